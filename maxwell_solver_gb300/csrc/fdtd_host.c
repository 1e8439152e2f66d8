/*
 * fdtd_host.c -- host side of the GB300 FDTD solver (plain C11).
 *
 * Implements the public C ABI of include/fdtd_gb300.h: the state and setup
 * of the reference's `simulation` class (enricoballini/maxwell_solver
 * src/simulation.h) and the dispatch of its per-op calls onto the fused
 * sm_103a kernels of fdtd_kernels.cu through the launchers declared in
 * fdtd_internal.h.
 *
 * Per-op calls are fused lazily: UpdateH_All, UpdateH_PlaneWave and
 * UpdateH_PML arriving in the reference order (highfrequency.m:85-91) are
 * queued and issued as one H half-step kernel when the next op needs their
 * result; the same for UpdateE_All / UpdateE_PlaneWave / UpdateE_PML /
 * AddCurrents.  Every op only touches its own cell's fields given the other
 * family, so the fused kernel applies exactly the same operations in the
 * same order.  Ops arriving out of that order flush the queue first.
 */
#define _GNU_SOURCE
#include <assert.h>
#include <math.h>
#include <pthread.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>
#include <time.h>

#include <cuda_runtime_api.h>

#include "../../include/fdtd_gb300.h"
#include "fdtd_internal.h"

/* physical constants, src/simulation.h:19-21 */
#define K_PI 3.14159265358979323846
static const double k_c0 = 299792458;
#define K_MU0 (4 * K_PI * 1e-7)
#define K_EPS0 (1 / k_c0 / k_c0 / K_MU0)

#define MAX_EVENTS 16
#define GRAPH_CHUNK 32
#define HASH_CAP 65536
#define MAX_MATERIALS 32768

/* ------------------------------------------------------------ errors */

static __thread char g_err[512];

static int fail(int code, const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
  return code;
}

const char *fdtd_last_error(void) { return g_err; }

/* Sets the thread's error message for entry points implemented in the
 * CUDA files (fdtd_internal.h). */
int fdtd_internal_fail(int code, const char *msg) { return fail(code, "%s", msg); }

#define CU(call)                                                           \
  do {                                                                     \
    cudaError_t e_ = (call);                                               \
    if (e_ != cudaSuccess)                                                 \
      return fail(e_ == cudaErrorMemoryAllocation ? FDTD_ERR_OOM : FDTD_ERR_CUDA, \
                  "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, \
                  __LINE__);                                               \
  } while (0)

#define KL(call)                                                           \
  do {                                                                     \
    int e_ = (call);                                                       \
    if (e_ != 0)                                                           \
      return fail(FDTD_ERR_CUDA, "%s: %s", #call,                          \
                  cudaGetErrorString((cudaError_t)e_));                    \
  } while (0)

/* ------------------------------------------------------------ state */

typedef struct {
  int active;      /* something queued */
  int h;           /* 1: H family, 0: E family */
  fdtd_op op;
} pending_t;

typedef struct sim {
  fdtd_params prm;
  int init_const, init_ready, init_1d, init_src, init_ant, init_mu;
  int32_t I, J, K, T, num_ant, p, size1d;
  int32_t Ip;            /* row pitch of the device field arrays */
  int64_t IJ, IJK, plane, cells;
  float fctr, delX, delT;
  float poly_m, alpha_m, sig_max, alpha_max, kappa_max;
  int32_t i0, i1, j0, j1, k0, k1;
  int64_t size_x, size_y, size_z;
  /* host copies (reference: pinned arrays of setConst / setSource) */
  float *d_raw[6];      /* sigma_x,y,z, eps_x,y,z as UpdateMaterial gave them
                           (device, packed I*J*K); unset: the defaults */
  int has_mat;          /* UpdateMaterial was called */
  /* media as shapes (fdtd_set_shapes): rasterised on the device instead */
  fdtd_shape *shapes;
  int32_t n_shapes;
  float bg_eps, bg_sigma;
  float *h_src;
  int64_t *h_probe_idx;
  float bE[2 * FDTD_MAX_PML], cE[2 * FDTD_MAX_PML];
  float bH[2 * FDTD_MAX_PML], cH[2 * FDTD_MAX_PML];
  float *h_den_ex, *h_den_hx;
  float Chh, Che;
  /* device */
  cudaStream_t stream;
  cudaEvent_t ev[MAX_EVENTS];
  float *d_f[6], *d_ce[6], *d_psi_pool, *d_psi[FDTD_NUM_PSI];
  float *d_den_ex, *d_den_hx, *d_inc[4], *d_src, *d_probes, *d_mu[3];
  /* per-cell H coefficients (fdtd_set_magnetic): mode 1 arrays, 2 indexed */
  int32_t hcoef_mode;
  float *d_hc, *d_htab;
  uint16_t *d_hmat;
  /* oblique plane wave (TF/SF mode 5) */
  int has_ob;
  double ob_theta, ob_phi, ob_psi;
  float ob_k[3], ob_e[3], ob_h[3], ob_x0, ob_speed, ob_rho;
  int32_t ob_r0[3], ob_w;
  float *d_ob[2];
  int64_t *d_probe_idx;
  int32_t *d_ctr; /* [0] step base, [1] probe row, [2..3] work queue */
  int32_t *d_err; /* device error word (bounded-wait timeouts) */
  uint16_t *d_mat;
  float *d_tab;
  unsigned long long *d_hkeys;
  int64_t *d_hrep;
  int32_t *d_hid, *d_hcnt;
  int32_t coef_mode, num_mat;
  int use_tma, allow_compress;
  fdtd_maps maps[FDTD_NUM_TILES]; /* per tile geometry (1: also the batch's) */
  int32_t tile_h, tile_e;          /* the autotuner's geometries */
  int32_t zc_h, zc_e; /* tuned z-planes per TMA work item (0: heuristic) */
  uint64_t device_bytes;
  fdtd_dev dev;
  pending_t pend;
  /* per-op steps in the reference order, held so that whole steps go to the
   * device as graph replays (like fdtd_step_n): UpdateH_All's probe gather
   * (belongs to the next H half-step), an H half-step waiting for the E
   * half-step of its step, and a run of complete steps */
  int gather_pending, held_h;
  fdtd_op held_op;
  int32_t run_first, run_n, run_mode;
  /* graph cache for fdtd_step_n */
  cudaGraphExec_t gexec;
  int g_mode, g_cur_mode, g_cur_box[6], g_probes;
  unsigned long long g_kernels;
  /* the fused step (fdtd_fused.cu): a second field buffer and second H psi
   * pairs, the descriptor with them (dev_b), the tensor maps of each buffer
   * as the step's source (fmaps[0]: the handle's, fmaps[1]: the second),
   * the z-run and whether the step uses it (fused: autotuned), its graph */
  float *d_fb[6], *d_psib_pool;
  fdtd_dev dev_b;
  fdtd_maps_fused fmaps[2];
  int32_t zc_f, fused;
  cudaGraphExec_t gexec_f;
  int gf_mode, gf_probes;
  unsigned long long gf_kernels;
} sim;

/* ------------------------------------------------------------ registry */

#define MAX_SIMS 4096
static pthread_mutex_t g_reg_lock = PTHREAD_MUTEX_INITIALIZER;
static sim *g_sims[MAX_SIMS];
static uint32_t g_gen[MAX_SIMS];
static unsigned long long g_graph_kernels = 0, g_captured_kernels = 0;

static sim *lookup(fdtd_handle h) {
  uint32_t slot = (uint32_t)(h & 0xffffffffu);
  uint32_t gen = (uint32_t)(h >> 32);
  if (slot == 0 || slot > MAX_SIMS) return NULL;
  pthread_mutex_lock(&g_reg_lock);
  sim *s = (g_gen[slot - 1] == gen) ? g_sims[slot - 1] : NULL;
  pthread_mutex_unlock(&g_reg_lock);
  return s;
}

#define GET(h)                                                             \
  sim *s = lookup(h);                                                      \
  if (!s) return fail(FDTD_ERR_INVALID_HANDLE, "invalid simulation handle")

/* ------------------------------------------------------------------
 * Division by the cell size.  The CPML recurrences divide by dx (12 times
 * in a corner cell); the kernels do it as a multiplication by y = RN(1/dx)
 * plus Markstein's correction step (P. Markstein, IBM J. Res. Dev. 34(1),
 * 1990; P. Cornea, J. Harrison, P. Tang, ARITH 14, 1999):
 * q0 = RN(a*y), r = RN(a - dx*q0), q = RN(q0 + r*y), one multiply and two
 * fused multiply-adds.  The plan says where that equals the IEEE quotient
 * RN(a/dx) bit for bit:
 *   - every significand of a in [1, 2) (2^23 values) is checked here
 *     against float division;
 *   - multiplying a by 2^e multiplies q0, r and q by 2^e with the same
 *     roundings as long as none of them (nor a/dx) leaves the normal
 *     range, so the check holds for every |a| in [lo, hi), the range where
 *     a*y and each nonzero r of the check, scaled, stay normal.
 * If any significand fails, lo = inf and every nonzero quotient is an
 * actual division.  Plans are cached per dx (grids share their cell size).
 * ------------------------------------------------------------------ */
static float f32_from_bits(uint32_t u) {
  float f;
  memcpy(&f, &u, sizeof(f));
  return f;
}

static fdtd_div_plan div_plan_compute(float dx) {
  fdtd_div_plan p = {dx, 1.0f / dx, INFINITY, 0.0f, INFINITY};
  if (!isnormal(dx) || !(dx > 0.0f)) return p;
  const float y = (float)(1.0 / (double)dx);
  if (!isnormal(y)) return p;
  float rmin = INFINITY; /* smallest nonzero |r| of the check */
  for (uint32_t m = 0; m < (1u << 23); ++m) {
    const float a = f32_from_bits(0x3F800000u | m);
    const float q0 = a * y;
    const float r = fmaf(-q0, dx, a);
    const float q = fmaf(r, y, q0);
    if (q != a / dx) return p;
    const float ar = fabsf(r);
    if (ar != 0.0f && ar < rmin) rmin = ar;
  }
  /* a = m * 2^e, m in [1, 2): need y*2^e >= 2^-126, rmin*2^e >= 2^-126 and
   * 2y*2^e < 2^127 (q0, q and a/dx are within an ulp of a*y); one binade
   * of margin on each side. */
  int ey, er;
  frexpf(y, &ey); /* y in [2^(ey-1), 2^ey) */
  int e_min = -125 - ey + 1;
  if (rmin != INFINITY) {
    frexpf(rmin, &er);
    if (-125 - er + 1 > e_min) e_min = -125 - er + 1;
  }
  int e_max = 126 - ey - 1;
  if (e_max > 125) e_max = 125;
  if (e_min < -125) e_min = -125;
  if (e_min > e_max) return p;
  p.rdx = y;
  p.lo = ldexpf(1.0f, e_min);
  p.hi = ldexpf(1.0f, e_max + 1);
  /* below lo: scale by 2^64 into [lo, hi), which needs |a| >= lo*2^-64 and
   * 2^64*lo <= hi; the scaled-back quotient is exact while it is normal,
   * |a/dx| >= 2^-126: |a| >= 2^-125*dx with one binade of margin */
  if (ldexpf(p.lo, 64) <= p.hi) {
    const float l1 = ldexpf(p.lo, -64), l2 = ldexpf(dx, -125);
    p.lo2 = l1 > l2 ? l1 : l2;
    if (!(p.lo2 < p.lo)) p.lo2 = p.lo;
  } else {
    p.lo2 = p.lo;
  }
  return p;
}

#define DIV_CACHE 8
static pthread_mutex_t g_div_lock = PTHREAD_MUTEX_INITIALIZER;
static fdtd_div_plan g_div_cache[DIV_CACHE];
static int g_div_used = 0, g_div_next = 0;

fdtd_div_plan fdtd_make_div_plan(float dx) {
  pthread_mutex_lock(&g_div_lock);
  for (int i = 0; i < g_div_used; ++i)
    if (memcmp(&g_div_cache[i].dx, &dx, sizeof(dx)) == 0) {
      const fdtd_div_plan p = g_div_cache[i];
      pthread_mutex_unlock(&g_div_lock);
      return p;
    }
  pthread_mutex_unlock(&g_div_lock);
  const fdtd_div_plan p = div_plan_compute(dx); /* ~50 ms, outside the lock */
  pthread_mutex_lock(&g_div_lock);
  g_div_cache[g_div_next] = p; /* round robin */
  g_div_next = (g_div_next + 1) % DIV_CACHE;
  if (g_div_used < DIV_CACHE) ++g_div_used;
  pthread_mutex_unlock(&g_div_lock);
  return p;
}

uint64_t fdtd_launch_count(void) {
  return (uint64_t)(fdtdk_launch_count() - g_captured_kernels + g_graph_kernels);
}

fdtd_params fdtd_default_params(void) {
  fdtd_params p;
  p.pml = 10;
  p.tfsf_width = 15;
  p.poly_m = 3;
  p.alpha_m = 1.0;
  p.alpha_max = 0.08;
  p.kappa_max = 1.0;
  p.sig_factor = 0.8;
  p.r0 = 0.0;
  return p;
}

/* Device memory comes from a pool owned by the library (one per device),
 * in stream order on the handle's stream: creating and deleting handles
 * while others run (as the serving loop does) never synchronises the
 * device the way cudaMalloc / cudaFree do.  Freed blocks stay in the pool
 * for the next handle; the pool gives them back when no handle is left. */
#define MAX_DEVICES 64
static pthread_mutex_t g_pool_lock = PTHREAD_MUTEX_INITIALIZER;
static cudaMemPool_t g_pool[MAX_DEVICES];
static int g_live_sims = 0;

static cudaError_t device_pool(cudaMemPool_t *out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= MAX_DEVICES) return cudaErrorInvalidDevice;
  pthread_mutex_lock(&g_pool_lock);
  if (!g_pool[dev]) {
    struct cudaMemPoolProps props;
    memset(&props, 0, sizeof(props));
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    e = cudaMemPoolCreate(&g_pool[dev], &props);
    if (e == cudaSuccess) {
      uint64_t keep = UINT64_MAX; /* cache freed blocks across handles */
      e = cudaMemPoolSetAttribute(g_pool[dev], cudaMemPoolAttrReleaseThreshold, &keep);
    }
    if (e != cudaSuccess) g_pool[dev] = NULL;
  }
  *out = g_pool[dev];
  pthread_mutex_unlock(&g_pool_lock);
  return e;
}

static void dfree_on(cudaStream_t st, void *p) {
  if (p) cudaFreeAsync(p, st);
}
#define dfree(p) dfree_on(s->stream, (p))

/* Stream-ordered allocation from the library's pool (see dalloc). */
static cudaError_t pool_alloc(void **p, size_t bytes, cudaStream_t st) {
  cudaMemPool_t pool;
  cudaError_t e = device_pool(&pool);
  if (e == cudaSuccess) e = cudaMallocFromPoolAsync(p, bytes ? bytes : 4, pool, st);
  if (e != cudaSuccess) *p = NULL;
  return e;
}


int fdtd_create(fdtd_handle *out) {
  if (!out) return fail(FDTD_ERR_INVALID_ARG, "null output handle");
  sim *s = (sim *)calloc(1, sizeof(sim));
  if (!s) return fail(FDTD_ERR_OOM, "out of host memory");
  s->prm = fdtd_default_params();
  /* FDTD_KERNELS=direct selects the direct kernels, FDTD_COEF=arrays the
   * per-cell coefficient arrays (both used by the comparison tests) */
  const char *ek = getenv("FDTD_KERNELS");
  const char *ec = getenv("FDTD_COEF");
  s->use_tma = !(ek && strcmp(ek, "direct") == 0);
  s->allow_compress = !(ec && strcmp(ec, "arrays") == 0);
  cudaError_t e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    free(s);
    return fail(FDTD_ERR_CUDA, "cudaStreamCreate: %s", cudaGetErrorString(e));
  }
  for (int i = 0; i < MAX_EVENTS; ++i) cudaEventCreate(&s->ev[i]);
  pthread_mutex_lock(&g_reg_lock);
  int slot = -1;
  for (int i = 0; i < MAX_SIMS; ++i)
    if (!g_sims[i]) {
      slot = i;
      break;
    }
  if (slot < 0) {
    pthread_mutex_unlock(&g_reg_lock);
    for (int i = 0; i < MAX_EVENTS; ++i) cudaEventDestroy(s->ev[i]);
    cudaStreamDestroy(s->stream);
    free(s);
    return fail(FDTD_ERR_OOM, "too many live simulations");
  }
  g_sims[slot] = s;
  g_gen[slot] += 1;
  *out = ((uint64_t)g_gen[slot] << 32) | (uint64_t)(slot + 1);
  pthread_mutex_unlock(&g_reg_lock);
  pthread_mutex_lock(&g_pool_lock);
  ++g_live_sims;
  pthread_mutex_unlock(&g_pool_lock);
  return FDTD_OK;
}


int fdtd_destroy(fdtd_handle h) {
  uint32_t slot = (uint32_t)(h & 0xffffffffu);
  sim *s = lookup(h);
  if (!s) return fail(FDTD_ERR_INVALID_HANDLE, "invalid simulation handle");
  pthread_mutex_lock(&g_reg_lock);
  g_sims[slot - 1] = NULL;
  pthread_mutex_unlock(&g_reg_lock);
  cudaStreamSynchronize(s->stream);
  if (s->gexec) cudaGraphExecDestroy(s->gexec);
  if (s->gexec_f) cudaGraphExecDestroy(s->gexec_f);
  dfree(s->d_psib_pool);
  for (int a = 0; a < 6; ++a) {
    dfree(s->d_fb[a]);
    dfree(s->d_f[a]);
    dfree(s->d_ce[a]);
    dfree(s->d_raw[a]);
  }
  free(s->shapes);
  for (int a = 0; a < 4; ++a) dfree(s->d_inc[a]);
  dfree(s->d_ob[0]);
  dfree(s->d_ob[1]);
  for (int a = 0; a < 3; ++a) dfree(s->d_mu[a]);
  dfree(s->d_hc);
  dfree(s->d_hmat);
  dfree(s->d_htab);
  dfree(s->d_psi_pool);
  dfree(s->d_den_ex);
  dfree(s->d_den_hx);
  dfree(s->d_src);
  dfree(s->d_probes);
  dfree(s->d_probe_idx);
  dfree(s->d_ctr);
  dfree(s->d_err);
  dfree(s->d_mat);
  dfree(s->d_tab);
  dfree(s->d_hkeys);
  dfree(s->d_hrep);
  dfree(s->d_hid);
  dfree(s->d_hcnt);
  free(s->h_src);
  free(s->h_probe_idx);
  free(s->h_den_ex);
  free(s->h_den_hx);
  for (int i = 0; i < MAX_EVENTS; ++i) cudaEventDestroy(s->ev[i]);
  cudaStreamSynchronize(s->stream); /* the frees above have run */
  cudaStreamDestroy(s->stream);
  free(s);
  pthread_mutex_lock(&g_pool_lock);
  if (--g_live_sims == 0)
    for (int d = 0; d < MAX_DEVICES; ++d)
      if (g_pool[d]) cudaMemPoolTrimTo(g_pool[d], 0);
  pthread_mutex_unlock(&g_pool_lock);
  return FDTD_OK;
}

/* Host-side fault injection (fdtd_inject_fault): the countdown of device
 * allocations until an injected failure; 0 = none armed. */
static int32_t g_fault_alloc = 0;

static int injected_alloc_failure(void) {
  int32_t v = __atomic_load_n(&g_fault_alloc, __ATOMIC_SEQ_CST);
  while (v > 0)
    if (__atomic_compare_exchange_n(&g_fault_alloc, &v, v - 1, 0, __ATOMIC_SEQ_CST,
                                    __ATOMIC_SEQ_CST))
      return v == 1;
  return 0;
}

int fdtd_inject_fault(int32_t kind, int32_t countdown) {
  if (kind == FDTD_FAULT_NONE) {
    __atomic_store_n(&g_fault_alloc, 0, __ATOMIC_SEQ_CST);
    return FDTD_OK;
  }
  if (kind != FDTD_FAULT_DEVICE_ALLOC || countdown < 1)
    return fail(FDTD_ERR_INVALID_ARG, "fault kind %d / countdown %d", kind, countdown);
  __atomic_store_n(&g_fault_alloc, countdown, __ATOMIC_SEQ_CST);
  return FDTD_OK;
}

static int dalloc(sim *s, void **p, size_t bytes) {
  if (injected_alloc_failure()) {
    *p = NULL;
    return fail(FDTD_ERR_OOM, "device allocation of %zu bytes: injected failure", bytes);
  }
  cudaMemPool_t pool;
  cudaError_t e = device_pool(&pool);
  if (e == cudaSuccess) e = cudaMallocFromPoolAsync(p, bytes ? bytes : 4, pool, s->stream);
  if (e != cudaSuccess) {
    *p = NULL;
    cudaGetLastError();
    return fail(FDTD_ERR_OOM, "device allocation of %zu bytes: %s", bytes,
                cudaGetErrorString(e));
  }
  s->device_bytes += bytes;
  return FDTD_OK;
}

/* ------------------------------------------------------------ setup */

int fdtd_set_params(fdtd_handle h, const fdtd_params *p) {
  GET(h);
  if (!p) return fail(FDTD_ERR_INVALID_ARG, "null params");
  if (s->init_const) return fail(FDTD_ERR_STATE, "SetParams must precede SetConst");
  if (p->pml < 2 || p->pml > FDTD_MAX_PML)
    return fail(FDTD_ERR_UNSUPPORTED, "pml must be in [2, %d]", FDTD_MAX_PML);
  if (p->tfsf_width < 1) return fail(FDTD_ERR_INVALID_ARG, "tfsf_width must be >= 1");
  s->prm = *p;
  return FDTD_OK;
}

/* src/simulation.h:79-131 */
int fdtd_set_const(fdtd_handle h, const float freqRes[3], const int32_t timeDim[5]) {
  GET(h);
  if (s->init_const)
    return fail(FDTD_ERR_ALREADY_INITIALIZED, "SetConst: already called.");
  if (!freqRes || !timeDim) return fail(FDTD_ERR_INVALID_ARG, "freqRes and TimeDim required.");
  const int32_t T = timeDim[0], I = timeDim[1], J = timeDim[2], K = timeDim[3];
  const int32_t na = timeDim[4];
  const int32_t p = s->prm.pml;
  if (T < 1 || na < 0) return fail(FDTD_ERR_INVALID_ARG, "TimeDim: T >= 1, numAnt >= 0");
  if (I < 2 * p + 2 || J < 2 * p + 2 || K < 2 * p + 2)
    return fail(FDTD_ERR_UNSUPPORTED, "grid %dx%dx%d too small for a %d-cell CPML", I, J, K, p);
  if (!(freqRes[1] > 0.0f) || !(freqRes[2] > 0.0f))
    return fail(FDTD_ERR_INVALID_ARG, "delX and delT must be positive");
  s->fctr = freqRes[0];
  s->delX = freqRes[1];
  s->delT = freqRes[2];
  s->poly_m = (float)s->prm.poly_m;
  s->alpha_m = (float)s->prm.alpha_m;
  if (s->prm.r0 > 0.0)
    s->sig_max = (float)(-((double)s->poly_m + 1.0) * log(s->prm.r0) /
                         (2.0 * sqrt(K_MU0 / K_EPS0) * (double)p * (double)s->delX));
  else
    s->sig_max = (float)(s->prm.sig_factor * ((double)s->poly_m + 1.0) /
                         (sqrt(K_MU0 / K_EPS0) * (double)s->delX));
  s->alpha_max = (float)s->prm.alpha_max;
  s->kappa_max = (float)s->prm.kappa_max;
  s->T = T;
  s->I = I;
  s->J = J;
  s->K = K;
  s->num_ant = na;
  s->p = p;
  s->IJ = (int64_t)I * J;
  s->IJK = s->IJ * K;
  s->Ip = (I + 7) / 8 * 8;
  s->plane = (int64_t)s->Ip * J;
  s->cells = s->plane * K;
  const int32_t w = s->prm.tfsf_width;
  s->i0 = w;
  s->i1 = I - w - 1;
  s->j0 = w;
  s->j1 = J - w - 1;
  s->k0 = w;
  s->k1 = K - w - 1;
  s->size_x = (int64_t)p * J * K;
  s->size_y = (int64_t)I * p * K;
  s->size_z = (int64_t)I * J * p;
  s->init_const = 1;
  return FDTD_OK;
}

/* Value of a material array (0..2 sigma, 3..5 eps) that UpdateMaterial
 * never set: sigma 0, eps 1. */
static float material_default(int a) { return a < 3 ? 0.0f : 1.0f; }

/* src/simulation.h:1068-1082 */
int fdtd_set_source(fdtd_handle h, const float *src, size_t n) {
  GET(h);
  if (!s->init_const) return fail(FDTD_ERR_STATE, "SetSource requires SetConst");
  if (!src || n < (size_t)s->T) return fail(FDTD_ERR_INVALID_ARG, "SourceIn needs T=%d values", s->T);
  if (s->init_src) return FDTD_OK; /* reference: "Source is already initialized" */
  s->h_src = (float *)malloc((size_t)s->T * sizeof(float));
  if (!s->h_src) return fail(FDTD_ERR_OOM, "out of host memory");
  memcpy(s->h_src, src, (size_t)s->T * sizeof(float));
  int rc = dalloc(s, (void **)&s->d_src, (size_t)s->T * sizeof(float));
  if (rc) return rc;
  CU(cudaMemcpyAsync(s->d_src, s->h_src, (size_t)s->T * sizeof(float),
                     cudaMemcpyHostToDevice, s->stream));
  CU(cudaStreamSynchronize(s->stream));
  s->dev.src = s->d_src;
  s->init_src = 1;
  return FDTD_OK;
}

static int flush(sim *s);
static int check_device_error(sim *s);
static int issue(sim *s, int hfam, const fdtd_op *op);

/* src/simulation.h:1084-1095 */
int fdtd_update_source(fdtd_handle h, const float *src, size_t n) {
  GET(h);
  if (!s->init_src) return FDTD_OK; /* reference: "Source is not initialized" */
  if (!src || n < (size_t)s->T) return fail(FDTD_ERR_INVALID_ARG, "SourceIn needs T=%d values", s->T);
  int rc = flush(s);
  if (rc) return rc;
  memcpy(s->h_src, src, (size_t)s->T * sizeof(float));
  CU(cudaMemcpyAsync(s->d_src, s->h_src, (size_t)s->T * sizeof(float),
                     cudaMemcpyHostToDevice, s->stream));
  CU(cudaStreamSynchronize(s->stream));
  return FDTD_OK;
}

/* src/simulation.h:288-328 */
int fdtd_update_material(fdtd_handle h, int32_t flag, const float *values, size_t n) {
  GET(h);
  if (!s->init_const) return fail(FDTD_ERR_STATE, "UpdateMaterial requires SetConst");
  if (flag < 1 || flag > 6) return FDTD_OK;
  if (!values || n < (size_t)s->IJK)
    return fail(FDTD_ERR_INVALID_ARG, "UpdateMaterial needs Imax*Jmax*Kmax=%lld values",
                (long long)s->IJK);
  if (s->shapes)
    return fail(FDTD_ERR_STATE, "UpdateMaterial after SetShapes: the media are the shapes");
  /* kept on the device as given; the copy is complete when this returns */
  const size_t bytes = (size_t)s->IJK * sizeof(float);
  int rc;
  if (!s->d_raw[flag - 1] && (rc = dalloc(s, (void **)&s->d_raw[flag - 1], bytes))) return rc;
  CU(cudaMemcpyAsync(s->d_raw[flag - 1], values, bytes, cudaMemcpyHostToDevice, s->stream));
  CU(cudaStreamSynchronize(s->stream));
  s->has_mat = 1;
  return FDTD_OK;
}

int fdtd_set_shapes(fdtd_handle h, float bg_eps_r, float bg_sigma, const fdtd_shape *shapes,
                    int32_t n) {
  GET(h);
  if (!s->init_const) return fail(FDTD_ERR_STATE, "SetShapes requires SetConst");
  if (s->has_mat) return fail(FDTD_ERR_STATE, "SetShapes after UpdateMaterial");
  if (n < 0 || (n > 0 && !shapes) || n > FDTD_MAX_SHAPES)
    return fail(FDTD_ERR_INVALID_ARG, "SetShapes takes 0..%d shapes", FDTD_MAX_SHAPES);
  for (int a = 0; a < n; ++a)
    if (shapes[a].kind < FDTD_SHAPE_SPHERE || shapes[a].kind > FDTD_SHAPE_BOX)
      return fail(FDTD_ERR_INVALID_ARG, "shape %d: unknown kind %d", a, shapes[a].kind);
  fdtd_shape *copy = (fdtd_shape *)malloc((size_t)(n > 0 ? n : 1) * sizeof(fdtd_shape));
  if (!copy) return fail(FDTD_ERR_OOM, "out of host memory");
  if (n) memcpy(copy, shapes, (size_t)n * sizeof(fdtd_shape));
  free(s->shapes);
  s->shapes = copy;
  s->n_shapes = n;
  s->bg_eps = bg_eps_r;
  s->bg_sigma = bg_sigma;
  /* taking effect needs ReadySimulation (or UpdateCuda after it), like
   * UpdateMaterial */
  return FDTD_OK;
}

/* src/simulation.h:1047-1067 */
int fdtd_set_antenna_locations(fdtd_handle h, const int32_t *loc, size_t n) {
  GET(h);
  if (!s->init_const) return fail(FDTD_ERR_STATE, "SetAntennaLocations requires SetConst");
  if (s->init_ready)
    return fail(FDTD_ERR_STATE, "SetAntennaLocations must precede ReadySimulation");
  if (n < (size_t)s->num_ant * 3 || (!loc && s->num_ant))
    return fail(FDTD_ERR_INVALID_ARG, "Locations needs numAnt x 3 = %d values", s->num_ant * 3);
  free(s->h_probe_idx);
  s->h_probe_idx = (int64_t *)calloc((size_t)(s->num_ant ? s->num_ant : 1), sizeof(int64_t));
  for (int a = 0; a < s->num_ant; ++a) {
    const int64_t x = (int64_t)s->p + loc[a + 0 * s->num_ant];
    const int64_t y = (int64_t)s->p + loc[a + 1 * s->num_ant];
    const int64_t z = (int64_t)s->p + loc[a + 2 * s->num_ant];
    const int inside = x >= 0 && x < s->I && y >= 0 && y < s->J && z >= 0 && z < s->K;
    s->h_probe_idx[a] = inside ? x + y * s->Ip + z * s->Ip * (int64_t)s->J : -1;
  }
  s->init_ant = 1;
  return FDTD_OK;
}

/* CPML grading samples, src/simulation.h:730-767 */
static void cpml_sample(const sim *s, double num_sig, double num_alpha, float *sig,
                        float *alpha, float *kappa) {
  const double pm1 = (double)s->p - 1.0;
  *sig = (float)((double)s->sig_max * pow(num_sig / pm1, (double)s->poly_m));
  *alpha = (float)((double)s->alpha_max * pow(num_alpha / pm1, (double)s->alpha_m));
  *kappa = (float)(1.0 + ((double)s->kappa_max - 1.0) * pow(num_sig / pm1, (double)s->poly_m));
}

static float cpml_b(const sim *s, float sig, float alpha, float kappa) {
  float t = sig / kappa;
  t = t + alpha;
  t = -t;
  t = t * s->delT;
  return (float)exp((double)t / K_EPS0);
}

static float cpml_c(float sig, float alpha, float kappa, float b) {
  const float u1 = sig / kappa;
  const float u2 = kappa * alpha;
  const float u3 = sig + u2;
  const float u4 = u1 / u3;
  return (float)((double)u4 * ((double)b - 1.0));
}

static void build_tables(sim *s, float *kaE, float *kaH) {
  const int p = s->p;
  float sigE[FDTD_MAX_PML], alE[FDTD_MAX_PML], bE1[FDTD_MAX_PML], cE1[FDTD_MAX_PML];
  float sigH[FDTD_MAX_PML], alH[FDTD_MAX_PML], bH1[FDTD_MAX_PML], cH1[FDTD_MAX_PML];
  memset(s->bE, 0, sizeof(s->bE));
  memset(s->cE, 0, sizeof(s->cE));
  memset(s->bH, 0, sizeof(s->bH));
  memset(s->cH, 0, sizeof(s->cH));
  for (int i = 0; i < p; ++i) { /* :730-749 */
    cpml_sample(s, (double)(p - i - 1), (double)(i + 1) - 1.0, &sigE[i], &alE[i], &kaE[i]);
    bE1[i] = cpml_b(s, sigE[i], alE[i], kaE[i]);
    if (sigE[i] == 0.0f && alE[i] == 0.0f && (i + 1) == (p - 1))
      cE1[i] = 0.0f;
    else
      cE1[i] = cpml_c(sigE[i], alE[i], kaE[i], bE1[i]);
  }
  for (int i = 0; i + 1 < p; ++i) { /* :752-767 */
    cpml_sample(s, (double)(p - i - 1) - 0.5, (double)(i + 1) - 0.5, &sigH[i], &alH[i], &kaH[i]);
    bH1[i] = cpml_b(s, sigH[i], alH[i], kaH[i]);
    cH1[i] = cpml_c(sigH[i], alH[i], kaH[i], bH1[i]);
  }
  for (int i = 0; i < p; ++i) { /* :772-822 */
    s->bE[i] = bE1[i];
    s->cE[i] = cE1[i];
    s->bE[p + i] = bE1[p - 1 - i];
    s->cE[p + i] = cE1[p - 1 - i];
  }
  for (int i = 0; i + 1 < p; ++i) {
    s->bH[i] = bH1[i];
    s->cH[i] = cH1[i];
    s->bH[p + i] = bH1[p - 2 - i];
    s->cH[p + i] = cH1[p - 2 - i];
  }
}

/* The second buffer's descriptor and both buffers' tensor maps for the
 * fused step, after every change of the handle's descriptor. */
static void fused_refresh(sim *s) {
  if (s->gexec_f) {
    cudaGraphExecDestroy(s->gexec_f);
    s->gexec_f = NULL;
  }
  s->fmaps[0].valid = s->fmaps[1].valid = 0;
  if (!s->d_fb[0] || !s->d_psib_pool) return;
  s->dev_b = s->dev;
  for (int a = 0; a < 6; ++a) s->dev_b.f[a] = s->d_fb[a];
  s->dev_b.psi[PSI_HY] = s->d_psib_pool;
  s->dev_b.psi[PSI_HX] = s->d_psib_pool + 4 * s->size_y;
  s->dev_b.psi[PSI_HZ] = s->d_psib_pool + 4 * (s->size_y + s->size_x);
  if (fdtdk_make_maps_fused(&s->dev, &s->fmaps[0])) s->fmaps[0].valid = 0;
  if (fdtdk_make_maps_fused(&s->dev_b, &s->fmaps[1])) s->fmaps[1].valid = 0;
}

static void fill_dev_struct(sim *s) {
  fdtd_dev *d = &s->dev;
  if (s->gexec) { /* a captured step graph holds the old descriptor */
    cudaGraphExecDestroy(s->gexec);
    s->gexec = NULL;
  }
  d->I = s->I;
  d->J = s->J;
  d->K = s->K;
  d->p = s->p;
  d->Ip = s->Ip;
  d->IJ = s->IJ;
  d->IJK = s->IJK;
  d->plane = s->plane;
  d->cells = s->cells;
  d->i0 = s->i0;
  d->i1 = s->i1;
  d->j0 = s->j0;
  d->j1 = s->j1;
  d->k0 = s->k0;
  d->k1 = s->k1;
  d->size1d = s->size1d;
  d->T = s->T;
  d->Chh = s->Chh;
  d->Che = s->Che;
  d->dx = s->delX;
  {
    const fdtd_div_plan dp = fdtd_make_div_plan(s->delX);
    d->rdx = dp.rdx;
    d->div_lo = dp.lo;
    d->div_hi = dp.hi;
    d->div_lo2 = dp.lo2;
  }
  memcpy(d->bE, s->bE, sizeof(d->bE));
  memcpy(d->cE, s->cE, sizeof(d->cE));
  memcpy(d->bH, s->bH, sizeof(d->bH));
  memcpy(d->cH, s->cH, sizeof(d->cH));
  for (int a = 0; a < 6; ++a) {
    d->f[a] = s->d_f[a];
    d->ce[a] = s->d_ce[a];
  }
  d->coef_mode = s->coef_mode;
  d->mat = s->d_mat;
  d->mat_tab = s->d_tab;
  d->n_mat = s->num_mat;
  d->hcoef_mode = s->hcoef_mode;
  d->hc = s->d_hc;
  d->hmat = s->d_hmat;
  d->hmat_tab = s->d_htab;
  d->err = s->d_err;
  d->zc_h = s->zc_h;
  d->zc_e = s->zc_e;
  d->tile_h = s->tile_h;
  d->tile_e = s->tile_e;
  for (int a = 0; a < FDTD_NUM_PSI; ++a) d->psi[a] = s->d_psi[a];
  for (int a = 0; a < 4; ++a) d->inc[a] = s->d_inc[a];
  d->src = s->d_src;
  for (int a = 0; a < 3; ++a) {
    d->ob_k[a] = s->ob_k[a];
    d->ob_e[a] = s->ob_e[a];
    d->ob_h[a] = s->ob_h[a];
    d->ob_r0[a] = s->ob_r0[a];
  }
  d->ob_x0 = s->ob_x0;
  d->ob_rho = s->ob_rho;
  d->ob_w = s->ob_w;
  d->ob_inc[0] = s->d_ob[0];
  d->ob_inc[1] = s->d_ob[1];
  d->step_base = s->d_ctr;
  d->probe_row = s->d_ctr ? s->d_ctr + 1 : NULL;
  d->work = s->d_ctr ? s->d_ctr + 2 : NULL;
  d->probes = s->d_probes;
  d->probe_idx = s->d_probe_idx;
  d->num_ant = (s->init_ant && s->d_probes) ? s->num_ant : 0;
  fused_refresh(s);
}

/* Material of cell (i,j,k) from the shapes (see k_rasterize; the same
 * double-precision tests, each operation rounded on its own). */
static void shape_material(const sim *s, int i, int j, int k, float *eps, float *sig) {
  float e = s->bg_eps, sg = s->bg_sigma;
  for (int a = 0; a < s->n_shapes; ++a) {
    const fdtd_shape *sh = &s->shapes[a];
    int in = 0;
    if (sh->kind == FDTD_SHAPE_SPHERE) {
      const double x = ((double)i + 0.5) - sh->g[0];
      const double y = ((double)j + 0.5) - sh->g[1];
      const double z = ((double)k + 0.5) - sh->g[2];
      const double xx = x * x, yy = y * y, zz = z * z;
      const double xy = xx + yy;
      const double d2 = xy + zz;
      const double rr = sh->g[3] * sh->g[3];
      in = d2 <= rr;
    } else if (sh->kind == FDTD_SHAPE_LAYER_Z) {
      in = (double)k >= sh->g[0] && (double)k < sh->g[1];
    } else if (sh->kind == FDTD_SHAPE_BOX) {
      in = (double)i >= sh->g[0] && (double)i < sh->g[1] && (double)j >= sh->g[2] &&
           (double)j < sh->g[3] && (double)k >= sh->g[4] && (double)k < sh->g[5];
    }
    if (in) {
      e = sh->eps_r;
      sg = sh->sigma;
    }
  }
  *eps = e;
  *sig = sg;
}

/* Fills the six material arrays on the device (from the shapes, or from
 * the host arrays UpdateMaterial filled), turns them into Cexe..Cezh in
 * place (src/simulation.h:924-951 / :1099-1126), and, when the grid's
 * coefficient tuples fit the material table, indexes them and releases the
 * per-cell arrays (the kernels then read the 2-byte ids only). */
static int upload_coefficients(sim *s) {
  const size_t bytes = (size_t)s->cells * sizeof(float);
  int rc = FDTD_OK;
  for (int a = 0; a < 6; ++a)
    if (!s->d_ce[a] && (rc = dalloc(s, (void **)&s->d_ce[a], bytes))) return rc;
  fill_dev_struct(s);
  /* sigma_x -> ce[0], sigma_y -> ce[1], sigma_z -> ce[2], eps -> ce[3..5]:
   * the kernel reads both inputs of a component before writing its outputs */
  if (s->shapes) {
    fdtd_shape *d_shapes = NULL;
    const size_t sb = (size_t)(s->n_shapes > 0 ? s->n_shapes : 1) * sizeof(fdtd_shape);
    CU(pool_alloc((void **)&d_shapes, sb, s->stream));
    if (s->n_shapes)
      CU(cudaMemcpyAsync(d_shapes, s->shapes, (size_t)s->n_shapes * sizeof(fdtd_shape),
                         cudaMemcpyHostToDevice, s->stream));
    float *sg[3] = {s->d_ce[0], s->d_ce[1], s->d_ce[2]};
    float *ep[3] = {s->d_ce[3], s->d_ce[4], s->d_ce[5]};
    const int e = fdtdk_rasterize(&s->dev, sg, ep, d_shapes, s->n_shapes, s->bg_eps,
                                  s->bg_sigma, s->stream);
    dfree(d_shapes);
    KL(e);
  } else {
    const size_t row = (size_t)s->I * sizeof(float);
    for (int a = 0; a < 6; ++a) {
      if (!s->d_raw[a]) {
        KL(fdtdk_fill_f32(s->d_ce[a], material_default(a), s->cells, s->stream));
      } else if (s->Ip == s->I) {
        CU(cudaMemcpyAsync(s->d_ce[a], s->d_raw[a], (size_t)s->IJK * sizeof(float),
                           cudaMemcpyDeviceToDevice, s->stream));
      } else { /* packed rows to pitched rows */
        CU(cudaMemcpy2DAsync(s->d_ce[a], (size_t)s->Ip * sizeof(float), s->d_raw[a], row, row,
                             (size_t)s->J * s->K, cudaMemcpyDeviceToDevice, s->stream));
      }
    }
  }
  float *ce[6];
  const float *eps[3], *sig[3];
  for (int a = 0; a < 6; ++a) ce[a] = s->d_ce[a];
  for (int a = 0; a < 3; ++a) {
    sig[a] = s->d_ce[a];
    eps[a] = s->d_ce[3 + a];
  }
  KL(fdtdk_compute_ce(&s->dev, ce, eps, sig, s->d_den_ex, s->delT, s->stream));
  /* material-indexed coefficients: the kernels then read a 2-byte id per
   * cell instead of six floats; falls back to the arrays when the grid has
   * more than MAX_MATERIALS distinct tuples */
  s->coef_mode = 0;
  s->num_mat = 0;
  if (s->allow_compress) {
    const float *cc[6];
    for (int a = 0; a < 6; ++a) cc[a] = s->d_ce[a];
    KL(fdtdk_compress_ce(&s->dev, cc, s->d_mat, s->d_tab, MAX_MATERIALS, s->d_hkeys, s->d_hrep,
                         s->d_hid, HASH_CAP, s->d_hcnt, s->stream));
    int32_t cnt[4];
    CU(cudaMemcpyAsync(cnt, s->d_hcnt, sizeof(cnt), cudaMemcpyDeviceToHost, s->stream));
    CU(cudaStreamSynchronize(s->stream));
    if (!cnt[1] && !cnt[2] && cnt[0] > 0 && cnt[0] <= MAX_MATERIALS) {
      s->coef_mode = 1;
      s->num_mat = cnt[0];
      for (int a = 0; a < 6; ++a) { /* UpdateCuda allocates them again */
        dfree(s->d_ce[a]);
        s->d_ce[a] = NULL;
        s->device_bytes -= bytes;
      }
    }
  }
  fill_dev_struct(s);
  return FDTD_OK;
}

static int zero_state(sim *s) {
  const size_t bytes = (size_t)s->cells * sizeof(float);
  for (int a = 0; a < 6; ++a) CU(cudaMemsetAsync(s->d_f[a], 0, bytes, s->stream));
  const size_t psi_total = (size_t)(4 * 2 * (s->size_x + s->size_y + s->size_z)) * sizeof(float);
  CU(cudaMemsetAsync(s->d_psi_pool, 0, psi_total, s->stream));
  CU(cudaMemsetAsync(s->d_ctr, 0, 4 * sizeof(int32_t), s->stream));
  for (int a = 0; a < 6; ++a)
    if (s->d_fb[a]) CU(cudaMemsetAsync(s->d_fb[a], 0, bytes, s->stream));
  if (s->d_psib_pool)
    CU(cudaMemsetAsync(s->d_psib_pool, 0, psi_total / 2, s->stream));
  return FDTD_OK;
}

/* ------------------------------------------------------------ autotune
 *
 * Measured once per grid shape at the end of ReadySimulation, while every
 * field and psi value is still exactly zero (a source-free step maps zero
 * to zero exactly, so the trial steps leave the state bit-identical and
 * need no snapshot):
 *   - the work-item height (z-planes per item, 2..32) of each half-step
 *     kernel: how many items keep the GPU busy, how wide a band of planes
 *     the blocks sweep together;
 *   - the fused H+E pass against the two half-step kernels (E/H fusion
 *     depth 2 or 1), and the fused pass's item height (8..64);
 * Results are kept per process and in a text file (FDTD_TUNE_CACHE, default
 * $HOME/.cache/fdtd_gb300/autotune.txt), keyed by the grid shape, the
 * coefficient layouts, the device (name and SM count) and the library
 * build (kernels change between builds), so an entry measured elsewhere is
 * not reused; FDTD_AUTOTUNE=0 disables it. */

#define TUNE_MAX 256
#define TUNE_MIN_CELLS ((int64_t)1 << 21) /* smaller grids: built-in heuristics */

static int tune_enabled(void) {
  const char *e = getenv("FDTD_AUTOTUNE");
  return !(e && strcmp(e, "0") == 0);
}
typedef struct {
  char key[96]; /* device and build */
  int32_t I, J, K, p, coef_mode, hcoef_mode, zh, ze, zf, fused, th, te;
} tune_entry;
static tune_entry g_tune[TUNE_MAX];
static int g_tune_n = 0, g_tune_loaded = 0;
static pthread_mutex_t g_tune_lock = PTHREAD_MUTEX_INITIALIZER;

/* "<device name>|sm<count>|<build>" with blanks replaced. */
static void tune_key(char *buf, size_t n) {
  int dev = 0, sms = 0;
  struct cudaDeviceProp pr;
  memset(&pr, 0, sizeof(pr));
  cudaGetDevice(&dev);
  if (cudaGetDeviceProperties(&pr, dev) != cudaSuccess) snprintf(pr.name, sizeof(pr.name), "?");
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  snprintf(buf, n, "%s|sm%d|%s_%s", pr.name, sms, __DATE__, __TIME__);
  for (char *c = buf; *c; ++c)
    if (*c == ' ' || *c == '\t') *c = '_';
}

static void tune_cache_path(char *buf, size_t n) {
  const char *e = getenv("FDTD_TUNE_CACHE");
  const char *home = getenv("HOME");
  if (e) snprintf(buf, n, "%s", e);
  else if (home) snprintf(buf, n, "%s/.cache/fdtd_gb300/autotune.txt", home);
  else buf[0] = '\0';
}

static void tune_load(void) {
  if (g_tune_loaded) return;
  g_tune_loaded = 1;
  char path[512], line[512];
  tune_cache_path(path, sizeof(path));
  if (!path[0]) return;
  FILE *f = fopen(path, "r");
  if (!f) return;
  while (g_tune_n < TUNE_MAX && fgets(line, sizeof(line), f)) {
    tune_entry t;
    if (sscanf(line, "v3 %95s %d %d %d %d %d %d %d %d %d %d %d %d", t.key, &t.I, &t.J, &t.K,
               &t.p, &t.coef_mode, &t.hcoef_mode, &t.zh, &t.ze, &t.zf, &t.fused, &t.th,
               &t.te) == 13)
      g_tune[g_tune_n++] = t; /* older formats are skipped */
  }
  fclose(f);
}

static void tune_store(const tune_entry *t) {
  if (g_tune_n < TUNE_MAX) g_tune[g_tune_n++] = *t;
  char path[512];
  tune_cache_path(path, sizeof(path));
  if (!path[0]) return;
  char dir[512];
  snprintf(dir, sizeof(dir), "%s", path);
  char *slash = strrchr(dir, '/');
  if (slash) { /* best effort: create the two last directory levels */
    *slash = '\0';
    char *up = strrchr(dir, '/');
    if (up) {
      *up = '\0';
      mkdir(dir, 0755);
      *up = '/';
    }
    mkdir(dir, 0755);
  }
  FILE *f = fopen(path, "a");
  if (!f) return;
  fprintf(f, "v3 %s %d %d %d %d %d %d %d %d %d %d %d %d\n", t->key, t->I, t->J, t->K, t->p,
          t->coef_mode, t->hcoef_mode, t->zh, t->ze, t->zf, t->fused, t->th, t->te);
  fclose(f);
}

/* Mean device time of the H and E half-steps over `steps` source-free steps
 * with z-run length z in tile geometry `tile` (after one untimed step). */
static int tune_measure(sim *s, int tile, int z, int steps, float *th, float *te) {
  fdtd_op op;
  memset(&op, 0, sizeof(op));
  op.curl = 1;
  op.pml = 1;
  s->dev.zc_h = s->dev.zc_e = z;
  s->dev.tile_h = s->dev.tile_e = tile;
  float sh = 0, se = 0;
  for (int c = -1; c < steps; ++c) {
    CU(cudaEventRecord(s->ev[12], s->stream));
    int rc = issue(s, 1, &op);
    if (rc) return rc;
    CU(cudaEventRecord(s->ev[13], s->stream));
    if ((rc = issue(s, 0, &op))) return rc;
    CU(cudaEventRecord(s->ev[14], s->stream));
    CU(cudaEventSynchronize(s->ev[14]));
    float a = 0, b = 0;
    CU(cudaEventElapsedTime(&a, s->ev[12], s->ev[13]));
    CU(cudaEventElapsedTime(&b, s->ev[13], s->ev[14]));
    if (c >= 0) {
      sh += a;
      se += b;
    }
  }
  *th = sh / steps;
  *te = se / steps;
  return FDTD_OK;
}

/* Mean device time per step of source-free fused pairs with item height z
 * (after one untimed pair). */
static int tune_measure_fused(sim *s, int z, int pairs, float *t) {
  fdtd_op op;
  memset(&op, 0, sizeof(op));
  op.curl = 1;
  op.pml = 1;
  float sum = 0;
  for (int c = -1; c < pairs; ++c) {
    CU(cudaEventRecord(s->ev[12], s->stream));
    KL(fdtdk_step_fused(&s->dev_b, &s->dev, &s->fmaps[0], &op, z, s->stream));
    KL(fdtdk_step_fused(&s->dev, &s->dev_b, &s->fmaps[1], &op, z, s->stream));
    CU(cudaEventRecord(s->ev[13], s->stream));
    CU(cudaEventSynchronize(s->ev[13]));
    float a = 0;
    CU(cudaEventElapsedTime(&a, s->ev[12], s->ev[13]));
    if (c >= 0) sum += a;
  }
  *t = sum / (2 * pairs);
  return FDTD_OK;
}

static int fused_usable(sim *s, int32_t mode, const fdtd_current *cur);
static int fused_mode(void);

/* The fused step's second buffer goes back to the pool when the autotuner
 * chose the half-step kernels. */
static void release_second_buffer(sim *s) {
  if (!s->d_fb[0]) return;
  for (int a = 0; a < 6; ++a) {
    dfree(s->d_fb[a]);
    s->d_fb[a] = NULL;
  }
  dfree(s->d_psib_pool);
  s->d_psib_pool = NULL;
  s->device_bytes -= (uint64_t)6 * s->cells * sizeof(float) +
                     (uint64_t)4 * (s->size_x + s->size_y + s->size_z) * sizeof(float);
  s->fused = 0;
}

static int autotune_zero_state(sim *s) {
  if (!tune_enabled() || !s->use_tma || !s->maps[0].valid) return FDTD_OK;
  if (s->cells < TUNE_MIN_CELLS) return FDTD_OK; /* small grids: heuristic */
  char key[96];
  tune_key(key, sizeof(key));
  pthread_mutex_lock(&g_tune_lock);
  tune_load();
  for (int i = 0; i < g_tune_n; ++i) {
    const tune_entry *t = &g_tune[i];
    if (t->I == s->I && t->J == s->J && t->K == s->K && t->p == s->p &&
        t->coef_mode == s->coef_mode && t->hcoef_mode == s->hcoef_mode &&
        strcmp(t->key, key) == 0) {
      s->zc_h = t->zh;
      s->zc_e = t->ze;
      s->tile_h = t->th;
      s->tile_e = t->te;
      s->zc_f = t->zf;
      s->fused = s->fused && (t->fused || fused_mode() == 1);
      pthread_mutex_unlock(&g_tune_lock);
      if (!s->fused) release_second_buffer(s);
      fill_dev_struct(s);
      return FDTD_OK;
    }
  }
  pthread_mutex_unlock(&g_tune_lock);
  static const int cand[] = {2, 4, 8, 16, 32};
  float best_h = 1e30f, best_e = 1e30f;
  int zh = 0, ze = 0, tlh = 0, tle = 0;
  for (int tile = 0; tile < FDTD_NUM_TILES; ++tile) {
    if (!s->maps[tile].valid) continue;
    for (size_t c = 0; c < sizeof(cand) / sizeof(cand[0]); ++c) {
      if (cand[c] > s->K) break;
      float th = 0, te = 0;
      int rc = tune_measure(s, tile, cand[c], 3, &th, &te);
      if (rc) return rc;
      if (th < best_h) { best_h = th; zh = cand[c]; tlh = tile; }
      if (te < best_e) { best_e = te; ze = cand[c]; tle = tile; }
    }
  }
  s->zc_h = zh;
  s->zc_e = ze;
  s->tile_h = tlh;
  s->tile_e = tle;
  fill_dev_struct(s); /* the tuned half-steps for the fused comparison */
  int zf = 0, fused = 0;
  if (fused_usable(s, 0, NULL)) {
    static const int fcand[] = {8, 16, 32, 64};
    float best_f = 1e30f;
    for (size_t c = 0; c < sizeof(fcand) / sizeof(fcand[0]); ++c) {
      if (fcand[c] > s->K && c > 0) break;
      float tf = 0;
      int rc = tune_measure_fused(s, fcand[c], 2, &tf);
      if (rc) return rc;
      if (tf < best_f) { best_f = tf; zf = fcand[c]; }
    }
    fused = best_f < best_h + best_e || fused_mode() == 1;
  }
  s->zc_f = zf;
  s->fused = s->fused && fused;
  if (!s->fused) release_second_buffer(s);
  fill_dev_struct(s);
  tune_entry t;
  memset(&t, 0, sizeof(t));
  snprintf(t.key, sizeof(t.key), "%s", key);
  t.I = s->I;
  t.J = s->J;
  t.K = s->K;
  t.p = s->p;
  t.coef_mode = s->coef_mode;
  t.hcoef_mode = s->hcoef_mode;
  t.zh = zh;
  t.ze = ze;
  t.zf = zf;
  t.fused = fused;
  t.th = tlh;
  t.te = tle;
  pthread_mutex_lock(&g_tune_lock);
  tune_store(&t);
  pthread_mutex_unlock(&g_tune_lock);
  return FDTD_OK;
}

/* The fused step: FDTD_FUSED=0 never, =1 always (no autotuning of the
 * choice), otherwise where the autotuner measures it faster (grids it
 * tunes).  Read at every ReadySimulation. */
static int fused_mode(void) {
  const char *e = getenv("FDTD_FUSED");
  if (e && strcmp(e, "0") == 0) return 0;
  if (e && strcmp(e, "1") == 0) return 1;
  return -1;
}

/* src/simulation.h:640-979 */
int fdtd_ready_simulation(fdtd_handle h) {
  GET(h);
  if (!s->init_const) return fail(FDTD_ERR_STATE, "ReadySimulation requires SetConst");
  if (s->init_ready) return fail(FDTD_ERR_STATE, "ReadySimulation already called");
  float kaE[FDTD_MAX_PML], kaH[FDTD_MAX_PML];
  build_tables(s, kaE, kaH);
  const int p = s->p;
  /* x-only stretch denominators, :861-912 (zero at i = Imax-1) */
  s->h_den_ex = (float *)calloc((size_t)s->I, sizeof(float));
  s->h_den_hx = (float *)calloc((size_t)s->I, sizeof(float));
  if (!s->h_den_ex || !s->h_den_hx) return fail(FDTD_ERR_OOM, "out of host memory");
  {
    int ii = p - 2;
    for (int i = 0; i + 1 < s->I; ++i) {
      if (i < p - 1) {
        s->h_den_hx[i] = (float)(1.0 / (double)(float)(s->delX * kaH[i]));
      } else if (i >= s->I - p) {
        s->h_den_hx[i] = (float)(1.0 / (double)(float)(s->delX * kaH[ii]));
        ii = ii - 1;
      } else {
        s->h_den_hx[i] = (float)(1.0 / (double)s->delX);
      }
    }
    ii = p - 1;
    for (int i = 0; i + 1 < s->I; ++i) {
      if (i < p) {
        s->h_den_ex[i] = (float)(1.0 / (double)(float)(s->delX * kaE[i]));
      } else if (i >= s->I - p) {
        s->h_den_ex[i] = (float)(1.0 / (double)(float)(s->delX * kaE[ii]));
        ii = ii - 1;
      } else {
        s->h_den_ex[i] = (float)(1.0 / (double)s->delX);
      }
    }
  }
  { /* :914-922, sigma_m = 0 */
    const float sigma_m = 0.0f;
    float t = sigma_m * s->delT;
    t = t / 2;
    const double q = (double)t / K_MU0;
    s->Chh = (float)((1 - q) / (1 + q));
    s->Che = (float)((double)s->delT / K_MU0 / (1 + q) / (double)s->delX);
  }
  const size_t bytes = (size_t)s->cells * sizeof(float);
  int rc;
  for (int a = 0; a < 6; ++a)
    if ((rc = dalloc(s, (void **)&s->d_f[a], bytes))) return rc;
  if ((rc = dalloc(s, (void **)&s->d_mat, (size_t)s->cells * sizeof(uint16_t)))) return rc;
  CU(cudaMemsetAsync(s->d_mat, 0, (size_t)s->cells * sizeof(uint16_t), s->stream));
  if (s->allow_compress) {
    if ((rc = dalloc(s, (void **)&s->d_tab, (size_t)MAX_MATERIALS * 6 * sizeof(float)))) return rc;
    if ((rc = dalloc(s, (void **)&s->d_hkeys, (size_t)HASH_CAP * sizeof(unsigned long long))))
      return rc;
    if ((rc = dalloc(s, (void **)&s->d_hrep, (size_t)HASH_CAP * sizeof(int64_t)))) return rc;
    if ((rc = dalloc(s, (void **)&s->d_hid, (size_t)HASH_CAP * sizeof(int32_t)))) return rc;
    if ((rc = dalloc(s, (void **)&s->d_hcnt, 4 * sizeof(int32_t)))) return rc;
  }
  if ((rc = dalloc(s, (void **)&s->d_err, sizeof(int32_t)))) return rc;
  CU(cudaMemsetAsync(s->d_err, 0, sizeof(int32_t), s->stream));
  /* floats per pair array: 2 slabs of size_* cells, 2 values per cell */
  const int64_t psi_n[FDTD_NUM_PSI] = {
      [PSI_EY] = 4 * s->size_y, [PSI_HY] = 4 * s->size_y, [PSI_EZ] = 4 * s->size_z,
      [PSI_HZ] = 4 * s->size_z, [PSI_EX] = 4 * s->size_x, [PSI_HX] = 4 * s->size_x};
  int64_t psi_total = 0;
  for (int a = 0; a < FDTD_NUM_PSI; ++a) psi_total += psi_n[a];
  if ((rc = dalloc(s, (void **)&s->d_psi_pool, (size_t)psi_total * sizeof(float)))) return rc;
  {
    int64_t off = 0;
    for (int a = 0; a < FDTD_NUM_PSI; ++a) {
      s->d_psi[a] = s->d_psi_pool + off;
      off += psi_n[a];
    }
  }
  const int fmode = fused_mode();
  if (s->use_tma && (fmode == 1 || (fmode < 0 && tune_enabled() &&
                                    s->cells >= TUNE_MIN_CELLS))) { /* the fused step's second buffer */
    for (int a = 0; a < 6; ++a)
      if ((rc = dalloc(s, (void **)&s->d_fb[a], bytes))) return rc;
    const int64_t hpsi = psi_n[PSI_HY] + psi_n[PSI_HX] + psi_n[PSI_HZ];
    if ((rc = dalloc(s, (void **)&s->d_psib_pool, (size_t)hpsi * sizeof(float)))) return rc;
    s->fused = 1;
  }
  if ((rc = dalloc(s, (void **)&s->d_den_ex, (size_t)s->I * sizeof(float)))) return rc;
  if ((rc = dalloc(s, (void **)&s->d_den_hx, (size_t)s->I * sizeof(float)))) return rc;
  if ((rc = dalloc(s, (void **)&s->d_ctr, 4 * sizeof(int32_t)))) return rc;
  CU(cudaMemcpyAsync(s->d_den_ex, s->h_den_ex, (size_t)s->I * sizeof(float),
                     cudaMemcpyHostToDevice, s->stream));
  CU(cudaMemcpyAsync(s->d_den_hx, s->h_den_hx, (size_t)s->I * sizeof(float),
                     cudaMemcpyHostToDevice, s->stream));
  if (s->init_ant && s->num_ant > 0) { /* :954-963 */
    const size_t pb = (size_t)s->T * s->num_ant * 6 * sizeof(float);
    if ((rc = dalloc(s, (void **)&s->d_probes, pb))) return rc;
    if ((rc = dalloc(s, (void **)&s->d_probe_idx, (size_t)s->num_ant * sizeof(int64_t)))) return rc;
    CU(cudaMemsetAsync(s->d_probes, 0, pb, s->stream));
    CU(cudaMemcpyAsync(s->d_probe_idx, s->h_probe_idx, (size_t)s->num_ant * sizeof(int64_t),
                       cudaMemcpyHostToDevice, s->stream));
  }
  fill_dev_struct(s);
  if ((rc = upload_coefficients(s))) return rc;
  if ((rc = zero_state(s))) return rc;
  if (s->use_tma) {
    for (int t = 0; t < FDTD_NUM_TILES; ++t)
      if (fdtdk_make_maps(&s->dev, t, &s->maps[t])) s->maps[t].valid = 0;
    if (!s->maps[0].valid) /* the direct kernels take over */
      for (int t = 1; t < FDTD_NUM_TILES; ++t) s->maps[t].valid = 0;
  }
  if ((rc = autotune_zero_state(s))) return rc;
  { /* FDTD_TILE=0|1|2: one tile geometry for both half-steps (comparisons) */
    const char *et = getenv("FDTD_TILE");
    if (et && et[0] >= '0' && et[0] < '0' + FDTD_NUM_TILES && !et[1]) {
      s->tile_h = s->tile_e = et[0] - '0';
      fill_dev_struct(s);
    }
  }
  CU(cudaStreamSynchronize(s->stream));
  s->init_ready = 1;
  return FDTD_OK;
}

/* src/simulation.h:1097-1127 */
int fdtd_update_cuda(fdtd_handle h) {
  GET(h);
  if (!s->init_ready) return fail(FDTD_ERR_STATE, "UpdateCuda requires ReadySimulation");
  int rc = flush(s);
  if (rc) return rc;
  if ((rc = upload_coefficients(s))) return rc;
  CU(cudaStreamSynchronize(s->stream));
  return FDTD_OK;
}

/* src/simulation.h:1128-1151 */
/* ------------------------------------------------------------ checkpoint
 * Image: header, the six pitched field arrays, the psi pool, the four
 * device counters, the probe record.  Loading checks the header against
 * the handle (same grid, CPML, steps, probes and coefficient mode). */
typedef struct {
  char magic[8];
  int32_t version, I, J, K, Ip, p, T, num_ant, coef_mode, pad;
  int64_t psi_floats, probe_floats;
} ckpt_header;

static void ckpt_describe(const sim *s, ckpt_header *hd) {
  memset(hd, 0, sizeof(*hd));
  memcpy(hd->magic, "FDTDCKP1", 8);
  hd->version = 1;
  hd->I = s->I;
  hd->J = s->J;
  hd->K = s->K;
  hd->Ip = s->Ip;
  hd->p = s->p;
  hd->T = s->T;
  hd->num_ant = s->d_probes ? s->num_ant : 0;
  hd->coef_mode = s->coef_mode;
  hd->psi_floats = 8 * (s->size_x + s->size_y + s->size_z);
  hd->probe_floats = s->d_probes ? (int64_t)s->T * s->num_ant * 6 : 0;
}

static size_t ckpt_bytes(const ckpt_header *hd, const sim *s) {
  return sizeof(*hd) + 6 * (size_t)s->cells * sizeof(float) +
         (size_t)hd->psi_floats * sizeof(float) + 4 * sizeof(int32_t) +
         (size_t)hd->probe_floats * sizeof(float);
}

int fdtd_checkpoint_size(fdtd_handle h, size_t *bytes) {
  GET(h);
  if (!bytes) return fail(FDTD_ERR_INVALID_ARG, "null output");
  if (!s->init_ready) return fail(FDTD_ERR_STATE, "checkpoints exist after ReadySimulation");
  ckpt_header hd;
  ckpt_describe(s, &hd);
  *bytes = ckpt_bytes(&hd, s);
  return FDTD_OK;
}

int fdtd_checkpoint_save(fdtd_handle h, void *buf, size_t n) {
  GET(h);
  if (!s->init_ready) return fail(FDTD_ERR_STATE, "checkpoints exist after ReadySimulation");
  ckpt_header hd;
  ckpt_describe(s, &hd);
  if (!buf || n < ckpt_bytes(&hd, s))
    return fail(FDTD_ERR_INVALID_ARG, "checkpoint needs %zu bytes", ckpt_bytes(&hd, s));
  int rc = flush(s);
  if (rc) return rc;
  unsigned char *o = (unsigned char *)buf;
  memcpy(o, &hd, sizeof(hd));
  o += sizeof(hd);
  const size_t fb = (size_t)s->cells * sizeof(float);
  for (int a = 0; a < 6; ++a, o += fb)
    CU(cudaMemcpyAsync(o, s->d_f[a], fb, cudaMemcpyDeviceToHost, s->stream));
  CU(cudaMemcpyAsync(o, s->d_psi_pool, (size_t)hd.psi_floats * sizeof(float),
                     cudaMemcpyDeviceToHost, s->stream));
  o += (size_t)hd.psi_floats * sizeof(float);
  CU(cudaMemcpyAsync(o, s->d_ctr, 4 * sizeof(int32_t), cudaMemcpyDeviceToHost, s->stream));
  o += 4 * sizeof(int32_t);
  if (hd.probe_floats)
    CU(cudaMemcpyAsync(o, s->d_probes, (size_t)hd.probe_floats * sizeof(float),
                       cudaMemcpyDeviceToHost, s->stream));
  CU(cudaStreamSynchronize(s->stream));
  return check_device_error(s);
}

int fdtd_checkpoint_load(fdtd_handle h, const void *buf, size_t n) {
  GET(h);
  if (!s->init_ready) return fail(FDTD_ERR_STATE, "checkpoints load after ReadySimulation");
  ckpt_header want, got;
  ckpt_describe(s, &want);
  if (!buf || n < sizeof(got)) return fail(FDTD_ERR_INVALID_ARG, "not a checkpoint");
  memcpy(&got, buf, sizeof(got));
  if (memcmp(&got, &want, sizeof(got)) != 0)
    return fail(FDTD_ERR_INVALID_ARG, "checkpoint of a different set-up (grid %dx%dx%d, "
                "pml %d, %d steps, %d probes, coefficient mode %d)", got.I, got.J, got.K,
                got.p, got.T, got.num_ant, got.coef_mode);
  if (n < ckpt_bytes(&want, s))
    return fail(FDTD_ERR_INVALID_ARG, "checkpoint truncated (%zu of %zu bytes)", n,
                ckpt_bytes(&want, s));
  int rc = flush(s);
  if (rc) return rc;
  const unsigned char *o = (const unsigned char *)buf + sizeof(got);
  const size_t fb = (size_t)s->cells * sizeof(float);
  for (int a = 0; a < 6; ++a, o += fb)
    CU(cudaMemcpyAsync(s->d_f[a], o, fb, cudaMemcpyHostToDevice, s->stream));
  CU(cudaMemcpyAsync(s->d_psi_pool, o, (size_t)want.psi_floats * sizeof(float),
                     cudaMemcpyHostToDevice, s->stream));
  o += (size_t)want.psi_floats * sizeof(float);
  CU(cudaMemcpyAsync(s->d_ctr, o, 4 * sizeof(int32_t), cudaMemcpyHostToDevice, s->stream));
  o += 4 * sizeof(int32_t);
  if (want.probe_floats)
    CU(cudaMemcpyAsync(s->d_probes, o, (size_t)want.probe_floats * sizeof(float),
                       cudaMemcpyHostToDevice, s->stream));
  CU(cudaStreamSynchronize(s->stream)); /* the host buffer may go away */
  return FDTD_OK;
}

int fdtd_reset_field_all(fdtd_handle h) {
  GET(h);
  if (!s->init_ready) return fail(FDTD_ERR_STATE, "ResetFieldAll requires ReadySimulation");
  int rc = flush(s);
  if (rc) return rc;
  return zero_state(s);
}

/* src/simulation.h:28-68.  The reference sets init_mu only when called
 * before ReadySimulation (where it reads unset state); after it, the
 * coefficients are computed and stored but the H update keeps the scalar
 * coefficient.  That reachable behaviour is what is reproduced here. */
int fdtd_create_mu(fdtd_handle h, const float *mu_x, const float *mu_y, const float *mu_z,
                   size_t n) {
  GET(h);
  if (!s->init_ready)
    return fail(FDTD_ERR_STATE, "CreateMu requires ReadySimulation (the reference reads "
                                "unset coefficients before it)");
  if (!mu_x || !mu_y || !mu_z || n < (size_t)s->IJK)
    return fail(FDTD_ERR_INVALID_ARG, "mu_x, mu_y, mu_z need Imax*Jmax*Kmax values");
  int rc = flush(s);
  if (rc) return rc;
  const float *mu[3] = {mu_x, mu_y, mu_z};
  const size_t bytes = (size_t)s->IJK * sizeof(float);
  float *tmp = NULL;
  if ((rc = dalloc(s, (void **)&tmp, bytes))) return rc;
  for (int a = 0; a < 3; ++a) {
    if (!s->d_mu[a] && (rc = dalloc(s, (void **)&s->d_mu[a], bytes))) {
      dfree(tmp);
      return rc;
    }
    CU(cudaMemcpyAsync(tmp, mu[a], bytes, cudaMemcpyHostToDevice, s->stream));
    KL(fdtdk_compute_mu(s->d_mu[a], tmp, s->d_den_hx, s->IJK, s->I, s->delT, 0.0f, s->stream));
  }
  CU(cudaStreamSynchronize(s->stream));
  dfree(tmp);
  s->device_bytes -= bytes;
  return FDTD_OK;
}

int fdtd_internal_record(fdtd_handle h, cudaEvent_t ev) {
  GET(h);
  int rc = flush(s);
  if (rc) return rc;
  CU(cudaEventRecord(ev, s->stream));
  return FDTD_OK;
}

/* Per-cell magnetic media: createMu's coefficient (src/simulation.h:28-68)
 * applied everywhere the H update uses Che (curl, CPML corrections, TF/SF
 * corrections), with a per-cell magnetic conductivity as well.  In double,
 * rounded once: q = sigma_m delT / 2 / mu0 / mu_r, Chh = (1 - q) / (1 + q),
 * Che = delT / mu0 / mu_r / (1 + q) / delX -- with mu_r = 1, sigma_m = 0
 * exactly the scalar pair of src/simulation.h:914-922. */
int fdtd_set_magnetic(fdtd_handle h, const float *mu_x, const float *mu_y, const float *mu_z,
                      const float *sm_x, const float *sm_y, const float *sm_z, size_t n) {
  GET(h);
  if (!s->init_ready) return fail(FDTD_ERR_STATE, "SetMagnetic requires ReadySimulation");
  if (!mu_x || !mu_y || !mu_z || n < (size_t)s->IJK)
    return fail(FDTD_ERR_INVALID_ARG, "mu_x, mu_y, mu_z need Imax*Jmax*Kmax values");
  if ((sm_x || sm_y || sm_z) && !(sm_x && sm_y && sm_z))
    return fail(FDTD_ERR_INVALID_ARG, "sigma_m: all three components or none");
  const float *mu[3] = {mu_x, mu_y, mu_z}, *sm[3] = {sm_x, sm_y, sm_z};
  const size_t IJK = (size_t)s->IJK;
  for (int a = 0; a < 3; ++a)
    for (size_t i = 0; i < IJK; ++i) {
      if (!(isfinite(mu[a][i]) && mu[a][i] > 0.0f))
        return fail(FDTD_ERR_INVALID_ARG, "mu_r must be finite and positive (cell %zu)", i);
      if (sm[a] && !(isfinite(sm[a][i]) && sm[a][i] >= 0.0f))
        return fail(FDTD_ERR_INVALID_ARG, "sigma_m must be finite and >= 0 (cell %zu)", i);
    }
  int rc = flush(s);
  if (rc) return rc;
  float *hh = (float *)malloc(2 * IJK * sizeof(float));
  if (!hh) return fail(FDTD_ERR_OOM, "out of host memory");
  float *he = hh + IJK;
  const size_t bytes = 6 * (size_t)s->cells * sizeof(float);
  if (!s->d_hc) {
    if ((rc = dalloc(s, (void **)&s->d_hc, bytes))) {
      free(hh);
      return rc;
    }
    CU(cudaMemsetAsync(s->d_hc, 0, bytes, s->stream));
  }
  const double dt = (double)s->delT, dx = (double)s->delX;
  for (int a = 0; a < 3; ++a) {
    for (size_t i = 0; i < IJK; ++i) {
      const double m = (double)mu[a][i];
      const double q = (sm[a] ? (double)sm[a][i] : 0.0) * dt / 2 / K_MU0 / m;
      hh[i] = (float)((1 - q) / (1 + q));
      he[i] = (float)(dt / K_MU0 / m / (1 + q) / dx);
    }
    const size_t row = (size_t)s->I * sizeof(float), pitch = (size_t)s->Ip * sizeof(float);
    cudaError_t e = cudaMemcpy2DAsync(s->d_hc + (size_t)a * s->cells, pitch, hh, row, row,
                                      (size_t)s->J * s->K, cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess)
      e = cudaMemcpy2DAsync(s->d_hc + (size_t)(3 + a) * s->cells, pitch, he, row, row,
                            (size_t)s->J * s->K, cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream); /* hh, he are reused */
    if (e != cudaSuccess) {
      free(hh);
      return fail(FDTD_ERR_CUDA, "SetMagnetic upload: %s", cudaGetErrorString(e));
    }
  }
  free(hh);
  /* 2-byte ids and a table, as for the E coefficients, when the tuples are
   * few; the per-cell arrays otherwise */
  s->hcoef_mode = 1;
  if (s->allow_compress && s->d_hkeys) {
    if (!s->d_hmat && (rc = dalloc(s, (void **)&s->d_hmat, (size_t)s->cells * sizeof(uint16_t))))
      return rc;
    if (!s->d_htab && (rc = dalloc(s, (void **)&s->d_htab, (size_t)MAX_MATERIALS * 6 * sizeof(float))))
      return rc;
    CU(cudaMemsetAsync(s->d_hmat, 0, (size_t)s->cells * sizeof(uint16_t), s->stream));
    const float *cc[6];
    for (int a = 0; a < 6; ++a) cc[a] = s->d_hc + (size_t)a * s->cells;
    KL(fdtdk_compress_ce(&s->dev, cc, s->d_hmat, s->d_htab, MAX_MATERIALS, s->d_hkeys, s->d_hrep,
                         s->d_hid, HASH_CAP, s->d_hcnt, s->stream));
    int32_t cnt[4];
    CU(cudaMemcpyAsync(cnt, s->d_hcnt, sizeof(cnt), cudaMemcpyDeviceToHost, s->stream));
    CU(cudaStreamSynchronize(s->stream));
    if (!cnt[1] && !cnt[2] && cnt[0] > 0 && cnt[0] <= MAX_MATERIALS) {
      s->hcoef_mode = 2;
      dfree(s->d_hc);
      s->d_hc = NULL;
      s->device_bytes -= bytes;
    }
  }
  fill_dev_struct(s);
  return FDTD_OK;
}

/* src/simulation.h:134-254 */
/* ------------------------------------------------------ oblique incidence */

int fdtd_set_incidence(fdtd_handle h, double theta, double phi, double psi) {
  GET(h);
  if (!s->init_const) return fail(FDTD_ERR_STATE, "SetIncidence requires SetConst");
  if (s->init_1d) return fail(FDTD_ERR_STATE, "SetIncidence must precede Init1D");
  if (!isfinite(theta) || !isfinite(phi) || !isfinite(psi))
    return fail(FDTD_ERR_INVALID_ARG, "incidence angles must be finite");
  s->has_ob = 1;
  s->ob_theta = theta;
  s->ob_phi = phi;
  s->ob_psi = psi;
  return FDTD_OK;
}

/* Numerical wavenumber of the 3D Yee grid in direction n at angular
 * frequency w (cubic cells of size dx, time step dt):
 * sum_a sin^2(k n_a dx / 2) = (dx / (c dt))^2 sin^2(w dt / 2), by Newton. */
static double yee_wavenumber(const double n[3], double w, double dx, double dt) {
  const double rhs = pow(dx / (k_c0 * dt) * sin(w * dt / 2), 2.0);
  double k = w / k_c0;
  for (int it = 0; it < 60; ++it) {
    double f = -rhs, df = 0.0;
    for (int a = 0; a < 3; ++a) {
      const double x = k * n[a] * dx / 2;
      f += sin(x) * sin(x);
      df += n[a] * dx * sin(x) * cos(x);
    }
    if (df == 0.0) break;
    const double step = f / df;
    k -= step;
    if (fabs(step) < 1e-15 * fabs(k)) break;
  }
  return k;
}

/* The 1D line of an oblique plane wave: direction k = (sin t cos p,
 * sin t sin p, cos t), E along cos(psi) theta_hat + sin(psi) phi_hat, H
 * along k x E.  Its spacing dx1 = dx sqrt(k_x^4 + k_y^4 + k_z^4) matches
 * the 3D grid's numerical dispersion in direction k to fourth order in
 * (k dx) at every frequency; its speed factor then makes the wavenumbers
 * equal at the source's centre frequency fctr.  The stored window spans
 * the TF/SF box's projection on k. */
static int init_1d_oblique(sim *s, float rate, const float *pw_source) {
  const double t = s->ob_theta, p = s->ob_phi, q = s->ob_psi;
  const double k[3] = {sin(t) * cos(p), sin(t) * sin(p), cos(t)};
  const double th[3] = {cos(t) * cos(p), cos(t) * sin(p), -sin(t)}, ph[3] = {-sin(p), cos(p), 0};
  double e[3], hv[3];
  for (int a = 0; a < 3; ++a) e[a] = cos(q) * th[a] + sin(q) * ph[a];
  hv[0] = k[1] * e[2] - k[2] * e[1];
  hv[1] = k[2] * e[0] - k[0] * e[2];
  hv[2] = k[0] * e[1] - k[1] * e[0];
  const int lo[3] = {s->i0, s->j0, s->k0}, hi[3] = {s->i1, s->j1, s->k1};
  double span = 0.0;
  for (int a = 0; a < 3; ++a) {
    s->ob_k[a] = (float)k[a];
    s->ob_e[a] = (float)e[a];
    s->ob_h[a] = (float)hv[a];
    s->ob_r0[a] = k[a] >= 0 ? lo[a] : hi[a];
    span += fabs(k[a]) * (double)(hi[a] - lo[a]);
  }
  /* window coordinates x = ob_x0 + k.(r - r0): positions used lie within
   * 1.5 cells of the box, i.e. |k.(r - r0)| beyond [0, span] by < 2.6 */
  const double dx = s->delX, dt = s->delT;
  double dx1 = dx * sqrt(pow(k[0], 4) + pow(k[1], 4) + pow(k[2], 4));
  if (k_c0 * dt / dx1 > 0.995) dx1 = k_c0 * dt / 0.995; /* keep the line stable */
  double speed = 1.0;
  const double w = 2.0 * K_PI * (double)s->fctr;
  if (w > 0) {
    const double kn = yee_wavenumber(k, w, dx, dt);
    const double sk = sin(kn * dx1 / 2);
    if (sk > 0) speed = sin(w * dt / 2) * dx1 / (k_c0 * dt * sk);
  }
  if (speed * k_c0 * dt / dx1 > 0.999) speed = 0.999 * dx1 / (k_c0 * dt);
  s->ob_speed = (float)speed;
  s->ob_rho = (float)(dx / dx1);
  /* window: positions used lie within 1.5 cells of the box */
  s->ob_x0 = 4.0f * s->ob_rho;
  s->ob_w = (int32_t)ceil((span + 2.6) * dx / dx1 + 4.0 * s->ob_rho) + 4;
  const int T = s->T, W = s->ob_w;
  const int m_src = T + 8, mb = m_src + 2, n1 = mb + W + T + 8;
  int rc;
  const size_t tab = (size_t)T * (size_t)W * sizeof(float);
  for (int a = 0; a < 2; ++a) {
    dfree(s->d_ob[a]);
    s->d_ob[a] = NULL;
    if ((rc = dalloc(s, (void **)&s->d_ob[a], tab))) return rc;
  }
  float *pw = (float *)malloc((size_t)T * sizeof(float));
  if (!pw) return fail(FDTD_ERR_OOM, "out of host memory");
  /* a soft source radiates ~1/(2 x Courant number) of its strength: scaled
   * by the line's Courant number over the 3D grid's, the plane wave has the
   * amplitude the axis-aligned modes give for the same PW_source */
  const float gain = (float)(speed * dx / dx1);
  for (int n = 0; n < T; ++n) {
    const float v = pw_source[n] * rate;
    pw[n] = v * gain;
  }
  float *d_pw = NULL, *scratch = NULL;
  if ((rc = dalloc(s, (void **)&d_pw, (size_t)T * sizeof(float)))) {
    free(pw);
    return rc;
  }
  if (2 * (size_t)n1 * sizeof(float) > 200 * 1024 &&
      (rc = dalloc(s, (void **)&scratch, 2 * (size_t)n1 * sizeof(float)))) {
    free(pw);
    return rc;
  }
  cudaMemcpyAsync(d_pw, pw, (size_t)T * sizeof(float), cudaMemcpyHostToDevice, s->stream);
  const float cE = (float)(speed * dt / K_EPS0 / dx1), cH = (float)(speed * dt / K_MU0 / dx1);
  const int e2 = fdtdk_init_1d_oblique(n1, m_src, mb, W, T, cE, cH, d_pw, s->d_ob[0], s->d_ob[1],
                                       scratch, s->stream);
  const cudaError_t se = cudaStreamSynchronize(s->stream);
  dfree(d_pw);
  s->device_bytes -= (size_t)T * sizeof(float);
  if (scratch) {
    dfree(scratch);
    s->device_bytes -= 2 * (size_t)n1 * sizeof(float);
  }
  free(pw);
  fill_dev_struct(s);
  if (e2) return fail(FDTD_ERR_CUDA, "oblique 1D launch: %s", cudaGetErrorString((cudaError_t)e2));
  if (se != cudaSuccess) return fail(FDTD_ERR_CUDA, "oblique 1D: %s", cudaGetErrorString(se));
  return FDTD_OK;
}

int fdtd_init_1d(fdtd_handle h, float rate, const float *pw_source, size_t n) {
  GET(h);
  if (!s->init_ready) return fail(FDTD_ERR_STATE, "Init1D requires ReadySimulation");
  if (!pw_source || n < (size_t)s->T)
    return fail(FDTD_ERR_INVALID_ARG, "PW_source needs T=%d values", s->T);
  int rc = flush(s);
  if (rc) return rc;
  int32_t S = s->I;
  if (s->J > S) S = s->J;
  if (s->K > S) S = s->K;
  if (S < 2 * s->p + 4)
    return fail(FDTD_ERR_UNSUPPORTED, "1D line of %d cells too short", S);
  s->size1d = S;
  const size_t tab = (size_t)s->T * (size_t)S * sizeof(float);
  for (int a = 0; a < 4; ++a) {
    if (!s->d_inc[a] && (rc = dalloc(s, (void **)&s->d_inc[a], tab))) return rc;
  }
  float *pw = (float *)malloc((size_t)s->T * sizeof(float));
  if (!pw) return fail(FDTD_ERR_OOM, "out of host memory");
  for (int t = 0; t < s->T; ++t) pw[t] = pw_source[t] * rate; /* :194-197 */
  float *d_pw = NULL, *scratch = NULL;
  if ((rc = dalloc(s, (void **)&d_pw, (size_t)s->T * sizeof(float)))) {
    free(pw);
    return rc;
  }
  const size_t smem = 2 * (size_t)S * sizeof(float);
  if (smem > fdtdk_init_1d_smem_limit()) {
    if ((rc = dalloc(s, (void **)&scratch, 4 * (size_t)S * sizeof(float)))) {
      dfree(d_pw);
      free(pw);
      return rc;
    }
  }
  cudaMemcpyAsync(d_pw, pw, (size_t)s->T * sizeof(float), cudaMemcpyHostToDevice, s->stream);
  fill_dev_struct(s);
  const float Ceh = (float)((double)s->delT / K_EPS0 / (double)s->delX); /* :144 */
  int e = fdtdk_init_1d(&s->dev, s->d_inc, d_pw, Ceh, scratch, s->stream);
  cudaError_t se = cudaStreamSynchronize(s->stream);
  dfree(d_pw);
  s->device_bytes -= (size_t)s->T * sizeof(float);
  if (scratch) {
    dfree(scratch);
    s->device_bytes -= 4 * (size_t)S * sizeof(float);
  }
  free(pw);
  if (e) return fail(FDTD_ERR_CUDA, "init_1d launch: %s", cudaGetErrorString((cudaError_t)e));
  if (se != cudaSuccess) return fail(FDTD_ERR_CUDA, "init_1d: %s", cudaGetErrorString(se));
  if (s->has_ob && (rc = init_1d_oblique(s, rate, pw_source))) return rc;
  s->init_1d = 1;
  return FDTD_OK;
}

/* ------------------------------------------------------------ step ops */

static int issue(sim *s, int hfam, const fdtd_op *op) {
  if (hfam) KL(fdtdk_half_h(&s->dev, s->maps, s->use_tma, op, s->stream));
  else KL(fdtdk_half_e(&s->dev, s->maps, s->use_tma, op, s->stream));
  return FDTD_OK;
}

/* Reads the device error word after a synchronisation point. */
static int check_device_error(sim *s) {
  if (!s->d_err) return FDTD_OK;
  int32_t e = 0;
  CU(cudaMemcpyAsync(&e, s->d_err, sizeof(e), cudaMemcpyDeviceToHost, s->stream));
  CU(cudaStreamSynchronize(s->stream));
  if (e) {
    cudaMemsetAsync(s->d_err, 0, sizeof(int32_t), s->stream);
    return fail(FDTD_ERR_CUDA, "a TMA pipeline wait timed out in a half-step kernel "
                               "(device error word %d); the fields are not valid", e);
  }
  return FDTD_OK;
}

int fdtd_inject_device_error(fdtd_handle h, int32_t value) {
  GET(h);
  if (!s->d_err) return fail(FDTD_ERR_STATE, "the handle has no device error word yet");
  int rc = flush(s);
  if (rc) return rc;
  CU(cudaMemcpyAsync(s->d_err, &value, sizeof(value), cudaMemcpyHostToDevice, s->stream));
  CU(cudaStreamSynchronize(s->stream));
  return FDTD_OK;
}

static int run_steps(sim *s, int32_t first, int32_t count, int32_t mode,
                     const fdtd_current *cur);

/* A half-step that is part of a plain step: curl, CPML and the step's
 * TF/SF (if any), no current source. */
static int plain_half(const fdtd_op *o) {
  return o->curl && o->pml && !o->cur_mode && !o->step_from_dev;
}

static int issue_gather(sim *s) {
  s->gather_pending = 0;
  if (s->dev.num_ant > 0) KL(fdtdk_probe_gather(&s->dev, s->stream));
  return FDTD_OK;
}

/* The held run of complete steps goes to the device. */
static int issue_run(sim *s) {
  if (!s->run_n) return FDTD_OK;
  const int32_t first = s->run_first, n = s->run_n;
  s->run_n = 0;
  return run_steps(s, first, n, s->run_mode, NULL);
}

/* The held H half-step (with its probe gather) goes to the device. */
static int issue_held(sim *s) {
  if (!s->held_h) return FDTD_OK;
  s->held_h = 0;
  int rc = issue_gather(s);
  if (rc) return rc;
  return issue(s, 1, &s->held_op);
}

/* The pending half-step leaves the queue: a plain H half-step after its
 * probe gather is held; the plain E half-step of the same step and mode
 * then joins it as one more step of the held run (issued every GRAPH_CHUNK
 * steps); anything else goes to the device after what is held, in order. */
static int retire(sim *s) {
  if (!s->pend.active) return FDTD_OK;
  s->pend.active = 0;
  const fdtd_op *o = &s->pend.op;
  int rc;
  if (s->pend.h == 1 && s->gather_pending && !s->held_h && plain_half(o)) {
    s->held_h = 1;
    s->held_op = *o;
    s->gather_pending = 0;
    return FDTD_OK;
  }
  if (s->pend.h == 0 && s->held_h && plain_half(o) && o->tfsf_mode == s->held_op.tfsf_mode &&
      (!o->tfsf_mode || o->step == s->held_op.step)) {
    const int32_t n = s->held_op.step, m = o->tfsf_mode;
    s->held_h = 0;
    if (s->run_n && (s->run_mode != m || (m && s->run_first + s->run_n != n)) &&
        (rc = issue_run(s)))
      return rc;
    if (!s->run_n) {
      s->run_first = n;
      s->run_mode = m;
    }
    if (++s->run_n >= GRAPH_CHUNK) return issue_run(s);
    return FDTD_OK;
  }
  if ((rc = issue_run(s)) || (rc = issue_held(s))) return rc;
  if (s->pend.h == 1 && s->gather_pending && (rc = issue_gather(s))) return rc;
  return issue(s, s->pend.h, o);
}

/* Everything queued or held goes to the device, in the call order. */
static int flush(sim *s) {
  int rc = retire(s);
  if (!rc) rc = issue_run(s);
  if (!rc) rc = issue_held(s);
  if (!rc && s->gather_pending) rc = issue_gather(s);
  return rc;
}

static int need_ready(sim *s) {
  if (!s->init_ready) return fail(FDTD_ERR_STATE, "operation requires ReadySimulation");
  return FDTD_OK;
}

static int tfsf_check(sim *s, int32_t step, int32_t mode) {
  if (!s->init_1d) return fail(FDTD_ERR_STATE, "PlaneWave update requires Init1D");
  if (step < 0 || step >= s->T)
    return fail(FDTD_ERR_INVALID_ARG, "time step %d outside [0, %d)", step, s->T);
  if (mode == FDTD_MODE_OBLIQUE) {
    if (!s->d_ob[0])
      return fail(FDTD_ERR_STATE, "mode 5 needs SetIncidence before Init1D");
    fdtd_op none;
    memset(&none, 0, sizeof(none));
    if (!fdtd_tfsf_faces_clear(&s->dev, &none))
      return fail(FDTD_ERR_UNSUPPORTED, "mode 5 needs the TF/SF box at least one cell inside "
                                        "the CPML (tfsf_width >= pml + 1)");
  }
  if (mode >= 1 && mode <= 4) {
    if (s->i0 < 1 || s->j0 < 1 || s->k0 < 1 || s->i1 <= s->i0 || s->j1 <= s->j0 ||
        s->k1 <= s->k0)
      return fail(FDTD_ERR_UNSUPPORTED, "TF/SF box does not fit the grid");
  }
  return FDTD_OK;
}

/* Queue stage ranks: curl 1, tfsf 2, pml 3, current 4. */
static int pend_rank(const fdtd_op *op) {
  if (op->cur_mode) return 4;
  if (op->pml) return 3;
  if (op->tfsf_mode) return 2;
  if (op->curl) return 1;
  return 0;
}

/* Adds one stage to the pending half-step, flushing first when the stage
 * would not follow the queued ones in the reference order. */
static int enqueue(sim *s, int hfam, int rank, const fdtd_op *stage) {
  /* stages that carry a step index (TF/SF, current) merge only with a
   * queue that refers to the same step */
  const int step_clash = (rank == 2 || rank == 4) && stage->step != s->pend.op.step &&
                         (s->pend.op.tfsf_mode || s->pend.op.cur_mode);
  if (s->pend.active &&
      (s->pend.h != hfam || pend_rank(&s->pend.op) >= rank || step_clash)) {
    int rc = retire(s);
    if (rc) return rc;
  }
  if (!s->pend.active) {
    memset(&s->pend, 0, sizeof(s->pend));
    s->pend.active = 1;
    s->pend.h = hfam;
  }
  fdtd_op *o = &s->pend.op;
  if (rank == 1) o->curl = 1;
  if (rank == 2) {
    o->tfsf_mode = stage->tfsf_mode;
    o->step = stage->step;
  }
  if (rank == 3) o->pml = 1;
  if (rank == 4) {
    o->cur_mode = stage->cur_mode;
    memcpy(o->cur_box, stage->cur_box, sizeof(o->cur_box));
    o->step = stage->step;
  }
  return FDTD_OK;
}

/* src/simulation.h:371-385; also records the probe row of this step */
int fdtd_update_h_all(fdtd_handle h) {
  GET(h);
  int rc = need_ready(s);
  if (rc) return rc;
  if ((rc = retire(s))) return rc;
  if (s->gather_pending && (rc = issue_gather(s))) return rc;
  s->gather_pending = 1; /* issued with the H half-step this call starts */
  fdtd_op st;
  memset(&st, 0, sizeof(st));
  return enqueue(s, 1, 1, &st);
}

/* src/simulation.h:386-391 */
int fdtd_update_e_all(fdtd_handle h) {
  GET(h);
  int rc = need_ready(s);
  if (rc) return rc;
  fdtd_op st;
  memset(&st, 0, sizeof(st));
  return enqueue(s, 0, 1, &st);
}

/* src/simulation.h:392-403 */
int fdtd_update_h_pml(fdtd_handle h) {
  GET(h);
  int rc = need_ready(s);
  if (rc) return rc;
  fdtd_op st;
  memset(&st, 0, sizeof(st));
  return enqueue(s, 1, 3, &st);
}

/* src/simulation.h:404-418 */
int fdtd_update_e_pml(fdtd_handle h) {
  GET(h);
  int rc = need_ready(s);
  if (rc) return rc;
  fdtd_op st;
  memset(&st, 0, sizeof(st));
  return enqueue(s, 0, 3, &st);
}

/* src/simulation.h:330-349 */
int fdtd_update_h_planewave(fdtd_handle h, int32_t step, int32_t mode) {
  GET(h);
  int rc = need_ready(s);
  if (rc) return rc;
  if ((rc = tfsf_check(s, step, mode))) return rc;
  if (mode < 1 || mode > FDTD_MODE_OBLIQUE) return FDTD_OK;
  fdtd_op st;
  memset(&st, 0, sizeof(st));
  st.tfsf_mode = mode;
  st.step = step;
  return enqueue(s, 1, 2, &st);
}

/* src/simulation.h:350-369 */
int fdtd_update_e_planewave(fdtd_handle h, int32_t step, int32_t mode) {
  GET(h);
  int rc = need_ready(s);
  if (rc) return rc;
  if ((rc = tfsf_check(s, step, mode))) return rc;
  if (mode < 1 || mode > FDTD_MODE_OBLIQUE) return FDTD_OK;
  fdtd_op st;
  memset(&st, 0, sizeof(st));
  st.tfsf_mode = mode;
  st.step = step;
  return enqueue(s, 0, 2, &st);
}

/* src/simulation.h:256-286 */
int fdtd_add_currents(fdtd_handle h, int32_t step, int32_t mode, const int32_t box[6]) {
  GET(h);
  int rc = need_ready(s);
  if (rc) return rc;
  if (!box) return fail(FDTD_ERR_INVALID_ARG, "time and indices required.");
  if (!s->init_src) return fail(FDTD_ERR_STATE, "AddCurrents requires SetSource");
  if (step < 0 || step >= s->T)
    return fail(FDTD_ERR_INVALID_ARG, "time step %d outside [0, %d)", step, s->T);
  if (mode < 1 || mode > 3) return FDTD_OK;
  for (int a = 0; a < 6; ++a)
    if (box[a] < 0) return FDTD_OK; /* reference: no cell is touched */
  if (box[1] < box[0] || box[3] < box[2] || box[5] < box[4]) return FDTD_OK;
  fdtd_op st;
  memset(&st, 0, sizeof(st));
  st.cur_mode = mode;
  memcpy(st.cur_box, box, sizeof(st.cur_box));
  st.step = step;
  return enqueue(s, 0, 4, &st);
}

/* ------------------------------------------------------------ fused loop */

static int step_ops(sim *s, int32_t step, int from_dev, int32_t mode, const fdtd_current *cur) {
  fdtd_op oh, oe;
  memset(&oh, 0, sizeof(oh));
  oh.curl = 1;
  oh.pml = 1;
  oh.tfsf_mode = mode;
  oh.step = step;
  oh.step_from_dev = from_dev;
  oe = oh;
  if (cur && cur->mode >= 1 && cur->mode <= 3) {
    int ok = 1;
    for (int a = 0; a < 6; ++a) ok &= cur->box[a] >= 0;
    ok &= cur->box[1] >= cur->box[0] && cur->box[3] >= cur->box[2] && cur->box[5] >= cur->box[4];
    if (ok) {
      oe.cur_mode = cur->mode;
      memcpy(oe.cur_box, cur->box, sizeof(oe.cur_box));
    }
  }
  if (s->dev.num_ant > 0) KL(fdtdk_probe_gather(&s->dev, s->stream));
  int rc = issue(s, 1, &oh);
  if (rc) return rc;
  return issue(s, 0, &oe);
}

int fdtd_step_n(fdtd_handle h, int32_t first, int32_t count, int32_t mode,
                const fdtd_current *cur) {
  GET(h);
  int rc = need_ready(s);
  if (rc) return rc;
  if (count < 0 || first < 0) return fail(FDTD_ERR_INVALID_ARG, "negative step range");
  if (count == 0) return FDTD_OK;
  if (mode < 1 || mode > FDTD_MODE_OBLIQUE) mode = 0;
  const int use_cur = cur && cur->mode >= 1 && cur->mode <= 3;
  if ((mode || use_cur) && (int64_t)first + count > s->T)
    return fail(FDTD_ERR_INVALID_ARG, "steps [%d, %d) exceed T=%d", first, first + count, s->T);
  if (mode && (rc = tfsf_check(s, first, mode))) return rc;
  if (use_cur && !s->init_src) return fail(FDTD_ERR_STATE, "current source requires SetSource");
  if ((rc = flush(s))) return rc;
  return run_steps(s, first, count, mode, cur);
}

/* Can steps of this mode (and current) run as fused pairs? */
static int fused_usable(sim *s, int32_t mode, const fdtd_current *cur) {
  if (!s->fused || !s->fmaps[0].valid || !s->fmaps[1].valid) return 0;
  if (cur && cur->mode >= 1 && cur->mode <= 3) return 0;
  if (mode == FDTD_MODE_OBLIQUE && !s->d_ob[0]) return 0;
  fdtd_op o;
  memset(&o, 0, sizeof(o));
  o.curl = 1;
  o.pml = 1;
  o.tfsf_mode = mode;
  return fdtd_fused_ok(&s->dev, &o);
}

/* One fused step out of buffer `from` (0: the handle's fields, 1: the
 * second buffer) into the other: the probe row of the state it starts
 * from, then the pass and its face / x-slab passes. */
static int fused_step(sim *s, int from, int32_t step, int from_dev, int32_t mode) {
  fdtd_op o;
  memset(&o, 0, sizeof(o));
  o.curl = 1;
  o.pml = 1;
  o.tfsf_mode = mode;
  o.step = step;
  o.step_from_dev = from_dev;
  const fdtd_dev *dold = from ? &s->dev_b : &s->dev, *dnew = from ? &s->dev : &s->dev_b;
  if (s->dev.num_ant > 0) KL(fdtdk_probe_gather(dold, s->stream));
  KL(fdtdk_step_fused(dnew, dold, &s->fmaps[from], &o, s->zc_f, s->stream));
  return FDTD_OK;
}

/* Steps first..first+count-1 as fused pairs: GRAPH_CHUNK-step graph
 * replays, then single pairs; an odd last step goes the plain way. */
static int run_fused(sim *s, int32_t first, int32_t count, int32_t mode) {
  int rc;
  const int probes = s->dev.num_ant > 0;
  int32_t done = 0;
  if (count >= GRAPH_CHUNK) {
    if (!(s->gexec_f && s->gf_mode == mode && s->gf_probes == probes)) {
      if (s->gexec_f) {
        cudaGraphExecDestroy(s->gexec_f);
        s->gexec_f = NULL;
      }
      cudaGraph_t g;
      const unsigned long long before = fdtdk_launch_count();
      CU(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
      int crc = FDTD_OK;
      for (int c = 0; c < GRAPH_CHUNK && !crc; ++c) crc = fused_step(s, c & 1, c, 1, mode);
      if (!crc) crc = fdtdk_add_i32(s->d_ctr, GRAPH_CHUNK, s->stream) ? FDTD_ERR_CUDA : FDTD_OK;
      cudaError_t ce = cudaStreamEndCapture(s->stream, &g);
      if (crc) return crc;
      if (ce != cudaSuccess) return fail(FDTD_ERR_CUDA, "graph capture: %s", cudaGetErrorString(ce));
      ce = cudaGraphInstantiate(&s->gexec_f, g, 0);
      cudaGraphDestroy(g);
      if (ce != cudaSuccess) {
        s->gexec_f = NULL;
        return fail(FDTD_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(ce));
      }
      s->gf_kernels = fdtdk_launch_count() - before;
      g_captured_kernels += s->gf_kernels;
      s->gf_mode = mode;
      s->gf_probes = probes;
    }
    KL(fdtdk_set_i32(s->d_ctr, first, s->stream));
    while (count - done >= GRAPH_CHUNK) {
      CU(cudaGraphLaunch(s->gexec_f, s->stream));
      g_graph_kernels += s->gf_kernels;
      done += GRAPH_CHUNK;
    }
  }
  for (; count - done >= 2; done += 2) {
    if ((rc = fused_step(s, 0, first + done, 0, mode))) return rc;
    if ((rc = fused_step(s, 1, first + done + 1, 0, mode))) return rc;
  }
  if (done < count) return step_ops(s, first + done, 0, mode, NULL);
  return FDTD_OK;
}

/* Steps first..first+count-1 as GRAPH_CHUNK-step graph replays and single
 * steps (the arguments already checked). */
static int run_steps(sim *s, int32_t first, int32_t count, int32_t mode,
                     const fdtd_current *cur) {
  int rc;
  const int use_cur = cur && cur->mode >= 1 && cur->mode <= 3;
  const int probes = s->dev.num_ant > 0;
  int32_t done = 0;
  if (count >= 2 && fused_usable(s, mode, cur)) return run_fused(s, first, count, mode);
  if (count >= GRAPH_CHUNK) {
    const int cm = use_cur ? cur->mode : 0;
    int same = s->gexec && s->g_mode == mode && s->g_cur_mode == cm && s->g_probes == probes;
    if (same && cm) same = memcmp(s->g_cur_box, cur->box, sizeof(s->g_cur_box)) == 0;
    if (!same) {
      if (s->gexec) {
        cudaGraphExecDestroy(s->gexec);
        s->gexec = NULL;
      }
      cudaGraph_t g;
      const unsigned long long before = fdtdk_launch_count();
      CU(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
      int crc = FDTD_OK;
      for (int c = 0; c < GRAPH_CHUNK && !crc; ++c) crc = step_ops(s, c, 1, mode, cur);
      if (!crc) crc = fdtdk_add_i32(s->d_ctr, GRAPH_CHUNK, s->stream) ? FDTD_ERR_CUDA : FDTD_OK;
      cudaError_t ce = cudaStreamEndCapture(s->stream, &g);
      if (crc) return crc;
      if (ce != cudaSuccess) return fail(FDTD_ERR_CUDA, "graph capture: %s", cudaGetErrorString(ce));
      ce = cudaGraphInstantiate(&s->gexec, g, 0);
      cudaGraphDestroy(g);
      if (ce != cudaSuccess) {
        s->gexec = NULL;
        return fail(FDTD_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(ce));
      }
      s->g_kernels = fdtdk_launch_count() - before;
      g_captured_kernels += s->g_kernels;
      s->g_mode = mode;
      s->g_cur_mode = cm;
      s->g_probes = probes;
      if (cm) memcpy(s->g_cur_box, cur->box, sizeof(s->g_cur_box));
    }
    KL(fdtdk_set_i32(s->d_ctr, first, s->stream));
    while (count - done >= GRAPH_CHUNK) {
      CU(cudaGraphLaunch(s->gexec, s->stream));
      g_graph_kernels += s->g_kernels;
      done += GRAPH_CHUNK;
    }
  }
  for (; done < count; ++done)
    if ((rc = step_ops(s, first + done, 0, mode, cur))) return rc;
  return FDTD_OK;
}

int fdtd_profile_steps(fdtd_handle h, int32_t first, int32_t count, int32_t mode,
                       const fdtd_current *cur, float ms_out[6]) {
  GET(h);
  int rc = need_ready(s);
  if (rc) return rc;
  if (!ms_out || count < 0) return fail(FDTD_ERR_INVALID_ARG, "bad profile arguments");
  if (mode < 1 || mode > FDTD_MODE_OBLIQUE) mode = 0;
  const int use_cur = cur && cur->mode >= 1 && cur->mode <= 3;
  if ((mode || use_cur) && (int64_t)first + count > s->T)
    return fail(FDTD_ERR_INVALID_ARG, "steps [%d, %d) exceed T=%d", first, first + count, s->T);
  if ((rc = flush(s))) return rc;
  cudaEvent_t *ev = s->ev;
  int32_t c0 = 0;
  if (count >= 2 && fused_usable(s, mode, cur)) {
    /* fused pairs: [2] the probe gathers, [5] the fused pass, [1] its
     * x-slab, face and fix-up passes */
    const int32_t nf = count & ~1;
    for (; c0 < nf; ++c0) {
      const int from = c0 & 1;
      const fdtd_dev *dold = from ? &s->dev_b : &s->dev, *dnew = from ? &s->dev : &s->dev_b;
      fdtd_op o;
      memset(&o, 0, sizeof(o));
      o.curl = 1;
      o.pml = 1;
      o.tfsf_mode = mode;
      o.step = first + c0;
      CU(cudaEventRecord(ev[8], s->stream));
      if (s->dev.num_ant > 0) KL(fdtdk_probe_gather(dold, s->stream));
      CU(cudaEventRecord(ev[9], s->stream));
      CU(cudaEventRecord(ev[12], s->stream));
      fdtdk_set_profile_mark(ev[12]);
      const int e = fdtdk_step_fused(dnew, dold, &s->fmaps[from], &o, s->zc_f, s->stream);
      fdtdk_set_profile_mark(NULL);
      KL(e);
      CU(cudaEventRecord(ev[10], s->stream));
      CU(cudaEventSynchronize(ev[10]));
      float d = 0, f = 0, r = 0;
      CU(cudaEventElapsedTime(&d, ev[8], ev[9]));
      CU(cudaEventElapsedTime(&f, ev[9], ev[12]));
      CU(cudaEventElapsedTime(&r, ev[12], ev[10]));
      ms_out[1] += r;
      ms_out[2] += d;
      ms_out[5] += f;
    }
  }
  for (int32_t c = c0; c < count; ++c) {
    fdtd_op oh, oe;
    memset(&oh, 0, sizeof(oh));
    oh.curl = 1;
    oh.pml = 1;
    oh.tfsf_mode = mode;
    oh.step = first + c;
    oe = oh;
    if (use_cur) {
      oe.cur_mode = cur->mode;
      memcpy(oe.cur_box, cur->box, sizeof(oe.cur_box));
    }
    /* ev[12] / ev[13]: recorded right after the H / E curl kernel (the
     * mark stays at the half-step's start when no curl kernel runs) */
    CU(cudaEventRecord(ev[8], s->stream));
    if (s->dev.num_ant > 0) KL(fdtdk_probe_gather(&s->dev, s->stream));
    CU(cudaEventRecord(ev[9], s->stream));
    CU(cudaEventRecord(ev[12], s->stream));
    fdtdk_set_profile_mark(ev[12]);
    rc = issue(s, 1, &oh);
    fdtdk_set_profile_mark(NULL);
    if (rc) return rc;
    CU(cudaEventRecord(ev[10], s->stream));
    CU(cudaEventRecord(ev[13], s->stream));
    fdtdk_set_profile_mark(ev[13]);
    rc = issue(s, 0, &oe);
    fdtdk_set_profile_mark(NULL);
    if (rc) return rc;
    CU(cudaEventRecord(ev[11], s->stream));
    CU(cudaEventSynchronize(ev[11]));
    float a = 0, b = 0, d = 0, hc = 0, ec = 0;
    CU(cudaEventElapsedTime(&d, ev[8], ev[9]));
    CU(cudaEventElapsedTime(&a, ev[9], ev[10]));
    CU(cudaEventElapsedTime(&b, ev[10], ev[11]));
    CU(cudaEventElapsedTime(&hc, ev[9], ev[12]));
    CU(cudaEventElapsedTime(&ec, ev[10], ev[13]));
    ms_out[0] += a;
    ms_out[1] += b;
    ms_out[2] += d;
    ms_out[3] += hc;
    ms_out[4] += ec;
  }
  return FDTD_OK;
}

int fdtd_set_device(int32_t device) {
  CU(cudaSetDevice(device));
  return FDTD_OK;
}

int fdtd_estimate_device_bytes(int32_t I, int32_t J, int32_t K, int32_t pml, int32_t T,
                               int32_t num_ant, uint64_t *bytes) {
  if (!bytes) return fail(FDTD_ERR_INVALID_ARG, "null output");
  if (I < 2 * pml + 2 || J < 2 * pml + 2 || K < 2 * pml + 2 || T < 1 || num_ant < 0 ||
      pml < 2 || pml > FDTD_MAX_PML)
    return fail(FDTD_ERR_INVALID_ARG, "grid %dx%dx%d, pml %d, %d steps is not valid", I, J, K,
                pml, T);
  const uint64_t Ip = (uint64_t)(I + 7) / 8 * 8, cells = Ip * (uint64_t)J * (uint64_t)K;
  const uint64_t S = (uint64_t)(I > J ? (I > K ? I : K) : (J > K ? J : K));
  const uint64_t sx = (uint64_t)pml * J * K, sy = (uint64_t)I * pml * K,
                 sz = (uint64_t)I * J * pml;
  uint64_t b = 6 * cells * 4;                      /* fields */
  b += 6 * cells * 4;                              /* coefficients (until indexed) */
  b += cells * 2 + (uint64_t)MAX_MATERIALS * 6 * 4; /* material ids + table */
  b += (uint64_t)HASH_CAP * (8 + 8 + 4) + 16 + 4;  /* indexing scratch, error word */
  b += 8 * (sx + sy + sz) * 4;                     /* psi pairs */
  if (fused_mode() == 1 || (fused_mode() < 0 && tune_enabled() &&
                              (int64_t)cells >= TUNE_MIN_CELLS))
    b += 6 * cells * 4 + 4 * (sx + sy + sz) * 4;   /* the fused step's second buffer
                                                      (held until the autotuner decides) */
  b += 2 * (uint64_t)I * 4 + 16;                   /* stretch denominators, counters */
  b += (uint64_t)T * num_ant * 6 * 4 + (uint64_t)num_ant * 8; /* probes */
  b += 4 * (uint64_t)T * S * 4 + (uint64_t)T * 4 + 16 * S + (uint64_t)T * 4; /* 1D tables */
  *bytes = b;
  return FDTD_OK;
}

int fdtd_division_plan(float dx, float out[4]) {
  if (!out) return fail(FDTD_ERR_INVALID_ARG, "null output");
  const fdtd_div_plan p = fdtd_make_div_plan(dx);
  out[0] = p.rdx;
  out[1] = p.lo;
  out[2] = p.hi;
  out[3] = p.lo2;
  return FDTD_OK;
}

int fdtd_check_division(float dx, uint64_t *mismatches) {
  if (!mismatches) return fail(FDTD_ERR_INVALID_ARG, "null output");
  const fdtd_div_plan p = fdtd_make_div_plan(dx);
  unsigned long long *d_bad = NULL, bad = 0;
  CU(cudaMalloc((void **)&d_bad, sizeof(*d_bad)));
  int rc = FDTD_OK;
  if (cudaMemset(d_bad, 0, sizeof(*d_bad)) != cudaSuccess ||
      fdtdk_check_division(p, 0, 1ull << 32, d_bad, 0) != 0 ||
      cudaMemcpy(&bad, d_bad, sizeof(bad), cudaMemcpyDeviceToHost) != cudaSuccess)
    rc = fail(FDTD_ERR_CUDA, "division check: %s", cudaGetErrorString(cudaGetLastError()));
  cudaFree(d_bad);
  if (rc == FDTD_OK) *mismatches = (uint64_t)bad;
  return rc;
}

int fdtd_check_bounded_wait(int32_t *timed_out, int32_t *completed, double *poll_ns,
                            double *limit_ms) {
  if (!timed_out || !completed || !poll_ns || !limit_ms)
    return fail(FDTD_ERR_INVALID_ARG, "null output");
  long long a[2] = {0, 0}, b[2] = {0, 0};
  int e = fdtdk_check_wait(0, a);
  if (!e) e = fdtdk_check_wait(1, b);
  if (e) return fail(FDTD_ERR_CUDA, "bounded-wait check: %s", cudaGetErrorString((cudaError_t)e));
  *timed_out = (int32_t)a[0];
  *completed = b[0] == 0;
  *poll_ns = (double)a[1]; /* the check's wait, limit fdtdk_check_ns() */
  *limit_ms = (double)fdtdk_wait_ns() * 1e-6;
  return FDTD_OK;
}

/* ------------------------------------------------------------ outputs */

int fdtd_synchronize(fdtd_handle h) {
  GET(h);
  int rc = flush(s);
  if (rc) return rc;
  CU(cudaStreamSynchronize(s->stream));
  return check_device_error(s);
}

/* src/simulation.h:572-619 */
int fdtd_output_vis(fdtd_handle h, float *out, size_t n, int32_t flag) {
  GET(h);
  if (!out && n) return fail(FDTD_ERR_INVALID_ARG, "null output");
  if (!s->init_const) return fail(FDTD_ERR_STATE, "OutputVis requires SetConst");
  const size_t cnt = n < (size_t)s->IJK ? n : (size_t)s->IJK;
  if (flag <= 0 && flag >= -5) {
    const int idx = -flag; /* 0,-1,-2 sigma_x,y,z; -3,-4,-5 eps_x,y,z */
    if (s->shapes) { /* the media are shapes: the same cells, rasterised here */
      for (size_t n2 = 0; n2 < cnt; ++n2) {
        const int64_t ii = (int64_t)n2 % s->I, rr = (int64_t)n2 / s->I;
        float e, sg;
        shape_material(s, (int)ii, (int)(rr % s->J), (int)(rr / s->J), &e, &sg);
        out[n2] = idx < 3 ? sg : e;
      }
      return FDTD_OK;
    }
    if (s->d_raw[idx]) {
      CU(cudaMemcpyAsync(out, s->d_raw[idx], cnt * sizeof(float), cudaMemcpyDeviceToHost,
                         s->stream));
      CU(cudaStreamSynchronize(s->stream));
    } else {
      const float v = material_default(idx);
      for (size_t n2 = 0; n2 < cnt; ++n2) out[n2] = v;
    }
    return FDTD_OK;
  }
  if (flag >= 1 && flag <= 6) {
    if (!s->init_ready) return fail(FDTD_ERR_STATE, "OutputVis of fields requires ReadySimulation");
    int rc = flush(s);
    if (rc) return rc;
    /* device rows are pitched: whole rows packed on the device (a 2D
     * device copy) and read back in one transfer, then the tail */
    const size_t rows = cnt / (size_t)s->I, tail = cnt % (size_t)s->I;
    const size_t row = (size_t)s->I * sizeof(float);
    const float *src = s->d_f[flag - 1];
    float *scratch = NULL;
    if (rows && s->Ip != s->I &&
        pool_alloc((void **)&scratch, rows * row, s->stream) != cudaSuccess)
      scratch = NULL;
    if (rows && s->Ip == s->I) {
      CU(cudaMemcpyAsync(out, src, rows * row, cudaMemcpyDeviceToHost, s->stream));
    } else if (rows && scratch) {
      cudaError_t e = cudaMemcpy2DAsync(scratch, row, src, (size_t)s->Ip * sizeof(float), row,
                                        rows, cudaMemcpyDeviceToDevice, s->stream);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(out, scratch, rows * row, cudaMemcpyDeviceToHost, s->stream);
      dfree(scratch);
      CU(e);
    } else if (rows) {
      CU(cudaMemcpy2DAsync(out, row, src, (size_t)s->Ip * sizeof(float), row, rows,
                           cudaMemcpyDeviceToHost, s->stream));
    }
    if (tail)
      CU(cudaMemcpyAsync(out + rows * s->I, src + rows * s->Ip, tail * sizeof(float),
                         cudaMemcpyDeviceToHost, s->stream));
    CU(cudaStreamSynchronize(s->stream));
    return check_device_error(s);
  }
  return FDTD_OK;
}

int fdtd_output_probes(fdtd_handle h, float *out, size_t n) {
  GET(h);
  if (!out && n) return fail(FDTD_ERR_INVALID_ARG, "null output");
  if (!s->d_probes) return fail(FDTD_ERR_STATE, "Antenna data is not initialized.");
  int rc = flush(s);
  if (rc) return rc;
  const size_t total = (size_t)s->T * s->num_ant * 6;
  CU(cudaMemcpyAsync(out, s->d_probes, (n < total ? n : total) * sizeof(float),
                     cudaMemcpyDeviceToHost, s->stream));
  CU(cudaStreamSynchronize(s->stream));
  return check_device_error(s);
}

/* src/simulation.h:621-638 */
int fdtd_output_ant(fdtd_handle h, float *out, size_t n) {
  GET(h);
  if (!out && n) return fail(FDTD_ERR_INVALID_ARG, "null output");
  if (!s->d_probes) return fail(FDTD_ERR_STATE, "Antenna data is not initialized.");
  const size_t rows = (size_t)s->T * s->num_ant;
  float *all = (float *)malloc(rows * 6 * sizeof(float));
  if (!all) return fail(FDTD_ERR_OOM, "out of host memory");
  int rc = fdtd_output_probes(h, all, rows * 6);
  if (!rc) {
    const size_t cnt = n < rows ? n : rows;
    for (size_t r = 0; r < cnt; ++r) out[r] = all[r * 6 + 2];
  }
  free(all);
  return rc;
}

int fdtd_get_info(fdtd_handle h, fdtd_info *o) {
  GET(h);
  if (!o) return fail(FDTD_ERR_INVALID_ARG, "null info");
  memset(o, 0, sizeof(*o));
  o->I = s->I;
  o->J = s->J;
  o->K = s->K;
  o->T = s->T;
  o->num_ant = s->num_ant;
  o->pml = s->p;
  o->size_1d = s->size1d;
  o->i0 = s->i0;
  o->i1 = s->i1;
  o->j0 = s->j0;
  o->j1 = s->j1;
  o->k0 = s->k0;
  o->k1 = s->k1;
  o->coef_mode = s->coef_mode;
  o->num_materials = s->num_mat;
  o->device_bytes = s->device_bytes;
  o->Chh = s->Chh;
  o->Che = s->Che;
  o->zchunk_h = s->zc_h;
  o->zchunk_e = s->zc_e;
  o->hcoef_mode = s->hcoef_mode;
  o->fused = s->fused && s->fmaps[0].valid && s->fmaps[1].valid;
  o->zchunk_f = s->zc_f;
  o->tile_h = s->tile_h;
  o->tile_e = s->tile_e;
  return FDTD_OK;
}

int fdtd_get_table(fdtd_handle h, int32_t which, float *out, size_t n) {
  GET(h);
  if (!s->init_ready) return fail(FDTD_ERR_STATE, "tables exist after ReadySimulation");
  if (which == 6) { /* material-indexed coefficient table: num_materials x 6 */
    if (s->coef_mode != 1) return fail(FDTD_ERR_STATE, "coefficients are not material-indexed");
    const size_t cnt = (size_t)s->num_mat * 6;
    if (!out || n < cnt) return fail(FDTD_ERR_INVALID_ARG, "table needs %zu values", cnt);
    int rc = flush(s);
    if (rc) return rc;
    CU(cudaMemcpyAsync(out, s->d_tab, cnt * sizeof(float), cudaMemcpyDeviceToHost, s->stream));
    CU(cudaStreamSynchronize(s->stream));
    return FDTD_OK;
  }
  const float *src = NULL;
  size_t cnt = 0;
  switch (which) {
    case 0: src = s->bE; cnt = 2 * (size_t)s->p; break;
    case 1: src = s->cE; cnt = 2 * (size_t)s->p; break;
    case 2: src = s->bH; cnt = 2 * (size_t)s->p; break;
    case 3: src = s->cH; cnt = 2 * (size_t)s->p; break;
    case 4: src = s->h_den_ex; cnt = (size_t)s->I; break;
    case 5: src = s->h_den_hx; cnt = (size_t)s->I; break;
    default: return fail(FDTD_ERR_INVALID_ARG, "unknown table %d", which);
  }
  if (!out || n < cnt) return fail(FDTD_ERR_INVALID_ARG, "table needs %zu values", cnt);
  memcpy(out, src, cnt * sizeof(float));
  return FDTD_OK;
}

int fdtd_event_record(fdtd_handle h, int32_t slot) {
  GET(h);
  if (slot < 0 || slot >= MAX_EVENTS) return fail(FDTD_ERR_INVALID_ARG, "event slot");
  int rc = flush(s);
  if (rc) return rc;
  CU(cudaEventRecord(s->ev[slot], s->stream));
  return FDTD_OK;
}

int fdtd_event_elapsed_ms(fdtd_handle h, int32_t a, int32_t b, float *ms) {
  GET(h);
  if (a < 0 || a >= MAX_EVENTS || b < 0 || b >= MAX_EVENTS || !ms)
    return fail(FDTD_ERR_INVALID_ARG, "event slot");
  CU(cudaEventSynchronize(s->ev[b]));
  CU(cudaEventElapsedTime(ms, s->ev[a], s->ev[b]));
  return FDTD_OK;
}

/* src/cpucode/FunLib.cpp:26-44 */
int fdtd_create_signal(double fctr, double delT, double percentage_bw, double num_side_lobes,
                       size_t time_steps, double *out, double *fmaxx_out) {
  if (!out && time_steps) return fail(FDTD_ERR_INVALID_ARG, "null output");
  const double fmaxx = fctr * percentage_bw / 2.0;
  if (fmaxx_out) *fmaxx_out = fmaxx;
  const double spread = 1.0 / (2.0 * delT * fmaxx);
  const double tto = num_side_lobes * spread;
  for (size_t n = 0; n < time_steps; ++n) {
    const double nn = (double)n + 1.0;
    double v = 0.0;
    if (nn < 2.0 * tto) {
      const double arg = 2.0 * K_PI * fmaxx * (nn - tto) * delT;
      const double den = (fabs(arg) < 1e-14) ? 1e-14 : arg;
      v = sin(arg) / den * sin(2.0 * K_PI * fctr * (nn - tto) * delT);
    }
    v *= cos(((nn - 1.0) / (double)time_steps) * (K_PI / 2.0));
    out[n] = v;
  }
  return FDTD_OK;
}

/* ==================================================================== batch
 *
 * A batch advances many simulation handles of different sizes together:
 * every batched step is one H and one E launch of the persistent TMA kernels
 * over the work items of all active members (plus a probe gather and a step
 * counter update), so small grids fill the GPU together instead of each
 * leaving most of it idle.  The per-cell arithmetic is the single-grid
 * kernels', so every member ends bit-identical to running it alone.
 */

#define MAX_BATCHES 256

/* FDTD_XSPLIT=0 keeps the batched E kernels' CPML X inline (the x-slab
 * pass is the default) */
static int xsplit_enabled(void) {
  static int v = -1;
  if (v < 0) {
    const char *e = getenv("FDTD_XSPLIT");
    v = !(e && strcmp(e, "0") == 0);
  }
  return v;
}

/* z-planes per batched work item: 16, or FDTD_BATCH_ZRUN (1..64) */
static int batch_zrun(void) {
  static int z = 0;
  if (!z) {
    const char *e = getenv("FDTD_BATCH_ZRUN");
    const int v = e ? atoi(e) : 0;
    z = v >= 1 && v <= 64 ? v : 16;
  }
  return z;
}

typedef struct {
  fdtd_handle h;
  int32_t first, count, done, mode, has_cur;
  fdtd_current cur;
} bmember;

typedef struct batch {
  bmember *m;
  int n, cap;
  cudaStream_t stream;
  cudaEvent_t ev;
  /* device mirrors of the active members, rebuilt when the set changes */
  fdtd_dev *d_devs;
  unsigned char *d_maps;
  fdtd_op *d_ops;
  int32_t *d_steps, *d_tab_h, *d_tab_e, *d_work, *d_err;
  int dev_cap, cap_h, cap_e;
  /* host staging */
  fdtd_dev *h_devs;
  unsigned char *h_maps;
  fdtd_op *h_ops;
  int32_t *h_steps, *h_tab_h, *h_tab_e;
  int *act;  /* member index of each active slot */
  int n_act, n_h, n_e, any_probes, dirty;
  int any_split;   /* some active member's TF/SF runs as the face pass */
  int any_oblique; /* ... in mode 5 */
  int32_t face_max; /* largest face-plane area of those members */
  int any_xsplit;   /* a member's E CPML X runs as the x-slab pass */
  int all_lean;     /* every member's E op satisfies fdtd_e_lean */
  int all_lean_h;   /* every member's op satisfies fdtd_h_lean */
  int64_t xs_max;   /* the largest member's 2p*J*K */
  /* GRAPH_CHUNK steps of the active set, captured after each rebuild */
  cudaGraphExec_t gexec;
  unsigned long long g_kernels;
  /* z-planes per work item, measured once (batch_tune) */
  int zrun, tuned;
  cudaEvent_t tev[2];
  /* rebuilds and graph captures so far, and their host seconds */
  uint64_t n_rebuild, n_capture;
  double t_rebuild, t_capture;
} batch;

static batch *g_batches[MAX_BATCHES];
static uint32_t g_bgen[MAX_BATCHES];

static batch *blookup(fdtd_batch b) {
  uint32_t slot = (uint32_t)(b & 0xffffffffu), gen = (uint32_t)(b >> 32);
  if (slot == 0 || slot > MAX_BATCHES) return NULL;
  pthread_mutex_lock(&g_reg_lock);
  batch *p = g_bgen[slot - 1] == gen ? g_batches[slot - 1] : NULL;
  pthread_mutex_unlock(&g_reg_lock);
  return p;
}

int fdtd_batch_create(fdtd_batch *out) {
  if (!out) return fail(FDTD_ERR_INVALID_ARG, "null output");
  batch *b = (batch *)calloc(1, sizeof(batch));
  if (!b) return fail(FDTD_ERR_OOM, "out of host memory");
  cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreate(&b->tev[0]);
  if (e == cudaSuccess) e = cudaEventCreate(&b->tev[1]);
  b->zrun = batch_zrun();
  /* the z-run is measured at the first large enough step unless fixed */
  b->tuned = getenv("FDTD_BATCH_ZRUN") != NULL || !tune_enabled();
  if (e == cudaSuccess) e = pool_alloc((void **)&b->d_work, 4 * sizeof(int32_t), b->stream);
  if (e == cudaSuccess) e = pool_alloc((void **)&b->d_err, sizeof(int32_t), b->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(b->d_work, 0, 4 * sizeof(int32_t), b->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(b->d_err, 0, sizeof(int32_t), b->stream);
  if (e != cudaSuccess) {
    free(b);
    return fail(FDTD_ERR_CUDA, "batch create: %s", cudaGetErrorString(e));
  }
  pthread_mutex_lock(&g_reg_lock);
  int slot = -1;
  for (int i = 0; i < MAX_BATCHES; ++i)
    if (!g_batches[i]) {
      slot = i;
      break;
    }
  if (slot < 0) {
    pthread_mutex_unlock(&g_reg_lock);
    dfree_on(b->stream, b->d_work);
    dfree_on(b->stream, b->d_err);
    cudaStreamSynchronize(b->stream);
    cudaStreamDestroy(b->stream);
    free(b);
    return fail(FDTD_ERR_OOM, "too many batches");
  }
  g_batches[slot] = b;
  g_bgen[slot] += 1;
  *out = ((uint64_t)g_bgen[slot] << 32) | (uint64_t)(slot + 1);
  pthread_mutex_unlock(&g_reg_lock);
  return FDTD_OK;
}

static void batch_free_mirrors(batch *b) {
  dfree_on(b->stream, b->d_devs);
  dfree_on(b->stream, b->d_maps);
  dfree_on(b->stream, b->d_ops);
  dfree_on(b->stream, b->d_steps);
  dfree_on(b->stream, b->d_tab_h);
  dfree_on(b->stream, b->d_tab_e);
  b->d_devs = NULL;
  b->d_maps = NULL;
  b->d_ops = NULL;
  b->d_steps = b->d_tab_h = b->d_tab_e = NULL;
  free(b->h_devs);
  free(b->h_maps);
  free(b->h_ops);
  free(b->h_steps);
  free(b->h_tab_h);
  free(b->h_tab_e);
  free(b->act);
  b->h_devs = NULL;
  b->h_maps = NULL;
  b->h_ops = NULL;
  b->h_steps = b->h_tab_h = b->h_tab_e = NULL;
  b->act = NULL;
  b->dev_cap = b->cap_h = b->cap_e = 0;
}

int fdtd_batch_destroy(fdtd_batch h) {
  uint32_t slot = (uint32_t)(h & 0xffffffffu);
  batch *b = blookup(h);
  if (!b) return fail(FDTD_ERR_INVALID_HANDLE, "invalid batch handle");
  pthread_mutex_lock(&g_reg_lock);
  g_batches[slot - 1] = NULL;
  pthread_mutex_unlock(&g_reg_lock);
  cudaStreamSynchronize(b->stream);
  if (b->gexec) cudaGraphExecDestroy(b->gexec);
  batch_free_mirrors(b);
  dfree_on(b->stream, b->d_work);
  dfree_on(b->stream, b->d_err);
  cudaStreamSynchronize(b->stream);
  cudaEventDestroy(b->ev);
  cudaEventDestroy(b->tev[0]);
  cudaEventDestroy(b->tev[1]);
  cudaStreamDestroy(b->stream);
  free(b->m);
  free(b);
  return FDTD_OK;
}

int fdtd_batch_add(fdtd_batch bh, fdtd_handle h, int32_t first, int32_t count, int32_t mode,
                   const fdtd_current *cur) {
  batch *b = blookup(bh);
  if (!b) return fail(FDTD_ERR_INVALID_HANDLE, "invalid batch handle");
  sim *s = lookup(h);
  if (!s) return fail(FDTD_ERR_INVALID_HANDLE, "invalid simulation handle");
  if (!s->init_ready) return fail(FDTD_ERR_STATE, "batch members need ReadySimulation");
  if (!s->maps[1].valid) return fail(FDTD_ERR_UNSUPPORTED, "batch members need the TMA kernels");
  if (s->hcoef_mode)
    return fail(FDTD_ERR_UNSUPPORTED, "batch members need uniform H coefficients (no SetMagnetic)");
  /* a work item packs its first z-plane into 16 bits (add_items) */
  if (s->K > 65535)
    return fail(FDTD_ERR_UNSUPPORTED, "batch members need K <= 65535 (K = %d)", s->K);
  if (first < 0 || count < 0) return fail(FDTD_ERR_INVALID_ARG, "negative step range");
  if (mode < 1 || mode > FDTD_MODE_OBLIQUE) mode = 0;
  const int use_cur = cur && cur->mode >= 1 && cur->mode <= 3;
  if ((mode || use_cur) && (int64_t)first + count > s->T)
    return fail(FDTD_ERR_INVALID_ARG, "steps [%d, %d) exceed T=%d", first, first + count, s->T);
  if (mode) {
    int rc = tfsf_check(s, first, mode);
    if (rc) return rc;
  }
  if (mode == FDTD_MODE_OBLIQUE && use_cur) { /* mode 5 runs as face passes only */
    fdtd_op o;
    memset(&o, 0, sizeof(o));
    o.cur_mode = cur->mode;
    memcpy(o.cur_box, cur->box, sizeof(o.cur_box));
    if (!fdtd_tfsf_faces_clear(&s->dev, &o))
      return fail(FDTD_ERR_UNSUPPORTED, "mode 5 with a current source on a TF/SF face");
  }
  if (use_cur && !s->init_src) return fail(FDTD_ERR_STATE, "current source requires SetSource");
  for (int i = 0; i < b->n; ++i)
    if (b->m[i].h == h && b->m[i].done < b->m[i].count)
      return fail(FDTD_ERR_STATE, "handle is already an active member of this batch");
  if (b->n == b->cap) {
    int nc = b->cap ? 2 * b->cap : 64;
    bmember *nm = (bmember *)realloc(b->m, (size_t)nc * sizeof(bmember));
    if (!nm) return fail(FDTD_ERR_OOM, "out of host memory");
    b->m = nm;
    b->cap = nc;
  }
  bmember *m = &b->m[b->n++];
  memset(m, 0, sizeof(*m));
  m->h = h;
  m->first = first;
  m->count = count;
  m->mode = mode;
  m->has_cur = 0;
  if (use_cur) {
    int ok = 1;
    for (int a = 0; a < 6; ++a) ok &= cur->box[a] >= 0;
    ok &= cur->box[1] >= cur->box[0] && cur->box[3] >= cur->box[2] && cur->box[5] >= cur->box[4];
    if (ok) {
      m->has_cur = 1;
      m->cur = *cur;
    }
  }
  b->dirty = 1;
  return FDTD_OK;
}

static int ensure_cap(void **d, void **hbuf, int *cap, int need, size_t elem, cudaStream_t st) {
  if (need <= *cap) return FDTD_OK;
  int nc = *cap ? *cap : 256;
  while (nc < need) nc *= 2;
  dfree_on(st, *d);
  free(*hbuf);
  *d = NULL;
  *hbuf = malloc((size_t)nc * elem);
  if (!*hbuf) return fail(FDTD_ERR_OOM, "out of host memory");
  cudaError_t e = pool_alloc(d, (size_t)nc * elem, st);
  if (e != cudaSuccess) return fail(FDTD_ERR_OOM, "device allocation: %s", cudaGetErrorString(e));
  *cap = nc;
  return FDTD_OK;
}

static int add_items(int32_t *tab, int n, int g, int ni, int nj, int nk, int zr) {
  assert(nk <= 65536 && zr < 32768); /* kb and np share one int32 (fdtd_batch_add) */
  for (int kb = 0; kb < nk; kb += zr) {
    const int np = nk - kb < zr ? nk - kb : zr;
    for (int y0 = 0; y0 < nj; y0 += FDTD_BTILE_Y)
      for (int x0 = 0; x0 < ni; x0 += FDTD_BTILE_X) {
        int32_t *e = tab + 4 * (size_t)n;
        e[0] = g;
        e[1] = x0;
        e[2] = y0;
        e[3] = kb | (np << 16);
        ++n;
      }
  }
  return n;
}

static int count_items(int ni, int nj, int nk, int zr) {
  return ((ni + FDTD_BTILE_X - 1) / FDTD_BTILE_X) * ((nj + FDTD_BTILE_Y - 1) / FDTD_BTILE_Y) *
         ((nk + zr - 1) / zr);
}

static double mono_s(void) {
  struct timespec t;
  clock_gettime(CLOCK_MONOTONIC, &t);
  return (double)t.tv_sec + 1e-9 * (double)t.tv_nsec;
}

static int batch_rebuild_(batch *b);
/* Builds and uploads the device mirrors of the active members. */
static int batch_rebuild(batch *b) {
  const double t0 = mono_s();
  const int rc = batch_rebuild_(b);
  b->t_rebuild += mono_s() - t0;
  b->n_rebuild += 1;
  return rc;
}
static int batch_rebuild_(batch *b) {
  int na = 0, nh = 0, ne = 0;
  for (int i = 0; i < b->n; ++i) {
    const bmember *m = &b->m[i];
    if (m->done >= m->count) continue;
    sim *s = lookup(m->h);
    if (!s) return fail(FDTD_ERR_INVALID_HANDLE, "a batch member was deleted");
    ++na;
    nh += count_items(s->I - 1, s->J - 1, s->K - 1, b->zrun);
    ne += count_items(s->I, s->J, s->K, b->zrun);
  }
  int rc;
  if (na > b->dev_cap) { /* per-member mirrors share one capacity */
    int cap = b->dev_cap ? b->dev_cap : 64;
    while (cap < na) cap *= 2;
    int c0 = 0, c1 = 0, c2 = 0, c3 = 0;
    dfree_on(b->stream, b->d_devs);
    dfree_on(b->stream, b->d_maps);
    dfree_on(b->stream, b->d_ops);
    dfree_on(b->stream, b->d_steps);
    b->d_devs = NULL;
    b->d_maps = NULL;
    b->d_ops = NULL;
    b->d_steps = NULL;
    free(b->act);
    b->act = (int *)malloc((size_t)cap * sizeof(int));
    if (!b->act) return fail(FDTD_ERR_OOM, "out of host memory");
    if ((rc = ensure_cap((void **)&b->d_devs, (void **)&b->h_devs, &c0, cap, sizeof(fdtd_dev),
                         b->stream)))
      return rc;
    if ((rc = ensure_cap((void **)&b->d_maps, (void **)&b->h_maps, &c1, cap,
                         sizeof(((fdtd_maps *)0)->bytes), b->stream)))
      return rc;
    if ((rc = ensure_cap((void **)&b->d_ops, (void **)&b->h_ops, &c2, cap, sizeof(fdtd_op),
                         b->stream)))
      return rc;
    if ((rc = ensure_cap((void **)&b->d_steps, (void **)&b->h_steps, &c3, cap, sizeof(int32_t),
                         b->stream)))
      return rc;
    b->dev_cap = cap;
  }
  if ((rc = ensure_cap((void **)&b->d_tab_h, (void **)&b->h_tab_h, &b->cap_h, nh,
                       4 * sizeof(int32_t), b->stream)))
    return rc;
  if ((rc = ensure_cap((void **)&b->d_tab_e, (void **)&b->h_tab_e, &b->cap_e, ne,
                       4 * sizeof(int32_t), b->stream)))
    return rc;
  b->any_split = 0;
  b->any_oblique = 0;
  b->face_max = 0;
  b->any_xsplit = 0;
  b->all_lean = 1;
  b->all_lean_h = 1;
  b->xs_max = 0;
  int g = 0;
  nh = ne = 0;
  b->any_probes = 0;
  const size_t mapsz = sizeof(((fdtd_maps *)0)->bytes);
  for (int i = 0; i < b->n; ++i) {
    const bmember *m = &b->m[i];
    if (m->done >= m->count) continue;
    sim *s = lookup(m->h);
    b->act[g] = i;
    b->h_devs[g] = s->dev;
    memcpy(b->h_maps + (size_t)g * mapsz, s->maps[1].bytes, mapsz);
    fdtd_op *op = &b->h_ops[g];
    memset(op, 0, sizeof(*op));
    op->curl = 1;
    op->pml = 1;
    op->tfsf_mode = m->mode;
    if (m->has_cur) {
      op->cur_mode = m->cur.mode;
      memcpy(op->cur_box, m->cur.box, sizeof(op->cur_box));
    }
    op->tfsf_split = fdtd_tfsf_split(&s->dev, op);
    op->xsplit = xsplit_enabled() && fdtd_xsplit(&s->dev, op);
    if (op->xsplit) {
      const int64_t xc = 2 * (int64_t)s->p * s->J * s->K;
      if (xc > b->xs_max) b->xs_max = xc;
      b->any_xsplit = 1;
    }
    if (!fdtd_e_lean(op)) b->all_lean = 0;
    if (!fdtd_h_lean(op)) b->all_lean_h = 0;
    if (op->tfsf_split) {
      const int32_t ax = s->I + 2, ay = s->J + 2, az = s->K + 2;
      int32_t f = ax * ay;
      if (ay * az > f) f = ay * az;
      if (ax * az > f) f = ax * az;
      if (f > b->face_max) b->face_max = f;
      /* the axis-mode face pass and the oblique one serve different members */
      if (op->tfsf_mode == FDTD_MODE_OBLIQUE) b->any_oblique = 1;
      else b->any_split = 1;
    }
    b->h_steps[g] = m->first + m->done;
    if (s->dev.num_ant > 0) b->any_probes = 1;
    nh = add_items(b->h_tab_h, nh, g, s->I - 1, s->J - 1, s->K - 1, b->zrun);
    ne = add_items(b->h_tab_e, ne, g, s->I, s->J, s->K, b->zrun);
    ++g;
  }
  b->n_act = na;
  b->n_h = nh;
  b->n_e = ne;
  if (na) {
    CU(cudaMemcpyAsync(b->d_devs, b->h_devs, (size_t)na * sizeof(fdtd_dev),
                       cudaMemcpyHostToDevice, b->stream));
    CU(cudaMemcpyAsync(b->d_maps, b->h_maps, (size_t)na * mapsz, cudaMemcpyHostToDevice,
                       b->stream));
    CU(cudaMemcpyAsync(b->d_ops, b->h_ops, (size_t)na * sizeof(fdtd_op), cudaMemcpyHostToDevice,
                       b->stream));
    CU(cudaMemcpyAsync(b->d_steps, b->h_steps, (size_t)na * sizeof(int32_t),
                       cudaMemcpyHostToDevice, b->stream));
    CU(cudaMemcpyAsync(b->d_tab_h, b->h_tab_h, (size_t)nh * 4 * sizeof(int32_t),
                       cudaMemcpyHostToDevice, b->stream));
    CU(cudaMemcpyAsync(b->d_tab_e, b->h_tab_e, (size_t)ne * 4 * sizeof(int32_t),
                       cudaMemcpyHostToDevice, b->stream));
    /* the staging buffers are reused by the next rebuild: wait for the copies */
    CU(cudaStreamSynchronize(b->stream));
  }
  b->dirty = 0;
  return FDTD_OK;
}

/* One step of every active member: the probe rows, H (+ faces), E (+ x-slab
 * pass unless the E kernel applies CPML X, faces) and the step counters. */
static int batch_step_ops(batch *b) {
  if (b->any_probes) KL(fdtdk_batch_probes(b->d_devs, b->n_act, b->stream));
  KL(fdtdk_batch_half(1, b->all_lean_h, b->d_devs, b->d_maps, b->d_ops, b->d_steps, b->d_tab_h,
                      b->n_h, b->d_work, b->d_err, b->stream));
  if (b->any_split)
    KL(fdtdk_batch_faces(1, b->d_devs, b->d_ops, b->d_steps, b->n_act, b->face_max,
                         b->stream));
  if (b->any_oblique)
    KL(fdtdk_batch_faces_oblique(1, b->d_devs, b->d_ops, b->d_steps, b->n_act, b->face_max,
                                 b->stream));
  KL(fdtdk_batch_half(0, b->all_lean, b->d_devs, b->d_maps, b->d_ops, b->d_steps,
                      b->d_tab_e, b->n_e, b->d_work + 2, b->d_err, b->stream));
  /* the lean E kernel may apply CPML X itself (compacted per warp) */
  if (b->any_xsplit && !(b->all_lean && fdtdk_batch_e_applies_x(1)))
    KL(fdtdk_batch_e_xslab(b->d_devs, b->d_ops, b->n_act, b->xs_max, b->stream));
  if (b->any_split)
    KL(fdtdk_batch_faces(0, b->d_devs, b->d_ops, b->d_steps, b->n_act, b->face_max,
                         b->stream));
  if (b->any_oblique)
    KL(fdtdk_batch_faces_oblique(0, b->d_devs, b->d_ops, b->d_steps, b->n_act, b->face_max,
                                 b->stream));
  KL(fdtdk_batch_advance(b->d_steps, b->n_act, b->stream));
  return FDTD_OK;
}

/* The batch's z-run (z-planes per work item) is measured once, on the
 * first step call with at least BATCH_TUNE_MIN_MEMBERS active members: a
 * few steps of the members with each candidate (the steps are real: the
 * result does not depend on the z-run), the fastest kept.  *steps_done
 * receives the steps taken.  The caller asks for more steps than the tuning
 * takes, so no member finishes inside it and every rebuild keeps them all. */
#define BATCH_TUNE_MIN_MEMBERS 8
#define BATCH_TUNE_CANDS 3
static int batch_tune(batch *b, int32_t *steps_done) {
  static const int cand[BATCH_TUNE_CANDS] = {8, 16, 32};
  float best = 1e30f;
  int bz = b->zrun, rc;
  for (int c = 0; c < BATCH_TUNE_CANDS; ++c) {
    b->zrun = cand[c];
    if (b->gexec) {
      cudaGraphExecDestroy(b->gexec);
      b->gexec = NULL;
    }
    if ((rc = batch_rebuild(b))) return rc;
    if ((rc = batch_step_ops(b))) return rc; /* untimed: the new tables */
    CU(cudaEventRecord(b->tev[0], b->stream));
    for (int k = 0; k < 3; ++k)
      if ((rc = batch_step_ops(b))) return rc;
    CU(cudaEventRecord(b->tev[1], b->stream));
    CU(cudaEventSynchronize(b->tev[1]));
    float ms = 0;
    CU(cudaEventElapsedTime(&ms, b->tev[0], b->tev[1]));
    if (ms < best) {
      best = ms;
      bz = cand[c];
    }
    /* the members' progress before the next rebuild uploads their steps */
    for (int g = 0; g < b->n_act; ++g) b->m[b->act[g]].done += 4;
    *steps_done += 4;
  }
  if (bz != b->zrun) {
    b->zrun = bz;
    if ((rc = batch_rebuild(b))) return rc;
  }
  b->tuned = 1;
  return FDTD_OK;
}

int fdtd_batch_get_zrun(fdtd_batch bh, int32_t *zrun) {
  batch *b = blookup(bh);
  if (!b) return fail(FDTD_ERR_INVALID_HANDLE, "invalid batch handle");
  if (!zrun) return fail(FDTD_ERR_INVALID_ARG, "null output");
  *zrun = b->tuned ? b->zrun : 0;
  return FDTD_OK;
}

/* Advances every active member by up to max_steps steps (all by the same
 * number: the fewest remaining steps of any active member, capped by
 * max_steps).  *active_left receives the number of members still running. */
int fdtd_batch_step(fdtd_batch bh, int32_t max_steps, int32_t *active_left) {
  batch *b = blookup(bh);
  if (!b) return fail(FDTD_ERR_INVALID_HANDLE, "invalid batch handle");
  int rc;
  int32_t left = 0;
  for (int i = 0; i < b->n; ++i) left += b->m[i].done < b->m[i].count;
  if (active_left) *active_left = left;
  if (!left || max_steps <= 0) return FDTD_OK;
  if (b->dirty) {
    /* new members: their own queued work must be on the device first */
    for (int i = 0; i < b->n; ++i) {
      if (b->m[i].done >= b->m[i].count) continue;
      sim *s = lookup(b->m[i].h);
      if (!s) return fail(FDTD_ERR_INVALID_HANDLE, "a batch member was deleted");
      if ((rc = flush(s))) return rc;
      CU(cudaEventRecord(s->ev[15], s->stream));
      CU(cudaStreamWaitEvent(b->stream, s->ev[15], 0));
    }
    if (b->gexec) { /* the mirrors and item tables change */
      cudaGraphExecDestroy(b->gexec);
      b->gexec = NULL;
    }
    if ((rc = batch_rebuild(b))) return rc;
  }
  int32_t nsteps = max_steps;
  for (int g = 0; g < b->n_act; ++g) {
    const bmember *m = &b->m[b->act[g]];
    if (m->count - m->done < nsteps) nsteps = m->count - m->done;
  }
  int32_t tuned = 0; /* steps the tuning took (already counted per member) */
  if (!b->tuned && b->n_act >= BATCH_TUNE_MIN_MEMBERS && nsteps > 4 * BATCH_TUNE_CANDS) {
    if ((rc = batch_tune(b, &tuned))) return rc;
  }
  int32_t t = tuned;
  if (nsteps - t >= GRAPH_CHUNK) {
    if (!b->gexec) {
      cudaGraph_t g;
      const double tc0 = mono_s();
      const unsigned long long before = fdtdk_launch_count();
      CU(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
      int crc = FDTD_OK;
      for (int c = 0; c < GRAPH_CHUNK && !crc; ++c) crc = batch_step_ops(b);
      cudaError_t ce = cudaStreamEndCapture(b->stream, &g);
      if (crc) return crc;
      if (ce != cudaSuccess) return fail(FDTD_ERR_CUDA, "graph capture: %s", cudaGetErrorString(ce));
      ce = cudaGraphInstantiate(&b->gexec, g, 0);
      cudaGraphDestroy(g);
      if (ce != cudaSuccess) {
        b->gexec = NULL;
        return fail(FDTD_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(ce));
      }
      b->g_kernels = fdtdk_launch_count() - before;
      g_captured_kernels += b->g_kernels;
      b->t_capture += mono_s() - tc0;
      b->n_capture += 1;
    }
    while (nsteps - t >= GRAPH_CHUNK) {
      t += GRAPH_CHUNK;
      CU(cudaGraphLaunch(b->gexec, b->stream));
      g_graph_kernels += b->g_kernels;
    }
  }
  for (; t < nsteps; ++t)
    if ((rc = batch_step_ops(b))) return rc;
  int finished = 0;
  for (int g = 0; g < b->n_act; ++g) {
    bmember *m = &b->m[b->act[g]];
    m->done += nsteps - tuned;
    if (m->done >= m->count) finished = 1;
  }
  if (finished) {
    /* finished members: later calls on their handles follow the batch */
    CU(cudaEventRecord(b->ev, b->stream));
    for (int g = 0; g < b->n_act; ++g) {
      bmember *m = &b->m[b->act[g]];
      if (m->done < m->count) continue;
      sim *s = lookup(m->h);
      if (s) CU(cudaStreamWaitEvent(s->stream, b->ev, 0));
    }
    b->dirty = 1;
  }
  left = 0;
  for (int i = 0; i < b->n; ++i) left += b->m[i].done < b->m[i].count;
  if (active_left) *active_left = left;
  return FDTD_OK;
}

int fdtd_internal_batch_counts(fdtd_batch bh, uint64_t n[2], double t[2]) {
  batch *b = blookup(bh);
  if (!b) return fail(FDTD_ERR_INVALID_HANDLE, "invalid batch handle");
  n[0] = b->n_rebuild;
  n[1] = b->n_capture;
  t[0] = b->t_rebuild;
  t[1] = b->t_capture;
  return FDTD_OK;
}

int fdtd_internal_batch_record(fdtd_batch bh, cudaEvent_t ev) {
  batch *b = blookup(bh);
  if (!b) return fail(FDTD_ERR_INVALID_HANDLE, "invalid batch handle");
  CU(cudaEventRecord(ev, b->stream));
  return FDTD_OK;
}

int fdtd_batch_status(fdtd_batch bh) {
  batch *b = blookup(bh);
  if (!b) return fail(FDTD_ERR_INVALID_HANDLE, "invalid batch handle");
  CU(cudaStreamSynchronize(b->stream));
  int32_t e = 0;
  CU(cudaMemcpy(&e, b->d_err, sizeof(e), cudaMemcpyDeviceToHost));
  if (e) {
    cudaMemset(b->d_err, 0, sizeof(int32_t));
    return fail(FDTD_ERR_CUDA, "a TMA pipeline wait timed out in a batched half-step "
                               "(device error word %d); member fields are not valid", e);
  }
  return FDTD_OK;
}

/* Runs every member to its last step. */
int fdtd_batch_run(fdtd_batch bh) {
  int32_t left = 1;
  while (left) {
    int rc = fdtd_batch_step(bh, 1 << 30, &left);
    if (rc) return rc;
  }
  return fdtd_batch_status(bh);
}

/* Drops the members (finished or not); device buffers are kept. */
int fdtd_batch_clear(fdtd_batch bh) {
  batch *b = blookup(bh);
  if (!b) return fail(FDTD_ERR_INVALID_HANDLE, "invalid batch handle");
  CU(cudaStreamSynchronize(b->stream));
  CU(cudaEventRecord(b->ev, b->stream));
  for (int i = 0; i < b->n; ++i) {
    sim *s = lookup(b->m[i].h);
    if (s) CU(cudaStreamWaitEvent(s->stream, b->ev, 0));
  }
  b->n = 0;
  b->n_act = 0;
  b->dirty = 1;
  return FDTD_OK;
}

/* Drops one member, finished or not; later calls on its handle follow the
 * batch's queued work. */
int fdtd_batch_remove(fdtd_batch bh, fdtd_handle h) {
  batch *b = blookup(bh);
  if (!b) return fail(FDTD_ERR_INVALID_HANDLE, "invalid batch handle");
  int idx = -1;
  for (int i = 0; i < b->n; ++i)
    if (b->m[i].h == h) idx = i;
  if (idx < 0) return fail(FDTD_ERR_INVALID_ARG, "not a member of this batch");
  CU(cudaEventRecord(b->ev, b->stream));
  sim *s = lookup(h);
  if (s) CU(cudaStreamWaitEvent(s->stream, b->ev, 0));
  memmove(&b->m[idx], &b->m[idx + 1], (size_t)(b->n - idx - 1) * sizeof(bmember));
  b->n -= 1;
  b->dirty = 1;
  return FDTD_OK;
}

/* Steps a member has completed in its batch (-1 if not a member). */
int fdtd_batch_progress(fdtd_batch bh, fdtd_handle h, int32_t *done) {
  batch *b = blookup(bh);
  if (!b) return fail(FDTD_ERR_INVALID_HANDLE, "invalid batch handle");
  if (!done) return fail(FDTD_ERR_INVALID_ARG, "null output");
  *done = -1;
  for (int i = 0; i < b->n; ++i)
    if (b->m[i].h == h) *done = b->m[i].done;
  return FDTD_OK;
}
