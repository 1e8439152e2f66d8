/*
 * fdtd_internal.h -- the thin C ABI between the host solver (fdtd_host.c,
 * plain C) and the sm_103a kernels (fdtd_kernels.cu).  Plain C structs
 * passed by value to the kernels; no C++ or torch types.
 */
#ifndef FDTD_INTERNAL_H
#define FDTD_INTERNAL_H

#include <stddef.h>
#include <stdint.h>

#include <cuda_runtime_api.h>

#include "fdtd_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

#define FDTD_MAX_PML 32
#define FDTD_NUM_PSI 6

/* CPML psi arrays: one per (field family, CPML axis), each storing the two
 * recurrences that share a slab index as an interleaved pair {first,
 * second}, so that a cell reads and writes both with one 8-byte access.
 * The reference keeps them as twelve separate arrays (src/simulation.h);
 * the values and their slab indexing are the same. */
enum {
  PSI_EY = 0, /* {psi_Exy, psi_Ezy}, index i + py*I + k*2p*I */
  PSI_EZ,     /* {psi_Exz, psi_Eyz}, index i + j*I + pz*I*J   */
  PSI_EX,     /* {psi_Eyx, psi_Ezx}, index px + j*2p + k*2p*J */
  PSI_HY,     /* {psi_Hxy, psi_Hzy} */
  PSI_HX,     /* {psi_Hyx, psi_Hzx} */
  PSI_HZ      /* {psi_Hxz, psi_Hyz} */
};

/* Everything a kernel needs to know about one grid (by value).
 * Field, coefficient and material-id arrays are pitched: cell (i,j,k) is
 * at i + j*Ip + k*Ip*J with Ip = I rounded up to a multiple of 8, so that
 * every row starts 32-byte aligned and TMA strides are multiples of 16 B.
 * CPML psi arrays and the 1D tables keep the reference's dense layouts. */
typedef struct {
  int32_t I, J, K, p;
  int32_t Ip;               /* row pitch (elements) */
  int64_t IJ, IJK;          /* logical I*J, I*J*K */
  int64_t plane;            /* Ip*J: plane stride */
  int64_t cells;            /* Ip*J*K: pitched array length */
  int32_t i0, i1, j0, j1, k0, k1;   /* TF/SF box */
  int32_t size1d, T;
  float Chh, Che, dx;
  /* quotient x/dx: see fdtd_make_div_plan (rdx = RN(1/dx); the corrected
   * product is used for div_lo <= |x| < div_hi, and on x*2^64 for
   * div_lo2 <= |x| < div_lo) */
  float rdx, div_lo, div_hi, div_lo2;
  float bE[2 * FDTD_MAX_PML], cE[2 * FDTD_MAX_PML];
  float bH[2 * FDTD_MAX_PML], cH[2 * FDTD_MAX_PML];
  float *f[6];              /* Ex Ey Ez Hx Hy Hz, x-fastest IJK each */
  const float *ce[6];       /* Cexe Ceye Ceze Cexh Ceyh Cezh (coef_mode 0) */
  int32_t coef_mode;        /* 0: per-cell arrays; 1: material-indexed */
  const uint16_t *mat;      /* coef_mode 1: coefficient-tuple id per cell */
  const float *mat_tab;     /* coef_mode 1: [n][6] Cexe..Cezh per id */
  int32_t n_mat;            /* coef_mode 1: number of ids */
  float *psi[FDTD_NUM_PSI];  /* pairs: [slab cells][2] */
  const float *inc[4];      /* Ez_1D, Hy_1D, E_inv_1D, H_inv_1D: [T][size1d] */
  const float *src;         /* current-source waveform [T] */
  int32_t *step_base;       /* device step base for graph-replayed steps */
  int32_t *work;            /* [0] work-item counter, [1] finished producers
                               (persistent kernels; zero between launches) */
  int32_t *probe_row;       /* device probe row counter */
  float *probes;            /* [T][num_ant][6] */
  const int64_t *probe_idx; /* [num_ant] pitched cell index, -1 if outside */
  int32_t num_ant;
  int32_t *err;             /* device error word (bounded-wait timeouts) */
  int32_t zc_h, zc_e;       /* z-planes per TMA work item (0: heuristic) */
  /* oblique plane wave (TF/SF mode 5): unit propagation direction, E
   * polarisation, H direction (k x e); the TF/SF box corner the wave reaches
   * first; its coordinate in the stored 1D window; 1D nodes per cell along
   * k; the window width; the window tables [T][ob_w] of the 1D E (at nodes)
   * and H (at half nodes) */
  float ob_k[3], ob_e[3], ob_h[3], ob_x0;
  int32_t ob_r0[3], ob_w;
  const float *ob_inc[2];
  float ob_rho;
  /* H coefficients: 0 uniform (Chh, Che); per cell (fdtd_set_magnetic):
   * 1 arrays hc[6 * cells] (Chh x, y, z, then Che x, y, z), 2 indexed
   * (hmat ids, hmat_tab [n][6] in the same order) */
  int32_t hcoef_mode;
  const float *hc;
  const uint16_t *hmat;
  const float *hmat_tab;
  /* tile geometry of the single-grid H and E curl kernels (autotuned):
   * 0 64 x 8, 1 32 x 16, 2 128 x 4 (size: a multiple of 16 bytes) */
  int32_t tile_h, tile_e;
} fdtd_dev;

/* TMA descriptors (CUtensorMap, 128 B each) of one grid in one tile
 * geometry: 0..5 = Ex Ey Ez Hx Hy Hz as E-half-step boxes, 6..11 the same
 * arrays as H-half-step boxes, 12 = material ids.  Opaque to C.  A handle
 * holds one set per geometry (FDTD_NUM_TILES: 64 x 8, 32 x 16 -- also the
 * batched kernels' -- and 128 x 4). */
#define FDTD_NUM_MAPS 13
#define FDTD_NUM_TILES 3
#ifdef __cplusplus
#define FDTD_ALIGN64 alignas(64)
#else
#define FDTD_ALIGN64 _Alignas(64)
#endif
typedef struct {
  FDTD_ALIGN64 unsigned char bytes[FDTD_NUM_MAPS][128];
  int32_t valid;            /* 1 when every map encoded */
} fdtd_maps;

/* One fused half-step: which parts run, for which step. */
typedef struct {
  int32_t curl;             /* Yee curl update */
  int32_t pml;              /* CPML psi recurrences + corrections */
  int32_t tfsf_mode;        /* 0 none, 1..4 reference plane-wave modes */
  int32_t step;             /* step index (offset when step_from_dev) */
  int32_t step_from_dev;    /* step = *step_base + step */
  int32_t cur_mode;         /* 0 none, 1..3 Ex/Ey/Ez current source */
  int32_t cur_box[6];
  int32_t tfsf_split;       /* TMA kernels: TF/SF applied by the face pass */
  int32_t xsplit;           /* TMA E kernel: CPML X applied by the x-slab pass */
  int32_t pad_[2];
} fdtd_op;

/* Can the TF/SF corrections of this half-step run as a separate pass over
 * the face cells after the curl kernel?  The reference applies, per cell,
 * curl, TF/SF, CPML (and, for E, the current source) in that order; a face
 * cell that is in no CPML slab and outside the current-source box has
 * curl then TF/SF only, so adding the correction afterwards gives the same
 * value.  Faces clear of every slab: i0 >= p+1 and i1 <= I-p-1 on each axis
 * (the H faces are at i0-1 and i1). */
static inline int fdtd_tfsf_faces_clear(const fdtd_dev *d, const fdtd_op *op) {
  const int p = d->p;
  if (d->i0 < p + 1 || d->j0 < p + 1 || d->k0 < p + 1) return 0;
  if (d->i1 > d->I - p - 1 || d->j1 > d->J - p - 1 || d->k1 > d->K - p - 1) return 0;
  if (d->i0 > d->i1 || d->j0 > d->j1 || d->k0 > d->k1) return 0;
  if (op->cur_mode) { /* current box against the six face planes */
    const int *b = op->cur_box;
    const int lo[3] = {d->i0, d->j0, d->k0}, hi[3] = {d->i1, d->j1, d->k1};
    for (int a = 0; a < 3; ++a) {
      const int u = (a + 1) % 3, v = (a + 2) % 3;
      const int cross = b[2 * u] <= hi[u] && b[2 * u + 1] >= lo[u] - 1 &&
                        b[2 * v] <= hi[v] && b[2 * v + 1] >= lo[v] - 1;
      const int on_lo = b[2 * a] <= lo[a] && b[2 * a + 1] >= lo[a] - 1;
      const int on_hi = b[2 * a] <= hi[a] && b[2 * a + 1] >= hi[a];
      if (cross && (on_lo || on_hi)) return 0;
    }
  }
  return 1;
}

static inline int fdtd_tfsf_split(const fdtd_dev *d, const fdtd_op *op) {
  if (!op->tfsf_mode || !op->curl) return 0;
  return fdtd_tfsf_faces_clear(d, op);
}

/* Can the E half-step's CPML X corrections run as a separate pass over the
 * x-slab cells after the curl kernel?  Per cell the reference applies curl,
 * TF/SF, CPML Y, Z, X and then the current source (src/simulation.h:386-418,
 * the source after them), so X is the last step of an x-slab cell unless the
 * current source reaches that column: E x slabs are i in [1, p) and
 * [I-p, I-1]. */
static inline int fdtd_xsplit(const fdtd_dev *d, const fdtd_op *op) {
  if (!op->pml || !op->curl || d->p < 1) return 0;
  if (2 * (int64_t)d->p * d->J * d->K > 0x7fffffff) return 0; /* the pass indexes in 32 bits */
  if (op->cur_mode >= 1 && op->cur_mode <= 3) {
    const int32_t a = op->cur_box[0], b = op->cur_box[1];
    if (a <= d->p - 1 && b >= 1) return 0;
    if (b >= d->I - d->p && a <= d->I - 1) return 0;
  }
  return 1;
}

/* The lean E curl kernel serves an op (tfsf_split and xsplit already set)
 * whose TF/SF corrections run in the face pass or are absent, whose CPML X
 * runs in the x-slab pass or is absent, and which has no current source. */
static inline int fdtd_e_lean(const fdtd_op *op) {
  return (!op->tfsf_mode || op->tfsf_split) && !op->cur_mode && (!op->pml || op->xsplit);
}

/* The lean H curl kernel: TF/SF corrections in the face pass or absent. */
static inline int fdtd_h_lean(const fdtd_op *op) { return !op->tfsf_mode || op->tfsf_split; }

/* TF/SF mode 5: an oblique plane wave (fdtd_set_incidence), applied only as
 * face passes after the curl / CPML kernels, which needs the faces clear of
 * the CPML and the current source (fdtd_tfsf_faces_clear). */
#define FDTD_MODE_OBLIQUE 5

/* The fused step (fdtd_fused.cu): H and E of a step in one pass that reads
 * the fields from one buffer and writes them to a second one (steps go in
 * pairs).  Tensor maps of the old buffer: Ex Ey Ez and Hx Hy Hz as boxes
 * with the tile's halo, the material ids. */
#define FDTD_FUSED_MAPS 7
typedef struct {
  FDTD_ALIGN64 unsigned char bytes[FDTD_FUSED_MAPS][128];
  int32_t valid;
} fdtd_maps_fused;

/* Can a step of this op run as the fused pass?  Curl and CPML, no current
 * source, uniform H coefficients, CPML X of E split off (fdtd_xsplit), and
 * TF/SF faces at least three cells inside every CPML slab (the E cells on
 * both sides of an H face plane, +-2 cells along it, are recomputed after
 * the H face pass and must hold no CPML work). */
static inline int fdtd_fused_ok(const fdtd_dev *d, const fdtd_op *op) {
  if (!op->curl || !op->pml || op->cur_mode || d->hcoef_mode || d->p < 1) return 0;
  if (d->I < 2 || d->J < 2 || d->K < 2) return 0;
  if (2 * (int64_t)d->p * d->J * d->K > 0x7fffffff) return 0; /* the x-slab pass */
  if (!op->tfsf_mode) return 1;
  const int p = d->p;
  if (d->i0 < p + 3 || d->j0 < p + 3 || d->k0 < p + 3) return 0;
  if (d->i1 > d->I - p - 3 || d->j1 > d->J - p - 3 || d->k1 > d->K - p - 3) return 0;
  return d->i0 <= d->i1 && d->j0 <= d->j1 && d->k0 <= d->k1;
}

/* Launchers (fdtd_kernels.cu).  Return cudaError_t as int.  m: the maps
 * of every tile geometry (FDTD_NUM_TILES).  With valid maps and op->curl
 * set, the TMA-pipelined kernels run (fdtd_tma.cu) in the descriptor's
 * tile geometries; otherwise the direct kernels.  use_tma = 0 forces the
 * direct kernels. */
int fdtdk_half_h(const fdtd_dev *d, const fdtd_maps *m, int use_tma, const fdtd_op *op,
                 cudaStream_t s);
int fdtdk_half_e(const fdtd_dev *d, const fdtd_maps *m, int use_tma, const fdtd_op *op,
                 cudaStream_t s);
/* Encodes the TMA descriptors for the current device pointers in tile
 * geometry `tile` (fdtd_tma.cu; tile 1 is the batched kernels'). */
int fdtdk_make_maps(const fdtd_dev *d, int tile, fdtd_maps *m);
int fdtdk_half_h_tma(const fdtd_dev *d, const fdtd_maps *m, const fdtd_op *op, cudaStream_t s);
int fdtdk_half_e_tma(const fdtd_dev *d, const fdtd_maps *m, const fdtd_op *op, cudaStream_t s);
/* The E CPML X corrections over the x-slab cells of a grid whose curl kernel
 * ran with op->xsplit (and of every batch member whose op has it set;
 * max_cells: the largest 2p*J*K among them). */
int fdtdk_e_xslab(const fdtd_dev *d, cudaStream_t s);
int fdtdk_batch_e_xslab(const fdtd_dev *devs, const fdtd_op *ops, int32_t n, int64_t max_cells,
                        cudaStream_t s);
/* Material-indexed E coefficients: dedupes the per-cell tuples of ce[6]
 * into mat[] ids and a [n][6] table.  Returns the number of distinct
 * tuples in *n_out, or 0 when they do not fit max_mat / collide. */
int fdtdk_compress_ce(const fdtd_dev *d, const float *const ce[6], uint16_t *mat,
                      float *tab, int32_t max_mat, unsigned long long *hash_keys,
                      int64_t *hash_rep, int32_t *hash_id, int32_t hash_cap,
                      int32_t *counters, cudaStream_t s);
/* Reads the compression counters: [0] distinct tuples, [1] overflow,
 * [2] collision. */
int fdtdk_probe_gather(const fdtd_dev *d, cudaStream_t s);
int fdtdk_set_i32(int32_t *dst, int32_t v, cudaStream_t s);
int fdtdk_fill_f32(float *dst, float v, int64_t n, cudaStream_t s);
int fdtdk_add_i32(int32_t *dst, int32_t v, cudaStream_t s);
/* Per-cell E coefficients from device eps/sigma (src/simulation.h:924-938). */
int fdtdk_compute_ce(const fdtd_dev *d, float *const ce[6],
                     const float *const eps[3], const float *const sig[3],
                     const float *den_ex, float delT, cudaStream_t s);
/* Forward + inverse 1D incident runs (src/simulation.h:134-254). */
int fdtdk_init_1d(const fdtd_dev *d, float *tab[4], const float *pw,
                  float Ceh, float *scratch, cudaStream_t s);
size_t fdtdk_init_1d_smem_limit(void);
/* Batched half-step over many grids (fdtd_tma.cu): table holds n_items
 * int4 {grid, x0, y0, kb | np << 16}; devs / maps (FDTD_NUM_MAPS x 128 B per
 * grid, 64-byte aligned) / ops / steps are per-grid device arrays; work is
 * a zeroed counter pair; lean when fdtd_e_lean (E) or fdtd_h_lean (H)
 * holds for every grid's op.  Every grid runs curl + CPML (+ its TF/SF mode and
 * current source) at step steps[g] + ops[g].step. */
int fdtdk_batch_half(int hfam, int lean, const fdtd_dev *devs, const void *maps,
                     const fdtd_op *ops, const int32_t *steps, const int32_t *table,
                     int32_t n_items, int32_t *work, int32_t *err, cudaStream_t s);
/* Probe rows of every grid of a batch, then +1 on each grid's probe row
 * and step (fdtd_kernels.cu). */
int fdtdk_batch_probes(const fdtd_dev *devs, int32_t n, cudaStream_t s);
/* 1 when the batched E kernel (lean variant when lean) applies the CPML X
 * corrections itself, so the batch needs no x-slab pass. */
int fdtdk_batch_e_applies_x(int lean);
int fdtdk_batch_advance(int32_t *steps, int32_t n, cudaStream_t s);
/* The fused pass's maps, its default z-run, the pass alone, and one whole
 * fused step: the pass from d_old (fields through m_old, H psi pairs) into
 * d_new (fields, H psi pairs; E psi in place), the E x-slab pass, the H
 * face pass, the E fix-up and the E face pass of op (zchunk 0: default). */
int fdtdk_make_maps_fused(const fdtd_dev *old, fdtd_maps_fused *m);
int fdtdk_fused_zchunk_default(int I, int J, int K);
int fdtdk_fused_pass(const fdtd_dev *d_new, const fdtd_dev *d_old, const fdtd_maps_fused *m_old,
                     int zchunk, cudaStream_t s);
int fdtdk_step_fused(const fdtd_dev *d_new, const fdtd_dev *d_old, const fdtd_maps_fused *m_old,
                     const fdtd_op *op, int zchunk, cudaStream_t s);
/* Batched-tile geometry of the TMA kernels. */
#define FDTD_TILE_X 64
#define FDTD_TILE_Y 8
#define FDTD_BTILE_X 32
#define FDTD_BTILE_Y 16

/* Per-cell mu coefficients (src/simulation.h:43-63). */
int fdtdk_compute_mu(float *out, const float *mu, const float *den_hx,
                     int64_t IJK, int32_t I, float delT, float sigma_m,
                     cudaStream_t s);
unsigned long long fdtdk_launch_count(void);
/* Measurement: while ev is set (not NULL), the half-step launchers of the
 * calling thread record it on the stream right after the curl kernel, so
 * that the curl kernel's time can be told from its passes' time. */
void fdtdk_set_profile_mark(cudaEvent_t ev);
void fdtdk_profile_mark(cudaStream_t s);
/* Records an error message for the calling thread (fdtd_last_error) and
 * returns code. */
int fdtd_internal_fail(int code, const char *msg);
/* Records ev on the stream a simulation's (or a batch's) work runs on, after
 * the work queued so far (the serving loop paces itself with these). */
int fdtd_internal_record(fdtd_handle h, cudaEvent_t ev);
int fdtd_internal_batch_record(fdtd_batch b, cudaEvent_t ev);
/* A batch's rebuilds and graph captures so far (n) and their host seconds
 * (t), for the serving loop's trace. */
int fdtd_internal_batch_counts(fdtd_batch b, uint64_t n[2], double t[2]);

/* TF/SF corrections of a split half-step over the face cells (single grid,
 * and every active member of a batch whose op has tfsf_split set;
 * max_cells_per_face sizes the blocks per member). */
int fdtdk_faces(int hfam, const fdtd_dev *d, const fdtd_op *op, cudaStream_t s);
int fdtdk_batch_faces(int hfam, const fdtd_dev *devs, const fdtd_op *ops, const int32_t *steps,
                      int32_t n, int32_t max_cells_per_face, cudaStream_t s);

int fdtdk_batch_faces_oblique(int hfam, const fdtd_dev *devs, const fdtd_op *ops,
                              const int32_t *steps, int32_t n, int32_t max_cells_per_face,
                              cudaStream_t s);
/* The 1D line of an oblique plane wave for all T steps (one block; the line
 * in shared memory, or in scratch[2*n1] when scratch is given). */
int fdtdk_init_1d_oblique(int n1, int m_src, int mb, int w, int T, float cE, float cH,
                          const float *pw, float *out_e, float *out_h, float *scratch,
                          cudaStream_t s);

/* Media from shapes into the six material arrays (sigma, eps; pitched). */
int fdtdk_rasterize(const fdtd_dev *d, float *const sig[3], float *const eps[3],
                    const fdtd_shape *shapes, int32_t n_shapes, float bg_eps, float bg_sig,
                    cudaStream_t s);

/* Plan for dividing by a fixed cell size (fdtd_host.c). */
typedef struct {
  float dx, rdx, lo, hi, lo2;
} fdtd_div_plan;
fdtd_div_plan fdtd_make_div_plan(float dx);
/* Adds to *out (device) the number of float bit patterns in
 * [first, first + count) whose plan quotient differs bitwise from the IEEE
 * division on the GPU. */
/* Bounded-wait self-check (fdtd_tma.cu): out[0] = 1 when the wait gave up,
 * out[1] = global-timer ns it took; the production limit and the check's
 * (ns). */
int fdtdk_check_wait(int arrive, long long out[2]);
unsigned long long fdtdk_wait_ns(void);
unsigned long long fdtdk_check_ns(void);
int fdtdk_check_division(fdtd_div_plan p, uint64_t first, uint64_t count,
                         unsigned long long *out, cudaStream_t s);

#ifdef __cplusplus
}
#endif
#endif
