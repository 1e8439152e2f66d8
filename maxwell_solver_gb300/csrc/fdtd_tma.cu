/*
 * fdtd_tma.cu -- TMA-pipelined half-step kernels for sm_103a.
 *
 * Each block owns a 64 x 8 (x, y) tile of a z-chunk and marches up in z.
 * One elected thread streams every z-plane the tile needs into a 4-stage
 * shared-memory ring with cp.async.bulk.tensor (TMA) copies completing on
 * per-stage mbarriers, so three to four planes of all fields are in flight
 * per block whatever the register count; the 256 threads compute from
 * shared memory (two cells each) and store their results with coalesced
 * stores.  The per-cell arithmetic is fdtd_device.cuh's, so results equal
 * the direct kernels' and the reference's bit for bit.
 *
 *   E half-step, plane k: E tile (64x8) + H tile with the x-1 / y-1 halo
 *     (68x9, box origin (x0-4, y0-1): the x origin stays 16-byte aligned)
 *     + the material-id tile; Hx, Hy of plane k-1 are carried in registers.
 *   H half-step, plane k: E tile with the x+1 / y+1 halo (68x9 at (x0, y0))
 *     + H tile; Ex, Ey of plane k+1 come from the next stage of the ring.
 *
 * Out-of-range boxes (grid edges, x < 0) are zero-filled by the TMA unit.
 * Every wait on an mbarrier is bounded: on a timeout the block drains its
 * own copies in flight (also bounded), raises the device error word and
 * returns.
 */
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include "fdtd_device.cuh"
#include "fdtd_internal.h"

using namespace fdtd;

extern "C" void fdtdk_count_launches(unsigned long long n);

namespace {

constexpr int BX = 64, BY = 8, NT = 256, NS = 4;
constexpr int HW = BX + 4;                  // halo box row (floats)
constexpr int HH = BY + 1;                  // halo box rows
constexpr int TILE_B = BX * BY * 4;         // 2048 B
constexpr int HALO_B = HW * HH * 4;         // 2448 B transferred
constexpr int HALO_SLOT = 2560;             // 128-byte aligned slot
constexpr int MAT_B = BX * BY * 2;          // 1024 B
constexpr int E_OFF_H = 3 * TILE_B;
constexpr int E_OFF_M = E_OFF_H + 3 * HALO_SLOT;
constexpr int E_STAGE = E_OFF_M + MAT_B;    // 14848 B
constexpr int H_OFF_H = 3 * HALO_SLOT;
constexpr int H_STAGE = H_OFF_H + 3 * TILE_B;  // 13824 B
constexpr int E_SMEM = NS * E_STAGE + 64;
constexpr int H_SMEM = NS * H_STAGE + 64;
constexpr unsigned kSpinLimit = 1u << 22;   // bounded mbarrier waits
static_assert(E_STAGE % 128 == 0 && H_STAGE % 128 == 0, "stage alignment");
static_assert((HW * 4) % 16 == 0 && (BX * 4) % 16 == 0 && (BX * 2) % 16 == 0,
              "TMA inner box extents must be multiples of 16 bytes");

struct Maps {
  CUtensorMap m[FDTD_NUM_MAPS];
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}

__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void proxy_fence() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait for phase `parity` of an mbarrier; false on timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
  for (unsigned it = 0; it < kSpinLimit; ++it)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, uint64_t *bar,
                                            int x, int y, int z) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}

// Timeout path of thread 0: wait (bounded) for the planes [from, issued)
// still in flight so no copy lands after the block is gone, then raise
// the error word.  A plane whose copies already completed returns at once
// (its stage has not been re-armed).
__device__ void drain_and_flag(uint64_t *bars, int from, int issued, int32_t *err, int code) {
  for (int q = from; q < issued; ++q) mbar_wait(&bars[q % NS], (uint32_t)((q / NS) & 1));
  if (err) atomicExch(err, code);
}

// ----------------------------------------------------------------- E half

template <bool PML>
__global__ void __launch_bounds__(NT, 3)
    k_half_e_tma(const fdtd_dev d, const fdtd_op op, const __grid_constant__ Maps mp, int zchunk) {
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem + NS * E_STAGE);
  const int tid = threadIdx.x, lane = tid & 31, ty = tid >> 5;
  const int x0 = blockIdx.x * BX, y0 = blockIdx.y * BY;
  const int I = d.I, J = d.J, K = d.K;
  const int kb = blockIdx.z * zchunk, ke = min(kb + zchunk, K);
  if (kb >= ke) return;
  const int np = ke - kb;
  const bool use_mat = d.coef_mode == 1;
  const uint32_t tx_bytes = 3 * TILE_B + 3 * HALO_B + (use_mat ? MAT_B : 0);
  int issued = 0;  // thread 0 only

  if (tid == 0) {
    for (int s = 0; s < NS; ++s) mbar_init(&bars[s], 1);
    mbar_init_fence();
  }
  __syncthreads();
  auto issue = [&](int q) {  // plane kb + q into stage q % NS
    unsigned char *st = smem + (q % NS) * E_STAGE;
    uint64_t *bar = &bars[q % NS];
    const int k = kb + q;
    proxy_fence();
    mbar_expect_tx(bar, tx_bytes);
    for (int c = 0; c < 3; ++c) tma_load_3d(st + c * TILE_B, &mp.m[c], bar, x0, y0, k);
    for (int c = 0; c < 3; ++c)
      tma_load_3d(st + E_OFF_H + c * HALO_SLOT, &mp.m[3 + c], bar, x0 - 4, y0 - 1, k);
    if (use_mat) tma_load_3d(st + E_OFF_M, &mp.m[12], bar, x0, y0, k);
  };
  if (tid == 0)
    for (; issued < NS && issued < np; ++issued) issue(issued);

  const int j = y0 + ty;
  const int mode = op.tfsf_mode;
  const int cm = op.cur_mode;
  const int step = (mode || cm) ? op_step(d, op) : 0;
  const float *inc = mode ? inc_e_row(d, mode, step) : nullptr;
  float hx_km[2] = {0.f, 0.f}, hy_km[2] = {0.f, 0.f};
  bool cur_col[2];
  float cur_src = 0.f;
#pragma unroll
  for (int c = 0; c < 2; ++c) {
    const int i = x0 + lane + 32 * c;
    cur_col[c] = cm && in_range(i, op.cur_box[0], op.cur_box[1]) &&
                 in_range(j, op.cur_box[2], op.cur_box[3]);
    if (kb > 0 && i < I && j < J) {
      const int64_t n = i + (int64_t)j * d.Ip + (int64_t)(kb - 1) * d.plane;
      hx_km[c] = d.f[3][n];
      hy_km[c] = d.f[4][n];
    }
  }
  if (cm && (cur_col[0] || cur_col[1])) cur_src = d.src[step];

  bool timeout = false;
  for (int t = 0; t < np; ++t) {
    const int s = t % NS;
    if (!timeout) timeout = !mbar_wait(&bars[s], (uint32_t)((t / NS) & 1));
    const int k = kb + t;
    const unsigned char *st = smem + s * E_STAGE;
    const float *sEx = reinterpret_cast<const float *>(st);
    const float *sEy = sEx + BX * BY;
    const float *sEz = sEy + BX * BY;
    const float *sHx = reinterpret_cast<const float *>(st + E_OFF_H);
    const float *sHy = sHx + HALO_SLOT / 4;
    const float *sHz = sHy + HALO_SLOT / 4;
    const uint16_t *sM = reinterpret_cast<const uint16_t *>(st + E_OFF_M);
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      const int xo = lane + 32 * c;
      const int i = x0 + xo;
      if (i < I && j < J && !timeout) {
        const int hb = (ty + 1) * HW + xo + 4;  // own cell in the halo tile
        const int eb = ty * BX + xo;            // own cell in the plain tile
        const float hx = sHx[hb], hy = sHy[hb], hz = sHz[hb];
        const int64_t n = i + (int64_t)j * d.Ip + (int64_t)k * d.plane;
        const Coef6 C = use_mat ? coef_from_table(d, sM[eb]) : coef_from_arrays(d, n);
        float ex = sEx[eb], ey = sEy[eb], ez = sEz[eb];
        int px = -1, py = -1, pz = -1;
        if (PML) e_slabs(d, i, j, k, px, py, pz);
        const bool cur = cur_col[c] && in_range(k, op.cur_box[4], op.cur_box[5]);
        update_e_cell<true, PML>(d, mode, inc, cm, cur_src, cur, i, j, k, px, py, pz, C, ex,
                                 ey, ez, hx, hy, hz, sHz[hb - HW], sHx[hb - HW], sHz[hb - 1],
                                 sHy[hb - 1], hx_km[c], hy_km[c]);
        d.f[0][n] = ex;
        d.f[1][n] = ey;
        d.f[2][n] = ez;
        hx_km[c] = hx;
        hy_km[c] = hy;
      }
    }
    if (__syncthreads_or(timeout)) {
      if (tid == 0) drain_and_flag(bars, t, issued, d.err, 1);
      return;
    }
    if (tid == 0 && issued < np) issue(issued++);
  }
}

// ----------------------------------------------------------------- H half

template <bool PML>
__global__ void __launch_bounds__(NT, 3)
    k_half_h_tma(const fdtd_dev d, const fdtd_op op, const __grid_constant__ Maps mp, int zchunk) {
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem + NS * H_STAGE);
  const int tid = threadIdx.x, lane = tid & 31, ty = tid >> 5;
  const int x0 = blockIdx.x * BX, y0 = blockIdx.y * BY;
  const int I = d.I, J = d.J, K = d.K, p = d.p;
  const int kb = blockIdx.z * zchunk, ke = min(kb + zchunk, K - 1);
  if (kb >= ke) return;
  const int np = ke - kb;  // planes computed
  const int nl = np + 1;   // planes loaded (E of plane k+1 is read)
  const uint32_t tx_bytes = 3 * HALO_B + 3 * TILE_B;
  int issued = 0;

  if (tid == 0) {
    for (int s = 0; s < NS; ++s) mbar_init(&bars[s], 1);
    mbar_init_fence();
  }
  __syncthreads();
  auto issue = [&](int q) {
    unsigned char *st = smem + (q % NS) * H_STAGE;
    uint64_t *bar = &bars[q % NS];
    const int k = kb + q;
    proxy_fence();
    mbar_expect_tx(bar, tx_bytes);
    for (int c = 0; c < 3; ++c) tma_load_3d(st + c * HALO_SLOT, &mp.m[6 + c], bar, x0, y0, k);
    for (int c = 0; c < 3; ++c)
      tma_load_3d(st + H_OFF_H + c * TILE_B, &mp.m[9 + c], bar, x0, y0, k);
  };
  if (tid == 0)
    for (; issued < NS && issued < nl; ++issued) issue(issued);

  const int j = y0 + ty;
  const int mode = op.tfsf_mode;
  const float *inc = mode ? inc_h_row(d, mode, op_step(d, op)) : nullptr;
  const int py = PML ? slab_h(j, J, p) : -1;

  bool timeout = !mbar_wait(&bars[0], 0u);
  for (int t = 0; t < np; ++t) {
    const int s0 = t % NS, s1 = (t + 1) % NS;
    if (!timeout) timeout = !mbar_wait(&bars[s1], (uint32_t)(((t + 1) / NS) & 1));
    const int k = kb + t;
    const unsigned char *st0 = smem + s0 * H_STAGE;
    const unsigned char *st1 = smem + s1 * H_STAGE;
    const float *sEx = reinterpret_cast<const float *>(st0);
    const float *sEy = sEx + HALO_SLOT / 4;
    const float *sEz = sEy + HALO_SLOT / 4;
    const float *sEx1 = reinterpret_cast<const float *>(st1);
    const float *sEy1 = sEx1 + HALO_SLOT / 4;
    const float *sHx = reinterpret_cast<const float *>(st0 + H_OFF_H);
    const float *sHy = sHx + BX * BY;
    const float *sHz = sHy + BX * BY;
    const int pz = PML ? slab_h(k, K, p) : -1;
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      const int xo = lane + 32 * c;
      const int i = x0 + xo;
      if (i < I - 1 && j < J - 1 && !timeout) {
        const int eb = ty * HW + xo;  // own cell in the halo tile
        const int hb = ty * BX + xo;  // own cell in the plain tile
        const float ex = sEx[eb], ey = sEy[eb], ez = sEz[eb];
        float hx = sHx[hb], hy = sHy[hb], hz = sHz[hb];
        const int px = PML ? slab_h(i, I, p) : -1;
        update_h_cell<true, PML>(d, mode, inc, i, j, k, px, py, pz, hx, hy, hz,
                                 sEz[eb + HW] - ez, sEx[eb + HW] - ex, sEz[eb + 1] - ez,
                                 sEy[eb + 1] - ey, sEy1[eb] - ey, sEx1[eb] - ex);
        const int64_t n = i + (int64_t)j * d.Ip + (int64_t)k * d.plane;
        d.f[3][n] = hx;
        d.f[4][n] = hy;
        d.f[5][n] = hz;
      }
    }
    if (__syncthreads_or(timeout)) {
      if (tid == 0) drain_and_flag(bars, t, issued, d.err, 2);
      return;
    }
    if (tid == 0 && issued < nl) issue(issued++);
  }
}

// z-chunk height: ~4 resident waves of 3 blocks per SM on 152 SMs.
inline int pick_zchunk(int bx, int by, int nk) {
  static int forced = -1;
  if (forced < 0) {
    const char *e = getenv("FDTD_TMA_ZCHUNK");
    forced = e ? atoi(e) : 0;
  }
  if (forced > 0) return forced;
  const long long xy = (long long)bx * by;
  const long long want = 152LL * 3 * 4;
  long long chunks = (want + xy - 1) / xy;
  if (chunks < 1) chunks = 1;
  if (chunks > nk) chunks = nk;
  int z = (int)((nk + chunks - 1) / chunks);
  if (z < 4) z = 4;
  if (z > 64) z = 64;
  return z;
}

template <class KH>
int launch(KH kern, int smem, const fdtd_dev *d, const fdtd_maps *m, const fdtd_op *op,
           cudaStream_t s, int ni, int nj, int nk) {
  static_assert(sizeof(Maps) == sizeof(((fdtd_maps *)0)->bytes), "map layout");
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return (int)e;
  Maps mp;
  memcpy(&mp, m->bytes, sizeof(Maps));
  const int bx = (ni + BX - 1) / BX, by = (nj + BY - 1) / BY;
  const int zc = pick_zchunk(bx, by, nk);
  dim3 grid(bx, by, (nk + zc - 1) / zc);
  kern<<<grid, NT, smem, s>>>(*d, *op, mp, zc);
  fdtdk_count_launches(1);
  return (int)cudaGetLastError();
}

PFN_cuTensorMapEncodeTiled_v12000 encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

int encode(CUtensorMap *out, void *base, CUtensorMapDataType dt, int esize, const fdtd_dev *d,
           int boxw, int boxh) {
  PFN_cuTensorMapEncodeTiled_v12000 enc = encoder();
  if (!enc) return (int)cudaErrorNotSupported;
  const cuuint64_t gdim[3] = {(cuuint64_t)d->I, (cuuint64_t)d->J, (cuuint64_t)d->K};
  const cuuint64_t gstride[2] = {(cuuint64_t)d->Ip * esize, (cuuint64_t)d->plane * esize};
  const cuuint32_t box[3] = {(cuuint32_t)boxw, (cuuint32_t)boxh, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = enc(out, dt, 3, base, gdim, gstride, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                   CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? 0 : (int)cudaErrorInvalidValue;
}

}  // namespace

extern "C" {

int fdtdk_make_maps(const fdtd_dev *d, fdtd_maps *m) {
  m->valid = 0;
  // TMA: 16-byte aligned base and strides; the pitch guarantees the strides
  if (((d->Ip * 4) % 16) || ((d->Ip * 2) % 16)) return (int)cudaErrorInvalidValue;
  CUtensorMap *maps = reinterpret_cast<CUtensorMap *>(m->bytes);
  for (int c = 0; c < 6; ++c)
    if (((uintptr_t)d->f[c]) % 16) return (int)cudaErrorInvalidValue;
  int e = 0;
  for (int c = 0; c < 3 && !e; ++c)
    e = encode(&maps[c], d->f[c], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, d, BX, BY);
  for (int c = 0; c < 3 && !e; ++c)
    e = encode(&maps[3 + c], d->f[3 + c], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, d, HW, HH);
  for (int c = 0; c < 3 && !e; ++c)
    e = encode(&maps[6 + c], d->f[c], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, d, HW, HH);
  for (int c = 0; c < 3 && !e; ++c)
    e = encode(&maps[9 + c], d->f[3 + c], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, d, BX, BY);
  if (!e) {
    if (!d->mat || ((uintptr_t)d->mat) % 16) return (int)cudaErrorInvalidValue;
    e = encode(&maps[12], (void *)d->mat, CU_TENSOR_MAP_DATA_TYPE_UINT16, 2, d, BX, BY);
  }
  if (!e) m->valid = 1;
  return e;
}

int fdtdk_half_e_tma(const fdtd_dev *d, const fdtd_maps *m, const fdtd_op *op, cudaStream_t s) {
  if (op->pml) return launch(k_half_e_tma<true>, E_SMEM, d, m, op, s, d->I, d->J, d->K);
  return launch(k_half_e_tma<false>, E_SMEM, d, m, op, s, d->I, d->J, d->K);
}

int fdtdk_half_h_tma(const fdtd_dev *d, const fdtd_maps *m, const fdtd_op *op, cudaStream_t s) {
  if (op->pml) return launch(k_half_h_tma<true>, H_SMEM, d, m, op, s, d->I - 1, d->J - 1, d->K - 1);
  return launch(k_half_h_tma<false>, H_SMEM, d, m, op, s, d->I - 1, d->J - 1, d->K - 1);
}

}  // extern "C"
