/*
 * fdtd_tma.cu -- persistent, warp-specialised TMA kernels of the two
 * half-steps for sm_103a.
 *
 * Work: the grid is cut into items of one (x, y) tile -- 64 x 8 in the
 * single-grid kernels, 32 x 16 in the batched ones -- and a run of
 * z-planes.  A launch is persistent (as many blocks as fit, at most one
 * per item): in every block one producer warp takes items from a global
 * atomic counter and streams every z-plane the item needs into a
 * shared-memory ring with cp.async.bulk.tensor (TMA) copies that complete
 * on the stage's "full" mbarrier; eight consumer warps wait on "full",
 * compute their cells from shared memory and release the stage on its
 * "empty" mbarrier.  There is no block-wide barrier in the steady state,
 * the ring stays full across item boundaries, and the dynamic queue keeps
 * the blocks busy to the end of the launch.  The producer that finishes
 * last rewinds the counter for the next launch.
 *
 *   E half-step, plane k: E tile (BX x BY) + H tile with the x-1 / y-1
 *     halo ((BX+4) x (BY+1), box origin (x0-4, y0-1): the x origin stays
 *     16-byte aligned) + the material-id tile; Hx, Hy of plane k-1 are
 *     carried in registers.
 *   H half-step, plane k: E tile with the x+1 / y+1 halo ((BX+4) x (BY+1)
 *     at (x0, y0)) + H tile.  Items march down in z: their first load is
 *     plane kb + np (Ex, Ey only), and Ex, Ey of plane k+1 are carried in
 *     registers.
 *
 * Cells with no CPML, TF/SF face or source in their warp take a lean
 * curl-only path; the others go through fdtd_device.cuh's full per-cell
 * functions.  Both compute the reference's operations in the reference's
 * order, so results equal the direct kernels' and the reference's bit for
 * bit.  Out-of-range boxes (grid edges, x < 0) are zero-filled by TMA.
 *
 * Every mbarrier wait is bounded.  A consumer that times out raises the
 * device error word and leaves; the producer, whose waits are bounded too,
 * then gives up, waits (bounded) for its own copies in flight and leaves.
 */
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <type_traits>

#include "fdtd_device.cuh"
#include "fdtd_internal.h"
#include "fdtd_pipe.cuh"

using namespace fdtd;
using namespace fdtd_pipe;

extern "C" void fdtdk_count_launches(unsigned long long n);

namespace {

constexpr int NCW = 8;                       // consumer warps
constexpr int NT = (NCW + 1) * 32;           // + one producer warp
#ifndef FDTD_NSE
#define FDTD_NSE 4
#endif
#ifndef FDTD_NSH
#define FDTD_NSH 4
#endif
// blocks per SM the single-grid kernels are compiled for (registers): the
// H kernel fits 4 (56 registers, 4 stages of 13.3 KB), the E kernel 3
// (72 registers; at 4 it spills)
#ifndef FDTD_MIN_BLOCKS_E
#define FDTD_MIN_BLOCKS_E 3
#endif
#ifndef FDTD_MIN_BLOCKS_H
#define FDTD_MIN_BLOCKS_H 4
#endif
constexpr int NSE = FDTD_NSE, NSH = FDTD_NSH;  // ring stages (E, H)
// Batch kernels: resident blocks per SM the register budget is sized for,
// and their ring depth (build-time tunables).
#ifndef FDTD_BATCH_MIN_BLOCKS_H
#define FDTD_BATCH_MIN_BLOCKS_H 3
#endif
#ifndef FDTD_BATCH_NS_H
#define FDTD_BATCH_NS_H 4
#endif
#ifndef FDTD_BATCH_MIN_BLOCKS
#define FDTD_BATCH_MIN_BLOCKS 3
#endif
#ifndef FDTD_BATCH_NS
#define FDTD_BATCH_NS 4
#endif
constexpr int kBatchMinBlocks = FDTD_BATCH_MIN_BLOCKS;  // E (and the default for H)
constexpr int kBatchNS = FDTD_BATCH_NS;
constexpr int kBatchMinBlocksH = FDTD_BATCH_MIN_BLOCKS_H;
constexpr int kBatchNSH = FDTD_BATCH_NS_H;
// Tile geometry: a work item is a BX x BY tile of cells over a run of
// z-planes.  The single-grid kernels use 64 x 8; the batched ones 32 x 16,
// since their grids are narrow (32..128 cells in x) and a 64-wide tile of a
// 70-cell axis leaves most lanes of its second tile idle.  Both have the
// same stage byte sizes.
template <int BX_, int BY_>
struct Geo {
  static constexpr int BX = BX_, BY = BY_;
  static constexpr int HW = BX + 4;                   // halo box row (floats)
  static constexpr int HH = BY + 1;                   // halo box rows
  static constexpr int TILE_B = BX * BY * 4;          // 2048 B
  static constexpr int HALO_B = HW * HH * 4;          // bytes transferred
  static constexpr int HALO_SLOT = (HALO_B + 127) / 128 * 128;  // 128-byte aligned slot
  static constexpr int MAT_B = BX * BY * 2;           // 1024 B
  static constexpr int E_OFF_H = 3 * TILE_B;
  static constexpr int E_OFF_M = E_OFF_H + 3 * HALO_SLOT;
  static constexpr int E_STAGE = E_OFF_M + MAT_B;
  static constexpr int H_OFF_H = 3 * HALO_SLOT;
  static constexpr int H_STAGE = H_OFF_H + 3 * TILE_B;
  static_assert(BX % 32 == 0 && (256 / 32) % (BX / 32) == 0 && BX * BY == 512,
                "8 consumer warps, two cells per thread");
  static_assert(E_STAGE % 128 == 0 && H_STAGE % 128 == 0, "stage alignment");
  static_assert((HW * 4) % 16 == 0 && (BX * 4) % 16 == 0 && (BX * 2) % 16 == 0,
                "TMA inner box extents must be multiples of 16 bytes");
};
using GS = Geo<64, 8>;   // single-grid kernels (tile 0, the default)
using GB = Geo<32, 16>;  // batched kernels; single-grid tile 1 (narrow grids)
using GW = Geo<128, 4>;  // single-grid tile 2 (wide grids)
template <bool BATCH>
using GeoOf = typename std::conditional<BATCH, GB, GS>::type;
// The single-grid tile geometry by index (fdtd_dev::tile_e / tile_h).
template <int T>
using TileGeo = typename std::conditional<T == 0, GS,
                                          typename std::conditional<T == 1, GB, GW>::type>::type;
constexpr int kSmemTabMax = 512;             // coefficient ids staged in shared memory
constexpr int CTRL_B = 512;                  // barriers + stage metadata
// Batch mode: every stage also carries its grid's descriptor and op (bulk
// copies completing on the stage's barrier), so the per-cell code reads
// them from shared memory instead of global memory; E stages also carry
// the grid's coefficient table when it has at most kStageTabMax ids.
constexpr int DESC_B = 1536;                 // >= sizeof(fdtd_dev), 128-aligned
constexpr int OPSLOT_B = 128;                // >= sizeof(fdtd_op)
constexpr int kStageTabMax = 64;
constexpr int TAB_B = kStageTabMax * 6 * 4;  // 1536 B
static_assert(sizeof(fdtd_dev) <= DESC_B && sizeof(fdtd_dev) % 16 == 0, "descriptor slot");
static_assert(sizeof(fdtd_op) <= OPSLOT_B && sizeof(fdtd_op) % 16 == 0, "op slot");
template <bool BATCH, class G = GeoOf<BATCH>>
struct EG {
  static constexpr int NS = BATCH ? kBatchNS : NSE;
  static constexpr int STAGE =
      BATCH ? G::E_STAGE + DESC_B + OPSLOT_B + TAB_B : G::E_STAGE;
  static constexpr int SMEM = NS * STAGE + CTRL_B + (BATCH ? 0 : kSmemTabMax * 6 * 4);
};
template <bool BATCH, class G = GeoOf<BATCH>>
struct HG {
  static constexpr int NS = BATCH ? kBatchNSH : NSH;
  static constexpr int STAGE = BATCH ? G::H_STAGE + DESC_B + OPSLOT_B : G::H_STAGE;
  static constexpr int SMEM = NS * STAGE + CTRL_B;
};
constexpr int E_SMEM = EG<false>::SMEM;
constexpr int H_SMEM = HG<false>::SMEM;
static_assert(EG<false, GW>::STAGE % 128 == 0 && HG<false, GW>::STAGE % 128 == 0,
              "stage alignment");
static_assert(EG<true>::STAGE % 128 == 0 && HG<true>::STAGE % 128 == 0, "batch stage alignment");
static_assert(kBatchMinBlocks * (EG<true>::SMEM + 1024) <= 228 * 1024 &&
                  kBatchMinBlocksH * (HG<true>::SMEM + 1024) <= 228 * 1024,
              "batch blocks per SM");
static_assert(NSH * (8 + 8 + 32) <= CTRL_B && NSE * (8 + 8 + 32) <= CTRL_B &&
                  kBatchNS * (8 + 8 + 32) <= CTRL_B && kBatchNSH * (8 + 8 + 32) <= CTRL_B,
              "control block");

struct Maps {
  CUtensorMap m[FDTD_NUM_MAPS];
};

// Work items of one launch.  Single grid: a regular decomposition of the
// grid (tiles_x * tiles_y tiles x z-runs of zchunk planes).  Batch: an
// explicit table over many grids, each with its descriptor, TMA maps, op
// and current step in device memory.
struct Items {
  int tiles_x, tiles_y, zchunk, nk, n_items;
  int32_t *work;             // [0] next item, [1] finished producers
  int32_t *err;              // device error word
  const int4 *table;         // batch: {grid, x0, y0, kb | np << 16} per item
  const fdtd_dev *devs;      // batch: per grid
  const CUtensorMap *maps;   // batch: FDTD_NUM_MAPS per grid
  const fdtd_op *ops;        // batch: per grid (step from steps[])
  const int32_t *steps;      // batch: step each grid is on
};

// Self-check of the bounded wait: one thread waits, with the production
// wait but a limit of kCheckNs, on a barrier that nothing completes
// (arrive = 0: it must give up and report it) or that it completes itself
// first (arrive = 1: it must succeed); out[0] = 1 when it gave up, out[1] =
// global-timer ns spent.
constexpr unsigned long long kCheckNs = 1000000ull;
__global__ void k_check_wait(long long *out, int arrive) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    mbar_init_fence();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (arrive) mbar_arrive(&bar);
    const unsigned long long t0 = global_ns();
    const bool ok = mbar_wait_for(&bar, 0, kCheckNs);
    out[1] = (long long)(global_ns() - t0);
    out[0] = ok ? 0 : 1;
  }
}

template <bool BATCH, class G>
__device__ __forceinline__ void decode_item(const Items &it, int w, int &g, int &x0, int &y0,
                                            int &kb, int &np) {
  if (BATCH) {
    const int4 e = it.table[w];
    g = e.x;
    x0 = e.y;
    y0 = e.z;
    kb = e.w & 0xFFFF;
    np = e.w >> 16;
  } else {
    const int nt = it.tiles_x * it.tiles_y;
    const int chunk = w / nt, tile = w - chunk * nt;
    g = 0;
    x0 = (tile % it.tiles_x) * G::BX;
    y0 = (tile / it.tiles_x) * G::BY;
    kb = chunk * it.zchunk;
    np = min(it.zchunk, it.nk - kb);
  }
}

// Stage metadata, written by the producer before it arms the stage:
// meta[2s] = {item, plane of the item, planes, first plane},
// meta[2s+1] = {grid, x0, y0, absolute step of the grid's op}.
// Producer side of one launch (lane 0 of the producer warp).  Up: the
// item's np planes from kb.  DOWN: `extra` more planes above the item come
// first (the H half-step reads plane k+1), then the item's planes from the
// top down; issue() is told which loads are such extra planes.
// Ends with a sentinel stage, rewinds the work counter when it is the last
// producer, and waits for its own copies before returning.
template <int NS, bool BATCH, bool DOWN, class G, class StepFn, class IssueFn>
__device__ void produce(const Items &it, int extra, uint64_t *full, uint64_t *empty, int4 *meta,
                        StepFn step_of, IssueFn issue) {
  int q = 0;
  bool ok = true;
  for (;;) {
    const int w = atomicAdd(&it.work[0], 1);
    if (w >= it.n_items) break;
    int g, x0, y0, kb, np;
    decode_item<BATCH, G>(it, w, g, x0, y0, kb, np);
    const int step = step_of(g);
    for (int t = 0; t < np + extra && ok; ++t, ++q) {
      const int s = q % NS;
      if (q >= NS) ok = mbar_wait(&empty[s], (uint32_t)(((q / NS) - 1) & 1));
      if (!ok) break;
      meta[2 * s] = make_int4(w, t, np, kb);
      meta[2 * s + 1] = make_int4(g, x0, y0, step);
      if (DOWN)
        issue(s, g, x0, y0, kb + np + extra - 1 - t, t < extra);
      else
        issue(s, g, x0, y0, kb + t, false);
    }
    if (!ok) break;
  }
  if (atomicAdd(&it.work[1], 1) == (int)gridDim.x - 1) {  // last producer: rewind
    atomicExch(&it.work[0], 0);
    atomicExch(&it.work[1], 0);
  }
  if (ok) {  // sentinel: tells the consumers there is no more work
    const int s = q % NS;
    if (q >= NS) ok = mbar_wait(&empty[s], (uint32_t)(((q / NS) - 1) & 1));
    if (ok) {
      meta[2 * s] = make_int4(-1, 0, 0, 0);
      mbar_arrive(&full[s]);
      ++q;
    }
  }
  if (!ok && it.err) atomicExch(it.err, 3);
  // drain: every copy issued by this block has landed before it retires
  for (int r = (q > NS ? q - NS : 0); r < q; ++r) mbar_wait(&full[r % NS], (uint32_t)((r / NS) & 1));
}

// Thread -> cell map of the consumer warps: warp w covers one 32-cell x run
// (run w % (BX/32) of the tile's row) of rows r0 = w / (BX/32) and
// r0 + BY/2, so that whole warps fall inside or outside the CPML x slabs and
// TF/SF x faces.
template <class G>
__device__ __forceinline__ void cell_map(int tid, int &xo, int &r0) {
  constexpr int WPR = G::BX / 32;  // warps per tile row
  const int w = tid >> 5;
  xo = 32 * (w % WPR) + (tid & 31);
  r0 = w / WPR;
}

// The CPML X columns of a warp's 32-cell run as at most two runs of lanes
// (the low and the high x slab): lanes a1 .. a1+len1-1 and a2 .. a2+len2-1.
struct XRuns {
  int a1, len1, a2, n;  // n = len1 + len2
};
__device__ __forceinline__ XRuns x_runs(unsigned mask) {
  XRuns r{0, 0, 0, __popc(mask)};
  if (!mask) return r;
  r.a1 = __ffs(mask) - 1;
  const unsigned up = mask >> r.a1;
  r.len1 = (~up == 0u) ? 32 - r.a1 : __ffs(~up) - 1;
  const unsigned rest = r.len1 >= 32 ? 0u : mask & ~(((1u << r.len1) - 1u) << r.a1);
  r.a2 = rest ? __ffs(rest) - 1 : 0;
  return r;
}
// Lane of the t-th X column (t < n).
__device__ __forceinline__ int x_run_lane(const XRuns &r, int t) {
  return t < r.len1 ? r.a1 + t : r.a2 + (t - r.len1);
}
// Generic-proxy writes into a ring stage before the stage goes back to the
// producer, whose TMA copies (async proxy) overwrite it next.
__device__ __forceinline__ void stage_writes_fence() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// ----------------------------------------------------------------- E half

// LEAN: every grid the launch serves has its TF/SF corrections in the face
// pass (or none), CPML X split from the per-cell path (or no CPML) and no
// current source, so the consumer drops those per-cell paths (fewer
// registers and branches; the cells it updates and their arithmetic are the
// same).
// XC (with LEAN and PML): the CPML X corrections, the last operation of an
// x-slab cell, run inside this kernel after each plane's curl and Y / Z
// corrections, compacted per warp: the warp's x-slab cells (a few lanes of
// each of its two rows) leave their Ey, Ez in the stage's E tile, and
// then the warp's lanes take them one per lane.  Without XC the x-slab pass
// (k_e_xslab) applies them after the kernel.
template <bool PML, bool BATCH, bool LEAN = false, bool XC = false, class GT = GeoOf<BATCH>>
__global__ void __launch_bounds__(NT, BATCH ? kBatchMinBlocks : FDTD_MIN_BLOCKS_E)
    k_half_e_tma(const __grid_constant__ fdtd_dev d0, const __grid_constant__ fdtd_op op0,
                 const __grid_constant__ Maps mp, const Items it) {
  static_assert(!XC || (LEAN && PML), "compacted CPML X needs the lean kernel with CPML");
  extern __shared__ __align__(128) unsigned char smem[];
  using G = GT;
  constexpr int ST = EG<BATCH, G>::STAGE;
  constexpr int NS = EG<BATCH, G>::NS;
  uint64_t *full = reinterpret_cast<uint64_t *>(smem + NS * ST);
  uint64_t *empty = full + NS;
  int4 *meta = reinterpret_cast<int4 *>(empty + NS);
  float *stab = reinterpret_cast<float *>(smem + NS * ST + CTRL_B);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // single grid: the coefficient table (if small) lives in shared memory
  const bool tab_in_smem = !BATCH && d0.coef_mode == 1 && d0.n_mat <= kSmemTabMax;
  // XC, single grid: the E grading tables for the per-lane X corrections
  __shared__ float s_xbcE[2][XC && !BATCH ? 2 * FDTD_MAX_PML : 1];
  if (XC && !BATCH)
    for (int t = tid; t < 2 * FDTD_MAX_PML; t += NT) {
      s_xbcE[0][t] = d0.bE[t];
      s_xbcE[1][t] = d0.cE[t];
    }

  if (tid == 0) {
    for (int s = 0; s < NS; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], NCW);
    }
    mbar_init_fence();
  }
  if (tab_in_smem)
    for (int t = tid; t < d0.n_mat * 6; t += NT) stab[t] = __ldg(d0.mat_tab + t);
  __syncthreads();

  if (warp == NCW) {  // ------------------------------------- producer
    if (lane == 0) {
      // per item (batch): the grid's coefficient mode and table size
      int g_um = -1;
      bool um = d0.coef_mode == 1;
      uint32_t tab_b = 0;
      const auto step_of = [&](int g) {
        return (BATCH ? it.steps[g] + it.ops[g].step : op_step(d0, op0));
      };
      produce<NS, BATCH, false, G>(it, 0, full, empty, meta, step_of, [&](int s, int g, int x0,
                                                                         int y0, int k, bool) {
        const CUtensorMap *mm = BATCH ? it.maps + (int64_t)g * FDTD_NUM_MAPS : mp.m;
        if (BATCH && g != g_um) {
          g_um = g;
          um = it.devs[g].coef_mode == 1;
          const int nm = it.devs[g].n_mat;
          // whole 16-byte units; the table allocation holds 32768 ids
          tab_b = (um && nm <= kStageTabMax) ? (uint32_t)((nm * 24 + 15) & ~15) : 0u;
        }
        unsigned char *st = smem + s * ST;
        const uint32_t desc_b = BATCH ? (uint32_t)(sizeof(fdtd_dev) + sizeof(fdtd_op)) : 0u;
        proxy_fence();
        // one arrive per phase: the stage's whole byte count at once
        mbar_expect_tx(&full[s], desc_b + 3 * G::TILE_B + 3 * G::HALO_B + (um ? G::MAT_B : 0) +
                                     (BATCH ? tab_b : 0u));
        if (BATCH) {
          bulk_g2s(st + G::E_STAGE, &it.devs[g], sizeof(fdtd_dev), &full[s]);
          bulk_g2s(st + G::E_STAGE + DESC_B, &it.ops[g], sizeof(fdtd_op), &full[s]);
          if (tab_b)
            bulk_g2s(st + G::E_STAGE + DESC_B + OPSLOT_B, it.devs[g].mat_tab, tab_b, &full[s]);
        }
        for (int c = 0; c < 3; ++c) tma_load_3d(st + c * G::TILE_B, &mm[c], &full[s], x0, y0, k);
        for (int c = 0; c < 3; ++c)
          tma_load_3d(st + G::E_OFF_H + c * G::HALO_SLOT, &mm[3 + c], &full[s], x0 - 4, y0 - 1, k);
        if (um) tma_load_3d(st + G::E_OFF_M, &mm[12], &full[s], x0, y0, k);
      });
    }
    return;
  }

  // ------------------------------------------------------------ consumers
  int xo, r0;
  cell_map<G>(tid, xo, r0);
  // per-item state
  int i = 0, y0 = 0, kb = 0, mode = 0, cm = 0;
  bool use_mat = false, tab_local = false;
  const float *inc = nullptr;
  float cur_src = 0.f;
  bool valid[2] = {false, false}, col_special[2] = {false, false}, cur_col[2] = {false, false};
  float hx_km[2] = {0.f, 0.f}, hy_km[2] = {0.f, 0.f};
  int64_t n0[2] = {0, 0};
  // XC: this warp's x-slab lanes and which of its rows hold x-slab cells
  XRuns xr{0, 0, 0, 0};
  bool x_lane = false, x_row[2] = {false, false};

  for (int q = 0;; ++q) {
    const int s = q % NS;
    if (!mbar_wait(&full[s], (uint32_t)((q / NS) & 1))) {
      if (it.err) atomicExch(it.err, 1);
      return;
    }
    const int4 m = meta[2 * s];
    if (m.x < 0) return;  // sentinel
    const unsigned char *st = smem + s * ST;
    const fdtd_dev &d = BATCH ? *reinterpret_cast<const fdtd_dev *>(st + G::E_STAGE) : d0;
    const fdtd_op &op = BATCH ? *reinterpret_cast<const fdtd_op *>(st + G::E_STAGE + DESC_B) : op0;
    const float *ttab = BATCH ? reinterpret_cast<const float *>(st + G::E_STAGE + DESC_B + OPSLOT_B)
                              : stab;
    const int I = d.I, J = d.J, K = d.K;
    const float *sHx = reinterpret_cast<const float *>(st + G::E_OFF_H);
    const float *sHy = sHx + G::HALO_SLOT / 4;
    const float *sHz = sHy + G::HALO_SLOT / 4;
    if (m.y == 0) {  // first plane of a new item: column constants
      const int4 m1 = meta[2 * s + 1];
      kb = m.w;
      y0 = m1.z;
      i = m1.y + xo;
      mode = (LEAN || op.tfsf_split) ? 0 : op.tfsf_mode;  // split: the face pass applies it
      cm = LEAN ? 0 : op.cur_mode;
      use_mat = d.coef_mode == 1;
      tab_local = BATCH ? (use_mat && d.n_mat <= kStageTabMax) : tab_in_smem;
      const int step = m1.w;
      inc = mode ? inc_e_row(d, mode, step) : nullptr;
      cur_src = cm ? d.src[step] : 0.f;
      const bool cur_x = cm && in_range(i, op.cur_box[0], op.cur_box[1]);
      // with xsplit the x-slab pass applies CPML X afterwards
      const bool x_special = (PML && !LEAN && !op.xsplit && slab_e(i, I, d.p) >= 0) ||
                             (mode && (i == d.i0 || i == d.i1)) || i == 0;
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        const int j = y0 + r0 + (G::BY / 2) * c;
        valid[c] = i < I && j < J;
        cur_col[c] = cur_x && in_range(j, op.cur_box[2], op.cur_box[3]);
        col_special[c] = x_special || (PML && slab_e(j, J, d.p) >= 0) ||
                         (mode && (j == d.j0 || j == d.j1)) || cur_col[c] || j == 0;
        n0[c] = valid[c] ? i + (int64_t)j * d.Ip + (int64_t)kb * d.plane : 0;
        hx_km[c] = hy_km[c] = 0.f;
        if (kb > 0 && valid[c]) {
          hx_km[c] = d.f[3][n0[c] - d.plane];
          hy_km[c] = d.f[4][n0[c] - d.plane];
        }
        // E x-slab cells: 1 <= j <= J-2 and 1 <= k <= K-2 (gpu.h:776-777)
        if (XC) x_row[c] = j >= 1 && j <= J - 2;
      }
      if (XC) {
        x_lane = i < I && slab_e(i, I, d.p) >= 0;
        xr = x_runs(__ballot_sync(0xffffffffu, x_lane));
      }
    }
    const int k = kb + m.y;
    const float *sEx = reinterpret_cast<const float *>(st);
    const float *sEy = sEx + G::BX * G::BY;
    const float *sEz = sEy + G::BX * G::BY;
    const uint16_t *sM = reinterpret_cast<const uint16_t *>(st + G::E_OFF_M);
    const bool plane_special = (PML && slab_e(k, K, d.p) >= 0) ||
                               (mode && (k == d.k0 || k == d.k1)) || k == 0 ||
                               (cm && in_range(k, op.cur_box[4], op.cur_box[5]));
    const int64_t off = (int64_t)m.y * d.plane;
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      const int ty = r0 + (G::BY / 2) * c;
      const bool act = valid[c];
      const int hb = (ty + 1) * G::HW + xo + 4;  // own cell in the halo tile
      const int eb = ty * G::BX + xo;            // own cell in the plain tile
      Coef6 C = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
      if (use_mat) {
        const int mi = sM[eb];
        if (tab_local) {
          const float *r = ttab + mi * 6;
          C.exe = r[0]; C.eye = r[1]; C.eze = r[2]; C.exh = r[3]; C.eyh = r[4]; C.ezh = r[5];
        } else {
          C = coef_from_table(d, mi);
        }
      } else if (act) {
        C = coef_from_arrays(d, n0[c] + off);
      }
      const float hx = sHx[hb], hy = sHy[hb], hz = sHz[hb];
      const float hz_jm = sHz[hb - G::HW], hx_jm = sHx[hb - G::HW];
      const float hz_im = sHz[hb - 1], hy_im = sHy[hb - 1];
      float ex = sEx[eb], ey = sEy[eb], ez = sEz[eb];
      if (__any_sync(0xffffffffu, act && (col_special[c] || plane_special))) {
        if (act) {
          const int j = y0 + ty;
          int px = -1, py = -1, pz = -1;
          if (PML) e_slabs(d, i, j, k, px, py, pz);
          if (LEAN || op.xsplit) px = -1;
          const bool cur = cur_col[c] && in_range(k, op.cur_box[4], op.cur_box[5]);
          update_e_cell<true, PML>(d, mode, inc, cm, cur_src, cur, i, j, k, px, py, pz, C, ex,
                                   ey, ez, hx, hy, hz, hz_jm, hx_jm, hz_im, hy_im, hx_km[c],
                                   hy_km[c]);
        }
      } else {  // interior warp: i, j, k >= 1, no CPML, TF/SF face or source
        ex = C.exe * ex + C.exh * (+(hz - hz_jm) - (hy - hy_km[c]));
        ey = C.eye * ey + C.eyh * (+(hx - hx_km[c]) - (hz - hz_im));
        ez = C.eze * ez + C.ezh * (+(hy - hy_im) - (hx - hx_jm));
      }
      const bool xcell = XC && x_lane && x_row[c] && k >= 1 && k <= K - 2;
      if (act) {
        d.f[0][n0[c] + off] = ex;
        if (xcell) {  // CPML X below: Ey, Ez wait in the stage's E tile
          const_cast<float *>(sEy)[eb] = ey;
          const_cast<float *>(sEz)[eb] = ez;
        } else {
          d.f[1][n0[c] + off] = ey;
          d.f[2][n0[c] + off] = ez;
        }
      }
      hx_km[c] = hx;
      hy_km[c] = hy;
    }
    if (XC && xr.n && k >= 1 && k <= K - 2 && (x_row[0] || x_row[1])) {
      // CPML X of the warp's x-slab cells (gpu.h:765-788), one per lane
      __syncwarp();
      const int nrow = (int)x_row[0] + (int)x_row[1];
      for (int t = lane; t < xr.n * nrow; t += 32) {
        const int c = x_row[0] ? t / xr.n : 1;
        const int xl = x_run_lane(xr, t % xr.n);
        const int ty = r0 + (G::BY / 2) * c;
        const int tcol = xo - lane + xl;  // the lane's column in the tile
        const int ix = i - xo + tcol, j = y0 + ty;
        const int eb = ty * G::BX + tcol, hb = (ty + 1) * G::HW + tcol + 4;
        const int px = slab_e(ix, I, d.p);
        const int64_t n = ix + (int64_t)j * d.Ip + (int64_t)k * d.plane;
        Coef6 C;
        if (use_mat) {
          const int mi = sM[eb];
          if (tab_local) {
            const float *r = ttab + mi * 6;
            C.eyh = r[4];
            C.ezh = r[5];
          } else {
            C = coef_from_table(d, mi);
          }
        } else {
          C = coef_from_arrays(d, n);
        }
        float ey = sEy[eb], ez = sEz[eb];
        float2 *X = psi_at_x(d, PSI_EX, px, j, k);
        const float xb = BATCH ? d.bE[px] : s_xbcE[0][px];
        const float xc = BATCH ? d.cE[px] : s_xbcE[1][px];
        e_corr_x_bc(d, xb, xc, *X, X, C, sHz[hb], sHz[hb - 1], sHy[hb], sHy[hb - 1], ey, ez);
        d.f[1][n] = ey;
        d.f[2][n] = ez;
      }
      stage_writes_fence();
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[s]);
  }
}

// ----------------------------------------------------------------- H half

// MU: per-cell H coefficients (fdtd_set_magnetic), read per cell from the
// material ids and table (or the arrays); compiled for 3 blocks per SM.
// LEAN: every grid the launch serves has its TF/SF corrections in the face
// pass (or none), so the consumer drops the inline TF/SF path.
// XC (with LEAN and PML, not MU): on planes outside the z slabs, the CPML X
// corrections (after curl and Y, gpu.h:604-642) run compacted per warp: the
// x-slab cells leave their Hy, Hz in the stage's H tile and the warp's
// lanes then take them one per lane, instead of every row of a warp that
// holds a few x-slab lanes taking the correction path.
template <bool PML, bool BATCH, bool MU = false, bool LEAN = false, bool XC = false,
          class GT = GeoOf<BATCH>>
__global__ void __launch_bounds__(NT, BATCH ? kBatchMinBlocksH : (MU ? 3 : FDTD_MIN_BLOCKS_H))
    k_half_h_tma(const __grid_constant__ fdtd_dev d0, const __grid_constant__ fdtd_op op0,
                 const __grid_constant__ Maps mp, const Items it) {
  static_assert(!XC || (LEAN && PML && !MU), "compacted CPML X needs the lean kernel with CPML");
  extern __shared__ __align__(128) unsigned char smem[];
  using G = GT;
  constexpr int ST = HG<BATCH, G>::STAGE;
  constexpr int NS = HG<BATCH, G>::NS;
  uint64_t *full = reinterpret_cast<uint64_t *>(smem + NS * ST);
  uint64_t *empty = full + NS;
  int4 *meta = reinterpret_cast<int4 *>(empty + NS);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

  // the X-axis CPML grading, read per lane below: a shared-memory copy
  // (indexed loads from the by-value descriptor would be divergent
  // constant-bank loads); in batch mode the staged descriptor has it
  __shared__ float s_xbc[2][2 * FDTD_MAX_PML];
  if (!BATCH && PML)
    for (int t = tid; t < 2 * FDTD_MAX_PML; t += NT) {
      s_xbc[0][t] = d0.bH[t];
      s_xbc[1][t] = d0.cH[t];
    }
  if (tid == 0) {
    for (int s = 0; s < NS; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], NCW);
    }
    mbar_init_fence();
  }
  __syncthreads();

  if (warp == NCW) {  // ------------------------------------- producer
    if (lane == 0) {
      const uint32_t tx_bytes = 3 * G::HALO_B + 3 * G::TILE_B;
      const auto step_of = [&](int g) {
        return (BATCH ? it.steps[g] + it.ops[g].step : op_step(d0, op0));
      };
      // planes from the top down; the item's first load is plane kb + np,
      // of which the consumers read Ex and Ey of their own cells
      produce<NS, BATCH, true, G>(it, 1, full, empty, meta, step_of, [&](int s, int g, int x0,
                                                                       int y0, int k,
                                                                       bool above) {
        const CUtensorMap *mm = BATCH ? it.maps + (int64_t)g * FDTD_NUM_MAPS : mp.m;
        unsigned char *st = smem + s * ST;
        proxy_fence();
        mbar_expect_tx(&full[s], (above ? 2 * G::HALO_B : tx_bytes) +
                                     (BATCH ? (uint32_t)(sizeof(fdtd_dev) + sizeof(fdtd_op))
                                            : 0u));
        if (BATCH) {
          bulk_g2s(st + G::H_STAGE, &it.devs[g], sizeof(fdtd_dev), &full[s]);
          bulk_g2s(st + G::H_STAGE + DESC_B, &it.ops[g], sizeof(fdtd_op), &full[s]);
        }
        for (int c = 0; c < (above ? 2 : 3); ++c)
          tma_load_3d(st + c * G::HALO_SLOT, &mm[6 + c], &full[s], x0, y0, k);
        if (!above)
          for (int c = 0; c < 3; ++c)
            tma_load_3d(st + G::H_OFF_H + c * G::TILE_B, &mm[9 + c], &full[s], x0, y0, k);
      });
    }
    return;
  }

  // ------------------------------------------------------------ consumers
  int xo, r0;
  cell_map<G>(tid, xo, r0);

  int q = 0;
  for (;;) {
    int s = q % NS;
    if (!mbar_wait(&full[s], (uint32_t)((q / NS) & 1))) {
      if (it.err) atomicExch(it.err, 2);
      return;
    }
    const int4 m = meta[2 * s];
    if (m.x < 0) return;  // sentinel
    const int4 m1 = meta[2 * s + 1];
    const int x0 = m1.y, y0 = m1.z, kb = m.w, np = m.z;
    // the item's descriptor and op: the first load's copies (every load of
    // the item carries the same ones)
    const unsigned char *st_item = smem + s * ST;
    const fdtd_dev &d = BATCH ? *reinterpret_cast<const fdtd_dev *>(st_item + G::H_STAGE) : d0;
    const fdtd_op &op =
        BATCH ? *reinterpret_cast<const fdtd_op *>(st_item + G::H_STAGE + DESC_B) : op0;
    const int I = d.I, J = d.J, K = d.K, p = d.p;
    // split: the face pass applies it
    const int mode = (LEAN || op.tfsf_split) ? 0 : op.tfsf_mode;
    const float *inc = mode ? inc_h_row(d, mode, m1.w) : nullptr;
    const float Chh = d.Chh, Che = d.Che;
    const int i = x0 + xo;
    const int px = PML ? slab_h(i, I, p) : -1;
    const bool x_face = mode && (i == d.i0 - 1 || i == d.i1);
    bool valid[2], col_face[2];  // col_face: a TF/SF face cell (not split off)
    bool valid_row[2];           // the row holds H cells (j <= J-2)
    bool ax[2];                  // a cell of the warp row is in an x slab
    int py[2];
    int64_t n0[2];
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      const int j = y0 + r0 + (G::BY / 2) * c;
      valid[c] = i < I - 1 && j < J - 1;
      valid_row[c] = j < J - 1;
      py[c] = PML ? slab_h(j, J, p) : -1;
      col_face[c] = x_face || (mode && (j == d.j0 - 1 || j == d.j1));
      n0[c] = valid[c] ? i + (int64_t)j * d.Ip + (int64_t)kb * d.plane : 0;
      ax[c] = PML && __any_sync(0xffffffffu, valid[c] && px >= 0);
    }
    // XC: the warp's x-slab lanes (i <= I-2: H cells) as runs
    const bool x_lane = XC && i < I - 1 && px >= 0;
    const XRuns xr = XC ? x_runs(__ballot_sync(0xffffffffu, x_lane)) : XRuns{0, 0, 0, 0};
    // the item's first load is plane kb + np: Ex, Ey of the own cells, the
    // upper ends of plane kb + np - 1's z differences; then the planes from
    // the top down, each carrying its own Ex, Ey to the plane below
    float ex1[2], ey1[2];
    {
      const float *sEx = reinterpret_cast<const float *>(st_item);
      const float *sEy = sEx + G::HALO_SLOT / 4;
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        const int eb = (r0 + (G::BY / 2) * c) * G::HW + xo;
        ex1[c] = sEx[eb];
        ey1[c] = sEy[eb];
      }
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[s]);
    ++q;
    for (int t = np - 1; t >= 0; --t, ++q) {
      s = q % NS;
      if (!mbar_wait(&full[s], (uint32_t)((q / NS) & 1))) {
        if (it.err) atomicExch(it.err, 2);
        return;
      }
      const int k = kb + t;
      const unsigned char *st0 = smem + s * ST;
      // descriptor of the stage in use (the item's first stage has been
      // handed back to the producer)
      const fdtd_dev &dp = BATCH ? *reinterpret_cast<const fdtd_dev *>(st0 + G::H_STAGE) : d0;
      const float *sEx = reinterpret_cast<const float *>(st0);
      const float *sEy = sEx + G::HALO_SLOT / 4;
      const float *sEz = sEy + G::HALO_SLOT / 4;
      const float *sHx = reinterpret_cast<const float *>(st0 + G::H_OFF_H);
      const float *sHy = sHx + G::BX * G::BY;
      const float *sHz = sHy + G::BX * G::BY;
      const int pz = PML ? slab_h(k, K, p) : -1;
      const bool plane_face = mode && (k == dp.k0 - 1 || k == dp.k1);
      const int64_t off = (int64_t)t * dp.plane;
      // XC on this plane: outside the z slabs, X is compacted below
      const bool xc_plane = XC && pz < 0 && xr.n > 0;
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        const int ty = r0 + (G::BY / 2) * c;
        const bool act = valid[c];
        const int eb = ty * G::HW + xo;  // own cell in the halo tile
        const int hb = ty * G::BX + xo;  // own cell in the plain tile
        const float ex = sEx[eb], ey = sEy[eb], ez = sEz[eb];
        const float dEz_y = sEz[eb + G::HW] - ez, dEx_y = sEx[eb + G::HW] - ex;
        const float dEz_x = sEz[eb + 1] - ez, dEy_x = sEy[eb + 1] - ey;
        const float dEy_z = ey1[c] - ey, dEx_z = ex1[c] - ex;
        ex1[c] = ex;
        ey1[c] = ey;
        float hx = sHx[hb], hy = sHy[hb], hz = sHz[hb];
        // lean path (curl, then at most one CPML axis) unless a cell is on
        // a TF/SF face or in two slabs
        const bool oth = !LEAN && __any_sync(0xffffffffu, act && (col_face[c] || plane_face));
        const bool ay = PML && py[c] >= 0, az = PML && pz >= 0;
        const int j = y0 + ty;
        const HCoef C = MU ? hcoef_at(dp, act ? n0[c] + off : 0) : HCoef{Chh, Chh, Chh, Che, Che, Che};
        if (xc_plane) {  // curl, Y (warp-uniform); X below for the x-slab lanes
          hx = C.hhx * hx + C.hex * (-dEz_y + dEy_z);
          hy = C.hhy * hy + C.hey * (-dEx_z + dEz_x);
          hz = C.hhz * hz + C.hez * (-dEy_x + dEx_y);
          if (ay && act) {
            float2 *Y = psi_at_y(dp, PSI_HY, i, py[c], k);
            h_corr_y(dp, py[c], *Y, Y, dEz_y, dEx_y, hx, hz, C.hex, C.hez);
          }
          if (act) {
            dp.f[3][n0[c] + off] = hx;
            if (x_lane) {  // Hy, Hz wait in the stage's H tile
              const_cast<float *>(sHy)[hb] = hy;
              const_cast<float *>(sHz)[hb] = hz;
            } else {
              dp.f[4][n0[c] + off] = hy;
              dp.f[5][n0[c] + off] = hz;
            }
          }
          continue;
        }
        if (oth || (int)ax[c] + (int)ay + (int)az > 1) {
          if (act) {
            update_h_cell<true, PML>(dp, C, mode, inc, i, j, k, px, py[c], pz,
                                     hx, hy, hz, dEz_y, dEx_y, dEz_x, dEy_x, dEy_z, dEx_z,
                                     BATCH ? dp.bH : s_xbc[0], BATCH ? dp.cH : s_xbc[1]);
          }
        } else {
          hx = C.hhx * hx + C.hex * (-dEz_y + dEy_z);
          hy = C.hhy * hy + C.hey * (-dEx_z + dEz_x);
          hz = C.hhz * hz + C.hez * (-dEy_x + dEx_y);
          if (PML && act) {
            if (ax[c]) {
              if (px >= 0) {
                float2 *X = psi_at_x(dp, PSI_HX, px, j, k);
                const float xb = BATCH ? dp.bH[px] : s_xbc[0][px];
                const float xc = BATCH ? dp.cH[px] : s_xbc[1][px];
                h_corr_x_bc(dp, xb, xc, *X, X, dEz_x, dEy_x, hy, hz, C.hey, C.hez);
              }
            } else if (ay) {
              float2 *Y = psi_at_y(dp, PSI_HY, i, py[c], k);
              h_corr_y(dp, py[c], *Y, Y, dEz_y, dEx_y, hx, hz, C.hex, C.hez);
            } else if (az) {
              float2 *Z = psi_at_z(dp, PSI_HZ, i, j, pz);
              h_corr_z(dp, pz, *Z, Z, dEy_z, dEx_z, hx, hy, C.hex, C.hey);
            }
          }
        }
        if (act) {
          dp.f[3][n0[c] + off] = hx;
          dp.f[4][n0[c] + off] = hy;
          dp.f[5][n0[c] + off] = hz;
        }
      }
      if (xc_plane) {
        // CPML X of the warp's x-slab cells, one per lane (H cells: j <= J-2)
        __syncwarp();
        const int nrow = (int)valid_row[0] + (int)valid_row[1];
        for (int u = lane; u < xr.n * nrow; u += 32) {
          const int c = valid_row[0] ? u / xr.n : 1;
          const int xl = x_run_lane(xr, u % xr.n);
          const int ty = r0 + (G::BY / 2) * c;
          const int tcol = xo - lane + xl;
          const int ix = x0 + tcol, j = y0 + ty;
          const int eb = ty * G::HW + tcol, hb = ty * G::BX + tcol;
          const int pxx = slab_h(ix, I, p);
          const int64_t n = ix + (int64_t)j * dp.Ip + (int64_t)k * dp.plane;
          float hy = sHy[hb], hz = sHz[hb];
          float2 *X = psi_at_x(dp, PSI_HX, pxx, j, k);
          const float xb = BATCH ? dp.bH[pxx] : s_xbc[0][pxx];
          const float xc = BATCH ? dp.cH[pxx] : s_xbc[1][pxx];
          h_corr_x_bc(dp, xb, xc, *X, X, sEz[eb + 1] - sEz[eb], sEy[eb + 1] - sEy[eb], hy, hz,
                      Che, Che);
          dp.f[4][n] = hy;
          dp.f[5][n] = hz;
        }
        stage_writes_fence();
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[s]);
    }
  }
}

// Item height: >= 4 items per resident block (dynamic balance), <= 32 planes.
inline int pick_zchunk(int tiles, int nk, int blocks) {
  static int forced = -1;
  if (forced < 0) {
    const char *e = getenv("FDTD_TMA_ZCHUNK");
    forced = e ? atoi(e) : 0;
  }
  if (forced > 0) return forced;
  const long long want = 4LL * blocks;
  long long chunks = (want + tiles - 1) / tiles;
  if (chunks < 1) chunks = 1;
  if (chunks > nk) chunks = nk;
  int z = (int)((nk + chunks - 1) / chunks);
  if (z < 2) z = 2;
  if (z > 32) z = 32;
  return z;
}

template <class G = GS, class KH>
int launch(KH kern, int smem, int *cached_blocks, const fdtd_dev *d, const fdtd_maps *m,
           const fdtd_op *op, cudaStream_t s, int ni, int nj, int nk, int zc_tuned) {
  static_assert(sizeof(Maps) == sizeof(((fdtd_maps *)0)->bytes), "map layout");
  if (!d->work) return (int)cudaErrorInvalidValue;
  if (*cached_blocks <= 0) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return (int)e;
    int per_sm = 0, sms = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, NT, smem);
    if (e != cudaSuccess) return (int)e;
    *cached_blocks = (per_sm > 0 ? per_sm : 1) * (sms > 0 ? sms : 1);
  }
  Maps mp;
  memcpy(&mp, m->bytes, sizeof(Maps));
  Items it;
  memset(&it, 0, sizeof(it));
  it.work = d->work;
  it.err = d->err;
  it.tiles_x = (ni + G::BX - 1) / G::BX;
  it.tiles_y = (nj + G::BY - 1) / G::BY;
  it.nk = nk;
  it.zchunk = pick_zchunk(it.tiles_x * it.tiles_y, nk, *cached_blocks);
  if (zc_tuned > 0 && !getenv("FDTD_TMA_ZCHUNK")) it.zchunk = zc_tuned < nk ? zc_tuned : nk;
  it.n_items = it.tiles_x * it.tiles_y * ((nk + it.zchunk - 1) / it.zchunk);
  const int blocks = it.n_items < *cached_blocks ? it.n_items : *cached_blocks;
  kern<<<blocks, NT, smem, s>>>(*d, *op, mp, it);
  fdtdk_count_launches(1);
  return (int)cudaGetLastError();
}

int g_blocks_e[5] = {0, 0, 0, 0, 0}, g_blocks_h[7] = {0, 0, 0, 0, 0, 0, 0};
int g_blocks_b[6] = {0, 0, 0, 0, 0, 0};

// The compacted CPML X kernels (XC) when FDTD_XC=1; by default the lean
// kernels without it, with E's CPML X as the x-slab pass.  Both give the
// same results.  Measured on GB300: XC is slower on the 256^3, 512x512x448
// and batched workloads (512x512x448 E half-step 0.833 vs 0.800 ms; 256
// grids of 32..128 cells a side 82.4 vs 88.4 solves/s): the warp that takes
// the x-slab cells waits on their psi loads while the stage it holds keeps
// the ring from advancing, where the separate pass has every thread of the
// GPU in flight.
bool use_xc() {
  static int v = -1;
  if (v < 0) {
    const char *e = getenv("FDTD_XC");
    v = e && strcmp(e, "1") == 0;
  }
  return v != 0;
}

// Resident blocks of a kernel on the current device (cached per kernel).
template <class KH>
int resident_blocks(KH kern, int smem, int *cached) {
  if (*cached > 0) return 0;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return (int)e;
  int per_sm = 0, sms = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, NT, smem);
  if (e != cudaSuccess) return (int)e;
  *cached = (per_sm > 0 ? per_sm : 1) * (sms > 0 ? sms : 1);
  return 0;
}

template <class G>
int make_maps(const fdtd_dev *d, fdtd_maps *m) {
  constexpr int BX = G::BX, BY = G::BY, HW = G::HW, HH = G::HH;
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


// The single-grid CPML curl kernels in the tile geometry T (maps: one set
// per geometry; blocks per SM cached per instance).
template <bool LEAN, int T>
int launch_e_pml(const fdtd_dev *d, const fdtd_maps *m, const fdtd_op *o, cudaStream_t s) {
  using G = TileGeo<T>;
  static int blocks = 0;
  return launch<G>(k_half_e_tma<true, false, LEAN, false, G>, EG<false, G>::SMEM, &blocks, d,
                   &m[T], o, s, d->I, d->J, d->K, d->zc_e);
}
template <bool LEAN, int T>
int launch_h_pml(const fdtd_dev *d, const fdtd_maps *m, const fdtd_op *o, cudaStream_t s) {
  using G = TileGeo<T>;
  static int blocks = 0;
  return launch<G>(k_half_h_tma<true, false, false, LEAN, false, G>, HG<false, G>::SMEM, &blocks,
                   d, &m[T], o, s, d->I - 1, d->J - 1, d->K - 1, d->zc_h);
}
// The tile the autotuner chose (when its maps encoded), else 64 x 8.
inline int tile_of(int t, const fdtd_maps *m) {
  return (t >= 0 && t < FDTD_NUM_TILES && m[t].valid) ? t : 0;
}
template <bool LEAN>
int launch_e_tiled(const fdtd_dev *d, const fdtd_maps *m, const fdtd_op *o, cudaStream_t s) {
  switch (tile_of(d->tile_e, m)) {
    case 1: return launch_e_pml<LEAN, 1>(d, m, o, s);
    case 2: return launch_e_pml<LEAN, 2>(d, m, o, s);
    default: return launch_e_pml<LEAN, 0>(d, m, o, s);
  }
}
template <bool LEAN>
int launch_h_tiled(const fdtd_dev *d, const fdtd_maps *m, const fdtd_op *o, cudaStream_t s) {
  switch (tile_of(d->tile_h, m)) {
    case 1: return launch_h_pml<LEAN, 1>(d, m, o, s);
    case 2: return launch_h_pml<LEAN, 2>(d, m, o, s);
    default: return launch_h_pml<LEAN, 0>(d, m, o, s);
  }
}

}  // namespace

extern "C" {

int fdtdk_make_maps(const fdtd_dev *d, int tile, fdtd_maps *m) {
  switch (tile) {
    case 0: return make_maps<GS>(d, m);
    case 1: return make_maps<GB>(d, m);
    case 2: return make_maps<GW>(d, m);
  }
  m->valid = 0;
  return (int)cudaErrorInvalidValue;
}

// The curl kernel, then the x-slab pass (CPML X, when it can be split off)
// and the face pass (TF/SF, when it can): their cells are disjoint.  m: the
// maps of every tile geometry (FDTD_NUM_TILES).
int fdtdk_half_e_tma(const fdtd_dev *d, const fdtd_maps *m, const fdtd_op *op, cudaStream_t s) {
  fdtd_op o = *op;
  o.tfsf_split = fdtd_tfsf_split(d, op);
  o.xsplit = fdtd_xsplit(d, op);
  const int I = d->I, J = d->J, K = d->K;
  int e;
  bool xslab_pass = o.xsplit;
  if (fdtd_e_lean(&o) && o.pml && use_xc()) {
    e = launch(k_half_e_tma<true, false, true, true>, E_SMEM, &g_blocks_e[4], d, m, &o, s, I, J,
               K, d->zc_e);
    xslab_pass = false;  // the kernel applied CPML X
  } else if (fdtd_e_lean(&o))
    e = o.pml ? launch_e_tiled<true>(d, m, &o, s)
              : launch(k_half_e_tma<false, false, true>, E_SMEM, &g_blocks_e[2], d, m, &o, s, I,
                       J, K, d->zc_e);
  else
    e = o.pml ? launch_e_tiled<false>(d, m, &o, s)
              : launch(k_half_e_tma<false, false>, E_SMEM, &g_blocks_e[0], d, m, &o, s, I, J, K,
                       d->zc_e);
  if (!e) fdtdk_profile_mark(s);
  if (!e && xslab_pass) e = fdtdk_e_xslab(d, s);
  if (e || !o.tfsf_split) return e;
  return fdtdk_faces(0, d, &o, s);
}

int fdtdk_half_h_tma(const fdtd_dev *d, const fdtd_maps *m, const fdtd_op *op, cudaStream_t s) {
  fdtd_op o = *op;
  o.tfsf_split = fdtd_tfsf_split(d, op);
  const int ni = d->I - 1, nj = d->J - 1, nk = d->K - 1;
  int e;
  if (d->hcoef_mode)  // per-cell H coefficients
    e = o.pml ? launch(k_half_h_tma<true, false, true>, H_SMEM, &g_blocks_h[3], d, m, &o, s, ni,
                       nj, nk, d->zc_h)
              : launch(k_half_h_tma<false, false, true>, H_SMEM, &g_blocks_h[2], d, m, &o, s,
                       ni, nj, nk, d->zc_h);
  else if (fdtd_h_lean(&o) && o.pml && use_xc())
    e = launch(k_half_h_tma<true, false, false, true, true>, H_SMEM, &g_blocks_h[6], d, m, &o, s,
               ni, nj, nk, d->zc_h);
  else if (fdtd_h_lean(&o))
    e = o.pml ? launch_h_tiled<true>(d, m, &o, s)
              : launch(k_half_h_tma<false, false, false, true>, H_SMEM, &g_blocks_h[4], d, m, &o,
                       s, ni, nj, nk, d->zc_h);
  else
    e = o.pml ? launch_h_tiled<false>(d, m, &o, s)
              : launch(k_half_h_tma<false, false>, H_SMEM, &g_blocks_h[0], d, m, &o, s, ni, nj,
                       nk, d->zc_h);
  if (!e) fdtdk_profile_mark(s);
  if (e || !o.tfsf_split) return e;
  return fdtdk_faces(1, d, &o, s);
}

int fdtdk_batch_half(int hfam, int lean, const fdtd_dev *devs, const void *maps,
                     const fdtd_op *ops, const int32_t *steps, const int32_t *table,
                     int32_t n_items, int32_t *work, int32_t *err, cudaStream_t s) {
  if (n_items <= 0) return 0;
  Items it;
  memset(&it, 0, sizeof(it));
  it.n_items = n_items;
  it.work = work;
  it.err = err;
  it.table = reinterpret_cast<const int4 *>(table);
  it.devs = devs;
  it.maps = static_cast<const CUtensorMap *>(maps);
  it.ops = ops;
  it.steps = steps;
  // the single-grid parameters are unused in batch mode
  static fdtd_dev d0;
  static fdtd_op op0;
  static Maps mp0;
  int e;
  if (hfam && lean && use_xc()) {
    e = resident_blocks(k_half_h_tma<true, true, false, true, true>, HG<true>::SMEM,
                        &g_blocks_b[4]);
    if (e) return e;
    const int blocks = n_items < g_blocks_b[4] ? n_items : g_blocks_b[4];
    k_half_h_tma<true, true, false, true, true><<<blocks, NT, HG<true>::SMEM, s>>>(d0, op0, mp0,
                                                                                  it);
  } else if (hfam && lean) {
    e = resident_blocks(k_half_h_tma<true, true, false, true>, HG<true>::SMEM, &g_blocks_b[3]);
    if (e) return e;
    const int blocks = n_items < g_blocks_b[3] ? n_items : g_blocks_b[3];
    k_half_h_tma<true, true, false, true><<<blocks, NT, HG<true>::SMEM, s>>>(d0, op0, mp0, it);
  } else if (hfam) {
    e = resident_blocks(k_half_h_tma<true, true>, HG<true>::SMEM, &g_blocks_b[0]);
    if (e) return e;
    const int blocks = n_items < g_blocks_b[0] ? n_items : g_blocks_b[0];
    k_half_h_tma<true, true><<<blocks, NT, HG<true>::SMEM, s>>>(d0, op0, mp0, it);
  } else if (lean && use_xc()) {
    e = resident_blocks(k_half_e_tma<true, true, true, true>, EG<true>::SMEM, &g_blocks_b[5]);
    if (e) return e;
    const int blocks = n_items < g_blocks_b[5] ? n_items : g_blocks_b[5];
    k_half_e_tma<true, true, true, true><<<blocks, NT, EG<true>::SMEM, s>>>(d0, op0, mp0, it);
  } else if (lean) {
    e = resident_blocks(k_half_e_tma<true, true, true>, EG<true>::SMEM, &g_blocks_b[2]);
    if (e) return e;
    const int blocks = n_items < g_blocks_b[2] ? n_items : g_blocks_b[2];
    k_half_e_tma<true, true, true><<<blocks, NT, EG<true>::SMEM, s>>>(d0, op0, mp0, it);
  } else {
    e = resident_blocks(k_half_e_tma<true, true>, EG<true>::SMEM, &g_blocks_b[1]);
    if (e) return e;
    const int blocks = n_items < g_blocks_b[1] ? n_items : g_blocks_b[1];
    k_half_e_tma<true, true><<<blocks, NT, EG<true>::SMEM, s>>>(d0, op0, mp0, it);
  }
  fdtdk_count_launches(1);
  return (int)cudaGetLastError();
}

}  // extern "C"

extern "C" int fdtdk_check_wait(int arrive, long long out[2]) {
  long long *d = nullptr;
  cudaError_t e = cudaMalloc((void **)&d, 2 * sizeof(long long));
  if (e != cudaSuccess) return (int)e;
  e = cudaMemset(d, 0, 2 * sizeof(long long));
  if (e == cudaSuccess) {
    k_check_wait<<<1, 32>>>(d, arrive);
    fdtdk_count_launches(1);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(out, d, 2 * sizeof(long long), cudaMemcpyDeviceToHost);
  cudaFree(d);
  return (int)e;
}

extern "C" unsigned long long fdtdk_wait_ns(void) { return kWaitNs; }
extern "C" int fdtdk_batch_e_applies_x(int lean) { return lean && use_xc(); }
extern "C" unsigned long long fdtdk_check_ns(void) { return kCheckNs; }
