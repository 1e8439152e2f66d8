/*
 * fdtd_fused.cu -- one whole FDTD step (the H half-step, then the E
 * half-step) in one persistent, warp-specialised TMA pass over a single
 * grid, for sm_103a.
 *
 * The two half-step kernels of fdtd_tma.cu each stream the six fields
 * through the GPU once per step: H reads 3 E + 3 H and writes 3 H, then E
 * reads 3 E + 3 H (+ material ids) and writes 3 E -- 74 compulsory bytes a
 * cell.  Here each work item (a 32 x 16 tile, a run of z-planes) computes
 * the new H of a plane and, from it, the new E of the same plane while both
 * are in shared memory: 3 E + 3 H + ids read, 3 E + 3 H written, 50 bytes
 * a cell.
 *
 * Two buffers.  The step reads the fields from one buffer ("old", through
 * TMA) and writes every cell of the other ("new").  A tile needs the new H
 * of its x-1 column and y-1 row, which belong to its neighbours: it
 * recomputes them from the old fields (and the old H psi pairs) instead of
 * waiting for them, so no item ever waits for another, and reading only the
 * old buffer makes that race-free.  The H psi pairs are double-buffered the
 * same way (old read, new written by the owner); the E psi pairs are only
 * touched by the owner of their cell and stay in place.  Steps go in pairs
 * (old -> new -> old), so between pairs the handle's fields are where they
 * always are.
 *
 * What stays outside the pass, in the reference's order per cell:
 *   - TF/SF.  The face cells are at least three cells inside the CPML, so
 *     each gets curl then TF/SF only; the H face pass corrects the new H
 *     after the pass, the E cells whose curl read a corrected H cell (the
 *     planes on both sides of each H face plane) are recomputed from the
 *     old E and the corrected new H (k_fix_e), then the E face pass runs.
 *   - CPML X of E, the last operation of an x-slab cell: the x-slab pass.
 *   - the probe gather, at the start of each step.
 * Every arithmetic operation is the reference's, in its order, rounded
 * separately (fdtd_device.cuh), so the result equals the two half-step
 * kernels', the oracle's and the reference's bit for bit.
 *
 * Per plane h of an item the consumers hold the stages of planes h and h+1
 * (the z differences of H reach up one plane): new H of plane h for the
 * tile and its x-1 / y-1 halo into a shared exchange buffer, a block-wide
 * bounded mbarrier sync, then new E of plane h, with the new H of plane h-1
 * carried in registers.  An item of np planes streams np + 2 planes (the
 * plane below, for that carried H, and the plane above).
 */
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "fdtd_device.cuh"
#include "fdtd_internal.h"
#include "fdtd_pipe.cuh"

using namespace fdtd;
using namespace fdtd_pipe;

extern "C" void fdtdk_count_launches(unsigned long long n);

namespace {

constexpr int NCW = 8;                   // consumer warps
constexpr int NT = (NCW + 1) * 32;       // + one producer warp
constexpr int BX = 32, BY = 16;          // tile: warp w owns rows w and w + 8
constexpr int EW = BX + 8, EH = BY + 2;  // old-E box: x0-4 .. x0+BX+3, y0-1 .. y0+BY
constexpr int HW = BX + 4, HH = BY + 1;  // old-H box: x0-4 .. x0+BX-1, y0-1 .. y0+BY-1
constexpr int E_BOX = EW * EH * 4;
constexpr int H_BOX = HW * HH * 4;
constexpr int E_SLOT = (E_BOX + 127) / 128 * 128;
constexpr int H_SLOT = (H_BOX + 127) / 128 * 128;
constexpr int M_BOX = BX * BY * 2;
constexpr int OFF_H = 3 * E_SLOT;
constexpr int OFF_M = OFF_H + 3 * H_SLOT;
constexpr int STAGE = OFF_M + M_BOX;
// exchange of a plane's new H: column 0 = x0-1, row 0 = y0-1
constexpr int XW = BX + 1, XH = BY + 1;
constexpr int XPLANE = XW * XH;                    // floats per component
constexpr int XB_B = (3 * XPLANE * 4 + 127) / 128 * 128;
constexpr int CTRL_B = 512;
#ifndef FDTD_FUSED_TAB
#define FDTD_FUSED_TAB 256
#endif
constexpr int kTabMax = FDTD_FUSED_TAB;  // coefficient ids staged in shared memory
#ifndef FDTD_FUSED_NS
#define FDTD_FUSED_NS 3
#endif
#ifndef FDTD_FUSED_MIN_BLOCKS
#define FDTD_FUSED_MIN_BLOCKS 3
#endif
constexpr int NS = FDTD_FUSED_NS;
constexpr int SMEM = NS * STAGE + 2 * XB_B + CTRL_B + kTabMax * 6 * 4;
static_assert(STAGE % 128 == 0 && E_SLOT % 128 == 0 && H_SLOT % 128 == 0, "stage alignment");
static_assert(NS * (8 + 8 + 32) + 2 * 8 <= CTRL_B, "control block");
static_assert((EW * 4) % 16 == 0 && (HW * 4) % 16 == 0 && (BX * 2) % 16 == 0,
              "TMA inner box extents must be multiples of 16 bytes");
static_assert(FDTD_FUSED_MIN_BLOCKS * (SMEM + 1024) <= 228 * 1024, "blocks per SM");

struct FusedParams {
  CUtensorMap m[FDTD_FUSED_MAPS];  // old Ex Ey Ez (E box), old Hx Hy Hz (H box), ids
  const float *psi_h_old[3];       // PSI_HY, PSI_HX, PSI_HZ pairs of the old buffer
  int tiles_x, tiles_y, zchunk, n_items;
  int32_t *work;                   // [0] next item, [1] finished producers
  int32_t *err;                    // device error word
};

// One CPML axis of a new H from the old psi pair (gpu.h:644-685 Y, :604-642 X,
// :687-725 Z): the same expressions as h_corr_y / h_corr_x_bc / h_corr_z,
// returning the new pair so that only the owner stores it.
__device__ __forceinline__ float2 hc_y(const fdtd_dev &d, float b, float c, float2 ps,
                                       float dEz_y, float dEx_y, float &hx, float &hz) {
  const float dx = d.dx, che = d.Che;
  const float v0 = b * ps.x + div_dx(d, c * dEz_y);
  hx = hx - che * v0 * dx;
  const float v1 = b * ps.y + div_dx(d, c * dEx_y);
  hz = hz + che * v1 * dx;
  return make_float2(v0, v1);
}
__device__ __forceinline__ float2 hc_x(const fdtd_dev &d, float b, float c, float2 ps,
                                       float dEz_x, float dEy_x, float &hy, float &hz) {
  const float dx = d.dx, che = d.Che;
  const float v0 = b * ps.x + div_dx(d, c * dEz_x);
  hy = hy + che * v0 * dx;
  const float v1 = b * ps.y + div_dx(d, c * dEy_x);
  hz = hz - che * v1 * dx;
  return make_float2(v0, v1);
}
__device__ __forceinline__ float2 hc_z(const fdtd_dev &d, float b, float c, float2 ps,
                                       float dEy_z, float dEx_z, float &hx, float &hy) {
  const float dx = d.dx, che = d.Che;
  const float v0 = b * ps.x + div_dx(d, c * dEy_z);
  hx = hx + che * v0 * dx;
  const float v1 = b * ps.y + div_dx(d, c * dEx_z);
  hy = hy - che * v1 * dx;
  return make_float2(v0, v1);
}

// Views of one ring stage.
struct StageView {
  const float *ex, *ey, *ez, *hx, *hy, *hz;
  const uint16_t *mat;
  __device__ __forceinline__ explicit StageView(const unsigned char *st)
      : ex(reinterpret_cast<const float *>(st)),
        ey(reinterpret_cast<const float *>(st + E_SLOT)),
        ez(reinterpret_cast<const float *>(st + 2 * E_SLOT)),
        hx(reinterpret_cast<const float *>(st + OFF_H)),
        hy(reinterpret_cast<const float *>(st + OFF_H + H_SLOT)),
        hz(reinterpret_cast<const float *>(st + OFF_H + 2 * H_SLOT)),
        mat(reinterpret_cast<const uint16_t *>(st + OFF_M)) {}
};

// New H of the cell at tile position (tx, ty) (tx in [-1, BX), ty in [-1, BY))
// of plane h: a from the stage of plane h, b from the stage of plane h + 1.
// Cells the reference does not update (i = I-1, j = J-1, h = K-1, or outside
// the grid) keep their old H.  The old psi pairs are read; when `own`, the
// new ones are stored.  Every lane of the warp calls it (the path vote).
__device__ __forceinline__ void new_h(const fdtd_dev &d, const FusedParams &fp,
                                      const StageView &a, const StageView &b, int x0, int y0,
                                      int tx, int ty, int h, bool own, const float *xb,
                                      const float *xc, const float *yb, const float *yc,
                                      float &hx, float &hy, float &hz) {
  const int I = d.I, J = d.J, K = d.K, p = d.p;
  const int i = x0 + tx, j = y0 + ty;
  const int e = (ty + 1) * EW + tx + 4, hb = (ty + 1) * HW + tx + 4;
  const float ex = a.ex[e], ey = a.ey[e], ez = a.ez[e];
  const float dEz_y = a.ez[e + EW] - ez, dEx_y = a.ex[e + EW] - ex;
  const float dEz_x = a.ez[e + 1] - ez, dEy_x = a.ey[e + 1] - ey;
  const float dEy_z = b.ey[e] - ey, dEx_z = b.ex[e] - ex;
  hx = a.hx[hb];
  hy = a.hy[hb];
  hz = a.hz[hb];
  const bool valid = i >= 0 && j >= 0 && i < I - 1 && j < J - 1 && h < K - 1;
  const int px = valid ? slab_h(i, I, p) : -1, py = valid ? slab_h(j, J, p) : -1;
  const int pz = valid ? slab_h(h, K, p) : -1;
  const float Chh = d.Chh, Che = d.Che;
  if (valid) {  // curl (gpu.h:575-602)
    hx = Chh * hx + Che * (-dEz_y + dEy_z);
    hy = Chh * hy + Che * (-dEx_z + dEz_x);
    hz = Chh * hz + Che * (-dEy_x + dEx_y);
  }
  if (__any_sync(0xffffffffu, px >= 0 || py >= 0 || pz >= 0)) {
    // CPML Y, X, Z (the reference's launch order); all pairs loaded first
    const int64_t Il = I, Jl = J, pj = 2 * (int64_t)p;
    const int64_t iy = i + py * Il + h * pj * Il, ix = px + j * pj + h * pj * Jl;
    const int64_t iz = i + j * Il + pz * d.IJ;
    float2 sy = make_float2(0.f, 0.f), sx = sy, sz = sy;
    if (py >= 0) sy = reinterpret_cast<const float2 *>(fp.psi_h_old[0])[iy];
    if (px >= 0) sx = reinterpret_cast<const float2 *>(fp.psi_h_old[1])[ix];
    if (pz >= 0) sz = reinterpret_cast<const float2 *>(fp.psi_h_old[2])[iz];
    if (py >= 0) {
      const float2 v = hc_y(d, yb[py], yc[py], sy, dEz_y, dEx_y, hx, hz);
      if (own) psi_pairs(d, PSI_HY)[iy] = v;
    }
    if (px >= 0) {
      const float2 v = hc_x(d, xb[px], xc[px], sx, dEz_x, dEy_x, hy, hz);
      if (own) psi_pairs(d, PSI_HX)[ix] = v;
    }
    if (pz >= 0) {
      const float2 v = hc_z(d, d.bH[pz], d.cH[pz], sz, dEy_z, dEx_z, hx, hy);
      if (own) psi_pairs(d, PSI_HZ)[iz] = v;
    }
  }
}

__global__ void __launch_bounds__(NT, FDTD_FUSED_MIN_BLOCKS)
    k_step_fused(const __grid_constant__ fdtd_dev d, const __grid_constant__ FusedParams fp) {
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t *full = reinterpret_cast<uint64_t *>(smem + NS * STAGE);
  uint64_t *empty = full + NS;
  int4 *meta = reinterpret_cast<int4 *>(empty + NS);
  uint64_t *xsync = reinterpret_cast<uint64_t *>(meta + 2 * NS);
  float *xbuf = reinterpret_cast<float *>(smem + NS * STAGE + CTRL_B);
  float *stab = reinterpret_cast<float *>(smem + NS * STAGE + CTRL_B + 2 * XB_B);
  // the H grading tables (read per lane by slab position) and the E table
  __shared__ float s_bc[2][2 * FDTD_MAX_PML];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const bool use_mat = d.coef_mode == 1;
  const bool tab_local = use_mat && d.n_mat <= kTabMax;
  for (int t = tid; t < 2 * FDTD_MAX_PML; t += NT) {
    s_bc[0][t] = d.bH[t];
    s_bc[1][t] = d.cH[t];
  }
  if (tab_local)
    for (int t = tid; t < d.n_mat * 6; t += NT) stab[t] = __ldg(d.mat_tab + t);
  if (tid == 0) {
    for (int s = 0; s < NS; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], NCW);
    }
    mbar_init(&xsync[0], NCW);
    mbar_init(&xsync[1], NCW);
    mbar_init_fence();
  }
  __syncthreads();
  const int K = d.K;

  if (warp == NCW) {  // ------------------------------------------ producer
    if (lane != 0) return;
    const int nt = fp.tiles_x * fp.tiles_y;
    int q = 0;
    bool ok = true;
    for (;;) {
      const int w = atomicAdd(&fp.work[0], 1);
      if (w >= fp.n_items) break;
      const int chunk = w / nt, tile = w - chunk * nt;
      const int x0 = (tile % fp.tiles_x) * BX, y0 = (tile / fp.tiles_x) * BY;
      const int kb = chunk * fp.zchunk;
      const int np = min(fp.zchunk, K - kb);
      for (int t = 0; t < np + 2 && ok; ++t, ++q) {
        const int s = q % NS;
        if (q >= NS) ok = mbar_wait(&empty[s], (uint32_t)(((q / NS) - 1) & 1));
        if (!ok) break;
        meta[2 * s] = make_int4(w, t, np, kb);
        meta[2 * s + 1] = make_int4(x0, y0, 0, 0);
        const int k = kb - 1 + t;
        // the plane above the item: Ex, Ey only (z differences of its top H);
        // the plane below: no ids (its E is not computed)
        const bool top = t == np + 1, bottom = t == 0;
        const uint32_t bytes = (top ? 2u : 3u) * E_BOX + (top ? 0u : 3u * H_BOX) +
                               ((top || bottom || !use_mat) ? 0u : (uint32_t)M_BOX);
        unsigned char *st = smem + s * STAGE;
        proxy_fence();
        mbar_expect_tx(&full[s], bytes);
        for (int c = 0; c < (top ? 2 : 3); ++c)
          tma_load_3d(st + c * E_SLOT, &fp.m[c], &full[s], x0 - 4, y0 - 1, k);
        if (!top)
          for (int c = 0; c < 3; ++c)
            tma_load_3d(st + OFF_H + c * H_SLOT, &fp.m[3 + c], &full[s], x0 - 4, y0 - 1, k);
        if (!top && !bottom && use_mat) tma_load_3d(st + OFF_M, &fp.m[6], &full[s], x0, y0, k);
      }
      if (!ok) break;
    }
    if (atomicAdd(&fp.work[1], 1) == (int)gridDim.x - 1) {  // last producer: rewind
      atomicExch(&fp.work[0], 0);
      atomicExch(&fp.work[1], 0);
    }
    if (ok) {  // sentinel
      const int s = q % NS;
      if (q >= NS) ok = mbar_wait(&empty[s], (uint32_t)(((q / NS) - 1) & 1));
      if (ok) {
        meta[2 * s] = make_int4(-1, 0, 0, 0);
        mbar_arrive(&full[s]);
        ++q;
      }
    }
    if (!ok && fp.err) atomicExch(fp.err, 4);
    for (int r = (q > NS ? q - NS : 0); r < q; ++r)
      mbar_wait(&full[r % NS], (uint32_t)((r / NS) & 1));
    return;
  }

  // ------------------------------------------------------------- consumers
  const int I = d.I, J = d.J;
  int q = 0, nsync = 0;
  for (;;) {
    int s = q % NS;
    if (!mbar_wait(&full[s], (uint32_t)((q / NS) & 1))) {
      if (fp.err) atomicExch(fp.err, 5);
      return;
    }
    const int4 m = meta[2 * s];
    if (m.x < 0) return;  // sentinel
    const int4 m1 = meta[2 * s + 1];
    const int kb = m.w, np = m.z, x0 = m1.x, y0 = m1.y;
    const int i = x0 + lane;
    float hxm[2] = {0.f, 0.f}, hym[2] = {0.f, 0.f};  // new Hx, Hy of plane h-1
    int sp = s;
    ++q;
    for (int t = 1; t <= np + 1; ++t, ++q) {
      s = q % NS;
      if (!mbar_wait(&full[s], (uint32_t)((q / NS) & 1))) {
        if (fp.err) atomicExch(fp.err, 5);
        return;
      }
      const int h = kb + t - 2;  // the plane of the previous stage
      const bool own = h >= kb;
      const StageView a(smem + sp * STAGE), b(smem + s * STAGE);
      float *X0 = xbuf + (nsync & 1) * (XB_B / 4);
      float *X1 = X0 + XPLANE, *X2 = X1 + XPLANE;
      float nhx[2] = {0.f, 0.f}, nhy[2] = {0.f, 0.f};
      if (h >= 0) {
#pragma unroll
        for (int c = 0; c < 2; ++c) {
          const int ty = warp + (BY / 2) * c;
          float hx, hy, hz;
          new_h(d, fp, a, b, x0, y0, lane, ty, h, own, s_bc[0], s_bc[1], d.bH, d.cH, hx, hy,
                hz);
          nhx[c] = hx;
          nhy[c] = hy;
          if (own) {
            const int xi = (ty + 1) * XW + lane + 1;
            X0[xi] = hx;
            X1[xi] = hy;
            X2[xi] = hz;
            const int j = y0 + ty;
            if (i < I && j < J) {
              const int64_t n = i + (int64_t)j * d.Ip + (int64_t)h * d.plane;
              d.f[3][n] = hx;
              d.f[4][n] = hy;
              d.f[5][n] = hz;
            }
          }
        }
        // the halo: warp 0 the y0-1 row, warp 1 the x0-1 column (recomputed,
        // not stored: they belong to the neighbouring tiles)
        if (own && warp < 2) {
          const int tx = warp == 0 ? lane : -1, ty = warp == 0 ? -1 : (lane < BY ? lane : BY - 1);
          float hx, hy, hz;
          new_h(d, fp, a, b, x0, y0, tx, ty, h, false, s_bc[0], s_bc[1], s_bc[0], s_bc[1], hx,
                hy, hz);
          const int xi = (ty + 1) * XW + tx + 1;
          if (warp == 0 || lane < BY) {
            X0[xi] = hx;
            X1[xi] = hy;
            X2[xi] = hz;
          }
        }
      }
      if (own) {
        // every warp's new H of plane h is in the exchange buffer
        __syncwarp();
        if (lane == 0) mbar_arrive(&xsync[nsync & 1]);
        if (!mbar_wait(&xsync[nsync & 1], (uint32_t)((nsync >> 1) & 1))) {
          if (fp.err) atomicExch(fp.err, 6);
          return;
        }
        ++nsync;
        // new E of plane h (gpu.h:727-763; CPML Y, Z :790-868; X in the
        // x-slab pass)
#pragma unroll
        for (int c = 0; c < 2; ++c) {
          const int ty = warp + (BY / 2) * c;
          const int j = y0 + ty;
          const bool act = i < I && j < J;
          const int e = (ty + 1) * EW + lane + 4, xi = (ty + 1) * XW + lane + 1;
          float ex = a.ex[e], ey = a.ey[e], ez = a.ez[e];
          const float hx = X0[xi], hy = X1[xi], hz = X2[xi];
          const float hz_jm = X2[xi - XW], hx_jm = X0[xi - XW];
          const float hz_im = X2[xi - 1], hy_im = X1[xi - 1];
          Coef6 C = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
          const int64_t n = act ? i + (int64_t)j * d.Ip + (int64_t)h * d.plane : 0;
          if (use_mat) {
            const int mi = a.mat[ty * BX + lane];
            if (tab_local) {
              const float *r = stab + mi * 6;
              C.exe = r[0]; C.eye = r[1]; C.eze = r[2]; C.exh = r[3]; C.eyh = r[4]; C.ezh = r[5];
            } else {
              C = coef_from_table(d, mi);
            }
          } else if (act) {
            C = coef_from_arrays(d, n);
          }
          int px = -1, py = -1, pz = -1;
          e_slabs(d, i, j, h, px, py, pz);
          const bool special = act && (i == 0 || j == 0 || h == 0 || py >= 0 || pz >= 0);
          if (__any_sync(0xffffffffu, special)) {
            if (act)
              update_e_cell<true, true>(d, 0, nullptr, 0, 0.f, false, i, j, h, -1, py, pz, C, ex,
                                        ey, ez, hx, hy, hz, hz_jm, hx_jm, hz_im, hy_im, hxm[c],
                                        hym[c]);
          } else {
            ex = C.exe * ex + C.exh * (+(hz - hz_jm) - (hy - hym[c]));
            ey = C.eye * ey + C.eyh * (+(hx - hxm[c]) - (hz - hz_im));
            ez = C.eze * ez + C.ezh * (+(hy - hy_im) - (hx - hx_jm));
          }
          if (act) {
            d.f[0][n] = ex;
            d.f[1][n] = ey;
            d.f[2][n] = ez;
          }
        }
      }
      hxm[0] = nhx[0];
      hxm[1] = nhx[1];
      hym[0] = nhy[0];
      hym[1] = nhy[1];
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[sp]);  // the stage of plane h
      sp = s;
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[sp]);  // the plane above the item
  }
}

// The E cells whose curl reads an H cell that the H face pass corrected:
// for each axis a whose faces the mode corrects H on, the planes on both
// sides of its two H face planes (a0-1, a0 and a1, a1+1), over the box's
// extent +-2 in the other two axes.  Each is recomputed from the old E and
// the corrected new H -- curl only (with the reference's guards): the cells
// are outside every CPML slab and the current source (fdtd_fused_ok).
// Overlapping regions give identical values.
__global__ void k_fix_e(const __grid_constant__ fdtd_dev d, const float *eox, const float *eoy,
                        const float *eoz, int axes) {
  const int r = blockIdx.y;  // 4 planes per axis in `axes` (bit a: axis a)
  int axis = 0;
  for (int n = r >> 2; n >= 0; ++axis)
    if ((axes >> axis) & 1) --n;
  --axis;
  const int which = r & 3;
  const int lo[3] = {d.i0, d.j0, d.k0}, hi[3] = {d.i1, d.j1, d.k1};
  // u: the faster-varying of the other two axes (x before y before z), so
  // that consecutive threads touch consecutive cells on y and z planes
  const int u = axis == 0 ? 1 : 0, v = axis == 2 ? 1 : 2;
  const int plane = which < 2 ? lo[axis] - 1 + which : hi[axis] + (which - 2);
  const int u0 = lo[u] - 2, nu = hi[u] - lo[u] + 5, v0 = lo[v] - 2, nv = hi[v] - lo[v] + 5;
  const int64_t cnt = (int64_t)nu * nv;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < cnt;
       t += (int64_t)gridDim.x * blockDim.x) {
    int c[3];
    c[axis] = plane;
    c[u] = u0 + (int)(t % nu);
    c[v] = v0 + (int)(t / nu);
    const int i = c[0], j = c[1], k = c[2];
    const int64_t n = i + (int64_t)j * d.Ip + (int64_t)k * d.plane;
    const Coef6 C = load_coef(d, n);
    float ex = eox[n], ey = eoy[n], ez = eoz[n];
    const float hx = d.f[3][n], hy = d.f[4][n], hz = d.f[5][n];
    const float hz_jm = d.f[5][n - d.Ip], hx_jm = d.f[3][n - d.Ip];
    const float hz_im = d.f[5][n - 1], hy_im = d.f[4][n - 1];
    const float hx_km = d.f[3][n - d.plane], hy_km = d.f[4][n - d.plane];
    update_e_cell<true, false>(d, 0, nullptr, 0, 0.f, false, i, j, k, -1, -1, -1, C, ex, ey, ez,
                               hx, hy, hz, hz_jm, hx_jm, hz_im, hy_im, hx_km, hy_km);
    d.f[0][n] = ex;
    d.f[1][n] = ey;
    d.f[2][n] = ez;
  }
}

int g_blocks_fused = 0;

}  // namespace

extern "C" {

int fdtdk_make_maps_fused(const fdtd_dev *old, fdtd_maps_fused *m) {
  m->valid = 0;
  if (((old->Ip * 4) % 16) || ((old->Ip * 2) % 16)) return (int)cudaErrorInvalidValue;
  for (int c = 0; c < 6; ++c)
    if (((uintptr_t)old->f[c]) % 16) return (int)cudaErrorInvalidValue;
  CUtensorMap *maps = reinterpret_cast<CUtensorMap *>(m->bytes);
  int e = 0;
  for (int c = 0; c < 3 && !e; ++c)
    e = encode(&maps[c], old->f[c], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, old, EW, EH);
  for (int c = 0; c < 3 && !e; ++c)
    e = encode(&maps[3 + c], old->f[3 + c], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, old, HW, HH);
  if (!e && old->coef_mode == 1) {
    if (!old->mat || ((uintptr_t)old->mat) % 16) return (int)cudaErrorInvalidValue;
    e = encode(&maps[6], (void *)old->mat, CU_TENSOR_MAP_DATA_TYPE_UINT16, 2, old, BX, BY);
  }
  if (!e) m->valid = 1;
  return e;
}

int fdtdk_fused_zchunk_default(int I, int J, int K) {
  const int tiles = ((I + BX - 1) / BX) * ((J + BY - 1) / BY);
  // >= 4 items per resident block, runs of 8..64 planes
  const long long want = 4LL * 2 * 152;
  long long chunks = (want + tiles - 1) / tiles;
  if (chunks < 1) chunks = 1;
  int z = (int)((K + chunks - 1) / chunks);
  if (z < 8) z = 8;
  if (z > 64) z = 64;
  return z < K ? z : K;
}

// The fused pass alone (old fields through m_old, H psi from d_old).
int fdtdk_fused_pass(const fdtd_dev *d_new, const fdtd_dev *d_old, const fdtd_maps_fused *m_old,
                     int zchunk, cudaStream_t s) {
  static_assert(sizeof(((FusedParams *)0)->m) == sizeof(((fdtd_maps_fused *)0)->bytes),
                "map layout");
  if (!m_old->valid || !d_new->work) return (int)cudaErrorInvalidValue;
  if (g_blocks_fused <= 0) {
    cudaError_t e = cudaFuncSetAttribute(k_step_fused, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         SMEM);
    if (e != cudaSuccess) return (int)e;
    int per_sm = 0, sms = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_step_fused, NT, SMEM);
    if (e != cudaSuccess) return (int)e;
    g_blocks_fused = (per_sm > 0 ? per_sm : 1) * (sms > 0 ? sms : 1);
  }
  FusedParams fp;
  memset(&fp, 0, sizeof(fp));
  memcpy(fp.m, m_old->bytes, sizeof(fp.m));
  fp.psi_h_old[0] = d_old->psi[PSI_HY];
  fp.psi_h_old[1] = d_old->psi[PSI_HX];
  fp.psi_h_old[2] = d_old->psi[PSI_HZ];
  fp.tiles_x = (d_new->I + BX - 1) / BX;
  fp.tiles_y = (d_new->J + BY - 1) / BY;
  static int forced = -1;  // FDTD_FUSED_ZCHUNK: a fixed item height (measurement sweeps)
  if (forced < 0) {
    const char *ev = getenv("FDTD_FUSED_ZCHUNK");
    forced = ev ? atoi(ev) : 0;
  }
  if (forced > 0) zchunk = forced;
  fp.zchunk = zchunk > 0 ? (zchunk < d_new->K ? zchunk : d_new->K)
                         : fdtdk_fused_zchunk_default(d_new->I, d_new->J, d_new->K);
  fp.n_items = fp.tiles_x * fp.tiles_y * ((d_new->K + fp.zchunk - 1) / fp.zchunk);
  fp.work = d_new->work;
  fp.err = d_new->err;
  const int blocks = fp.n_items < g_blocks_fused ? fp.n_items : g_blocks_fused;
  k_step_fused<<<blocks, NT, SMEM, s>>>(*d_new, fp);
  fdtdk_count_launches(1);
  return (int)cudaGetLastError();
}

// One fused step: the pass, the E x-slab pass, the H face pass, the E
// fix-up and the E face pass (op: curl + pml, TF/SF mode 0..5, no current).
int fdtdk_step_fused(const fdtd_dev *d_new, const fdtd_dev *d_old, const fdtd_maps_fused *m_old,
                     const fdtd_op *op, int zchunk, cudaStream_t s) {
  int e = fdtdk_fused_pass(d_new, d_old, m_old, zchunk, s);
  if (!e) fdtdk_profile_mark(s);
  if (!e) e = fdtdk_e_xslab(d_new, s);
  if (e || !op->tfsf_mode) return e;
  fdtd_op o = *op;
  o.tfsf_split = 1;
  e = fdtdk_faces(1, d_new, &o, s);
  if (e) return e;
  int a = (d_new->j1 - d_new->j0 + 5) * (d_new->k1 - d_new->k0 + 5);
  const int b2 = (d_new->i1 - d_new->i0 + 5) * (d_new->k1 - d_new->k0 + 5);
  const int c2 = (d_new->i1 - d_new->i0 + 5) * (d_new->j1 - d_new->j0 + 5);
  if (b2 > a) a = b2;
  if (c2 > a) a = c2;
  int bx = (a + 255) / 256;
  bx = bx < 1 ? 1 : (bx > 64 ? 64 : bx);
  // the axes whose faces carry H corrections: mode 1 x, z; 2 y, z; 3 x, y;
  // 4 x, z (src/gpu.h:152-573); 5 all
  static const int kAxes[6] = {0, 5, 6, 3, 5, 7};
  const int axes = kAxes[op->tfsf_mode];
  const int naxes = (axes & 1) + ((axes >> 1) & 1) + ((axes >> 2) & 1);
  k_fix_e<<<dim3(bx, 4 * naxes), 256, 0, s>>>(*d_new, d_old->f[0], d_old->f[1], d_old->f[2],
                                              axes);
  fdtdk_count_launches(1);
  e = (int)cudaGetLastError();
  if (e) return e;
  return fdtdk_faces(0, d_new, &o, s);
}

}  // extern "C"
