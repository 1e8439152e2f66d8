/*
 * fdtd_kernels.cu -- direct sm_103a kernels of the FDTD step loop, the
 * setup kernels and the launch dispatch.
 *
 * The reference (enricoballini/maxwell_solver src/gpu.h) runs one step as
 * 12 launches: the curl kernels GPU_updateH / GPU_updateE (one thread per
 * cell, 64-bit div/mod indexing), 2+2 TF/SF face kernels and 3+3 CPML slab
 * kernels that re-read the fields.  Here one step is two launches, one per
 * half-step, each fusing curl + TF/SF + CPML (+ current source) per cell
 * through the shared cell functions of fdtd_device.cuh.
 *
 * The production half-steps are the TMA-pipelined kernels of fdtd_tma.cu.
 * The direct kernels below (each thread owns an (i,j) column of a z-chunk,
 * loads straight from global memory) serve the op combinations that skip
 * the curl (a lone UpdateH_PML, say) and the comparison tests.
 *
 * Both half-steps only read the other field family and read-modify-write
 * their own cell, so in-place update is race free.
 */
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdlib.h>

#include "fdtd_device.cuh"
#include "fdtd_internal.h"

using namespace fdtd;

namespace {

constexpr int TX = 32;  // x extent of a block (one warp)
constexpr int TY = 8;   // y extent of a block

unsigned long long g_launches = 0;  // host-side count of our launches

// ----------------------------------------------------------------- H half

template <bool CURL, bool PML>
__global__ void __launch_bounds__(TX *TY) k_half_h(const fdtd_dev d, const fdtd_op op,
                                                    int zchunk) {
  const int i = blockIdx.x * TX + threadIdx.x;
  const int j = blockIdx.y * TY + threadIdx.y;
  const int I = d.I, J = d.J, K = d.K, p = d.p;
  if (i >= I - 1 || j >= J - 1) return;
  const int kb = blockIdx.z * zchunk;
  const int ke = min(kb + zchunk, K - 1);
  if (kb >= ke) return;
  const int64_t sI = d.Ip, sIJ = d.plane;
  const float *__restrict__ Ex = d.f[0];
  const float *__restrict__ Ey = d.f[1];
  const float *__restrict__ Ez = d.f[2];
  float *__restrict__ Hx = d.f[3];
  float *__restrict__ Hy = d.f[4];
  float *__restrict__ Hz = d.f[5];
  const int mode = op.tfsf_mode;
  const float *inc = mode ? inc_h_row(d, mode, op_step(d, op)) : nullptr;
  const int px = PML ? slab_h(i, I, p) : -1;
  const int py = PML ? slab_h(j, J, p) : -1;

  int64_t n = i + (int64_t)j * sI + (int64_t)kb * sIJ;
  float ex = 0.f, ey = 0.f;
  if (CURL) {
    ex = Ex[n];
    ey = Ey[n];
  }
  for (int k = kb; k < ke; ++k, n += sIJ) {
    const int pz = PML ? slab_h(k, K, p) : -1;
    if (!CURL) {
      if (!(px >= 0 || py >= 0 || pz >= 0) && !tfsf_h_touches(d, mode, i, j, k)) continue;
      ex = Ex[n];
      ey = Ey[n];
    }
    const float ez = Ez[n];
    const float ex_k1 = Ex[n + sIJ], ey_k1 = Ey[n + sIJ];
    float hx = Hx[n], hy = Hy[n], hz = Hz[n];
    update_h_cell<CURL, PML>(d, hcoef_at(d, n), mode, inc, i, j, k, px, py, pz, hx, hy, hz,
                             Ez[n + sI] - ez,
                             Ex[n + sI] - ex, Ez[n + 1] - ez, Ey[n + 1] - ey, ey_k1 - ey,
                             ex_k1 - ex, d.bH, d.cH);
    Hx[n] = hx;
    Hy[n] = hy;
    Hz[n] = hz;
    if (CURL) {
      ex = ex_k1;
      ey = ey_k1;
    }
  }
}

// ----------------------------------------------------------------- E half

template <bool CURL, bool PML>
__global__ void __launch_bounds__(TX *TY) k_half_e(const fdtd_dev d, const fdtd_op op,
                                                    int zchunk) {
  const int i = blockIdx.x * TX + threadIdx.x;
  const int j = blockIdx.y * TY + threadIdx.y;
  const int I = d.I, J = d.J, K = d.K;
  if (i >= I || j >= J) return;
  const int kb = blockIdx.z * zchunk;
  const int ke = min(kb + zchunk, K);
  if (kb >= ke) return;
  const int64_t sI = d.Ip, sIJ = d.plane;
  float *__restrict__ Ex = d.f[0];
  float *__restrict__ Ey = d.f[1];
  float *__restrict__ Ez = d.f[2];
  const float *__restrict__ Hx = d.f[3];
  const float *__restrict__ Hy = d.f[4];
  const float *__restrict__ Hz = d.f[5];
  const int mode = op.tfsf_mode;
  const int step = (mode || op.cur_mode) ? op_step(d, op) : 0;
  const float *inc = mode ? inc_e_row(d, mode, step) : nullptr;
  const int cm = op.cur_mode;
  const bool cur_col = cm && in_range(i, op.cur_box[0], op.cur_box[1]) &&
                       in_range(j, op.cur_box[2], op.cur_box[3]);
  const float cur_src = cur_col ? d.src[step] : 0.f;

  int64_t n = i + (int64_t)j * sI + (int64_t)kb * sIJ;
  float hx_km = 0.f, hy_km = 0.f;
  if (CURL && kb > 0) {
    hx_km = Hx[n - sIJ];
    hy_km = Hy[n - sIJ];
  }
  for (int k = kb; k < ke; ++k, n += sIJ) {
    int px = -1, py = -1, pz = -1;
    if (PML) e_slabs(d, i, j, k, px, py, pz);
    const bool cur = cur_col && in_range(k, op.cur_box[4], op.cur_box[5]);
    if (!CURL) {
      if (!(px >= 0 || py >= 0 || pz >= 0) && !tfsf_e_touches(d, mode, i, j, k) && !cur)
        continue;
      if (k > 0) {
        hx_km = Hx[n - sIJ];
        hy_km = Hy[n - sIJ];
      }
    }
    const float hx = Hx[n], hy = Hy[n], hz = Hz[n];
    const float hz_jm = j > 0 ? Hz[n - sI] : 0.f;
    const float hx_jm = j > 0 ? Hx[n - sI] : 0.f;
    const float hz_im = i > 0 ? Hz[n - 1] : 0.f;
    const float hy_im = i > 0 ? Hy[n - 1] : 0.f;
    const Coef6 C = load_coef(d, n);
    float ex = Ex[n], ey = Ey[n], ez = Ez[n];
    update_e_cell<CURL, PML>(d, mode, inc, cm, cur_src, cur, i, j, k, px, py, pz, C, ex, ey,
                             ez, hx, hy, hz, hz_jm, hx_jm, hz_im, hy_im, hx_km, hy_km);
    Ex[n] = ex;
    Ey[n] = ey;
    Ez[n] = ez;
    hx_km = hx;
    hy_km = hy;
  }
}

// ------------------------------------------------------ TF/SF face pass
//
// After a TMA curl kernel that skipped the TF/SF corrections
// (fdtd_tfsf_split), they are applied here to the face cells.  In every
// mode each corrected component takes corrections from the two faces of
// one axis only (tfsf_e / tfsf_h), so the pass walks those face planes and
// each thread writes the one component its plane's axis owns: no two
// threads write the same value, and a cell on two faces gets each
// component's correction exactly once, with the reference's expression.

// Component (0..2 = x,y,z) whose correction comes from the faces normal to
// `axis` in `mode`, or -1.  E: mode 1 ey<-z ez<-y; 2 ex<-z ez<-x;
// 3 ex<-z ez<-x; 4 ex<-y ey<-x.  H: 1 hx<-z hz<-x; 2 hy<-z hz<-y;
// 3 hx<-y hy<-x; 4 hx<-z hz<-x.
__host__ __device__ __forceinline__ int face_owner(bool hfam, int mode, int axis) {
  static constexpr signed char e_tab[5][3] = {{-1, -1, -1}, {-1, 2, 1}, {2, -1, 0},
                                              {2, -1, 0}, {1, 0, -1}};
  static constexpr signed char h_tab[5][3] = {{-1, -1, -1}, {2, -1, 0}, {-1, 2, 1},
                                              {1, 0, -1}, {2, -1, 0}};
  if (mode < 1 || mode > 4) return -1;
  return hfam ? h_tab[mode][axis] : e_tab[mode][axis];
}

// One face plane of the pass (q = 0..3: the low and high face of the first
// axis that owns a component, then of the second), as scalars: the plane
// sits at index `at` on `axis`, and its cells run over u (x when the plane
// contains x, so that a warp's accesses are contiguous) and v, both across
// the TF/SF box widened by one cell below (the H faces sit at i0-1).
struct FacePlane {
  int axis, at, comp, nu, nv, u0, v0;
  bool valid;
};

__device__ __forceinline__ int box_lo(const fdtd_dev &d, int a) {
  return a == 0 ? d.i0 : (a == 1 ? d.j0 : d.k0);
}
__device__ __forceinline__ int box_hi(const fdtd_dev &d, int a) {
  return a == 0 ? d.i1 : (a == 1 ? d.j1 : d.k1);
}

template <bool HFAM>
__device__ __forceinline__ FacePlane face_plane(const fdtd_dev &d, int mode, int q) {
  FacePlane f;
  f.valid = false;
  int seen = 0;
  for (int a = 0; a < 3; ++a) {
    const int c = face_owner(HFAM, mode, a);
    if (c < 0) continue;
    if (seen++ != q / 2) continue;
    const int p0 = HFAM ? box_lo(d, a) - 1 : box_lo(d, a), p1 = box_hi(d, a);
    if ((q & 1) && p1 == p0) return f;  // both faces on one plane: done once
    f.axis = a;
    f.at = (q & 1) ? p1 : p0;
    f.comp = c;
    const int u = a == 0 ? 1 : 0, v = a == 2 ? 1 : 2;
    f.u0 = box_lo(d, u) - 1;
    f.nu = box_hi(d, u) - f.u0 + 1;
    f.v0 = box_lo(d, v) - 1;
    f.nv = box_hi(d, v) - f.v0 + 1;
    f.valid = true;
  }
  return f;
}

// The TF/SF expressions of tfsf_e / tfsf_h for one face cell, on the owned
// component only (the corrections of the three components are independent).
template <bool HFAM>
__device__ __forceinline__ void face_cell(const fdtd_dev &d, int mode, const float *inc, int comp,
                                          int i, int j, int k) {
  const int64_t n = i + (int64_t)j * d.Ip + (int64_t)k * d.plane;
  float *f = d.f[(HFAM ? 3 : 0) + comp] + n;
  const float v0 = *f;
  float vx = comp == 0 ? v0 : 0.f, vy = comp == 1 ? v0 : 0.f, vz = comp == 2 ? v0 : 0.f;
  if (HFAM) {
    const HCoef C = hcoef_at(d, n);
    tfsf_h(d, mode, inc, i, j, k, vx, vy, vz, C.hex, C.hey, C.hez);
  } else {
    const Coef6 C = load_coef(d, n);
    tfsf_e(d, mode, inc, i, j, k, C.exh, C.eyh, C.ezh, vx, vy, vz);
  }
  *f = comp == 0 ? vx : (comp == 1 ? vy : vz);
}

template <bool HFAM>
__device__ __forceinline__ void face_plane_cells(const fdtd_dev &d, int mode, const float *inc,
                                                 int q, int first, int stride) {
  const FacePlane f = face_plane<HFAM>(d, mode, q);
  if (!f.valid) return;
  const int64_t total = (int64_t)f.nu * f.nv;
  for (int64_t t = first; t < total; t += stride) {
    const int u = f.u0 + (int)(t % f.nu), v = f.v0 + (int)(t / f.nu);
    if (f.axis == 0) face_cell<HFAM>(d, mode, inc, f.comp, f.at, u, v);
    else if (f.axis == 1) face_cell<HFAM>(d, mode, inc, f.comp, u, f.at, v);
    else face_cell<HFAM>(d, mode, inc, f.comp, u, v, f.at);
  }
}

// blockIdx.y = face plane 0..3
template <bool HFAM>
__global__ void k_faces(const fdtd_dev d, const fdtd_op op) {
  const int mode = op.tfsf_mode, step = op_step(d, op);
  const float *inc = HFAM ? inc_h_row(d, mode, step) : inc_e_row(d, mode, step);
  face_plane_cells<HFAM>(d, mode, inc, blockIdx.y, blockIdx.x * blockDim.x + threadIdx.x,
                         gridDim.x * blockDim.x);
}

// Batched passes: the block's member descriptor is copied into shared
// memory once (every thread of the block calls this, after any block-uniform
// early return), so that the per-cell code reads it there; stores to the
// fields (global memory) cannot alias it, so the compiler keeps the fields
// it reads in registers instead of reloading them after every store.
__device__ __forceinline__ const fdtd_dev &stage_desc(const fdtd_dev *src) {
  __shared__ __align__(16) fdtd_dev sd;
  static_assert(sizeof(fdtd_dev) % 16 == 0, "descriptor copy in 16-byte units");
  const int4 *s4 = reinterpret_cast<const int4 *>(src);
  int4 *d4 = reinterpret_cast<int4 *>(&sd);
  for (int t = threadIdx.x; t < (int)(sizeof(fdtd_dev) / 16); t += blockDim.x) d4[t] = s4[t];
  __syncthreads();
  return sd;
}

// Batched: blockIdx.z = active member g (its op says whether it split),
// blockIdx.y = face plane.
template <bool HFAM>
__global__ void k_batch_faces(const fdtd_dev *devs, const fdtd_op *ops, const int32_t *steps) {
  const int g = blockIdx.z;
  const fdtd_op &op = ops[g];
  if (!op.tfsf_split) return;
  const fdtd_dev &d = stage_desc(&devs[g]);
  const int mode = op.tfsf_mode, step = steps[g] + op.step;
  const float *inc = HFAM ? inc_h_row(d, mode, step) : inc_e_row(d, mode, step);
  face_plane_cells<HFAM>(d, mode, inc, blockIdx.y, blockIdx.x * blockDim.x + threadIdx.x,
                         gridDim.x * blockDim.x);
}

// ------------------------------------------------------- E x-slab pass
//
// With fdtd_xsplit the TMA E kernel leaves out CPML X, the last step of an
// x-slab cell's E update; this pass applies it (e_corr_x, the expression of
// gpu.h:765-788) to the x-slab cells, one thread per psi pair in the pairs'
// own order (px fastest, then j, then k; fdtd_xsplit keeps their count
// below 2^31): i = px below p and px + I - 2p above; px in [1, 2p), j and k
// inside [1, n-2] (gpu.h:776-777).
__device__ __forceinline__ void e_xslab_cell(const fdtd_dev &d, const float *sb, const float *sc,
                                             int px, int j, int k) {
  const int p2 = 2 * d.p;
  if (px < 1 || px >= p2 || j < 1 || j > d.J - 2 || k < 1 || k > d.K - 2) return;
  const int i = px < d.p ? px : px + d.I - p2;
  const int64_t n = i + (int64_t)j * d.Ip + (int64_t)k * d.plane;
  const Coef6 C = load_coef(d, n);
  const float hz = d.f[5][n], hz_im = d.f[5][n - 1];
  const float hy = d.f[4][n], hy_im = d.f[4][n - 1];
  float ey = d.f[1][n], ez = d.f[2][n];
  float2 *X = psi_at_x(d, PSI_EX, px, j, k);
  e_corr_x_bc(d, sb[px], sc[px], *X, X, C, hz, hz_im, hy, hy_im, ey, ez);
  d.f[1][n] = ey;
  d.f[2][n] = ez;
}

// The CPML grading is staged in shared memory: indexed per lane from the
// by-value descriptor it would be a divergent constant-bank load.
__device__ __forceinline__ void e_xslab_range(const fdtd_dev &d, uint32_t first,
                                              uint32_t stride) {
  __shared__ float sb[2 * FDTD_MAX_PML], sc[2 * FDTD_MAX_PML];
  for (int t = threadIdx.x; t < 2 * d.p && t < 2 * FDTD_MAX_PML; t += blockDim.x) {
    sb[t] = d.bE[t];
    sc[t] = d.cE[t];
  }
  __syncthreads();
  const uint32_t p2 = 2u * (uint32_t)d.p, J = (uint32_t)d.J;
  const uint32_t total = p2 * J * (uint32_t)d.K;
  for (uint32_t t = first; t < total; t += stride) {
    const uint32_t r = t / p2, k = r / J;
    e_xslab_cell(d, sb, sc, (int)(t - r * p2), (int)(r - k * J), (int)k);
  }
}

__global__ void k_e_xslab(const fdtd_dev d) {
  e_xslab_range(d, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
}

// Batched: blockIdx.y = active member (members without xsplit skip).
__global__ void k_batch_e_xslab(const fdtd_dev *devs, const fdtd_op *ops) {
  if (!ops[blockIdx.y].xsplit) return;
  e_xslab_range(stage_desc(&devs[blockIdx.y]), blockIdx.x * blockDim.x + threadIdx.x,
                gridDim.x * blockDim.x);
}

// ---------------------------------------------- oblique plane wave (mode 5)
//
// The incident field of an oblique plane wave comes from a 1D FDTD line
// along the propagation direction k (E at nodes, H at half nodes), run once
// for all steps (k_init_1d_oblique) with its speed scaled so that its
// numerical phase velocity equals the 3D grid's in direction k at the
// source's centre frequency; the line extends T cells beyond the source on
// both sides, so nothing reflected returns within T steps.  Only the window
// spanning the TF/SF box's projection on k is stored per step:
// ob_inc[0][n][w] = E before step n, ob_inc[1][n][w] = H after the H update
// of step n (the reference's 1D bookkeeping, src/simulation.h:201-215).
//
// The line's spacing is dx * sqrt(k_x^4 + k_y^4 + k_z^4), which makes its
// numerical dispersion agree with the 3D grid's in direction k to fourth
// order in (k dx) at every frequency; the speed factor removes the residual
// at the centre frequency.  A Yee component at position r (cells; Ex at
// (i+1/2, j, k), Hx at (i, j+1/2, k+1/2), ...) sees e_c * E1(x) and
// h_c * H1(x - 1/2) with x = ob_x0 + ob_rho * k . (r - r0) (1D nodes),
// linearly interpolated in the window.

// 1D line, one block: E[0..n1), H[0..n1-1) (H[m] at m + 1/2).
__global__ void k_init_1d_oblique(float *E, float *H, int n1, int m_src, int mb, int w, int T,
                                  float cE, float cH, const float *pw, float *out_e,
                                  float *out_h) {
  extern __shared__ float sh1d[];
  if (!E) {  // the line fits in shared memory
    E = sh1d;
    H = sh1d + n1;
  }
  for (int m = threadIdx.x; m < n1; m += blockDim.x) E[m] = H[m] = 0.f;
  __syncthreads();
  for (int n = 0; n < T; ++n) {
    for (int t = threadIdx.x; t < w; t += blockDim.x) out_e[(int64_t)n * w + t] = E[mb + t];
    for (int m = threadIdx.x; m < n1 - 1; m += blockDim.x) H[m] = H[m] - cH * (E[m + 1] - E[m]);
    __syncthreads();
    for (int t = threadIdx.x; t < w; t += blockDim.x) out_h[(int64_t)n * w + t] = H[mb + t];
    for (int m = 1 + threadIdx.x; m < n1 - 1; m += blockDim.x)
      E[m] = E[m] - cE * (H[m] - H[m - 1]);
    __syncthreads();
    if (threadIdx.x == 0) E[m_src] = E[m_src] + pw[n];
    __syncthreads();
  }
}

// Window value at coordinate x (linear interpolation between nodes).
__device__ __forceinline__ float ob_interp(const float *row, float x, int w) {
  int m = (int)floorf(x);
  m = m < 0 ? 0 : (m > w - 2 ? w - 2 : m);
  const float f = x - (float)m;
  return row[m] + f * (row[m + 1] - row[m]);
}

// Window coordinate of a point (px, py, pz) in cells: ob_rho 1D nodes per
// cell of distance along k.
__device__ __forceinline__ float ob_coord(const fdtd_dev &d, float px, float py, float pz) {
  const float s = d.ob_k[0] * (px - (float)d.ob_r0[0]) + d.ob_k[1] * (py - (float)d.ob_r0[1]) +
                  d.ob_k[2] * (pz - (float)d.ob_r0[2]);
  return d.ob_x0 + d.ob_rho * s;
}

// The oblique TF/SF corrections, one face plane per blockIdx.y = q (0..11):
// the faces normal to AXIS = q / 4, SIDE = (q / 2) % 2 (low, high), pair
// P = q % 2 (0: E_u with H_v, 1: E_v with H_u; u, v = the axes after AXIS).
// E pass: E_ce on the face's E plane takes +-C * h_ch * H1 of the H cell
// half a cell outside; H pass: H_ch at that half cell takes +-Che * e_ce *
// E1 of the face plane.  Sign: + for (E_u, H_v) on the low face, - on the
// high face, opposite for (E_v, H_u) -- the reference's axis modes are the
// special cases.  Tangential ranges: E_ce and H_ch span [lo, hi-1] along ce
// and [lo, hi] along ch.
//
// The corrections are applied plane after plane in the order (AXIS, SIDE)
// (the oracle's loops).  H planes never share an element: H_ch is corrected
// by the faces of AXIS and of ce, and along ce the H_ch plane of AXIS spans
// [lo, hi-1], inside the ce faces' H planes at lo-1 and hi.  E planes share
// the box edges: E_ce is corrected by the faces of AXIS and of ch, and along
// ch the E_ce plane of AXIS spans [lo, hi], which holds the ch faces.
// The plane that comes first in the order owns such an element and applies
// all its corrections in order, so that each element has one writer and its
// additions happen in the oracle's sequence.
template <int A, int CE>
__device__ __forceinline__ float ob_e_corr(const fdtd_dev &d, const float *rowH, int x0, int x1,
                                           int x2, int side, float c, float val) {
  constexpr int CH = 3 - A - CE;            // the H component the face pairs with E_ce
  constexpr bool T0 = CE == (A + 1) % 3;    // pair (E_u, H_v)
  const int lo = A == 0 ? d.i0 : (A == 1 ? d.j0 : d.k0);
  const int hi = A == 0 ? d.i1 : (A == 1 ? d.j1 : d.k1);
  const int xa = side ? hi : lo - 1;        // the H cell outside the face
  const float p0 = (float)(A == 0 ? xa : x0) + (CH != 0 ? 0.5f : 0.f);
  const float p1 = (float)(A == 1 ? xa : x1) + (CH != 1 ? 0.5f : 0.f);
  const float p2 = (float)(A == 2 ? xa : x2) + (CH != 2 ? 0.5f : 0.f);
  const float inc = d.ob_h[CH] * ob_interp(rowH, ob_coord(d, p0, p1, p2) - 0.5f, d.ob_w);
  const float t = c * inc;
  return (T0 == (side == 0)) ? val + t : val - t;
}

template <bool HFAM, int Q>
__device__ __forceinline__ void ob_plane(const fdtd_dev &d, int step, int first, int stride) {
  constexpr int AXIS = Q >> 2, SIDE = (Q >> 1) & 1, P = Q & 1;
  constexpr int U = (AXIS + 1) % 3, V = (AXIS + 2) % 3;
  constexpr int CE = P == 0 ? U : V, CH = P == 0 ? V : U;
  constexpr int F = U < V ? U : V, G = U < V ? V : U;  // F: the thread-fastest axis
  const int lo[3] = {d.i0, d.j0, d.k0}, hi[3] = {d.i1, d.j1, d.k1};
  const int nf = hi[F] - lo[F] + (CE == F ? 0 : 1), ng = hi[G] - lo[G] + (CE == G ? 0 : 1);
  const int64_t total = (int64_t)nf * ng;
  const int w = d.ob_w;
  const float *row = d.ob_inc[HFAM ? 0 : 1] + (int64_t)step * w;
  for (int64_t r = first; r < total; r += stride) {
    int x[3];
    x[F] = lo[F] + (int)(r % nf);
    x[G] = lo[G] + (int)(r / nf);
    if (HFAM) {  // H_ch at the half cell outside += +- Che * e_ce * E1(E_ce position)
      x[AXIS] = SIDE ? hi[AXIS] : lo[AXIS];
      const float p0 = (float)x[0] + (CE == 0 ? 0.5f : 0.f);
      const float p1 = (float)x[1] + (CE == 1 ? 0.5f : 0.f);
      const float p2 = (float)x[2] + (CE == 2 ? 0.5f : 0.f);
      const float inc = d.ob_e[CE] * ob_interp(row, ob_coord(d, p0, p1, p2), w);
      x[AXIS] = SIDE ? hi[AXIS] : lo[AXIS] - 1;
      const int64_t n = x[0] + (int64_t)x[1] * d.Ip + (int64_t)x[2] * d.plane;
      float *f = d.f[3 + CH] + n;
      const float t = hche_at(d, n, CH) * inc;
      *f = (P == 0) == (SIDE == 0) ? *f + t : *f - t;
    } else {
      x[AXIS] = SIDE ? hi[AXIS] : lo[AXIS];
      const bool on_ch_lo = x[CH] == lo[CH], on_ch_hi = x[CH] == hi[CH];
      const bool flat = lo[AXIS] == hi[AXIS];  // both faces of AXIS on one plane
      if (CH < AXIS && (on_ch_lo || on_ch_hi)) continue;  // owned by a face of CH
      if (SIDE == 1 && flat) continue;                    // owned by the low face
      const int64_t n = x[0] + (int64_t)x[1] * d.Ip + (int64_t)x[2] * d.plane;
      const Coef6 C = load_coef(d, n);
      const float c = CE == 0 ? C.exh : (CE == 1 ? C.eyh : C.ezh);
      float *f = d.f[CE] + n;
      float val = ob_e_corr<AXIS, CE>(d, row, x[0], x[1], x[2], SIDE, c, *f);
      if (SIDE == 0 && flat) val = ob_e_corr<AXIS, CE>(d, row, x[0], x[1], x[2], 1, c, val);
      if (CH > AXIS) {
        if (on_ch_lo) val = ob_e_corr<CH, CE>(d, row, x[0], x[1], x[2], 0, c, val);
        if (on_ch_hi) val = ob_e_corr<CH, CE>(d, row, x[0], x[1], x[2], 1, c, val);
      }
      *f = val;
    }
  }
}

template <bool HFAM>
__device__ __forceinline__ void ob_planes(const fdtd_dev &d, int q, int step, int first,
                                          int stride) {
  switch (q) {
#define OB_Q(Q) \
  case Q: ob_plane<HFAM, Q>(d, step, first, stride); break;
    OB_Q(0) OB_Q(1) OB_Q(2) OB_Q(3) OB_Q(4) OB_Q(5)
    OB_Q(6) OB_Q(7) OB_Q(8) OB_Q(9) OB_Q(10) OB_Q(11)
#undef OB_Q
    default: break;
  }
}

template <bool HFAM>
__global__ void k_faces_oblique(const fdtd_dev d, const fdtd_op op) {
  ob_planes<HFAM>(d, blockIdx.y, op_step(d, op), blockIdx.x * blockDim.x + threadIdx.x,
                  gridDim.x * blockDim.x);
}

// Batched: blockIdx.z = active member; members in other modes skip.
template <bool HFAM>
__global__ void k_batch_faces_oblique(const fdtd_dev *devs, const fdtd_op *ops,
                                      const int32_t *steps) {
  const int g = blockIdx.z;
  const fdtd_op &op = ops[g];
  if (!op.tfsf_split || op.tfsf_mode != FDTD_MODE_OBLIQUE) return;
  ob_planes<HFAM>(stage_desc(&devs[g]), blockIdx.y, steps[g] + op.step,
                  blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
}

// --------------------------------------------------------------- probes

// Records the six components at every probe into row *probe_row and
// advances the row: one block, every thread reads the row before the
// barrier, then thread 0 advances it (one launch per step).
__global__ void k_probe_gather(const fdtd_dev d) {
  const int row = *d.probe_row;
  if (row < d.T)
    for (int t = threadIdx.x; t < d.num_ant * 6; t += blockDim.x) {
      const int a = t / 6, c = t - a * 6;
      const int64_t id = d.probe_idx[a];
      d.probes[((int64_t)row * d.num_ant + a) * 6 + c] = id >= 0 ? d.f[c][id] : 0.f;
    }
  __syncthreads();
  if (threadIdx.x == 0) *d.probe_row = row + 1;
}

// Batched probe gather: block g records grid g's probes into its current
// row, then advances the row.
__global__ void k_batch_probes(const fdtd_dev *devs, int n) {
  const int g = blockIdx.x;
  if (g >= n) return;
  const fdtd_dev &d = devs[g];
  if (d.num_ant <= 0 || !d.probes) return;
  const int row = *d.probe_row;
  if (row < d.T) {
    for (int t = threadIdx.x; t < d.num_ant * 6; t += blockDim.x) {
      const int a = t / 6, c = t - a * 6;
      const int64_t id = d.probe_idx[a];
      d.probes[((int64_t)row * d.num_ant + a) * 6 + c] = id >= 0 ? d.f[c][id] : 0.f;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) *d.probe_row = row + 1;
}

__global__ void k_batch_advance(int32_t *steps, int n) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g < n) steps[g] += 1;
}

__global__ void k_add_i32(int32_t *p, int32_t v) { *p += v; }

// Self-check of the division plan: over the float bit patterns
// [first, first + count), counts inputs where fdtd::div_by differs bitwise
// from the IEEE quotient a / dx computed by this GPU.
__global__ void k_check_division(fdtd_div_plan p, uint64_t first, uint64_t count,
                                 unsigned long long *out) {
  unsigned long long bad = 0;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < count; t += stride) {
    const float a = __uint_as_float((uint32_t)(first + t));
    const float q = div_by(a, p.dx, p.rdx, p.lo, p.hi, p.lo2);
    const float r = a / p.dx;
    bad += __float_as_uint(q) != __float_as_uint(r);
  }
  for (int o = 16; o > 0; o >>= 1) bad += __shfl_xor_sync(0xffffffffu, bad, o);
  if ((threadIdx.x & 31) == 0 && bad) atomicAdd(out, bad);
}
__global__ void k_set_i32(int32_t *p, int32_t v) { *p = v; }

__global__ void k_fill_f32(float *p, float v, int64_t n) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x)
    p[t] = v;
}

// ------------------------------------------------------ coefficients (setup)

// src/simulation.h:924-938 in the reference's precision: 2*eps0*eps and the
// quotient in double, sigma*delT in float, the result rounded to float.
// Inputs arrive in the output buffers (sigma_x,y,z in ce[0..2], eps_x,y,z in
// ce[3..5]); each component's two inputs are read before its two outputs
// are written.  Padding columns (i >= I) are left alone.
__global__ void k_compute_ce(float *ce0, float *ce1, float *ce2, float *ce3, float *ce4,
                             float *ce5, const float *eps0_, const float *eps1_,
                             const float *eps2_, const float *sig0, const float *sig1,
                             const float *sig2, const float *den_ex, int64_t cells, int Ip,
                             int I, float delT, double two_eps0) {
  float *ce[6] = {ce0, ce1, ce2, ce3, ce4, ce5};
  const float *eps[3] = {eps0_, eps1_, eps2_};
  const float *sig[3] = {sig0, sig1, sig2};
  const float two_dt = 2 * delT;
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < cells;
       n += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(n % Ip);
    if (i >= I) continue;
    const double den = (double)den_ex[i];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const float sd = __fmul_rn(sig[a][n], delT);
      const double te = __dmul_rn(two_eps0, (double)eps[a][n]);
      const double lo = __dadd_rn(te, (double)sd);
      ce[a][n] = __double2float_rn(__ddiv_rn(__dsub_rn(te, (double)sd), lo));
      ce[3 + a][n] = __double2float_rn(__dmul_rn(__ddiv_rn((double)two_dt, lo), den));
    }
  }
}

// Media from shapes: sigma into sig[0..2], eps_r into eps[0..2] (pitched),
// starting from the background and applying the shapes in order.  The
// tests are done in double arithmetic with each operation rounded on its
// own, so the host rasteriser (OutputVis) and any double-precision
// restatement give the same cells.
__global__ void k_rasterize(float *sg0, float *sg1, float *sg2, float *ep0, float *ep1,
                            float *ep2, const fdtd_shape *shapes, int n_shapes, float bg_eps,
                            float bg_sig, int64_t cells, int Ip, int I, int J) {
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < cells;
       n += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(n % Ip);
    if (i >= I) continue;
    const int64_t r = n / Ip;
    const int j = (int)(r % J), k = (int)(r / J);
    float e = bg_eps, sg = bg_sig;
    for (int a = 0; a < n_shapes; ++a) {
      const fdtd_shape &sh = shapes[a];
      bool in = false;
      if (sh.kind == FDTD_SHAPE_SPHERE) {
        const double x = __dsub_rn((double)i + 0.5, sh.g[0]);
        const double y = __dsub_rn((double)j + 0.5, sh.g[1]);
        const double z = __dsub_rn((double)k + 0.5, sh.g[2]);
        const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z));
        in = d2 <= __dmul_rn(sh.g[3], sh.g[3]);
      } else if (sh.kind == FDTD_SHAPE_LAYER_Z) {
        in = (double)k >= sh.g[0] && (double)k < sh.g[1];
      } else if (sh.kind == FDTD_SHAPE_BOX) {
        in = (double)i >= sh.g[0] && (double)i < sh.g[1] && (double)j >= sh.g[2] &&
             (double)j < sh.g[3] && (double)k >= sh.g[4] && (double)k < sh.g[5];
      }
      if (in) {
        e = sh.eps_r;
        sg = sh.sigma;
      }
    }
    sg0[n] = sg;
    sg1[n] = sg;
    sg2[n] = sg;
    ep0[n] = e;
    ep1[n] = e;
    ep2[n] = e;
  }
}

// src/simulation.h:43-63: delT/mu0/mu/(1 + sigma_m*delT/2/mu0/mu) * den_hx
// (dense layout: these coefficients are stored, never read by a kernel).
__global__ void k_compute_mu(float *out, const float *mu, const float *den_hx, int64_t IJK,
                             int I, float delT, float sigma_m, double mu0) {
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < IJK;
       n += (int64_t)gridDim.x * blockDim.x) {
    const double m = (double)mu[n];
    const float st = __fdiv_rn(__fmul_rn(sigma_m, delT), 2.0f);
    const double q = __ddiv_rn(__ddiv_rn((double)st, mu0), m);
    const double a = __ddiv_rn(__ddiv_rn((double)delT, mu0), m);
    out[n] = __double2float_rn(__dmul_rn(__ddiv_rn(a, __dadd_rn(1.0, q)),
                                         (double)den_hx[n % I]));
  }
}

// ----------------------------------------- material-indexed coefficients

__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

__device__ __forceinline__ unsigned long long tuple_hash(const float v[6]) {
  unsigned long long h = 0x9E3779B97F4A7C15ULL;
#pragma unroll
  for (int c = 0; c < 6; ++c) h = mix64(h ^ (unsigned long long)__float_as_uint(v[c]) ^
                                        ((unsigned long long)c << 40));
  return h ? h : 1ULL;
}

constexpr int kMaxProbe = 128;

// Inserts each cell's coefficient tuple hash into an open-addressing table
// (bounded probing); the first inserter of a hash records its cell as the
// representative.  mat[n] receives the slot.  counters: [0] distinct,
// [1] overflow.
__global__ void k_hash_insert(const fdtd_dev d, const float *c0, const float *c1,
                              const float *c2, const float *c3, const float *c4,
                              const float *c5, uint16_t *mat, unsigned long long *keys,
                              int64_t *rep, int cap, int max_mat, int *counters) {
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < d.cells;
       n += (int64_t)gridDim.x * blockDim.x) {
    if ((int)(n % d.Ip) >= d.I) continue;
    if (*(volatile int *)&counters[1]) return;
    const float v[6] = {c0[n], c1[n], c2[n], c3[n], c4[n], c5[n]};
    const unsigned long long h = tuple_hash(v);
    int slot = (int)(h & (unsigned long long)(cap - 1));
    int found = -1;
    for (int probe = 0; probe < kMaxProbe; ++probe) {
      unsigned long long cur = *(volatile unsigned long long *)&keys[slot];
      if (cur == h) {
        found = slot;
        break;
      }
      if (cur == 0ULL) {
        cur = atomicCAS(&keys[slot], 0ULL, h);
        if (cur == 0ULL) {
          rep[slot] = n;
          if (atomicAdd(&counters[0], 1) + 1 > max_mat) atomicExch(&counters[1], 1);
          found = slot;
          break;
        }
        if (cur == h) {
          found = slot;
          break;
        }
      }
      slot = (slot + 1) & (cap - 1);
    }
    if (found < 0) {
      atomicExch(&counters[1], 1);
      return;
    }
    mat[n] = (uint16_t)found;
  }
}

// One block: compact ids for the occupied slots (exclusive scan) and the
// [n][6] table from each slot's representative cell.
__global__ void __launch_bounds__(1024) k_hash_compact(const float *c0, const float *c1,
                                                       const float *c2, const float *c3,
                                                       const float *c4, const float *c5,
                                                       const unsigned long long *keys,
                                                       const int64_t *rep, int *ids, int cap,
                                                       float *tab, int max_mat,
                                                       int *counters) {
  __shared__ int part[1024];
  const int t = threadIdx.x, per = (cap + 1023) / 1024;
  const int lo = t * per, hi = min(lo + per, cap);
  int cnt = 0;
  for (int s = lo; s < hi; ++s) cnt += keys[s] != 0ULL;
  part[t] = cnt;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {  // inclusive Hillis-Steele scan
    const int v = t >= off ? part[t - off] : 0;
    __syncthreads();
    part[t] += v;
    __syncthreads();
  }
  int id = part[t] - cnt;
  if (t == 1023 && part[t] > max_mat) counters[1] = 1;
  for (int s = lo; s < hi; ++s) {
    if (keys[s] == 0ULL) continue;
    ids[s] = id;
    if (id < max_mat) {
      const int64_t r = rep[s];
      float *row = tab + (int64_t)id * 6;
      row[0] = c0[r];
      row[1] = c1[r];
      row[2] = c2[r];
      row[3] = c3[r];
      row[4] = c4[r];
      row[5] = c5[r];
    }
    ++id;
  }
}

// Slot -> compact id for every cell, verifying that the cell's tuple equals
// its id's table row bit for bit (a hash collision sets counters[2]).
__global__ void k_hash_remap(const fdtd_dev d, const float *c0, const float *c1,
                             const float *c2, const float *c3, const float *c4,
                             const float *c5, uint16_t *mat, const int *ids, const float *tab,
                             int max_mat, int *counters) {
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < d.cells;
       n += (int64_t)gridDim.x * blockDim.x) {
    if ((int)(n % d.Ip) >= d.I) {
      mat[n] = 0;
      continue;
    }
    const int id = ids[mat[n]];
    if (id < 0 || id >= max_mat) {  // only after an overflow: fall back
      atomicExch(&counters[1], 1);
      return;
    }
    const float *row = tab + (int64_t)id * 6;
    const float v[6] = {c0[n], c1[n], c2[n], c3[n], c4[n], c5[n]};
    bool same = true;
#pragma unroll
    for (int c = 0; c < 6; ++c) same &= __float_as_uint(v[c]) == __float_as_uint(row[c]);
    if (!same) atomicExch(&counters[2], 1);
    mat[n] = (uint16_t)id;
  }
}

// ------------------------------------------------------------ 1D incident

// Forward (block 0, source near the high end) and inverse (block 1, source
// near the low end) runs of the auxiliary 1D Ez/Hy grid for all T steps in
// one launch, replacing init1D's 2 x T x 7 launches (src/simulation.h:
// 198-244) of the kernels at src/gpu.h:40-53 and :84-149.  The line lives in
// shared memory when it fits (use_smem) or in `scratch` (2 x 2 x S floats).
__global__ void __launch_bounds__(1024) k_init_1d(const fdtd_dev d, float *Ef, float *Hf,
                                                   float *Ei, float *Hi, const float *pw,
                                                   float Ceh, float *scratch, int use_smem) {
  extern __shared__ float sm[];
  const int S = d.size1d, p = d.p, T = d.T;
  const int fwd = blockIdx.x == 0;
  float *E, *H;
  if (use_smem) {
    E = sm;
    H = sm + S;
  } else {
    E = scratch + (int64_t)blockIdx.x * 2 * S;
    H = E + S;
  }
  __shared__ float psiE[2 * FDTD_MAX_PML], psiH[2 * FDTD_MAX_PML];
  float *Es = fwd ? Ef : Ei;
  float *Hs = fwd ? Hf : Hi;
  // reference: S-13 and 13 for its 10-cell CPML (src/simulation.h:213, :241),
  // i.e. 3 cells inside the 1D CPML; kept 3 cells inside for other thicknesses
  const int src_at = fwd ? S - (p + 3) : p + 3;
  const float Che = d.Che, dx = d.dx;
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int t = tid; t < S; t += nt) {
    E[t] = 0.f;
    H[t] = 0.f;
  }
  for (int t = tid; t < 2 * p; t += nt) {
    psiE[t] = 0.f;
    psiH[t] = 0.f;
  }
  __syncthreads();
  for (int n = 0; n < T; ++n) {
    float *erow = Es + (int64_t)n * S;
    for (int t = tid; t < S; t += nt) {  // copy1d (E before the step)
      const float e = E[t];
      erow[t] = e;
      if (t < S - 1) H[t] = H[t] + Che * (E[t + 1] - e);  // GPU_updateH_1D
    }
    __syncthreads();
    for (int t = tid; t < 2 * p - 1; t += nt) {  // GPU_updateHPml_1D
      const int idx = t < p ? t : t + S - 2 * p;
      const float v = d.bH[t] * psiH[t] + d.cH[t] * (E[idx + 1] - E[idx]) / dx;
      psiH[t] = v;
      H[idx] = H[idx] + Che * v * dx;
    }
    __syncthreads();
    float *hrow = Hs + (int64_t)n * S;
    for (int t = tid; t < S; t += nt) {  // GPU_updateE_1D + copy1d of H
      const float h = H[t];
      hrow[t] = h;
      if (t > 0) E[t] = E[t] + Ceh * (h - H[t - 1]);
    }
    __syncthreads();
    for (int t = tid + 1; t < 2 * p; t += nt) {  // GPU_updateEPml_1D
      const int idx = t < p ? t : t + S - 2 * p;
      const float v = d.bE[t] * psiE[t] + d.cE[t] * (H[idx] - H[idx - 1]) / dx;
      psiE[t] = v;
      E[idx] = E[idx] + Ceh * v * dx;
    }
    __syncthreads();
    if (tid == 0) E[src_at] = E[src_at] + pw[n];  // AddSource_GPU_1D
    __syncthreads();
  }
}

inline int grid_chunks(int extent, int zchunk) { return (extent + zchunk - 1) / zchunk; }

// z-chunk height: enough blocks for ~4 resident waves on 152 SMs, at most 64.
inline int pick_zchunk(int bx, int by, int K) {
  const long long xy = (long long)bx * by;
  const long long want = 152LL * 8 * 4;
  long long chunks = (want + xy - 1) / xy;
  if (chunks < 1) chunks = 1;
  if (chunks > K) chunks = K;
  int z = (int)((K + chunks - 1) / chunks);
  if (z > 64) z = 64;
  if (z < 1) z = 1;
  return z;
}

template <class KH>
int launch_half(KH kern, const fdtd_dev *d, const fdtd_op *op, cudaStream_t s, int ni,
                int nj, int nk) {
  const int bx = (ni + TX - 1) / TX, by = (nj + TY - 1) / TY;
  const int zc = pick_zchunk(bx, by, nk);
  dim3 grid(bx, by, grid_chunks(nk, zc));
  kern<<<grid, dim3(TX, TY), 0, s>>>(*d, *op, zc);
  ++g_launches;
  return (int)cudaGetLastError();
}

}  // namespace

extern "C" {

// Mode 5 (oblique): the curl / CPML / source kernels without TF/SF, then the
// face passes (valid when the faces are clear of the CPML and the source).
static int half_oblique(int hfam, const fdtd_dev *d, const fdtd_maps *m, int use_tma,
                        const fdtd_op *op, cudaStream_t s) {
  if (!d->ob_inc[0] || !fdtd_tfsf_faces_clear(d, op)) return (int)cudaErrorNotSupported;
  fdtd_op o = *op;
  o.tfsf_mode = 0;
  int e = 0;
  if (o.curl || o.pml || (!hfam && o.cur_mode))
    e = hfam ? fdtdk_half_h(d, m, use_tma, &o, s) : fdtdk_half_e(d, m, use_tma, &o, s);
  if (e) return e;
  return fdtdk_faces(hfam, d, op, s);
}

int fdtdk_half_h(const fdtd_dev *d, const fdtd_maps *m, int use_tma, const fdtd_op *op,
                 cudaStream_t s) {
  if (op->tfsf_mode == FDTD_MODE_OBLIQUE) return half_oblique(1, d, m, use_tma, op, s);
  if (use_tma && m && m[0].valid && op->curl) return fdtdk_half_h_tma(d, m, op, s);
  const int ni = d->I - 1, nj = d->J - 1, nk = d->K - 1;
  if (op->curl && op->pml) return launch_half(k_half_h<true, true>, d, op, s, ni, nj, nk);
  if (op->curl) return launch_half(k_half_h<true, false>, d, op, s, ni, nj, nk);
  if (op->pml) return launch_half(k_half_h<false, true>, d, op, s, ni, nj, nk);
  if (op->tfsf_mode) return launch_half(k_half_h<false, false>, d, op, s, ni, nj, nk);
  return 0;
}

int fdtdk_half_e(const fdtd_dev *d, const fdtd_maps *m, int use_tma, const fdtd_op *op,
                 cudaStream_t s) {
  if (op->tfsf_mode == FDTD_MODE_OBLIQUE) return half_oblique(0, d, m, use_tma, op, s);
  if (use_tma && m && m[0].valid && op->curl) return fdtdk_half_e_tma(d, m, op, s);
  const int ni = d->I, nj = d->J, nk = d->K;
  if (op->curl && op->pml) return launch_half(k_half_e<true, true>, d, op, s, ni, nj, nk);
  if (op->curl) return launch_half(k_half_e<true, false>, d, op, s, ni, nj, nk);
  if (op->pml) return launch_half(k_half_e<false, true>, d, op, s, ni, nj, nk);
  if (op->tfsf_mode || op->cur_mode)
    return launch_half(k_half_e<false, false>, d, op, s, ni, nj, nk);
  return 0;
}

int fdtdk_faces(int hfam, const fdtd_dev *d, const fdtd_op *op, cudaStream_t s) {
  if (op->tfsf_mode == FDTD_MODE_OBLIQUE) {  // the twelve face planes in one launch
    int32_t a = (d->j1 - d->j0 + 1) * (d->k1 - d->k0 + 1);
    if ((d->i1 - d->i0 + 1) * (d->k1 - d->k0 + 1) > a) a = (d->i1 - d->i0 + 1) * (d->k1 - d->k0 + 1);
    if ((d->i1 - d->i0 + 1) * (d->j1 - d->j0 + 1) > a) a = (d->i1 - d->i0 + 1) * (d->j1 - d->j0 + 1);
    int bx = (a + 255) / 256;
    bx = bx < 1 ? 1 : (bx > 152 * 2 ? 152 * 2 : bx);
    if (hfam) k_faces_oblique<true><<<dim3(bx, 12), 256, 0, s>>>(*d, *op);
    else k_faces_oblique<false><<<dim3(bx, 12), 256, 0, s>>>(*d, *op);
    ++g_launches;
    return (int)cudaGetLastError();
  }
  int32_t a = (d->I + 2) * (d->J + 2);
  if ((d->J + 2) * (d->K + 2) > a) a = (d->J + 2) * (d->K + 2);
  if ((d->I + 2) * (d->K + 2) > a) a = (d->I + 2) * (d->K + 2);
  int bx = (a + 255) / 256;
  if (bx > 152 * 2) bx = 152 * 2;
  const dim3 grid(bx > 0 ? bx : 1, 4);
  if (hfam) k_faces<true><<<grid, 256, 0, s>>>(*d, *op);
  else k_faces<false><<<grid, 256, 0, s>>>(*d, *op);
  ++g_launches;
  return (int)cudaGetLastError();
}

int fdtdk_e_xslab(const fdtd_dev *d, cudaStream_t s) {
  const int64_t total = 2 * (int64_t)d->p * d->J * d->K;
  if (total <= 0 || total > INT32_MAX) return total > 0 ? (int)cudaErrorInvalidValue : 0;
  int64_t bx = (total + 255) / 256;
  if (bx > 152 * 16) bx = 152 * 16;
  k_e_xslab<<<(unsigned)bx, 256, 0, s>>>(*d);
  ++g_launches;
  return (int)cudaGetLastError();
}

// Blocks per member of the batched x-slab and face passes (environment
// FDTD_BATCH_XSLAB_BLOCKS, FDTD_BATCH_FACE_BLOCKS; read once).
static int batch_blocks(const char *name, int def) {
  const char *e = getenv(name);
  const int v = e ? atoi(e) : def;
  return v >= 1 && v <= 4096 ? v : def;
}

int fdtdk_batch_e_xslab(const fdtd_dev *devs, const fdtd_op *ops, int32_t n, int64_t max_cells,
                        cudaStream_t s) {
  static const int cap = batch_blocks("FDTD_BATCH_XSLAB_BLOCKS", 64);
  if (n <= 0 || max_cells <= 0) return 0;
  int64_t bx = (max_cells + 255) / 256;
  if (bx > cap) bx = cap;
  k_batch_e_xslab<<<dim3((unsigned)bx, (unsigned)n), 256, 0, s>>>(devs, ops);
  ++g_launches;
  return (int)cudaGetLastError();
}

int fdtdk_batch_faces(int hfam, const fdtd_dev *devs, const fdtd_op *ops, const int32_t *steps,
                      int32_t n, int32_t max_cells_per_face, cudaStream_t s) {
  static const int cap = batch_blocks("FDTD_BATCH_FACE_BLOCKS", 4);
  if (n <= 0) return 0;
  int bx = (max_cells_per_face + 255) / 256;
  if (bx > cap) bx = cap;
  const dim3 grid(bx > 0 ? bx : 1, 4, (unsigned)n);
  if (hfam) k_batch_faces<true><<<grid, 256, 0, s>>>(devs, ops, steps);
  else k_batch_faces<false><<<grid, 256, 0, s>>>(devs, ops, steps);
  ++g_launches;
  return (int)cudaGetLastError();
}

int fdtdk_batch_faces_oblique(int hfam, const fdtd_dev *devs, const fdtd_op *ops,
                              const int32_t *steps, int32_t n, int32_t max_cells_per_face,
                              cudaStream_t s) {
  static const int cap = batch_blocks("FDTD_BATCH_FACE_BLOCKS", 4);
  if (n <= 0) return 0;
  int bx = (max_cells_per_face + 255) / 256;
  bx = bx < 1 ? 1 : (bx > cap ? cap : bx);
  if (hfam) k_batch_faces_oblique<true><<<dim3(bx, 12, n), 256, 0, s>>>(devs, ops, steps);
  else k_batch_faces_oblique<false><<<dim3(bx, 12, n), 256, 0, s>>>(devs, ops, steps);
  ++g_launches;
  return (int)cudaGetLastError();
}

int fdtdk_init_1d_oblique(int n1, int m_src, int mb, int w, int T, float cE, float cH,
                          const float *pw, float *out_e, float *out_h, float *scratch,
                          cudaStream_t s) {
  const size_t smem = 2 * (size_t)n1 * sizeof(float);
  if (!scratch) {
    cudaError_t e = cudaFuncSetAttribute(k_init_1d_oblique,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return (int)e;
  }
  k_init_1d_oblique<<<1, 1024, scratch ? 0 : smem, s>>>(scratch, scratch ? scratch + n1 : nullptr,
                                                        n1, m_src, mb, w, T, cE, cH, pw, out_e,
                                                        out_h);
  ++g_launches;
  return (int)cudaGetLastError();
}

int fdtdk_probe_gather(const fdtd_dev *d, cudaStream_t s) {
  if (d->num_ant <= 0 || !d->probes) return 0;
  k_probe_gather<<<1, 1024, 0, s>>>(*d);
  ++g_launches;
  return (int)cudaGetLastError();
}

int fdtdk_fill_f32(float *dst, float v, int64_t n, cudaStream_t s) {
  if (n <= 0) return 0;
  int64_t bx = (n + 255) / 256;
  if (bx > 152 * 16) bx = 152 * 16;
  k_fill_f32<<<(unsigned)bx, 256, 0, s>>>(dst, v, n);
  ++g_launches;
  return (int)cudaGetLastError();
}

int fdtdk_set_i32(int32_t *dst, int32_t v, cudaStream_t s) {
  k_set_i32<<<1, 1, 0, s>>>(dst, v);
  ++g_launches;
  return (int)cudaGetLastError();
}

int fdtdk_add_i32(int32_t *dst, int32_t v, cudaStream_t s) {
  k_add_i32<<<1, 1, 0, s>>>(dst, v);
  ++g_launches;
  return (int)cudaGetLastError();
}

int fdtdk_compute_ce(const fdtd_dev *d, float *const ce[6], const float *const eps[3],
                     const float *const sig[3], const float *den_ex, float delT,
                     cudaStream_t s) {
  const double mu0 = 4 * 3.14159265358979323846 * 1e-7;
  const double c0 = 299792458;
  const double eps0 = 1 / c0 / c0 / mu0;
  k_compute_ce<<<152 * 8, 256, 0, s>>>(ce[0], ce[1], ce[2], ce[3], ce[4], ce[5], eps[0], eps[1],
                                        eps[2], sig[0], sig[1], sig[2], den_ex, d->cells, d->Ip,
                                        d->I, delT, 2 * eps0);
  ++g_launches;
  return (int)cudaGetLastError();
}

int fdtdk_compute_mu(float *out, const float *mu, const float *den_hx, int64_t IJK, int32_t I,
                     float delT, float sigma_m, cudaStream_t s) {
  const double mu0 = 4 * 3.14159265358979323846 * 1e-7;
  k_compute_mu<<<152 * 8, 256, 0, s>>>(out, mu, den_hx, IJK, I, delT, sigma_m, mu0);
  ++g_launches;
  return (int)cudaGetLastError();
}

int fdtdk_compress_ce(const fdtd_dev *d, const float *const ce[6], uint16_t *mat, float *tab,
                      int32_t max_mat, unsigned long long *hash_keys, int64_t *hash_rep,
                      int32_t *hash_id, int32_t hash_cap, int32_t *counters, cudaStream_t s) {
  // the slot index is carried in the u16 id array: every u16 must be a slot
  if (hash_cap != 65536) return (int)cudaErrorInvalidValue;
  cudaError_t e = cudaMemsetAsync(hash_keys, 0, (size_t)hash_cap * sizeof(unsigned long long), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(hash_id, 0xFF, (size_t)hash_cap * sizeof(int32_t), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(counters, 0, 4 * sizeof(int32_t), s);
  if (e != cudaSuccess) return (int)e;
  k_hash_insert<<<152 * 8, 256, 0, s>>>(*d, ce[0], ce[1], ce[2], ce[3], ce[4], ce[5], mat,
                                         hash_keys, hash_rep, hash_cap, max_mat, counters);
  k_hash_compact<<<1, 1024, 0, s>>>(ce[0], ce[1], ce[2], ce[3], ce[4], ce[5], hash_keys,
                                     hash_rep, hash_id, hash_cap, tab, max_mat, counters);
  k_hash_remap<<<152 * 8, 256, 0, s>>>(*d, ce[0], ce[1], ce[2], ce[3], ce[4], ce[5], mat,
                                        hash_id, tab, max_mat, counters);
  g_launches += 3;
  return (int)cudaGetLastError();
}

size_t fdtdk_init_1d_smem_limit(void) { return 160 * 1024; }

int fdtdk_init_1d(const fdtd_dev *d, float *tab[4], const float *pw, float Ceh, float *scratch,
                  cudaStream_t s) {
  const size_t smem = 2 * (size_t)d->size1d * sizeof(float);
  const int use_smem = smem <= fdtdk_init_1d_smem_limit();
  if (use_smem) {
    cudaError_t e = cudaFuncSetAttribute(k_init_1d, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)fdtdk_init_1d_smem_limit());
    if (e != cudaSuccess) return (int)e;
  } else if (!scratch) {
    return (int)cudaErrorInvalidValue;
  }
  int threads = d->size1d < 1024 ? ((d->size1d + 31) / 32) * 32 : 1024;
  if (threads < 64) threads = 64;
  k_init_1d<<<2, threads, use_smem ? smem : 0, s>>>(*d, tab[0], tab[1], tab[2], tab[3], pw, Ceh,
                                                    scratch, use_smem);
  ++g_launches;
  return (int)cudaGetLastError();
}

int fdtdk_batch_probes(const fdtd_dev *devs, int32_t n, cudaStream_t s) {
  if (n <= 0) return 0;
  k_batch_probes<<<n, 256, 0, s>>>(devs, n);
  ++g_launches;
  return (int)cudaGetLastError();
}

int fdtdk_rasterize(const fdtd_dev *d, float *const sig[3], float *const eps[3],
                    const fdtd_shape *shapes, int32_t n_shapes, float bg_eps, float bg_sig,
                    cudaStream_t s) {
  k_rasterize<<<152 * 8, 256, 0, s>>>(sig[0], sig[1], sig[2], eps[0], eps[1], eps[2],
                                                  shapes, n_shapes, bg_eps, bg_sig, d->cells,
                                                  d->Ip, d->I, d->J);
  ++g_launches;
  return (int)cudaGetLastError();
}

int fdtdk_check_division(fdtd_div_plan p, uint64_t first, uint64_t count,
                         unsigned long long *out, cudaStream_t s) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  k_check_division<<<(sms > 0 ? sms : 1) * 8, 256, 0, s>>>(p, first, count, out);
  ++g_launches;
  return (int)cudaGetLastError();
}

int fdtdk_batch_advance(int32_t *steps, int32_t n, cudaStream_t s) {
  if (n <= 0) return 0;
  k_batch_advance<<<(n + 255) / 256, 256, 0, s>>>(steps, n);
  ++g_launches;
  return (int)cudaGetLastError();
}

void fdtdk_count_launches(unsigned long long n) { g_launches += n; }

static thread_local cudaEvent_t g_profile_mark = nullptr;
void fdtdk_set_profile_mark(cudaEvent_t ev) { g_profile_mark = ev; }
void fdtdk_profile_mark(cudaStream_t s) {
  if (g_profile_mark) cudaEventRecord(g_profile_mark, s);
}

unsigned long long fdtdk_launch_count(void) { return g_launches; }

}  // extern "C"

// ------------------------------------------------------------------------
// Allocation-free coefficient indexing.
//
// Some callers cannot call cudaMalloc: hosts that own all device memory
// through their own pool or a fixed budget (an embedding application's
// allocator, a serving loop that admits work against an exact HBM budget)
// and loops that must not stall other streams with the device-wide
// synchronisation cudaMalloc/cudaFree imply.  fdtd_index_coefficients_static
// serves them: the same indexing kernels as ReadySimulation's, with their
// hash-table scratch in the file-scope array below instead of allocated
// memory.  Every GPU that loads the library holds this array (1.25 MiB)
// until the process exits.
// ------------------------------------------------------------------------

#include <mutex>

namespace {

constexpr int kStaticHashCap = 65536;   // slots (fixed: ids ride in a u16)
constexpr int kStaticMaxIds = 32768;    // largest max_ids accepted
constexpr size_t kStaticKeysOff = 0;
constexpr size_t kStaticRepOff = kStaticKeysOff + kStaticHashCap * sizeof(unsigned long long);
constexpr size_t kStaticIdsOff = kStaticRepOff + kStaticHashCap * sizeof(int64_t);
constexpr size_t kStaticCntOff = kStaticIdsOff + kStaticHashCap * sizeof(int32_t);
constexpr size_t kStaticScratchBytes = kStaticCntOff + 256;

static __device__ __align__(256) unsigned char g_index_scratch[kStaticScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_static_lock;
unsigned char *g_static_ptr[kMaxDevices];  // device address of g_index_scratch, per device

// Device address of the scratch array for the current device.  The first
// call on a device looks it up (cudaGetSymbolAddress), so that first call
// should come before any stream capture on that device.
int static_scratch(unsigned char **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return (int)e;
  if (dev < 0 || dev >= kMaxDevices) return (int)cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> guard(g_static_lock);
  if (!g_static_ptr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_index_scratch);
    if (e != cudaSuccess) return (int)e;
    g_static_ptr[dev] = static_cast<unsigned char *>(p);
  }
  *out = g_static_ptr[dev];
  return 0;
}

}  // namespace

extern "C" int fdtd_index_coefficients_static(const float *const ce[6], int32_t I, int32_t J,
                                              int32_t K, int32_t pitch, uint16_t *ids,
                                              float *table, int32_t max_ids, int32_t *n_ids,
                                              void *stream) {
  if (n_ids) *n_ids = 0;
  if (!ce || !ids || !table || !n_ids)
    return fdtd_internal_fail(2, "fdtd_index_coefficients_static: null pointer argument");
  for (int a = 0; a < 6; ++a)
    if (!ce[a]) return fdtd_internal_fail(2, "fdtd_index_coefficients_static: null ce array");
  if (I < 1 || J < 1 || K < 1 || pitch < I)
    return fdtd_internal_fail(2, "fdtd_index_coefficients_static: need I, J, K >= 1 and "
                                 "pitch >= I");
  if (max_ids < 1 || max_ids > kStaticMaxIds)
    return fdtd_internal_fail(2, "fdtd_index_coefficients_static: max_ids must be in "
                                 "[1, 32768], the capacity of the static scratch table");
  unsigned char *base = nullptr;
  int e = static_scratch(&base);
  if (e) return fdtd_internal_fail(5, cudaGetErrorString((cudaError_t)e));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  unsigned long long *keys = reinterpret_cast<unsigned long long *>(base + kStaticKeysOff);
  int64_t *rep = reinterpret_cast<int64_t *>(base + kStaticRepOff);
  int32_t *sid = reinterpret_cast<int32_t *>(base + kStaticIdsOff);
  int32_t *cnt = reinterpret_cast<int32_t *>(base + kStaticCntOff);

  fdtd_dev d;
  memset(&d, 0, sizeof(d));
  d.I = I;
  d.J = J;
  d.K = K;
  d.Ip = pitch;
  d.plane = (int64_t)pitch * J;
  d.cells = d.plane * K;
  // the array keeps the previous call's contents: clear what starts at zero
  cudaError_t ce_ = cudaMemsetAsync(keys, 0, kStaticHashCap * sizeof(unsigned long long), s);
  if (ce_ == cudaSuccess) ce_ = cudaMemsetAsync(sid, 0xFF, kStaticHashCap * sizeof(int32_t), s);
  if (ce_ == cudaSuccess) ce_ = cudaMemsetAsync(cnt, 0, 4 * sizeof(int32_t), s);
  if (ce_ != cudaSuccess) return fdtd_internal_fail(5, cudaGetErrorString(ce_));
  k_hash_insert<<<152 * 8, 256, 0, s>>>(d, ce[0], ce[1], ce[2], ce[3], ce[4], ce[5], ids, keys,
                                         rep, kStaticHashCap, max_ids, cnt);
  k_hash_compact<<<1, 1024, 0, s>>>(ce[0], ce[1], ce[2], ce[3], ce[4], ce[5], keys, rep, sid,
                                     kStaticHashCap, table, max_ids, cnt);
  k_hash_remap<<<152 * 8, 256, 0, s>>>(d, ce[0], ce[1], ce[2], ce[3], ce[4], ce[5], ids, sid,
                                        table, max_ids, cnt);
  g_launches += 3;
  int32_t h_cnt[4] = {0, 0, 0, 0};
  ce_ = cudaGetLastError();
  if (ce_ == cudaSuccess)
    ce_ = cudaMemcpyAsync(h_cnt, cnt, sizeof(h_cnt), cudaMemcpyDeviceToHost, s);
  if (ce_ == cudaSuccess) ce_ = cudaStreamSynchronize(s);
  if (ce_ != cudaSuccess) return fdtd_internal_fail(5, cudaGetErrorString(ce_));
  if (h_cnt[1] || h_cnt[0] > max_ids)
    return fdtd_internal_fail(7, "fdtd_index_coefficients_static: more distinct coefficient "
                                 "tuples than max_ids");
  if (h_cnt[2])
    return fdtd_internal_fail(7, "fdtd_index_coefficients_static: hash collision between "
                                 "distinct coefficient tuples");
  *n_ids = h_cnt[0];
  return 0;
}
