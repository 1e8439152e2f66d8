/*
 * fdtd_kernels.cu -- sm_103a kernels of the FDTD step loop.
 *
 * The reference (enricoballini/maxwell_solver src/gpu.h) runs one step as
 * 12 launches: the curl kernels GPU_updateH / GPU_updateE (one thread per
 * cell, 64-bit div/mod indexing), 2+2 TF/SF face kernels and 3+3 CPML slab
 * kernels that re-read the fields.  Here one step is two launches:
 *
 *   k_half_h : H curl (gpu.h:575-602) + H TF/SF faces (gpu.h:152-541)
 *              + H CPML Y, X, Z (gpu.h:604-725), fused per cell;
 *   k_half_e : E curl (gpu.h:727-763) + E TF/SF faces + E CPML Y, Z, X
 *              (gpu.h:765-868) + current source (gpu.h:55-82), fused.
 *
 * Each thread owns one (i, j) column of a z-chunk and marches up in z; the
 * z-neighbour read by the stencil is carried in registers, the x and y
 * neighbours come from the same warp / block through L1.  Every cell applies
 * the reference's operations in the reference's order (curl, TF/SF, then
 * the CPML axes in launch order), each rounded separately (the library is
 * built with --fmad=false), so the result is bitwise the reference's.
 *
 * Both half-steps only read the other field family and read-modify-write
 * their own cell, so in-place update is race free.
 */
#include <cuda_runtime.h>
#include <stdint.h>

#include "fdtd_internal.h"

namespace {

constexpr int TX = 32;  // x extent of a block (one warp)
constexpr int TY = 8;   // y extent of a block

unsigned long long g_launches = 0;  // host-side count of our launches

__device__ __forceinline__ bool in_range(int v, int lo, int hi) {
  return v >= lo && v <= hi;
}

// Slab position of index v in a CPML of thickness p on an axis of length n.
// H cells: low side [0,p) -> v, high side [n-p, n-2] -> v-n+2p.
__device__ __forceinline__ int slab_h(int v, int n, int p) {
  if (v < p) return v;
  if (v >= n - p && v <= n - 2) return v - n + 2 * p;
  return -1;
}
// E cells: low side [1,p) -> v, high side [n-p, n-1] -> v-n+2p.
__device__ __forceinline__ int slab_e(int v, int n, int p) {
  if (v >= 1 && v < p) return v;
  if (v >= n - p && v <= n - 1) return v - n + 2 * p;
  return -1;
}

__device__ __forceinline__ int op_step(const fdtd_dev &d, const fdtd_op &op) {
  return op.step_from_dev ? (*d.step_base + op.step) : op.step;
}

// Incident-table row used by the H side at step n (src/simulation.h:330-349).
__device__ __forceinline__ const float *inc_h_row(const fdtd_dev &d, int mode, int n) {
  const int64_t S = d.size1d;
  switch (mode) {
    case 1:
    case 2: return d.inc[0] + (int64_t)n * S + S - d.K;
    case 3: return d.inc[0] + (int64_t)n * S + S - d.I;
    case 4: return d.inc[2] + (int64_t)n * S + S - d.I;
  }
  return nullptr;
}
// ... and by the E side (src/simulation.h:350-369).
__device__ __forceinline__ const float *inc_e_row(const fdtd_dev &d, int mode, int n) {
  const int64_t S = d.size1d;
  switch (mode) {
    case 1:
    case 2: return d.inc[1] + (int64_t)n * S + S - d.K;
    case 3: return d.inc[1] + (int64_t)n * S + S - d.I;
    case 4: return d.inc[3] + (int64_t)n * S + S - d.I;
  }
  return nullptr;
}

// H-side TF/SF corrections of one cell (all launchers pass c = +1):
// mode 3 gpu.h:152-182, mode 4 :217-247, mode 1 :424-477, mode 2 :512-541.
__device__ __forceinline__ void tfsf_h(const fdtd_dev &d, int mode, const float *inc,
                                       int i, int j, int k, float &hx, float &hy,
                                       float &hz) {
  const float Ch = d.Che;
  const int i0 = d.i0, i1 = d.i1, j0 = d.j0, j1 = d.j1, k0 = d.k0, k1 = d.k1;
  if (mode == 3) {
    if (in_range(i, i0, i1) && in_range(k, k0, k1 - 1)) {
      if (j == j0 - 1) hx = hx + Ch * inc[i];
      if (j == j1) hx = hx - Ch * inc[i];
    }
    if (in_range(j, j0, j1) && in_range(k, k0, k1 - 1)) {
      if (i == i0 - 1) hy = hy - Ch * inc[i0];
      if (i == i1) hy = hy + Ch * inc[i1];
    }
  } else if (mode == 4) {
    if (in_range(i, i0, i1) && in_range(j, j0, j1 - 1)) {
      if (k == k0 - 1) hx = hx - Ch * inc[i];
      if (k == k1) hx = hx + Ch * inc[i];
    }
    if (in_range(j, j0, j1 - 1) && in_range(k, k0, k1)) {
      if (i == i0 - 1) hz = hz + Ch * inc[i0];
      if (i == i1) hz = hz - Ch * inc[i1];
    }
  } else if (mode == 1) {
    if (in_range(i, i0, i1) && in_range(j, j0, j1 - 1)) {
      if (k == k0 - 1) hx = hx - Ch * inc[k0];
      if (k == k1) hx = hx + Ch * inc[k1];
    }
    if (in_range(j, j0, j1 - 1) && in_range(k, k0, k1)) {
      if (i == i0 - 1) hz = hz + Ch * inc[k];
      if (i == i1) hz = hz - Ch * inc[k];
    }
  } else if (mode == 2) {
    if (in_range(i, i0, i1 - 1) && in_range(j, j0, j1)) {
      if (k == k0 - 1) hy = hy + Ch * inc[k0];
      if (k == k1) hy = hy - Ch * inc[k1];
    }
    if (in_range(i, i0, i1 - 1) && in_range(k, k0, k1)) {
      if (j == j0 - 1) hz = hz - Ch * inc[k];
      if (j == j1) hz = hz + Ch * inc[k];
    }
  }
}

// E-side TF/SF corrections of one cell.  Modes 1 and 3 are launched with
// c = +1, modes 2 and 4 with c = -1 (src/simulation.h:493-570); x - (a*-1)
// is computed as x + a, which IEEE arithmetic makes identical.
// mode 3 gpu.h:184-214, mode 4 :249-291, mode 1 :479-509, mode 2 :543-573.
__device__ __forceinline__ void tfsf_e(const fdtd_dev &d, int mode, const float *inc,
                                       int i, int j, int k, float cxh, float cyh,
                                       float czh, float &ex, float &ey, float &ez) {
  const int i0 = d.i0, i1 = d.i1, j0 = d.j0, j1 = d.j1, k0 = d.k0, k1 = d.k1;
  if (mode == 3) {
    if (in_range(i, i0, i1 - 1) && in_range(j, j0, j1)) {
      if (k == k0) ex = ex + cxh * inc[i];
      if (k == k1) ex = ex - cxh * inc[i];
    }
    if (in_range(j, j0, j1) && in_range(k, k0, k1 - 1)) {
      if (i == i0) ez = ez - czh * inc[i0 - 1];
      if (i == i1) ez = ez + czh * inc[i1];
    }
  } else if (mode == 4) {
    if (in_range(i, i0, i1 - 1) && in_range(k, k0, k1)) {
      if (j == j0) ex = ex + cxh * inc[i];
      if (j == j1) ex = ex - cxh * inc[i];
    }
    if (in_range(j, j0, j1 - 1) && in_range(k, k0, k1)) {
      if (i == i0) ey = ey - cyh * inc[i0 - 1];
      if (i == i1) ey = ey + cyh * inc[i1];
    }
  } else if (mode == 1) {
    if (in_range(i, i0, i1) && in_range(j, j0, j1 - 1)) {
      if (k == k0) ey = ey - cyh * inc[k0 - 1];
      if (k == k1) ey = ey + cyh * inc[k1];
    }
    if (in_range(i, i0, i1) && in_range(k, k0, k1 - 1)) {
      if (j == j0) ez = ez + czh * inc[k];
      if (j == j1) ez = ez - czh * inc[k];
    }
  } else if (mode == 2) {
    if (in_range(i, i0, i1 - 1) && in_range(j, j0, j1)) {
      if (k == k0) ex = ex - cxh * inc[k0 - 1];
      if (k == k1) ex = ex + cxh * inc[k1];
    }
    if (in_range(j, j0, j1) && in_range(k, k0, k1 - 1)) {
      if (i == i0) ez = ez + czh * inc[k];
      if (i == i1) ez = ez - czh * inc[k];
    }
  }
}

// Does the H-side TF/SF of `mode` touch cell (i,j,k)?  (Only used by the
// non-curl variant, which skips untouched cells.)
__device__ __forceinline__ bool tfsf_h_touches(const fdtd_dev &d, int mode, int i, int j,
                                               int k) {
  if (!mode) return false;
  const bool xf = (i == d.i0 - 1 || i == d.i1), yf = (j == d.j0 - 1 || j == d.j1),
             zf = (k == d.k0 - 1 || k == d.k1);
  return xf || yf || zf;
}
__device__ __forceinline__ bool tfsf_e_touches(const fdtd_dev &d, int mode, int i, int j,
                                               int k) {
  if (!mode) return false;
  const bool xf = (i == d.i0 || i == d.i1), yf = (j == d.j0 || j == d.j1),
             zf = (k == d.k0 || k == d.k1);
  return xf || yf || zf;
}

struct Coef6 {
  float exe, eye, eze, exh, eyh, ezh;
};

__device__ __forceinline__ Coef6 load_coef(const fdtd_dev &d, int64_t n, int i) {
  Coef6 c;
  if (d.coef_mode == 0) {
    c.exe = __ldg(d.ce[0] + n);
    c.eye = __ldg(d.ce[1] + n);
    c.eze = __ldg(d.ce[2] + n);
    c.exh = __ldg(d.ce[3] + n);
    c.eyh = __ldg(d.ce[4] + n);
    c.ezh = __ldg(d.ce[5] + n);
  } else {
    const int m = __ldg(d.mat + n);
    const float *t = d.mat_tab + ((int64_t)m * d.n_xclass + __ldg(d.xclass + i)) * 6;
    c.exe = __ldg(t + 0);
    c.eye = __ldg(t + 1);
    c.eze = __ldg(t + 2);
    c.exh = __ldg(t + 3);
    c.eyh = __ldg(t + 4);
    c.ezh = __ldg(t + 5);
  }
  return c;
}

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
  const int64_t sI = I, sIJ = d.IJ;
  const float *__restrict__ Ex = d.f[0];
  const float *__restrict__ Ey = d.f[1];
  const float *__restrict__ Ez = d.f[2];
  float *__restrict__ Hx = d.f[3];
  float *__restrict__ Hy = d.f[4];
  float *__restrict__ Hz = d.f[5];
  const float Chh = d.Chh, Che = d.Che, dx = d.dx;
  const int mode = op.tfsf_mode;
  const float *inc = mode ? inc_h_row(d, mode, op_step(d, op)) : nullptr;
  const int px = PML ? slab_h(i, I, p) : -1;
  const int py = PML ? slab_h(j, J, p) : -1;
  const int64_t pj = 2 * (int64_t)p;

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
    const float dEz_y = Ez[n + sI] - ez;
    const float dEx_y = Ex[n + sI] - ex;
    const float dEz_x = Ez[n + 1] - ez;
    const float dEy_x = Ey[n + 1] - ey;
    const float dEy_z = ey_k1 - ey;
    const float dEx_z = ex_k1 - ex;
    float hx, hy, hz;
    if (CURL) {
      hx = Chh * Hx[n] + Che * (-dEz_y + dEy_z);
      hy = Chh * Hy[n] + Che * (-dEx_z + dEz_x);
      hz = Chh * Hz[n] + Che * (-dEy_x + dEx_y);
    } else {
      hx = Hx[n];
      hy = Hy[n];
      hz = Hz[n];
    }
    if (mode) tfsf_h(d, mode, inc, i, j, k, hx, hy, hz);
    if (PML) {
      if (py >= 0) {  // gpu.h:644-685
        const int64_t t = i + py * sI + k * pj * sI;
        const float b = d.bH[py], c = d.cH[py];
        float *ps = d.psi[PSI_HXY] + t;
        float v = b * *ps + c * dEz_y / dx;
        *ps = v;
        hx = hx - Che * v * dx;
        ps = d.psi[PSI_HZY] + t;
        v = b * *ps + c * dEx_y / dx;
        *ps = v;
        hz = hz + Che * v * dx;
      }
      if (px >= 0) {  // gpu.h:604-642
        const int64_t t = px + j * pj + k * pj * J;
        const float b = d.bH[px], c = d.cH[px];
        float *ps = d.psi[PSI_HYX] + t;
        float v = b * *ps + c * dEz_x / dx;
        *ps = v;
        hy = hy + Che * v * dx;
        ps = d.psi[PSI_HZX] + t;
        v = b * *ps + c * dEy_x / dx;
        *ps = v;
        hz = hz - Che * v * dx;
      }
      if (pz >= 0) {  // gpu.h:687-725
        const int64_t t = i + j * sI + pz * sIJ;
        const float b = d.bH[pz], c = d.cH[pz];
        float *ps = d.psi[PSI_HXZ] + t;
        float v = b * *ps + c * dEy_z / dx;
        *ps = v;
        hx = hx + Che * v * dx;
        ps = d.psi[PSI_HYZ] + t;
        v = b * *ps + c * dEx_z / dx;
        *ps = v;
        hy = hy - Che * v * dx;
      }
    }
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
  const int I = d.I, J = d.J, K = d.K, p = d.p;
  if (i >= I || j >= J) return;
  const int kb = blockIdx.z * zchunk;
  const int ke = min(kb + zchunk, K);
  if (kb >= ke) return;
  const int64_t sI = I, sIJ = d.IJ;
  float *__restrict__ Ex = d.f[0];
  float *__restrict__ Ey = d.f[1];
  float *__restrict__ Ez = d.f[2];
  const float *__restrict__ Hx = d.f[3];
  const float *__restrict__ Hy = d.f[4];
  const float *__restrict__ Hz = d.f[5];
  const float dx = d.dx;
  const int mode = op.tfsf_mode;
  const int step = (mode || op.cur_mode) ? op_step(d, op) : 0;
  const float *inc = mode ? inc_e_row(d, mode, step) : nullptr;
  // PML slab positions; the X and Y slabs exclude the first and last
  // planes of the other two axes (gpu.h:776-777, :800-801, :839-840)
  const bool i_in = i >= 1 && i <= I - 2, j_in = j >= 1 && j <= J - 2;
  const int px = (PML && j_in) ? slab_e(i, I, p) : -1;
  const int py = (PML && i_in) ? slab_e(j, J, p) : -1;
  const bool zs = PML && i_in && j_in;
  const int64_t pj = 2 * (int64_t)p;
  // current source (gpu.h:55-82): box clipped to the grid
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
    const bool k_in = k >= 1 && k <= K - 2;
    const int py_k = k_in ? py : -1;
    const int px_k = k_in ? px : -1;
    const int pz = zs ? slab_e(k, K, p) : -1;
    const bool cur = cur_col && in_range(k, op.cur_box[4], op.cur_box[5]);
    if (!CURL) {
      if (!(px_k >= 0 || py_k >= 0 || pz >= 0) && !tfsf_e_touches(d, mode, i, j, k) &&
          !cur)
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
    const Coef6 C = load_coef(d, n, i);
    float ex = Ex[n], ey = Ey[n], ez = Ez[n];
    if (CURL) {
      if (j != 0 && k != 0) ex = C.exe * ex + C.exh * (+(hz - hz_jm) - (hy - hy_km));
      if (i != 0 && k != 0) ey = C.eye * ey + C.eyh * (+(hx - hx_km) - (hz - hz_im));
      if (i != 0 && j != 0) ez = C.eze * ez + C.ezh * (+(hy - hy_im) - (hx - hx_jm));
    }
    if (mode) tfsf_e(d, mode, inc, i, j, k, C.exh, C.eyh, C.ezh, ex, ey, ez);
    if (PML) {
      if (py_k >= 0) {  // gpu.h:790-827
        const int64_t t = i + py_k * sI + k * pj * sI;
        const float b = d.bE[py_k], c = d.cE[py_k];
        float *ps = d.psi[PSI_EXY] + t;
        float v = b * *ps + c * (hz - hz_jm) / dx;
        *ps = v;
        ex = ex + C.exh * v * dx;
        ps = d.psi[PSI_EZY] + t;
        v = b * *ps + c * (hx - hx_jm) / dx;
        *ps = v;
        ez = ez - C.ezh * v * dx;
      }
      if (pz >= 0) {  // gpu.h:829-868
        const int64_t t = i + j * sI + pz * sIJ;
        const float b = d.bE[pz], c = d.cE[pz];
        float *ps = d.psi[PSI_EXZ] + t;
        float v = b * *ps + c * (hy - hy_km) / dx;
        *ps = v;
        ex = ex - C.exh * v * dx;
        ps = d.psi[PSI_EYZ] + t;
        v = b * *ps + c * (hx - hx_km) / dx;
        *ps = v;
        ey = ey + C.eyh * v * dx;
      }
      if (px_k >= 0) {  // gpu.h:765-788
        const int64_t t = px_k + j * pj + k * pj * J;
        const float b = d.bE[px_k], c = d.cE[px_k];
        float *ps = d.psi[PSI_EYX] + t;
        float v = b * *ps + c * (hz - hz_im) / dx;
        *ps = v;
        ey = ey - C.eyh * v * dx;
        ps = d.psi[PSI_EZX] + t;
        v = b * *ps + c * (hy - hy_im) / dx;
        *ps = v;
        ez = ez + C.ezh * v * dx;
      }
    }
    if (cur) {  // E -= Ce?h * source * dx / dx / dx
      if (cm == 1) ex = ex - C.exh * cur_src * dx / dx / dx;
      else if (cm == 2) ey = ey - C.eyh * cur_src * dx / dx / dx;
      else ez = ez - C.ezh * cur_src * dx / dx / dx;
    }
    Ex[n] = ex;
    Ey[n] = ey;
    Ez[n] = ez;
    hx_km = hx;
    hy_km = hy;
  }
}

// --------------------------------------------------------------- probes

// Records the six components at every probe into row *probe_row and
// advances the row (one thread per probe and component).
__global__ void k_probe_gather(const fdtd_dev d) {
  const int row = *d.probe_row;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (row < d.T && t < d.num_ant * 6) {
    const int a = t / 6, c = t - a * 6;
    const int64_t id = d.probe_idx[a];
    d.probes[((int64_t)row * d.num_ant + a) * 6 + c] = id >= 0 ? d.f[c][id] : 0.f;
  }
}

__global__ void k_add_i32(int32_t *p, int32_t v) { *p += v; }
__global__ void k_set_i32(int32_t *p, int32_t v) { *p = v; }

// ------------------------------------------------------ coefficients (setup)

// src/simulation.h:924-938 in the reference's precision: 2*eps0*eps and the
// quotient in double, sigma*delT in float, the result rounded to float.
__global__ void k_compute_ce(float *ce0, float *ce1, float *ce2, float *ce3, float *ce4,
                             float *ce5, const float *eps0_, const float *eps1_,
                             const float *eps2_, const float *sig0, const float *sig1,
                             const float *sig2, const float *den_ex, int64_t IJK, int I,
                             float delT, double two_eps0) {
  float *ce[6] = {ce0, ce1, ce2, ce3, ce4, ce5};
  const float *eps[3] = {eps0_, eps1_, eps2_};
  const float *sig[3] = {sig0, sig1, sig2};
  const float two_dt = 2 * delT;
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < IJK;
       n += (int64_t)gridDim.x * blockDim.x) {
    const double den = (double)den_ex[n % I];
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

// src/simulation.h:43-63: delT/mu0/mu/(1 + sigma_m*delT/2/mu0/mu) * den_hx.
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

// ------------------------------------------------------------ 1D incident

// Forward (block 0, source at S-13) and inverse (block 1, source at 13) runs
// of the auxiliary 1D Ez/Hy grid for all T steps in one launch, replacing
// init1D's 2 x T x 7 launches (src/simulation.h:198-244) of the kernels at
// src/gpu.h:40-53 and :84-149.  The line lives in shared memory when it fits
// (dyn_smem > 0) or in `scratch` (2 x 2 x S floats) otherwise.
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

int fdtdk_half_h(const fdtd_dev *d, const fdtd_op *op, cudaStream_t s) {
  if (op->curl && op->pml) return launch_half(k_half_h<true, true>, d, op, s, d->I - 1, d->J - 1, d->K - 1);
  if (op->curl) return launch_half(k_half_h<true, false>, d, op, s, d->I - 1, d->J - 1, d->K - 1);
  if (op->pml) return launch_half(k_half_h<false, true>, d, op, s, d->I - 1, d->J - 1, d->K - 1);
  if (op->tfsf_mode) return launch_half(k_half_h<false, false>, d, op, s, d->I - 1, d->J - 1, d->K - 1);
  return 0;
}

int fdtdk_half_e(const fdtd_dev *d, const fdtd_op *op, cudaStream_t s) {
  if (op->curl && op->pml) return launch_half(k_half_e<true, true>, d, op, s, d->I, d->J, d->K);
  if (op->curl) return launch_half(k_half_e<true, false>, d, op, s, d->I, d->J, d->K);
  if (op->pml) return launch_half(k_half_e<false, true>, d, op, s, d->I, d->J, d->K);
  if (op->tfsf_mode || op->cur_mode) return launch_half(k_half_e<false, false>, d, op, s, d->I, d->J, d->K);
  return 0;
}

int fdtdk_probe_gather(const fdtd_dev *d, cudaStream_t s) {
  if (d->num_ant <= 0 || !d->probes) return 0;
  const int nt = d->num_ant * 6;
  k_probe_gather<<<(nt + 255) / 256, 256, 0, s>>>(*d);
  k_add_i32<<<1, 1, 0, s>>>(d->probe_row, 1);
  g_launches += 2;
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
  const int blocks = 152 * 8;
  k_compute_ce<<<blocks, 256, 0, s>>>(ce[0], ce[1], ce[2], ce[3], ce[4], ce[5], eps[0],
                                      eps[1], eps[2], sig[0], sig[1], sig[2], den_ex,
                                      d->IJK, d->I, delT, 2 * eps0);
  ++g_launches;
  return (int)cudaGetLastError();
}

int fdtdk_compute_mu(float *out, const float *mu, const float *den_hx, int64_t IJK,
                     int32_t I, float delT, float sigma_m, cudaStream_t s) {
  const double mu0 = 4 * 3.14159265358979323846 * 1e-7;
  k_compute_mu<<<152 * 8, 256, 0, s>>>(out, mu, den_hx, IJK, I, delT, sigma_m, mu0);
  ++g_launches;
  return (int)cudaGetLastError();
}

size_t fdtdk_init_1d_smem_limit(void) { return 160 * 1024; }

int fdtdk_init_1d(const fdtd_dev *d, float *tab[4], const float *pw, float Ceh,
                  float *scratch, cudaStream_t s) {
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
  k_init_1d<<<2, threads, use_smem ? smem : 0, s>>>(*d, tab[0], tab[1], tab[2], tab[3], pw,
                                                    Ceh, scratch, use_smem);
  ++g_launches;
  return (int)cudaGetLastError();
}

unsigned long long fdtdk_launch_count(void) { return g_launches; }

}  // extern "C"
