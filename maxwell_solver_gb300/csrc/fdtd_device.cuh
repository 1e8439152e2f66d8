/*
 * fdtd_device.cuh -- per-cell update functions shared by the direct
 * kernels (fdtd_kernels.cu) and the TMA-pipelined kernels (fdtd_tma.cu).
 *
 * Each function applies, to one cell, the reference's operations in the
 * reference's order (enricoballini/maxwell_solver src/gpu.h): the Yee curl,
 * then the TF/SF face correction, then the CPML axes in the order the
 * reference launches them, then (E only) the current source.  Every
 * operation is rounded separately (the library is built with --fmad=false),
 * so any kernel built from these functions reproduces the reference bit
 * for bit, however it stages its loads.
 */
#pragma once
#include <stdint.h>

#include "fdtd_internal.h"

namespace fdtd {

__device__ __forceinline__ bool in_range(int v, int lo, int hi) { return v >= lo && v <= hi; }

// IEEE quotient a / b, kept out of line of the fast paths below (an asm
// statement is never evaluated speculatively).
__device__ __forceinline__ float div_ieee(float a, float b) {
  float q;
  asm volatile("div.rn.f32 %0, %1, %2;" : "=f"(q) : "f"(a), "f"(b));
  return q;
}

// RN(a / b) for a fixed divisor b with y = RN(1/b): one rounded product and
// Markstein's correction step, q0 = RN(a*y), r = RN(a - b*q0),
// q = RN(q0 + r*y), which the host has shown equal to the IEEE quotient
// for lo <= |a| < hi (fdtd_make_div_plan).  For lo2 <= |a| < lo the same
// is done on a*2^64 and the result scaled back by 2^-64: both scalings are
// exact (the quotient is normal there).  A zero numerator gives a*y = +-0
// = a/b; the rest (tiny, huge, inf, NaN) is divided.
__device__ __forceinline__ float div_by(float a, float b, float y, float lo, float hi,
                                        float lo2) {
  const float aa = fabsf(a);
  const bool small = aa < lo;
  const float as = a * (small ? 0x1p64f : 1.0f);
  const float q0 = as * y;
  const float q = __fmaf_rn(__fmaf_rn(-q0, b, as), y, q0) * (small ? 0x1p-64f : 1.0f);
  if (aa >= lo2 && aa < hi) return q;
  if (aa == 0.f) return a * y;
  return div_ieee(a, b);
}
// RN(a / dx): the CPML recurrences' c * difference / dx.
__device__ __forceinline__ float div_dx(const fdtd_dev &d, float a) {
  return div_by(a, d.dx, d.rdx, d.div_lo, d.div_hi, d.div_lo2);
}

__device__ __forceinline__ float2 *psi_pairs(const fdtd_dev &d, int a) {
  return reinterpret_cast<float2 *>(d.psi[a]);
}

// Slab position of index v in a CPML of thickness p on an axis of length n.
// H cells: low side [0,p) -> v, high side [n-p, n-2] -> v-n+2p
// (src/gpu.h:615-617, :654-656, :698-700).
__device__ __forceinline__ int slab_h(int v, int n, int p) {
  if (v < p) return v;
  if (v >= n - p && v <= n - 2) return v - n + 2 * p;
  return -1;
}
// E cells: low side [1,p) -> v, high side [n-p, n-1] -> v-n+2p
// (src/gpu.h:776-778, :800-802, :839-841).
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
// chx, chy, chz: the Che of each component (the reference's scalar Che, or
// per cell).
__device__ __forceinline__ void tfsf_h(const fdtd_dev &d, int mode, const float *inc, int i,
                                       int j, int k, float &hx, float &hy, float &hz,
                                       float chx, float chy, float chz) {
  const int i0 = d.i0, i1 = d.i1, j0 = d.j0, j1 = d.j1, k0 = d.k0, k1 = d.k1;
  if (mode == 3) {
    if (in_range(i, i0, i1) && in_range(k, k0, k1 - 1)) {
      if (j == j0 - 1) hx = hx + chx * inc[i];
      if (j == j1) hx = hx - chx * inc[i];
    }
    if (in_range(j, j0, j1) && in_range(k, k0, k1 - 1)) {
      if (i == i0 - 1) hy = hy - chy * inc[i0];
      if (i == i1) hy = hy + chy * inc[i1];
    }
  } else if (mode == 4) {
    if (in_range(i, i0, i1) && in_range(j, j0, j1 - 1)) {
      if (k == k0 - 1) hx = hx - chx * inc[i];
      if (k == k1) hx = hx + chx * inc[i];
    }
    if (in_range(j, j0, j1 - 1) && in_range(k, k0, k1)) {
      if (i == i0 - 1) hz = hz + chz * inc[i0];
      if (i == i1) hz = hz - chz * inc[i1];
    }
  } else if (mode == 1) {
    if (in_range(i, i0, i1) && in_range(j, j0, j1 - 1)) {
      if (k == k0 - 1) hx = hx - chx * inc[k0];
      if (k == k1) hx = hx + chx * inc[k1];
    }
    if (in_range(j, j0, j1 - 1) && in_range(k, k0, k1)) {
      if (i == i0 - 1) hz = hz + chz * inc[k];
      if (i == i1) hz = hz - chz * inc[k];
    }
  } else if (mode == 2) {
    if (in_range(i, i0, i1 - 1) && in_range(j, j0, j1)) {
      if (k == k0 - 1) hy = hy + chy * inc[k0];
      if (k == k1) hy = hy - chy * inc[k1];
    }
    if (in_range(i, i0, i1 - 1) && in_range(k, k0, k1)) {
      if (j == j0 - 1) hz = hz - chz * inc[k];
      if (j == j1) hz = hz + chz * inc[k];
    }
  }
}

// E-side TF/SF corrections of one cell.  Modes 1 and 3 are launched with
// c = +1, modes 2 and 4 with c = -1 (src/simulation.h:493-570); x - (a*-1)
// is computed as x + a, which IEEE arithmetic makes identical.
// mode 3 gpu.h:184-214, mode 4 :249-291, mode 1 :479-509, mode 2 :543-573.
__device__ __forceinline__ void tfsf_e(const fdtd_dev &d, int mode, const float *inc, int i,
                                       int j, int k, float cxh, float cyh, float czh,
                                       float &ex, float &ey, float &ez) {
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

// Does the TF/SF of `mode` touch cell (i,j,k)?  (Used by the variants that
// skip the curl and visit only the cells other stages touch.)
__device__ __forceinline__ bool tfsf_h_touches(const fdtd_dev &d, int mode, int i, int j, int k) {
  if (!mode) return false;
  return i == d.i0 - 1 || i == d.i1 || j == d.j0 - 1 || j == d.j1 || k == d.k0 - 1 ||
         k == d.k1;
}
__device__ __forceinline__ bool tfsf_e_touches(const fdtd_dev &d, int mode, int i, int j, int k) {
  if (!mode) return false;
  return i == d.i0 || i == d.i1 || j == d.j0 || j == d.j1 || k == d.k0 || k == d.k1;
}

struct Coef6 {
  float exe, eye, eze, exh, eyh, ezh;
};

__device__ __forceinline__ Coef6 coef_from_table(const fdtd_dev &d, int m) {
  const float *t = d.mat_tab + (int64_t)m * 6;
  Coef6 c;
  c.exe = __ldg(t + 0);
  c.eye = __ldg(t + 1);
  c.eze = __ldg(t + 2);
  c.exh = __ldg(t + 3);
  c.eyh = __ldg(t + 4);
  c.ezh = __ldg(t + 5);
  return c;
}

__device__ __forceinline__ Coef6 coef_from_arrays(const fdtd_dev &d, int64_t n) {
  Coef6 c;
  c.exe = __ldg(d.ce[0] + n);
  c.eye = __ldg(d.ce[1] + n);
  c.eze = __ldg(d.ce[2] + n);
  c.exh = __ldg(d.ce[3] + n);
  c.eyh = __ldg(d.ce[4] + n);
  c.ezh = __ldg(d.ce[5] + n);
  return c;
}

__device__ __forceinline__ Coef6 load_coef(const fdtd_dev &d, int64_t n) {
  return d.coef_mode == 0 ? coef_from_arrays(d, n) : coef_from_table(d, __ldg(d.mat + n));
}

// H update coefficients of one cell: Chh and Che per component.  Uniform
// (the reference's scalars) unless fdtd_set_magnetic gave per-cell ones.
struct HCoef {
  float hhx, hhy, hhz, hex, hey, hez;
};
__device__ __forceinline__ HCoef hcoef_uniform(const fdtd_dev &d) {
  return HCoef{d.Chh, d.Chh, d.Chh, d.Che, d.Che, d.Che};
}
__device__ __forceinline__ HCoef hcoef_at(const fdtd_dev &d, int64_t n) {
  if (d.hcoef_mode == 0) return hcoef_uniform(d);
  if (d.hcoef_mode == 2) {
    const float *t = d.hmat_tab + 6 * (int)__ldg(d.hmat + n);
    return HCoef{__ldg(t), __ldg(t + 1), __ldg(t + 2), __ldg(t + 3), __ldg(t + 4), __ldg(t + 5)};
  }
  const int64_t c = d.cells;
  return HCoef{__ldg(d.hc + n), __ldg(d.hc + c + n), __ldg(d.hc + 2 * c + n),
               __ldg(d.hc + 3 * c + n), __ldg(d.hc + 4 * c + n), __ldg(d.hc + 5 * c + n)};
}
// Che of component comp (0..2) at cell n.
__device__ __forceinline__ float hche_at(const fdtd_dev &d, int64_t n, int comp) {
  if (d.hcoef_mode == 0) return d.Che;
  if (d.hcoef_mode == 2) return __ldg(d.hmat_tab + 6 * (int)__ldg(d.hmat + n) + 3 + comp);
  return __ldg(d.hc + (3 + comp) * d.cells + n);
}

// One CPML axis of a cell's H update: the psi pair's recurrence from its
// old value ps (stored back to *dst) and the field corrections
// (gpu.h:644-685 Y, :604-642 X, :687-725 Z), with the Che of each
// corrected component (the reference's scalar Che, or per cell).
__device__ __forceinline__ void h_corr_y(const fdtd_dev &d, int py, float2 ps, float2 *dst,
                                         float dEz_y, float dEx_y, float &hx, float &hz,
                                         float che_x, float che_z) {
  const float dx = d.dx;  // {psi_Hxy, psi_Hzy}
  const float b = d.bH[py], c = d.cH[py];
  const float v0 = b * ps.x + div_dx(d, c * dEz_y);
  hx = hx - che_x * v0 * dx;
  const float v1 = b * ps.y + div_dx(d, c * dEx_y);
  hz = hz + che_z * v1 * dx;
  *dst = make_float2(v0, v1);
}
// (b, c: the grading at the cell's slab position px; indexed per lane, so
// the callers read them from shared memory where they can)
__device__ __forceinline__ void h_corr_x_bc(const fdtd_dev &d, float b, float c, float2 ps,
                                            float2 *dst, float dEz_x, float dEy_x, float &hy,
                                            float &hz, float che_y, float che_z) {
  const float dx = d.dx;  // {psi_Hyx, psi_Hzx}
  const float v0 = b * ps.x + div_dx(d, c * dEz_x);
  hy = hy + che_y * v0 * dx;
  const float v1 = b * ps.y + div_dx(d, c * dEy_x);
  hz = hz - che_z * v1 * dx;
  *dst = make_float2(v0, v1);
}
__device__ __forceinline__ void h_corr_x(const fdtd_dev &d, int px, float2 ps, float2 *dst,
                                         float dEz_x, float dEy_x, float &hy, float &hz,
                                         float che_y, float che_z) {
  h_corr_x_bc(d, d.bH[px], d.cH[px], ps, dst, dEz_x, dEy_x, hy, hz, che_y, che_z);
}
__device__ __forceinline__ void h_corr_z(const fdtd_dev &d, int pz, float2 ps, float2 *dst,
                                         float dEy_z, float dEx_z, float &hx, float &hy,
                                         float che_x, float che_y) {
  const float dx = d.dx;  // {psi_Hxz, psi_Hyz}
  const float b = d.bH[pz], c = d.cH[pz];
  const float v0 = b * ps.x + div_dx(d, c * dEy_z);
  hx = hx + che_x * v0 * dx;
  const float v1 = b * ps.y + div_dx(d, c * dEx_z);
  hy = hy - che_y * v1 * dx;
  *dst = make_float2(v0, v1);
}

// psi pair addresses of a cell (H and E share the slab layouts).
__device__ __forceinline__ float2 *psi_at_y(const fdtd_dev &d, int a, int i, int py, int k) {
  return psi_pairs(d, a) + (i + py * (int64_t)d.I + k * 2 * (int64_t)d.p * d.I);
}
__device__ __forceinline__ float2 *psi_at_x(const fdtd_dev &d, int a, int px, int j, int k) {
  return psi_pairs(d, a) + (px + j * 2 * (int64_t)d.p + k * 2 * (int64_t)d.p * d.J);
}
__device__ __forceinline__ float2 *psi_at_z(const fdtd_dev &d, int a, int i, int j, int pz) {
  return psi_pairs(d, a) + (i + j * (int64_t)d.I + pz * d.IJ);
}

// New H of one cell from its old H and the six forward E differences:
// curl (gpu.h:575-602), TF/SF, CPML Y (gpu.h:644-685), X (:604-642),
// Z (:687-725).  px/py/pz: H-slab positions (-1 outside).  C: the cell's
// coefficients (hcoef_uniform: the reference's scalars).  xb, xc: the H
// grading tables (d.bH, d.cH, or a shared-memory copy) for the X axis, whose
// slab position differs between the lanes of a warp.
template <bool CURL, bool PML>
__device__ __forceinline__ void update_h_cell(const fdtd_dev &d, const HCoef &C, int mode,
                                              const float *inc, int i, int j, int k, int px,
                                              int py, int pz, float &hx, float &hy, float &hz,
                                              float dEz_y, float dEx_y, float dEz_x,
                                              float dEy_x, float dEy_z, float dEx_z,
                                              const float *xb, const float *xc) {
  if (CURL) {
    hx = C.hhx * hx + C.hex * (-dEz_y + dEy_z);
    hy = C.hhy * hy + C.hey * (-dEx_z + dEz_x);
    hz = C.hhz * hz + C.hez * (-dEy_x + dEx_y);
  }
  if (mode) tfsf_h(d, mode, inc, i, j, k, hx, hy, hz, C.hex, C.hey, C.hez);
  if (PML) {
    // Each psi pair belongs to one cell, so all of the cell's pairs are
    // loaded before its first psi store: one memory round trip.
    const int64_t I = d.I, J = d.J, pj = 2 * (int64_t)d.p;
    float2 *Y = psi_pairs(d, PSI_HY) + (i + py * I + k * pj * I);
    float2 *X = psi_pairs(d, PSI_HX) + (px + j * pj + k * pj * J);
    float2 *Z = psi_pairs(d, PSI_HZ) + (i + j * I + pz * d.IJ);
    float2 y = make_float2(0.f, 0.f), x = y, z = y;
    if (py >= 0) y = *Y;
    if (px >= 0) x = *X;
    if (pz >= 0) z = *Z;
    if (py >= 0) h_corr_y(d, py, y, Y, dEz_y, dEx_y, hx, hz, C.hex, C.hez);
    if (px >= 0) h_corr_x_bc(d, xb[px], xc[px], x, X, dEz_x, dEy_x, hy, hz, C.hey, C.hez);
    if (pz >= 0) h_corr_z(d, pz, z, Z, dEy_z, dEx_z, hx, hy, C.hex, C.hey);
  }
}

// E-slab positions of cell (i,j,k) with the reference's exclusions of the
// first and last planes of the other two axes (gpu.h:776-777, :800-801,
// :839-840).
__device__ __forceinline__ void e_slabs(const fdtd_dev &d, int i, int j, int k, int &px,
                                        int &py, int &pz) {
  const bool i_in = i >= 1 && i <= d.I - 2, j_in = j >= 1 && j <= d.J - 2,
             k_in = k >= 1 && k <= d.K - 2;
  px = (j_in && k_in) ? slab_e(i, d.I, d.p) : -1;
  py = (i_in && k_in) ? slab_e(j, d.J, d.p) : -1;
  pz = (i_in && j_in) ? slab_e(k, d.K, d.p) : -1;
}

// One CPML axis of a cell's E update (gpu.h:790-827 Y, :829-868 Z,
// :765-788 X), as h_corr_*.
__device__ __forceinline__ void e_corr_y(const fdtd_dev &d, int py, float2 ps, float2 *dst,
                                         const Coef6 &C, float hz, float hz_jm, float hx,
                                         float hx_jm, float &ex, float &ez) {
  const float dx = d.dx;  // {psi_Exy, psi_Ezy}
  const float b = d.bE[py], c = d.cE[py];
  const float v0 = b * ps.x + div_dx(d, c * (hz - hz_jm));
  ex = ex + C.exh * v0 * dx;
  const float v1 = b * ps.y + div_dx(d, c * (hx - hx_jm));
  ez = ez - C.ezh * v1 * dx;
  *dst = make_float2(v0, v1);
}
__device__ __forceinline__ void e_corr_z(const fdtd_dev &d, int pz, float2 ps, float2 *dst,
                                         const Coef6 &C, float hy, float hy_km, float hx,
                                         float hx_km, float &ex, float &ey) {
  const float dx = d.dx;  // {psi_Exz, psi_Eyz}
  const float b = d.bE[pz], c = d.cE[pz];
  const float v0 = b * ps.x + div_dx(d, c * (hy - hy_km));
  ex = ex - C.exh * v0 * dx;
  const float v1 = b * ps.y + div_dx(d, c * (hx - hx_km));
  ey = ey + C.eyh * v1 * dx;
  *dst = make_float2(v0, v1);
}
// (b, c: the grading at the cell's slab position px)
__device__ __forceinline__ void e_corr_x_bc(const fdtd_dev &d, float b, float c, float2 ps,
                                            float2 *dst, const Coef6 &C, float hz, float hz_im,
                                            float hy, float hy_im, float &ey, float &ez) {
  const float dx = d.dx;  // {psi_Eyx, psi_Ezx}
  const float v0 = b * ps.x + div_dx(d, c * (hz - hz_im));
  ey = ey - C.eyh * v0 * dx;
  const float v1 = b * ps.y + div_dx(d, c * (hy - hy_im));
  ez = ez + C.ezh * v1 * dx;
  *dst = make_float2(v0, v1);
}
__device__ __forceinline__ void e_corr_x(const fdtd_dev &d, int px, float2 ps, float2 *dst,
                                         const Coef6 &C, float hz, float hz_im, float hy,
                                         float hy_im, float &ey, float &ez) {
  e_corr_x_bc(d, d.bE[px], d.cE[px], ps, dst, C, hz, hz_im, hy, hy_im, ey, ez);
}

// New E of one cell: curl with the reference's guards (gpu.h:727-763),
// TF/SF, CPML Y (gpu.h:790-827), Z (:829-868), X (:765-788), then the
// current source (gpu.h:55-82) when `cur` is set.
template <bool CURL, bool PML>
__device__ __forceinline__ void update_e_cell(const fdtd_dev &d, int mode, const float *inc,
                                              int cur_mode, float cur_src, bool cur, int i,
                                              int j, int k, int px, int py, int pz,
                                              const Coef6 &C, float &ex, float &ey, float &ez,
                                              float hx, float hy, float hz, float hz_jm,
                                              float hx_jm, float hz_im, float hy_im,
                                              float hx_km, float hy_km) {
  const float dx = d.dx;
  if (CURL) {
    if (j != 0 && k != 0) ex = C.exe * ex + C.exh * (+(hz - hz_jm) - (hy - hy_km));
    if (i != 0 && k != 0) ey = C.eye * ey + C.eyh * (+(hx - hx_km) - (hz - hz_im));
    if (i != 0 && j != 0) ez = C.eze * ez + C.ezh * (+(hy - hy_im) - (hx - hx_jm));
  }
  if (mode) tfsf_e(d, mode, inc, i, j, k, C.exh, C.eyh, C.ezh, ex, ey, ez);
  if (PML) {
    // all psi pairs of the cell first (see update_h_cell)
    const int64_t I = d.I, J = d.J, pj = 2 * (int64_t)d.p;
    float2 *Y = psi_pairs(d, PSI_EY) + (i + py * I + k * pj * I);
    float2 *Z = psi_pairs(d, PSI_EZ) + (i + j * I + pz * d.IJ);
    float2 *X = psi_pairs(d, PSI_EX) + (px + j * pj + k * pj * J);
    float2 y = make_float2(0.f, 0.f), z = y, x = y;
    if (py >= 0) y = *Y;
    if (pz >= 0) z = *Z;
    if (px >= 0) x = *X;
    if (py >= 0) e_corr_y(d, py, y, Y, C, hz, hz_jm, hx, hx_jm, ex, ez);
    if (pz >= 0) e_corr_z(d, pz, z, Z, C, hy, hy_km, hx, hx_km, ex, ey);
    if (px >= 0) e_corr_x(d, px, x, X, C, hz, hz_im, hy, hy_im, ey, ez);
  }
  if (cur) {  // E -= Ce?h * source * dx / dx / dx
    if (cur_mode == 1) ex = ex - C.exh * cur_src * dx / dx / dx;
    else if (cur_mode == 2) ey = ey - C.eyh * cur_src * dx / dx / dx;
    else ez = ez - C.ezh * cur_src * dx / dx / dx;
  }
}

}  // namespace fdtd
