/*
 * fdtd_oracle.c -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of the reference's 3D Yee FDTD step loop
 * (enricoballini/maxwell_solver, src/simulation.h + src/gpu.h).  It is the
 * checker the CUDA product is compared against; nothing in the product links
 * it.  Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline /
 * reference legs load it.
 *
 * Every routine follows one reference routine (cited file:line) with the same
 * index ranges, guards, update order and float/double mixing, so that an
 * FP32 build reproduces the reference bit for bit when both are compiled
 * without FMA contraction (-ffp-contract=off).  The file is compiled twice:
 *   OR_REAL=float  -> symbols ora_f32_*   (parity oracle)
 *   OR_REAL=double -> symbols ora_f64_*   (error floor)
 *
 * Pinning: tests/golden/ holds vectors produced by the reference's own
 * sources built for the host (oracle/ref_build.sh -> oracle/_ref/), and
 * tests/test_oracle_golden.py checks this file against them.
 *
 * Extensions over the reference (all default to the reference's constants):
 * runtime CPML thickness / grading, TF/SF inset, a probe gather that
 * records (Ex,Ey,Ez,Hx,Hy,Hz) at each probe at the start of every step, and
 * TF/SF mode 5, an oblique plane wave (set_incidence): a 1D line along the
 * propagation direction with its speed matched to the 3D grid's numerical
 * phase velocity there, the incident field linearly interpolated from it at
 * every Yee position of the six faces, faces corrected axis by axis (x, y,
 * z).  It has no reference counterpart; it restates the library's mode 5.
 */
#define _GNU_SOURCE
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef OR_REAL
#define OR_REAL float
#define OR_SUFFIX f32
#endif

#define OR_CAT2(a, b) a##_##b
#define OR_CAT(a, b) OR_CAT2(a, b)
#define OR(name) OR_CAT(OR_CAT(ora, OR_SUFFIX), name)

typedef OR_REAL real;

/* Physical constants: src/simulation.h:19-21 (glibc M_PI). */
static const double k_c0 = 299792458;
#define K_MU0 (4 * 3.14159265358979323846 * 1e-7)
#define K_EPS0 (1 / k_c0 / k_c0 / K_MU0)

enum { F_EX = 0, F_EY, F_EZ, F_HX, F_HY, F_HZ };
/* psi slots, named as in src/simulation.h:1298-1312 */
enum {
  P_EXY = 0, P_EXZ, P_EYX, P_EYZ, P_EZX, P_EZY,
  P_HXY, P_HXZ, P_HYX, P_HYZ, P_HZX, P_HZY, P_COUNT
};

typedef struct {
  int pml;          /* CPML thickness (reference: constexpr 10) */
  int tfsf_width;   /* TF/SF inset (reference: 15) */
  double poly_m, alpha_m, alpha_max, kappa_max, sig_factor, r0;
} or_params;

typedef struct or_sim {
  or_params prm;
  int init_const, init_ready, init_1d, init_src, init_ant;
  size_t I, J, K, IJ, IJK, T, numAnt, p;
  real fctr, delX, delT;
  real poly_m, alpha_m, sig_max, alpha_max, kappa_max;
  size_t i0, i1, j0, j1, k0, k1;
  size_t size_x, size_y, size_z;
  real *eps[3], *sig[3];
  real *bE, *cE, *bH, *cH;
  real *den_ex, *den_hx; /* per x index: x-only in the reference */
  real Chh, Che;
  real *Ce[6]; /* Cexe Ceye Ceze Cexh Ceyh Cezh */
  real *f[6];  /* Ex Ey Ez Hx Hy Hz */
  real *psi[P_COUNT];
  real *src;
  size_t size1d;
  real *Ez1d, *Hy1d, *Einv1d, *Hinv1d;
  size_t *ant_idx;
  real *probes; /* [T][numAnt][6] */
  /* TF/SF mode 5 */
  int has_ob;
  double ob_theta, ob_phi, ob_psi;
  real ob_k[3], ob_e[3], ob_h[3], ob_x0, ob_rho;
  long ob_r0[3];
  size_t ob_w;
  real *obE, *obH; /* [T][ob_w] */
  /* extension: per-cell H coefficients (set_magnetic) -- Chh x, y, z, then
   * Che x, y, z; NULL: the scalar Chh, Che */
  real *hc[6];
} or_sim;

/* H coefficients of component a (0..2) at cell n */
#define CHH(a, n) (s->hc[a] ? s->hc[a][n] : s->Chh)
#define CHE(a, n) (s->hc[3 + (a)] ? s->hc[3 + (a)][n] : s->Che)

static void *xcalloc(size_t n, size_t sz) {
  void *p = calloc(n ? n : 1, sz);
  if (!p) {
    fprintf(stderr, "oracle: out of memory\n");
    abort();
  }
  return p;
}

/* OpenMP threads of the oracle's loops: set (n >= 1) and read back. */
void OR(set_threads)(int n) {
#ifdef _OPENMP
  if (n >= 1) omp_set_num_threads(n);
#else
  (void)n;
#endif
}
int OR(threads)(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

or_sim *OR(create)(void) {
  or_sim *s = (or_sim *)xcalloc(1, sizeof(or_sim));
  s->prm.pml = 10;
  s->prm.tfsf_width = 15;
  s->prm.poly_m = 3;
  s->prm.alpha_m = 1.0;
  s->prm.alpha_max = 0.08;
  s->prm.kappa_max = 1.0;
  s->prm.sig_factor = 0.8;
  s->prm.r0 = 0.0;
  return s;
}

void OR(destroy)(or_sim *s) {
  if (!s) return;
  for (int a = 0; a < 3; ++a) { free(s->eps[a]); free(s->sig[a]); }
  free(s->bE); free(s->cE); free(s->bH); free(s->cH);
  free(s->den_ex); free(s->den_hx);
  for (int a = 0; a < 6; ++a) { free(s->Ce[a]); free(s->f[a]); }
  for (int a = 0; a < P_COUNT; ++a) free(s->psi[a]);
  free(s->src);
  free(s->Ez1d); free(s->Hy1d); free(s->Einv1d); free(s->Hinv1d);
  free(s->ant_idx); free(s->probes);
  free(s->obE); free(s->obH);
  for (int a = 0; a < 6; ++a) free(s->hc[a]);
  free(s);
}

int OR(set_incidence)(or_sim *s, double theta, double phi, double psi) {
  if (!s->init_const || s->init_1d) return -1;
  s->has_ob = 1;
  s->ob_theta = theta;
  s->ob_phi = phi;
  s->ob_psi = psi;
  return 0;
}

/* Extension: per-cell magnetic media (what createMu, src/simulation.h:28-68,
 * sets out to do): mu_r and magnetic conductivity sigma_m (sm may be NULL)
 * per H component; in double, rounded once:
 * q = sm delT / 2 / mu0 / mu_r, Chh = (1 - q) / (1 + q),
 * Che = delT / mu0 / mu_r / (1 + q) / delX.  After ready_simulation. */
int OR(set_magnetic)(or_sim *s, const float *mu_x, const float *mu_y, const float *mu_z,
                     const float *sm_x, const float *sm_y, const float *sm_z) {
  if (!s->init_ready) return -1;
  const float *mu[3] = {mu_x, mu_y, mu_z}, *sm[3] = {sm_x, sm_y, sm_z};
  const double dt = (double)s->delT, dx = (double)s->delX;
  for (int a = 0; a < 3; ++a) {
    if (!s->hc[a]) s->hc[a] = (real *)xcalloc(s->IJK, sizeof(real));
    if (!s->hc[3 + a]) s->hc[3 + a] = (real *)xcalloc(s->IJK, sizeof(real));
    for (size_t i = 0; i < s->IJK; ++i) {
      const double m = (double)mu[a][i];
      const double q = (sm[a] ? (double)sm[a][i] : 0.0) * dt / 2 / K_MU0 / m;
      s->hc[a][i] = (real)((1 - q) / (1 + q));
      s->hc[3 + a][i] = (real)(dt / K_MU0 / m / (1 + q) / dx);
    }
  }
  return 0;
}

/* Extension: CPML / TF/SF parameters; must precede set_const. */
int OR(set_params)(or_sim *s, int pml, int tfsf_width, double poly_m,
                   double alpha_m, double alpha_max, double kappa_max,
                   double sig_factor, double r0) {
  if (s->init_const) return -1;
  if (pml < 2) return -2;
  s->prm.pml = pml;
  s->prm.tfsf_width = tfsf_width;
  s->prm.poly_m = poly_m;
  s->prm.alpha_m = alpha_m;
  s->prm.alpha_max = alpha_max;
  s->prm.kappa_max = kappa_max;
  s->prm.sig_factor = sig_factor;
  s->prm.r0 = r0;
  return 0;
}

/* src/simulation.h:79-131 (setConst) */
int OR(set_const)(or_sim *s, const float *freqRes, const int32_t *timeDim) {
  if (s->init_const) return -1;
  s->fctr = (real)freqRes[0];
  s->delX = (real)freqRes[1];
  s->delT = (real)freqRes[2];
  s->poly_m = (real)s->prm.poly_m;
  s->alpha_m = (real)s->prm.alpha_m;
  if (s->prm.r0 > 0.0)
    s->sig_max = (real)(-((double)s->poly_m + 1.0) * log(s->prm.r0) /
                        (2.0 * sqrt(K_MU0 / K_EPS0) * (double)s->prm.pml *
                         (double)s->delX));
  else
    s->sig_max = (real)(s->prm.sig_factor * ((double)s->poly_m + 1.0) /
                        (sqrt(K_MU0 / K_EPS0) * (double)s->delX));
  s->alpha_max = (real)s->prm.alpha_max;
  s->kappa_max = (real)s->prm.kappa_max;
  s->T = (size_t)timeDim[0];
  s->I = (size_t)timeDim[1];
  s->J = (size_t)timeDim[2];
  s->K = (size_t)timeDim[3];
  s->numAnt = (size_t)timeDim[4];
  s->p = (size_t)s->prm.pml;
  s->IJ = s->I * s->J;
  s->IJK = s->IJ * s->K;
  size_t w = (size_t)s->prm.tfsf_width;
  s->i0 = w; s->i1 = s->I - w - 1;
  s->j0 = w; s->j1 = s->J - w - 1;
  s->k0 = w; s->k1 = s->K - w - 1;
  s->size_x = s->p * s->J * s->K;
  s->size_y = s->I * s->p * s->K;
  s->size_z = s->I * s->J * s->p;
  for (int a = 0; a < 3; ++a) {
    s->eps[a] = (real *)xcalloc(s->IJK, sizeof(real));
    s->sig[a] = (real *)xcalloc(s->IJK, sizeof(real));
    for (size_t n = 0; n < s->IJK; ++n) s->eps[a][n] = (real)1.0;
  }
  s->init_const = 1;
  return 0;
}

/* src/simulation.h:1068-1082 (setSource) and :1084-1095 (updateSource) */
int OR(set_source)(or_sim *s, const float *in) {
  if (!s->src) s->src = (real *)xcalloc(s->T, sizeof(real));
  for (size_t n = 0; n < s->T; ++n) s->src[n] = (real)in[n];
  s->init_src = 1;
  return 0;
}

/* src/simulation.h:288-328 (updateMaterial): flag 1..3 sigma, 4..6 eps */
int OR(update_material)(or_sim *s, int flag, const float *values) {
  real *dst = NULL;
  if (flag >= 1 && flag <= 3) dst = s->sig[flag - 1];
  else if (flag >= 4 && flag <= 6) dst = s->eps[flag - 4];
  if (!dst) return 0;
  for (size_t n = 0; n < s->IJK; ++n) dst[n] = (real)values[n];
  return 0;
}

/* src/simulation.h:1047-1067 (setAntennaLocations): numAnt x 3 column-major,
 * each coordinate offset by the CPML thickness. */
int OR(set_antenna_locations)(or_sim *s, const int32_t *loc) {
  free(s->ant_idx);
  s->ant_idx = (size_t *)xcalloc(s->numAnt, sizeof(size_t));
  for (size_t a = 0; a < s->numAnt; ++a) {
    size_t x = s->p + (size_t)loc[a + 0 * s->numAnt];
    size_t y = s->p + (size_t)loc[a + 1 * s->numAnt];
    size_t z = s->p + (size_t)loc[a + 2 * s->numAnt];
    s->ant_idx[a] = x + y * s->I + z * s->IJ;
  }
  s->init_ant = 1;
  return 0;
}

/* Per-cell E coefficients: src/simulation.h:924-938 (== updateCuda :1099-1113).
 * Mixed precision exactly as the reference: 2*eps0*eps in double, sigma*delT
 * in real, the quotient in double, stored as real. */
static void compute_ce(or_sim *s) {
  const double eps0 = K_EPS0;
  const real dt = s->delT;
  const real two_dt = (real)(2 * dt);
#pragma omp parallel for schedule(static)
  for (long long kk = 0; kk < (long long)s->K; ++kk) {
    for (size_t j = 0; j < s->J; ++j) {
      for (size_t i = 0; i < s->I; ++i) {
        size_t n = i + j * s->I + (size_t)kk * s->IJ;
        for (int a = 0; a < 3; ++a) {
          real sd = (real)(s->sig[a][n] * dt);
          double two_eps = 2 * eps0 * (double)s->eps[a][n];
          s->Ce[a][n] = (real)((two_eps - (double)sd) / (two_eps + (double)sd));
          s->Ce[3 + a][n] =
              (real)((double)two_dt / (two_eps + (double)sd) * (double)s->den_ex[i]);
        }
      }
    }
  }
}

/* One CPML grading sample: src/simulation.h:730-749 (E) and :752-767 (H). */
static void cpml_sample(const or_sim *s, double num_sig, double num_alpha,
                        real *sig, real *alpha, real *kappa) {
  const double pm1 = (double)s->p - 1.0;
  *sig = (real)((double)s->sig_max * pow(num_sig / pm1, (double)s->poly_m));
  *alpha = (real)((double)s->alpha_max * pow(num_alpha / pm1, (double)s->alpha_m));
  *kappa = (real)(1.0 + ((double)s->kappa_max - 1.0) *
                            pow(num_sig / pm1, (double)s->poly_m));
}

static real cpml_b(const or_sim *s, real sig, real alpha, real kappa) {
  real t = sig / kappa;
  t = t + alpha;
  t = -t;
  t = t * s->delT;
  return (real)exp((double)t / K_EPS0);
}

static real cpml_c(real sig, real alpha, real kappa, real b) {
  real u1 = sig / kappa;
  real u2 = kappa * alpha;
  real u3 = sig + u2;
  real u4 = u1 / u3;
  return (real)((double)u4 * ((double)b - 1.0));
}

/* src/simulation.h:640-979 (readySimulation) incl. initField :980-1045 */
int OR(ready_simulation)(or_sim *s) {
  const size_t p = s->p;
  real *sigE = (real *)xcalloc(p, sizeof(real));
  real *alE = (real *)xcalloc(p, sizeof(real));
  real *kaE = (real *)xcalloc(p, sizeof(real));
  real *sigH = (real *)xcalloc(p, sizeof(real));
  real *alH = (real *)xcalloc(p, sizeof(real));
  real *kaH = (real *)xcalloc(p, sizeof(real));
  real *bE1 = (real *)xcalloc(p, sizeof(real)), *cE1 = (real *)xcalloc(p, sizeof(real));
  real *bH1 = (real *)xcalloc(p, sizeof(real)), *cH1 = (real *)xcalloc(p, sizeof(real));
  s->bE = (real *)xcalloc(2 * p, sizeof(real));
  s->cE = (real *)xcalloc(2 * p, sizeof(real));
  s->bH = (real *)xcalloc(2 * p, sizeof(real));
  s->cH = (real *)xcalloc(2 * p, sizeof(real));
  /* E grading, :730-749, incl. the (never-taken) zero-c guard at :742-744 */
  for (size_t i = 0; i < p; ++i) {
    cpml_sample(s, (double)(p - i - 1), (double)(i + 1) - 1.0, &sigE[i], &alE[i], &kaE[i]);
    bE1[i] = cpml_b(s, sigE[i], alE[i], kaE[i]);
    if (sigE[i] == 0.0 && alE[i] == 0.0 && (i + 1) == (p - 1))
      cE1[i] = 0;
    else
      cE1[i] = cpml_c(sigE[i], alE[i], kaE[i], bE1[i]);
  }
  /* H grading at half-cell offsets, p-1 entries, :752-767 */
  for (size_t i = 0; i + 1 < p; ++i) {
    cpml_sample(s, (double)(p - i - 1) - 0.5, (double)(i + 1) - 0.5, &sigH[i], &alH[i], &kaH[i]);
    bH1[i] = cpml_b(s, sigH[i], alH[i], kaH[i]);
    cH1[i] = cpml_c(sigH[i], alH[i], kaH[i], bH1[i]);
  }
  /* Assemble [low | reversed high], :772-822.  The H table keeps zeros at
   * p-1 and 2p-1 (fill at :701-703). */
  for (size_t i = 0; i < p; ++i) {
    s->bE[i] = bE1[i];
    s->cE[i] = cE1[i];
    s->bE[p + i] = bE1[p - 1 - i];
    s->cE[p + i] = cE1[p - 1 - i];
  }
  for (size_t i = 0; i + 1 < p; ++i) {
    s->bH[i] = bH1[i];
    s->cH[i] = cH1[i];
    s->bH[p + i] = bH1[p - 2 - i];
    s->cH[p + i] = cH1[p - 2 - i];
  }
  /* x-only stretch denominators, :861-912; zero at i = I-1 (fill :714-715) */
  s->den_ex = (real *)xcalloc(s->I, sizeof(real));
  s->den_hx = (real *)xcalloc(s->I, sizeof(real));
  {
    size_t ii = p - 2;
    for (size_t i = 0; i + 1 < s->I; ++i) {
      if (i < p - 1) {
        s->den_hx[i] = (real)(1.0 / (double)(real)(s->delX * kaH[i]));
      } else if (i >= s->I - p) {
        /* kappa_Hx_PML_2 holds the same values as kappa_Hx_PML_1 */
        s->den_hx[i] = (real)(1.0 / (double)(real)(s->delX * kaH[ii]));
        ii = ii - 1;
      } else {
        s->den_hx[i] = (real)(1.0 / (double)s->delX);
      }
    }
    ii = p - 1;
    for (size_t i = 0; i + 1 < s->I; ++i) {
      if (i < p) {
        s->den_ex[i] = (real)(1.0 / (double)(real)(s->delX * kaE[i]));
      } else if (i >= s->I - p) {
        s->den_ex[i] = (real)(1.0 / (double)(real)(s->delX * kaE[ii]));
        ii = ii - 1;
      } else {
        s->den_ex[i] = (real)(1.0 / (double)s->delX);
      }
    }
  }
  /* Scalar H coefficients, :914-922 (sigma_m = 0) */
  {
    real sigma_m = 0;
    real t = (real)(sigma_m * s->delT);
    t = t / 2;
    double q = (double)t / K_MU0;
    s->Chh = (real)((1 - q) / (1 + q));
    s->Che = (real)((double)s->delT / K_MU0 / (1 + q) / (double)s->delX);
  }
  for (int a = 0; a < 6; ++a) s->Ce[a] = (real *)xcalloc(s->IJK, sizeof(real));
  compute_ce(s);
  /* probe buffer, :954-963 (only if antennas were set first) */
  if (s->init_ant) s->probes = (real *)xcalloc(s->T * s->numAnt * 6, sizeof(real));
  /* initField, :980-1045 */
  for (int a = 0; a < 6; ++a) s->f[a] = (real *)xcalloc(s->IJK, sizeof(real));
  s->psi[P_EXY] = (real *)xcalloc(2 * s->size_y, sizeof(real));
  s->psi[P_EZY] = (real *)xcalloc(2 * s->size_y, sizeof(real));
  s->psi[P_HXY] = (real *)xcalloc(2 * s->size_y, sizeof(real));
  s->psi[P_HZY] = (real *)xcalloc(2 * s->size_y, sizeof(real));
  s->psi[P_EXZ] = (real *)xcalloc(2 * s->size_z, sizeof(real));
  s->psi[P_EYZ] = (real *)xcalloc(2 * s->size_z, sizeof(real));
  s->psi[P_HXZ] = (real *)xcalloc(2 * s->size_z, sizeof(real));
  s->psi[P_HYZ] = (real *)xcalloc(2 * s->size_z, sizeof(real));
  s->psi[P_EYX] = (real *)xcalloc(2 * s->size_x, sizeof(real));
  s->psi[P_EZX] = (real *)xcalloc(2 * s->size_x, sizeof(real));
  s->psi[P_HYX] = (real *)xcalloc(2 * s->size_x, sizeof(real));
  s->psi[P_HZX] = (real *)xcalloc(2 * s->size_x, sizeof(real));
  free(sigE); free(alE); free(kaE); free(sigH); free(alH); free(kaH);
  free(bE1); free(cE1); free(bH1); free(cH1);
  s->init_ready = 1;
  return 0;
}

/* src/simulation.h:1097-1127 (updateCuda) */
int OR(update_cuda)(or_sim *s) {
  compute_ce(s);
  return 0;
}

/* src/simulation.h:1128-1151 (ResetFieldAll) */
int OR(reset_field_all)(or_sim *s) {
  for (int a = 0; a < 6; ++a) memset(s->f[a], 0, s->IJK * sizeof(real));
  const size_t sizes[P_COUNT] = {
      [P_EXY] = 2 * s->size_y, [P_EZY] = 2 * s->size_y, [P_HXY] = 2 * s->size_y,
      [P_HZY] = 2 * s->size_y, [P_EXZ] = 2 * s->size_z, [P_EYZ] = 2 * s->size_z,
      [P_HXZ] = 2 * s->size_z, [P_HYZ] = 2 * s->size_z, [P_EYX] = 2 * s->size_x,
      [P_EZX] = 2 * s->size_x, [P_HYX] = 2 * s->size_x, [P_HZX] = 2 * s->size_x};
  for (int a = 0; a < P_COUNT; ++a) memset(s->psi[a], 0, sizes[a] * sizeof(real));
  return 0;
}

/* ---------------------------------------------------------------- 1D grid */

/* One run of the auxiliary 1D Ez/Hy grid, src/simulation.h:198-217 (forward,
 * source at size_1D-13) and :222-244 (inverse, source at 13), with the 1D
 * kernels of src/gpu.h:40-53 and :84-149. */
static void run_1d(or_sim *s, real *Estore, real *Hstore, size_t src_at,
                   const real *pw) {
  const size_t S = s->size1d, p = s->p;
  real *E = (real *)xcalloc(S, sizeof(real));
  real *H = (real *)xcalloc(S, sizeof(real));
  real *psiE = (real *)xcalloc(2 * p, sizeof(real));
  real *psiH = (real *)xcalloc(2 * p, sizeof(real));
  const real Che = s->Che;
  const real Ceh = (real)((double)s->delT / K_EPS0 / (double)s->delX);
  const real dx = s->delX;
  for (size_t n = 0; n < s->T; ++n) {
    memcpy(Estore + n * S, E, S * sizeof(real));                  /* copy1d */
    for (size_t t = 0; t + 1 < S; ++t) H[t] = H[t] + Che * (E[t + 1] - E[t]);
    for (size_t t = 0; t < 2 * p; ++t) {                          /* :84-107 */
      int c1 = t < p, c2 = (t < 2 * p - 1) && (t >= p);
      if (!(c1 || c2)) continue;
      size_t idx = c1 ? t : t + S - 2 * p;
      real q = s->cH[t] * (E[idx + 1] - E[idx]);
      psiH[t] = s->bH[t] * psiH[t] + q / dx;
      H[idx] = H[idx] + Che * psiH[t] * dx;
    }
    for (size_t t = 1; t < S; ++t) E[t] = E[t] + Ceh * (H[t] - H[t - 1]);
    for (size_t t = 0; t < 2 * p; ++t) {                          /* :109-132 */
      int c1 = (t > 0) && (t < p), c2 = (t < 2 * p) && (t >= p);
      if (!(c1 || c2)) continue;
      size_t idx = c1 ? t : t + S - 2 * p;
      real q = s->cE[t] * (H[idx] - H[idx - 1]);
      psiE[t] = s->bE[t] * psiE[t] + q / dx;
      E[idx] = E[idx] + Ceh * psiE[t] * dx;
    }
    E[src_at] = E[src_at] + pw[n];                                /* :48-53 */
    memcpy(Hstore + n * S, H, S * sizeof(real));
  }
  free(E); free(H); free(psiE); free(psiH);
}

/* Mode 5: numerical wavenumber of the 3D grid in direction n at angular
 * frequency w, sum_a sin^2(k n_a dx/2) = (dx/(c dt))^2 sin^2(w dt/2). */
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

/* Mode 5: the 1D line (E at nodes, H at half nodes) for all T steps; the
 * window [mb, mb + ob_w) of E before each step and of H after its H
 * update. */
static void init_1d_oblique(or_sim *s, const real *pw) {
  const double t = s->ob_theta, p = s->ob_phi, q = s->ob_psi;
  const double k[3] = {sin(t) * cos(p), sin(t) * sin(p), cos(t)};
  const double th[3] = {cos(t) * cos(p), cos(t) * sin(p), -sin(t)}, ph[3] = {-sin(p), cos(p), 0};
  double e[3], hv[3];
  for (int a = 0; a < 3; ++a) e[a] = cos(q) * th[a] + sin(q) * ph[a];
  hv[0] = k[1] * e[2] - k[2] * e[1];
  hv[1] = k[2] * e[0] - k[0] * e[2];
  hv[2] = k[0] * e[1] - k[1] * e[0];
  const size_t lo[3] = {s->i0, s->j0, s->k0}, hi[3] = {s->i1, s->j1, s->k1};
  double span = 0.0;
  for (int a = 0; a < 3; ++a) {
    s->ob_k[a] = (real)k[a];
    s->ob_e[a] = (real)e[a];
    s->ob_h[a] = (real)hv[a];
    s->ob_r0[a] = (long)(k[a] >= 0 ? lo[a] : hi[a]);
    span += fabs(k[a]) * (double)(hi[a] - lo[a]);
  }
  const double dx = (double)(float)s->delX, dt = (double)(float)s->delT;
  double dx1 = dx * sqrt(pow(k[0], 4) + pow(k[1], 4) + pow(k[2], 4));
  if (k_c0 * dt / dx1 > 0.995) dx1 = k_c0 * dt / 0.995;
  double speed = 1.0;
  const double w = 2.0 * 3.14159265358979323846 * (double)(float)s->fctr;
  if (w > 0) {
    const double kn = yee_wavenumber(k, w, dx, dt);
    const double sk = sin(kn * dx1 / 2);
    if (sk > 0) speed = sin(w * dt / 2) * dx1 / (k_c0 * dt * sk);
  }
  if (speed * k_c0 * dt / dx1 > 0.999) speed = 0.999 * dx1 / (k_c0 * dt);
  const float rho = (float)(dx / dx1);
  s->ob_rho = (real)rho;
  s->ob_x0 = (real)(4.0f * rho);
  s->ob_w = (size_t)ceil((span + 2.6) * dx / dx1 + 4.0 * rho) + 4;
  const size_t T = s->T, W = s->ob_w;
  const size_t m_src = T + 8, mb = m_src + 2, n1 = mb + W + T + 8;
  const real cE = (real)(speed * dt / K_EPS0 / dx1), cH = (real)(speed * dt / K_MU0 / dx1);
  const real gain = (real)(float)(speed * dx / dx1); /* source strength per line Courant */
  real *E = (real *)xcalloc(n1, sizeof(real)), *H = (real *)xcalloc(n1, sizeof(real));
  free(s->obE); free(s->obH);
  s->obE = (real *)xcalloc(T * W, sizeof(real));
  s->obH = (real *)xcalloc(T * W, sizeof(real));
  for (size_t n = 0; n < T; ++n) {
    memcpy(s->obE + n * W, E + mb, W * sizeof(real));
    for (size_t m = 0; m + 1 < n1; ++m) H[m] = H[m] - cH * (E[m + 1] - E[m]);
    memcpy(s->obH + n * W, H + mb, W * sizeof(real));
    for (size_t m = 1; m + 1 < n1; ++m) E[m] = E[m] - cE * (H[m] - H[m - 1]);
    E[m_src] = E[m_src] + pw[n] * gain;
  }
  free(E); free(H);
}

/* src/simulation.h:134-254 (init1D) */
int OR(init_1d)(or_sim *s, float rate, const float *pw_source) {
  size_t S = s->I;
  if (s->J > S) S = s->J;
  if (s->K > S) S = s->K;
  s->size1d = S;
  free(s->Ez1d); free(s->Hy1d); free(s->Einv1d); free(s->Hinv1d);
  s->Ez1d = (real *)xcalloc(s->T * S, sizeof(real));
  s->Hy1d = (real *)xcalloc(s->T * S, sizeof(real));
  s->Einv1d = (real *)xcalloc(s->T * S, sizeof(real));
  s->Hinv1d = (real *)xcalloc(s->T * S, sizeof(real));
  real *pw = (real *)xcalloc(s->T, sizeof(real));
  for (size_t n = 0; n < s->T; ++n) pw[n] = (real)((real)pw_source[n] * (real)rate);
  /* sources at S-13 / 13 for the reference's 10-cell CPML: 3 cells inside
   * the 1D CPML, kept so for other thicknesses (extension) */
  run_1d(s, s->Ez1d, s->Hy1d, S - (s->p + 3), pw);
  run_1d(s, s->Einv1d, s->Hinv1d, s->p + 3, pw);
  if (s->has_ob) init_1d_oblique(s, pw);
  free(pw);
  s->init_1d = 1;
  return 0;
}

/* ------------------------------------------------------------ 3D kernels */

#define IDX(i, j, k) ((i) + (j)*s->I + (k)*s->IJ)

/* src/gpu.h:575-602 (GPU_updateH), launched by src/simulation.h:371-385 */
void OR(update_h_all)(or_sim *s) {
  real *Hx = s->f[F_HX], *Hy = s->f[F_HY], *Hz = s->f[F_HZ];
  const real *Ex = s->f[F_EX], *Ey = s->f[F_EY], *Ez = s->f[F_EZ];
  const size_t I = s->I, IJ = s->IJ;
#pragma omp parallel for schedule(static)
  for (long long kk = 0; kk < (long long)s->K - 1; ++kk)
    for (size_t j = 0; j + 1 < s->J; ++j)
      for (size_t i = 0; i + 1 < s->I; ++i) {
        size_t n = i + j * I + (size_t)kk * IJ;
        real ez = Ez[n], ey = Ey[n], ex = Ex[n];
        Hx[n] = CHH(0, n) * Hx[n] + CHE(0, n) * (-(Ez[n + I] - ez) + (Ey[n + IJ] - ey));
        Hy[n] = CHH(1, n) * Hy[n] + CHE(1, n) * (-(Ex[n + IJ] - ex) + (Ez[n + 1] - ez));
        Hz[n] = CHH(2, n) * Hz[n] + CHE(2, n) * (-(Ey[n + 1] - ey) + (Ex[n + I] - ex));
      }
}

/* src/gpu.h:727-763 (GPU_updateE), launched by src/simulation.h:386-391 */
void OR(update_e_all)(or_sim *s) {
  real *Ex = s->f[F_EX], *Ey = s->f[F_EY], *Ez = s->f[F_EZ];
  const real *Hx = s->f[F_HX], *Hy = s->f[F_HY], *Hz = s->f[F_HZ];
  real *const *C = s->Ce;
  const size_t I = s->I, IJ = s->IJ;
#pragma omp parallel for schedule(static)
  for (long long kk = 0; kk < (long long)s->K; ++kk)
    for (size_t j = 0; j < s->J; ++j)
      for (size_t i = 0; i < s->I; ++i) {
        size_t k = (size_t)kk, n = i + j * I + k * IJ;
        real hx = Hx[n], hy = Hy[n], hz = Hz[n];
        if (j != 0 && k != 0)
          Ex[n] = C[0][n] * Ex[n] + C[3][n] * (+(hz - Hz[n - I]) - (hy - Hy[n - IJ]));
        if (i != 0 && k != 0)
          Ey[n] = C[1][n] * Ey[n] + C[4][n] * (+(hx - Hx[n - IJ]) - (hz - Hz[n - 1]));
        if (i != 0 && j != 0)
          Ez[n] = C[2][n] * Ez[n] + C[5][n] * (+(hy - Hy[n - 1]) - (hx - Hx[n - I]));
      }
}

/* H-field CPML, src/simulation.h:392-403: Y (gpu.h:644-685), X (:604-642),
 * Z (:687-725), in that order. */
void OR(update_h_pml)(or_sim *s) {
  real *Hx = s->f[F_HX], *Hy = s->f[F_HY], *Hz = s->f[F_HZ];
  const real *Ex = s->f[F_EX], *Ey = s->f[F_EY], *Ez = s->f[F_EZ];
  const size_t I = s->I, J = s->J, K = s->K, IJ = s->IJ, p = s->p;
  const real d = s->delX;
  const real *b = s->bH, *c = s->cH;
  /* Y faces: psi layout [k][2p][i] */
  {
    real *pxy = s->psi[P_HXY], *pzy = s->psi[P_HZY];
#pragma omp parallel for schedule(static)
    for (long long kk = 0; kk < (long long)K - 1; ++kk)
      for (size_t y = 0; y < 2 * p - 1; ++y)
        for (size_t x = 0; x + 1 < I; ++x) {
          size_t t = x + y * I + (size_t)kk * (2 * p * I);
          size_t j = y < p ? y : y + J - 2 * p;
          size_t id = x + j * I + (size_t)kk * IJ;
          pxy[t] = b[y] * pxy[t] + c[y] * (Ez[id + I] - Ez[id]) / d;
          Hx[id] = Hx[id] - CHE(0, id) * pxy[t] * d;
          pzy[t] = b[y] * pzy[t] + c[y] * (Ex[id + I] - Ex[id]) / d;
          Hz[id] = Hz[id] + CHE(2, id) * pzy[t] * d;
        }
  }
  /* X faces: psi layout [k][j][2p] */
  {
    real *pyx = s->psi[P_HYX], *pzx = s->psi[P_HZX];
#pragma omp parallel for schedule(static)
    for (long long kk = 0; kk < (long long)K - 1; ++kk)
      for (size_t j = 0; j + 1 < J; ++j)
        for (size_t x = 0; x < 2 * p - 1; ++x) {
          size_t t = x + j * (2 * p) + (size_t)kk * (2 * p * J);
          size_t i = x < p ? x : I - 2 * p + x;
          size_t id = i + j * I + (size_t)kk * IJ;
          pyx[t] = b[x] * pyx[t] + c[x] * (Ez[id + 1] - Ez[id]) / d;
          Hy[id] = Hy[id] + CHE(1, id) * pyx[t] * d;
          pzx[t] = b[x] * pzx[t] + c[x] * (Ey[id + 1] - Ey[id]) / d;
          Hz[id] = Hz[id] - CHE(2, id) * pzx[t] * d;
        }
  }
  /* Z faces: psi layout [2p][j][i] */
  {
    real *pxz = s->psi[P_HXZ], *pyz = s->psi[P_HYZ];
#pragma omp parallel for schedule(static)
    for (long long zz = 0; zz < (long long)(2 * p - 1); ++zz)
      for (size_t j = 0; j + 1 < J; ++j)
        for (size_t x = 0; x + 1 < I; ++x) {
          size_t z = (size_t)zz;
          size_t t = x + j * I + z * IJ;
          size_t k = z < p ? z : z + K - 2 * p;
          size_t id = x + j * I + k * IJ;
          pxz[t] = b[z] * pxz[t] + c[z] * (Ey[id + IJ] - Ey[id]) / d;
          Hx[id] = Hx[id] + CHE(0, id) * pxz[t] * d;
          pyz[t] = b[z] * pyz[t] + c[z] * (Ex[id + IJ] - Ex[id]) / d;
          Hy[id] = Hy[id] - CHE(1, id) * pyz[t] * d;
        }
  }
}

/* E-field CPML, src/simulation.h:404-418: Y (gpu.h:790-827), Z (:829-868),
 * X (:765-788), in that order. */
void OR(update_e_pml)(or_sim *s) {
  real *Ex = s->f[F_EX], *Ey = s->f[F_EY], *Ez = s->f[F_EZ];
  const real *Hx = s->f[F_HX], *Hy = s->f[F_HY], *Hz = s->f[F_HZ];
  const size_t I = s->I, J = s->J, K = s->K, IJ = s->IJ, p = s->p;
  const real d = s->delX;
  const real *b = s->bE, *c = s->cE;
  const real *Cxh = s->Ce[3], *Cyh = s->Ce[4], *Czh = s->Ce[5];
  {
    real *pxy = s->psi[P_EXY], *pzy = s->psi[P_EZY];
#pragma omp parallel for schedule(static)
    for (long long kk = 1; kk < (long long)K - 1; ++kk)
      for (size_t y = 1; y < 2 * p; ++y)
        for (size_t x = 1; x + 1 < I; ++x) {
          size_t t = x + y * I + (size_t)kk * (2 * p * I);
          size_t j = y < p ? y : y + J - 2 * p;
          size_t id = x + j * I + (size_t)kk * IJ;
          pxy[t] = b[y] * pxy[t] + c[y] * (Hz[id] - Hz[id - I]) / d;
          Ex[id] = Ex[id] + Cxh[id] * pxy[t] * d;
          pzy[t] = b[y] * pzy[t] + c[y] * (Hx[id] - Hx[id - I]) / d;
          Ez[id] = Ez[id] - Czh[id] * pzy[t] * d;
        }
  }
  {
    real *pxz = s->psi[P_EXZ], *pyz = s->psi[P_EYZ];
#pragma omp parallel for schedule(static)
    for (long long zz = 1; zz < (long long)(2 * p); ++zz)
      for (size_t j = 1; j + 1 < J; ++j)
        for (size_t x = 1; x + 1 < I; ++x) {
          size_t z = (size_t)zz;
          size_t t = x + j * I + z * IJ;
          size_t k = z < p ? z : z + K - 2 * p;
          size_t id = x + j * I + k * IJ;
          pxz[t] = b[z] * pxz[t] + c[z] * (Hy[id] - Hy[id - IJ]) / d;
          Ex[id] = Ex[id] - Cxh[id] * pxz[t] * d;
          pyz[t] = b[z] * pyz[t] + c[z] * (Hx[id] - Hx[id - IJ]) / d;
          Ey[id] = Ey[id] + Cyh[id] * pyz[t] * d;
        }
  }
  {
    real *pyx = s->psi[P_EYX], *pzx = s->psi[P_EZX];
#pragma omp parallel for schedule(static)
    for (long long kk = 1; kk < (long long)K - 1; ++kk)
      for (size_t j = 1; j + 1 < J; ++j)
        for (size_t x = 1; x < 2 * p; ++x) {
          size_t t = x + j * (2 * p) + (size_t)kk * (2 * p * J);
          size_t i = x < p ? x : x + I - 2 * p;
          size_t id = i + j * I + (size_t)kk * IJ;
          pyx[t] = b[x] * pyx[t] + c[x] * (Hz[id] - Hz[id - 1]) / d;
          Ey[id] = Ey[id] - Cyh[id] * pyx[t] * d;
          pzx[t] = b[x] * pzx[t] + c[x] * (Hy[id] - Hy[id - 1]) / d;
          Ez[id] = Ez[id] + Czh[id] * pzx[t] * d;
        }
  }
}

/* ----------------------------------------------------------- TF/SF faces */

/* Mode 5 helpers: window value at coordinate x, window coordinate of a
 * point, position of Yee component c of family E / H at cell x[3]. */
static real ob_interp(const real *row, real x, size_t w) {
  long m = (long)floor((double)x);
  m = m < 0 ? 0 : (m > (long)w - 2 ? (long)w - 2 : m);
  const real f = x - (real)m;
  return row[m] + f * (row[m + 1] - row[m]);
}
static real ob_coord(const or_sim *s, real px, real py, real pz) {
  const real v = s->ob_k[0] * (px - (real)s->ob_r0[0]) + s->ob_k[1] * (py - (real)s->ob_r0[1]) +
                 s->ob_k[2] * (pz - (real)s->ob_r0[2]);
  return s->ob_x0 + s->ob_rho * v;
}
static void yee_pos(int hfam, int c, const long x[3], real p[3]) {
  for (int a = 0; a < 3; ++a) {
    const int half = hfam ? (a != c) : (a == c);
    p[a] = (real)x[a] + (half ? (real)0.5 : (real)0);
  }
}

/* Mode 5, faces normal to each axis in turn (x, y, z): E pass, E_u and E_v
 * on the face planes take +-C * h_{v,u} H1 at the half cell outside; H pass,
 * H_v and H_u at that half cell take +-Che * e_{u,v} E1 of the face plane;
 * + for (E_u, H_v) on the low face, - on the high face, opposite for
 * (E_v, H_u). */
static void oblique_faces(or_sim *s, int hfam, int n) {
  const long lo[3] = {(long)s->i0, (long)s->j0, (long)s->k0};
  const long hi[3] = {(long)s->i1, (long)s->j1, (long)s->k1};
  const size_t W = s->ob_w;
  const real *rowE = s->obE + (size_t)n * W, *rowH = s->obH + (size_t)n * W;
  for (int axis = 0; axis < 3; ++axis) {
    const int u = (axis + 1) % 3, v = (axis + 2) % 3;
    for (int side = 0; side < 2; ++side)
      for (int t = 0; t < 2; ++t) {
        const int ce = t == 0 ? u : v, ch = t == 0 ? v : u;
        const int plus = (t == 0) == (side == 0);
        const long nu = hi[u] - lo[u] + (ce == u ? 0 : 1), nv = hi[v] - lo[v] + (ce == v ? 0 : 1);
        for (long b = 0; b < nv; ++b)
          for (long a = 0; a < nu; ++a) {
            long xe[3], xh[3];
            xe[u] = lo[u] + a;
            xe[v] = lo[v] + b;
            xe[axis] = side ? hi[axis] : lo[axis];
            xh[u] = xe[u];
            xh[v] = xe[v];
            xh[axis] = side ? hi[axis] : lo[axis] - 1;
            real p[3];
            if (hfam) {
              yee_pos(0, ce, xe, p);
              const real inc = s->ob_e[ce] * ob_interp(rowE, ob_coord(s, p[0], p[1], p[2]), W);
              const size_t id = IDX(xh[0], xh[1], xh[2]);
              real *f = &s->f[F_HX + ch][id];
              const real val = CHE(ch, id) * inc;
              *f = plus ? *f + val : *f - val;
            } else {
              yee_pos(1, ch, xh, p);
              const real inc =
                  s->ob_h[ch] * ob_interp(rowH, ob_coord(s, p[0], p[1], p[2]) - (real)0.5, W);
              const size_t id = IDX(xe[0], xe[1], xe[2]);
              real *f = &s->f[F_EX + ce][id];
              const real val = s->Ce[3 + ce][id] * inc;
              *f = plus ? *f + val : *f - val;
            }
          }
      }
  }
}

/* H-side TF/SF corrections, src/simulation.h:330-349 with the launchers at
 * :421-492 and kernels at src/gpu.h:152-182 (mode 3), :217-247 (mode 4),
 * :424-477 (mode 1), :512-541 (mode 2).  c = +1 for every H launcher. */
int OR(update_h_planewave)(or_sim *s, int n, int mode) {
  if (!s->init_1d || n < 0 || (size_t)n >= s->T) return -1;
  if (mode == 5) {
    if (!s->obE) return -1;
    oblique_faces(s, 1, n);
    return 0;
  }
  const size_t I = s->I, IJ = s->IJ, S = s->size1d;
  const size_t i0 = s->i0, i1 = s->i1, j0 = s->j0, j1 = s->j1, k0 = s->k0, k1 = s->k1;
  /* Chxe = Chye = Chze = Che, :920-922 (per cell after set_magnetic) */
  real *Hx = s->f[F_HX], *Hy = s->f[F_HY], *Hz = s->f[F_HZ];
  const real c = 1;
  if (mode == 1) { /* ZY */
    const real *E = s->Ez1d + (size_t)n * S + S - s->K;
    for (size_t y = j0; y <= j1 - 1; ++y)
      for (size_t x = i0; x <= i1; ++x) {
        Hx[IDX(x, y, k0 - 1)] = Hx[IDX(x, y, k0 - 1)] - CHE(0, IDX(x, y, k0 - 1)) * E[k0] * c;
        Hx[IDX(x, y, k1)] = Hx[IDX(x, y, k1)] + CHE(0, IDX(x, y, k1)) * E[k1] * c;
      }
    for (size_t z = k0; z <= k1; ++z)
      for (size_t y = j0; y <= j1 - 1; ++y) {
        Hz[IDX(i0 - 1, y, z)] = Hz[IDX(i0 - 1, y, z)] + CHE(2, IDX(i0 - 1, y, z)) * E[z] * c;
        Hz[IDX(i1, y, z)] = Hz[IDX(i1, y, z)] - CHE(2, IDX(i1, y, z)) * E[z] * c;
      }
  } else if (mode == 2) { /* ZX */
    const real *E = s->Ez1d + (size_t)n * S + S - s->K;
    for (size_t y = j0; y <= j1; ++y)
      for (size_t x = i0; x <= i1 - 1; ++x) {
        Hy[IDX(x, y, k0 - 1)] = Hy[IDX(x, y, k0 - 1)] + CHE(1, IDX(x, y, k0 - 1)) * E[k0] * c;
        Hy[IDX(x, y, k1)] = Hy[IDX(x, y, k1)] - CHE(1, IDX(x, y, k1)) * E[k1] * c;
      }
    for (size_t z = k0; z <= k1; ++z)
      for (size_t x = i0; x <= i1 - 1; ++x) {
        Hz[IDX(x, j0 - 1, z)] = Hz[IDX(x, j0 - 1, z)] - CHE(2, IDX(x, j0 - 1, z)) * E[z] * c;
        Hz[IDX(x, j1, z)] = Hz[IDX(x, j1, z)] + CHE(2, IDX(x, j1, z)) * E[z] * c;
      }
  } else if (mode == 3) { /* XZ */
    const real *E = s->Ez1d + (size_t)n * S + S - s->I;
    for (size_t z = k0; z <= k1 - 1; ++z)
      for (size_t x = i0; x <= i1; ++x) {
        Hx[IDX(x, j0 - 1, z)] = Hx[IDX(x, j0 - 1, z)] + CHE(0, IDX(x, j0 - 1, z)) * E[x] * c;
        Hx[IDX(x, j1, z)] = Hx[IDX(x, j1, z)] - CHE(0, IDX(x, j1, z)) * E[x] * c;
      }
    for (size_t z = k0; z <= k1 - 1; ++z)
      for (size_t y = j0; y <= j1; ++y) {
        Hy[IDX(i0 - 1, y, z)] = Hy[IDX(i0 - 1, y, z)] - CHE(1, IDX(i0 - 1, y, z)) * E[i0] * c;
        Hy[IDX(i1, y, z)] = Hy[IDX(i1, y, z)] + CHE(1, IDX(i1, y, z)) * E[i1] * c;
      }
  } else if (mode == 4) { /* XY, inverse run */
    const real *E = s->Einv1d + (size_t)n * S + S - s->I;
    for (size_t y = j0; y <= j1 - 1; ++y)
      for (size_t x = i0; x <= i1; ++x) {
        Hx[IDX(x, y, k0 - 1)] = Hx[IDX(x, y, k0 - 1)] - CHE(0, IDX(x, y, k0 - 1)) * E[x] * c;
        Hx[IDX(x, y, k1)] = Hx[IDX(x, y, k1)] + CHE(0, IDX(x, y, k1)) * E[x] * c;
      }
    for (size_t z = k0; z <= k1; ++z)
      for (size_t y = j0; y <= j1 - 1; ++y) {
        Hz[IDX(i0 - 1, y, z)] = Hz[IDX(i0 - 1, y, z)] + CHE(2, IDX(i0 - 1, y, z)) * E[i0] * c;
        Hz[IDX(i1, y, z)] = Hz[IDX(i1, y, z)] - CHE(2, IDX(i1, y, z)) * E[i1] * c;
      }
  }
  (void)I; (void)IJ;
  return 0;
}

/* E-side TF/SF corrections, src/simulation.h:350-369 with launchers
 * :493-570 and kernels src/gpu.h:184-214 (mode 3, c=+1), :249-291 (mode 4,
 * c=-1), :479-509 (mode 1, c=+1), :543-573 (mode 2, c=-1). */
int OR(update_e_planewave)(or_sim *s, int n, int mode) {
  if (!s->init_1d || n < 0 || (size_t)n >= s->T) return -1;
  if (mode == 5) {
    if (!s->obE) return -1;
    oblique_faces(s, 0, n);
    return 0;
  }
  const size_t I = s->I, IJ = s->IJ, S = s->size1d;
  const size_t i0 = s->i0, i1 = s->i1, j0 = s->j0, j1 = s->j1, k0 = s->k0, k1 = s->k1;
  real *Ex = s->f[F_EX], *Ey = s->f[F_EY], *Ez = s->f[F_EZ];
  const real *Cxh = s->Ce[3], *Cyh = s->Ce[4], *Czh = s->Ce[5];
  if (mode == 1) { /* ZY */
    const real c = 1;
    const real *H = s->Hy1d + (size_t)n * S + S - s->K;
    for (size_t y = j0; y <= j1 - 1; ++y)
      for (size_t x = i0; x <= i1; ++x) {
        size_t a = IDX(x, y, k0), b = IDX(x, y, k1);
        Ey[a] = Ey[a] - Cyh[a] * H[k0 - 1] * c;
        Ey[b] = Ey[b] + Cyh[b] * H[k1] * c;
      }
    for (size_t z = k0; z <= k1 - 1; ++z)
      for (size_t x = i0; x <= i1; ++x) {
        size_t a = IDX(x, j0, z), b = IDX(x, j1, z);
        Ez[a] = Ez[a] + Czh[a] * H[z] * c;
        Ez[b] = Ez[b] - Czh[b] * H[z] * c;
      }
  } else if (mode == 2) { /* ZX */
    const real c = -1;
    const real *H = s->Hy1d + (size_t)n * S + S - s->K;
    for (size_t y = j0; y <= j1; ++y)
      for (size_t x = i0; x <= i1 - 1; ++x) {
        size_t a = IDX(x, y, k0), b = IDX(x, y, k1);
        Ex[a] = Ex[a] + Cxh[a] * H[k0 - 1] * c;
        Ex[b] = Ex[b] - Cxh[b] * H[k1] * c;
      }
    for (size_t z = k0; z <= k1 - 1; ++z)
      for (size_t y = j0; y <= j1; ++y) {
        size_t a = IDX(i0, y, z), b = IDX(i1, y, z);
        Ez[a] = Ez[a] - Czh[a] * H[z] * c;
        Ez[b] = Ez[b] + Czh[b] * H[z] * c;
      }
  } else if (mode == 3) { /* XZ */
    const real c = 1;
    const real *H = s->Hy1d + (size_t)n * S + S - s->I;
    for (size_t y = j0; y <= j1; ++y)
      for (size_t x = i0; x <= i1 - 1; ++x) {
        size_t a = IDX(x, y, k0), b = IDX(x, y, k1);
        Ex[a] = Ex[a] + Cxh[a] * H[x] * c;
        Ex[b] = Ex[b] - Cxh[b] * H[x] * c;
      }
    for (size_t z = k0; z <= k1 - 1; ++z)
      for (size_t y = j0; y <= j1; ++y) {
        size_t a = IDX(i0, y, z), b = IDX(i1, y, z);
        Ez[a] = Ez[a] - Czh[a] * H[i0 - 1] * c;
        Ez[b] = Ez[b] + Czh[b] * H[i1] * c;
      }
  } else if (mode == 4) { /* XY, inverse run */
    const real c = -1;
    const real *H = s->Hinv1d + (size_t)n * S + S - s->I;
    for (size_t z = k0; z <= k1; ++z)
      for (size_t x = i0; x <= i1 - 1; ++x) {
        size_t a = IDX(x, j0, z), b = IDX(x, j1, z);
        Ex[a] = Ex[a] - Cxh[a] * H[x] * c;
        Ex[b] = Ex[b] + Cxh[b] * H[x] * c;
      }
    for (size_t z = k0; z <= k1; ++z)
      for (size_t y = j0; y <= j1 - 1; ++y) {
        size_t a = IDX(i0, y, z), b = IDX(i1, y, z);
        Ey[a] = Ey[a] + Cyh[a] * H[i0 - 1] * c;
        Ey[b] = Ey[b] - Cyh[b] * H[i1] * c;
      }
  }
  (void)I; (void)IJ;
  return 0;
}

/* src/simulation.h:256-286 (addCurrents) -> src/gpu.h:55-82 */
int OR(add_currents)(or_sim *s, int n, int mode, const int32_t *ind) {
  if (!s->init_src || n < 0 || (size_t)n >= s->T) return -1;
  if (mode < 1 || mode > 3) return 0;
  for (int a = 0; a < 6; ++a) if (ind[a] < 0) return -2;
  size_t i0 = (size_t)ind[0], i1 = (size_t)ind[1], j0 = (size_t)ind[2],
         j1 = (size_t)ind[3], k0 = (size_t)ind[4], k1 = (size_t)ind[5];
  if (i1 < i0 || j1 < j0 || k1 < k0) return 0;
  real *E = s->f[mode - 1];
  const real *Ch = s->Ce[3 + mode - 1];
  const real src = s->src[n], dx = s->delX;
  for (size_t k = k0; k <= k1; ++k)
    for (size_t j = j0; j <= j1; ++j)
      for (size_t i = i0; i <= i1; ++i) {
        if (i < s->I && j < s->J && k < s->K) {
          size_t id = IDX(i, j, k);
          E[id] = E[id] - Ch[id] * src * dx / dx / dx;
        }
      }
  return 0;
}

/* Extension: probe gather.  Row n of the [T][numAnt][6] record holds the six
 * components at each probe at the start of step n (before its H update). */
int OR(sample_probes)(or_sim *s, int n) {
  if (!s->probes || n < 0 || (size_t)n >= s->T) return -1;
  for (size_t a = 0; a < s->numAnt; ++a) {
    size_t id = s->ant_idx[a];
    if (id >= s->IJK) continue;
    for (int cpt = 0; cpt < 6; ++cpt)
      s->probes[((size_t)n * s->numAnt + a) * 6 + cpt] = s->f[cpt][id];
  }
  return 0;
}

/* One full step in the order of highfrequency.m:85-91 (probe row first). */
int OR(step)(or_sim *s, int n, int mode) {
  if (s->probes) OR(sample_probes)(s, n);
  OR(update_h_all)(s);
  if (mode) OR(update_h_planewave)(s, n, mode);
  OR(update_h_pml)(s);
  OR(update_e_all)(s);
  if (mode) OR(update_e_planewave)(s, n, mode);
  OR(update_e_pml)(s);
  return 0;
}

/* ---------------------------------------------------------------- access */

real *OR(field)(or_sim *s, int which) {
  if (which >= 0 && which < 6) return s->f[which];
  if (which >= 6 && which < 12) return s->Ce[which - 6];
  if (which >= 12 && which < 15) return s->sig[which - 12];
  if (which >= 15 && which < 18) return s->eps[which - 15];
  return NULL;
}
real *OR(psi)(or_sim *s, int which) {
  return (which >= 0 && which < P_COUNT) ? s->psi[which] : NULL;
}
/* which: 0 bE, 1 cE, 2 bH, 3 cH, 4 den_ex, 5 den_hx, 6 Ez1d, 7 Hy1d, 8 Einv, 9 Hinv, 10 probes */
real *OR(array)(or_sim *s, int which) {
  switch (which) {
    case 0: return s->bE;
    case 1: return s->cE;
    case 2: return s->bH;
    case 3: return s->cH;
    case 4: return s->den_ex;
    case 5: return s->den_hx;
    case 6: return s->Ez1d;
    case 7: return s->Hy1d;
    case 8: return s->Einv1d;
    case 9: return s->Hinv1d;
    case 10: return s->probes;
    case 11: return s->obE;
    case 12: return s->obH;
  }
  return NULL;
}
/* 0 I,1 J,2 K,3 T,4 numAnt,5 p,6 size1d,7 i0,8 i1,9 j0,10 j1,11 k0,12 k1,
 * 13 ob_w */
long long OR(dim)(or_sim *s, int which) {
  switch (which) {
    case 0: return (long long)s->I;
    case 1: return (long long)s->J;
    case 2: return (long long)s->K;
    case 3: return (long long)s->T;
    case 4: return (long long)s->numAnt;
    case 5: return (long long)s->p;
    case 6: return (long long)s->size1d;
    case 7: return (long long)s->i0;
    case 8: return (long long)s->i1;
    case 9: return (long long)s->j0;
    case 10: return (long long)s->j1;
    case 11: return (long long)s->k0;
    case 12: return (long long)s->k1;
    case 13: return (long long)s->ob_w;
  }
  return -1;
}
/* 0 Chh, 1 Che, 2 sig_max, 3 Ceh_1D */
double OR(scalar)(or_sim *s, int which) {
  switch (which) {
    case 0: return (double)s->Chh;
    case 1: return (double)s->Che;
    case 2: return (double)s->sig_max;
    case 3: return (double)(real)((double)s->delT / K_EPS0 / (double)s->delX);
  }
  return 0;
}
