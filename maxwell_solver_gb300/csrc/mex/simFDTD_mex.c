/*
 * simFDTD_mex.c -- drop-in MATLAB entry point over the GB300 C ABI.
 *
 * Same signature, op strings (case-insensitive), argument classes, outputs
 * and error identifiers as the reference dispatcher
 * (enricoballini/maxwell_solver src/simFDTD.cu:19-187), so the reference's
 * scripts (highfrequency.m, GICsimulation.m) run unchanged:
 *
 *   P = simFDTD('CreateSimulation');
 *   simFDTD('SetConst', P, single([fctr delX delT]), int32([T I J K nAnt]));
 *   ...
 *   simFDTD('UpdateH_All', P); simFDTD('UpdateH_PlaneWave', P, int32([n 3])); ...
 *
 * Build (MATLAB):  mex -R2018a simFDTD_mex.c -output simFDTD \
 *                      -I<repo>/include -L<lib dir> -lfdtd_gb300
 *
 * Failures the reference leaves undefined (bad handle, calls out of order,
 * CUDA errors) raise simFDTD:InvalidHandle / :InvalidState / :CudaError /
 * :OutOfMemory / :Unsupported instead of crashing MATLAB.
 *
 * Extension ops: 'SetParams' (CPML / TF/SF settings), 'StepN'
 * [first count mode] (+ optional [curmode i0 i1 j0 j1 k0 k1]),
 * 'OutputProbes' N, 'Synchronize'.
 */
#include <ctype.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "mex.h"
#include "fdtd_gb300.h"

static void raise_status(int rc) {
  const char *id = "simFDTD:Failed";
  switch (rc) {
    case FDTD_ERR_INVALID_HANDLE: id = "simFDTD:InvalidHandle"; break;
    case FDTD_ERR_INVALID_ARG: id = "simFDTD:InvalidInput"; break;
    case FDTD_ERR_STATE: id = "simFDTD:InvalidState"; break;
    case FDTD_ERR_ALREADY_INITIALIZED: id = "simFDTD:AlreadyInitialized"; break;
    case FDTD_ERR_CUDA: id = "simFDTD:CudaError"; break;
    case FDTD_ERR_OOM: id = "simFDTD:OutOfMemory"; break;
    case FDTD_ERR_UNSUPPORTED: id = "simFDTD:Unsupported"; break;
    case FDTD_ERR_CANCELLED: id = "simFDTD:Cancelled"; break;
  }
  mexErrMsgIdAndTxt(id, "%s", fdtd_last_error());
}

#define CHECK(call)               \
  do {                            \
    int rc_ = (call);             \
    if (rc_ != FDTD_OK) raise_status(rc_); \
  } while (0)

/* Numeric argument as int32 / float, whatever numeric class MATLAB passed
 * (the reference reinterprets the raw data; int32 and single are what its
 * scripts pass). */
static int32_t *as_i32(const mxArray *a, size_t *n) {
  size_t cnt = mxGetNumberOfElements(a);
  int32_t *out = (int32_t *)malloc((cnt ? cnt : 1) * sizeof(int32_t));
  const void *d = mxGetData(a);
  for (size_t i = 0; i < cnt; ++i) {
    switch (mxGetClassID(a)) {
      case mxINT32_CLASS: out[i] = ((const int32_t *)d)[i]; break;
      case mxUINT32_CLASS: out[i] = (int32_t)((const uint32_t *)d)[i]; break;
      case mxDOUBLE_CLASS: out[i] = (int32_t)((const double *)d)[i]; break;
      case mxSINGLE_CLASS: out[i] = (int32_t)((const float *)d)[i]; break;
      case mxUINT64_CLASS: out[i] = (int32_t)((const uint64_t *)d)[i]; break;
      default: out[i] = 0;
    }
  }
  if (n) *n = cnt;
  return out;
}

static float *as_f32(const mxArray *a, size_t *n) {
  size_t cnt = mxGetNumberOfElements(a);
  if (n) *n = cnt;
  float *out = (float *)malloc((cnt ? cnt : 1) * sizeof(float));
  const void *d = mxGetData(a);
  if (mxGetClassID(a) == mxSINGLE_CLASS) {
    memcpy(out, d, cnt * sizeof(float));
    return out;
  }
  for (size_t i = 0; i < cnt; ++i) {
    switch (mxGetClassID(a)) {
      case mxDOUBLE_CLASS: out[i] = (float)((const double *)d)[i]; break;
      case mxINT32_CLASS: out[i] = (float)((const int32_t *)d)[i]; break;
      default: out[i] = 0.0f;
    }
  }
  return out;
}

static double *as_f64(const mxArray *a, size_t *n) {
  size_t cnt = mxGetNumberOfElements(a);
  if (n) *n = cnt;
  double *out = (double *)malloc((cnt ? cnt : 1) * sizeof(double));
  const void *d = mxGetData(a);
  for (size_t i = 0; i < cnt; ++i) {
    switch (mxGetClassID(a)) {
      case mxDOUBLE_CLASS: out[i] = ((const double *)d)[i]; break;
      case mxSINGLE_CLASS: out[i] = (double)((const float *)d)[i]; break;
      case mxINT32_CLASS: out[i] = (double)((const int32_t *)d)[i]; break;
      default: out[i] = 0.0;
    }
  }
  return out;
}

static size_t scalar_count(const mxArray *a) {
  switch (mxGetClassID(a)) {
    case mxUINT32_CLASS: return *(const uint32_t *)mxGetData(a);
    case mxINT32_CLASS: return (size_t)*(const int32_t *)mxGetData(a);
    case mxDOUBLE_CLASS: return (size_t)*(const double *)mxGetData(a);
    case mxUINT64_CLASS: return (size_t)*(const uint64_t *)mxGetData(a);
    default: return 0;
  }
}

static mxArray *single_row(size_t n) {
  const mwSize dims[2] = {1, (mwSize)n};
  return mxCreateNumericArray(2, dims, mxSINGLE_CLASS, mxREAL);
}

void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[]) {
  (void)nlhs;
  if (nrhs < 1) {
    mexErrMsgIdAndTxt("simFDTD:InvalidInput", "At least one input required: operation string.");
    return;
  }
  char *op = mxArrayToString(prhs[0]);
  if (!op) {
    mexErrMsgIdAndTxt("simFDTD:InvalidInput", "At least one input required: operation string.");
    return;
  }
  for (char *c = op; *c; ++c) *c = (char)tolower((unsigned char)*c);

  if (strcmp(op, "createsimulation") == 0) {
    fdtd_handle h = 0;
    int rc = fdtd_create(&h);
    mxFree(op);
    if (rc) raise_status(rc);
    const mwSize dims[2] = {1, 1};
    mxArray *out = mxCreateNumericArray(2, dims, mxUINT64_CLASS, mxREAL);
    *(uint64_t *)mxGetData(out) = h;
    plhs[0] = out;
    return;
  }
  if (nrhs < 2) {
    mxFree(op);
    mexErrMsgIdAndTxt("simFDTD:InvalidInput", "Simulation pointer required for this operation.");
    return;
  }
  const fdtd_handle P = (fdtd_handle)(mxGetClassID(prhs[1]) == mxUINT64_CLASS
                                          ? *(const uint64_t *)mxGetData(prhs[1])
                                          : 0);
  /* Arguments are copied to plain buffers so that an error raised below
   * (which does not return) only leaks into MATLAB's allocator scope. */
  char opbuf[64];
  strncpy(opbuf, op, sizeof(opbuf) - 1);
  opbuf[sizeof(opbuf) - 1] = '\0';
  mxFree(op);
  const char *o = opbuf;

  if (strcmp(o, "deletesimulation") == 0) {
    CHECK(fdtd_destroy(P));
  } else if (strcmp(o, "updatee_all") == 0) {
    CHECK(fdtd_update_e_all(P));
  } else if (strcmp(o, "updateh_all") == 0) {
    CHECK(fdtd_update_h_all(P));
  } else if (strcmp(o, "updatee_pml") == 0) {
    CHECK(fdtd_update_e_pml(P));
  } else if (strcmp(o, "updateh_pml") == 0) {
    CHECK(fdtd_update_h_pml(P));
  } else if (strcmp(o, "updatecuda") == 0) {
    CHECK(fdtd_update_cuda(P));
  } else if (strcmp(o, "addcurrents") == 0) {
    if (nrhs < 4) mexErrMsgIdAndTxt("simFDTD:InvalidInput", "time and indices required.");
    size_t nt = 0, nb = 0;
    int32_t *t = as_i32(prhs[2], &nt), *b = as_i32(prhs[3], &nb);
    int32_t tt[2] = {nt > 0 ? t[0] : 0, nt > 1 ? t[1] : 0}, bb[6] = {0, -1, 0, -1, 0, -1};
    for (size_t i = 0; i < 6 && i < nb; ++i) bb[i] = b[i];
    free(t);
    free(b);
    if (nt < 2 || nb < 6) mexErrMsgIdAndTxt("simFDTD:InvalidInput", "time and indices required.");
    CHECK(fdtd_add_currents(P, tt[0], tt[1], bb));
  } else if (strcmp(o, "readysimulation") == 0) {
    CHECK(fdtd_ready_simulation(P));
  } else if (strcmp(o, "resetfieldall") == 0) {
    CHECK(fdtd_reset_field_all(P));
  } else if (strcmp(o, "updatee_planewave") == 0 || strcmp(o, "updateh_planewave") == 0) {
    if (nrhs < 3) mexErrMsgIdAndTxt("simFDTD:InvalidInput", "time required.");
    size_t nt = 0;
    int32_t *t = as_i32(prhs[2], &nt);
    int32_t tt[2] = {nt > 0 ? t[0] : 0, nt > 1 ? t[1] : 0};
    free(t);
    if (nt < 2) mexErrMsgIdAndTxt("simFDTD:InvalidInput", "time required.");
    if (o[6] == 'e') CHECK(fdtd_update_e_planewave(P, tt[0], tt[1]));
    else CHECK(fdtd_update_h_planewave(P, tt[0], tt[1]));
  } else if (strcmp(o, "setconst") == 0) {
    if (nrhs < 4) mexErrMsgIdAndTxt("simFDTD:InvalidInput", "freqRes and TimeDim required.");
    size_t nf = 0, nd = 0;
    float *f = as_f32(prhs[2], &nf);
    int32_t *d = as_i32(prhs[3], &nd);
    float ff[3] = {0, 0, 0};
    int32_t dd[5] = {0, 0, 0, 0, 0};
    for (size_t i = 0; i < 3 && i < nf; ++i) ff[i] = f[i];
    for (size_t i = 0; i < 5 && i < nd; ++i) dd[i] = d[i];
    free(f);
    free(d);
    if (nf < 3 || nd < 5) mexErrMsgIdAndTxt("simFDTD:InvalidInput", "freqRes and TimeDim required.");
    CHECK(fdtd_set_const(P, ff, dd));
  } else if (strcmp(o, "setsource") == 0) {
    if (nrhs < 3) mexErrMsgIdAndTxt("simFDTD:InvalidInput", "SourceIn required.");
    size_t n = 0;
    float *src = as_f32(prhs[2], &n);
    int rc;
    if (nrhs > 3) {
      mexPrintf("Update Source Mode!\n");
      rc = fdtd_update_source(P, src, n);
    } else {
      rc = fdtd_set_source(P, src, n);
    }
    free(src);
    CHECK(rc);
  } else if (strcmp(o, "setantennalocations") == 0) {
    if (nrhs < 3) mexErrMsgIdAndTxt("simFDTD:InvalidInput", "Locations required.");
    size_t n = 0;
    int32_t *loc = as_i32(prhs[2], &n);
    int rc = fdtd_set_antenna_locations(P, loc, n);
    free(loc);
    CHECK(rc);
  } else if (strcmp(o, "createmu") == 0) {
    if (nrhs < 5) mexErrMsgIdAndTxt("simFDTD:InvalidInput", "mu_x, mu_y, mu_z required.");
    size_t nx = 0, ny = 0, nz = 0;
    float *mx = as_f32(prhs[2], &nx), *my = as_f32(prhs[3], &ny), *mz = as_f32(prhs[4], &nz);
    size_t n = nx < ny ? nx : ny;
    n = n < nz ? n : nz;
    int rc = fdtd_create_mu(P, mx, my, mz, n);
    free(mx);
    free(my);
    free(mz);
    CHECK(rc);
  } else if (strcmp(o, "setmagnetic") == 0) {
    /* simFDTD('SetMagnetic', P, mu_x, mu_y, mu_z [, sm_x, sm_y, sm_z]) */
    if (nrhs != 5 && nrhs != 8)
      mexErrMsgIdAndTxt("simFDTD:InvalidInput", "mu_x, mu_y, mu_z [, sm_x, sm_y, sm_z] required.");
    size_t nv[6] = {0, 0, 0, 0, 0, 0};
    float *v[6] = {NULL, NULL, NULL, NULL, NULL, NULL};
    for (int a = 0; a < nrhs - 2; ++a) v[a] = as_f32(prhs[2 + a], &nv[a]);
    size_t n = nv[0];
    for (int a = 1; a < nrhs - 2; ++a) n = nv[a] < n ? nv[a] : n;
    int rc = fdtd_set_magnetic(P, v[0], v[1], v[2], v[3], v[4], v[5], n);
    for (int a = 0; a < 6; ++a) free(v[a]);
    CHECK(rc);
  } else if (strcmp(o, "init1d") == 0) {
    if (nrhs < 4) mexErrMsgIdAndTxt("simFDTD:InvalidInput", "rate and PW_source required.");
    size_t nr = 0, n = 0;
    float *rate = as_f32(prhs[2], &nr), *pw = as_f32(prhs[3], &n);
    const float r = nr ? rate[0] : 0.0f;
    int rc = fdtd_init_1d(P, r, pw, n);
    free(rate);
    free(pw);
    CHECK(rc);
  } else if (strcmp(o, "updatematerial") == 0) {
    if (nrhs < 4) mexErrMsgIdAndTxt("simFDTD:InvalidInput", "flag, values required.");
    size_t nf = 0, n = 0;
    int32_t *flag = as_i32(prhs[2], &nf);
    float *v = as_f32(prhs[3], &n);
    const int32_t fl = nf ? flag[0] : 0;
    int rc = fdtd_update_material(P, fl, v, n);
    free(flag);
    free(v);
    CHECK(rc);
  } else if (strcmp(o, "setincidence") == 0) {
    /* SetIncidence(P, [theta phi psi]) in radians: TF/SF mode 5 */
    if (nrhs < 3) mexErrMsgIdAndTxt("simFDTD:InvalidInput", "[theta phi psi] required.");
    size_t na = 0;
    double *ang = as_f64(prhs[2], &na);
    if (na < 3) {
      free(ang);
      mexErrMsgIdAndTxt("simFDTD:InvalidInput", "[theta phi psi] required.");
    }
    int rc = fdtd_set_incidence(P, ang[0], ang[1], ang[2]);
    free(ang);
    CHECK(rc);
  } else if (strcmp(o, "setshapes") == 0) {
    /* SetShapes(P, [bg_eps_r bg_sigma], S): S is n x 9, one shape per row
     * [kind eps_r sigma g1 .. g6] (column-major, as MATLAB stores it) */
    if (nrhs < 4) mexErrMsgIdAndTxt("simFDTD:InvalidInput", "background and shapes required.");
    size_t nb = 0, ns = 0;
    float *bg = as_f32(prhs[2], &nb);
    double *sv = as_f64(prhs[3], &ns);
    const size_t rows = mxGetNumberOfElements(prhs[3]) ? mxGetM(prhs[3]) : 0;
    if (nb < 2 || (rows && mxGetN(prhs[3]) < 9)) {
      free(bg);
      free(sv);
      mexErrMsgIdAndTxt("simFDTD:InvalidInput", "background and shapes required.");
    }
    fdtd_shape *sh = (fdtd_shape *)calloc(rows ? rows : 1, sizeof(fdtd_shape));
    for (size_t r = 0; r < rows; ++r) {
      sh[r].kind = (int32_t)sv[r];
      sh[r].eps_r = (float)sv[r + rows];
      sh[r].sigma = (float)sv[r + 2 * rows];
      for (int g = 0; g < 6; ++g) sh[r].g[g] = sv[r + (size_t)(3 + g) * rows];
    }
    int rc = fdtd_set_shapes(P, bg[0], bg[1], sh, (int32_t)rows);
    free(sh);
    free(bg);
    free(sv);
    CHECK(rc);
  } else if (strcmp(o, "savecheckpoint") == 0) {
    size_t n = 0;
    CHECK(fdtd_checkpoint_size(P, &n));
    const mwSize dims[2] = {1, (mwSize)n};
    plhs[0] = mxCreateNumericArray(2, dims, mxUINT8_CLASS, mxREAL);
    CHECK(fdtd_checkpoint_save(P, mxGetData(plhs[0]), n));
  } else if (strcmp(o, "loadcheckpoint") == 0) {
    if (nrhs < 3) mexErrMsgIdAndTxt("simFDTD:InvalidInput", "checkpoint required.");
    if (mxGetClassID(prhs[2]) != mxUINT8_CLASS)
      mexErrMsgIdAndTxt("simFDTD:InvalidInput", "checkpoint must be uint8.");
    CHECK(fdtd_checkpoint_load(P, mxGetData(prhs[2]), mxGetNumberOfElements(prhs[2])));
  } else if (strcmp(o, "outputant") == 0) {
    if (nrhs < 3) mexErrMsgIdAndTxt("simFDTD:InvalidInput", "OutAntSize required.");
    const size_t n = scalar_count(prhs[2]);
    plhs[0] = single_row(n);
    int rc = fdtd_output_ant(P, (float *)mxGetData(plhs[0]), n);
    /* reference: prints "Antenna data is not initialized." and returns zeros */
    if (rc == FDTD_ERR_STATE) mexPrintf("Antenna data is not initialized.\n");
    else CHECK(rc);
  } else if (strcmp(o, "outputvis") == 0) {
    if (nrhs < 4) mexErrMsgIdAndTxt("simFDTD:InvalidInput", "OutAntSize and flag required.");
    const size_t n = scalar_count(prhs[2]);
    size_t nf = 0;
    int32_t *flag = as_i32(prhs[3], &nf);
    const int32_t fl = nf ? flag[0] : 0;
    free(flag);
    plhs[0] = single_row(n);
    CHECK(fdtd_output_vis(P, (float *)mxGetData(plhs[0]), n, fl));
  } else if (strcmp(o, "outputprobes") == 0) {
    if (nrhs < 3) mexErrMsgIdAndTxt("simFDTD:InvalidInput", "OutSize required.");
    const size_t n = scalar_count(prhs[2]);
    plhs[0] = single_row(n);
    CHECK(fdtd_output_probes(P, (float *)mxGetData(plhs[0]), n));
  } else if (strcmp(o, "stepn") == 0) {
    if (nrhs < 3) mexErrMsgIdAndTxt("simFDTD:InvalidInput", "[first count mode] required.");
    size_t nt = 0;
    int32_t *t = as_i32(prhs[2], &nt);
    int32_t tt[3] = {nt > 0 ? t[0] : 0, nt > 1 ? t[1] : 0, nt > 2 ? t[2] : 0};
    free(t);
    fdtd_current cur;
    memset(&cur, 0, sizeof(cur));
    if (nrhs > 3) {
      size_t nc = 0;
      int32_t *c = as_i32(prhs[3], &nc);
      if (nc >= 7) {
        cur.mode = c[0];
        for (int i = 0; i < 6; ++i) cur.box[i] = c[1 + i];
      }
      free(c);
    }
    CHECK(fdtd_step_n(P, tt[0], tt[1], tt[2], cur.mode ? &cur : NULL));
  } else if (strcmp(o, "setparams") == 0) {
    if (nrhs < 3) mexErrMsgIdAndTxt("simFDTD:InvalidInput", "params required.");
    size_t n = 0;
    float *v = as_f32(prhs[2], &n);
    fdtd_params pr = fdtd_default_params();
    if (n > 0) pr.pml = (int32_t)v[0];
    if (n > 1) pr.tfsf_width = (int32_t)v[1];
    if (n > 2) pr.poly_m = v[2];
    if (n > 3) pr.alpha_m = v[3];
    if (n > 4) pr.alpha_max = v[4];
    if (n > 5) pr.kappa_max = v[5];
    if (n > 6) pr.sig_factor = v[6];
    if (n > 7) pr.r0 = v[7];
    free(v);
    CHECK(fdtd_set_params(P, &pr));
  } else if (strcmp(o, "synchronize") == 0) {
    CHECK(fdtd_synchronize(P));
  } else {
    mexErrMsgIdAndTxt("simFDTD:UnknownOperation", "Unknown operation: %s", o);
  }
}
