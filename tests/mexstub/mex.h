/*
 * Minimal stand-in for MATLAB's MEX API (mex.h / matrix.h), for tests only.
 *
 * MATLAB is not installed here, so tests drive mexFunction implementations
 * through this stub: mxArrays are plain heap objects, mexErrMsgIdAndTxt
 * long-jumps back to mexstub_call(), which reports the error identifier
 * and message to the caller (as MATLAB would raise an MException).
 */
#ifndef MEXSTUB_MEX_H
#define MEXSTUB_MEX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef size_t mwSize;
typedef uint64_t uint64_T;
typedef int32_t int32_T;
typedef uint32_t uint32_T;

typedef enum {
  mxUNKNOWN_CLASS = 0,
  mxCHAR_CLASS = 4,
  mxDOUBLE_CLASS = 6,
  mxSINGLE_CLASS = 7,
  mxUINT8_CLASS = 9,
  mxINT32_CLASS = 12,
  mxUINT32_CLASS = 13,
  mxUINT64_CLASS = 15
} mxClassID;

typedef enum { mxREAL = 0, mxCOMPLEX = 1 } mxComplexity;

typedef struct mxArray_tag mxArray;

mxArray *mxCreateNumericArray(mwSize ndim, const mwSize *dims, mxClassID cls,
                              mxComplexity cplx);
mxArray *mxCreateNumericMatrix(mwSize m, mwSize n, mxClassID cls,
                               mxComplexity cplx);
mxArray *mxCreateDoubleScalar(double v);
mxArray *mxCreateDoubleMatrix(mwSize m, mwSize n, mxComplexity cplx);
mxArray *mxCreateString(const char *s);
void mxDestroyArray(mxArray *a);
void *mxGetData(const mxArray *a);
double *mxGetPr(const mxArray *a);
size_t mxGetNumberOfElements(const mxArray *a);
size_t mxGetM(const mxArray *a);
size_t mxGetN(const mxArray *a);
mxClassID mxGetClassID(const mxArray *a);
int mxIsChar(const mxArray *a);
double mxGetScalar(const mxArray *a);
char *mxArrayToString(const mxArray *a);
int mxGetString(const mxArray *a, char *buf, mwSize buflen);
void mxFree(void *p);

void mexErrMsgIdAndTxt(const char *id, const char *fmt, ...);
/* The MEX file's entry point (C linkage, as MATLAB's own header gives it). */
void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[]);
int mexPrintf(const char *fmt, ...);

/* ---- harness side (not part of MATLAB's API) ---- */
typedef void (*mexstub_fn)(int nlhs, mxArray *plhs[], int nrhs,
                           const mxArray *prhs[]);
/* Calls fn under an error trap.  Returns 0 on success; 1 when the callee
 * raised mexErrMsgIdAndTxt, with the identifier and message copied out. */
int mexstub_call(mexstub_fn fn, int nlhs, mxArray **plhs, int nrhs,
                 const mxArray **prhs, char *err_id, size_t id_len,
                 char *err_msg, size_t msg_len);
/* Wraps caller memory (copied) in a new 2-D numeric array. */
mxArray *mexstub_numeric(mxClassID cls, mwSize m, mwSize n, const void *src);
size_t mexstub_elsize(mxClassID cls);
/* Captured mexPrintf output since the last call (for tests). */
const char *mexstub_printed(void);

#ifdef __cplusplus
}
#endif
#endif
