/* Implementation of the test-only MEX API stand-in declared in mex.h. */
#include "mex.h"

#include <setjmp.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

struct mxArray_tag {
  mxClassID cls;
  size_t m, n;
  size_t elsize;
  void *data;
};

static jmp_buf *g_trap = NULL;
static char g_err_id[128];
static char g_err_msg[512];
static char g_printed[4096];
static size_t g_printed_len = 0;

size_t mexstub_elsize(mxClassID cls) {
  switch (cls) {
    case mxCHAR_CLASS: return 2;
    case mxDOUBLE_CLASS: return 8;
    case mxSINGLE_CLASS: return 4;
    case mxINT32_CLASS: return 4;
    case mxUINT32_CLASS: return 4;
    case mxUINT64_CLASS: return 8;
    default: return 1;
  }
}

mxArray *mxCreateNumericMatrix(mwSize m, mwSize n, mxClassID cls,
                               mxComplexity cplx) {
  (void)cplx;
  mxArray *a = (mxArray *)calloc(1, sizeof(mxArray));
  a->cls = cls;
  a->m = m;
  a->n = n;
  a->elsize = mexstub_elsize(cls);
  a->data = calloc(m * n ? m * n : 1, a->elsize);
  return a;
}

mxArray *mxCreateNumericArray(mwSize ndim, const mwSize *dims, mxClassID cls,
                              mxComplexity cplx) {
  size_t m = ndim > 0 ? dims[0] : 1, n = 1;
  for (mwSize d = 1; d < ndim; ++d) n *= dims[d];
  return mxCreateNumericMatrix(m, n, cls, cplx);
}

mxArray *mxCreateDoubleScalar(double v) {
  mxArray *a = mxCreateNumericMatrix(1, 1, mxDOUBLE_CLASS, mxREAL);
  *(double *)a->data = v;
  return a;
}

mxArray *mxCreateDoubleMatrix(mwSize m, mwSize n, mxComplexity cplx) {
  return mxCreateNumericMatrix(m, n, mxDOUBLE_CLASS, cplx);
}

mxArray *mxCreateString(const char *s) {
  size_t len = strlen(s);
  mxArray *a = mxCreateNumericMatrix(1, len, mxCHAR_CLASS, mxREAL);
  uint16_t *d = (uint16_t *)a->data;
  for (size_t i = 0; i < len; ++i) d[i] = (uint16_t)(unsigned char)s[i];
  return a;
}

mxArray *mexstub_numeric(mxClassID cls, mwSize m, mwSize n, const void *src) {
  mxArray *a = mxCreateNumericMatrix(m, n, cls, mxREAL);
  if (src) memcpy(a->data, src, m * n * a->elsize);
  return a;
}

void mxDestroyArray(mxArray *a) {
  if (!a) return;
  free(a->data);
  free(a);
}

void *mxGetData(const mxArray *a) { return a->data; }
double *mxGetPr(const mxArray *a) { return (double *)a->data; }
size_t mxGetNumberOfElements(const mxArray *a) { return a->m * a->n; }
size_t mxGetM(const mxArray *a) { return a->m; }
size_t mxGetN(const mxArray *a) { return a->n; }
mxClassID mxGetClassID(const mxArray *a) { return a->cls; }
int mxIsChar(const mxArray *a) { return a->cls == mxCHAR_CLASS; }

double mxGetScalar(const mxArray *a) {
  if (a->m * a->n == 0) return 0.0;
  switch (a->cls) {
    case mxDOUBLE_CLASS: return ((double *)a->data)[0];
    case mxSINGLE_CLASS: return ((float *)a->data)[0];
    case mxINT32_CLASS: return ((int32_t *)a->data)[0];
    case mxUINT32_CLASS: return ((uint32_t *)a->data)[0];
    case mxUINT64_CLASS: return (double)((uint64_t *)a->data)[0];
    default: return 0.0;
  }
}

char *mxArrayToString(const mxArray *a) {
  if (!a || a->cls != mxCHAR_CLASS) return NULL;
  size_t len = a->m * a->n;
  char *s = (char *)malloc(len + 1);
  const uint16_t *d = (const uint16_t *)a->data;
  for (size_t i = 0; i < len; ++i) s[i] = (char)d[i];
  s[len] = '\0';
  return s;
}

int mxGetString(const mxArray *a, char *buf, mwSize buflen) {
  char *s = mxArrayToString(a);
  if (!s || buflen == 0) { free(s); return 1; }
  strncpy(buf, s, buflen - 1);
  buf[buflen - 1] = '\0';
  int truncated = strlen(s) >= buflen;
  free(s);
  return truncated;
}

void mxFree(void *p) { free(p); }

int mexPrintf(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  int room = (int)(sizeof(g_printed) - g_printed_len);
  int n = 0;
  if (room > 1) {
    n = vsnprintf(g_printed + g_printed_len, (size_t)room, fmt, ap);
    if (n > 0) g_printed_len += (size_t)(n < room ? n : room - 1);
  }
  va_end(ap);
  return n;
}

const char *mexstub_printed(void) { return g_printed; }

void mexErrMsgIdAndTxt(const char *id, const char *fmt, ...) {
  snprintf(g_err_id, sizeof(g_err_id), "%s", id ? id : "");
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err_msg, sizeof(g_err_msg), fmt, ap);
  va_end(ap);
  if (g_trap) longjmp(*g_trap, 1);
  fprintf(stderr, "mexErrMsgIdAndTxt outside mexstub_call: %s: %s\n", g_err_id,
          g_err_msg);
  abort();
}

int mexstub_call(mexstub_fn fn, int nlhs, mxArray **plhs, int nrhs,
                 const mxArray **prhs, char *err_id, size_t id_len,
                 char *err_msg, size_t msg_len) {
  jmp_buf trap;
  jmp_buf *saved = g_trap;
  g_printed_len = 0;
  g_printed[0] = '\0';
  g_trap = &trap;
  if (setjmp(trap) != 0) {
    g_trap = saved;
    if (err_id && id_len) snprintf(err_id, id_len, "%s", g_err_id);
    if (err_msg && msg_len) snprintf(err_msg, msg_len, "%s", g_err_msg);
    return 1;
  }
  fn(nlhs, plhs, nrhs, prhs);
  g_trap = saved;
  return 0;
}
