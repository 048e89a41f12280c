/*
 * Implementation of the stand-in MEX API (mex.h in this folder) plus the entry points the
 * Python tests call through ctypes to build arguments, call mexFunction and read results.
 * Test infrastructure only.
 */
#include <setjmp.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "mex.h"

struct mxArray_tag {
  int cell;         /* 1: cell array, 0: real double matrix */
  int complex_flag; /* a flag the tests set to check the gateways' type checks */
  size_t m, n;
  double* data;     /* m*n doubles, column-major */
  mxArray** cells;  /* m*n elements */
};

static jmp_buf g_jmp;
static int g_in_call = 0;
static char g_err_id[128], g_err_msg[1024];
static int g_locked = 0;
static void (*g_exit_fn)(void) = NULL;

size_t mxGetM(const mxArray* a) { return a->m; }
size_t mxGetN(const mxArray* a) { return a->n; }
size_t mxGetNumberOfElements(const mxArray* a) { return a->m * a->n; }
double* mxGetDoubles(const mxArray* a) { return a->cell ? NULL : a->data; }
double mxGetScalar(const mxArray* a) { return (!a->cell && a->m * a->n > 0) ? a->data[0] : 0.0; }
int mxIsDouble(const mxArray* a) { return !a->cell; }
int mxIsCell(const mxArray* a) { return a->cell; }
int mxIsComplex(const mxArray* a) { return a->complex_flag; }
mxArray* mxGetCell(const mxArray* a, size_t i) { return (a->cell && i < a->m * a->n) ? a->cells[i] : NULL; }
void mxSetCell(mxArray* a, size_t i, mxArray* v) {
  if (a->cell && i < a->m * a->n) a->cells[i] = v;
}
mxArray* mxCreateDoubleMatrix(size_t m, size_t n, mxComplexity c) {
  mxArray* a = (mxArray*)calloc(1, sizeof(mxArray));
  a->m = m;
  a->n = n;
  a->complex_flag = c == mxCOMPLEX;
  a->data = (double*)calloc(m * n > 0 ? m * n : 1, sizeof(double));
  return a;
}
mxArray* mxCreateCellMatrix(size_t m, size_t n) {
  mxArray* a = (mxArray*)calloc(1, sizeof(mxArray));
  a->cell = 1;
  a->m = m;
  a->n = n;
  a->cells = (mxArray**)calloc(m * n > 0 ? m * n : 1, sizeof(mxArray*));
  return a;
}
void* mxMalloc(size_t n) { return malloc(n > 0 ? n : 1); }
void mxFree(void* p) { free(p); }
void mexErrMsgIdAndTxt(const char* id, const char* fmt, ...) {
  snprintf(g_err_id, sizeof g_err_id, "%s", id);
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err_msg, sizeof g_err_msg, fmt, ap);
  va_end(ap);
  if (g_in_call) longjmp(g_jmp, 1);
  abort(); /* a MEX error outside a harness call */
}
void mexLock(void) { g_locked = 1; }
void mexUnlock(void) { g_locked = 0; }
int mexIsLocked(void) { return g_locked; }
int mexAtExit(void (*fn)(void)) {
  g_exit_fn = fn;
  return 0;
}

/* ---- harness entry points (ctypes) ---- */
mxArray* stub_double(size_t m, size_t n, const double* src) {
  mxArray* a = mxCreateDoubleMatrix(m, n, mxREAL);
  if (src && m * n > 0) memcpy(a->data, src, m * n * sizeof(double));
  return a;
}
mxArray* stub_cell(size_t m, size_t n) { return mxCreateCellMatrix(m, n); }
void stub_set_cell(mxArray* a, size_t i, mxArray* v) { mxSetCell(a, i, v); }
mxArray* stub_get_cell(const mxArray* a, size_t i) { return mxGetCell(a, i); }
void stub_set_complex(mxArray* a, int flag) { a->complex_flag = flag; }
size_t stub_m(const mxArray* a) { return a->m; }
size_t stub_n(const mxArray* a) { return a->n; }
int stub_is_cell(const mxArray* a) { return a->cell; }
double* stub_data(const mxArray* a) { return a->data; }
void stub_destroy(mxArray* a) {
  if (!a) return;
  if (a->cell)
    for (size_t i = 0; i < a->m * a->n; ++i) stub_destroy(a->cells[i]);
  free(a->cells);
  free(a->data);
  free(a);
}
/* 0 on success, 1 when the gateway raised an error (id and message kept). */
int stub_call(int nlhs, mxArray** plhs, int nrhs, mxArray** prhs) {
  g_err_id[0] = g_err_msg[0] = '\0';
  for (int i = 0; i < nlhs; ++i) plhs[i] = NULL;
  g_in_call = 1;
  if (setjmp(g_jmp)) {
    g_in_call = 0;
    return 1;
  }
  mexFunction(nlhs, plhs, nrhs, (const mxArray**)prhs);
  g_in_call = 0;
  return 0;
}
const char* stub_err_id(void) { return g_err_id; }
const char* stub_err_msg(void) { return g_err_msg; }
int stub_locked(void) { return g_locked; }
/* What MATLAB does on "clear mex": run the gateway's exit hook and unlock it. */
void stub_clear(void) {
  if (g_exit_fn) g_exit_fn();
  g_exit_fn = NULL;
  g_locked = 0;
}
