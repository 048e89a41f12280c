/*
 * Minimal stand-in for MATLAB's mex.h / matrix.h, for compiling and exercising the MEX
 * gateways of this repository without MATLAB or Octave (test infrastructure).  It declares
 * only the part of the documented MEX C API (interleaved-complex, R2018a) the gateways use;
 * mexstub.c implements it with plain C structures and turns mexErrMsgIdAndTxt into a
 * longjmp back to the test harness.
 */
#ifndef ASG_TEST_MEX_H
#define ASG_TEST_MEX_H

#include <stddef.h>

typedef struct mxArray_tag mxArray;
typedef enum { mxREAL = 0, mxCOMPLEX = 1 } mxComplexity;

size_t mxGetM(const mxArray* a);
size_t mxGetN(const mxArray* a);
size_t mxGetNumberOfElements(const mxArray* a);
double* mxGetDoubles(const mxArray* a);
double mxGetScalar(const mxArray* a);
int mxIsDouble(const mxArray* a);
int mxIsCell(const mxArray* a);
int mxIsComplex(const mxArray* a);
mxArray* mxGetCell(const mxArray* a, size_t i);
void mxSetCell(mxArray* a, size_t i, mxArray* v);
mxArray* mxCreateDoubleMatrix(size_t m, size_t n, mxComplexity c);
mxArray* mxCreateCellMatrix(size_t m, size_t n);
void* mxMalloc(size_t n);
void mxFree(void* p);
void mexErrMsgIdAndTxt(const char* id, const char* fmt, ...);
void mexLock(void);
void mexUnlock(void);
int mexIsLocked(void);
int mexAtExit(void (*fn)(void));
void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]);

#endif
