/* Declarations of the MATLAB MEX / matrix API functions that
 * gmgs-3d_gb300/matlab/gmgs_mex.c calls, so the shim can be compiled and
 * linked here without MATLAB (tests/test_mex_shim.py).  Declarations only:
 * the shim is built against MATLAB's own headers with `mex`. */
#ifndef GMGS_TEST_MEX_STUB_H
#define GMGS_TEST_MEX_STUB_H
#include <stddef.h>

typedef struct mxArray_tag mxArray;
typedef size_t mwSize;
typedef enum { mxREAL = 0, mxCOMPLEX = 1 } mxComplexity;

mwSize mxGetNumberOfDimensions(const mxArray* a);
const mwSize* mxGetDimensions(const mxArray* a);
size_t mxGetM(const mxArray* a);
size_t mxGetN(const mxArray* a);
size_t mxGetNumberOfElements(const mxArray* a);
int mxIsInt32(const mxArray* a);
int mxIsDouble(const mxArray* a);
void* mxGetData(const mxArray* a);
double* mxGetPr(const mxArray* a);
double mxGetScalar(const mxArray* a);
mxArray* mxCreateDoubleMatrix(mwSize m, mwSize n, mxComplexity c);
mxArray* mxCreateDoubleScalar(double v);
void* mxMalloc(size_t n);
void mxFree(void* p);
void mexErrMsgIdAndTxt(const char* id, const char* fmt, ...);
void mexWarnMsgIdAndTxt(const char* id, const char* fmt, ...);
#endif
