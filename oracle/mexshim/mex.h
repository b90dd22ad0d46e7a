/*
 * mex.h -- minimal stand-in for MATLAB's C MEX API (separate-complex storage,
 * the pre-R2018a API the reference gateways use), written for this project so
 * that the reference's C++ gateways can be compiled and called without
 * MATLAB.  TEST INFRASTRUCTURE ONLY: used to build the reference under
 * oracle/_ref, never by the shipped library.
 */
#ifndef FTE_MEXSHIM_MEX_H
#define FTE_MEXSHIM_MEX_H
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef size_t mwSize;
typedef enum { mxREAL = 0, mxCOMPLEX = 1 } mxComplexity;
typedef struct mxArray_tag mxArray;

double* mxGetPr(const mxArray* a);
double* mxGetPi(const mxArray* a);
size_t mxGetM(const mxArray* a);
size_t mxGetN(const mxArray* a);
double mxGetScalar(const mxArray* a);
mxArray* mxCreateDoubleMatrix(mwSize m, mwSize n, mxComplexity c);
void mxDestroyArray(mxArray* a);
void* mxMalloc(size_t n);
void* mxCalloc(size_t n, size_t size);
void mxFree(void* p);
void mxSetPr(mxArray* a, double* p);
void mxSetPi(mxArray* a, double* p);
void mexErrMsgTxt(const char* msg);
int mexPrintf(const char* fmt, ...);
int mexCallMATLAB(int nlhs, mxArray* plhs[], int nrhs, mxArray* prhs[], const char* name);

void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]);

#ifdef __cplusplus
}
#endif
#endif
