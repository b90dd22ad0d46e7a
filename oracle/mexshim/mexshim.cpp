/*
 * mexshim.cpp -- implementation of the MEX stand-in (see mex.h) plus the
 * C entry point ref_call() through which tests and the CPU baseline call a
 * compiled reference gateway.  fft2/ifft2 requested through mexCallMATLAB
 * are served by or_fft.c.  mexErrMsgTxt unwinds to ref_call with longjmp.
 * TEST INFRASTRUCTURE ONLY.
 */
#include "mex.h"

#include <setjmp.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "or_fft.h"

struct mxArray_tag {
    size_t m, n;
    double* pr;
    double* pi;
};

static jmp_buf g_jmp;
static char g_err[512];

extern "C" {

double* mxGetPr(const mxArray* a) { return a->pr; }
double* mxGetPi(const mxArray* a) { return a->pi; }
size_t mxGetM(const mxArray* a) { return a->m; }
size_t mxGetN(const mxArray* a) { return a->n; }
double mxGetScalar(const mxArray* a) { return (a->m * a->n > 0 && a->pr) ? a->pr[0] : 0.0; }

mxArray* mxCreateDoubleMatrix(mwSize m, mwSize n, mxComplexity c) {
    mxArray* a = (mxArray*)calloc(1, sizeof(mxArray));
    a->m = m;
    a->n = n;
    size_t cnt = m * n > 0 ? m * n : 1;
    a->pr = (double*)calloc(cnt, sizeof(double));
    a->pi = c == mxCOMPLEX ? (double*)calloc(cnt, sizeof(double)) : NULL;
    return a;
}

void mxDestroyArray(mxArray* a) {
    if (!a) return;
    free(a->pr);
    free(a->pi);
    free(a);
}

void* mxMalloc(size_t n) { return malloc(n > 0 ? n : 1); }
void* mxCalloc(size_t n, size_t size) { return calloc(n > 0 ? n : 1, size > 0 ? size : 1); }
void mxFree(void* p) { free(p); }
void mxSetPr(mxArray* a, double* p) { if (a->pr != p) free(a->pr); a->pr = p; }
void mxSetPi(mxArray* a, double* p) { if (a->pi != p) free(a->pi); a->pi = p; }

void mexErrMsgTxt(const char* msg) {
    snprintf(g_err, sizeof(g_err), "%s", msg);
    longjmp(g_jmp, 1);
}

int mexPrintf(const char* fmt, ...) {
    (void)fmt;
    return 0;
}

int mexCallMATLAB(int nlhs, mxArray* plhs[], int nrhs, mxArray* prhs[], const char* name) {
    if (nlhs != 1 || nrhs != 1) mexErrMsgTxt("mexshim: only one-in/one-out calls are supported");
    int inverse;
    if (!strcmp(name, "fft2"))
        inverse = 0;
    else if (!strcmp(name, "ifft2"))
        inverse = 1;
    else
        mexErrMsgTxt("mexshim: unsupported MATLAB function");
    const mxArray* in = prhs[0];
    mxArray* out = mxCreateDoubleMatrix(in->m, in->n, mxCOMPLEX);
    size_t cnt = in->m * in->n;
    memcpy(out->pr, in->pr, cnt * sizeof(double));
    if (in->pi) memcpy(out->pi, in->pi, cnt * sizeof(double));
    if (or_fft2((int)in->m, (int)in->n, out->pr, out->pi, inverse)) mexErrMsgTxt("mexshim: fft failed");
    plhs[0] = out;
    return 0;
}

/*
 * Call the gateway linked into this library.  rhs i is an m[i] x n[i]
 * column-major double matrix; the first output is copied to `out` (at most
 * out_len values).  Returns 0, or -1 with the gateway's error text in err.
 */
int ref_call(int nrhs, const double* const* data, const long* m, const long* n, double* out, long out_len,
             char* err, int errlen) {
    mxArray* prhs[32];
    mxArray* plhs[1] = {NULL};
    if (nrhs > 32) return -2;
    for (int i = 0; i < nrhs; i++) {
        prhs[i] = mxCreateDoubleMatrix((mwSize)m[i], (mwSize)n[i], mxREAL);
        if (m[i] * n[i] > 0) memcpy(prhs[i]->pr, data[i], sizeof(double) * (size_t)(m[i] * n[i]));
    }
    int rc = 0;
    if (setjmp(g_jmp) == 0) {
        mexFunction(1, plhs, nrhs, (const mxArray**)prhs);
        if (plhs[0]) {
            long cnt = (long)(plhs[0]->m * plhs[0]->n);
            if (cnt > out_len) cnt = out_len;
            memcpy(out, plhs[0]->pr, sizeof(double) * (size_t)cnt);
        }
    } else {
        rc = -1;
        if (err && errlen > 0) snprintf(err, (size_t)errlen, "%s", g_err);
    }
    for (int i = 0; i < nrhs; i++) mxDestroyArray(prhs[i]);
    if (plhs[0]) mxDestroyArray(plhs[0]);
    return rc;
}

}  // extern "C"
