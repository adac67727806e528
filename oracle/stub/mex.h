/*
 * Minimal stand-in for MATLAB's separate-complex MEX API (test infrastructure).
 *
 * MATLAB is not available on either build machine.  This header declares the
 * handful of mx/mex calls that the Helmholtz MEX gateways use, with MATLAB's
 * pre-R2018a semantics: real and imaginary parts live in separate column-major
 * double arrays (mxGetPr / mxGetPi).  mexstub.c implements them; a Python
 * ctypes harness builds mxArray structs around numpy buffers and calls the
 * gateway's mexFunction through mexstub_call(), which turns
 * mexErrMsgIdAndTxt into an error return instead of a MATLAB exception.
 *
 * Used by: oracle/Makefile (reference gateways, compiled unmodified) and the
 * drop-in gateway slim-release-apps_gb300/mex/h3d_mex_gateway.c.
 */
#ifndef H3D_MEXSTUB_MEX_H
#define H3D_MEXSTUB_MEX_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef size_t mwSize;
typedef size_t mwIndex;

typedef enum { mxREAL = 0, mxCOMPLEX = 1 } mxComplexity;

typedef struct mxArray_tag {
    size_t m;        /* rows */
    size_t n;        /* columns */
    double *pr;      /* real part, column-major, m*n doubles */
    double *pi;      /* imaginary part or NULL */
    int owns;        /* 1 if pr/pi were allocated by mxCreateDoubleMatrix */
} mxArray;

double *mxGetPr(const mxArray *a);
double *mxGetPi(const mxArray *a);
size_t mxGetM(const mxArray *a);
size_t mxGetN(const mxArray *a);
int mxIsComplex(const mxArray *a);
double mxGetScalar(const mxArray *a);
void *mxCalloc(size_t n, size_t size);
void mxFree(void *p);
mxArray *mxCreateDoubleMatrix(size_t m, size_t n, mxComplexity c);
void mexErrMsgIdAndTxt(const char *id, const char *fmt, ...);
int mexPrintf(const char *fmt, ...);

/* The gateway entry point every MEX file defines. */
void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[]);

/* Harness helpers (not part of MATLAB's API). */
int mexstub_call(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[],
                 char *err_id, size_t err_id_len);
void mexstub_destroy(mxArray *a);

#ifdef __cplusplus
}
#endif

#endif
