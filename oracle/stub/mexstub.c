/*
 * Implementation of the minimal MEX API declared in mex.h (test infrastructure).
 *
 * mexErrMsgIdAndTxt longjmps back into mexstub_call, which reports the error
 * identifier to the caller; this mirrors how MATLAB aborts a MEX call on error.
 * Memory handed out by mxCalloc during a call is not tracked: the Helmholtz
 * gateways free what they allocate before returning.
 */
#include <setjmp.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "mex.h"

static __thread jmp_buf *g_jmp = NULL;
static __thread char g_err_id[256];

double *mxGetPr(const mxArray *a) { return a->pr; }
double *mxGetPi(const mxArray *a) { return a->pi; }
size_t mxGetM(const mxArray *a) { return a->m; }
size_t mxGetN(const mxArray *a) { return a->n; }
int mxIsComplex(const mxArray *a) { return a->pi != NULL; }
double mxGetScalar(const mxArray *a) { return a->pr[0]; }

void *mxCalloc(size_t n, size_t size) { return calloc(n ? n : 1, size ? size : 1); }
void mxFree(void *p) { free(p); }

mxArray *mxCreateDoubleMatrix(size_t m, size_t n, mxComplexity c)
{
    mxArray *a = (mxArray *)calloc(1, sizeof(mxArray));
    size_t cnt = m * n ? m * n : 1;
    a->m = m;
    a->n = n;
    a->pr = (double *)calloc(cnt, sizeof(double));
    a->pi = (c == mxCOMPLEX) ? (double *)calloc(cnt, sizeof(double)) : NULL;
    a->owns = 1;
    return a;
}

void mexstub_destroy(mxArray *a)
{
    if (!a) return;
    if (a->owns) {
        free(a->pr);
        free(a->pi);
    }
    free(a);
}

int mexPrintf(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    int r = vprintf(fmt, ap);
    va_end(ap);
    return r;
}

void mexErrMsgIdAndTxt(const char *id, const char *fmt, ...)
{
    (void)fmt;
    snprintf(g_err_id, sizeof g_err_id, "%s", id ? id : "");
    if (g_jmp) longjmp(*g_jmp, 1);
    fprintf(stderr, "mexErrMsgIdAndTxt outside mexstub_call: %s\n", g_err_id);
    abort();
}

int mexstub_call(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[],
                 char *err_id, size_t err_id_len)
{
    jmp_buf env;
    jmp_buf *prev = g_jmp;
    g_jmp = &env;
    if (setjmp(env)) {
        g_jmp = prev;
        if (err_id && err_id_len) snprintf(err_id, err_id_len, "%s", g_err_id);
        return 1;
    }
    mexFunction(nlhs, plhs, nrhs, prhs);
    g_jmp = prev;
    if (err_id && err_id_len) err_id[0] = '\0';
    return 0;
}
