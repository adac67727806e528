/*
 * Drop-in MEX gateway for the GB300 Helmholtz library.
 *
 * One source, compiled once per reference binary name (the flag matrix of
 * ibin/install_MEX:88-114 in SLIM-release-apps):
 *
 *   -DH3D_GATEWAY_MVP   [-DADJ] [-DDERIV] [-DWNCMPLX]  -> Helm3dmvp_*_mex
 *       y = Helm3dmvp_xxx_mex(wn, h, n, npml, x, nthreads)       (Helm3dmvp_mex.c:17-48)
 *   -DH3D_GATEWAY_SWEEP [-DADJ] [-DWNCMPLX]            -> Helm3d_kacz_sweep_*_mex
 *       y = Helm3d_kacz_sweep_xxx_mex(wn, h, n, npml, w, x, b)   (Helm3dkaczswp_mex.c:21-50)
 *   -DH3D_GATEWAY_BAND_MVP                             -> Hmvp_MT_mex (install_MEX:75-76)
 *       y = Hmvp_MT_mex(coef, offset, x, nthreads)               (Hmvp_MT_mex.c:12-45)
 *   -DH3D_GATEWAY_BAND_SWEEP                           -> sweep_MT_mex (install_MEX:78-86)
 *       y = sweep_MT_mex(coef, offset, x, b, w, row_norms_sq)    (sweep_MT_mex.c:12-47)
 *   -DH3D_GATEWAY_SOLVE                                -> h3d_solve_mex (no reference binary)
 *       u = h3d_solve_mex(wn, h, n, npml, b, mode, tol, maxit[, precision[, stop]])
 *       the whole linearsolve.m:148-168 + CGMN.m:36-94 solve of a Helmholtz operator
 *       (H\b for mode 1, H'\b otherwise) in one call: precision 0 = FP64 (default), 1 =
 *       complex64 inner solves under FP64 refinement; stop 1 = true residual (default), 0 =
 *       CGMN.m:79's preconditioned residual.  Returns the last iterate when maxit is reached,
 *       as CGMN.m does.
 *
 *   -DH3D_GATEWAY_MLGMRES                              -> h3d_mlgmres_mex (no reference binary)
 *       u = h3d_mlgmres_mex(v, h, n, npml, freq, b, mode, tol, maxit[, precision[, unit]])
 *       linearsolve.m:139-141 with SOLVE_FGMRES preconditioned by ML_GMRES
 *       (discrete_helmholtz.m:349-350): the three-level hierarchy of construct_multigrid.m
 *       built from the physical model v (n = its three sizes, npml PML points added on every
 *       face, h the spacing, unit 0 = m/s (default), 1 = s2/m2, 2 = s2/km2) and FGMRES
 *       (restart 5) to tol on the PML grid; precision 0 = FP64 (default), 1 = complex64
 *       V-cycle under the complex128 FGMRES.  Each column of b is solved independently.
 *
 * Same argument order, same checks and error identifiers as the reference
 * gateways, same output (a new N x 1 or N x P complex double matrix).  The
 * arithmetic runs on the GPU through libh3d (include/h3d.h); nthreads is
 * accepted and ignored.  The sweep uses the reference's lexicographic row order
 * (H3D_ORDER_LEX), so results match the CPU gateway to rounding.
 *
 * Deliberate differences:
 *   - Helm3d_kacz_sweep_wnc_mex uses the imaginary part of wn (the reference's
 *     install line spells the flag -DWNCMPLEX, so its build silently drops it);
 *   - a b with fewer columns than x is rejected with the Bsize identifier instead
 *     of being read out of bounds;
 *   - sweep_MT_mex takes the 27 bands of a grid stencil (as helmholtz_3d.m builds them;
 *     the grid is read off the offsets), which the GPU sweeps as parallel hyperplanes;
 *     other band matrices are rejected;
 *   - Hmvp_MT_mex accepts at most 64 bands and at most 65535 right-hand-side columns per
 *     call (the reference has neither limit); larger calls are rejected with an error
 *     instead of being split.
 */
#include <stddef.h>
#include <stdio.h>

#include "h3d.h"
#include "mex.h"

#define ID_PREFIX "SLIM_release_apps:tools:algorithms:ThreeDFreqModeling:"

static void fail(int status, const char *gateway)
{
    static char id[160];
    const char *which = "h3d";
    switch (status) {
    case H3D_ERR_NSIZE: which = "Nsize"; break;
    case H3D_ERR_XSIZE: which = "Xsize"; break;
    case H3D_ERR_BSIZE: which = "Bsize"; break;
    default: break;
    }
    if (which[0] == 'h') {
        mexErrMsgIdAndTxt(h3d_status_id(status), "%s", h3d_last_error());
        return;
    }
    /* The reference's matvec reports an x-size error with the sweep gateway's prefix
     * (Helm3dmvp_mex.c:83); keep that. */
    if (status == H3D_ERR_XSIZE) gateway = "Helm3dkaczswp_mex";
    snprintf(id, sizeof id, ID_PREFIX "%s:%s", gateway, which);
    mexErrMsgIdAndTxt(id, "%s", h3d_last_error());
}

#ifdef ADJ
#define H3D_MODE H3D_ADJOINT
#else
#define H3D_MODE H3D_FORWARD
#endif

#ifdef DERIV
#define H3D_DERIV 1
#else
#define H3D_DERIV 0
#endif

static size_t n_len_of(const mxArray *n)
{
    /* Helm3dmvp_mex.c:75 / Helm3dkaczswp_mex.c:143: accepted when either dimension is 3. */
    return (mxGetM(n) == 3 || mxGetN(n) == 3) ? 3 : 0;
}

#if defined(H3D_GATEWAY_MVP)

void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[])
{
    (void)nlhs;
    if (nrhs < 5) mexErrMsgIdAndTxt("h3d:badArgument", "expected (wn,h,n,npml,x[,nthreads])");
    const mxArray *WN = prhs[0], *H = prhs[1], *N = prhs[2], *NPML = prhs[3], *X = prhs[4];
    const size_t nl = n_len_of(N);
    if (nl != 3) {
        fail(H3D_ERR_NSIZE, "Helm3dmvp_mex");
        return;
    }
    const double *n = mxGetPr(N);
    const size_t numel = (size_t)n[0] * (size_t)n[1] * (size_t)n[2];
    if (mxGetM(X) != numel) {
        fail(H3D_ERR_XSIZE, "Helm3dmvp_mex");
        return;
    }
#ifdef WNCMPLX
    const double *wni = mxIsComplex(WN) ? mxGetPi(WN) : NULL;
#else
    const double *wni = NULL;
#endif
    plhs[0] = mxCreateDoubleMatrix(numel, 1, mxCOMPLEX);
    int rc = h3d_mex_mvp(mxGetPr(WN), wni, mxGetPr(H), n, nl, mxGetPr(NPML), mxGetPr(X),
                         mxIsComplex(X) ? mxGetPi(X) : NULL, mxGetM(X), mxGetPr(plhs[0]),
                         mxGetPi(plhs[0]), H3D_MODE, H3D_DERIV);
    if (rc != H3D_OK) fail(rc, "Helm3dmvp_mex");
}

#elif defined(H3D_GATEWAY_SWEEP)

void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[])
{
    (void)nlhs;
    if (nrhs < 7) mexErrMsgIdAndTxt("h3d:badArgument", "expected (wn,h,n,npml,w,x,b)");
    const mxArray *WN = prhs[0], *H = prhs[1], *N = prhs[2], *NPML = prhs[3], *OMEGA = prhs[4],
                  *X = prhs[5], *B = prhs[6];
    const size_t nl = n_len_of(N);
    if (nl != 3) {
        fail(H3D_ERR_NSIZE, "Helm3dkaczswp_mex");
        return;
    }
    const double *n = mxGetPr(N);
    const size_t numel = (size_t)n[0] * (size_t)n[1] * (size_t)n[2];
    if (mxGetM(X) != numel) {
        fail(H3D_ERR_XSIZE, "Helm3dkaczswp_mex");
        return;
    }
    const size_t P = mxGetN(X);
    if (mxGetM(B) != numel || mxGetN(B) < P) {
        fail(H3D_ERR_BSIZE, "Helm3dkaczswp_mex");
        return;
    }
#ifdef WNCMPLX
    const double *wni = mxIsComplex(WN) ? mxGetPi(WN) : NULL;
#else
    const double *wni = NULL;
#endif
    plhs[0] = mxCreateDoubleMatrix(numel, P, mxCOMPLEX);
    int rc = h3d_mex_kacz_sweep(mxGetPr(WN), wni, mxGetPr(H), n, nl, mxGetPr(NPML),
                                mxGetScalar(OMEGA), mxGetPr(X), mxIsComplex(X) ? mxGetPi(X) : NULL,
                                mxGetM(X), P, mxGetPr(B), mxIsComplex(B) ? mxGetPi(B) : NULL,
                                mxGetM(B), mxGetPr(plhs[0]), mxGetPi(plhs[0]), H3D_MODE,
                                H3D_ORDER_LEX);
    if (rc != H3D_OK) fail(rc, "Helm3dkaczswp_mex");
}

#elif defined(H3D_GATEWAY_SOLVE)

void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[])
{
    (void)nlhs;
    if (nrhs < 8) mexErrMsgIdAndTxt("h3d:badArgument", "expected (wn,h,n,npml,b,mode,tol,maxit[,precision[,stop]])");
    const mxArray *WN = prhs[0], *H = prhs[1], *N = prhs[2], *NPML = prhs[3], *B = prhs[4];
    const size_t nl = n_len_of(N);
    if (nl != 3) {
        fail(H3D_ERR_NSIZE, "h3d_solve_mex");
        return;
    }
    const double *n = mxGetPr(N);
    const size_t numel = (size_t)n[0] * (size_t)n[1] * (size_t)n[2];
    if (mxGetM(B) != numel) {
        fail(H3D_ERR_BSIZE, "h3d_solve_mex");
        return;
    }
    h3d_solve_opts o;
    h3d_default_opts(&o);
    o.tol = mxGetScalar(prhs[6]);
    o.maxit = (int32_t)mxGetScalar(prhs[7]);
    if (nrhs > 8) o.precision = mxGetScalar(prhs[8]) != 0.0 ? H3D_PREC_MIXED : H3D_PREC_FP64;
    if (nrhs > 9) o.stop_rule = mxGetScalar(prhs[9]) != 0.0 ? H3D_STOP_TRUE_RESIDUAL : H3D_STOP_PRECONDITIONED;
    const int mode = mxGetScalar(prhs[5]) == 1.0 ? H3D_FORWARD : H3D_ADJOINT;   /* linearsolve.m:52-60 */
    const size_t P = mxGetN(B);
    plhs[0] = mxCreateDoubleMatrix(numel, P, mxCOMPLEX);
    int rc = h3d_mex_solve(mxGetPr(WN), mxIsComplex(WN) ? mxGetPi(WN) : NULL, mxGetPr(H), n, nl, mxGetPr(NPML),
                           mxGetPr(B), mxIsComplex(B) ? mxGetPi(B) : NULL, mxGetM(B), P, mxGetPr(plhs[0]),
                           mxGetPi(plhs[0]), mode, &o, NULL);
    if (rc != H3D_OK && rc != H3D_ERR_NOT_CONVERGED) fail(rc, "h3d_solve_mex");
}

#elif defined(H3D_GATEWAY_MLGMRES)

void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[])
{
    (void)nlhs;
    if (nrhs < 9)
        mexErrMsgIdAndTxt("h3d:badArgument", "expected (v,h,n,npml,freq,b,mode,tol,maxit[,precision[,unit]])");
    const mxArray *V = prhs[0], *H = prhs[1], *N = prhs[2], *B = prhs[5];
    const size_t nl = n_len_of(N);
    if (nl != 3) {
        fail(H3D_ERR_NSIZE, "h3d_mlgmres_mex");
        return;
    }
    const double *n = mxGetPr(N);
    const double npml = mxGetScalar(prhs[3]);
    h3d_ml_opts o;
    h3d_ml_default_opts(&o);
    o.tol = mxGetScalar(prhs[7]);
    o.maxit = (int32_t)mxGetScalar(prhs[8]);
    if (nrhs > 9) o.precision = mxGetScalar(prhs[9]) != 0.0 ? H3D_PREC_MIXED : H3D_PREC_FP64;
    const int unit = nrhs > 10 ? (int)mxGetScalar(prhs[10]) : H3D_UNIT_M_PER_S;
    const int mode = mxGetScalar(prhs[6]) == 1.0 ? H3D_FORWARD : H3D_ADJOINT;   /* linearsolve.m:52-60 */
    const size_t P = mxGetN(B), rows = mxGetM(B);
    plhs[0] = mxCreateDoubleMatrix(rows, P, mxCOMPLEX);
    int rc = h3d_mex_mlgmres(mxGetPr(V), n, nl, mxGetPr(H), npml, mxGetScalar(prhs[4]), unit, 3, mxGetPr(B),
                             mxIsComplex(B) ? mxGetPi(B) : NULL, rows, P, mxGetPr(plhs[0]), mxGetPi(plhs[0]), mode,
                             &o, NULL);
    if (rc != H3D_OK) fail(rc, "h3d_mlgmres_mex");
}

#elif defined(H3D_GATEWAY_BAND_MVP) || defined(H3D_GATEWAY_BAND_SWEEP)

#define BAND_ID ID_PREFIX "HMvp_MT_mex:NumElements"

static void band_fail(int status)
{
    if (status == H3D_ERR_XSIZE || status == H3D_ERR_BSIZE)
        mexErrMsgIdAndTxt(BAND_ID, "%s", h3d_last_error());
    else
        mexErrMsgIdAndTxt(h3d_status_id(status), "%s", h3d_last_error());
}

#if defined(H3D_GATEWAY_BAND_MVP)

void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[])
{
    (void)nlhs;
    if (nrhs < 3) mexErrMsgIdAndTxt("h3d:badArgument", "expected (coef,offset,x[,nthreads])");
    const mxArray *COEF = prhs[0], *OFF = prhs[1], *X = prhs[2];
    const size_t n = mxGetN(COEF), nd = mxGetM(COEF);
    if (mxGetM(X) != n) {
        mexErrMsgIdAndTxt(BAND_ID, "The row size of the vector x and the column size of the matrix A must match");
        return;
    }
    const size_t P = mxGetN(X);
    plhs[0] = mxCreateDoubleMatrix(n, P, mxCOMPLEX);
    int rc = h3d_mex_band_mvp(mxGetPr(COEF), mxIsComplex(COEF) ? mxGetPi(COEF) : NULL, nd, n, mxGetPr(OFF),
                              mxGetPr(X), mxIsComplex(X) ? mxGetPi(X) : NULL, mxGetM(X), P, mxGetPr(plhs[0]),
                              mxGetPi(plhs[0]));
    if (rc != H3D_OK) band_fail(rc);
}

#else

void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[])
{
    (void)nlhs;
    if (nrhs < 6) mexErrMsgIdAndTxt("h3d:badArgument", "expected (coef,offset,x,b,w,row_norms_sq)");
    const mxArray *COEF = prhs[0], *OFF = prhs[1], *X = prhs[2], *B = prhs[3], *OMEGA = prhs[4], *RN = prhs[5];
    const size_t n = mxGetN(COEF), nd = mxGetM(COEF);
    if (mxGetM(X) != n) {
        mexErrMsgIdAndTxt(BAND_ID, "The row size of the vector x and the column size of the matrix A must match");
        return;
    }
    if (mxGetM(RN) != n) {
        mexErrMsgIdAndTxt(BAND_ID, "The size of the row norms vector and the rows size of the matrix A must match");
        return;
    }
    const size_t P = mxGetN(X);
    if (mxGetM(B) != n || mxGetN(B) < P) {
        mexErrMsgIdAndTxt(BAND_ID, "b must have as many rows as x and at least as many columns");
        return;
    }
    plhs[0] = mxCreateDoubleMatrix(n, P, mxCOMPLEX);
    int rc = h3d_mex_band_sweep(mxGetPr(COEF), mxIsComplex(COEF) ? mxGetPi(COEF) : NULL, nd, n, mxGetPr(OFF),
                                mxGetPr(X), mxIsComplex(X) ? mxGetPi(X) : NULL, mxGetM(X), P, mxGetPr(B),
                                mxIsComplex(B) ? mxGetPi(B) : NULL, mxGetM(B), mxGetScalar(OMEGA), mxGetPr(RN),
                                mxGetM(RN), mxGetPr(plhs[0]), mxGetPi(plhs[0]));
    if (rc != H3D_OK) band_fail(rc);
}

#endif

#else
#error "define H3D_GATEWAY_MVP, _SWEEP, _SOLVE, _MLGMRES, _BAND_MVP or _BAND_SWEEP"
#endif
