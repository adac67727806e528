// extern "C" entry points for operator application (matvec and Kaczmarz sweep), in the
// device-pointer form and in the MATLAB host layout used by the drop-in MEX gateway.
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "h3d_b8.cuh"
#include "h3d_internal.cuh"
#include "h3d_kernels.cuh"
#include "h3d_vec.cuh"

using namespace h3d;

namespace h3d {
const char *last_error();

// COLOUR27 and BLOCK8 (12x12x12 blocks) run on stored row coefficients formed here for
// this call, unless block[0] is -1 or they do not fit in device memory; then the kernels
// that form the coefficients themselves run (COLOUR27: the shared-memory tile kernel).
// Both give the same row order's result to rounding.
template <typename T>
static int kacz_sweep_t(const Op<T> &op, cplx<T> *x, const cplx<T> *b, int nrhs, T w, bool adj, int order,
                        const int32_t *block, cudaStream_t st)
{
    if (order == H3D_ORDER_COLOUR27 && !(block && block[0] == -1)) {
        DevBuf cb, rb;
        if (cb.alloc(sizeof(cplx<T>) * 27 * (size_t)op.N, st) == H3D_OK &&
            rb.alloc(sizeof(T) * (size_t)op.N, st) == H3D_OK) {
            int rc = store_row_coefs<T>(op, adj, cb.as<cplx<T>>(), st);
            if (!rc) rc = row_inv_norms<T>(op, adj, rb.as<T>(), st);
            if (!rc) rc = launch_sweep<T>(op, x, b, nrhs, w, adj, order, block, nullptr, st, rb.as<T>(), -1, cb.as<cplx<T>>());
            return rc;
        }
        (void)cudaGetLastError();  // out of memory is not sticky: fall back to the tile kernel
    }
    const bool blk12 = !block || block[0] == 0 || (block[0] == 12 && block[1] == 12 && block[2] == 12);
    if (order == H3D_ORDER_BLOCK8 && blk12) {
        // the batched BLOCK8 kernel on one problem (stored coefficients, bulk-copied slabs);
        // its status word is read back, so this call synchronises the stream
        B8Batch<T> batch;
        batch.add(op, adj, 0, 0, nrhs);
        int rc = batch.setup(st);
        if (rc == H3D_ERR_NO_MEMORY) {
            (void)cudaGetLastError();  // out of memory is not sticky: fall back below
        } else {
            if (rc) return rc;
            const bool fp64 = sizeof(T) == 8;
            int c = 0;  // the largest right-hand-side group the columns fill
            for (int k = 1; k < b8_num_cfgs(fp64); ++k)
                if (b8_cfg(fp64, k).r <= nrhs) c = k;
            // H3D_BLOCK8_CONFIG=<index> fixes the configuration (for tests of each of them)
            if (const char *env = std::getenv("H3D_BLOCK8_CONFIG")) {
                const int k = std::atoi(env);
                if (k >= 0 && k < b8_num_cfgs(fp64)) c = k;
            }
            if ((rc = batch.configure(c, st)) || (rc = batch.dsweep(x, b, w, nullptr, st))) return rc;
            int status = 0;
            H3D_CUDA_TRY(cudaMemcpyAsync(&status, batch.err, sizeof(int), cudaMemcpyDeviceToHost, st));
            H3D_CUDA_TRY(cudaStreamSynchronize(st));
            if (status) {
                set_error("a bounded wait of the BLOCK8 sweep expired (device status %d)", status);
                return H3D_ERR_TIMEOUT;
            }
            return H3D_OK;
        }
    }
    return launch_sweep<T>(op, x, b, nrhs, w, adj, order, block, nullptr, st);
}

}  // namespace h3d

extern "C" {

int h3d_version(void) { return H3D_API_VERSION; }

const char *h3d_last_error(void) { return h3d::last_error(); }

const char *h3d_status_id(int status)
{
    // Identifiers of the reference gateways (Helm3dmvp_mex.c:77,83; Helm3dkaczswp_mex.c:145,157,162).
    switch (status) {
    case H3D_OK: return "";
    case H3D_ERR_NSIZE: return "SLIM_release_apps:tools:algorithms:ThreeDFreqModeling:Helm3dmvp_mex:Nsize";
    case H3D_ERR_XSIZE: return "SLIM_release_apps:tools:algorithms:ThreeDFreqModeling:Helm3dkaczswp_mex:Xsize";
    case H3D_ERR_BSIZE: return "SLIM_release_apps:tools:algorithms:ThreeDFreqModeling:Helm3dkaczswp_mex:Bsize";
    case H3D_ERR_BAD_ARG: return "h3d:badArgument";
    case H3D_ERR_NOT_CONVERGED: return "h3d:notConverged";
    case H3D_ERR_TIMEOUT: return "h3d:deviceTimeout";
    case H3D_ERR_CUDA: return "h3d:cudaError";
    case H3D_ERR_NO_MEMORY: return "h3d:outOfMemory";
    case H3D_ERR_NONFINITE: return "h3d:nonFinite";
    default: return "h3d:unknown";
    }
}

void h3d_default_opts(h3d_solve_opts *o)
{
    if (!o) return;
    std::memset(o, 0, sizeof *o);
    o->tol = 1e-6;
    o->maxit = 10000;
    o->w = 1.5;
    o->precision = H3D_PREC_FP64;
    o->order = H3D_ORDER_BLOCK8;
    o->stop_rule = H3D_STOP_TRUE_RESIDUAL;
    o->check_every = 25;
    o->inner_tol = 1e-3;
    o->max_outer = 20;
    o->use_graphs = 1;
}

int h3d_mvp(const h3d_grid *g, const void *wn_re, const void *wn_im, const void *x, void *y,
            int nrhs, int mode, int deriv, int dtype, void *stream)
{
    if (!wn_re || !x || !y || nrhs < 1 || (mode != H3D_FORWARD && mode != H3D_ADJOINT)) {
        set_error("h3d_mvp: bad argument");
        return H3D_ERR_BAD_ARG;
    }
    cudaStream_t st = (cudaStream_t)stream;
    if (dtype == H3D_C128) {
        Op<double> op;
        int rc = make_op_f64(g, (const double *)wn_re, (const double *)wn_im, &op);
        if (rc) return rc;
        return launch_mvp<double>(op, (const cplx<double> *)x, (cplx<double> *)y, nrhs,
                                  mode == H3D_ADJOINT, deriv != 0, st);
    }
    if (dtype == H3D_C64) {
        Op<float> op;
        int rc = make_op_f32(g, (const float *)wn_re, (const float *)wn_im, &op);
        if (rc) return rc;
        return launch_mvp<float>(op, (const cplx<float> *)x, (cplx<float> *)y, nrhs,
                                 mode == H3D_ADJOINT, deriv != 0, st);
    }
    set_error("h3d_mvp: unknown dtype %d", dtype);
    return H3D_ERR_BAD_ARG;
}

int h3d_kacz_sweep(const h3d_grid *g, const void *wn_re, const void *wn_im, double w, void *x,
                   const void *b, int nrhs, int mode, int order, const int32_t *block, int dtype,
                   void *stream)
{
    if (!wn_re || !x || nrhs < 1 || (mode != H3D_FORWARD && mode != H3D_ADJOINT) || !std::isfinite(w)) {
        set_error("h3d_kacz_sweep: bad argument");
        return H3D_ERR_BAD_ARG;
    }
    cudaStream_t st = (cudaStream_t)stream;
    if (dtype == H3D_C128) {
        Op<double> op;
        int rc = make_op_f64(g, (const double *)wn_re, (const double *)wn_im, &op);
        if (rc) return rc;
        return kacz_sweep_t<double>(op, (cplx<double> *)x, (const cplx<double> *)b, nrhs, w,
                                    mode == H3D_ADJOINT, order, block, st);
    }
    if (dtype == H3D_C64) {
        Op<float> op;
        int rc = make_op_f32(g, (const float *)wn_re, (const float *)wn_im, &op);
        if (rc) return rc;
        return kacz_sweep_t<float>(op, (cplx<float> *)x, (const cplx<float> *)b, nrhs, (float)w,
                                   mode == H3D_ADJOINT, order, block, st);
    }
    set_error("h3d_kacz_sweep: unknown dtype %d", dtype);
    return H3D_ERR_BAD_ARG;
}

// ---- MATLAB host layout -------------------------------------------------------------------

static int grid_from_mex(const double *h, const double *n, size_t n_len, const double *npml,
                         h3d_grid *g)
{
    if (!n || n_len != 3) {
        set_error("n must be a 3-length vector");
        return H3D_ERR_NSIZE;
    }
    if (!h || !npml) {
        set_error("h and npml are required");
        return H3D_ERR_BAD_ARG;
    }
    for (int a = 0; a < 3; ++a) {
        g->n[a] = (int32_t)n[a];
        g->h[a] = h[a];
    }
    for (int a = 0; a < 6; ++a) g->npml[a] = (int32_t)npml[a];
    return check_grid(g);
}

int h3d_mex_mvp(const double *wn_re, const double *wn_im, const double *h, const double *n,
                size_t n_len, const double *npml, const double *x_re, const double *x_im,
                size_t x_rows, double *y_re, double *y_im, int mode, int deriv)
{
    h3d_grid g;
    int rc = grid_from_mex(h, n, n_len, npml, &g);
    if (rc) return rc;
    const long long N = (long long)g.n[0] * g.n[1] * g.n[2];
    if ((long long)x_rows != N) {
        set_error("x must have nx*ny*nz elements");
        return H3D_ERR_XSIZE;
    }
    if (!wn_re || !x_re || !y_re || !y_im) {
        set_error("h3d_mex_mvp: NULL array");
        return H3D_ERR_BAD_ARG;
    }
    cudaStream_t st = nullptr;
    H3D_CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    rc = [&]() -> int {
        DevBuf dwr, dwi, dpl, dx, dy;
        const size_t pb = (size_t)N * sizeof(double);
        if ((rc = dwr.alloc(pb, st)) || (wn_im && (rc = dwi.alloc(pb, st))) ||
            (rc = dpl.alloc(2 * pb, st)) || (rc = dx.alloc(2 * pb, st)) || (rc = dy.alloc(2 * pb, st)))
            return rc;
        H3D_CUDA_TRY(cudaMemcpyAsync(dwr.p, wn_re, pb, cudaMemcpyHostToDevice, st));
        if (wn_im) H3D_CUDA_TRY(cudaMemcpyAsync(dwi.p, wn_im, pb, cudaMemcpyHostToDevice, st));
        double *pre = dpl.as<double>(), *pim = pre + N;
        H3D_CUDA_TRY(cudaMemcpyAsync(pre, x_re, pb, cudaMemcpyHostToDevice, st));
        if (x_im) H3D_CUDA_TRY(cudaMemcpyAsync(pim, x_im, pb, cudaMemcpyHostToDevice, st));
        if ((rc = interleave<double>(pre, x_im ? pim : nullptr, dx.as<cplx<double>>(), N, st))) return rc;
        if ((rc = h3d_mvp(&g, dwr.p, wn_im ? dwi.p : nullptr, dx.p, dy.p, 1, mode, deriv, H3D_C128, st)))
            return rc;
        if ((rc = deinterleave<double>(dy.as<cplx<double>>(), pre, pim, N, st))) return rc;
        H3D_CUDA_TRY(cudaMemcpyAsync(y_re, pre, pb, cudaMemcpyDeviceToHost, st));
        H3D_CUDA_TRY(cudaMemcpyAsync(y_im, pim, pb, cudaMemcpyDeviceToHost, st));
        return H3D_OK;
    }();
    cudaError_t e = cudaStreamSynchronize(st);
    cudaStreamDestroy(st);
    if (rc) return rc;
    if (e != cudaSuccess) return cuda_fail(e, "h3d_mex_mvp");
    return H3D_OK;
}

int h3d_mex_kacz_sweep(const double *wn_re, const double *wn_im, const double *h,
                       const double *n, size_t n_len, const double *npml, double w,
                       const double *x_re, const double *x_im, size_t x_rows, size_t nrhs,
                       const double *b_re, const double *b_im, size_t b_rows, double *y_re,
                       double *y_im, int mode, int order)
{
    h3d_grid g;
    int rc = grid_from_mex(h, n, n_len, npml, &g);
    if (rc) return rc;
    const long long N = (long long)g.n[0] * g.n[1] * g.n[2];
    if ((long long)x_rows != N) {
        set_error("x must have nx*ny*nz elements");
        return H3D_ERR_XSIZE;
    }
    if ((long long)b_rows != N) {
        set_error("b must have nx*ny*nz elements");
        return H3D_ERR_BSIZE;
    }
    if (!wn_re || !x_re || !b_re || !y_re || !y_im || nrhs < 1) {
        set_error("h3d_mex_kacz_sweep: bad argument");
        return H3D_ERR_BAD_ARG;
    }
    const long long M = N * (long long)nrhs;
    cudaStream_t st = nullptr;
    H3D_CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    rc = [&]() -> int {
        DevBuf dwr, dwi, dpl, dx, db;
        const size_t pb = (size_t)N * sizeof(double), mb = (size_t)M * sizeof(double);
        if ((rc = dwr.alloc(pb, st)) || (wn_im && (rc = dwi.alloc(pb, st))) ||
            (rc = dpl.alloc(2 * mb, st)) || (rc = dx.alloc(2 * mb, st)) || (rc = db.alloc(2 * mb, st)))
            return rc;
        H3D_CUDA_TRY(cudaMemcpyAsync(dwr.p, wn_re, pb, cudaMemcpyHostToDevice, st));
        if (wn_im) H3D_CUDA_TRY(cudaMemcpyAsync(dwi.p, wn_im, pb, cudaMemcpyHostToDevice, st));
        double *pre = dpl.as<double>(), *pim = pre + M;
        H3D_CUDA_TRY(cudaMemcpyAsync(pre, x_re, mb, cudaMemcpyHostToDevice, st));
        if (x_im) H3D_CUDA_TRY(cudaMemcpyAsync(pim, x_im, mb, cudaMemcpyHostToDevice, st));
        if ((rc = interleave<double>(pre, x_im ? pim : nullptr, dx.as<cplx<double>>(), M, st))) return rc;
        H3D_CUDA_TRY(cudaMemcpyAsync(pre, b_re, mb, cudaMemcpyHostToDevice, st));
        if (b_im) H3D_CUDA_TRY(cudaMemcpyAsync(pim, b_im, mb, cudaMemcpyHostToDevice, st));
        if ((rc = interleave<double>(pre, b_im ? pim : nullptr, db.as<cplx<double>>(), M, st))) return rc;
        if ((rc = h3d_kacz_sweep(&g, dwr.p, wn_im ? dwi.p : nullptr, w, dx.p, db.p, (int)nrhs, mode,
                                 order, nullptr, H3D_C128, st)))
            return rc;
        if ((rc = deinterleave<double>(dx.as<cplx<double>>(), pre, pim, M, st))) return rc;
        H3D_CUDA_TRY(cudaMemcpyAsync(y_re, pre, mb, cudaMemcpyDeviceToHost, st));
        H3D_CUDA_TRY(cudaMemcpyAsync(y_im, pim, mb, cudaMemcpyDeviceToHost, st));
        return H3D_OK;
    }();
    cudaError_t e = cudaStreamSynchronize(st);
    cudaStreamDestroy(st);
    if (rc) return rc;
    if (e != cudaSuccess) return cuda_fail(e, "h3d_mex_kacz_sweep");
    return H3D_OK;
}

int h3d_check_wait_timeout(double limit_ms)
{
    if (!(limit_ms > 0) || limit_ms > 1000) {
        set_error("h3d_check_wait_timeout: limit_ms must lie in (0, 1000]");
        return H3D_ERR_BAD_ARG;
    }
    // An internal 24 x 24 x 24 problem (PML 6, h 20 m, 5 Hz, wavenumber of 2000 m/s): every
    // block has PML rows, so every step of the BLOCK8 kernel waits on a bulk copy.
    const int n = 24;
    const long long N = (long long)n * n * n;
    h3d_grid g{};
    for (int a = 0; a < 3; ++a) {
        g.n[a] = n;
        g.h[a] = 20.0;
    }
    for (int a = 0; a < 6; ++a) g.npml[a] = 6;
    cudaStream_t st = nullptr;
    H3D_CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    int status = 0;
    int rc = [&]() -> int {
        DevBuf wn, x;
        int r;
        if ((r = wn.alloc(sizeof(float) * (size_t)N, st)) || (r = x.alloc(sizeof(cplx<float>) * (size_t)N, st))) return r;
        const double k2 = std::pow(2.0 * M_PI * 5.0 / 2000.0, 2);
        std::vector<float> h((size_t)N, (float)k2);
        H3D_CUDA_TRY(cudaMemcpyAsync(wn.p, h.data(), sizeof(float) * (size_t)N, cudaMemcpyHostToDevice, st));
        H3D_CUDA_TRY(cudaMemsetAsync(x.p, 0, sizeof(cplx<float>) * (size_t)N, st));
        Op<float> op;
        if ((r = make_op_f32(&g, wn.as<float>(), nullptr, &op))) return r;
        B8Batch<float> batch;
        batch.add(op, false, 0, 0, 1);
        if ((r = batch.setup(st)) || (r = batch.configure(0, st))) return r;
        batch.wait_limit_ns = (unsigned long long)(limit_ms * 1e6);
        if ((r = batch.dsweep(x.as<cplx<float>>(), nullptr, 1.5f, nullptr, st, 1))) return r;
        H3D_CUDA_TRY(cudaMemcpyAsync(&status, batch.err, sizeof(int), cudaMemcpyDeviceToHost, st));
        H3D_CUDA_TRY(cudaStreamSynchronize(st));
        return H3D_OK;
    }();
    cudaError_t e = cudaStreamSynchronize(st);
    cudaStreamDestroy(st);
    if (rc) return rc;
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamSynchronize");
    if (status) set_error("the BLOCK8 sweep reported an expired wait (status %d)", status);
    return status;
}

}  // extern "C"
