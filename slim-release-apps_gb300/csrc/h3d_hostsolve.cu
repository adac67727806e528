// Host-buffer entry points above sweep granularity: the solve behind linearsolve / CGMN with
// MATLAB's split-complex arrays (what the h3d_solve_mex gateway calls), and PDEfunc OBJ for
// one frequency and a batch of sources (what a MATLAB PDEfunc or a C caller reaches without
// any per-iteration host round trip).  Both are synchronous and own their device buffers.
#include <cmath>
#include <cstring>
#include <vector>

#include "h3d_internal.cuh"
#include "h3d_kernels.cuh"
#include "h3d_vec.cuh"

using namespace h3d;

namespace {

// Run f on a private non-blocking stream, synchronise it and destroy it.
template <typename F>
int on_private_stream(F f)
{
    cudaStream_t st = nullptr;
    H3D_CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    int rc = f(st);
    cudaError_t e = cudaStreamSynchronize(st);
    cudaStreamDestroy(st);
    if (rc) return rc;
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamSynchronize");
    return H3D_OK;
}

int grid_of_mex(const double *h, const double *n, size_t n_len, const double *npml, h3d_grid *g)
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
        if (!(n[a] >= 1) || n[a] > 2147483647.0 || n[a] != std::floor(n[a])) {
            set_error("n must hold three positive integer sizes");
            return H3D_ERR_NSIZE;
        }
        g->n[a] = (int32_t)n[a];
        g->h[a] = h[a];
    }
    for (int a = 0; a < 6; ++a) g->npml[a] = (int32_t)npml[a];
    return check_grid(g);
}

}  // namespace

extern "C" {

int h3d_mex_solve(const double *wn_re, const double *wn_im, const double *h, const double *n, size_t n_len,
                  const double *npml, const double *b_re, const double *b_im, size_t b_rows, size_t nrhs,
                  double *u_re, double *u_im, int mode, const h3d_solve_opts *opts, h3d_solve_info *info)
{
    h3d_grid g;
    int rc = grid_of_mex(h, n, n_len, npml, &g);
    if (rc) return rc;
    const long long N = (long long)g.n[0] * g.n[1] * g.n[2];
    if ((long long)b_rows != N) {
        set_error("b must have nx*ny*nz rows");
        return H3D_ERR_BSIZE;
    }
    if (!wn_re || !b_re || !u_re || !u_im || nrhs < 1 || nrhs > 2147483647u ||
        (mode != H3D_FORWARD && mode != H3D_ADJOINT)) {
        set_error("h3d_mex_solve: bad argument");
        return H3D_ERR_BAD_ARG;
    }
    const long long M = N * (long long)nrhs;
    int solve_rc = H3D_OK;
    rc = on_private_stream([&](cudaStream_t st) -> int {
        DevBuf dw, dpl, db, du;
        const size_t pb = (size_t)N * sizeof(double), mb = (size_t)M * sizeof(double);
        int r;
        if ((r = dw.alloc(pb * (wn_im ? 2 : 1), st)) || (r = dpl.alloc(2 * mb, st)) ||
            (r = db.alloc(2 * mb, st)) || (r = du.alloc(2 * mb, st)))
            return r;
        H3D_CUDA_TRY(cudaMemcpyAsync(dw.p, wn_re, pb, cudaMemcpyHostToDevice, st));
        if (wn_im) H3D_CUDA_TRY(cudaMemcpyAsync(dw.as<double>() + N, wn_im, pb, cudaMemcpyHostToDevice, st));
        double *pre = dpl.as<double>(), *pim = pre + M;
        H3D_CUDA_TRY(cudaMemcpyAsync(pre, b_re, mb, cudaMemcpyHostToDevice, st));
        if (b_im) H3D_CUDA_TRY(cudaMemcpyAsync(pim, b_im, mb, cudaMemcpyHostToDevice, st));
        if ((r = interleave<double>(pre, b_im ? pim : nullptr, db.as<cplx<double>>(), M, st))) return r;
        solve_rc = h3d_solve(&g, dw.as<double>(), wn_im ? dw.as<double>() + N : nullptr, db.p, du.p, (int)nrhs,
                             mode, opts, info, nullptr, 0, st);
        if (solve_rc && solve_rc != H3D_ERR_NOT_CONVERGED) return solve_rc;
        if ((r = deinterleave<double>(du.as<cplx<double>>(), pre, pim, M, st))) return r;
        H3D_CUDA_TRY(cudaMemcpyAsync(u_re, pre, mb, cudaMemcpyDeviceToHost, st));
        H3D_CUDA_TRY(cudaMemcpyAsync(u_im, pim, mb, cudaMemcpyDeviceToHost, st));
        return H3D_OK;
    });
    return rc ? rc : solve_rc;
}

int h3d_fwi_grad(const h3d_grid *g, const double *wn, const double *dwn, const double *src_pts, int nsrc,
                 const double *src_amp, const double *rec_pts, int nrec, const double *dobs,
                 const h3d_solve_opts *opts, double *f, double *g_phys, h3d_solve_info *info)
{
    int rc = check_grid(g);
    if (rc) return rc;
    if (!wn || !dwn || !src_pts || nsrc < 1 || !src_amp || !rec_pts || nrec < 1 || !dobs || !f || !g_phys) {
        set_error("h3d_fwi_grad: bad argument");
        return H3D_ERR_BAD_ARG;
    }
    const long long N = (long long)g->n[0] * g->n[1] * g->n[2];
    long long nphys = 1;
    for (int a = 0; a < 3; ++a) {
        const long long m = (long long)g->n[a] - g->npml[2 * a] - g->npml[2 * a + 1];
        if (m < 1) {
            set_error("h3d_fwi_grad: the PML leaves no physical grid");
            return H3D_ERR_NSIZE;
        }
        nphys *= m;
    }
    // sinc-Kaiser weights of the sources and receivers (opInterp.m, opSincInterp.m)
    std::vector<int32_t> sbase((size_t)nsrc * 3), rbase((size_t)nrec * 3);
    std::vector<double> sw((size_t)nsrc * 27), rw((size_t)nrec * 27);
    if ((rc = h3d_sinc_weights(g, src_pts, nsrc, sbase.data(), sw.data()))) return rc;
    if ((rc = h3d_sinc_weights(g, rec_pts, nrec, rbase.data(), rw.data()))) return rc;
    int solve_rc = H3D_OK;
    rc = on_private_stream([&](cudaStream_t st) -> int {
        DevBuf dw, dd, dsb, dsw, drb, drw, dsa, dU, dV, dres, dg;
        const size_t vb = sizeof(cplx<double>) * (size_t)N * nsrc;
        int r;
        if ((r = dw.alloc(sizeof(double) * (size_t)N, st)) || (r = dd.alloc(sizeof(double) * (size_t)N, st)) ||
            (r = dsb.alloc(sizeof(int32_t) * sbase.size(), st)) || (r = dsw.alloc(sizeof(double) * sw.size(), st)) ||
            (r = drb.alloc(sizeof(int32_t) * rbase.size(), st)) || (r = drw.alloc(sizeof(double) * rw.size(), st)) ||
            (r = dsa.alloc(sizeof(double) * 2 * (size_t)nsrc, st)) || (r = dU.alloc(vb, st)) ||
            (r = dV.alloc(vb, st)) || (r = dres.alloc(sizeof(cplx<double>) * (size_t)nrec * nsrc, st)) ||
            (r = dg.alloc(sizeof(double) * (size_t)nphys, st)))
            return r;
        H3D_CUDA_TRY(cudaMemcpyAsync(dw.p, wn, sizeof(double) * (size_t)N, cudaMemcpyHostToDevice, st));
        H3D_CUDA_TRY(cudaMemcpyAsync(dd.p, dwn, sizeof(double) * (size_t)N, cudaMemcpyHostToDevice, st));
        H3D_CUDA_TRY(cudaMemcpyAsync(dsb.p, sbase.data(), sizeof(int32_t) * sbase.size(), cudaMemcpyHostToDevice, st));
        H3D_CUDA_TRY(cudaMemcpyAsync(dsw.p, sw.data(), sizeof(double) * sw.size(), cudaMemcpyHostToDevice, st));
        H3D_CUDA_TRY(cudaMemcpyAsync(drb.p, rbase.data(), sizeof(int32_t) * rbase.size(), cudaMemcpyHostToDevice, st));
        H3D_CUDA_TRY(cudaMemcpyAsync(drw.p, rw.data(), sizeof(double) * rw.size(), cudaMemcpyHostToDevice, st));
        H3D_CUDA_TRY(cudaMemcpyAsync(dsa.p, src_amp, sizeof(double) * 2 * (size_t)nsrc, cudaMemcpyHostToDevice, st));
        // Q = Ps (w Q_s) (PDEfunc.m:330-339), U = H \ Q (PDEfunc.m:347)
        H3D_CUDA_TRY(cudaMemsetAsync(dV.p, 0, vb, st));
        if ((r = h3d_src_inject(g, dsb.as<int32_t>(), dsw.as<double>(), dsa.as<double>(), dV.p, nsrc, st))) return r;
        solve_rc = h3d_solve(g, dw.as<double>(), nullptr, dV.p, dU.p, nsrc, H3D_FORWARD, opts, info, nullptr, 0, st);
        if (solve_rc && solve_rc != H3D_ERR_NOT_CONVERGED) return solve_rc;
        // D = Pr U; the residual and f = 1/2 ||D - Dobs||^2 on the host (LS_misfit.m:21-26)
        if ((r = h3d_rec_sample(g, drb.as<int32_t>(), drw.as<double>(), nrec, dU.p, nsrc, dres.p, st))) return r;
        std::vector<double> res((size_t)nrec * nsrc * 2);
        H3D_CUDA_TRY(cudaMemcpyAsync(res.data(), dres.p, sizeof(double) * res.size(), cudaMemcpyDeviceToHost, st));
        H3D_CUDA_TRY(cudaStreamSynchronize(st));
        double fsum = 0.0;
        for (size_t e = 0; e < res.size(); ++e) {
            res[e] -= dobs[e];
            fsum += res[e] * res[e];
        }
        *f = 0.5 * fsum;
        H3D_CUDA_TRY(cudaMemcpyAsync(dres.p, res.data(), sizeof(double) * res.size(), cudaMemcpyHostToDevice, st));
        // V = H^H \ (-Pr^T (D - Dobs)) (PDEfunc.m:393); the source buffer holds the adjoint
        // right-hand sides now
        if ((r = h3d_rec_spread(g, drb.as<int32_t>(), drw.as<double>(), nrec, dres.p, nsrc, -1.0, dV.p, st))) return r;
        DevBuf dZ;
        if ((r = dZ.alloc(vb, st))) return r;
        h3d_solve_info ainfo;
        const int arc = h3d_solve(g, dw.as<double>(), nullptr, dV.p, dZ.p, nsrc, H3D_ADJOINT, opts, info ? &ainfo : nullptr,
                                  nullptr, 0, st);
        if (arc && arc != H3D_ERR_NOT_CONVERGED) return arc;
        if (arc) solve_rc = arc;
        if (info) {  // the two solves of the call
            info->iters = info->iters > ainfo.iters ? info->iters : ainfo.iters;
            info->converged = info->converged && ainfo.converged;
            info->rel_res_true = std::fmax(info->rel_res_true, ainfo.rel_res_true);
            info->rel_res_prec = std::fmax(info->rel_res_prec, ainfo.rel_res_prec);
            info->seconds += ainfo.seconds;
            info->sweep_seconds += ainfo.sweep_seconds;
            info->sweep_bytes += ainfo.sweep_bytes;
            info->sweep_samples += ainfo.sweep_samples;
            info->kernel_launches += ainfo.kernel_launches;
        }
        // g = crop(sum_s Re(conj(U_s) .* (dH^H V_s))) (discrete_helmholtz.m:288, PDEfunc.m:394)
        H3D_CUDA_TRY(cudaMemsetAsync(dg.p, 0, sizeof(double) * (size_t)nphys, st));
        if ((r = h3d_grad_accum(g, dd.as<double>(), dU.p, dZ.p, nsrc, 1.0, dg.as<double>(), st))) return r;
        H3D_CUDA_TRY(cudaMemcpyAsync(g_phys, dg.p, sizeof(double) * (size_t)nphys, cudaMemcpyDeviceToHost, st));
        return H3D_OK;
    });
    return rc ? rc : solve_rc;
}

}  // extern "C"
