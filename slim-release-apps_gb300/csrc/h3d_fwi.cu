// FWI building blocks around the solves of PDEfunc (tools/algorithms/CommonFreqModeling/
// PDEfunc.m:324-394):
//   - separable sinc x Kaiser interpolation weights (opSincInterp.m:26-52 with r = 4,
//     beta = 6.31 from opInterp.m:108 / opSincInterp.m:46), used for source injection Ps
//     and receiver sampling Pr (DataGrid.m:22-44);
//   - the gradient accumulation g += to_phys * sum_src Re(conj(u) .* (dH' * v))
//     (discrete_helmholtz.m:288, PDEfunc.m:386,394), fused over sources and cropped to
//     the physical grid (cut_pml = true, discrete_helmholtz.m:231-232).
#include <cmath>
#include <cstring>

#include "h3d_internal.cuh"
#include "h3d_reduce.cuh"

namespace h3d {

// Modified Bessel function I0 by its power series sum_k ((x/2)^(2k)) / (k!)^2
// (Abramowitz & Stegun 9.6.10); for the |x| <= 8 used here it converges in < 40 terms.
static double bessel_i0(double x)
{
    const double q = 0.25 * x * x;
    double term = 1.0, sum = 1.0;
    for (int k = 1; k < 200; ++k) {
        term *= q / ((double)k * (double)k);
        sum += term;
        if (term < 1e-18 * sum) break;
    }
    return sum;
}

// sinc(x) = sin(pi x)/(pi x), 1 at 0 (tools/functions/misc/sinc.m); Kaiser window
// I0(b sqrt(1-(x/r)^2)) / I0(b) for |x| <= r, else 0 (kaiser_window.m:16-19).
static double sinc_kaiser(double x, double r, double beta)
{
    if (std::fabs(x) > r) return 0.0;
    const double s = x == 0.0 ? 1.0 : std::sin(M_PI * x) / (M_PI * x);
    const double t = x / r;
    return s * bessel_i0(beta * std::sqrt(1.0 - t * t)) / bessel_i0(beta);
}

constexpr double kSincR = 4.0;       // opInterp.m:108 (sinc_window = 4)
constexpr double kSincBeta = 6.31;   // opSincInterp.m:46, r_b(4)
constexpr int kTaps = 9;

// ---------------------------------------------------------------------------------------
__global__ void k_src_inject(int nx, int ny, int nz, long long N, const int32_t *__restrict__ base,
                             const double *__restrict__ w, const double *__restrict__ scale,
                             cplx<double> *__restrict__ b)
{
    const int s = blockIdx.x;
    const int tid = threadIdx.x;  // 0 .. 728
    if (tid >= kTaps * kTaps * kTaps) return;
    const int ox = tid % kTaps, oy = (tid / kTaps) % kTaps, oz = tid / (kTaps * kTaps);
    const int i = base[3 * s] + ox, j = base[3 * s + 1] + oy, k = base[3 * s + 2] + oz;
    if (i < 0 || i >= nx || j < 0 || j >= ny || k < 0 || k >= nz) return;
    const double wt = w[(3 * s + 0) * kTaps + ox] * w[(3 * s + 1) * kTaps + oy] * w[(3 * s + 2) * kTaps + oz];
    if (wt == 0.0) return;
    cplx<double> *p = b + (long long)s * N + i + (long long)nx * j + (long long)nx * ny * k;
    cplx<double> v = *p;
    v.re += wt * scale[2 * s];
    v.im += wt * scale[2 * s + 1];
    *p = v;
}

// One warp per (receiver, rhs): d = sum over the 9^3 taps of w * u.
__global__ void k_rec_sample(int nx, int ny, int nz, long long N, const int32_t *__restrict__ base,
                             const double *__restrict__ w, int nrec, const cplx<double> *__restrict__ u,
                             int nrhs, cplx<double> *__restrict__ d)
{
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= nrec * nrhs) return;
    const int r = warp % nrec, s = warp / nrec;
    double are = 0.0, aim = 0.0;
    for (int t = lane; t < kTaps * kTaps * kTaps; t += 32) {
        const int ox = t % kTaps, oy = (t / kTaps) % kTaps, oz = t / (kTaps * kTaps);
        const int i = base[3 * r] + ox, j = base[3 * r + 1] + oy, k = base[3 * r + 2] + oz;
        if (i < 0 || i >= nx || j < 0 || j >= ny || k < 0 || k >= nz) continue;
        const double wt = w[(3 * r + 0) * kTaps + ox] * w[(3 * r + 1) * kTaps + oy] * w[(3 * r + 2) * kTaps + oz];
        const cplx<double> v = u[(long long)s * N + i + (long long)nx * j + (long long)nx * ny * k];
        are += wt * v.re;
        aim += wt * v.im;
    }
    for (int o = 16; o > 0; o >>= 1) {
        are += __shfl_down_sync(0xffffffffu, are, o);
        aim += __shfl_down_sync(0xffffffffu, aim, o);
    }
    if (lane == 0) d[(long long)s * nrec + r] = mk(are, aim);
}

// b_s = scale * Pr^T d_s: one CTA per RHS adds the receivers one after another (their
// footprints overlap), so the sum order is fixed and no atomics are needed.
__global__ void k_rec_spread(int nx, int ny, int nz, long long N, const int32_t *__restrict__ base,
                             const double *__restrict__ w, int nrec, const cplx<double> *__restrict__ d,
                             double scale, cplx<double> *__restrict__ b)
{
    const int s = blockIdx.x;
    for (int r = 0; r < nrec; ++r) {
        const cplx<double> dv = d[(long long)s * nrec + r];
        for (int t = threadIdx.x; t < kTaps * kTaps * kTaps; t += blockDim.x) {
            const int ox = t % kTaps, oy = (t / kTaps) % kTaps, oz = t / (kTaps * kTaps);
            const int i = base[3 * r] + ox, j = base[3 * r + 1] + oy, k = base[3 * r + 2] + oz;
            if (i < 0 || i >= nx || j < 0 || j >= ny || k < 0 || k >= nz) continue;
            const double wt = scale * w[(3 * r + 0) * kTaps + ox] * w[(3 * r + 1) * kTaps + oy] *
                              w[(3 * r + 2) * kTaps + oz];
            if (wt == 0.0) continue;
            cplx<double> *p = b + (long long)s * N + i + (long long)nx * j + (long long)nx * ny * k;
            cplx<double> v = *p;
            v.re += wt * dv.re;
            v.im += wt * dv.im;
            *p = v;
        }
        __syncthreads();
    }
}

// g_phys += scale * sum_s Re( conj(u_s) * dwn * (M z_s) ), M = the 27-point mass stencil
// of the adjoint derivative operator (Helm3d_27pt.h:718-752 with DERIV: every coefficient
// -WM_t * dwn[centre], centre wn_coef * dwn[centre], x outside the grid = 0).
__global__ void __launch_bounds__(256) k_grad(int nx, int ny, int nz, long long N, int lo0, int lo1, int lo2,
                                              int px, int py, int pz, const double *__restrict__ dwn,
                                              const cplx<double> *__restrict__ u,
                                              const cplx<double> *__restrict__ z, int nrhs,
                                              double scale, double wn_c, double *__restrict__ g)
{
    const int ip = blockIdx.x * blockDim.x + threadIdx.x;
    const int jp = blockIdx.y * blockDim.y + threadIdx.y;
    const int kp = blockIdx.z;
    if (ip >= px || jp >= py || kp >= pz) return;
    const int i = ip + lo0, j = jp + lo1, k = kp + lo2;
    const uint32_t m = inside_mask(i, j, k, nx, ny, nz);
    const long long sy = nx, sz = (long long)nx * ny;
    const long long ctr = i + sy * j + sz * k;
    const double dw = dwn[ctr];
    double acc_g = 0.0;
    for (int s = 0; s < nrhs; ++s) {
        const cplx<double> *zs = z + (long long)s * N + ctr;
        double f1r = 0, f1i = 0, f2r = 0, f2i = 0, f3r = 0, f3i = 0;
#define H3D_MASS(t, dx, dy, dz)                                                                \
    if (t != 13 && (m & (1u << t))) {                                                          \
        const cplx<double> v = zs[dx + sy * dy + sz * dz];                                     \
        constexpr int nzc = (dx != 0) + (dy != 0) + (dz != 0);                                 \
        if (nzc == 1) { f1r += v.re; f1i += v.im; }                                            \
        else if (nzc == 2) { f2r += v.re; f2i += v.im; }                                       \
        else { f3r += v.re; f3i += v.im; }                                                     \
    }
        H3D_FOR_27(H3D_MASS)
#undef H3D_MASS
        const cplx<double> zc = zs[0];
        const double mr = wn_c * zc.re - kWM2 * f1r - kWM3 * f2r - kWM4 * f3r;
        const double mi = wn_c * zc.im - kWM2 * f1i - kWM3 * f2i - kWM4 * f3i;
        const cplx<double> uv = u[(long long)s * N + ctr];
        // Re(conj(u) * dwn * (mr + i mi))
        acc_g += dw * (uv.re * mr + uv.im * mi);
    }
    g[ip + (long long)px * jp + (long long)px * py * kp] += scale * acc_g;
}

}  // namespace h3d

using namespace h3d;

extern "C" {

int h3d_sinc_weights(const h3d_grid *g, const double *pts, int npts, int32_t *base, double *w)
{
    int rc = check_grid(g);
    if (rc) return rc;
    if (!pts || !base || !w || npts < 0) {
        set_error("h3d_sinc_weights: bad argument");
        return H3D_ERR_BAD_ARG;
    }
    for (int p = 0; p < npts; ++p) {
        for (int a = 0; a < 3; ++a) {
            const double x = pts[3 * p + a];
            if (!std::isfinite(x)) {
                set_error("non-finite point coordinate");
                return H3D_ERR_BAD_ARG;
            }
            const int b0 = (int)std::floor(x) - 4;
            base[3 * p + a] = b0;
            for (int o = 0; o < kTaps; ++o) {
                const int idx = b0 + o;
                double v = 0.0;
                if (idx >= 0 && idx < g->n[a]) v = sinc_kaiser((double)idx - x, kSincR, kSincBeta);
                w[(3 * p + a) * kTaps + o] = v;
            }
        }
    }
    return H3D_OK;
}

int h3d_src_inject(const h3d_grid *g, const int32_t *base, const double *w, const double *scale,
                   void *b, int nsrc, void *stream)
{
    int rc = check_grid(g);
    if (rc) return rc;
    if (!base || !w || !scale || !b || nsrc < 0) {
        set_error("h3d_src_inject: bad argument");
        return H3D_ERR_BAD_ARG;
    }
    if (nsrc == 0) return H3D_OK;
    const long long N = (long long)g->n[0] * g->n[1] * g->n[2];
    k_src_inject<<<nsrc, 736, 0, (cudaStream_t)stream>>>(g->n[0], g->n[1], g->n[2], N, base, w, scale,
                                                          (cplx<double> *)b);
    H3D_CUDA_TRY(cudaGetLastError());
    return H3D_OK;
}

int h3d_rec_sample(const h3d_grid *g, const int32_t *base, const double *w, int nrec,
                   const void *u, int nrhs, void *d, void *stream)
{
    int rc = check_grid(g);
    if (rc) return rc;
    if (!base || !w || !u || !d || nrec < 0 || nrhs < 1) {
        set_error("h3d_rec_sample: bad argument");
        return H3D_ERR_BAD_ARG;
    }
    if (nrec == 0) return H3D_OK;
    const long long N = (long long)g->n[0] * g->n[1] * g->n[2];
    const long long warps = (long long)nrec * nrhs;
    const int blocks = (int)((warps * 32 + 255) / 256);
    k_rec_sample<<<blocks, 256, 0, (cudaStream_t)stream>>>(g->n[0], g->n[1], g->n[2], N, base, w, nrec,
                                                            (const cplx<double> *)u, nrhs, (cplx<double> *)d);
    H3D_CUDA_TRY(cudaGetLastError());
    return H3D_OK;
}

int h3d_rec_spread(const h3d_grid *g, const int32_t *base, const double *w, int nrec,
                   const void *d, int nrhs, double scale, void *b, void *stream)
{
    int rc = check_grid(g);
    if (rc) return rc;
    if (!base || !w || !d || !b || nrec < 0 || nrhs < 1) {
        set_error("h3d_rec_spread: bad argument");
        return H3D_ERR_BAD_ARG;
    }
    const long long N = (long long)g->n[0] * g->n[1] * g->n[2];
    cudaStream_t st = (cudaStream_t)stream;
    H3D_CUDA_TRY(cudaMemsetAsync(b, 0, sizeof(cplx<double>) * (size_t)N * nrhs, st));
    if (nrec == 0) return H3D_OK;
    k_rec_spread<<<nrhs, 256, 0, st>>>(g->n[0], g->n[1], g->n[2], N, base, w, nrec,
                                       (const cplx<double> *)d, scale, (cplx<double> *)b);
    H3D_CUDA_TRY(cudaGetLastError());
    return H3D_OK;
}

int h3d_grad_accum(const h3d_grid *g, const double *dwn, const void *u, const void *z,
                   int nrhs, double scale, double *g_phys, void *stream)
{
    int rc = check_grid(g);
    if (rc) return rc;
    if (!dwn || !u || !z || !g_phys || nrhs < 1) {
        set_error("h3d_grad_accum: bad argument");
        return H3D_ERR_BAD_ARG;
    }
    const int px = g->n[0] - g->npml[0] - g->npml[1];
    const int py = g->n[1] - g->npml[2] - g->npml[3];
    const int pz = g->n[2] - g->npml[4] - g->npml[5];
    if (px < 1 || py < 1 || pz < 1) {
        set_error("the PML leaves no physical grid");
        return H3D_ERR_NSIZE;
    }
    const double hx2 = g->h[0] * g->h[0], hy2 = g->h[1] * g->h[1], hz2 = g->h[2] * g->h[2];
    const double hxyz = hx2 + hy2 + hz2;
    const double w3a = kW3 * 3 / (4 * hxyz);
    const double wn_c = -(kW1 + 3 * kW2 + 16 * w3a * hxyz / 3 + kWM1 - 1);
    const long long N = (long long)g->n[0] * g->n[1] * g->n[2];
    const dim3 blk(32, 8), grd((px + 31) / 32, (py + 7) / 8, pz);
    k_grad<<<grd, blk, 0, (cudaStream_t)stream>>>(g->n[0], g->n[1], g->n[2], N, g->npml[0], g->npml[2],
                                                   g->npml[4], px, py, pz, dwn, (const cplx<double> *)u,
                                                   (const cplx<double> *)z, nrhs, scale, wn_c, g_phys);
    H3D_CUDA_TRY(cudaGetLastError());
    return H3D_OK;
}

}  // extern "C"
