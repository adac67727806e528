// Band storage: the reference's mat_free = false path (helmholtz_3d.m, opBandStorage.m,
// Hmvp_MT_mex.c, sweep_MT_mex.c).  A band matrix holds, for every row i, the coefficients
// of its ndiags couplings: coef[k + ndiags i] = A(i, i + offsets[k]) (the reference's
// ndiags x N column-major array, complex interleaved here).
//
//  * band_coefs_kernel: the 27 x N bands of the operator the matrix-free kernels apply --
//    forward H (helmholtz_3d.m:35-190: couplings to points outside the grid zeroed,
//    :158-190) or the band storage of H^H (conj(Htransp(H)), opBandStorage.m:127-129,
//    Htransp.m:21-35), whose band k holds the offset -offsets[k].  One thread per row, the
//    coefficient rule shared with every other kernel (row_coefs).
//  * band_mvp_kernel: y = A x for any ndiags <= kMaxBands (Hmvp_MT_mex.c:53-73), couplings
//    outside 0 <= i + offset < N skipped as the reference does; one thread per (row, rhs).
//  * band_lex_kernel: the Kaczmarz double sweep of sweep_MT_mex.c:55-97 (rows 0..N-1, then
//    N-1..0).  The rows run as the hyperplanes t = i + 3j + 9k of the grid, the schedule of
//    the matrix-free LEX sweep: rows of one hyperplane share no grid neighbour, and every
//    earlier row that shares one has a smaller t, so the result is the sequential one as
//    long as the bands couple grid neighbours only: the 27 offsets of the grid, with zero
//    couplings across a grid face (what helmholtz_3d.m and band_coefs_kernel produce).
//    Each band is mapped to its grid direction and a row skips the directions that leave
//    the grid.  The reference instead adds those zero couplings through its linear bounds
//    test (a face row's +1 reaches the next line's first point): the values are the same,
//    and skipping them keeps two rows of one hyperplane from writing the same point.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "h3d_internal.cuh"
#include "h3d_kernels.cuh"
#include "h3d_vec.cuh"

namespace h3d {

constexpr int kMaxBands = 64;

struct BandOffsets {
    long long v[kMaxBands];     // linear offset of band k
    unsigned char t[kMaxBands];  // band sweep: grid direction (dx+1) + 3(dy+1) + 9(dz+1) of band k
};

template <typename T, bool ADJ, bool WNC>
__global__ void __launch_bounds__(128) band_coefs_kernel(Op<T> op, cplx<T> *__restrict__ coef)
{
    const long long row = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (row >= op.N) return;
    const int i = (int)(row % op.nx), j = (int)((row / op.nx) % op.ny), k = (int)(row / op.sz);
    const uint32_t m = inside_mask(i, j, k, op.nx, op.ny, op.nz);
    cplx<T> c[27];
    row_coefs<T, ADJ, false, WNC>(op, i, j, k, ADJ ? 0x7ffffffu : m, c);
    cplx<T> *dst = coef + 27 * row;
#pragma unroll
    for (int t = 0; t < 27; ++t) {
        const cplx<T> v = (m >> t) & 1u ? c[t] : mk<T>(T(0), T(0));
        // adjoint: band 26 - t carries the offset -offsets[26 - t] = offsets[t]
        dst[ADJ ? 26 - t : t] = v;
    }
}

template <typename T>
__global__ void __launch_bounds__(256) band_mvp_kernel(const cplx<T> *__restrict__ coef, BandOffsets offs,
                                                       int nd, long long N, const cplx<T> *__restrict__ x,
                                                       cplx<T> *__restrict__ y)
{
    const long long row = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (row >= N) return;
    const long long s = blockIdx.y;
    const cplx<T> *a = coef + (long long)nd * row;
    const cplx<T> *xs = x + s * N;
    cplx<T> acc = mk<T>(T(0), T(0));
    for (int k = 0; k < nd; ++k) {
        const long long q = row + offs.v[k];
        if (q >= 0 && q < N) cmac(acc, a[k], xs[q]);
    }
    y[s * N + row] = acc;
}

// One hyperplane t = i + 3j + 9k of the band sweep; (i, j, k) from (t, j) as in the LEX
// kernel.  rn: squared row norms (NULL: the sum over all 27 bands, opBandStorage.m:139-144).
template <typename T>
__global__ void __launch_bounds__(128) band_lex_kernel(int nx, int ny, int nz, long long N,
                                                       const cplx<T> *__restrict__ coef, BandOffsets offs,
                                                       const T *__restrict__ rn, cplx<T> *x,
                                                       const cplx<T> *__restrict__ b, int nrhs, int t, T w)
{
    const int kk = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (j >= ny) return;
    const int r = t - 3 * j;  // = i + 9k
    if (r < 0) return;
    const int kmax = min(r / 9, nz - 1);
    const int kmin = r - (nx - 1) <= 0 ? 0 : (r - (nx - 1) + 8) / 9;
    const int k = kmin + kk;
    if (k > kmax) return;
    const int i = r - 9 * k;
    const long long row = i + (long long)nx * (j + (long long)ny * k);
    const uint32_t m = inside_mask(i, j, k, nx, ny, nz);
    cplx<T> c[27];
    const cplx<T> *a = coef + 27 * row;
#pragma unroll
    for (int q = 0; q < 27; ++q) c[q] = a[q];
    T nrm;
    if (rn) {
        nrm = rn[row];
    } else {
        nrm = T(0);
#pragma unroll
        for (int q = 0; q < 27; ++q) nrm += cabs2(c[q]);
    }
    for (int s = 0; s < nrhs; ++s) {
        cplx<T> *xs = x + (long long)s * N;
        cplx<T> atx = mk<T>(T(0), T(0));
#pragma unroll
        for (int q = 0; q < 27; ++q)
            if ((m >> offs.t[q]) & 1u) cmac(atx, c[q], xs[row + offs.v[q]]);
        const cplx<T> bv = b ? b[(long long)s * N + row] : mk<T>(T(0), T(0));
        const cplx<T> d = mk<T>(w * (bv.re - atx.re) / nrm, w * (bv.im - atx.im) / nrm);
#pragma unroll
        for (int q = 0; q < 27; ++q)
            if ((m >> offs.t[q]) & 1u) cmac_cb(xs[row + offs.v[q]], d, c[q]);
    }
}

// The 27 linear offsets of grid g in band order t = (dx+1) + 3(dy+1) + 9(dz+1).
static void grid_offsets(const h3d_grid *g, long long off[27])
{
    const long long nx = g->n[0], nxy = (long long)g->n[0] * g->n[1];
    int t = 0;
    for (int dz = -1; dz <= 1; ++dz)
        for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) off[t++] = dx + nx * dy + nxy * dz;
}

template <typename T>
static int band_coefs_t(const h3d_grid *g, const T *wr, const T *wi, bool adj, cplx<T> *coef, cudaStream_t st)
{
    Op<T> op;
    int rc;
    if constexpr (sizeof(T) == 8) rc = make_op_f64(g, wr, wi, &op);
    else rc = make_op_f32(g, wr, wi, &op);
    if (rc) return rc;
    const long long blocks = (op.N + 127) / 128;
    if (blocks > 0x7fffffffLL) {
        set_error("h3d_band_coefs: grid too large");
        return H3D_ERR_NSIZE;
    }
    const bool wnc = wi != nullptr;
#define H3D_BC(A, W) band_coefs_kernel<T, A, W><<<(unsigned)blocks, 128, 0, st>>>(op, coef)
    if (!adj && !wnc) H3D_BC(false, false);
    else if (!adj && wnc) H3D_BC(false, true);
    else if (adj && !wnc) H3D_BC(true, false);
    else H3D_BC(true, true);
#undef H3D_BC
    H3D_CUDA_TRY(cudaGetLastError());
    return H3D_OK;
}

}  // namespace h3d

using namespace h3d;

extern "C" int h3d_band_coefs(const h3d_grid *g, const void *wn_re, const void *wn_im, int mode, void *coef,
                              int64_t offsets_out[27], int dtype, void *stream)
{
    if (!wn_re || !coef || !offsets_out || (mode != H3D_FORWARD && mode != H3D_ADJOINT)) {
        set_error("h3d_band_coefs: bad argument");
        return H3D_ERR_BAD_ARG;
    }
    int rc = check_grid(g);
    if (rc) return rc;
    long long off[27];
    grid_offsets(g, off);
    // adjoint band k: offset -off[k] (Htransp.m:29)
    for (int k = 0; k < 27; ++k) offsets_out[k] = mode == H3D_ADJOINT ? -off[k] : off[k];
    cudaStream_t st = (cudaStream_t)stream;
    if (dtype == H3D_C128)
        return band_coefs_t<double>(g, (const double *)wn_re, (const double *)wn_im, mode == H3D_ADJOINT,
                                    (cplx<double> *)coef, st);
    if (dtype == H3D_C64)
        return band_coefs_t<float>(g, (const float *)wn_re, (const float *)wn_im, mode == H3D_ADJOINT,
                                   (cplx<float> *)coef, st);
    set_error("h3d_band_coefs: unknown dtype %d", dtype);
    return H3D_ERR_BAD_ARG;
}

extern "C" int h3d_band_mvp(const void *coef, const int64_t *offsets, int ndiags, int64_t n, const void *x,
                            void *y, int nrhs, int dtype, void *stream)
{
    if (!coef || !offsets || !x || !y || ndiags < 1 || ndiags > kMaxBands || n < 1 || nrhs < 1 ||
        nrhs > 65535) {
        set_error("h3d_band_mvp: bad argument (ndiags 1..%d, n >= 1, nrhs 1..65535)", kMaxBands);
        return H3D_ERR_BAD_ARG;
    }
    BandOffsets offs{};
    for (int k = 0; k < ndiags; ++k) offs.v[k] = offsets[k];
    const long long blocks = (n + 255) / 256;
    if (blocks > 0x7fffffffLL) {
        set_error("h3d_band_mvp: n too large");
        return H3D_ERR_NSIZE;
    }
    cudaStream_t st = (cudaStream_t)stream;
    const dim3 grd((unsigned)blocks, nrhs);
    if (dtype == H3D_C128)
        band_mvp_kernel<double><<<grd, 256, 0, st>>>((const cplx<double> *)coef, offs, ndiags, n,
                                                    (const cplx<double> *)x, (cplx<double> *)y);
    else if (dtype == H3D_C64)
        band_mvp_kernel<float><<<grd, 256, 0, st>>>((const cplx<float> *)coef, offs, ndiags, n,
                                                   (const cplx<float> *)x, (cplx<float> *)y);
    else {
        set_error("h3d_band_mvp: unknown dtype %d", dtype);
        return H3D_ERR_BAD_ARG;
    }
    H3D_CUDA_TRY(cudaGetLastError());
    return H3D_OK;
}

extern "C" int h3d_band_sweep(const h3d_grid *g, const void *coef, const int64_t *offsets, const void *row_norms,
                              double w, void *x, const void *b, int nrhs, int dtype, void *stream)
{
    if (!coef || !offsets || !x || nrhs < 1 || !std::isfinite(w)) {
        set_error("h3d_band_sweep: bad argument");
        return H3D_ERR_BAD_ARG;
    }
    int rc = check_grid(g);
    if (rc) return rc;
    if (g->n[0] < 3 || g->n[1] < 3 || g->n[2] < 3) {
        // below 3 points an axis' offsets coincide with another axis' and a band's
        // direction is ambiguous
        set_error("h3d_band_sweep: every axis needs at least 3 points");
        return H3D_ERR_NSIZE;
    }
    // the bands must be the 27 couplings of grid g, in any order: map each to its direction
    long long off[27];
    grid_offsets(g, off);
    BandOffsets offs{};
    bool used[27] = {false};
    for (int k = 0; k < 27; ++k) {
        int dir = -1;
        for (int t = 0; t < 27; ++t)
            if (!used[t] && off[t] == offsets[k]) dir = t;
        if (dir < 0) {
            set_error("h3d_band_sweep: the 27 offsets are not the 27-point neighbourhood of the %dx%dx%d grid",
                      g->n[0], g->n[1], g->n[2]);
            return H3D_ERR_BAD_ARG;
        }
        used[dir] = true;
        offs.v[k] = offsets[k];
        offs.t[k] = (unsigned char)dir;
    }
    const int nx = g->n[0], ny = g->n[1], nz = g->n[2];
    const long long N = (long long)nx * ny * nz;
    const int tmax = (nx - 1) + 3 * (ny - 1) + 9 * (nz - 1);
    const int kw = (nx + 8) / 9 + 1;  // k values per (t, j)
    const dim3 blk(32, 4);
    const dim3 grd((kw + 31) / 32, (ny + 3) / 4);
    if (grd.y > 65535) {
        set_error("h3d_band_sweep: ny too large");
        return H3D_ERR_NSIZE;
    }
    cudaStream_t st = (cudaStream_t)stream;
    for (int pass = 0; pass < 2; ++pass) {
        for (int tt = 0; tt <= tmax; ++tt) {
            const int t = pass == 0 ? tt : tmax - tt;
            if (dtype == H3D_C128)
                band_lex_kernel<double><<<grd, blk, 0, st>>>(nx, ny, nz, N, (const cplx<double> *)coef, offs,
                                                             (const double *)row_norms, (cplx<double> *)x,
                                                             (const cplx<double> *)b, nrhs, t, w);
            else if (dtype == H3D_C64)
                band_lex_kernel<float><<<grd, blk, 0, st>>>(nx, ny, nz, N, (const cplx<float> *)coef, offs,
                                                            (const float *)row_norms, (cplx<float> *)x,
                                                            (const cplx<float> *)b, nrhs, t, (float)w);
            else {
                set_error("h3d_band_sweep: unknown dtype %d", dtype);
                return H3D_ERR_BAD_ARG;
            }
        }
    }
    H3D_CUDA_TRY(cudaGetLastError());
    return H3D_OK;
}

// ---------------------------------------------------------------------------------------
// Host entries of the drop-in band gateways (Hmvp_MT_mex.c:76-141, sweep_MT_mex.c:100-188):
// MATLAB's split-complex column-major arrays in host memory, copied to the device,
// interleaved, processed, copied back.

namespace h3d {

static int offsets_from_mex(const double *offsets, size_t ndiags, int64_t *off)
{
    for (size_t k = 0; k < ndiags; ++k) {
        const double v = offsets[k];
        if (!std::isfinite(v) || v != std::floor(v) || std::fabs(v) > 9.0e15) {
            set_error("offset %zu is not an integer", k);
            return H3D_ERR_BAD_ARG;
        }
        off[k] = (int64_t)v;
    }
    return H3D_OK;
}

// Split (re, im) host planes of n values -> interleaved device buffer (im may be NULL).
static int upload_split(const double *re, const double *im, long long n, DevBuf &stage, DevBuf &out, cudaStream_t st)
{
    int rc;
    const size_t pb = (size_t)n * sizeof(double);
    if ((rc = stage.alloc(2 * pb, st)) || (rc = out.alloc(2 * pb, st))) return rc;
    double *pre = stage.as<double>(), *pim = pre + n;
    H3D_CUDA_TRY(cudaMemcpyAsync(pre, re, pb, cudaMemcpyHostToDevice, st));
    if (im) H3D_CUDA_TRY(cudaMemcpyAsync(pim, im, pb, cudaMemcpyHostToDevice, st));
    return interleave<double>(pre, im ? pim : nullptr, out.as<cplx<double>>(), n, st);
}

static int download_split(const DevBuf &in, long long n, DevBuf &stage, double *re, double *im, cudaStream_t st)
{
    int rc;
    const size_t pb = (size_t)n * sizeof(double);
    if ((rc = stage.alloc(2 * pb, st))) return rc;
    double *pre = stage.as<double>(), *pim = pre + n;
    if ((rc = deinterleave<double>(in.as<cplx<double>>(), pre, pim, n, st))) return rc;
    H3D_CUDA_TRY(cudaMemcpyAsync(re, pre, pb, cudaMemcpyDeviceToHost, st));
    H3D_CUDA_TRY(cudaMemcpyAsync(im, pim, pb, cudaMemcpyDeviceToHost, st));
    return H3D_OK;
}

// The grid of a 27-point band matrix from its offsets: the positive offsets in ascending
// order are 1, nx-1, nx, nx+1, nxy-nx-1, ..., nxy, ... (every axis >= 3 points), so nx is the
// third and nx*ny the ninth.
static int grid_from_offsets(const int64_t *off, long long n, h3d_grid *g)
{
    long long pos[27];
    int np = 0;
    for (int k = 0; k < 27; ++k)
        if (off[k] > 0) pos[np++] = off[k];
    if (np != 13) {
        set_error("the 27 offsets are not a 27-point grid neighbourhood");
        return H3D_ERR_BAD_ARG;
    }
    std::sort(pos, pos + np);
    const long long nx = pos[2], nxy = pos[8];
    if (nx < 3 || nxy % nx != 0 || nxy / nx < 3 || n % nxy != 0 || n / nxy < 3 || n / nxy > 0x7fffffffLL ||
        nxy / nx > 0x7fffffffLL || nx > 0x7fffffffLL) {
        set_error("the 27 offsets are not the neighbourhood of a grid of n = %lld points", n);
        return H3D_ERR_BAD_ARG;
    }
    std::memset(g, 0, sizeof *g);
    g->n[0] = (int32_t)nx;
    g->n[1] = (int32_t)(nxy / nx);
    g->n[2] = (int32_t)(n / nxy);
    g->h[0] = g->h[1] = g->h[2] = 1.0;  // the band sweep reads only the sizes
    // all 27 offsets must be that grid's (checked here, before any device work)
    long long want[27], have[27];
    grid_offsets(g, want);
    for (int k = 0; k < 27; ++k) have[k] = off[k];
    std::sort(want, want + 27);
    std::sort(have, have + 27);
    for (int k = 0; k < 27; ++k)
        if (want[k] != have[k]) {
            set_error("the 27 offsets are not the neighbourhood of a grid of n = %lld points", n);
            return H3D_ERR_BAD_ARG;
        }
    return H3D_OK;
}

}  // namespace h3d

extern "C" int h3d_mex_band_mvp(const double *coef_re, const double *coef_im, size_t ndiags, size_t n,
                                const double *offsets, const double *x_re, const double *x_im, size_t x_rows,
                                size_t nrhs, double *y_re, double *y_im)
{
    if (x_rows != n) {
        set_error("The row size of the vector x and the column size of the matrix A must match");
        return H3D_ERR_XSIZE;
    }
    if (!coef_re || !offsets || !x_re || !y_re || !y_im || ndiags < 1 || ndiags > (size_t)kMaxBands || n < 1 ||
        nrhs < 1 || nrhs > 65535) {
        set_error("h3d_mex_band_mvp: bad argument");
        return H3D_ERR_BAD_ARG;
    }
    int64_t off[kMaxBands];
    int rc = offsets_from_mex(offsets, ndiags, off);
    if (rc) return rc;
    cudaStream_t st = nullptr;
    H3D_CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    rc = [&]() -> int {
        DevBuf sc, dc, sx, dx, dy, sy;
        const long long nc = (long long)ndiags * (long long)n, nv = (long long)n * (long long)nrhs;
        int r;
        if ((r = upload_split(coef_re, coef_im, nc, sc, dc, st))) return r;
        sc.release();
        if ((r = upload_split(x_re, x_im, nv, sx, dx, st))) return r;
        if ((r = dy.alloc((size_t)nv * sizeof(cplx<double>), st))) return r;
        if ((r = h3d_band_mvp(dc.p, off, (int)ndiags, (int64_t)n, dx.p, dy.p, (int)nrhs, H3D_C128, st))) return r;
        return download_split(dy, nv, sy, y_re, y_im, st);
    }();
    cudaError_t e = cudaStreamSynchronize(st);
    cudaStreamDestroy(st);
    if (rc) return rc;
    if (e != cudaSuccess) return cuda_fail(e, "h3d_mex_band_mvp");
    return H3D_OK;
}

extern "C" int h3d_mex_band_sweep(const double *coef_re, const double *coef_im, size_t ndiags, size_t n,
                                  const double *offsets, const double *x_re, const double *x_im, size_t x_rows,
                                  size_t nrhs, const double *b_re, const double *b_im, size_t b_rows, double w,
                                  const double *row_norms, size_t rn_rows, double *y_re, double *y_im)
{
    if (x_rows != n) {
        set_error("The row size of the vector x and the column size of the matrix A must match");
        return H3D_ERR_XSIZE;
    }
    if (b_rows != n) {
        set_error("b must have N rows");
        return H3D_ERR_BSIZE;
    }
    if (rn_rows != n) {
        set_error("The size of the row norms vector and the rows size of the matrix A must match");
        return H3D_ERR_XSIZE;
    }
    if (!coef_re || !offsets || !x_re || !b_re || !row_norms || !y_re || !y_im || ndiags != 27 || n < 27 ||
        nrhs < 1 || !std::isfinite(w)) {
        set_error("h3d_mex_band_sweep: bad argument (the GPU band sweep takes the 27 bands of a grid stencil)");
        return H3D_ERR_BAD_ARG;
    }
    int64_t off[27];
    int rc = offsets_from_mex(offsets, 27, off);
    if (rc) return rc;
    h3d_grid g;
    if ((rc = grid_from_offsets(off, (long long)n, &g))) return rc;
    cudaStream_t st = nullptr;
    H3D_CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    rc = [&]() -> int {
        DevBuf sc, dc, sx, dx, sb, db, rn, sy;
        const long long nc = 27LL * (long long)n, nv = (long long)n * (long long)nrhs;
        int r;
        if ((r = upload_split(coef_re, coef_im, nc, sc, dc, st))) return r;
        sc.release();
        if ((r = upload_split(x_re, x_im, nv, sx, dx, st))) return r;
        if ((r = upload_split(b_re, b_im, nv, sb, db, st))) return r;
        if ((r = rn.alloc((size_t)n * sizeof(double), st))) return r;
        H3D_CUDA_TRY(cudaMemcpyAsync(rn.p, row_norms, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, st));
        if ((r = h3d_band_sweep(&g, dc.p, off, rn.p, w, dx.p, db.p, (int)nrhs, H3D_C128, st))) return r;
        return download_split(dx, nv, sy, y_re, y_im, st);
    }();
    cudaError_t e = cudaStreamSynchronize(st);
    cudaStreamDestroy(st);
    if (rc) return rc;
    if (e != cudaSuccess) return cuda_fail(e, "h3d_mex_band_sweep");
    return H3D_OK;
}
