// Matrix-free 27-point Helmholtz operator kernels: matvec (forward, adjoint, derivative,
// complex-wavenumber variants) and Kaczmarz double sweeps in three row orderings.
//
// Reference semantics: do_Hmvp (tools/algorithms/3DFreqModeling/Helm3d_27pt.h:827-875) and
// do_sweep (Helm3dkaczswp_mex.c:60-120).  Layout: interleaved complex, x fastest,
// right-hand side s at offset s*N.
#include <algorithm>

#include "h3d_internal.cuh"
#include "h3d_kernels.cuh"
#include "h3d_rowops.cuh"

namespace h3d {

// ---------------------------------------------------------------------------------------
// Matvec: one thread per output row, coefficients built once and applied to every
// right-hand side.  x outside the grid is zero (load_nbrhoodc, Helm3d_27pt.h:483-520).
template <typename T, bool ADJ, bool DERIV, bool WNC>
__global__ void __launch_bounds__(256) mvp_kernel(Op<T> op, const cplx<T> *__restrict__ x,
                                                  cplx<T> *__restrict__ y, int nrhs)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= op.nx || j >= op.ny) return;
    const uint32_t m = inside_mask(i, j, k, op.nx, op.ny, op.nz);
    cplx<T> c[27];
    row_coefs<T, ADJ, DERIV, WNC>(op, i, j, k, m, c);
    const long long ctr = i + op.sy * j + op.sz * k;
    for (int s = 0; s < nrhs; ++s) {
        const cplx<T> *xs = x + (long long)s * op.N + ctr;
        cplx<T> acc = mk<T>(T(0), T(0));
#define H3D_ACC(t, dx, dy, dz) \
    if (m & (1u << t)) cmac(acc, c[t], ldg_c(xs + (dx + op.sy * dy + op.sz * dz)));
        H3D_FOR_27(H3D_ACC)
#undef H3D_ACC
        y[(long long)s * op.N + ctr] = acc;
    }
}

// COLOUR27: every row of colour (a, bq, cq) = (i%3, j%3, k%3) in one launch.  Their
// 3x3x3 footprints are disjoint, so the rows run concurrently without atomics.
template <typename T, bool ADJ, bool WNC>
__global__ void __launch_bounds__(256) sweep_colour_kernel(Op<T> op, cplx<T> *x,
                                                           const cplx<T> *b, int nrhs, int a,
                                                           int bq, int cq, T w,
                                                           const int *active)
{
    const int u = blockIdx.x * blockDim.x + threadIdx.x;
    const int v = blockIdx.y * blockDim.y + threadIdx.y;
    const int i = a + 3 * u, j = bq + 3 * v, k = cq + 3 * (int)blockIdx.z;
    if (i >= op.nx || j >= op.ny || k >= op.nz) return;
    project_row<T, ADJ, WNC>(op, x, b, nrhs, i, j, k, w, active);
}

// LEX: the reference order executed as hyperplanes t = i + 3j + 9k.  Rows on one plane
// never share a neighbour (|di + 3dj| <= 8 < 9 forces dk = 0, then di = -3dj forces
// dj = di = 0), and any two rows whose footprints overlap (all |d*| <= 2) that come
// earlier in k,j,i order have a smaller t, so the result equals the sequential sweep.
template <typename T, bool ADJ, bool WNC>
__global__ void __launch_bounds__(128) sweep_lex_kernel(Op<T> op, cplx<T> *x, const cplx<T> *b,
                                                        int nrhs, int t, T w, const int *active)
{
    const int kk = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (j >= op.ny) return;
    const int r = t - 3 * j;  // = i + 9k
    if (r < 0) return;
    const int kmax = min(r / 9, op.nz - 1);
    const int kmin = r - (op.nx - 1) <= 0 ? 0 : (r - (op.nx - 1) + 8) / 9;
    const int k = kmin + kk;
    if (k > kmax) return;
    const int i = r - 9 * k;
    project_row<T, ADJ, WNC>(op, x, b, nrhs, i, j, k, w, active);
}

// ---------------------------------------------------------------------------------------
// Dispatch.

template <typename T>
int launch_mvp(const Op<T> &op, const cplx<T> *x, cplx<T> *y, int nrhs, bool adj, bool deriv,
               cudaStream_t st)
{
    const dim3 blk(32, 8);
    const dim3 grd((op.nx + 31) / 32, (op.ny + 7) / 8, op.nz);
    if (op.nz > 65535) {
        set_error("nz > 65535 is not supported");
        return H3D_ERR_NSIZE;
    }
    const bool wnc = op.wni != nullptr;
#define H3D_LAUNCH_MVP(A, D, W) mvp_kernel<T, A, D, W><<<grd, blk, 0, st>>>(op, x, y, nrhs)
    if (!adj && !deriv && !wnc) H3D_LAUNCH_MVP(false, false, false);
    else if (!adj && !deriv && wnc) H3D_LAUNCH_MVP(false, false, true);
    else if (!adj && deriv && !wnc) H3D_LAUNCH_MVP(false, true, false);
    else if (!adj && deriv && wnc) H3D_LAUNCH_MVP(false, true, true);
    else if (adj && !deriv && !wnc) H3D_LAUNCH_MVP(true, false, false);
    else if (adj && !deriv && wnc) H3D_LAUNCH_MVP(true, false, true);
    else if (adj && deriv && !wnc) H3D_LAUNCH_MVP(true, true, false);
    else H3D_LAUNCH_MVP(true, true, true);
#undef H3D_LAUNCH_MVP
    H3D_CUDA_TRY(cudaGetLastError());
    return H3D_OK;
}

template <typename T, bool ADJ, bool WNC>
static int sweep_colour_pass(const Op<T> &op, cplx<T> *x, const cplx<T> *b, int nrhs, T w,
                             const int *active, bool backward, cudaStream_t st)
{
    for (int qq = 0; qq < 27; ++qq) {
        const int q = backward ? 26 - qq : qq;
        const int a = q % 3, bq = (q / 3) % 3, cq = q / 9;
        const int nu = (op.nx - a + 2) / 3, nv = (op.ny - bq + 2) / 3, nw = (op.nz - cq + 2) / 3;
        if (nu <= 0 || nv <= 0 || nw <= 0) continue;
        const dim3 blk(32, 8);
        const dim3 grd((nu + 31) / 32, (nv + 7) / 8, nw);
        sweep_colour_kernel<T, ADJ, WNC><<<grd, blk, 0, st>>>(op, x, b, nrhs, a, bq, cq, w, active);
    }
    return H3D_OK;
}

template <typename T, bool ADJ, bool WNC>
static int sweep_lex_pass(const Op<T> &op, cplx<T> *x, const cplx<T> *b, int nrhs, T w,
                          const int *active, bool backward, cudaStream_t st)
{
    const int tmax = (op.nx - 1) + 3 * (op.ny - 1) + 9 * (op.nz - 1);
    const int kw = (op.nx + 8) / 9 + 1;  // k values per (t, j)
    const dim3 blk(32, 4);
    const dim3 grd((kw + 31) / 32, (op.ny + 3) / 4);
    for (int tt = 0; tt <= tmax; ++tt) {
        const int t = backward ? tmax - tt : tt;
        sweep_lex_kernel<T, ADJ, WNC><<<grd, blk, 0, st>>>(op, x, b, nrhs, t, w, active);
    }
    return H3D_OK;
}

template <typename T, bool ADJ, bool WNC>
static int sweep_dispatch(const Op<T> &op, cplx<T> *x, const cplx<T> *b, int nrhs, T w,
                          int order, const int32_t *block, const int *active, cudaStream_t st)
{
    int rc = H3D_OK;
    if (order == H3D_ORDER_LEX) {
        rc = sweep_lex_pass<T, ADJ, WNC>(op, x, b, nrhs, w, active, false, st);
        if (!rc) rc = sweep_lex_pass<T, ADJ, WNC>(op, x, b, nrhs, w, active, true, st);
    } else if (order == H3D_ORDER_COLOUR27) {
        rc = sweep_colour_pass<T, ADJ, WNC>(op, x, b, nrhs, w, active, false, st);
        if (!rc) rc = sweep_colour_pass<T, ADJ, WNC>(op, x, b, nrhs, w, active, true, st);
    } else if (order == H3D_ORDER_BLOCK) {
        rc = sweep_block(op, x, b, nrhs, w, block, active, ADJ, st);
    } else {
        set_error("unknown sweep order %d", order);
        return H3D_ERR_BAD_ARG;
    }
    if (rc) return rc;
    H3D_CUDA_TRY(cudaGetLastError());
    return H3D_OK;
}

template <typename T>
int launch_sweep(const Op<T> &op, cplx<T> *x, const cplx<T> *b, int nrhs, T w, bool adj,
                 int order, const int32_t *block, const int *active, cudaStream_t st)
{
    const bool wnc = op.wni != nullptr;
    if (!adj && !wnc) return sweep_dispatch<T, false, false>(op, x, b, nrhs, w, order, block, active, st);
    if (!adj && wnc) return sweep_dispatch<T, false, true>(op, x, b, nrhs, w, order, block, active, st);
    if (adj && !wnc) return sweep_dispatch<T, true, false>(op, x, b, nrhs, w, order, block, active, st);
    return sweep_dispatch<T, true, true>(op, x, b, nrhs, w, order, block, active, st);
}

template int launch_mvp<double>(const Op<double> &, const cplx<double> *, cplx<double> *, int, bool, bool, cudaStream_t);
template int launch_mvp<float>(const Op<float> &, const cplx<float> *, cplx<float> *, int, bool, bool, cudaStream_t);
template int launch_sweep<double>(const Op<double> &, cplx<double> *, const cplx<double> *, int, double, bool, int, const int32_t *, const int *, cudaStream_t);
template int launch_sweep<float>(const Op<float> &, cplx<float> *, const cplx<float> *, int, float, bool, int, const int32_t *, const int *, cudaStream_t);

}  // namespace h3d
