// Kaczmarz double sweeps of the 27-point Helmholtz operator: row-order dispatch and the
// exact-LEX hyperplane kernel (the COLOUR27 and BLOCK kernels live in their own files).
//
// Reference semantics: do_Hmvp (tools/algorithms/3DFreqModeling/Helm3d_27pt.h:827-875) and
// do_sweep (Helm3dkaczswp_mex.c:60-120).  Layout: interleaved complex, x fastest,
// right-hand side s at offset s*N.
#include <algorithm>

#include "h3d_internal.cuh"
#include "h3d_kernels.cuh"
#include "h3d_rowops.cuh"

namespace h3d {

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
                          int order, const int32_t *block, const int *active, cudaStream_t st,
                          const T *rinv, int shape, const cplx<T> *coef)
{
    int rc = H3D_OK;
    if (order == H3D_ORDER_LEX) {
        rc = sweep_lex_pass<T, ADJ, WNC>(op, x, b, nrhs, w, active, false, st);
        if (!rc) rc = sweep_lex_pass<T, ADJ, WNC>(op, x, b, nrhs, w, active, true, st);
    } else if (order == H3D_ORDER_COLOUR27 && coef && rinv) {
        rc = sweep_colour_direct<T>(op, x, b, nrhs, w, active, rinv, coef, ADJ, st);
    } else if (order == H3D_ORDER_COLOUR27) {
        rc = sweep_colour_tiled<T>(op, x, b, nrhs, w, active, rinv, shape, ADJ, false, st);
        if (!rc) rc = sweep_colour_tiled<T>(op, x, b, nrhs, w, active, rinv, shape, ADJ, true, st);
    } else if (order == H3D_ORDER_BLOCK) {
        rc = sweep_block(op, x, b, nrhs, w, block, active, ADJ, st, rinv, shape);
    } else if (order == H3D_ORDER_BLOCK8) {
        rc = sweep_block8(op, x, b, nrhs, w, block, active, ADJ, st, rinv, shape, coef);
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
                 int order, const int32_t *block, const int *active, cudaStream_t st,
                 const T *rinv, int shape, const cplx<T> *coef)
{
    const bool wnc = op.wni != nullptr;
    if (!adj && !wnc) return sweep_dispatch<T, false, false>(op, x, b, nrhs, w, order, block, active, st, rinv, shape, coef);
    if (!adj && wnc) return sweep_dispatch<T, false, true>(op, x, b, nrhs, w, order, block, active, st, rinv, shape, coef);
    if (adj && !wnc) return sweep_dispatch<T, true, false>(op, x, b, nrhs, w, order, block, active, st, rinv, shape, coef);
    return sweep_dispatch<T, true, true>(op, x, b, nrhs, w, order, block, active, st, rinv, shape, coef);
}

template int launch_sweep<double>(const Op<double> &, cplx<double> *, const cplx<double> *, int, double, bool, int, const int32_t *, const int *, cudaStream_t, const double *, int, const cplx<double> *);
template int launch_sweep<float>(const Op<float> &, cplx<float> *, const cplx<float> *, int, float, bool, int, const int32_t *, const int *, cudaStream_t, const float *, int, const cplx<float> *);

}  // namespace h3d
