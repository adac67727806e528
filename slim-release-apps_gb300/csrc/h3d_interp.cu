// One-dimensional sparse operators applied along one axis of a complex 3D field: the
// grid transfers of the multigrid preconditioner (construct_multigrid.m:45-51, built from
// LinInterp1D / opLInterp1D rows as fine2coarse.m does) are Kronecker products of three
// such operators, applied as three launches.
//
//   y[.., o, ..] = sum_{p in row o} val[p] * x[.., col[p], ..]      (o along `axis`)
//
// One thread per output value; a row has a handful of entries (two for linear
// interpolation, about four for its adjoint), read through the L1 cache.  The multigrid
// solver folds the restriction's 1/8 into its last axis (scale) and adds the prolongated
// correction to the fine solution in the same launch (accum: y += result, the result rounded
// to the field's precision first, as a separate sum would).
#include "h3d_kernels.cuh"

namespace h3d {

template <typename T>
__global__ void __launch_bounds__(256) axis_apply_kernel(const int32_t *__restrict__ rowptr,
                                                         const int32_t *__restrict__ col,
                                                         const double *__restrict__ val, int axis, int ox,
                                                         int oy, int oz, int ix, int iy, const cplx<T> *__restrict__ x,
                                                         cplx<T> *__restrict__ y, long long nout, long long nin,
                                                         double scale, int accum)
{
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const int s = blockIdx.y;
    if (q >= nout) return;
    const int i = (int)(q % ox), j = (int)((q / ox) % oy), k = (int)(q / ((long long)ox * oy));
    (void)oz;
    const int o = axis == 0 ? i : (axis == 1 ? j : k);
    const cplx<T> *xs = x + (long long)s * nin;
    double re = 0.0, im = 0.0;
    for (int p = rowptr[o]; p < rowptr[o + 1]; ++p) {
        const int c = col[p];
        const long long src = axis == 0 ? c + (long long)ix * (j + (long long)iy * k)
                              : axis == 1 ? i + (long long)ix * (c + (long long)iy * k)
                                          : i + (long long)ix * (j + (long long)iy * c);
        const cplx<T> v = xs[src];
        re += val[p] * (double)v.re;
        im += val[p] * (double)v.im;
    }
    cplx<T> v = mk<T>((T)(re * scale), (T)(im * scale));
    if (accum) v = y[(long long)s * nout + q] + v;
    y[(long long)s * nout + q] = v;
}

template <typename T>
int launch_axis(const int32_t *rowptr, const int32_t *col, const double *val, int n_out, int axis,
                const int32_t dims_in[3], const cplx<T> *x, cplx<T> *y, int nrhs, double scale, bool accum,
                cudaStream_t st)
{
    int od[3] = {dims_in[0], dims_in[1], dims_in[2]};
    od[axis] = n_out;
    const long long nout = (long long)od[0] * od[1] * od[2];
    const long long nin = (long long)dims_in[0] * dims_in[1] * dims_in[2];
    const long long blocks = (nout + 255) / 256;
    if (blocks > 0x7fffffffLL) {
        set_error("axis transfer: field too large");
        return H3D_ERR_NSIZE;
    }
    const dim3 grd((unsigned)blocks, nrhs);
    axis_apply_kernel<T><<<grd, 256, 0, st>>>(rowptr, col, val, axis, od[0], od[1], od[2], dims_in[0], dims_in[1], x,
                                              y, nout, nin, scale, accum ? 1 : 0);
    H3D_CUDA_TRY(cudaGetLastError());
    return H3D_OK;
}

template int launch_axis<double>(const int32_t *, const int32_t *, const double *, int, int, const int32_t[3],
                                 const cplx<double> *, cplx<double> *, int, double, bool, cudaStream_t);
template int launch_axis<float>(const int32_t *, const int32_t *, const double *, int, int, const int32_t[3],
                                const cplx<float> *, cplx<float> *, int, double, bool, cudaStream_t);

}  // namespace h3d

using namespace h3d;

extern "C" int h3d_axis_apply(const int32_t *rowptr, const int32_t *col, const double *val, int n_out, int axis,
                              const int32_t dims_in[3], const void *x, void *y, int nrhs, int dtype,
                              void *stream)
{
    if (!rowptr || !col || !val || !dims_in || !x || !y || n_out < 1 || axis < 0 || axis > 2 || nrhs < 1 ||
        dims_in[0] < 1 || dims_in[1] < 1 || dims_in[2] < 1 || nrhs > 65535) {
        set_error("h3d_axis_apply: bad argument");
        return H3D_ERR_BAD_ARG;
    }
    cudaStream_t st = (cudaStream_t)stream;
    if (dtype == H3D_C128)
        return launch_axis<double>(rowptr, col, val, n_out, axis, dims_in, (const cplx<double> *)x,
                                   (cplx<double> *)y, nrhs, 1.0, false, st);
    if (dtype == H3D_C64)
        return launch_axis<float>(rowptr, col, val, n_out, axis, dims_in, (const cplx<float> *)x,
                                  (cplx<float> *)y, nrhs, 1.0, false, st);
    set_error("h3d_axis_apply: unknown dtype %d", dtype);
    return H3D_ERR_BAD_ARG;
}
