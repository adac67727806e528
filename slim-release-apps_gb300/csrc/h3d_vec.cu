// Layout conversion kernels between MATLAB's separate real/imaginary planes and the
// interleaved complex vectors the stencil kernels use, plus precision casts.
#include "h3d_internal.cuh"
#include "h3d_vec.cuh"

namespace h3d {

template <typename T>
__global__ void interleave_kernel(const double *__restrict__ re, const double *__restrict__ im,
                                  cplx<T> *__restrict__ out, long long n)
{
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
         q += (long long)gridDim.x * blockDim.x)
        out[q] = mk<T>((T)re[q], im ? (T)im[q] : T(0));
}

template <typename T>
__global__ void deinterleave_kernel(const cplx<T> *__restrict__ in, double *__restrict__ re,
                                    double *__restrict__ im, long long n)
{
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
         q += (long long)gridDim.x * blockDim.x) {
        const cplx<T> v = in[q];
        re[q] = (double)v.re;
        im[q] = (double)v.im;
    }
}

template <typename S, typename D>
__global__ void cast_kernel(const S *__restrict__ in, D *__restrict__ out, long long n)
{
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
         q += (long long)gridDim.x * blockDim.x)
        out[q] = (D)in[q];
}

static inline unsigned grid_for(long long n)
{
    long long g = (n + 255) / 256;
    if (g > 152 * 32) g = 152 * 32;
    if (g < 1) g = 1;
    return (unsigned)g;
}

template <typename T>
int interleave(const double *re, const double *im, cplx<T> *out, long long n, cudaStream_t st)
{
    interleave_kernel<T><<<grid_for(n), 256, 0, st>>>(re, im, out, n);
    H3D_CUDA_TRY(cudaGetLastError());
    return H3D_OK;
}

template <typename T>
int deinterleave(const cplx<T> *in, double *re, double *im, long long n, cudaStream_t st)
{
    deinterleave_kernel<T><<<grid_for(n), 256, 0, st>>>(in, re, im, n);
    H3D_CUDA_TRY(cudaGetLastError());
    return H3D_OK;
}

template <typename S, typename D>
int cast(const S *in, D *out, long long n, cudaStream_t st)
{
    cast_kernel<S, D><<<grid_for(n), 256, 0, st>>>(in, out, n);
    H3D_CUDA_TRY(cudaGetLastError());
    return H3D_OK;
}

template int interleave<double>(const double *, const double *, cplx<double> *, long long, cudaStream_t);
template int interleave<float>(const double *, const double *, cplx<float> *, long long, cudaStream_t);
template int deinterleave<double>(const cplx<double> *, double *, double *, long long, cudaStream_t);
template int deinterleave<float>(const cplx<float> *, double *, double *, long long, cudaStream_t);
template int cast<double, float>(const double *, float *, long long, cudaStream_t);
template int cast<float, double>(const float *, double *, long long, cudaStream_t);

}  // namespace h3d
