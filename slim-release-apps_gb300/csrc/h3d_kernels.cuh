// Host-callable launchers of the device kernels (one translation unit each).
#pragma once

#include "h3d_internal.cuh"

namespace h3d {

// L2-coherent load (bypasses L1), for data another CTA may have written in the same launch.
template <typename T>
__device__ __forceinline__ cplx<T> load_cg(const cplx<T> *p);
template <>
__device__ __forceinline__ cplx<double> load_cg(const cplx<double> *p)
{
    const double2 v = __ldcg(reinterpret_cast<const double2 *>(p));
    return {v.x, v.y};
}
template <>
__device__ __forceinline__ cplx<float> load_cg(const cplx<float> *p)
{
    const float2 v = __ldcg(reinterpret_cast<const float2 *>(p));
    return {v.x, v.y};
}

// h3d_stencil.cu
template <typename T>
int launch_mvp(const Op<T> &op, const cplx<T> *x, cplx<T> *y, int nrhs, bool adj, bool deriv,
               cudaStream_t st);
template <typename T>
int launch_sweep(const Op<T> &op, cplx<T> *x, const cplx<T> *b, int nrhs, T w, bool adj,
                 int order, const int32_t *block, const int *active, cudaStream_t st);

// h3d_block.cu: the BLOCK ordering (block wavefront, 27 colours inside a block).
template <typename T>
int sweep_block(const Op<T> &op, cplx<T> *x, const cplx<T> *b, int nrhs, T w,
                const int32_t *block, const int *active, bool adj, cudaStream_t st);

}  // namespace h3d
