// Layout conversions (h3d_vec.cu).
#pragma once

#include "h3d_internal.cuh"

namespace h3d {

template <typename T>
int interleave(const double *re, const double *im, cplx<T> *out, long long n, cudaStream_t st);
template <typename T>
int deinterleave(const cplx<T> *in, double *re, double *im, long long n, cudaStream_t st);
template <typename S, typename D>
int cast(const S *in, D *out, long long n, cudaStream_t st);

// RAII device buffer from the stream-ordered allocator.
struct DevBuf {
    void *p = nullptr;
    cudaStream_t st = nullptr;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf()
    {
        if (p) cudaFreeAsync(p, st);
    }
    int alloc(size_t bytes, cudaStream_t s)
    {
        st = s;
        cudaError_t e = cudaMallocAsync(&p, bytes ? bytes : 16, s);
        if (e != cudaSuccess) {
            p = nullptr;
            return cuda_fail(e, "cudaMallocAsync");
        }
        return H3D_OK;
    }
    void release()
    {
        if (p) cudaFreeAsync(p, st);
        p = nullptr;
    }
    template <typename U>
    U *as() const { return static_cast<U *>(p); }
};

}  // namespace h3d
