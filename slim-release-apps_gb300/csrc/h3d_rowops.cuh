// Per-row device routines shared by the sweep kernels (one Kaczmarz row projection).
#pragma once

#include "h3d_internal.cuh"

namespace h3d {

template <typename T>
__device__ __forceinline__ cplx<T> ldg_c(const cplx<T> *p);
template <>
__device__ __forceinline__ cplx<double> ldg_c(const cplx<double> *p)
{
    const double2 v = __ldg(reinterpret_cast<const double2 *>(p));
    return {v.x, v.y};
}
template <>
__device__ __forceinline__ cplx<float> ldg_c(const cplx<float> *p)
{
    const float2 v = __ldg(reinterpret_cast<const float2 *>(p));
    return {v.x, v.y};
}

// One Kaczmarz row projection on every active right-hand side (do_sweep body,
// Helm3dkaczswp_mex.c:93-118): d = w (b_i - a_i.x) / ||a_i||^2, x_nbr += d conj(a_i).
// The row norm runs over all 27 coefficients: masked ones are zero in forward mode, but
// the adjoint coefficients of outside neighbours are not masked and do count.
template <typename T, bool ADJ, bool WNC>
__device__ __forceinline__ void project_row(const Op<T> &op, cplx<T> *x, const cplx<T> *b,
                                            int nrhs, int i, int j, int k, T w,
                                            const int *active)
{
    const uint32_t m = inside_mask(i, j, k, op.nx, op.ny, op.nz);
    cplx<T> c[27];
    row_coefs<T, ADJ, false, WNC>(op, i, j, k, m, c);
    T nrm = T(0);
#pragma unroll
    for (int t = 0; t < 27; ++t) nrm += cabs2(c[t]);
    const long long ctr = i + op.sy * j + op.sz * k;
    for (int s = 0; s < nrhs; ++s) {
        if (active && !active[s]) continue;
        cplx<T> *xs = x + (long long)s * op.N + ctr;
        cplx<T> atx = mk<T>(T(0), T(0));
#define H3D_GATHER(t, dx, dy, dz)                                                              \
    if (m & (1u << t)) {                                                                       \
        cmac(atx, c[t], xs[dx + op.sy * dy + op.sz * dz]);                                     \
    }
        H3D_FOR_27(H3D_GATHER)
#undef H3D_GATHER
        cplx<T> bv = b ? b[(long long)s * op.N + ctr] : mk<T>(T(0), T(0));
        cplx<T> d = w * (bv - atx);
        d.re = d.re / nrm;
        d.im = d.im / nrm;
#define H3D_SCATTER(t, dx, dy, dz)                                                             \
    if (m & (1u << t)) {                                                                       \
        cplx<T> *p = xs + (dx + op.sy * dy + op.sz * dz);                                      \
        const cplx<T> u = d * cconj(c[t]);                                                     \
        cplx<T> o = *p;                                                                        \
        o.re += u.re;                                                                          \
        o.im += u.im;                                                                          \
        *p = o;                                                                                \
    }
        H3D_FOR_27(H3D_SCATTER)
#undef H3D_SCATTER
    }
}

}  // namespace h3d
