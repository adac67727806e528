// One Kaczmarz row projection on a block of x held in shared memory, shared by the two
// block orderings (h3d_block.cu: wavefront of blocks; h3d_block8.cu: parity classes of
// blocks).  The block's box has a one-point halo: PX x PY x PZ points, x fastest.
//
//   a.x = sum_t a_t x_t over the footprint,
//   d = w (b_i - a.x) / ||a||^2                         (Helm3dkaczswp_mex.c:93-112),
//   x_nbr += d conj(a_nbr) for neighbours inside the grid (Helm3dkaczswp_mex.c:114-117).
//
// The box stays resident across the 27 colours of a block, so its points outside the grid
// must keep reading as zero (the zero boundary of the gather, Helm3d_27pt.h:483-520):
// adjoint coefficients of outside neighbours are not zero, so the scatter is masked.
#pragma once

#include "h3d_internal.cuh"

namespace h3d {

template <int BYTES>
__device__ __forceinline__ void blk_cp_async(void *sdst, const void *gsrc, bool valid)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(sdst);
    const int n = valid ? BYTES : 0;
    if constexpr (BYTES == 16)
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gsrc), "r"(n) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], %2, %3;\n" ::"r"(s), "l"(gsrc), "n"(BYTES), "r"(n) : "memory");
}

__device__ __forceinline__ void blk_cp_async_wait_all()
{
    asm volatile("cp.async.commit_group;\n" ::: "memory");
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
}

template <int BX, int BY, int BZ>
struct BlockGeom {
    static constexpr int PX = BX + 2, PY = BY + 2, PZ = BZ + 2;  // box with a one-point halo
    static constexpr int PXY = PX * PY;
    static constexpr int NB = PXY * PZ;
};

template <typename T, bool WNC, int BX, int BY, int BZ, int R>
__host__ __device__ constexpr size_t block_smem()
{
    using G = BlockGeom<BX, BY, BZ>;
    return sizeof(cplx<T>) * G::NB * R + sizeof(T) * G::NB * (WNC ? 2 : 1);
}

// Copy the halo'd box at global origin (i0, j0, k0) of the wavenumber and of the right-hand
// sides s0 + r with bit r of act set (zero fill outside the grid); NT threads.
template <typename T, bool WNC, int PX, int PY, int NB, int R, int NT>
__device__ __forceinline__ void block_stage(const Op<T> &op, const cplx<T> *x, int s0, unsigned act,
                                            int i0, int j0, int k0, cplx<T> *sx, T *swr, T *swi)
{
    for (int e = threadIdx.x; e < NB; e += NT) {
        const int li = e % PX, lj = (e / PX) % PY, lk = e / (PX * PY);
        const int gi = i0 + li, gj = j0 + lj, gk = k0 + lk;
        const bool in = gi >= 0 && gi < op.nx && gj >= 0 && gj < op.ny && gk >= 0 && gk < op.nz;
        const long long g = in ? gi + op.sy * gj + op.sz * gk : 0;
        blk_cp_async<sizeof(T)>(swr + e, op.wn + g, in);
        if constexpr (WNC) blk_cp_async<sizeof(T)>(swi + e, op.wni + g, in);
#pragma unroll
        for (int r = 0; r < R; ++r)
            if (act & (1u << r))
                blk_cp_async<sizeof(cplx<T>)>(sx + (size_t)r * NB + e, x + (long long)(s0 + r) * op.N + g, in);
    }
    blk_cp_async_wait_all();
}

// Store the box back (halo included: the rows at the block's faces update the neighbouring
// blocks' edge points), points inside the grid only.
template <typename T, int PX, int PY, int NB, int R, int NT>
__device__ __forceinline__ void block_store(const Op<T> &op, cplx<T> *x, int s0, unsigned act, int i0,
                                            int j0, int k0, const cplx<T> *sx)
{
    for (int e = threadIdx.x; e < NB; e += NT) {
        const int li = e % PX, lj = (e / PX) % PY, lk = e / (PX * PY);
        const int gi = i0 + li, gj = j0 + lj, gk = k0 + lk;
        if (gi < 0 || gi >= op.nx || gj < 0 || gj >= op.ny || gk < 0 || gk >= op.nz) continue;
        const long long g = gi + op.sy * gj + op.sz * gk;
#pragma unroll
        for (int r = 0; r < R; ++r)
            if (act & (1u << r)) x[(long long)(s0 + r) * op.N + g] = sx[(size_t)r * NB + e];
    }
}

// Project row (i, j, k) at box index lc for one right-hand side (box bx; bv = b_i and
// inv = 1/||a_i||^2, loaded by the caller so that it can fetch them ahead of time).  The 27
// coefficients are formed once, in registers, and serve both the gather (three partial
// sums, one per plane dz, each in offset order) and the scatter.  Rows whose whole footprint has PML values of exactly 1 have real
// coefficients: K_t - WM_t wn.
template <typename T, bool ADJ, bool WNC, int PX, int PY>
__device__ __forceinline__ void block_row(const Op<T> &op, cplx<T> *bx, const T *swr, const T *swi,
                                          cplx<T> bv, T inv, T w, int i, int j, int k, int lc)
{
    const int *ilo = ADJ ? op.int_lo_a : op.int_lo_f, *ihi = ADJ ? op.int_hi_a : op.int_hi_f;
    const bool interior =
        !WNC && i >= ilo[0] && i < ihi[0] && j >= ilo[1] && j < ihi[1] && k >= ilo[2] && k < ihi[2];
    auto wnf = [&](int dx, int dy, int dz) {
        const int qd = lc + dx + PX * (dy + PY * dz);
        return mk<T>(swr[qd], WNC ? swi[qd] : T(0));
    };
    auto wnr = [&](int dx, int dy, int dz) { return swr[lc + dx + PX * (dy + PY * dz)]; };
    if (interior) {
        T cr[27];
#define H3D_CI(t, dx, dy, dz) cr[t] = coef_int<t, dx, dy, dz, T, ADJ>(op, wnr);
        H3D_FOR_27(H3D_CI)
#undef H3D_CI
        // one partial sum per plane dz: three shorter dependency chains
        cplx<T> acc[3] = {mk<T>(T(0), T(0)), mk<T>(T(0), T(0)), mk<T>(T(0), T(0))};
        cplx<T> xv[27];  // kept for the scatter (the footprint is this row's alone in the colour)
#define H3D_GI(t, dx, dy, dz)                                                                  \
    {                                                                                          \
        xv[t] = bx[lc + dx + PX * (dy + PY * dz)];                                             \
        fma_rc(acc[dz + 1], cr[t], xv[t]);                                                     \
    }
        H3D_FOR_27(H3D_GI)
#undef H3D_GI
        const cplx<T> atx = cadd(cadd(acc[0], acc[1]), acc[2]);
        const cplx<T> d = (w * inv) * (bv - atx);
#define H3D_SI(t, dx, dy, dz)                                                                  \
    {                                                                                          \
        cplx<T> o = xv[t];                                                                     \
        fma_rc(o, cr[t], d);                                                                   \
        bx[lc + dx + PX * (dy + PY * dz)] = o;                                                 \
    }
        H3D_FOR_27(H3D_SI)
#undef H3D_SI
    } else {
        const RowPml<T> pml = load_row_pml<T, ADJ>(op, i, j, k);
        const uint32_t m = inside_mask(i, j, k, op.nx, op.ny, op.nz);
        cplx<T> c[27];
        // forward coefficients of outside neighbours are zero (m); adjoint ones are not, so
        // the scatter is masked to keep the box's outside points at zero
#define H3D_CC(t, dx, dy, dz) c[t] = coef_at<t, dx, dy, dz, T, ADJ, false, WNC>(op, pml, ADJ ? 0x7ffffffu : m, wnf);
        H3D_FOR_27(H3D_CC)
#undef H3D_CC
        const cplx<T> z = mk<T>(T(0), T(0));
        CSum<T> acc[3] = {csum_init(z), csum_init(z), csum_init(z)};
        cplx<T> xv[27];  // kept for the scatter (the footprint is this row's alone in the colour)
#define H3D_GC(t, dx, dy, dz)                                                                  \
    {                                                                                          \
        xv[t] = bx[lc + dx + PX * (dy + PY * dz)];                                             \
        csum_mac(acc[dz + 1], c[t], xv[t]);                                                    \
    }
        H3D_FOR_27(H3D_GC)
#undef H3D_GC
        const cplx<T> atx = cadd(cadd(csum_value(acc[0]), csum_value(acc[1])), csum_value(acc[2]));
        const Scat<T> sd = scat_of((w * inv) * (bv - atx));
#define H3D_SC(t, dx, dy, dz)                                                                  \
    if (m & (1u << t)) {                                                                       \
        cplx<T> o = xv[t];                                                                     \
        scat_mac(o, sd, c[t]);                                                                 \
        bx[lc + dx + PX * (dy + PY * dz)] = o;                                                 \
    }
        H3D_FOR_27(H3D_SC)
#undef H3D_SC
    }
}

// Project row (i, j, k) with its 27 coefficients read from shared memory (sc[t * NR + row],
// staged from the stored coefficients).  Neighbours outside the grid are masked as above;
// EDGE = false: the caller's block has no row on a face of the grid, nothing is masked.
template <typename T, int PX, int PY, bool EDGE>
__device__ __forceinline__ void block_row_stored(const Op<T> &op, cplx<T> *bx, const cplx<T> *sc, int NR, int row,
                                                 cplx<T> bv, T inv, T w, int i, int j, int k, int lc)
{
    uint32_t m = 0x7ffffffu;
    if constexpr (EDGE) {
        const bool edge = i == 0 || j == 0 || k == 0 || i == op.nx - 1 || j == op.ny - 1 || k == op.nz - 1;
        if (edge) m = inside_mask(i, j, k, op.nx, op.ny, op.nz);
    }
    cplx<T> c[27], xv[27];
#pragma unroll
    for (int t = 0; t < 27; ++t) c[t] = sc[t * NR + row];
    const cplx<T> z = mk<T>(T(0), T(0));
    CSum<T> acc[3] = {csum_init(z), csum_init(z), csum_init(z)};
    // the gathered values stay in registers for the scatter: no other row of this colour
    // touches the footprint, so they are still current when it is written back
#define H3D_GS(t, dx, dy, dz)                                                                  \
    {                                                                                          \
        xv[t] = bx[lc + dx + PX * (dy + PY * dz)];                                             \
        csum_mac(acc[dz + 1], c[t], xv[t]);                                                    \
    }
    H3D_FOR_27(H3D_GS)
#undef H3D_GS
    const cplx<T> atx = cadd(cadd(csum_value(acc[0]), csum_value(acc[1])), csum_value(acc[2]));
    const Scat<T> sd = scat_of((w * inv) * (bv - atx));
#define H3D_SS(t, dx, dy, dz)                                                                  \
    if (m & (1u << t)) {                                                                       \
        cplx<T> o = xv[t];                                                                     \
        scat_mac(o, sd, c[t]);                                                                 \
        bx[lc + dx + PX * (dy + PY * dz)] = o;                                                 \
    }
    H3D_FOR_27(H3D_SS)
#undef H3D_SS
}

// Row projections with the coefficients already in registers, so that one thread can project
// the same row for several right-hand sides from one load of its coefficients.
//   row_project_c: complex coefficients; the scatter skips the neighbours outside m
//   row_project_r: real coefficients of an interior row (nothing outside the grid)
// The gathered values stay in registers for the scatter (the footprint is the row's alone
// within its colour).
template <typename T, int PX, int PY>
__device__ __forceinline__ void row_project_c(cplx<T> *bx, const cplx<T> (&c)[27], uint32_t m, cplx<T> bv, T inv,
                                              T w, int lc)
{
    cplx<T> xv[27];
    const cplx<T> z = mk<T>(T(0), T(0));
    CSum<T> acc[3] = {csum_init(z), csum_init(z), csum_init(z)};
#define H3D_GP(t, dx, dy, dz)                                                                  \
    {                                                                                          \
        xv[t] = bx[lc + dx + PX * (dy + PY * dz)];                                             \
        csum_mac(acc[dz + 1], c[t], xv[t]);                                                    \
    }
    H3D_FOR_27(H3D_GP)
#undef H3D_GP
    const cplx<T> atx = cadd(cadd(csum_value(acc[0]), csum_value(acc[1])), csum_value(acc[2]));
    const Scat<T> sd = scat_of((w * inv) * (bv - atx));
#define H3D_SP(t, dx, dy, dz)                                                                  \
    if (m & (1u << t)) {                                                                       \
        cplx<T> o = xv[t];                                                                     \
        scat_mac(o, sd, c[t]);                                                                 \
        bx[lc + dx + PX * (dy + PY * dz)] = o;                                                 \
    }
    H3D_FOR_27(H3D_SP)
#undef H3D_SP
}

template <typename T, int PX, int PY>
__device__ __forceinline__ void row_project_r(cplx<T> *bx, const T (&cr)[27], cplx<T> bv, T inv, T w, int lc)
{
    cplx<T> xv[27];
    cplx<T> acc[3] = {mk<T>(T(0), T(0)), mk<T>(T(0), T(0)), mk<T>(T(0), T(0))};
#define H3D_GR(t, dx, dy, dz)                                                                  \
    {                                                                                          \
        xv[t] = bx[lc + dx + PX * (dy + PY * dz)];                                             \
        fma_rc(acc[dz + 1], cr[t], xv[t]);                                                     \
    }
    H3D_FOR_27(H3D_GR)
#undef H3D_GR
    const cplx<T> atx = cadd(cadd(acc[0], acc[1]), acc[2]);
    const cplx<T> d = (w * inv) * (bv - atx);
#define H3D_SR(t, dx, dy, dz)                                                                  \
    {                                                                                          \
        cplx<T> o = xv[t];                                                                     \
        fma_rc(o, cr[t], d);                                                                   \
        bx[lc + dx + PX * (dy + PY * dz)] = o;                                                 \
    }
    H3D_FOR_27(H3D_SR)
#undef H3D_SR
}

// The 27 real coefficients of an interior row (all PML values 1, real wavenumber) from the
// wavenumber box: K_t - WM_t wn (Helm3d_27pt.h:676-825 with xi = 1).
template <typename T, bool ADJ, int PX, int PY>
__device__ __forceinline__ void interior_coefs(const Op<T> &op, const T *swr, int lc, T (&cr)[27])
{
    auto wnr = [&](int dx, int dy, int dz) { return swr[lc + dx + PX * (dy + PY * dz)]; };
#define H3D_CIR(t, dx, dy, dz) cr[t] = coef_int<t, dx, dy, dz, T, ADJ>(op, wnr);
    H3D_FOR_27(H3D_CIR)
#undef H3D_CIR
}

}  // namespace h3d
