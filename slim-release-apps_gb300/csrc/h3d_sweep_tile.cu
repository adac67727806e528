// COLOUR27 Kaczmarz phase with the footprint box staged in shared memory.
//
// For one colour (a, b, c) = (i%3, j%3, k%3) the 3x3x3 footprints of the rows tile the
// grid.  A CTA owns TU x TV x TW rows of the colour; their footprints form one box of
// (3TU) x (3TV) x (3TW) points, disjoint from the boxes of the other CTAs.  The box is
// 27 copies of the CTA shape, so thread (u,v,w) copies the points (ox TU + u, oy TV + v,
// oz TW + w), ox,oy,oz in 0..2: coalesced along x, no index division.  Per right-hand
// side the CTA
//   1. copies the x box in (asynchronous, zero-filled outside the grid),
//   2. forms a_i.x from the three planes of its footprint with the plane-sum algebra of
//      the matvec, scales by the precomputed 1/||a_i||^2 (the norms do not change between
//      sweeps), d = w (b_i - a_i.x) / ||a_i||^2     (Helm3dkaczswp_mex.c:93-112),
//   3. scatters x_nbr += d conj(a_i,nbr) in shared memory (Helm3dkaczswp_mex.c:114-117),
//   4. writes the box back (only points inside the grid).
// Points outside the grid read as zero and are never stored: that is the zero boundary
// of the gather (Helm3d_27pt.h:483-520) and the masked scatter (Helm3d_27pt.h:522-590).
// Forward coefficients of outside neighbours still count as zero in the row norm.  CTAs
// whose rows all have PML values of exactly 1 scatter with real coefficients.
#include "h3d_internal.cuh"
#include "h3d_kernels.cuh"
#include "h3d_planes.cuh"

namespace h3d {

template <int BYTES>
__device__ __forceinline__ void cp_async_zfill(void *sdst, const void *gsrc, bool valid)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(sdst);
    const int n = valid ? BYTES : 0;
    if constexpr (BYTES == 16)
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gsrc), "r"(n) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], %2, %3;\n" ::"r"(s), "l"(gsrc), "n"(BYTES), "r"(n) : "memory");
}

__device__ __forceinline__ void cp_async_wait_all()
{
    asm volatile("cp.async.commit_group;\n" ::: "memory");
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
}

template <int TU, int TV, int TW>
struct TileGeom {
    static constexpr int NT = TU * TV * TW;
    static constexpr int BX = 3 * TU, BY = 3 * TV, BZ = 3 * TW;
    static constexpr int PX = BX + 1;  // padded pitch: rows of neighbouring threads fall on other banks
    static constexpr int PXY = PX * BY;
    static constexpr int NBP = PXY * BZ;
};

template <typename T, bool WNC, int TU, int TV, int TW>
constexpr size_t tile_smem()
{
    using G = TileGeom<TU, TV, TW>;
    return sizeof(cplx<T>) * G::NBP + sizeof(T) * G::NBP * (WNC ? 2 : 1);
}

// MINB: CTAs per SM the register allocation must allow (complex64: 2 caps a thread at 128
// registers, 1 lets the 27 coefficients of a PML row stay in registers without spilling).
template <typename T, bool ADJ, bool WNC, int TU, int TV, int TW, int MINB>
__global__ void __launch_bounds__(TU *TV *TW, MINB) sweep_tile_kernel(Op<T> op, cplx<T> *x, const cplx<T> *b,
                                                                int nrhs, int a, int bq, int cq, T w,
                                                                const int *active, const T *rinv)
{
    using G = TileGeom<TU, TV, TW>;
    constexpr int PX = G::PX, BY = G::BY, PXY = G::PXY, NBP = G::NBP;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cplx<T> *sx = reinterpret_cast<cplx<T> *>(smem_raw);
    T *swr = reinterpret_cast<T *>(sx + NBP);
    T *swi = WNC ? swr + NBP : nullptr;

    const int tu = threadIdx.x, tv = threadIdx.y, tw = threadIdx.z;
    const int u0 = blockIdx.x * TU, v0 = blockIdx.y * TV, w0 = blockIdx.z * TW;
    const int i0 = a - 1 + 3 * u0, j0 = bq - 1 + 3 * v0, k0 = cq - 1 + 3 * w0;  // box origin

    auto for_box = [&](auto &&f) {
#pragma unroll
        for (int oz = 0; oz < 3; ++oz) {
            const int bk = oz * TW + tw, gk = k0 + bk;
            const bool kin = gk >= 0 && gk < op.nz;
#pragma unroll
            for (int oy = 0; oy < 3; ++oy) {
                const int bj = oy * TV + tv, gj = j0 + bj;
                const bool jin = kin && gj >= 0 && gj < op.ny;
                const long long gjk = op.sy * gj + op.sz * gk;
#pragma unroll
                for (int ox = 0; ox < 3; ++ox) {
                    const int bi = ox * TU + tu, gi = i0 + bi;
                    const bool in = jin && gi >= 0 && gi < op.nx;
                    f(bi + PX * (bj + BY * bk), in, in ? gi + gjk : 0LL);
                }
            }
        }
    };

    for_box([&](int q, bool in, long long g) {
        cp_async_zfill<sizeof(T)>(swr + q, op.wn + g, in);
        if constexpr (WNC) cp_async_zfill<sizeof(T)>(swi + q, op.wni + g, in);
    });

    const int i = a + 3 * (u0 + tu), j = bq + 3 * (v0 + tv), k = cq + 3 * (w0 + tw);
    const bool valid = i < op.nx && j < op.ny && k < op.nz;
    const int lc = (3 * tu + 1) + PX * ((3 * tv + 1) + BY * (3 * tw + 1));
    const long long ctr = (long long)i + op.sy * j + op.sz * k;

    // Every row of this CTA has PML values of exactly 1 -> real coefficients.
    const int *ilo = ADJ ? op.int_lo_a : op.int_lo_f, *ihi = ADJ ? op.int_hi_a : op.int_hi_f;
    const int ri1 = a + 3 * (u0 + TU - 1), rj1 = bq + 3 * (v0 + TV - 1), rk1 = cq + 3 * (w0 + TW - 1);
    const bool interior = !WNC && a + 3 * u0 >= ilo[0] && ri1 < ihi[0] && bq + 3 * v0 >= ilo[1] &&
                          rj1 < ihi[1] && cq + 3 * w0 >= ilo[2] && rk1 < ihi[2] && ri1 < op.nx &&
                          rj1 < op.ny && rk1 < op.nz;

    cp_async_wait_all();
    __syncthreads();

    auto wnf = [&](int dx, int dy, int dz) {
        const int q = lc + dx + PX * (dy + BY * dz);
        return mk<T>(swr[q], WNC ? swi[q] : T(0));
    };
    auto wnr = [&](int dx, int dy, int dz) { return swr[lc + dx + PX * (dy + BY * dz)]; };

    // Per right-hand side: box in, project this thread's row (rows inside the grid only), box
    // out.  The row's 27 coefficients are formed in registers right before its gather and
    // reused by its scatter; they are formed again for every right-hand side, which keeps
    // them out of the registers that live across the box copies (multi-RHS solves are
    // better served by the BLOCK8 order, whose groups of right-hand sides share a block).
    auto run_rhs = [&](auto &&project) {
        for (int s = 0; s < nrhs; ++s) {
            if (active && !active[s]) continue;  // uniform over the CTA
            cplx<T> *xs = x + (long long)s * op.N;
            if (s > 0) __syncthreads();  // the previous box is fully written back
            for_box([&](int q, bool in, long long g) { cp_async_zfill<sizeof(cplx<T>)>(sx + q, xs + g, in); });
            cp_async_wait_all();
            __syncthreads();
            if (valid) project(b ? b + (long long)s * op.N : nullptr);
            __syncthreads();
            for_box([&](int q, bool in, long long g) {
                if (in) xs[g] = sx[q];
            });
        }
    };

    if (interior) {
        // every row of the CTA has PML values of exactly 1: real coefficients K_t - WM_t wn
        run_rhs([&](const cplx<T> *bs) {
            T cr[27];
#define H3D_CI(t, dx, dy, dz) cr[t] = coef_int<t, dx, dy, dz, T, ADJ>(op, wnr);
            H3D_FOR_27(H3D_CI)
#undef H3D_CI
            T inv;
            if (rinv) {
                inv = rinv[ctr];
            } else {
                T nrm = T(0);
#pragma unroll
                for (int t = 0; t < 27; ++t) nrm += cr[t] * cr[t];
                inv = T(1) / nrm;
            }
            // one partial sum per plane dz: three shorter dependency chains
        cplx<T> acc[3] = {mk<T>(T(0), T(0)), mk<T>(T(0), T(0)), mk<T>(T(0), T(0))};
#define H3D_GI(t, dx, dy, dz)                                                                  \
    {                                                                                          \
        const cplx<T> xv = sx[lc + dx + PX * (dy + BY * dz)];                                  \
        fma_rc(acc[dz + 1], cr[t], xv);                                                        \
    }
            H3D_FOR_27(H3D_GI)
#undef H3D_GI
        const cplx<T> atx = (acc[0] + acc[1]) + acc[2];
            const cplx<T> bv = bs ? bs[ctr] : mk<T>(T(0), T(0));
            const cplx<T> d = (w * inv) * (bv - atx);
#define H3D_SI(t, dx, dy, dz)                                                                  \
    {                                                                                          \
        cplx<T> &o = sx[lc + dx + PX * (dy + BY * dz)];                                        \
        fma_rc(o, cr[t], d);                                                                   \
    }
            H3D_FOR_27(H3D_SI)
#undef H3D_SI
        });
    } else {
        run_rhs([&](const cplx<T> *bs) {
            const RowPml<T> pml = load_row_pml<T, ADJ>(op, i, j, k);
            const uint32_t m = ADJ ? 0x7ffffffu : inside_mask(i, j, k, op.nx, op.ny, op.nz);
            // forward coefficients of outside neighbours are zero; adjoint ones are not (they
            // count in the norm), and x outside the grid is never stored (for_box)
            cplx<T> c[27];
#define H3D_CC(t, dx, dy, dz) c[t] = coef_at<t, dx, dy, dz, T, ADJ, false, WNC>(op, pml, m, wnf);
            H3D_FOR_27(H3D_CC)
#undef H3D_CC
            T inv;
            if (rinv) {
                inv = rinv[ctr];
            } else {
                T nrm = T(0);
#pragma unroll
                for (int t = 0; t < 27; ++t) nrm += cabs2(c[t]);
                inv = T(1) / nrm;
            }
            const cplx<T> z = mk<T>(T(0), T(0));
            CSum<T> acc[3] = {csum_init(z), csum_init(z), csum_init(z)};
#define H3D_GC(t, dx, dy, dz)                                                                  \
    {                                                                                          \
        const cplx<T> xv = sx[lc + dx + PX * (dy + BY * dz)];                                  \
        csum_mac(acc[dz + 1], c[t], xv);                                                       \
    }
            H3D_FOR_27(H3D_GC)
#undef H3D_GC
            const cplx<T> atx = cadd(cadd(csum_value(acc[0]), csum_value(acc[1])), csum_value(acc[2]));
            const cplx<T> bv = bs ? bs[ctr] : mk<T>(T(0), T(0));
            const Scat<T> sd = scat_of((w * inv) * (bv - atx));
#define H3D_SC(t, dx, dy, dz)                                                                  \
    {                                                                                          \
        cplx<T> &o = sx[lc + dx + PX * (dy + BY * dz)];                                        \
        scat_mac(o, sd, c[t]);                                                                 \
    }
            H3D_FOR_27(H3D_SC)
#undef H3D_SC
        });
    }
}

// 1/||a_i||^2 for every row (iteration-invariant), in the storage precision of the sweep.
template <typename T, bool ADJ, bool WNC>
__global__ void __launch_bounds__(256) rownorm_kernel(Op<T> op, T *rinv)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= op.nx || j >= op.ny) return;
    const uint32_t m = ADJ ? 0x7ffffffu : inside_mask(i, j, k, op.nx, op.ny, op.nz);
    cplx<T> c[27];
    row_coefs<T, ADJ, false, WNC>(op, i, j, k, m, c);
    T nrm = T(0);
#pragma unroll
    for (int t = 0; t < 27; ++t) nrm += cabs2(c[t]);
    rinv[i + op.sy * j + op.sz * k] = T(1) / nrm;
}

template <typename T>
int row_inv_norms(const Op<T> &op, bool adj, T *rinv, cudaStream_t st)
{
    const dim3 blk(32, 8), grd((op.nx + 31) / 32, (op.ny + 7) / 8, op.nz);
    const bool wnc = op.wni != nullptr;
    if (!adj && !wnc) rownorm_kernel<T, false, false><<<grd, blk, 0, st>>>(op, rinv);
    else if (!adj && wnc) rownorm_kernel<T, false, true><<<grd, blk, 0, st>>>(op, rinv);
    else if (adj && !wnc) rownorm_kernel<T, true, false><<<grd, blk, 0, st>>>(op, rinv);
    else rownorm_kernel<T, true, true><<<grd, blk, 0, st>>>(op, rinv);
    H3D_CUDA_TRY(cudaGetLastError());
    return H3D_OK;
}

// Candidate tile shapes (rows of one colour per CTA).
struct Shape {
    int tu, tv, tw, minb;
};
static const Shape kShapes[] = {{32, 4, 2, 2}, {16, 8, 2, 2}, {8, 8, 4, 2}, {32, 4, 2, 1}};
constexpr int kNumShapes = 4;

int num_tile_shapes() { return kNumShapes; }

// Launched rows that exist, summed over the 27 colours: least padding wins, ties go to
// the wider x extent (longer coalesced runs).
int pick_tile_shape(int nx, int ny, int nz)
{
    int best = 0;
    double best_eff = -1;
    for (int s = 0; s < 3; ++s) {  // the register-rich variant is left to the measured tuner
        double eff = 0;
        for (int q = 0; q < 27; ++q) {
            const int a = q % 3, b = (q / 3) % 3, c = q / 9;
            const long long nu = (nx - a + 2) / 3, nv = (ny - b + 2) / 3, nw = (nz - c + 2) / 3;
            if (nu <= 0 || nv <= 0 || nw <= 0) continue;
            const long long pu = (nu + kShapes[s].tu - 1) / kShapes[s].tu * kShapes[s].tu;
            const long long pv = (nv + kShapes[s].tv - 1) / kShapes[s].tv * kShapes[s].tv;
            const long long pw = (nw + kShapes[s].tw - 1) / kShapes[s].tw * kShapes[s].tw;
            eff += (double)(nu * nv * nw) / (double)(pu * pv * pw);
        }
        if (eff > best_eff + 1e-9) {
            best = s;
            best_eff = eff;
        }
    }
    return best;
}

template <typename T, bool ADJ, bool WNC, int TU, int TV, int TW, int MINB>
static int tile_pass_shape(const Op<T> &op, cplx<T> *x, const cplx<T> *b, int nrhs, T w,
                           const int *active, const T *rinv, bool backward, cudaStream_t st)
{
    constexpr size_t smem = tile_smem<T, WNC, TU, TV, TW>();
    static bool attr_set = false;  // per template instance and process
    if (!attr_set) {
        H3D_CUDA_TRY(cudaFuncSetAttribute(sweep_tile_kernel<T, ADJ, WNC, TU, TV, TW, MINB>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        attr_set = true;
    }
    const dim3 blk(TU, TV, TW);
    for (int qq = 0; qq < 27; ++qq) {
        const int q = backward ? 26 - qq : qq;
        const int a = q % 3, bq = (q / 3) % 3, cq = q / 9;
        const int nu = (op.nx - a + 2) / 3, nv = (op.ny - bq + 2) / 3, nw = (op.nz - cq + 2) / 3;
        if (nu <= 0 || nv <= 0 || nw <= 0) continue;
        const dim3 grd((nu + TU - 1) / TU, (nv + TV - 1) / TV, (nw + TW - 1) / TW);
        sweep_tile_kernel<T, ADJ, WNC, TU, TV, TW, MINB><<<grd, blk, smem, st>>>(op, x, b, nrhs, a, bq, cq, w,
                                                                          active, rinv);
    }
    H3D_CUDA_TRY(cudaGetLastError());
    return H3D_OK;
}

template <typename T, bool ADJ, bool WNC>
static int tile_pass(const Op<T> &op, cplx<T> *x, const cplx<T> *b, int nrhs, T w,
                     const int *active, const T *rinv, int shape, bool backward, cudaStream_t st)
{
    switch (shape) {
    case 1: return tile_pass_shape<T, ADJ, WNC, 16, 8, 2, sizeof(T) == 4 ? 2 : 1>(op, x, b, nrhs, w, active, rinv, backward, st);
    case 2: return tile_pass_shape<T, ADJ, WNC, 8, 8, 4, sizeof(T) == 4 ? 2 : 1>(op, x, b, nrhs, w, active, rinv, backward, st);
    case 3: return tile_pass_shape<T, ADJ, WNC, 32, 4, 2, 1>(op, x, b, nrhs, w, active, rinv, backward, st);
    default: return tile_pass_shape<T, ADJ, WNC, 32, 4, 2, sizeof(T) == 4 ? 2 : 1>(op, x, b, nrhs, w, active, rinv, backward, st);
    }
}

template <typename T>
int sweep_colour_tiled(const Op<T> &op, cplx<T> *x, const cplx<T> *b, int nrhs, T w,
                       const int *active, const T *rinv, int shape, bool adj, bool backward,
                       cudaStream_t st)
{
    if (shape < 0) shape = pick_tile_shape(op.nx, op.ny, op.nz);
    const bool wnc = op.wni != nullptr;
    if (!adj && !wnc) return tile_pass<T, false, false>(op, x, b, nrhs, w, active, rinv, shape, backward, st);
    if (!adj && wnc) return tile_pass<T, false, true>(op, x, b, nrhs, w, active, rinv, shape, backward, st);
    if (adj && !wnc) return tile_pass<T, true, false>(op, x, b, nrhs, w, active, rinv, shape, backward, st);
    return tile_pass<T, true, true>(op, x, b, nrhs, w, active, rinv, shape, backward, st);
}

template int sweep_colour_tiled<double>(const Op<double> &, cplx<double> *, const cplx<double> *, int, double, const int *, const double *, int, bool, bool, cudaStream_t);
template int sweep_colour_tiled<float>(const Op<float> &, cplx<float> *, const cplx<float> *, int, float, const int *, const float *, int, bool, bool, cudaStream_t);
template int row_inv_norms<double>(const Op<double> &, bool, double *, cudaStream_t);
template int row_inv_norms<float>(const Op<float> &, bool, float *, cudaStream_t);

}  // namespace h3d
