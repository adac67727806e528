// COLOUR27 Kaczmarz sweep on stored row coefficients ("direct" implementation).
//
// Same row order and arithmetic as sweep_tile_kernel (one launch per colour q = i%3 +
// 3(j%3) + 9(k%3), ascending then descending), without the shared-memory box: the rows of
// one colour have disjoint 3x3x3 footprints, so every thread gathers its footprint straight
// from x (L1/L2) and writes its footprint back with no other row touching it in the launch.
//
// The 27 complex coefficients of every row are formed once per operator (coef_store_kernel,
// the same coef_at arithmetic as every other kernel) and kept in HBM in colour-major order:
// colour q owns M_q = nu nv nw rows (its own sub-grid, u fastest), and coefficient t of row
// lin sits at base_q + t M_q + lin, so a warp of consecutive rows reads 32 consecutive
// values per offset.  Rows whose PML values are all exactly 1 (the interior) do not read
// them: their real coefficients K_t - WM_t wn cost one FMA each.  A PML row then costs 27
// coalesced loads instead of ~27 complex PML expressions, and the coefficient stream is
// reused by every right-hand side of the launch.
//
// Storage: 27 N complex values (complex64: 216 B per grid point), allocated by the solver
// when it fits the coefficient budget; otherwise the shared-memory tile kernel runs.
#include "h3d_internal.cuh"
#include "h3d_kernels.cuh"

namespace h3d {

// Colour q sub-grid of rows (a + 3u, b + 3v, c + 3w).
struct ColourGrid {
    int a, b, c, nu, nv, nw;
    long long base, M;  // first coefficient of the colour, rows in the colour
};

__host__ __device__ inline ColourGrid colour_grid(int nx, int ny, int nz, int q)
{
    ColourGrid g;
    g.a = q % 3;
    g.b = (q / 3) % 3;
    g.c = q / 9;
    g.nu = nx > g.a ? (nx - g.a + 2) / 3 : 0;
    g.nv = ny > g.b ? (ny - g.b + 2) / 3 : 0;
    g.nw = nz > g.c ? (nz - g.c + 2) / 3 : 0;
    g.M = (long long)g.nu * g.nv * g.nw;
    g.base = 0;
    for (int p = 0; p < q; ++p) {
        const int a = p % 3, b = (p / 3) % 3, c = p / 9;
        const long long nu = nx > a ? (nx - a + 2) / 3 : 0, nv = ny > b ? (ny - b + 2) / 3 : 0,
                        nw = nz > c ? (nz - c + 2) / 3 : 0;
        g.base += 27 * nu * nv * nw;
    }
    return g;
}

// coef[base_q + t M_q + lin] = coefficient t of row (i, j, k) of the forward (ADJ = false) or
// adjoint operator, for every row.  One thread per row, rows of colour q.
template <typename T, bool ADJ, bool WNC>
__global__ void __launch_bounds__(128) coef_store_kernel(Op<T> op, cplx<T> *coef, ColourGrid g)
{
    const int u = blockIdx.x * blockDim.x + threadIdx.x, v = blockIdx.y, w = blockIdx.z;
    if (u >= g.nu) return;
    const int i = g.a + 3 * u, j = g.b + 3 * v, k = g.c + 3 * w;
    const uint32_t m = ADJ ? 0x7ffffffu : inside_mask(i, j, k, op.nx, op.ny, op.nz);
    cplx<T> c[27];
    row_coefs<T, ADJ, false, WNC>(op, i, j, k, m, c);
    const long long lin = u + (long long)g.nu * (v + (long long)g.nv * w);
    cplx<T> *dst = coef + g.base + lin;
#pragma unroll
    for (int t = 0; t < 27; ++t) dst[t * g.M] = c[t];
}

template <typename T>
int store_row_coefs(const Op<T> &op, bool adj, cplx<T> *coef, cudaStream_t st)
{
    const bool wnc = op.wni != nullptr;
    for (int q = 0; q < 27; ++q) {
        const ColourGrid g = colour_grid(op.nx, op.ny, op.nz, q);
        if (g.M == 0) continue;
        if (g.nv > 65535 || g.nw > 65535) {
            set_error("grid too large for the coefficient store");
            return H3D_ERR_NSIZE;
        }
        const dim3 grd((g.nu + 127) / 128, g.nv, g.nw);
        if (!adj && !wnc) coef_store_kernel<T, false, false><<<grd, 128, 0, st>>>(op, coef, g);
        else if (!adj && wnc) coef_store_kernel<T, false, true><<<grd, 128, 0, st>>>(op, coef, g);
        else if (adj && !wnc) coef_store_kernel<T, true, false><<<grd, 128, 0, st>>>(op, coef, g);
        else coef_store_kernel<T, true, true><<<grd, 128, 0, st>>>(op, coef, g);
    }
    H3D_CUDA_TRY(cudaGetLastError());
    return H3D_OK;
}

// One colour phase: thread (u, v, w) projects row (a + 3u, b + 3v, c + 3w) for every active
// right-hand side.
template <typename T, bool ADJ, bool WNC>
__global__ void __launch_bounds__(128) sweep_direct_kernel(Op<T> op, cplx<T> *x, const cplx<T> *b, int nrhs,
                                                           T w, const int *active, const T *rinv,
                                                           const cplx<T> *coef, ColourGrid g)
{
    const int u = blockIdx.x * blockDim.x + threadIdx.x, v = blockIdx.y, wq = blockIdx.z;
    if (u >= g.nu) return;
    const int i = g.a + 3 * u, j = g.b + 3 * v, k = g.c + 3 * wq;
    const long long ctr = i + op.sy * j + op.sz * k;
    const int *ilo = ADJ ? op.int_lo_a : op.int_lo_f, *ihi = ADJ ? op.int_hi_a : op.int_hi_f;
    const bool interior =
        !WNC && i >= ilo[0] && i < ihi[0] && j >= ilo[1] && j < ihi[1] && k >= ilo[2] && k < ihi[2];
    // rows on the grid's faces have neighbours outside: those read as zero and are not stored
    const bool edge = i == 0 || j == 0 || k == 0 || i == op.nx - 1 || j == op.ny - 1 || k == op.nz - 1;
    const uint32_t m = edge ? inside_mask(i, j, k, op.nx, op.ny, op.nz) : 0x7ffffffu;
    const T inv = rinv[ctr];

    cplx<T> c[27];
    if (interior) {
        // K_t - WM_t wn (forward: wn of the neighbour; adjoint: of the row)
#define H3D_DI(t, dx, dy, dz)                                                                  \
    {                                                                                          \
        constexpr int nzc = (dx != 0) + (dy != 0) + (dz != 0);                                 \
        constexpr int cls = nzc == 0 ? 0 : nzc == 3 ? 7 : nzc == 1 ? (dx ? 1 : dy ? 2 : 3) : (!dz ? 4 : !dy ? 5 : 6); \
        const T wv = ADJ ? op.wn[ctr] : op.wn[ctr + dx + op.sy * dy + op.sz * dz];             \
        c[t].re = (t == 13) ? op.wn_c * wv + op.kint[0] : op.kint[cls] - T(WM<dx, dy, dz>::value) * wv; \
        c[t].im = T(0);                                                                        \
    }
        H3D_FOR_27(H3D_DI)
#undef H3D_DI
    } else {
        const cplx<T> *src = coef + g.base + u + (long long)g.nu * (v + (long long)g.nv * wq);
#pragma unroll
        for (int t = 0; t < 27; ++t) c[t] = src[t * g.M];
    }

    for (int s = 0; s < nrhs; ++s) {
        if (active && !active[s]) continue;
        cplx<T> *xs = x + (long long)s * op.N + ctr;
        cplx<T> xv[27];
#define H3D_DG(t, dx, dy, dz) xv[t] = (m >> t) & 1u ? xs[dx + op.sy * dy + op.sz * dz] : mk<T>(T(0), T(0));
        H3D_FOR_27(H3D_DG)
#undef H3D_DG
        // one partial sum per plane dz, each in offset order
        const cplx<T> z = mk<T>(T(0), T(0));
        CSum<T> acc[3] = {csum_init(z), csum_init(z), csum_init(z)};
#pragma unroll
        for (int t = 0; t < 27; ++t) csum_mac(acc[t / 9], c[t], xv[t]);
        const cplx<T> atx = cadd(cadd(csum_value(acc[0]), csum_value(acc[1])), csum_value(acc[2]));
        const cplx<T> bv = b ? b[(long long)s * op.N + ctr] : mk<T>(T(0), T(0));
        const Scat<T> sd = scat_of((w * inv) * (bv - atx));
#define H3D_DS(t, dx, dy, dz)                                                                  \
    if ((m >> t) & 1u) {                                                                       \
        cplx<T> o = xv[t];                                                                     \
        scat_mac(o, sd, c[t]);                                                                 \
        xs[dx + op.sy * dy + op.sz * dz] = o;                                                  \
    }
        H3D_FOR_27(H3D_DS)
#undef H3D_DS
    }
}

template <typename T, bool ADJ, bool WNC>
static int direct_pass(const Op<T> &op, cplx<T> *x, const cplx<T> *b, int nrhs, T w, const int *active,
                       const T *rinv, const cplx<T> *coef, bool backward, cudaStream_t st)
{
    for (int qq = 0; qq < 27; ++qq) {
        const int q = backward ? 26 - qq : qq;
        const ColourGrid g = colour_grid(op.nx, op.ny, op.nz, q);
        if (g.M == 0) continue;
        const dim3 grd((g.nu + 127) / 128, g.nv, g.nw);
        sweep_direct_kernel<T, ADJ, WNC><<<grd, 128, 0, st>>>(op, x, b, nrhs, w, active, rinv, coef, g);
    }
    H3D_CUDA_TRY(cudaGetLastError());
    return H3D_OK;
}

template <typename T>
int sweep_colour_direct(const Op<T> &op, cplx<T> *x, const cplx<T> *b, int nrhs, T w, const int *active,
                        const T *rinv, const cplx<T> *coef, bool adj, cudaStream_t st)
{
    if (op.ny > 3 * 65535 || op.nz > 3 * 65535) {
        set_error("grid too large for the direct COLOUR27 sweep");
        return H3D_ERR_NSIZE;
    }
    const bool wnc = op.wni != nullptr;
    for (int pass = 0; pass < 2; ++pass) {
        const bool bw = pass == 1;
        int rc;
        if (!adj && !wnc) rc = direct_pass<T, false, false>(op, x, b, nrhs, w, active, rinv, coef, bw, st);
        else if (!adj && wnc) rc = direct_pass<T, false, true>(op, x, b, nrhs, w, active, rinv, coef, bw, st);
        else if (adj && !wnc) rc = direct_pass<T, true, false>(op, x, b, nrhs, w, active, rinv, coef, bw, st);
        else rc = direct_pass<T, true, true>(op, x, b, nrhs, w, active, rinv, coef, bw, st);
        if (rc) return rc;
    }
    return H3D_OK;
}

template int store_row_coefs<double>(const Op<double> &, bool, cplx<double> *, cudaStream_t);
template int store_row_coefs<float>(const Op<float> &, bool, cplx<float> *, cudaStream_t);
template int sweep_colour_direct<double>(const Op<double> &, cplx<double> *, const cplx<double> *, int, double,
                                         const int *, const double *, const cplx<double> *, bool, cudaStream_t);
template int sweep_colour_direct<float>(const Op<float> &, cplx<float> *, const cplx<float> *, int, float,
                                        const int *, const float *, const cplx<float> *, bool, cudaStream_t);

}  // namespace h3d
