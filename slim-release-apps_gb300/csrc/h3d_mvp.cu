// Matrix-free matvec y = H x (and H^H x, dH x, dH^H x) as a z-marching stencil.
//
// A CTA owns a 32 x 8 column of rows and marches a chunk of planes in z.  Each plane of
// x (and, forward, of the wavenumber) is staged in shared memory with its one-point xy
// halo by asynchronous copies (double-buffered: plane p+1 streams in while plane p is
// used).  From a plane every thread forms the partial sums of its 3 x 3 in-plane
// neighbourhood that the stencil needs -- centre, the two x-faces, the two y-faces and
// the corner pairs grouped by the sign of dx and of dy -- and keeps the last three planes
// in registers (a register queue along z).  One output row then combines planes k-1,
// k, k+1 with its own PML values: the 27 coefficients of Helm3d_27pt.h:676-825 regroup
// into 9 complex factors (xi_lo / xi_hi per axis and the per-axis sums S) multiplying
// real-weighted brackets of plane sums, plus the wavenumber (mass) part.  The adjoint
// uses the same algebra with the neighbour-shifted, conjugated PML values and the
// centre wavenumber; the derivative variants keep only the mass part.
//
// The same kernel produces the FP64 residual r = b - A x with per-block partial sums of
// ||r||^2 and ||b||^2 (RESID).
#include "h3d_internal.cuh"
#include "h3d_kernels.cuh"
#include "h3d_reduce.cuh"
#include "h3d_planes.cuh"

namespace h3d {

constexpr int kMX = 32, kMY = 8;                 // CTA columns
constexpr int kPX = kMX + 2, kPY = kMY + 2;      // staged plane with halo
constexpr int kPN = kPX * kPY;

template <int BYTES>
__device__ __forceinline__ void mv_cp_async(void *sdst, const void *gsrc, bool valid)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(sdst);
    const int n = valid ? BYTES : 0;
    if constexpr (BYTES == 16)
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gsrc), "r"(n) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], %2, %3;\n" ::"r"(s), "l"(gsrc), "n"(BYTES), "r"(n) : "memory");
}

// Origin shift of the column tiling along one axis: with tiles of t columns starting at
// -shift, a tile boundary falls on the first row whose forward PML values are all 1 (lo), so
// the interior columns fill whole tiles and take the folded-bracket path.
__host__ __device__ inline int tile_shift(int lo, int hi, int t)
{
    return (lo > 0 && lo < hi && lo % t != 0) ? t - lo % t : 0;
}

template <typename T, bool ADJ, bool DERIV, bool WNC, bool RESID>
__global__ void __launch_bounds__(kMX *kMY) mvp_zmarch_kernel(Op<T> op, const cplx<T> *__restrict__ x,
                                                              cplx<T> *__restrict__ y,
                                                              const cplx<T> *__restrict__ b, int kz,
                                                              int nchunks, double *part)
{
    constexpr bool NEED_WN = !ADJ;  // forward: neighbour wavenumbers; adjoint: centre only
    __shared__ __align__(16) cplx<T> sx[2][kPN];
    __shared__ T swr[NEED_WN ? 2 : 1][NEED_WN ? kPN : 1];
    __shared__ T swi[NEED_WN && WNC ? 2 : 1][NEED_WN && WNC ? kPN : 1];

    const int tid = threadIdx.x + kMX * threadIdx.y;
    const int s = blockIdx.z / nchunks, chunk = blockIdx.z % nchunks;
    const int kb = chunk * kz, ke = min(op.nz, kb + kz);
    const int i0 = blockIdx.x * kMX - tile_shift(op.int_lo_f[0], op.int_hi_f[0], kMX);
    const int j0 = blockIdx.y * kMY - tile_shift(op.int_lo_f[1], op.int_hi_f[1], kMY);
    const int i = i0 + threadIdx.x, j = j0 + threadIdx.y;
    const bool valid = i >= 0 && i < op.nx && j >= 0 && j < op.ny;
    const cplx<T> *xs = x + (long long)s * op.N;

    // Staging: the CTA's halo'd plane has kPN points; thread tid copies points tid and
    // tid + kMX*kMY.  Their in-plane offsets (32-bit: the host refuses nx*ny >= 2^31) and
    // x/y bounds are fixed for the march; per plane only the plane's base pointers change
    // (the same for every thread).  Points outside the grid copy nothing (zero fill) from a
    // valid address: the plane base, or plane 0 for planes outside the grid.
    constexpr int kNT = kMX * kMY;
    constexpr int kSlots = (kPN + kNT - 1) / kNT;
    int goff[kSlots];
    bool gin[kSlots];
#pragma unroll
    for (int q = 0; q < kSlots; ++q) {
        const int e = tid + q * kNT;
        const int li = e % kPX, lj = e / kPX;
        const int gi = i0 - 1 + li, gj = j0 - 1 + lj;
        gin[q] = e < kPN && gi >= 0 && gi < op.nx && gj >= 0 && gj < op.ny;
        goff[q] = gin[q] ? gi + op.nx * gj : 0;
    }
    auto stage = [&](int buf, int pk) {
        const bool kin = pk >= 0 && pk < op.nz;
        const long long zo = kin ? op.sz * pk : 0;
        const cplx<T> *xp = xs + zo;
        const T *wp = op.wn + zo;
        const T *wip = WNC ? op.wni + zo : nullptr;
#pragma unroll
        for (int q = 0; q < kSlots; ++q) {
            const int e = tid + q * kNT;
            if (e < kPN) {
                const bool in = kin && gin[q];
                const int g = in ? goff[q] : 0;
                mv_cp_async<sizeof(cplx<T>)>(&sx[buf][e], xp + g, in);
                if constexpr (NEED_WN) {
                    mv_cp_async<sizeof(T)>(&swr[buf][e], wp + g, in);
                    if constexpr (WNC) mv_cp_async<sizeof(T)>(&swi[buf][e], wip + g, in);
                }
            }
        }
        asm volatile("cp.async.commit_group;\n" ::: "memory");
    };

    RowPml<T> pml{};
    if (valid && !DERIV) pml = load_row_pml<T, ADJ>(op, i, j, 0);
    // Columns whose x and y PML values are all 1 across the CTA (uniform): folded brackets;
    // rows inside the z interior as well: the interior class constants.
    const int *ilo = ADJ ? op.int_lo_a : op.int_lo_f, *ihi = ADJ ? op.int_hi_a : op.int_hi_f;
    const bool xyint = !DERIV && !WNC && i0 >= ilo[0] && i0 + kMX <= ihi[0] && j0 >= ilo[1] &&
                       j0 + kMY <= ihi[1];
    auto zint = [&](int k) { return k >= ilo[2] && k < ihi[2]; };
    const int l = (threadIdx.x + 1) + kPX * (threadIdx.y + 1);
    const long long col = i + op.sy * j;  // the thread's column: row k at col + k sz
    double rr = 0.0, bb = 0.0;

    // One plane pk: add it to the pending rows pk-1 (lo), pk (mid) and pk+1 (hi) and finish
    // row pk-1, whose accumulator then serves row pk+2 (its first plane sets every bracket,
    // so nothing is cleared).  The caller rotates the three accumulators' roles, so no
    // accumulator is ever copied.
    auto step = [&](int pk, RowAcc<T> &lo, RowAcc<T> &mid, RowAcc<T> &hi) {
        const int buf = (pk - (kb - 1)) & 1;
        if (pk + 1 <= ke) {
            stage(buf ^ 1, pk + 1);
            asm volatile("cp.async.wait_group 1;\n" ::: "memory");
        } else {
            asm volatile("cp.async.wait_group 0;\n" ::: "memory");
        }
        __syncthreads();
        {
            const PlaneSums<T> P = plane_sums<T, ADJ, WNC, kPX>(sx[buf], NEED_WN ? swr[buf] : nullptr,
                                                                NEED_WN && WNC ? swi[buf] : nullptr, l);
            if (xyint) {
                if (zint(pk - 1)) acc_plane_xy<2, T, true>(lo, P, op);
                else acc_plane_xy<2, T, false>(lo, P, op);
                if (zint(pk)) acc_plane_xy<1, T, true>(mid, P, op);
                else acc_plane_xy<1, T, false>(mid, P, op);
                if (zint(pk + 1)) acc_plane_xy<0, T, true>(hi, P, op);
                else acc_plane_xy<0, T, false>(hi, P, op);
            } else {
                acc_plane<2, T, DERIV>(lo, P, op);
                acc_plane<1, T, DERIV>(mid, P, op);
                acc_plane<0, T, DERIV>(hi, P, op);
            }
        }
        __syncthreads();
        const int k = pk - 1;  // row completed by this plane
        if (k >= kb && valid) {
            RowPml<T> p = pml;
            if constexpr (!DERIV) {
                // only the z values change along the march
                const cplx<T> *t = op.tab;
                p.Sz = t[op.sum[2] + k + 1];
                if constexpr (!ADJ) {
                    p.Azm = t[op.lo[2] + k + 1];
                    p.Azp = t[op.hi[2] + k + 1];
                } else {
                    p.Azm = t[op.hi[2] + k];
                    p.Azp = t[op.lo[2] + k + 2];
                }
            }
            const long long ctr = col + op.sz * k;
            cplx<T> wc = mk<T>(T(0), T(0));
            if constexpr (ADJ) wc = load_wn<T, WNC>(op, ctr);
            const cplx<T> v = !xyint     ? acc_finish<T, ADJ, DERIV, WNC>(lo, p, wc)
                              : zint(k) ? acc_finish_xy<T, ADJ, true>(lo, p, wc)
                                        : acc_finish_xy<T, ADJ, false>(lo, p, wc);
            if constexpr (RESID) {
                const cplx<T> bv = b[(long long)s * op.N + ctr];
                const cplx<T> r = bv - v;
                y[(long long)s * op.N + ctr] = r;
                rr += (double)cabs2(r);
                bb += (double)cabs2(bv);
            } else {
                y[(long long)s * op.N + ctr] = v;
            }
        }
    };

    RowAcc<T> Q0, Q1, Q2;  // rows pk-1, pk, pk+1 at the top of the loop
    acc_zero(Q0);
    acc_zero(Q1);
    acc_zero(Q2);
    stage(0, kb - 1);
    for (int pk = kb - 1; pk <= ke; pk += 3) {
        step(pk, Q0, Q1, Q2);
        if (pk + 1 <= ke) step(pk + 1, Q1, Q2, Q0);
        if (pk + 2 <= ke) step(pk + 2, Q2, Q0, Q1);
    }
    if constexpr (RESID) {
        const double2 t = block_sum2_r(rr, bb);
        if (tid == 0) {
            const long long G = (long long)gridDim.x * gridDim.y * nchunks;
            const long long blin = blockIdx.x + gridDim.x * (blockIdx.y + (long long)gridDim.y * chunk);
            part[2 * (s * G + blin)] = t.x;
            part[2 * (s * G + blin) + 1] = t.y;
        }
    }
}

// CTAs of the z-march kernel resident on the whole device (occupancy of the forward
// variant of the precision and mode), queried once per device and kept for the process:
// the residual's partial-sum buffer is sized from the same grid as the launch, so the
// answer never changes (a failed query is remembered as "unknown").  make_op primes it,
// outside any stream capture.
template <typename T, bool RESID>
static int zmarch_slots()
{
    static int cache[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        cudaGetLastError();
        return 0;
    }
    if (cache[dev] == 0) {
        int per_sm = 0, sms = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mvp_zmarch_kernel<T, false, false, false, RESID>,
                                                          kMX * kMY, 0) != cudaSuccess ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
            cudaGetLastError();
            per_sm = 0;
        }
        cache[dev] = per_sm * sms > 0 ? per_sm * sms : -1;
    }
    return cache[dev] > 0 ? cache[dev] : 0;
}

void mvp_prime_occupancy()
{
    zmarch_slots<float, false>();
    zmarch_slots<double, false>();
    zmarch_slots<float, true>();
    zmarch_slots<double, true>();
}

// Split of the z axis into marching chunks.  A CTA's time grows with the planes it marches
// (its rows plus the two halo planes), and the launch takes as many rounds of resident CTAs
// as the grid needs: the split minimises rounds x (chunk + 2), which balances the halo
// overhead of short chunks against the partly empty last round of a grid that does not fill
// the device (config 1, 201 x 201 x 101: 5 chunks of 21 planes, 910 CTAs in 3 full rounds
// of 304).  Without an occupancy figure, chunks of 16 planes.
template <typename T, bool RESID>
static dim3 zmarch_grid(const Op<T> &op, int nrhs, int *kz, int *nchunks)
{
    const long long gx = (op.nx + tile_shift(op.int_lo_f[0], op.int_hi_f[0], kMX) + kMX - 1) / kMX;
    const long long gy = (op.ny + tile_shift(op.int_lo_f[1], op.int_hi_f[1], kMY) + kMY - 1) / kMY;
    const int slots = zmarch_slots<T, RESID>();
    int best_kz = op.nz < 32 ? op.nz : 16;
    if (slots > 0) {
        long long best = -1;
        const int nmax = op.nz < 64 ? op.nz : 64;
        for (int n = 1; n <= nmax; ++n) {
            const int k = (op.nz + n - 1) / n;
            const long long ctas = gx * gy * (long long)((op.nz + k - 1) / k) * nrhs;
            const long long cost = ((ctas + slots - 1) / slots) * (k + 2);
            if (best < 0 || cost < best) {
                best = cost;
                best_kz = k;
            }
        }
    }
    *kz = best_kz;
    *nchunks = (op.nz + *kz - 1) / *kz;
    return dim3((unsigned)gx, (unsigned)gy, *nchunks * nrhs);
}

template <typename T, bool RESID>
static int zmarch_dispatch(const Op<T> &op, const cplx<T> *x, cplx<T> *y, const cplx<T> *b, int nrhs,
                           bool adj, bool deriv, double *part, int parts, cudaStream_t st)
{
    if ((long long)op.nx * op.ny >= (1LL << 31)) {
        set_error("a z plane of more than 2^31 - 1 points is not supported by the matvec");
        return H3D_ERR_NSIZE;
    }
    int kz, nch;
    const dim3 grd = zmarch_grid<T, RESID>(op, nrhs, &kz, &nch);
    if ((long long)nch * nrhs > 65535) {
        set_error("too many right-hand sides for one launch");
        return H3D_ERR_BAD_ARG;
    }
    if (RESID && (long long)grd.x * grd.y * nch != parts) {
        // the partial-sum buffer was sized for another grid: refuse rather than overrun it
        set_error("residual: %lld column blocks per right-hand side, buffer sized for %d",
                  (long long)grd.x * grd.y * nch, parts);
        return H3D_ERR_BAD_ARG;
    }
    const dim3 blk(kMX, kMY);
    const bool wnc = op.wni != nullptr;
#define H3D_ZM(A, D, W) mvp_zmarch_kernel<T, A, D, W, RESID><<<grd, blk, 0, st>>>(op, x, y, b, kz, nch, part)
    if (!adj && !deriv && !wnc) H3D_ZM(false, false, false);
    else if (!adj && !deriv && wnc) H3D_ZM(false, false, true);
    else if (!adj && deriv && !wnc) H3D_ZM(false, true, false);
    else if (!adj && deriv && wnc) H3D_ZM(false, true, true);
    else if (adj && !deriv && !wnc) H3D_ZM(true, false, false);
    else if (adj && !deriv && wnc) H3D_ZM(true, false, true);
    else if (adj && deriv && !wnc) H3D_ZM(true, true, false);
    else H3D_ZM(true, true, true);
#undef H3D_ZM
    H3D_CUDA_TRY(cudaGetLastError());
    return H3D_OK;
}

template <typename T>
int launch_mvp(const Op<T> &op, const cplx<T> *x, cplx<T> *y, int nrhs, bool adj, bool deriv,
               cudaStream_t st)
{
    return zmarch_dispatch<T, false>(op, x, y, nullptr, nrhs, adj, deriv, nullptr, 0, st);
}

int mvp_residual_parts(const Op<double> &op, int nrhs)
{
    int kz, nch;
    const dim3 g = zmarch_grid<double, true>(op, nrhs, &kz, &nch);
    return (int)(g.x * g.y * nch);
}

int launch_residual(const Op<double> &op, const cplx<double> *b, const cplx<double> *x, cplx<double> *r,
                    int nrhs, bool adj, double *part, int parts, cudaStream_t st)
{
    return zmarch_dispatch<double, true>(op, x, r, b, nrhs, adj, false, part, parts, st);
}

template int launch_mvp<double>(const Op<double> &, const cplx<double> *, cplx<double> *, int, bool, bool, cudaStream_t);
template int launch_mvp<float>(const Op<float> &, const cplx<float> *, cplx<float> *, int, bool, bool, cudaStream_t);

}  // namespace h3d
