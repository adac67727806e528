// Batched BLOCK8 Kaczmarz double sweep: one launch per block parity over a table of problems
// of any sizes, the stored coefficients of each colour staged by bulk copies into a ring of
// shared-memory buffers that complete on mbarriers.
//
// Row order and arithmetic are those of the BLOCK8 sweep (h3d_block8.cu, h3d_blockrow.cuh):
// 12^3 blocks in eight parity classes, 27 colours inside a block, forward then backward
// (Helm3dkaczswp_mex.c:60-120 with another row order).  What changes is how work and data
// reach a CTA:
//
//  * Work list.  A launch of parity p runs sum over problems of (blocks of parity p) x
//    (groups of R right-hand sides) CTAs, problem-major, block-major, group fastest (the CTAs
//    of one block sit side by side and share its coefficient slabs through L2).  A CTA finds
//    its problem by a binary search over the per-parity prefix counts.
//  * Staging.  Thread 0 issues, per colour step, one cp.async.bulk of the colour's 13.8 KB
//    coefficient slab (complex64; 27.6 KB complex128) and one of its 64 inverse row norms,
//    both completing on the step's mbarrier, S steps ahead into an S-deep ring; no other
//    thread spends instructions on the copies.  Interior blocks (all PML values 1, real
//    wavenumber) form their real coefficients from the staged wavenumber box instead and
//    fetch only the row norms; the wavenumber box shares its space with the ring.
//  * Bounded waits.  Every mbarrier wait gives up after wait_limit_ns (globaltimer); the CTA
//    then records H3D_ERR_TIMEOUT in the status word, waits (bounded again) for the copies
//    it still has in flight, and returns without writing its box back.  The host reads the
//    status word and fails the call; the context stays usable.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>

#include "h3d_b8.cuh"
#include "h3d_blockrow.cuh"
#include "h3d_kernels.cuh"

namespace h3d {

namespace {

constexpr int kBS = 12;                 // block side
constexpr int kNR = 64;                 // rows per colour and block (4 x 4 x 4)
constexpr int kPX = kBS + 2, kPY = kBS + 2;
constexpr int kNB = kPX * kPY * (kBS + 2);  // halo'd box points

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"(bytes) : "memory");
}

// Global -> shared bulk copy (16-byte aligned ends, size a multiple of 16) completing on bar.
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Wait for the completion of the phase with the given parity; false after limit_ns.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, unsigned long long limit_ns)
{
    if (mbar_try(bar, parity)) return true;
    const unsigned long long t0 = global_ns();
    for (;;) {
        if (mbar_try(bar, parity)) return true;
        if (global_ns() - t0 > limit_ns) return false;
    }
}

template <typename T>
constexpr uint32_t slab_bytes() { return 27u * kNR * sizeof(cplx<T>); }
template <typename T>
constexpr uint32_t rinv_bytes() { return kNR * sizeof(T); }
template <typename T, int S>
constexpr size_t ring_bytes()
{
    return std::max((size_t)kNB * sizeof(T), (size_t)S * slab_bytes<T>());
}
// [S mbarriers, padded to 128 B] [R x-boxes] [ring, or the wavenumber box] [S row-norm buffers]
template <typename T, int R, int S>
constexpr size_t b8_smem() { return 128 + (size_t)R * kNB * sizeof(cplx<T>) + ring_bytes<T, S>() + S * rinv_bytes<T>(); }

// selftest != 0 (h3d_check_wait_timeout only): the first step's copies are announced on its
// mbarrier but never issued, so that every wait of the first colour step expires.
//
// R right-hand sides per CTA; each thread projects one row of every colour for RPT of them,
// from one load of the row's coefficients (64 R / RPT threads).
template <typename T, int R, int RPT, int S>
__global__ void __launch_bounds__(kNR *R / RPT) sweep_b8_kernel(const B8Prob<T> *__restrict__ probs,
                                                                const int *__restrict__ starts, int nprob, cplx<T> *x,
                                                                const cplx<T> *b, T w, const int *active, int par,
                                                                int backward, int nsteps, int *err,
                                                                unsigned long long limit_ns, int selftest)
{
    static_assert(R % RPT == 0, "RPT must divide R");
    constexpr int NT = kNR * R / RPT, SLAB = 27 * kNR;
    constexpr uint32_t SLABB = slab_bytes<T>(), RVB = rinv_bytes<T>();
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ B8Prob<T> sp;
    __shared__ int s_pi;
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem);
    cplx<T> *sx = reinterpret_cast<cplx<T> *>(smem + 128);
    unsigned char *ring = smem + 128 + (size_t)R * kNB * sizeof(cplx<T>);
    T *rv = reinterpret_cast<T *>(ring + ring_bytes<T, S>());
    const int tid = threadIdx.x;

    const int *st0 = starts + par * (nprob + 1);
    if (tid == 0) {  // the problem whose CTA range holds this CTA
        int lo = 0, hi = nprob - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (st0[mid] <= (int)blockIdx.x) lo = mid;
            else hi = mid - 1;
        }
        s_pi = lo;
    }
    __syncthreads();
    {
        const int *src = reinterpret_cast<const int *>(probs + s_pi);
        int *dst = reinterpret_cast<int *>(&sp);
        for (int e = tid; e < (int)(sizeof(B8Prob<T>) / sizeof(int)); e += NT) dst[e] = src[e];
    }
    __syncthreads();
    const Op<T> &op = sp.op;
    const int local = (int)blockIdx.x - st0[s_pi];
    const int blk = local / sp.ngrp, grp = local - blk * sp.ngrp;
    const int nI = (sp.NI - (par & 1) + 1) >> 1, nJ = (sp.NJ - ((par >> 1) & 1) + 1) >> 1;
    const int Ib = (par & 1) + 2 * (blk % nI);
    const int Jb = ((par >> 1) & 1) + 2 * ((blk / nI) % nJ);
    const int Kb = (par >> 2) + 2 * (blk / (nI * nJ));
    const int bi0 = Ib * kBS, bj0 = Jb * kBS, bk0 = Kb * kBS;
    const int s0 = grp * R;
    unsigned act = 0;  // bit r: column s0 + r of the problem takes part
#pragma unroll
    for (int r = 0; r < R; ++r)
        if (s0 + r < sp.nrhs && (!active || active[sp.c0 + s0 + r])) act |= 1u << r;
    if (!act) return;  // uniform over the CTA, before any barrier or copy

    const int *ilo = sp.adj ? op.int_lo_a : op.int_lo_f, *ihi = sp.adj ? op.int_hi_a : op.int_hi_f;
    const bool interior = !sp.wnc && bi0 >= ilo[0] && min(bi0 + kBS, op.nx) <= ihi[0] && bj0 >= ilo[1] &&
                          min(bj0 + kBS, op.ny) <= ihi[1] && bk0 >= ilo[2] && min(bk0 + kBS, op.nz) <= ihi[2];
    const bool edge_block = bi0 == 0 || bj0 == 0 || bk0 == 0 || bi0 + kBS >= op.nx || bj0 + kBS >= op.ny ||
                            bk0 + kBS >= op.nz;
    const long long bid = Ib + (long long)sp.NI * (Jb + (long long)sp.NJ * Kb);
    const cplx<T> *slab0 = sp.coef + bid * 27 * SLAB;
    const T *rv0 = sp.rinv8 + bid * 27 * kNR;
    auto colour_of = [&](int st) { return st < 27 ? (backward ? 26 - st : st) : 53 - st; };
    auto issue = [&](int st) {  // thread 0: step st's slab and row norms -> ring buffer st % S
        const int q = colour_of(st), buf = st % S;
        const uint32_t bar = smem_u32(bars + buf);
        mbar_expect_tx(bar, (interior ? 0u : SLABB) + RVB);
        if (selftest && st == 0) return;
        if (!interior) bulk_g2s(smem_u32(ring + (size_t)buf * SLABB), slab0 + (size_t)q * SLAB, SLABB, bar);
        bulk_g2s(smem_u32(rv + buf * kNR), rv0 + q * kNR, RVB, bar);
    };

    if (tid == 0) {
#pragma unroll
        for (int s = 0; s < S; ++s) mbar_init(smem_u32(bars + s), 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();
    if (tid == 0)
        for (int st = 0; st < S && st < nsteps; ++st) issue(st);

    // the halo'd boxes of x (and the wavenumber box of an interior block), zero outside the grid,
    // one box row (14 points along x) at a time.  One right-hand side: a thread per row, its 14
    // points unrolled (fewest instructions; the 64 threads have 196 rows to copy).  Several: a
    // half-warp per row, lane l on point l (the copies of a warp stay contiguous).
    const int i0 = bi0 - 1, j0 = bj0 - 1, k0 = bk0 - 1;
    constexpr int kRows = kPY * (kBS + 2);
    T *swr = reinterpret_cast<T *>(ring);
    const int li_lo = max(0, -i0), li_hi = min(kPX, op.nx - i0);  // box columns inside the grid
    if constexpr (R == 1) {
        for (int rw = tid; rw < kRows; rw += NT) {
            const int lj = rw % kPY, lk = rw / kPY;
            const int gj = j0 + lj, gk = k0 + lk;
            const bool rin = gj >= 0 && gj < op.ny && gk >= 0 && gk < op.nz;
            const long long g0 = rin ? (long long)i0 + op.sy * gj + op.sz * gk : 0;
            const cplx<T> *xr = x + sp.col0 + s0 * sp.cstride + g0;
#pragma unroll
            for (int li = 0; li < kPX; ++li) {
                const bool in = rin && li >= li_lo && li < li_hi;
                if (interior) blk_cp_async<sizeof(T)>(swr + rw * kPX + li, op.wn + (in ? g0 + li : 0), in);
                blk_cp_async<sizeof(cplx<T>)>(sx + rw * kPX + li, in ? xr + li : x, in);
            }
        }
    } else {
        constexpr int kSlots = NT / 16;
        const int li = tid & 15, slot = tid >> 4;
        const bool lin = li >= li_lo && li < li_hi;
        const cplx<T> *xcol = x + sp.col0 + s0 * sp.cstride;
        for (int rw = slot; rw < kRows; rw += kSlots) {
            if (li >= kPX) continue;
            const int lj = rw % kPY, lk = rw / kPY;
            const int gj = j0 + lj, gk = k0 + lk;
            const bool in = lin && gj >= 0 && gj < op.ny && gk >= 0 && gk < op.nz;
            const long long g = in ? (long long)(i0 + li) + op.sy * gj + op.sz * gk : 0;
            const int e = rw * kPX + li;
            if (interior) blk_cp_async<sizeof(T)>(swr + e, op.wn + g, in);
#pragma unroll
            for (int r = 0; r < R; ++r)
                if (act & (1u << r))
                    blk_cp_async<sizeof(cplx<T>)>(sx + (size_t)r * kNB + e, xcol + r * sp.cstride + g, in);
        }
    }
    blk_cp_async_wait_all();
    __syncthreads();

    // thread slot: row (u, v, w) of every colour, right-hand sides s0 + r0 .. s0 + r0 + RPT - 1
    // (a half-warp spans (u, w): conflict-free box offsets, as the BLOCK8 kernel)
    const int r0 = (tid / kNR) * RPT, row = tid % kNR;
    const int u = row % 4, ww = (row / 4) % 4, v = row / 16;
    const unsigned mine = (act >> r0) & ((1u << RPT) - 1u);
    cplx<T> bv_n[RPT];
#pragma unroll
    for (int kk = 0; kk < RPT; ++kk) bv_n[kk] = mk<T>(T(0), T(0));
    auto fetch_b = [&](int q) {  // b_i of the next colour's row, one step ahead
        const int i = bi0 + q % 3 + 3 * u, j = bj0 + (q / 3) % 3 + 3 * v, k = bk0 + q / 9 + 3 * ww;
        if (i < op.nx && j < op.ny && k < op.nz) {
            const long long ctr = i + op.sy * j + op.sz * k;
#pragma unroll
            for (int kk = 0; kk < RPT; ++kk)
                if (mine & (1u << kk)) bv_n[kk] = b[sp.col0 + (s0 + r0 + kk) * sp.cstride + ctr];
        }
    };
    if (b) fetch_b(colour_of(0));
    for (int qq = 0; qq < nsteps; ++qq) {
        const int q = colour_of(qq), buf = qq % S;
        cplx<T> bv[RPT];
#pragma unroll
        for (int kk = 0; kk < RPT; ++kk) bv[kk] = bv_n[kk];
        if (b && qq + 1 < nsteps) fetch_b(colour_of(qq + 1));
        const bool ok = mbar_wait(smem_u32(bars + buf), (uint32_t)((qq / S) & 1), limit_ns);
        const int a = q % 3, bq = (q / 3) % 3, cq = q / 9;
        const int i = bi0 + a + 3 * u, j = bj0 + bq + 3 * v, k = bk0 + cq + 3 * ww;
        if (ok && mine && i < op.nx && j < op.ny && k < op.nz) {
            const T inv = rv[buf * kNR + row];
            const int lc = (1 + a + 3 * u) + kPX * ((1 + bq + 3 * v) + kPY * (1 + cq + 3 * ww));
            if (!interior) {
                const cplx<T> *sc = reinterpret_cast<const cplx<T> *>(ring + (size_t)buf * SLABB);
                cplx<T> c[27];
#pragma unroll
                for (int t = 0; t < 27; ++t) c[t] = sc[t * kNR + row];
                // neighbours outside the grid keep reading zero: a row on a face of the grid
                // scatters to its inside neighbours only
                uint32_t m = 0x7ffffffu;
                if (edge_block && (i == 0 || j == 0 || k == 0 || i == op.nx - 1 || j == op.ny - 1 || k == op.nz - 1))
                    m = inside_mask(i, j, k, op.nx, op.ny, op.nz);
#pragma unroll
                for (int kk = 0; kk < RPT; ++kk)
                    if (mine & (1u << kk))
                        row_project_c<T, kPX, kPY>(sx + (size_t)(r0 + kk) * kNB, c, m, bv[kk], inv, w, lc);
            } else {
                T cr[27];
                if (sp.adj) interior_coefs<T, true, kPX, kPY>(op, swr, lc, cr);
                else interior_coefs<T, false, kPX, kPY>(op, swr, lc, cr);
#pragma unroll
                for (int kk = 0; kk < RPT; ++kk)
                    if (mine & (1u << kk)) row_project_r<T, kPX, kPY>(sx + (size_t)(r0 + kk) * kNB, cr, bv[kk], inv, w, lc);
            }
        }
        if (__syncthreads_or(!ok)) {
            // a wait expired: report it, let the copies still in flight land, leave x alone
            if (tid == 0) {
                atomicCAS(err, 0, (int)H3D_ERR_TIMEOUT);
                for (int st = qq; st < qq + S && st < nsteps; ++st)
                    if (!(selftest && st == 0)) (void)mbar_wait(smem_u32(bars + st % S), (uint32_t)((st / S) & 1), limit_ns);
            }
            __syncthreads();
            return;
        }
        if (tid == 0 && qq + S < nsteps) issue(qq + S);  // the buffer this step used is free
    }
    // write the box back (halo included), points inside the grid only, as staged
    cplx<T> *xw = x + sp.col0 + s0 * sp.cstride;
    if constexpr (R == 1) {
        for (int rw = tid; rw < kRows; rw += NT) {
            const int lj = rw % kPY, lk = rw / kPY;
            const int gj = j0 + lj, gk = k0 + lk;
            if (gj < 0 || gj >= op.ny || gk < 0 || gk >= op.nz) continue;
            cplx<T> *xr = xw + (long long)i0 + op.sy * gj + op.sz * gk;
#pragma unroll
            for (int li = 0; li < kPX; ++li)
                if (li >= li_lo && li < li_hi) xr[li] = sx[rw * kPX + li];
        }
    } else {
        constexpr int kSlots = NT / 16;
        const int li = tid & 15, slot = tid >> 4;
        if (li < kPX && li >= li_lo && li < li_hi) {
            for (int rw = slot; rw < kRows; rw += kSlots) {
                const int lj = rw % kPY, lk = rw / kPY;
                const int gj = j0 + lj, gk = k0 + lk;
                if (gj < 0 || gj >= op.ny || gk < 0 || gk >= op.nz) continue;
                const long long g = (long long)(i0 + li) + op.sy * gj + op.sz * gk;
                const int e = rw * kPX + li;
#pragma unroll
                for (int rr = 0; rr < R; ++rr)
                    if (act & (1u << rr)) xw[rr * sp.cstride + g] = sx[(size_t)rr * kNB + e];
            }
        }
    }
}

// 1/||a_i||^2 from the grid layout into the block- and colour-major layout of the slabs
// (0 for the slots of rows outside the grid).
template <typename T>
__global__ void rinv8_kernel(const T *__restrict__ rinv, T *__restrict__ rinv8, int nx, int ny, int nz,
                             long long sy, long long sz, int NI, int NJ, long long nslab)
{
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= nslab * kNR) return;
    const long long bq = e / kNR;
    const int row = (int)(e % kNR);
    const long long bid = bq / 27;
    const int q = (int)(bq % 27);
    const int Ib = (int)(bid % NI), Jb = (int)((bid / NI) % NJ), Kb = (int)(bid / ((long long)NI * NJ));
    const int u = row % 4, w = (row / 4) % 4, v = row / 16;
    const int i = Ib * kBS + q % 3 + 3 * u, j = Jb * kBS + (q / 3) % 3 + 3 * v, k = Kb * kBS + q / 9 + 3 * w;
    rinv8[e] = (i < nx && j < ny && k < nz) ? rinv[i + sy * j + sz * k] : T(0);
}

// Compiled configurations (R right-hand sides per CTA, RPT per thread, ring depth S):
// complex64 with a 3-deep ring; complex128 with a 2-deep ring (its R = 4 boxes would exceed a
// CTA's 227 KB of shared memory).
const B8Cfg kCfgF32[] = {{1, 1, 3}, {2, 1, 3}, {4, 1, 3}, {4, 2, 3}, {8, 1, 3}, {8, 2, 3}};
const B8Cfg kCfgF64[] = {{1, 1, 2}, {2, 1, 2}, {2, 2, 2}};

template <typename T, int R, int RPT, int S>
int launch_b8(const B8Prob<T> *probs, const int *starts, int nprob, long long nctas, cplx<T> *x, const cplx<T> *b,
              T w, const int *active, int par, int backward, int nsteps, int *err, unsigned long long limit_ns,
              int selftest, cudaStream_t st)
{
    constexpr size_t smem = b8_smem<T, R, S>();
    static_assert(smem + sizeof(B8Prob<T>) + 16 <= 232448, "batched BLOCK8 configuration exceeds shared memory");
    static bool attr_set = false;  // per instantiation and process
    if (!attr_set) {
        H3D_CUDA_TRY(cudaFuncSetAttribute(sweep_b8_kernel<T, R, RPT, S>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)smem));
        attr_set = true;
    }
    sweep_b8_kernel<T, R, RPT, S><<<(unsigned)nctas, kNR * R / RPT, smem, st>>>(
        probs, starts, nprob, x, b, w, active, par, backward, nsteps, err, limit_ns, selftest);
    return H3D_OK;
}

template <typename T>
int launch_b8_cfg(int cfg, const B8Prob<T> *probs, const int *starts, int nprob, long long nctas, cplx<T> *x,
                  const cplx<T> *b, T w, const int *active, int par, int backward, int nsteps, int *err,
                  unsigned long long limit_ns, int selftest, cudaStream_t st)
{
#define H3D_B8_ARGS probs, starts, nprob, nctas, x, b, w, active, par, backward, nsteps, err, limit_ns, selftest, st
    if constexpr (sizeof(T) == 4) {
        switch (cfg) {
        case 0: return launch_b8<T, 1, 1, 3>(H3D_B8_ARGS);
        case 1: return launch_b8<T, 2, 1, 3>(H3D_B8_ARGS);
        case 2: return launch_b8<T, 4, 1, 3>(H3D_B8_ARGS);
        case 3: return launch_b8<T, 4, 2, 3>(H3D_B8_ARGS);
        case 4: return launch_b8<T, 8, 1, 3>(H3D_B8_ARGS);
        case 5: return launch_b8<T, 8, 2, 3>(H3D_B8_ARGS);
        default: break;
        }
    } else {
        switch (cfg) {
        case 0: return launch_b8<T, 1, 1, 2>(H3D_B8_ARGS);
        case 1: return launch_b8<T, 2, 1, 2>(H3D_B8_ARGS);
        case 2: return launch_b8<T, 2, 2, 2>(H3D_B8_ARGS);
        default: break;
        }
    }
#undef H3D_B8_ARGS
    set_error("batched BLOCK8 configuration %d out of range", cfg);
    return H3D_ERR_BAD_ARG;
}

// Tuner cache: batch shape (grid sizes, columns, precision) -> configuration.
std::mutex g_b8_mutex;
std::map<std::vector<long long>, int> g_b8_cache;

}  // namespace

int b8_num_cfgs(bool fp64) { return fp64 ? (int)(sizeof(kCfgF64) / sizeof(B8Cfg)) : (int)(sizeof(kCfgF32) / sizeof(B8Cfg)); }
B8Cfg b8_cfg(bool fp64, int c) { return fp64 ? kCfgF64[c] : kCfgF32[c]; }

template <typename T>
static void block_counts(const Op<T> &op, int *NI, int *NJ, int *NK)
{
    *NI = (op.nx + kBS - 1) / kBS;
    *NJ = (op.ny + kBS - 1) / kBS;
    *NK = (op.nz + kBS - 1) / kBS;
}

template <typename T>
size_t B8Batch<T>::bytes_needed() const
{
    size_t tot = 0;
    for (const Item &it : items) {
        int NI, NJ, NK;
        block_counts(it.op, &NI, &NJ, &NK);
        const size_t nslab = (size_t)NI * NJ * NK * 27;
        tot += nslab * 27 * kNR * sizeof(cplx<T>) + nslab * kNR * sizeof(T) + (size_t)it.op.N * sizeof(T);
    }
    return tot;
}

template <typename T>
int B8Batch<T>::setup(cudaStream_t st)
{
    int rc;
    if (items.empty()) {
        set_error("batched BLOCK8 sweep without problems");
        return H3D_ERR_BAD_ARG;
    }
    coefs.clear();
    rinvs.clear();
    for (const Item &it : items) {
        int NI, NJ, NK;
        block_counts(it.op, &NI, &NJ, &NK);
        const long long nslab = (long long)NI * NJ * NK * 27;
        if (nslab * kNR > 0x7fffffffLL * 64LL) {
            set_error("grid too large for the batched BLOCK8 sweep");
            return H3D_ERR_NSIZE;
        }
        auto cb = std::make_unique<DevBuf>();
        auto rb = std::make_unique<DevBuf>();
        if ((rc = cb->alloc(sizeof(cplx<T>) * block8_coef_count(it.op.nx, it.op.ny, it.op.nz), st))) return rc;
        if ((rc = rb->alloc(sizeof(T) * (size_t)nslab * kNR, st))) return rc;
        if ((rc = store_block8_coefs<T>(it.op, it.adj, cb->as<cplx<T>>(), st))) return rc;
        DevBuf grid_rinv;
        if ((rc = grid_rinv.alloc(sizeof(T) * (size_t)it.op.N, st))) return rc;
        if ((rc = row_inv_norms<T>(it.op, it.adj, grid_rinv.as<T>(), st))) return rc;
        const long long n = nslab * kNR;
        rinv8_kernel<T><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(grid_rinv.as<T>(), rb->as<T>(), it.op.nx, it.op.ny,
                                                                       it.op.nz, it.op.sy, it.op.sz, NI, NJ, nslab);
        H3D_CUDA_TRY(cudaGetLastError());
        coefs.push_back(std::move(cb));
        rinvs.push_back(std::move(rb));
    }
    if (!errb.p && (rc = errb.alloc(sizeof(int), st))) return rc;
    err = errb.as<int>();
    H3D_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), st));
    return H3D_OK;
}

template <typename T>
int B8Batch<T>::configure(int c, cudaStream_t st)
{
    const bool fp64 = sizeof(T) == 8;
    if (c < 0 || c >= b8_num_cfgs(fp64)) {
        set_error("batched BLOCK8 configuration %d out of range", c);
        return H3D_ERR_BAD_ARG;
    }
    const int R = b8_cfg(fp64, c).r;
    const int np = (int)items.size();
    std::vector<B8Prob<T>> h(np);
    std::vector<int> hs(8 * (np + 1), 0);
    long long tot[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int i = 0; i < np; ++i) {
        const Item &it = items[i];
        B8Prob<T> &d = h[i];
        std::memset(&d, 0, sizeof d);
        d.op = it.op;
        d.coef = coefs[i]->as<cplx<T>>();
        d.rinv8 = rinvs[i]->as<T>();
        d.col0 = it.col0;
        d.cstride = it.op.N;
        d.c0 = it.c0;
        d.nrhs = it.nrhs;
        d.ngrp = (it.nrhs + R - 1) / R;
        d.adj = it.adj ? 1 : 0;
        d.wnc = it.op.wni != nullptr;
        block_counts(it.op, &d.NI, &d.NJ, &d.NK);
        for (int p = 0; p < 8; ++p) {
            const long long nI = (d.NI - (p & 1) + 1) / 2, nJ = (d.NJ - ((p >> 1) & 1) + 1) / 2,
                            nK = (d.NK - (p >> 2) + 1) / 2;
            hs[p * (np + 1) + i] = (int)tot[p];
            tot[p] += nI * nJ * nK * d.ngrp;
        }
    }
    for (int p = 0; p < 8; ++p) {
        if (tot[p] > 0x7fffffffLL) {
            set_error("batched BLOCK8 launch too large (%lld CTAs)", tot[p]);
            return H3D_ERR_BAD_ARG;
        }
        hs[p * (np + 1) + np] = (int)tot[p];
        nctas[p] = tot[p];
    }
    int rc;
    desc.release();
    starts.release();
    if ((rc = desc.alloc(sizeof(B8Prob<T>) * np, st)) || (rc = starts.alloc(sizeof(int) * hs.size(), st))) return rc;
    // pageable sources: staged before the calls return
    H3D_CUDA_TRY(cudaMemcpyAsync(desc.p, h.data(), sizeof(B8Prob<T>) * np, cudaMemcpyHostToDevice, st));
    H3D_CUDA_TRY(cudaMemcpyAsync(starts.p, hs.data(), sizeof(int) * hs.size(), cudaMemcpyHostToDevice, st));
    cfg = c;
    return H3D_OK;
}

template <typename T>
int B8Batch<T>::launches() const
{
    int n = 0;
    for (int pp = 0; pp < 15; ++pp) n += nctas[pp < 8 ? pp : 14 - pp] > 0;
    return n;
}

template <typename T>
int B8Batch<T>::dsweep(cplx<T> *x, const cplx<T> *b, T w, const int *active, cudaStream_t st, int selftest)
{
    if (cfg < 0) {
        set_error("batched BLOCK8 sweep used before configure()");
        return H3D_ERR_BAD_ARG;
    }
    const int np = (int)items.size();
    // forward parities 0..6, parity 7 up and down in one launch, backward parities 6..0
    for (int pp = 0; pp < 15; ++pp) {
        const int par = pp < 8 ? pp : 14 - pp;
        if (!nctas[par]) continue;
        int rc = launch_b8_cfg<T>(cfg, desc.as<B8Prob<T>>(), starts.as<int>(), np, nctas[par], x, b, w, active, par,
                                  pp < 8 ? 0 : 1, pp == 7 ? 54 : 27, err, wait_limit_ns, selftest, st);
        if (rc) return rc;
    }
    H3D_CUDA_TRY(cudaGetLastError());
    return H3D_OK;
}

template <typename T>
int B8Batch<T>::max_nrhs() const
{
    int m = 0;
    for (const Item &it : items) m = std::max(m, it.nrhs);
    return m;
}

template <typename T>
int B8Batch<T>::tune(cplx<T> *y, long long len, cudaStream_t st)
{
    const bool fp64 = sizeof(T) == 8;
    std::vector<long long> key{(long long)sizeof(T)};
    for (const Item &it : items) {
        key.push_back(it.op.nx);
        key.push_back(it.op.ny);
        key.push_back(it.op.nz);
        key.push_back(it.nrhs);
        key.push_back(it.adj);
    }
    {
        std::lock_guard<std::mutex> lk(g_b8_mutex);
        auto f = g_b8_cache.find(key);
        if (f != g_b8_cache.end()) return configure(f->second, st);
    }
    const int mx = max_nrhs();
    int best = -1;
    float best_ms = 1e30f;
    cudaEvent_t e0, e1;
    H3D_CUDA_TRY(cudaEventCreate(&e0));
    H3D_CUDA_TRY(cudaEventCreate(&e1));
    int rc = H3D_OK;
    for (int c = 0; c < b8_num_cfgs(fp64) && !rc; ++c) {
        if (c > 0 && b8_cfg(fp64, c).r > mx) break;  // only groups the columns fill
        if ((rc = configure(c, st))) break;
        H3D_CUDA_TRY(cudaMemsetAsync(y, 0, sizeof(cplx<T>) * (size_t)len, st));
        if ((rc = dsweep(y, nullptr, T(1.5), nullptr, st))) break;  // warm-up
        cudaEventRecord(e0, st);
        for (int rep = 0; rep < 2 && !rc; ++rep) rc = dsweep(y, nullptr, T(1.5), nullptr, st);
        cudaEventRecord(e1, st);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (verbose) fprintf(stderr, "[h3d] tune batched BLOCK8 R=%d: %.3f ms per double sweep\n", b8_cfg(fp64, c).r, 0.5 * ms);
        if (ms < best_ms) {
            best_ms = ms;
            best = c;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    {
        std::lock_guard<std::mutex> lk(g_b8_mutex);
        g_b8_cache[key] = best;
    }
    return configure(best, st);
}

template struct B8Batch<float>;
template struct B8Batch<double>;

}  // namespace h3d
