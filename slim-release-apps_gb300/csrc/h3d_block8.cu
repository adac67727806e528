// BLOCK8 row ordering of the Kaczmarz double sweep: blocks in eight parity classes, each
// block resident in shared memory for all 27 of its colours.
//
// The grid is cut into blocks of BX x BY x BZ points (each a multiple of 3).  Block (I,J,K)
// has parity p = I%2 + 2(J%2) + 4(K%2); the forward pass visits p = 0..7, and inside a block
// the 27 colours q = i%3 + 3(j%3) + 9(k%3) in ascending order.  Two blocks of one parity are
// a whole block apart in some axis, so their rows share no column and their halo'd boxes are
// disjoint: each parity is one launch, one CTA per (block, group of R right-hand sides), no
// ordering between CTAs.  The backward pass reverses both levels, so the double sweep is a
// symmetric product of row projections (Helm3dkaczswp_mex.c:60-120 with another row order)
// and stays a valid CGMN preconditioner.
//
// Against the COLOUR27 order (27 grid-wide launches per pass, each re-reading its footprint
// boxes), x and the wavenumber cross HBM/L2 about once per pass (plus the one-point halo),
// and a pass is 8 parity phases (a double sweep 15 launches: the forward pass's last
// parity runs its colours up and back down in one launch).  With block sides divisible by 3
// every colour has the same (BX/3)(BY/3)(BZ/3) rows in a block (fewer at the grid's far
// faces), so thread t owns one fixed (row, right-hand side) slot for all colours: no index
// division in the colour loop.
//
// Stored coefficients (12x12x12 blocks): the 27 coefficients of every row are formed once
// per operator (coef8_store_kernel) and kept block- and colour-major, so the coefficients of
// one colour of one block are one contiguous slab of 27 x 64 values (13.8 KB complex64).
// A block that is not entirely interior copies the next colour's slab into shared memory
// (cp.async, double-buffered) while it projects the current colour, and its rows read their
// coefficients from there instead of forming complex PML expressions; interior blocks keep
// forming their real coefficients from the wavenumber.
#include "h3d_blockrow.cuh"
#include "h3d_kernels.cuh"
#include "h3d_vec.cuh"

namespace h3d {

// Stored-coefficient layout of BXxBYxBZ blocks: slab (block bid, colour q) starts at
// (bid * 27 + q) * 27 * NR; coefficient t of row r = u + U (w + W v) of the slab at
// + t * NR + r (the kernel's thread order).
template <int BX, int BY, int BZ>
struct Coef8Layout {
    static constexpr int U = BX / 3, V = BY / 3, W = BZ / 3, NR = U * V * W;
    static constexpr int SLAB = 27 * NR;  // complex values per (block, colour)
};

template <typename T, bool ADJ, bool WNC, int BX, int BY, int BZ>
__global__ void __launch_bounds__(128) coef8_store_kernel(Op<T> op, cplx<T> *coef, int NI, int NJ)
{
    using L = Coef8Layout<BX, BY, BZ>;
    const int bq = blockIdx.x;  // block * 27 + colour
    const int bid = bq / 27, q = bq % 27;
    const int Ib = bid % NI, Jb = (bid / NI) % NJ, Kb = bid / (NI * NJ);
    const int a = q % 3, b = (q / 3) % 3, c = q / 9;
    for (int row = threadIdx.x; row < L::NR; row += blockDim.x) {
        const int u = row % L::U, w = (row / L::U) % L::W, v = row / (L::U * L::W);
        const int i = Ib * BX + a + 3 * u, j = Jb * BY + b + 3 * v, k = Kb * BZ + c + 3 * w;
        if (i >= op.nx || j >= op.ny || k >= op.nz) continue;
        const uint32_t m = ADJ ? 0x7ffffffu : inside_mask(i, j, k, op.nx, op.ny, op.nz);
        cplx<T> cc[27];
        row_coefs<T, ADJ, false, WNC>(op, i, j, k, m, cc);
        cplx<T> *dst = coef + (size_t)bq * L::SLAB + row;
#pragma unroll
        for (int t = 0; t < 27; ++t) dst[t * L::NR] = cc[t];
    }
}

template <typename T, bool ADJ, bool WNC, int BX, int BY, int BZ, int R>
__global__ void __launch_bounds__((BX / 3) * (BY / 3) * (BZ / 3) * R) sweep_block8_kernel(
    Op<T> op, cplx<T> *x, const cplx<T> *b, int nrhs, T w, const int *active, const T *rinv,
    const cplx<T> *coef, int NI, int NJ, int NIp, int NJp, int par, int backward, int nsteps)
{
    static_assert(BX % 3 == 0 && BY % 3 == 0 && BZ % 3 == 0, "block sides must be multiples of 3");
    constexpr int U = BX / 3, V = BY / 3, W = BZ / 3, NR = U * V * W, NT = NR * R;
    constexpr int SLAB = 27 * NR;
    using G = BlockGeom<BX, BY, BZ>;
    constexpr int PX = G::PX, PY = G::PY, NB = G::NB;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cplx<T> *sx = reinterpret_cast<cplx<T> *>(smem_raw);  // [R][NB]
    T *swr = reinterpret_cast<T *>(sx + (size_t)R * NB);
    T *swi = WNC ? swr + NB : nullptr;
    // [2][SLAB] staged coefficients, after the wavenumber box (16-byte aligned)
    cplx<T> *sc = reinterpret_cast<cplx<T> *>(smem_raw + ((block_smem<T, WNC, BX, BY, BZ, R>() + 15) / 16) * 16);

    const int bid = blockIdx.x;
    const int Ib = (par & 1) + 2 * (bid % NIp);
    const int Jb = ((par >> 1) & 1) + 2 * ((bid / NIp) % NJp);
    const int Kb = (par >> 2) + 2 * (bid / (NIp * NJp));
    const int bi0 = Ib * BX, bj0 = Jb * BY, bk0 = Kb * BZ;
    if (bi0 >= op.nx || bj0 >= op.ny || bk0 >= op.nz) return;  // uniform over the CTA
    const int s0 = blockIdx.y * R;
    if (s0 >= nrhs) return;
    const int i0 = bi0 - 1, j0 = bj0 - 1, k0 = bk0 - 1;  // box origin (halo)

    unsigned act = 0;  // bit r: right-hand side s0 + r takes part
#pragma unroll
    for (int r = 0; r < R; ++r)
        if (s0 + r < nrhs && (!active || active[s0 + r])) act |= 1u << r;
    if (!act) return;

    // every row of the block has PML values of exactly 1 (CTA-uniform)
    const int *ilo = ADJ ? op.int_lo_a : op.int_lo_f, *ihi = ADJ ? op.int_hi_a : op.int_hi_f;
    const bool interior_block = !WNC && bi0 >= ilo[0] && min(bi0 + BX, op.nx) <= ihi[0] && bj0 >= ilo[1] &&
                                min(bj0 + BY, op.ny) <= ihi[1] && bk0 >= ilo[2] && min(bk0 + BZ, op.nz) <= ihi[2];
    const bool stored = coef != nullptr && !interior_block;
    // the block holds a row on a face of the grid (CTA-uniform): its scatter is masked
    const bool edge_block = bi0 == 0 || bj0 == 0 || bk0 == 0 || bi0 + BX >= op.nx || bj0 + BY >= op.ny ||
                            bk0 + BZ >= op.nz;
    // Colour of step s: the forward pass (q = 0..26), the backward pass (q = 26..0), or both in
    // one launch (nsteps = 54: the last parity of the forward pass is the first of the backward
    // pass, so one CTA runs the block's 27 colours up and then down)
    auto colour_of = [&](int st) { return st < 27 ? (backward ? 26 - st : st) : 53 - st; };
    const cplx<T> *slab0 = stored ? coef + (size_t)((Ib + NI * (Jb + NJ * Kb)) * 27) * SLAB : nullptr;
    auto stage = [&](int q, int buf) {  // colour q's slab -> sc[buf], 16-byte copies
        constexpr int CH = SLAB * (int)sizeof(cplx<T>) / 16;
        const char *src = reinterpret_cast<const char *>(slab0 + (size_t)q * SLAB);
        char *dst = reinterpret_cast<char *>(sc + buf * SLAB);
        for (int e = threadIdx.x; e < CH; e += NT) blk_cp_async<16>(dst + 16 * e, src + 16 * e, true);
    };

    block_stage<T, WNC, PX, PY, NB, R, NT>(op, x, s0, act, i0, j0, k0, sx, swr, swi);
    if (stored) {
        stage(colour_of(0), 0);
        asm volatile("cp.async.commit_group;\n" ::: "memory");
        asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    }
    __syncthreads();

    // this thread's slot: row (u, v, w) of every colour, right-hand side s0 + r.  u, then w,
    // then v: a half-warp spans (u, w), whose box offsets 3u + 3 PX PY w hit 16 distinct
    // 8-byte bank pairs for the 14-point box pitch (no shared-memory bank conflicts).
    const int tid = threadIdx.x;
    const int r = tid / NR, row = tid % NR;
    const int u = row % U, ww = (row / U) % W, v = row / (U * W);
    const bool mine = (act >> r) & 1u;
    cplx<T> *bx = sx + (size_t)r * NB;
    const cplx<T> *bs = b ? b + (long long)(s0 + r) * op.N : nullptr;
    // b_i and 1/||a_i||^2 of the next colour's row are fetched one colour step ahead, so
    // their global-memory latency overlaps the current step
    T inv_n = T(0);
    cplx<T> bv_n = mk<T>(T(0), T(0));
    auto fetch = [&](int q) {
        const int i = bi0 + q % 3 + 3 * u, j = bj0 + (q / 3) % 3 + 3 * v, k = bk0 + q / 9 + 3 * ww;
        if (mine && i < op.nx && j < op.ny && k < op.nz) {
            const long long ctr = i + op.sy * j + op.sz * k;
            inv_n = rinv[ctr];
            if (bs) bv_n = bs[ctr];
        }
    };
    fetch(colour_of(0));
    for (int qq = 0; qq < nsteps; ++qq) {
        const int q = colour_of(qq);
        const T inv = inv_n;
        const cplx<T> bv = bv_n;
        if (qq + 1 < nsteps) fetch(colour_of(qq + 1));
        if (stored) {
            // prefetch the next colour's coefficients into the other buffer (its previous
            // colour finished at the barrier that ended the last iteration)
            if (qq + 1 < nsteps) stage(colour_of(qq + 1), (qq + 1) & 1);
            asm volatile("cp.async.commit_group;\n" ::: "memory");
            asm volatile("cp.async.wait_group 1;\n" ::: "memory");  // this colour's slab landed
            __syncthreads();
        }
        const int a = q % 3, bq = (q / 3) % 3, cq = q / 9;
        const int i = bi0 + a + 3 * u, j = bj0 + bq + 3 * v, k = bk0 + cq + 3 * ww;
        if (mine && i < op.nx && j < op.ny && k < op.nz) {
            const int lc = (1 + a + 3 * u) + PX * ((1 + bq + 3 * v) + PY * (1 + cq + 3 * ww));
            if (stored && edge_block)
                block_row_stored<T, PX, PY, true>(op, bx, sc + (qq & 1) * SLAB, NR, row, bv, inv, w, i, j, k, lc);
            else if (stored)
                block_row_stored<T, PX, PY, false>(op, bx, sc + (qq & 1) * SLAB, NR, row, bv, inv, w, i, j, k, lc);
            else
                block_row<T, ADJ, WNC, PX, PY>(op, bx, swr, swi, bv, inv, w, i, j, k, lc);
        }
        __syncthreads();
    }
    block_store<T, PX, PY, NB, R, NT>(op, x, s0, act, i0, j0, k0, sx);
}

// Block shapes and right-hand-side group sizes the BLOCK8 path can use.
struct Block8Cfg {
    int bx, by, bz, r;
};
static const Block8Cfg kBlock8Cfgs[] = {{12, 12, 12, 1}, {12, 12, 12, 2}, {12, 12, 12, 4}, {24, 12, 12, 1}};
constexpr int kNumBlock8Cfgs = sizeof(kBlock8Cfgs) / sizeof(kBlock8Cfgs[0]);

int num_block8_cfgs() { return kNumBlock8Cfgs; }

size_t block8_cfg_smem(int c, bool fp64, bool wnc)
{
    const Block8Cfg &k = kBlock8Cfgs[c];
    const size_t nb = (size_t)(k.bx + 2) * (k.by + 2) * (k.bz + 2);
    const size_t bytes = nb * k.r * (fp64 ? 16 : 8) + nb * (fp64 ? 8 : 4) * (wnc ? 2 : 1);
    return bytes > 232448 ? 0 : bytes;
}

void block8_cfg_dims(int c, int32_t *blk, int *r)
{
    blk[0] = kBlock8Cfgs[c].bx;
    blk[1] = kBlock8Cfgs[c].by;
    blk[2] = kBlock8Cfgs[c].bz;
    *r = kBlock8Cfgs[c].r;
}

template <typename T, bool ADJ, bool WNC, int BX, int BY, int BZ, int R>
static int block8_pass_t(const Op<T> &op, cplx<T> *x, const cplx<T> *b, int nrhs, T w, const int *active,
                         const T *rinv, const cplx<T> *coef, cudaStream_t st)
{
    constexpr size_t smem_box = block_smem<T, WNC, BX, BY, BZ, R>();
    constexpr size_t smem_coef = ((smem_box + 15) / 16) * 16 + 2 * sizeof(cplx<T>) * Coef8Layout<BX, BY, BZ>::SLAB;
    constexpr int NT = (BX / 3) * (BY / 3) * (BZ / 3) * R;
    if constexpr (smem_box > 232448) {  // 227 KB: the per-CTA shared-memory limit
        set_error("BLOCK8 configuration %dx%dx%d x %d right-hand sides exceeds shared memory", BX, BY, BZ, R);
        return H3D_ERR_BAD_ARG;
    } else {
        // stored coefficients only where their double buffer fits next to the box
        if (smem_coef > 232448) coef = nullptr;
        const size_t smem = coef ? smem_coef : smem_box;
        static bool attr_set = false;  // per template instance and process
        if (!attr_set) {
            const size_t mx = smem_coef > 232448 ? smem_box : smem_coef;
            H3D_CUDA_TRY(cudaFuncSetAttribute(sweep_block8_kernel<T, ADJ, WNC, BX, BY, BZ, R>,
                                              cudaFuncAttributeMaxDynamicSharedMemorySize, (int)mx));
            attr_set = true;
        }
        const int NI = (op.nx + BX - 1) / BX, NJ = (op.ny + BY - 1) / BY, NK = (op.nz + BZ - 1) / BZ;
        // block counts of parity 0 per axis (the largest); other parities skip the excess
        const int NIp = (NI + 1) / 2, NJp = (NJ + 1) / 2, NKp = (NK + 1) / 2;
        const long long nblk = (long long)NIp * NJp * NKp;
        if (nblk > 0x7fffffffLL) {
            set_error("grid too large for the BLOCK8 launch");
            return H3D_ERR_NSIZE;
        }
        const int ngrp = (nrhs + R - 1) / R;
        if (ngrp > 65535) {
            set_error("too many right-hand sides for one BLOCK8 launch (%d groups of %d)", ngrp, R);
            return H3D_ERR_BAD_ARG;
        }
        const dim3 grd((unsigned)nblk, ngrp);
        // forward pass: parities 0..6, then parity 7 up and down in one launch, then the
        // backward pass: parities 6..0 -- 15 launches per double sweep
        for (int pp = 0; pp < 15; ++pp) {
            const int par = pp < 8 ? pp : 14 - pp;
            const int bw = pp < 8 ? 0 : 1;
            const int nsteps = pp == 7 ? 54 : 27;
            sweep_block8_kernel<T, ADJ, WNC, BX, BY, BZ, R><<<grd, NT, smem, st>>>(
                op, x, b, nrhs, w, active, rinv, coef, NI, NJ, NIp, NJp, par, bw, nsteps);
        }
        H3D_CUDA_TRY(cudaGetLastError());
        return H3D_OK;
    }
}

template <typename T, bool ADJ, bool WNC>
static int block8_pass_cfg(const Op<T> &op, cplx<T> *x, const cplx<T> *b, int nrhs, T w, const int *active,
                           const T *rinv, const cplx<T> *coef, int cfg, cudaStream_t st)
{
    // the stored layout is the 12x12x12 one: the 24x12x12 configuration forms coefficients itself
    switch (cfg) {
    case 1: return block8_pass_t<T, ADJ, WNC, 12, 12, 12, 2>(op, x, b, nrhs, w, active, rinv, coef, st);
    case 2: return block8_pass_t<T, ADJ, WNC, 12, 12, 12, 4>(op, x, b, nrhs, w, active, rinv, coef, st);
    case 3: return block8_pass_t<T, ADJ, WNC, 24, 12, 12, 1>(op, x, b, nrhs, w, active, rinv, nullptr, st);
    default: return block8_pass_t<T, ADJ, WNC, 12, 12, 12, 1>(op, x, b, nrhs, w, active, rinv, coef, st);
    }
}

size_t block8_coef_count(int nx, int ny, int nz)
{
    const size_t NI = (nx + 11) / 12, NJ = (ny + 11) / 12, NK = (nz + 11) / 12;
    return NI * NJ * NK * 27 * Coef8Layout<12, 12, 12>::SLAB;
}

template <typename T>
int store_block8_coefs(const Op<T> &op, bool adj, cplx<T> *coef, cudaStream_t st)
{
    const int NI = (op.nx + 11) / 12, NJ = (op.ny + 11) / 12, NK = (op.nz + 11) / 12;
    const long long nbq = (long long)NI * NJ * NK * 27;
    if (nbq > 0x7fffffffLL) {
        set_error("grid too large for the BLOCK8 coefficient store");
        return H3D_ERR_NSIZE;
    }
    const bool wnc = op.wni != nullptr;
    if (!adj && !wnc) coef8_store_kernel<T, false, false, 12, 12, 12><<<(unsigned)nbq, 64, 0, st>>>(op, coef, NI, NJ);
    else if (!adj && wnc) coef8_store_kernel<T, false, true, 12, 12, 12><<<(unsigned)nbq, 64, 0, st>>>(op, coef, NI, NJ);
    else if (adj && !wnc) coef8_store_kernel<T, true, false, 12, 12, 12><<<(unsigned)nbq, 64, 0, st>>>(op, coef, NI, NJ);
    else coef8_store_kernel<T, true, true, 12, 12, 12><<<(unsigned)nbq, 64, 0, st>>>(op, coef, NI, NJ);
    H3D_CUDA_TRY(cudaGetLastError());
    return H3D_OK;
}

// Configuration for an explicit block size: the matching shape with the largest group that
// the right-hand sides fill, or -1 when the size is not one of the compiled shapes.
static int cfg8_for_block(const int32_t *blk, int nrhs)
{
    int best = -1;
    for (int c = 0; c < kNumBlock8Cfgs; ++c) {
        const Block8Cfg &k = kBlock8Cfgs[c];
        if (k.bx != blk[0] || k.by != blk[1] || k.bz != blk[2]) continue;
        if (best < 0 || (k.r <= nrhs && k.r > kBlock8Cfgs[best].r)) best = c;
    }
    return best;
}

template <typename T>
int sweep_block8(const Op<T> &op, cplx<T> *x, const cplx<T> *b, int nrhs, T w, const int32_t *block,
                 const int *active, bool adj, cudaStream_t st, const T *rinv, int cfg, const cplx<T> *coef)
{
    if (cfg < 0) {
        int32_t blk[3] = {12, 12, 12};
        if (block && block[0] > 0)
            for (int a = 0; a < 3; ++a) blk[a] = block[a];
        cfg = cfg8_for_block(blk, nrhs);
        if (cfg < 0) {
            set_error("BLOCK8 order supports block sizes 12x12x12 and 24x12x12");
            return H3D_ERR_BAD_ARG;
        }
    }
    if (cfg >= kNumBlock8Cfgs) {
        set_error("BLOCK8 configuration %d out of range", cfg);
        return H3D_ERR_BAD_ARG;
    }
    const bool wnc = op.wni != nullptr;
    DevBuf norms;  // callers outside the solver pass no row norms: form them here
    if (!rinv) {
        int rc = norms.alloc(sizeof(T) * (size_t)op.N, st);
        if (!rc) rc = row_inv_norms<T>(op, adj, norms.as<T>(), st);
        if (rc) return rc;
        rinv = norms.as<T>();
    }
    int rc;
    if (!adj && !wnc) rc = block8_pass_cfg<T, false, false>(op, x, b, nrhs, w, active, rinv, coef, cfg, st);
    else if (!adj && wnc) rc = block8_pass_cfg<T, false, true>(op, x, b, nrhs, w, active, rinv, coef, cfg, st);
    else if (adj && !wnc) rc = block8_pass_cfg<T, true, false>(op, x, b, nrhs, w, active, rinv, coef, cfg, st);
    else rc = block8_pass_cfg<T, true, true>(op, x, b, nrhs, w, active, rinv, coef, cfg, st);
    if (rc) return rc;
    return H3D_OK;
}

template int sweep_block8<double>(const Op<double> &, cplx<double> *, const cplx<double> *, int, double, const int32_t *, const int *, bool, cudaStream_t, const double *, int, const cplx<double> *);
template int sweep_block8<float>(const Op<float> &, cplx<float> *, const cplx<float> *, int, float, const int32_t *, const int *, bool, cudaStream_t, const float *, int, const cplx<float> *);
template int store_block8_coefs<double>(const Op<double> &, bool, cplx<double> *, cudaStream_t);
template int store_block8_coefs<float>(const Op<float> &, bool, cplx<float> *, cudaStream_t);

}  // namespace h3d
