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
// and a pass is 8 launches.  With block sides divisible by 3 every colour has the same
// (BX/3)(BY/3)(BZ/3) rows in a block (fewer at the grid's far faces), so thread t owns one
// fixed (row, right-hand side) slot for all colours: no index division in the colour loop.
#include "h3d_blockrow.cuh"
#include "h3d_kernels.cuh"
#include "h3d_vec.cuh"

namespace h3d {

template <typename T, bool ADJ, bool WNC, int BX, int BY, int BZ, int R>
__global__ void __launch_bounds__((BX / 3) * (BY / 3) * (BZ / 3) * R) sweep_block8_kernel(
    Op<T> op, cplx<T> *x, const cplx<T> *b, int nrhs, T w, const int *active, const T *rinv,
    int NIp, int NJp, int par, int backward)
{
    static_assert(BX % 3 == 0 && BY % 3 == 0 && BZ % 3 == 0, "block sides must be multiples of 3");
    constexpr int U = BX / 3, V = BY / 3, W = BZ / 3, NR = U * V * W, NT = NR * R;
    using G = BlockGeom<BX, BY, BZ>;
    constexpr int PX = G::PX, PY = G::PY, NB = G::NB;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cplx<T> *sx = reinterpret_cast<cplx<T> *>(smem_raw);  // [R][NB]
    T *swr = reinterpret_cast<T *>(sx + (size_t)R * NB);
    T *swi = WNC ? swr + NB : nullptr;

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

    block_stage<T, WNC, PX, PY, NB, R, NT>(op, x, s0, act, i0, j0, k0, sx, swr, swi);
    __syncthreads();

    // this thread's slot: row (u, v, w) of every colour, right-hand side s0 + r
    const int tid = threadIdx.x;
    const int r = tid / NR, row = tid % NR;
    const int u = row % U, v = (row / U) % V, ww = row / (U * V);
    const bool mine = (act >> r) & 1u;
    cplx<T> *bx = sx + (size_t)r * NB;
    const cplx<T> *bs = b ? b + (long long)(s0 + r) * op.N : nullptr;
    for (int qq = 0; qq < 27; ++qq) {
        const int q = backward ? 26 - qq : qq;
        const int a = q % 3, bq = (q / 3) % 3, cq = q / 9;
        const int i = bi0 + a + 3 * u, j = bj0 + bq + 3 * v, k = bk0 + cq + 3 * ww;
        if (mine && i < op.nx && j < op.ny && k < op.nz) {
            const int lc = (1 + a + 3 * u) + PX * ((1 + bq + 3 * v) + PY * (1 + cq + 3 * ww));
            block_row<T, ADJ, WNC, PX, PY>(op, bx, swr, swi, bs, rinv, w, i, j, k, lc);
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
                         const T *rinv, bool backward, cudaStream_t st)
{
    constexpr size_t smem = block_smem<T, WNC, BX, BY, BZ, R>();
    constexpr int NT = (BX / 3) * (BY / 3) * (BZ / 3) * R;
    if constexpr (smem > 232448) {  // 227 KB: the per-CTA shared-memory limit
        set_error("BLOCK8 configuration %dx%dx%d x %d right-hand sides exceeds shared memory", BX, BY, BZ, R);
        return H3D_ERR_BAD_ARG;
    } else {
        static bool attr_set = false;  // per template instance and process
        if (!attr_set) {
            H3D_CUDA_TRY(cudaFuncSetAttribute(sweep_block8_kernel<T, ADJ, WNC, BX, BY, BZ, R>,
                                              cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
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
        for (int pp = 0; pp < 8; ++pp) {
            const int par = backward ? 7 - pp : pp;
            sweep_block8_kernel<T, ADJ, WNC, BX, BY, BZ, R>
                <<<grd, NT, smem, st>>>(op, x, b, nrhs, w, active, rinv, NIp, NJp, par, backward ? 1 : 0);
        }
        H3D_CUDA_TRY(cudaGetLastError());
        return H3D_OK;
    }
}

template <typename T, bool ADJ, bool WNC>
static int block8_pass_cfg(const Op<T> &op, cplx<T> *x, const cplx<T> *b, int nrhs, T w, const int *active,
                           const T *rinv, int cfg, bool backward, cudaStream_t st)
{
    switch (cfg) {
    case 1: return block8_pass_t<T, ADJ, WNC, 12, 12, 12, 2>(op, x, b, nrhs, w, active, rinv, backward, st);
    case 2: return block8_pass_t<T, ADJ, WNC, 12, 12, 12, 4>(op, x, b, nrhs, w, active, rinv, backward, st);
    case 3: return block8_pass_t<T, ADJ, WNC, 24, 12, 12, 1>(op, x, b, nrhs, w, active, rinv, backward, st);
    default: return block8_pass_t<T, ADJ, WNC, 12, 12, 12, 1>(op, x, b, nrhs, w, active, rinv, backward, st);
    }
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
                 const int *active, bool adj, cudaStream_t st, const T *rinv, int cfg)
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
    for (int pass = 0; pass < 2; ++pass) {
        const bool bw = pass == 1;
        int rc;
        if (!adj && !wnc) rc = block8_pass_cfg<T, false, false>(op, x, b, nrhs, w, active, rinv, cfg, bw, st);
        else if (!adj && wnc) rc = block8_pass_cfg<T, false, true>(op, x, b, nrhs, w, active, rinv, cfg, bw, st);
        else if (adj && !wnc) rc = block8_pass_cfg<T, true, false>(op, x, b, nrhs, w, active, rinv, cfg, bw, st);
        else rc = block8_pass_cfg<T, true, true>(op, x, b, nrhs, w, active, rinv, cfg, bw, st);
        if (rc) return rc;
    }
    return H3D_OK;
}

template int sweep_block8<double>(const Op<double> &, cplx<double> *, const cplx<double> *, int, double, const int32_t *, const int *, bool, cudaStream_t, const double *, int);
template int sweep_block8<float>(const Op<float> &, cplx<float> *, const cplx<float> *, int, float, const int32_t *, const int *, bool, cudaStream_t, const float *, int);

}  // namespace h3d
