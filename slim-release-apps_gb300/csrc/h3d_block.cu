// BLOCK row ordering of the Kaczmarz double sweep, with each block resident in shared
// memory for a group of right-hand sides.
//
// The grid is cut into blocks of BX x BY x BZ points.  Blocks (I,J,K) are visited along
// the wavefront T = I + 2J + 4K: two blocks with equal T are never adjacent
// (|dI + 2dJ| <= 3 < 4 forces dK = 0, then dI = -2dJ forces dJ = dI = 0), so a full block
// separates them in some axis and their one-point-halo boxes are disjoint; adjacent blocks
// keep a fixed order.  Inside a block, rows go by the 27 global colours
// q = i%3 + 3(j%3) + 9(k%3).  The backward pass reverses both levels, which keeps the double
// sweep symmetric (a valid CGMN preconditioner; Helm3dkaczswp_mex.c:60-120 with another row
// order).  Information still crosses the whole grid in one pass, as in the reference's
// lexicographic order.
//
// One CTA per (block, group of R right-hand sides): the halo'd box of x for the R right-hand
// sides and of the wavenumber are copied into shared memory (cp.async, zero fill outside the
// grid), the 27 colour phases run there (CTA barriers between colours), and the box goes
// back to global memory once: about one read and one write of x per pass instead of 27.
#include "h3d_blockrow.cuh"
#include "h3d_kernels.cuh"
#include "h3d_vec.cuh"

namespace h3d {

constexpr int kBlockThreads = 256;

template <typename T, bool ADJ, bool WNC, int BX, int BY, int BZ, int R>
__global__ void __launch_bounds__(kBlockThreads) sweep_block_smem_kernel(
    Op<T> op, cplx<T> *x, const cplx<T> *b, int nrhs, T w, const int *active, const T *rinv, int NI,
    int NJ, int Tph, int backward)
{
    using G = BlockGeom<BX, BY, BZ>;
    constexpr int PX = G::PX, PY = G::PY, NB = G::NB;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cplx<T> *sx = reinterpret_cast<cplx<T> *>(smem_raw);  // [R][NB]
    T *swr = reinterpret_cast<T *>(sx + (size_t)R * NB);
    T *swi = WNC ? swr + NB : nullptr;

    const int Jb = blockIdx.x % NJ, Kb = blockIdx.x / NJ;
    const int Ib = Tph - 2 * Jb - 4 * Kb;
    if (Ib < 0 || Ib >= NI) return;
    const int s0 = blockIdx.y * R;
    if (s0 >= nrhs) return;
    const int tid = threadIdx.x;
    const int i0 = Ib * BX - 1, j0 = Jb * BY - 1, k0 = Kb * BZ - 1;  // box origin (halo)

    unsigned act = 0;  // bit r: right-hand side s0 + r takes part
    for (int r = 0; r < R; ++r)
        if (s0 + r < nrhs && (!active || active[s0 + r])) act |= 1u << r;
    if (!act) return;

    block_stage<T, WNC, PX, PY, NB, R, kBlockThreads>(op, x, s0, act, i0, j0, k0, sx, swr, swi);
    __syncthreads();

    const int bi0 = Ib * BX, bj0 = Jb * BY, bk0 = Kb * BZ;
    for (int qq = 0; qq < 27; ++qq) {
        const int q = backward ? 26 - qq : qq;
        const int a = q % 3, bq = (q / 3) % 3, cq = q / 9;
        // first row of this colour inside the block, and the colour's row counts
        const int fi = bi0 + ((a - bi0 % 3) + 3) % 3, fj = bj0 + ((bq - bj0 % 3) + 3) % 3,
                  fk = bk0 + ((cq - bk0 % 3) + 3) % 3;
        const int hi_i = min(bi0 + BX, op.nx), hi_j = min(bj0 + BY, op.ny), hi_k = min(bk0 + BZ, op.nz);
        const int nu = fi < hi_i ? (hi_i - fi + 2) / 3 : 0;
        const int nv = fj < hi_j ? (hi_j - fj + 2) / 3 : 0;
        const int nw = fk < hi_k ? (hi_k - fk + 2) / 3 : 0;
        const int nrow = nu * nv * nw;
        for (int pr = tid; pr < nrow * R; pr += kBlockThreads) {
            const int r = pr / nrow, row = pr % nrow;
            if (!(act & (1u << r))) continue;
            const int i = fi + 3 * (row % nu), j = fj + 3 * ((row / nu) % nv), k = fk + 3 * (row / (nu * nv));
            const int lc = (i - i0) + PX * ((j - j0) + PY * (k - k0));
            const long long ctr = i + op.sy * j + op.sz * k;
            const cplx<T> bv = b ? b[(long long)(s0 + r) * op.N + ctr] : mk<T>(T(0), T(0));
            block_row<T, ADJ, WNC, PX, PY>(op, sx + (size_t)r * NB, swr, swi, bv, rinv[ctr], w, i, j, k, lc);
        }
        __syncthreads();
    }
    block_store<T, PX, PY, NB, R, kBlockThreads>(op, x, s0, act, i0, j0, k0, sx);
}

// Block shapes and right-hand-side group sizes the BLOCK path can use.
struct BlockCfg {
    int bx, by, bz, r;
};
static const BlockCfg kBlockCfgs[] = {{8, 8, 8, 1}, {16, 8, 8, 1}, {8, 8, 8, 4}};
constexpr int kNumBlockCfgs = sizeof(kBlockCfgs) / sizeof(kBlockCfgs[0]);

int num_block_cfgs() { return kNumBlockCfgs; }

// Shared memory one CTA of configuration c needs (0 if it does not fit).
size_t block_cfg_smem(int c, bool fp64, bool wnc)
{
    const BlockCfg &k = kBlockCfgs[c];
    const size_t nb = (size_t)(k.bx + 2) * (k.by + 2) * (k.bz + 2);
    const size_t bytes = nb * k.r * (fp64 ? 16 : 8) + nb * (fp64 ? 8 : 4) * (wnc ? 2 : 1);
    return bytes > 232448 ? 0 : bytes;
}

void block_cfg_dims(int c, int32_t *blk, int *r)
{
    blk[0] = kBlockCfgs[c].bx;
    blk[1] = kBlockCfgs[c].by;
    blk[2] = kBlockCfgs[c].bz;
    *r = kBlockCfgs[c].r;
}

template <typename T, bool ADJ, bool WNC, int BX, int BY, int BZ, int R>
static int block_pass_t(const Op<T> &op, cplx<T> *x, const cplx<T> *b, int nrhs, T w, const int *active,
                        const T *rinv, bool backward, cudaStream_t st)
{
    constexpr size_t smem = block_smem<T, WNC, BX, BY, BZ, R>();
    if constexpr (smem > 232448) {  // 227 KB: the per-CTA shared-memory limit
        set_error("BLOCK configuration %dx%dx%d x %d right-hand sides exceeds shared memory", BX, BY, BZ, R);
        return H3D_ERR_BAD_ARG;
    } else {
    static bool attr_set = false;  // per template instance and process
    if (!attr_set) {
        H3D_CUDA_TRY(cudaFuncSetAttribute(sweep_block_smem_kernel<T, ADJ, WNC, BX, BY, BZ, R>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        attr_set = true;
    }
    const int NI = (op.nx + BX - 1) / BX, NJ = (op.ny + BY - 1) / BY, NK = (op.nz + BZ - 1) / BZ;
    const int Tmax = (NI - 1) + 2 * (NJ - 1) + 4 * (NK - 1);
    const dim3 grd(NJ * NK, (nrhs + R - 1) / R);
    for (int tt = 0; tt <= Tmax; ++tt) {
        const int Tph = backward ? Tmax - tt : tt;
        sweep_block_smem_kernel<T, ADJ, WNC, BX, BY, BZ, R>
            <<<grd, kBlockThreads, smem, st>>>(op, x, b, nrhs, w, active, rinv, NI, NJ, Tph, backward ? 1 : 0);
    }
    H3D_CUDA_TRY(cudaGetLastError());
    return H3D_OK;
    }
}

template <typename T, bool ADJ, bool WNC>
static int block_pass_cfg(const Op<T> &op, cplx<T> *x, const cplx<T> *b, int nrhs, T w, const int *active,
                          const T *rinv, int cfg, bool backward, cudaStream_t st)
{
    switch (cfg) {
    case 1: return block_pass_t<T, ADJ, WNC, 16, 8, 8, 1>(op, x, b, nrhs, w, active, rinv, backward, st);
    case 2: return block_pass_t<T, ADJ, WNC, 8, 8, 8, 4>(op, x, b, nrhs, w, active, rinv, backward, st);
    default: return block_pass_t<T, ADJ, WNC, 8, 8, 8, 1>(op, x, b, nrhs, w, active, rinv, backward, st);
    }
}

// Configuration for an explicit block size: the matching shape with the largest group that
// the right-hand sides fill, or -1 when the size is not one of the compiled shapes.
static int cfg_for_block(const int32_t *blk, int nrhs)
{
    int best = -1;
    for (int c = 0; c < kNumBlockCfgs; ++c) {
        const BlockCfg &k = kBlockCfgs[c];
        if (k.bx != blk[0] || k.by != blk[1] || k.bz != blk[2]) continue;
        if (best < 0 || (k.r <= nrhs && k.r > kBlockCfgs[best].r)) best = c;
    }
    return best;
}

template <typename T>
int sweep_block(const Op<T> &op, cplx<T> *x, const cplx<T> *b, int nrhs, T w,
                const int32_t *block, const int *active, bool adj, cudaStream_t st,
                const T *rinv, int cfg)
{
    if (cfg < 0) {
        int32_t blk[3] = {8, 8, 8};
        if (block && block[0] > 0)
            for (int a = 0; a < 3; ++a) blk[a] = block[a];
        cfg = cfg_for_block(blk, nrhs);
        if (cfg < 0) {
            set_error("BLOCK order supports block sizes 8x8x8 and 16x8x8");
            return H3D_ERR_BAD_ARG;
        }
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
        if (!adj && !wnc) rc = block_pass_cfg<T, false, false>(op, x, b, nrhs, w, active, rinv, cfg, bw, st);
        else if (!adj && wnc) rc = block_pass_cfg<T, false, true>(op, x, b, nrhs, w, active, rinv, cfg, bw, st);
        else if (adj && !wnc) rc = block_pass_cfg<T, true, false>(op, x, b, nrhs, w, active, rinv, cfg, bw, st);
        else rc = block_pass_cfg<T, true, true>(op, x, b, nrhs, w, active, rinv, cfg, bw, st);
        if (rc) return rc;
    }
    return H3D_OK;
}

template int sweep_block<double>(const Op<double> &, cplx<double> *, const cplx<double> *, int, double, const int32_t *, const int *, bool, cudaStream_t, const double *, int);
template int sweep_block<float>(const Op<float> &, cplx<float> *, const cplx<float> *, int, float, const int32_t *, const int *, bool, cudaStream_t, const float *, int);

}  // namespace h3d
