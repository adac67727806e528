// BLOCK row ordering of the Kaczmarz double sweep.
//
// The grid is cut into blocks of bx*by*bz points (each >= 2).  Blocks (I,J,K) are visited
// along the block wavefront T = I + 2J + 4K: two blocks with equal T are never adjacent
// (|dI + 2dJ| <= 3 < 4 forces dK = 0, then dI = -2dJ forces dJ = dI = 0), so their rows
// share no neighbour and one CTA per block can run them concurrently, while adjacent
// blocks keep a fixed order.  Inside a block, rows go by the 27 global colours
// q = i%3 + 3(j%3) + 9(k%3), with a CTA barrier between colours.  The backward pass
// reverses both levels, which keeps the double sweep symmetric (a valid CGMN
// preconditioner, Helm3dkaczswp_mex.c:60-120 with a different row order).
#include "h3d_internal.cuh"
#include "h3d_kernels.cuh"
#include "h3d_rowops.cuh"

namespace h3d {

template <typename T, bool ADJ, bool WNC>
__global__ void __launch_bounds__(256) sweep_block_kernel(Op<T> op, cplx<T> *x, const cplx<T> *b,
                                                          int nrhs, int rhs_per_cta, T w,
                                                          const int *active, int bx, int by,
                                                          int bz, int NI, int NJ, int Tph,
                                                          int backward)
{
    const int J = blockIdx.x % NJ, K = blockIdx.x / NJ;
    const int I = Tph - 2 * J - 4 * K;
    if (I < 0 || I >= NI) return;
    const int s0 = blockIdx.y * rhs_per_cta;
    const int ns = min(rhs_per_cta, nrhs - s0);
    if (ns <= 0) return;
    const int lo0 = I * bx, lo1 = J * by, lo2 = K * bz;
    const int hi0 = min(lo0 + bx, op.nx), hi1 = min(lo1 + by, op.ny), hi2 = min(lo2 + bz, op.nz);
    cplx<T> *xs = x + (long long)s0 * op.N;
    const cplx<T> *bs = b ? b + (long long)s0 * op.N : nullptr;
    const int *act = active ? active + s0 : nullptr;
    for (int qq = 0; qq < 27; ++qq) {
        const int q = backward ? 26 - qq : qq;
        const int a = q % 3, bq = (q / 3) % 3, cq = q / 9;
        const int i0 = lo0 + ((a - lo0 % 3) + 3) % 3;
        const int j0 = lo1 + ((bq - lo1 % 3) + 3) % 3;
        const int k0 = lo2 + ((cq - lo2 % 3) + 3) % 3;
        const int nu = i0 < hi0 ? (hi0 - i0 + 2) / 3 : 0;
        const int nv = j0 < hi1 ? (hi1 - j0 + 2) / 3 : 0;
        const int nw = k0 < hi2 ? (hi2 - k0 + 2) / 3 : 0;
        const int cnt = nu * nv * nw;
        for (int r = threadIdx.x; r < cnt; r += blockDim.x) {
            const int u = r % nu, v = (r / nu) % nv, ww = r / (nu * nv);
            project_row<T, ADJ, WNC>(op, xs, bs, ns, i0 + 3 * u, j0 + 3 * v, k0 + 3 * ww, w, act);
        }
        __syncthreads();
    }
}

template <typename T, bool ADJ, bool WNC>
static void block_pass(const Op<T> &op, cplx<T> *x, const cplx<T> *b, int nrhs, T w,
                       const int32_t *blk, const int *active, bool backward, cudaStream_t st)
{
    const int bx = blk[0], by = blk[1], bz = blk[2];
    const int NI = (op.nx + bx - 1) / bx, NJ = (op.ny + by - 1) / by, NK = (op.nz + bz - 1) / bz;
    const int Tmax = (NI - 1) + 2 * (NJ - 1) + 4 * (NK - 1);
    const int rpc = nrhs < 4 ? nrhs : 4;
    const dim3 grd(NJ * NK, (nrhs + rpc - 1) / rpc);
    for (int tt = 0; tt <= Tmax; ++tt) {
        const int Tph = backward ? Tmax - tt : tt;
        sweep_block_kernel<T, ADJ, WNC><<<grd, 128, 0, st>>>(op, x, b, nrhs, rpc, w, active, bx, by,
                                                             bz, NI, NJ, Tph, backward ? 1 : 0);
    }
}

template <typename T>
int sweep_block(const Op<T> &op, cplx<T> *x, const cplx<T> *b, int nrhs, T w,
                const int32_t *block, const int *active, bool adj, cudaStream_t st)
{
    int32_t blk[3] = {8, 8, 8};
    if (block && block[0] > 0) {
        for (int a = 0; a < 3; ++a) blk[a] = block[a];
    }
    for (int a = 0; a < 3; ++a)
        if (blk[a] < 2) {
            set_error("BLOCK order needs block sizes >= 2");
            return H3D_ERR_BAD_ARG;
        }
    const bool wnc = op.wni != nullptr;
    for (int pass = 0; pass < 2; ++pass) {
        const bool bw = pass == 1;
        if (!adj && !wnc) block_pass<T, false, false>(op, x, b, nrhs, w, blk, active, bw, st);
        else if (!adj && wnc) block_pass<T, false, true>(op, x, b, nrhs, w, blk, active, bw, st);
        else if (adj && !wnc) block_pass<T, true, false>(op, x, b, nrhs, w, blk, active, bw, st);
        else block_pass<T, true, true>(op, x, b, nrhs, w, blk, active, bw, st);
    }
    H3D_CUDA_TRY(cudaGetLastError());
    return H3D_OK;
}

template int sweep_block<double>(const Op<double> &, cplx<double> *, const cplx<double> *, int, double, const int32_t *, const int *, bool, cudaStream_t);
template int sweep_block<float>(const Op<float> &, cplx<float> *, const cplx<float> *, int, float, const int32_t *, const int *, bool, cudaStream_t);

}  // namespace h3d
