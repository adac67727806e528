// Host-callable launchers of the device kernels (one translation unit each).
#pragma once

#include "h3d_internal.cuh"

namespace h3d {

// L2-coherent load (bypasses L1), for data another CTA may have written in the same launch.
template <typename T>
__device__ __forceinline__ cplx<T> load_cg(const cplx<T> *p);
template <>
__device__ __forceinline__ cplx<double> load_cg(const cplx<double> *p)
{
    const double2 v = __ldcg(reinterpret_cast<const double2 *>(p));
    return {v.x, v.y};
}
template <>
__device__ __forceinline__ cplx<float> load_cg(const cplx<float> *p)
{
    const float2 v = __ldcg(reinterpret_cast<const float2 *>(p));
    return {v.x, v.y};
}

// h3d_mvp.cu: z-marching matvec, and the FP64 residual b - A x with per-block norms.
// mvp_prime_occupancy: fixes the device occupancy the matvec grids are cut by (called when
// an operator is made).
void mvp_prime_occupancy();
int mvp_residual_parts(const Op<double> &op, int nrhs);
// parts: the partial-sum count per right-hand side the buffer was sized for
// (mvp_residual_parts); a launch needing another count is refused.
int launch_residual(const Op<double> &op, const cplx<double> *b, const cplx<double> *x, cplx<double> *r,
                    int nrhs, bool adj, double *part, int parts, cudaStream_t st);

// h3d_mvp.cu / h3d_stencil.cu
template <typename T>
int launch_mvp(const Op<T> &op, const cplx<T> *x, cplx<T> *y, int nrhs, bool adj, bool deriv,
               cudaStream_t st);
// rinv: optional 1/||a_i||^2 per row (COLOUR27 only; NULL = computed in the kernel);
// shape: COLOUR27 tile shape index (-1 = chosen from the grid).  coef (with rinv): stored
// row coefficients; COLOUR27 then runs the direct kernel instead of the tile kernel.
template <typename T>
int launch_sweep(const Op<T> &op, cplx<T> *x, const cplx<T> *b, int nrhs, T w, bool adj,
                 int order, const int32_t *block, const int *active, cudaStream_t st,
                 const T *rinv = nullptr, int shape = -1, const cplx<T> *coef = nullptr);

// h3d_sweep_direct.cu: COLOUR27 on stored row coefficients (27 N complex values, colour-major).
template <typename T>
int store_row_coefs(const Op<T> &op, bool adj, cplx<T> *coef, cudaStream_t st);
template <typename T>
int sweep_colour_direct(const Op<T> &op, cplx<T> *x, const cplx<T> *b, int nrhs, T w, const int *active,
                        const T *rinv, const cplx<T> *coef, bool adj, cudaStream_t st);

// h3d_sweep_tile.cu: one COLOUR27 pass (27 colour launches) with shared-memory boxes.
template <typename T>
int sweep_colour_tiled(const Op<T> &op, cplx<T> *x, const cplx<T> *b, int nrhs, T w,
                       const int *active, const T *rinv, int shape, bool adj, bool backward,
                       cudaStream_t st);
template <typename T>
int row_inv_norms(const Op<T> &op, bool adj, T *rinv, cudaStream_t st);
int pick_tile_shape(int nx, int ny, int nz);
int num_tile_shapes();

// h3d_block.cu: the BLOCK ordering (block wavefront, 27 colours inside a block).
// cfg: index of a compiled (block shape, right-hand-side group) configuration, or -1 to
// derive it from `block` (8x8x8 by default).
template <typename T>
int sweep_block(const Op<T> &op, cplx<T> *x, const cplx<T> *b, int nrhs, T w,
                const int32_t *block, const int *active, bool adj, cudaStream_t st,
                const T *rinv = nullptr, int cfg = -1);
int num_block_cfgs();
void block_cfg_dims(int c, int32_t *blk, int *r);
size_t block_cfg_smem(int c, bool fp64, bool wnc);

// h3d_block8.cu: the BLOCK8 ordering (eight parity classes of blocks, 27 colours inside a
// block); cfg as for sweep_block (12x12x12 by default).
// coef: stored coefficients in the 12x12x12 block layout (store_block8_coefs), or null.
template <typename T>
int sweep_block8(const Op<T> &op, cplx<T> *x, const cplx<T> *b, int nrhs, T w,
                 const int32_t *block, const int *active, bool adj, cudaStream_t st,
                 const T *rinv = nullptr, int cfg = -1, const cplx<T> *coef = nullptr);
size_t block8_coef_count(int nx, int ny, int nz);  // complex values of the stored layout
template <typename T>
int store_block8_coefs(const Op<T> &op, bool adj, cplx<T> *coef, cudaStream_t st);
int num_block8_cfgs();
void block8_cfg_dims(int c, int32_t *blk, int *r);
size_t block8_cfg_smem(int c, bool fp64, bool wnc);

// h3d_interp.cu: y = scale * A x along one axis (A in CSR form), or y += that (accum).
template <typename T>
int launch_axis(const int32_t *rowptr, const int32_t *col, const double *val, int n_out, int axis,
                const int32_t dims_in[3], const cplx<T> *x, cplx<T> *y, int nrhs, double scale, bool accum,
                cudaStream_t st);

}  // namespace h3d
