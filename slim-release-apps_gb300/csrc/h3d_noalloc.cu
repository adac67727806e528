// h3d_residual_noalloc: the FP64 residual r = b - A x with per-RHS ||r||^2 and ||b||^2,
// for callers that cannot allocate device memory (their device memory belongs to their
// own allocator or to a fixed budget).  It runs the same kernels as h3d_residual; the
// only difference is where the scratch lives: one file-scope device array, sized once,
// instead of buffers from the stream-ordered allocator and the per-grid table cache.
//
// Scratch layout (doubles): [PML tables: 2 * sum_a 3 (n_a + 2), i.e. three complex tables of
// n_a + 2 entries per axis] [partials: 2 * G * nrhs]
// The tables are rewritten on every call; every partial is written by its block before
// the reduction reads it, so nothing has to start at zero.
#include <cstring>
#include <mutex>
#include <vector>

#include "h3d_internal.cuh"
#include "h3d_kernels.cuh"
#include "h3d_krylov.cuh"

namespace h3d {

constexpr size_t kNoAllocDoubles = H3D_NOALLOC_SCRATCH_BYTES / sizeof(double);

// Held by every GPU that loads the library, until the process exits.
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocDoubles];

constexpr int kMaxDevices = 64;
static std::mutex g_noalloc_mutex;
static double *g_noalloc_ptr[kMaxDevices];

// Device address of the scratch array on the current device, looked up once per device.
static int noalloc_scratch(double **out)
{
    int dev = 0;
    H3D_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) {
        set_error("device ordinal %d out of range", dev);
        return H3D_ERR_BAD_ARG;
    }
    std::lock_guard<std::mutex> lk(g_noalloc_mutex);
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(noalloc scratch)");
        g_noalloc_ptr[dev] = static_cast<double *>(p);
    }
    *out = g_noalloc_ptr[dev];
    return H3D_OK;
}

}  // namespace h3d

using namespace h3d;

extern "C" int h3d_residual_noalloc(const h3d_grid *g, const double *wn_re, const double *wn_im,
                                    const void *b, const void *x, void *r, double *rr2, double *bb2,
                                    int nrhs, int mode, void *stream)
{
    if (nrhs < 1 || (mode != H3D_FORWARD && mode != H3D_ADJOINT)) {
        set_error("h3d_residual_noalloc: bad argument");
        return H3D_ERR_BAD_ARG;
    }
    int rc = check_grid(g);
    if (rc) return rc;
    // Size check first, before any launch or copy and before the pointers are looked at: a
    // call with the data pointers left NULL asks only whether the problem fits the scratch,
    // and can never launch.  The count of partial sums follows the matvec's z split, which
    // is chosen from the current device's occupancy (a CUDA query, no launch), so the largest
    // problem accepted depends on the device.
    size_t tab_entries = 0;
    for (int a = 0; a < 3; ++a) tab_entries += 3 * (size_t)(g->n[a] + 2);
    const size_t tab_doubles = (2 * tab_entries + 31) / 32 * 32;  // keep the partials 256-byte aligned
    Op<double> probe{};
    probe.nx = g->n[0];
    probe.ny = g->n[1];
    probe.nz = g->n[2];
    const long long G = mvp_residual_parts(probe, nrhs);
    const size_t need = tab_doubles + 2 * (size_t)G * (size_t)nrhs;
    if (need > kNoAllocDoubles) {
        set_error("h3d_residual_noalloc: grid %dx%dx%d with %d right-hand sides needs %zu bytes of scratch, "
                  "more than the fixed %u bytes",
                  g->n[0], g->n[1], g->n[2], nrhs, need * sizeof(double), (unsigned)H3D_NOALLOC_SCRATCH_BYTES);
        return H3D_ERR_BAD_ARG;
    }
    if (!wn_re || !b || !x || !r) {
        set_error("h3d_residual_noalloc: bad argument");
        return H3D_ERR_BAD_ARG;
    }
    double *scratch = nullptr;
    if ((rc = noalloc_scratch(&scratch))) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    std::vector<cplx<double>> host_tab;
    Op<double> op;
    if ((rc = make_op_f64_at(g, wn_re, wn_im, scratch, &host_tab, &op))) return rc;
    // Pageable source: the copy is staged before cudaMemcpyAsync returns.
    H3D_CUDA_TRY(cudaMemcpyAsync(scratch, host_tab.data(), host_tab.size() * sizeof(cplx<double>),
                                 cudaMemcpyHostToDevice, st));
    double *part = scratch + tab_doubles;
    return residual_f64(op, (const cplx<double> *)b, (const cplx<double> *)x, (cplx<double> *)r, rr2, bb2,
                        nrhs, mode == H3D_ADJOINT, part, (int)G, st);
}
