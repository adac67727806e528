// Solvers: u = H \ b and H^H \ b by CGMN on the Kaczmarz-preconditioned system
// (tools/solvers/Krylov/linearsolve.m:148-168 + CGMN.m:36-94), in plain FP64 or as
// complex64 inner solves under FP64 iterative refinement.
//
//   b~ = DSWP(0, b),  (I - Q) u = b~,  Q y = DSWP(y, 0),  w = 1.5, one double sweep
//   (linearsolve.m:150-152); zero start (linearsolve.m:117-119).
//
// Iterations are recorded once into a CUDA graph (check_every iterations per graph) and
// replayed; per-RHS masks freeze converged right-hand sides on the device, and the host
// only reads the mask every check_every iterations.
#include <chrono>
#include <map>
#include <mutex>
#include <tuple>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "h3d_internal.cuh"
#include "h3d_kernels.cuh"
#include "h3d_krylov.cuh"
#include "h3d_reduce.cuh"
#include "h3d_vec.cuh"

namespace h3d {

// FP64 residual r = b - A x (z-marching matvec kernel with fused norms), then one block
// per right-hand side sums the per-block partials in a fixed order.
__global__ void residual_reduce(const double *part, int G, double *rr2, double *bb2)
{
    const int s = blockIdx.x;
    double a = 0.0, b = 0.0;
    for (int q = threadIdx.x; q < G; q += blockDim.x) {
        a += part[2 * ((long long)s * G + q)];
        b += part[2 * ((long long)s * G + q) + 1];
    }
    const double2 t = block_sum2_r(a, b);
    if (threadIdx.x == 0) {
        if (rr2) rr2[s] = t.x;
        if (bb2) bb2[s] = t.y;
    }
}

int residual_f64(const Op<double> &op, const cplx<double> *b, const cplx<double> *x,
                 cplx<double> *r, double *rr2, double *bb2, int nrhs, bool adj, double *part,
                 int G, cudaStream_t st)
{
    int rc = launch_residual(op, b, x, r, nrhs, adj, part, G, st);
    if (rc) return rc;
    residual_reduce<<<nrhs, 256, 0, st>>>(part, G, rr2, bb2);
    H3D_CUDA_TRY(cudaGetLastError());
    return H3D_OK;
}

// ---------------------------------------------------------------------------------------
// Autotuner cache: (nx, ny, nz, element size, adjoint, complex wn, nrhs) -> tile shape.
using TuneKey = std::tuple<int, int, int, int, int, int, int>;
static std::mutex g_tune_mutex;
static std::map<TuneKey, int> g_tune_cache;

static bool tune_lookup(const TuneKey &k, int *shape)
{
    std::lock_guard<std::mutex> lk(g_tune_mutex);
    auto it = g_tune_cache.find(k);
    if (it == g_tune_cache.end()) return false;
    *shape = it->second;
    return true;
}

static void tune_store(const TuneKey &k, int shape)
{
    std::lock_guard<std::mutex> lk(g_tune_mutex);
    g_tune_cache[k] = shape;
}

// ---------------------------------------------------------------------------------------
// One CGMN instance over nrhs right-hand sides in storage precision T.
template <typename T>
struct CgRun {
    Op<T> op{};
    long long N = 0;
    int nrhs = 0;
    bool adj = false;
    T w = T(1.5);
    int order = H3D_ORDER_COLOUR27;
    int32_t block[3] = {0, 0, 0};
    int maxit = 10000;
    int method = H3D_METHOD_CGMN;
    int verbose = 0;
    cplx<T> *x = nullptr, *r = nullptr, *p = nullptr, *y = nullptr;
    cplx<T> *ap = nullptr;  // CRMN: A p
    T *rinv = nullptr;   // 1/||a_i||^2 per row, computed once (all orders but LEX)
    int shape = -1;      // COLOUR27 tile shape (num_tile_shapes(): stored coefficients), BLOCK cfg
    cplx<T> *coef = nullptr;  // stored row coefficients (COLOUR27: colour-major 27 N; BLOCK8: 12^3 block layout)
    CgState s{};
    DevBuf vecs, scal, ints, parts, norms, coefs;
    cudaGraphExec_t exec = nullptr;
    int graph_iters = 0;
    // Timing of the last double sweep of every replayed block: two timing events recorded
    // as event nodes of the graph, read after the block completes.
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    bool timed_pending = false;
    double sweep_seconds = 0.0;
    int sweep_samples = 0;
    long long launches = 0;        // kernels executed by this instance
    long long block_launches = 0;  // kernels in one replayed block

    ~CgRun()
    {
        if (exec) cudaGraphExecDestroy(exec);
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
    }

    int iteration_launches() const { return sweep_launches() + (method == H3D_METHOD_CRMN ? 6 : 5); }

    // Fold the last timed sweep into the totals (the stream has been synchronised).
    void harvest_timing()
    {
        if (!timed_pending) return;
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, ev0, ev1) == cudaSuccess) {
            sweep_seconds += 1e-3 * ms;
            ++sweep_samples;
        }
        timed_pending = false;
    }

    int alloc(cudaStream_t st)
    {
        const size_t vb = sizeof(cplx<T>) * (size_t)N * nrhs;
        int rc;
        const bool cr = method == H3D_METHOD_CRMN;
        if ((rc = vecs.alloc((cr ? 5 : 4) * vb, st))) return rc;
        x = vecs.as<cplx<T>>();
        r = x + N * nrhs;
        p = r + N * nrhs;
        y = p + N * nrhs;
        ap = cr ? y + N * nrhs : nullptr;
        s.G = reduction_blocks(N);
        if ((rc = scal.alloc(sizeof(double) * (size_t)nrhs * (cr ? 12 : 7), st))) return rc;
        double *d = scal.as<double>();
        s.rr = d;
        s.bb = d + nrhs;
        s.ratio = d + 2 * nrhs;
        s.tolp = d + 3 * nrhs;
        s.beta = d + 4 * nrhs;
        s.alpha = d + 5 * nrhs;  // 2 * nrhs
        if (cr) {
            s.rar = d + 7 * nrhs;    // 2 * nrhs
            s.cbeta = d + 9 * nrhs;  // 2 * nrhs
            s.nap2 = d + 11 * nrhs;
        }
        if ((rc = ints.alloc(sizeof(int) * (size_t)nrhs * 4, st))) return rc;
        int *q = ints.as<int>();
        s.active = q;
        s.upd = q + nrhs;
        s.iters = q + 2 * nrhs;
        s.status = q + 3 * nrhs;
        if ((rc = parts.alloc(sizeof(double) * 2 * (size_t)s.G * nrhs, st))) return rc;
        s.part = parts.as<double>();
        if (order != H3D_ORDER_LEX) {
            if ((rc = norms.alloc(sizeof(T) * (size_t)N, st))) return rc;
            rinv = norms.as<T>();
            if ((rc = row_inv_norms<T>(op, adj, rinv, st))) return rc;
            ++launches;
        }
        if (order == H3D_ORDER_COLOUR27) {
            // stored coefficients when they take at most half of the free device memory
            size_t fr = 0, tot = 0;
            const size_t bytes = sizeof(cplx<T>) * 27 * (size_t)N;
            if (cudaMemGetInfo(&fr, &tot) == cudaSuccess && bytes <= fr / 2 && coefs.alloc(bytes, st) == H3D_OK) {
                coef = coefs.as<cplx<T>>();
                if ((rc = store_row_coefs<T>(op, adj, coef, st))) return rc;
                launches += 27;
            }
            (void)cudaGetLastError();
        }
        const bool blk12 = block[0] <= 0 || (block[0] == 12 && block[1] == 12 && block[2] == 12);
        if (order == H3D_ORDER_BLOCK8 && blk12) {
            size_t fr = 0, tot = 0;
            const size_t bytes = sizeof(cplx<T>) * block8_coef_count(op.nx, op.ny, op.nz);
            if (cudaMemGetInfo(&fr, &tot) == cudaSuccess && bytes <= fr / 2 && coefs.alloc(bytes, st) == H3D_OK) {
                coef = coefs.as<cplx<T>>();
                if ((rc = store_block8_coefs<T>(op, adj, coef, st))) return rc;
                launches += 1;
            }
            (void)cudaGetLastError();
        }
        return H3D_OK;
    }

    int sweep_launches() const
    {
        if (order == H3D_ORDER_LEX) return 2 * ((op.nx - 1) + 3 * (op.ny - 1) + 9 * (op.nz - 1) + 1);
        if (order == H3D_ORDER_BLOCK) {
            int32_t bd[3] = {block[0] > 0 ? block[0] : 8, block[1] > 0 ? block[1] : 8, block[2] > 0 ? block[2] : 8};
            if (shape >= 0) {
                int r = 1;
                block_cfg_dims(shape, bd, &r);
            }
            const int bx = bd[0], by = bd[1], bz = bd[2];
            return 2 * (((op.nx + bx - 1) / bx - 1) + 2 * ((op.ny + by - 1) / by - 1) +
                        4 * ((op.nz + bz - 1) / bz - 1) + 1);
        }
        if (order == H3D_ORDER_BLOCK8) return 15;
        int n = 0;
        for (int q = 0; q < 27; ++q) {
            const int a = q % 3, bq = (q / 3) % 3, cq = q / 9;
            n += (op.nx > a && op.ny > bq && op.nz > cq) ? 1 : 0;
        }
        return 2 * n;
    }

    // Tile-shape autotuner for the COLOUR27 sweep: time one double sweep per candidate
    // shape on the scratch vector y (its contents are overwritten by setup right after)
    // and keep the fastest; decisions are cached per (grid, precision, mode, nrhs).
    int tune(cudaStream_t st)
    {
        if (order == H3D_ORDER_LEX || shape >= 0) return H3D_OK;
        if (order != H3D_ORDER_COLOUR27 && block[0] > 0) return H3D_OK;  // explicit block size
        const TuneKey key{op.nx, op.ny, op.nz, (int)sizeof(T) + 100 * order, adj ? 1 : 0, op.wni ? 1 : 0, nrhs};
        if (tune_lookup(key, &shape)) {
            settle_coefs();
            return H3D_OK;
        }
        cudaEvent_t e0, e1;
        H3D_CUDA_TRY(cudaEventCreate(&e0));
        H3D_CUDA_TRY(cudaEventCreate(&e1));
        float best = 1e30f;
        int best_shape = 0;
        int rc = zero_vec<T>(y, N, nrhs, st);
        const int ncand = order == H3D_ORDER_BLOCK    ? num_block_cfgs()
                          : order == H3D_ORDER_BLOCK8 ? num_block8_cfgs()
                                                      : num_tile_shapes() + (coef ? 1 : 0);
        for (int sh = 0; sh < ncand && !rc; ++sh) {
            if (order != H3D_ORDER_COLOUR27) {
                int32_t bd[3];
                int r = 1;
                const bool f64 = sizeof(T) == 8, wnc = op.wni != nullptr;
                size_t smem;
                if (order == H3D_ORDER_BLOCK) {
                    block_cfg_dims(sh, bd, &r);
                    smem = block_cfg_smem(sh, f64, wnc);
                } else {
                    block8_cfg_dims(sh, bd, &r);
                    smem = block8_cfg_smem(sh, f64, wnc);
                }
                // only groups the right-hand sides fill, and configurations that fit
                if (r > nrhs || smem == 0) continue;
            }
            const cplx<T> *cf = (order == H3D_ORDER_COLOUR27 && sh == num_tile_shapes()) || order == H3D_ORDER_BLOCK8
                                    ? coef : nullptr;
            if ((rc = launch_sweep<T>(op, y, nullptr, nrhs, w, adj, order, block, nullptr, st, rinv, sh, cf))) break;
            cudaEventRecord(e0, st);
            for (int rep = 0; rep < 2 && !rc; ++rep)
                rc = launch_sweep<T>(op, y, nullptr, nrhs, w, adj, order, block, nullptr, st, rinv, sh, cf);
            cudaEventRecord(e1, st);
            cudaEventSynchronize(e1);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (verbose)
                fprintf(stderr, "[h3d] tune order %d candidate %d: %.3f ms per double sweep\n", order, sh, 0.5 * ms);
            if (ms < best) {
                best = ms;
                best_shape = sh;
            }
            launches += 3LL * sweep_launches();
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if (rc) return rc;
        shape = best_shape;
        tune_store(key, shape);
        settle_coefs();
        return H3D_OK;
    }

    // Keep the stored coefficients only if the chosen implementation uses them
    // (a cached choice of them without room for them falls back to the grid's tile shape).
    void settle_coefs()
    {
        if (order == H3D_ORDER_BLOCK8 && coef && shape >= 0) {
            int32_t bd[3];
            int r = 1;
            block8_cfg_dims(shape, bd, &r);
            if (bd[0] != 12 || bd[1] != 12 || bd[2] != 12) {  // only the 12^3 kernels read them
                coefs.release();
                coef = nullptr;
            }
        }
        if (order != H3D_ORDER_COLOUR27) return;
        if (shape == num_tile_shapes() && !coef) shape = pick_tile_shape(op.nx, op.ny, op.nz);
        if (shape != num_tile_shapes() && coef) {
            coefs.release();
            coef = nullptr;
        }
    }

    // Stored coefficients for the sweep launches (null: the chosen kernel does not use them).
    const cplx<T> *cf() const
    {
        if (order == H3D_ORDER_BLOCK8) return coef;
        return (order == H3D_ORDER_COLOUR27 && shape == num_tile_shapes()) ? coef : nullptr;
    }

    // b~ = DSWP(0, b) into y, then x = 0, r = p = y.
    int setup(const cplx<T> *b, const double *bnorm2_orig, double zero_tol2, cudaStream_t st)
    {
        int rc;
        if ((rc = tune(st))) return rc;
        if ((rc = zero_vec<T>(y, N, nrhs, st))) return rc;
        if ((rc = launch_sweep<T>(op, y, b, nrhs, w, adj, order, block, nullptr, st, rinv, shape, cf()))) return rc;
        launches += sweep_launches() + 2;
        if ((rc = cg_init<T>(y, x, r, p, N, nrhs, s, bnorm2_orig, zero_tol2, maxit, st))) return rc;
        if (method != H3D_METHOD_CRMN) return H3D_OK;
        // CRMN.m:54-56, 66-69 with the zero start of linearsolve: r = b~ (y holds it too),
        // Ar = A r, p = r, Ap = Ar, gamma; then the first x, r update and stop test
        // (CRMN.m:79-92).  Every later iteration starts at Ar = A r (CRMN.m:94), so a
        // right-hand side stopped by the test resumes exactly where CRMN.m would continue.
        if ((rc = zero_vec<T>(ap, N, nrhs, st))) return rc;
        if ((rc = launch_sweep<T>(op, y, nullptr, nrhs, w, adj, order, block, s.active, st, rinv, shape, cf()))) return rc;
        if ((rc = cr_ar_dot<T>(r, y, N, nrhs, s, st))) return rc;
        if ((rc = cr_update_p<T>(p, ap, r, y, N, nrhs, s, true, st))) return rc;
        if ((rc = cr_update_xr<T>(x, r, p, ap, y, N, nrhs, s, maxit, st))) return rc;
        launches += sweep_launches() + 6;
        return H3D_OK;
    }

    int enqueue_iteration(cudaStream_t st, bool timed)
    {
        int rc;
        if (method == H3D_METHOD_CRMN) {
            // CRMN.m:94-105 then 73-92: Ar = A r (y = r on entry), rAr, beta, p, Ap, ||Ap||,
            // gamma; x, r, y = r, the stop test
            if (timed) H3D_CUDA_TRY(cudaEventRecordWithFlags(ev0, st, cudaEventRecordExternal));
            if ((rc = launch_sweep<T>(op, y, nullptr, nrhs, w, adj, order, block, s.active, st, rinv, shape, cf()))) return rc;
            if (timed) H3D_CUDA_TRY(cudaEventRecordWithFlags(ev1, st, cudaEventRecordExternal));
            if ((rc = cr_ar_dot<T>(r, y, N, nrhs, s, st))) return rc;
            if ((rc = cr_update_p<T>(p, ap, r, y, N, nrhs, s, false, st))) return rc;
            return cr_update_xr<T>(x, r, p, ap, y, N, nrhs, s, maxit, st);
        }
        if (timed) H3D_CUDA_TRY(cudaEventRecordWithFlags(ev0, st, cudaEventRecordExternal));
        if ((rc = launch_sweep<T>(op, y, nullptr, nrhs, w, adj, order, block, s.active, st, rinv, shape, cf()))) return rc;
        if (timed) H3D_CUDA_TRY(cudaEventRecordWithFlags(ev1, st, cudaEventRecordExternal));
        if ((rc = cg_ap_dot<T>(p, y, N, nrhs, s, st))) return rc;
        if ((rc = cg_update_xr<T>(x, r, p, y, N, nrhs, s, maxit, st))) return rc;
        return cg_update_p<T>(p, r, y, N, nrhs, s, st);
    }

    int run_block(int iters, bool use_graph, cudaStream_t st)
    {
        if (!ev0) {
            H3D_CUDA_TRY(cudaEventCreate(&ev0));
            H3D_CUDA_TRY(cudaEventCreate(&ev1));
        }
        block_launches = (long long)iters * iteration_launches();
        if (!use_graph) {
            for (int q = 0; q < iters; ++q) {
                int rc = enqueue_iteration(st, q == iters - 1);
                if (rc) return rc;
            }
            launches += block_launches;
            timed_pending = true;
            return H3D_OK;
        }
        if (!exec || graph_iters != iters) {
            if (exec) cudaGraphExecDestroy(exec);
            exec = nullptr;
            cudaGraph_t g = nullptr;
            H3D_CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
            int rc = H3D_OK;
            for (int q = 0; q < iters && !rc; ++q) rc = enqueue_iteration(st, q == iters - 1);
            cudaError_t e = cudaStreamEndCapture(st, &g);
            if (rc) {
                if (g) cudaGraphDestroy(g);
                return rc;
            }
            if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
            e = cudaGraphInstantiate(&exec, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
            graph_iters = iters;
        }
        H3D_CUDA_TRY(cudaGraphLaunch(exec, st));
        launches += block_launches;
        timed_pending = true;
        return H3D_OK;
    }
};

struct HostState {
    std::vector<int> active, iters, status;
    std::vector<double> ratio;
    int *h_ints = nullptr;
    double *h_dbl = nullptr;
    int n = 0;
    ~HostState()
    {
        if (h_ints) cudaFreeHost(h_ints);
        if (h_dbl) cudaFreeHost(h_dbl);
    }
    int init(int nrhs)
    {
        n = nrhs;
        H3D_CUDA_TRY(cudaMallocHost(&h_ints, sizeof(int) * 3 * nrhs));
        H3D_CUDA_TRY(cudaMallocHost(&h_dbl, sizeof(double) * 4 * nrhs));
        active.resize(nrhs);
        iters.resize(nrhs);
        status.resize(nrhs);
        ratio.resize(nrhs);
        return H3D_OK;
    }
    template <typename T>
    int fetch(const CgRun<T> &cg, cudaStream_t st)
    {
        H3D_CUDA_TRY(cudaMemcpyAsync(h_ints, cg.s.active, sizeof(int) * n, cudaMemcpyDeviceToHost, st));
        H3D_CUDA_TRY(cudaMemcpyAsync(h_ints + n, cg.s.iters, sizeof(int) * n, cudaMemcpyDeviceToHost, st));
        H3D_CUDA_TRY(cudaMemcpyAsync(h_ints + 2 * n, cg.s.status, sizeof(int) * n, cudaMemcpyDeviceToHost, st));
        H3D_CUDA_TRY(cudaMemcpyAsync(h_dbl, cg.s.ratio, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
        H3D_CUDA_TRY(cudaStreamSynchronize(st));
        for (int q = 0; q < n; ++q) {
            active[q] = h_ints[q];
            iters[q] = h_ints[n + q];
            status[q] = h_ints[2 * n + q];
            ratio[q] = h_dbl[q];
        }
        return H3D_OK;
    }
};

// Run a CGMN instance until every right-hand side is inactive.
template <typename T>
static int cg_drive(CgRun<T> &cg, HostState &hs, const h3d_solve_opts &o, double *res_hist,
                    int res_hist_len, int *hist_pos, cudaStream_t st)
{
    const int per_iter = cg.sweep_launches() + 6;
    int block_iters = o.check_every > 0 ? o.check_every : 25;
    if (block_iters * per_iter > 20000) block_iters = std::max(1, 20000 / per_iter);
    for (;;) {
        int rc = hs.fetch(cg, st);
        if (rc) return rc;
        cg.harvest_timing();
        bool any = false;
        double mx = 0.0;
        for (int q = 0; q < hs.n; ++q) {
            any |= hs.active[q] != 0;
            if (hs.iters[q] > 0) mx = std::max(mx, hs.ratio[q]);
        }
        if (res_hist && hist_pos && *hist_pos < res_hist_len) res_hist[(*hist_pos)++] = mx;
        if (o.verbose) {
            int it = 0;
            for (int q = 0; q < hs.n; ++q) it = std::max(it, hs.iters[q]);
            fprintf(stderr, "[h3d] cgmn(%s) it %d max-ratio %.3e\n", sizeof(T) == 8 ? "c128" : "c64", it, mx);
        }
        if (!any) return H3D_OK;
        if ((rc = cg.run_block(block_iters, o.use_graphs != 0, st))) return rc;
    }
}

struct Timer {
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
    double seconds() const
    {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
};

// ---------------------------------------------------------------------------------------
// Core solve on an internal stream.  b, u: complex128 interleaved device vectors.
static int solve_impl(const h3d_grid *g, const double *wn_re, const double *wn_im,
                      const cplx<double> *b, cplx<double> *u, int nrhs, int mode,
                      const h3d_solve_opts &o, h3d_solve_info *info, double *res_hist,
                      int res_hist_len, cudaStream_t st)
{
    Timer timer;
    int rc;
    Op<double> op64;
    if ((rc = make_op_f64(g, wn_re, wn_im, &op64))) return rc;
    const long long N = op64.N;
    const bool adj = mode == H3D_ADJOINT;
    const double zero_tol2 = 1e-24;  // (1e-12)^2, opAbstractMatrix.m:118

    // FP64 residual machinery: r64 = b - A u, per-RHS norms.
    const int Gr = mvp_residual_parts(op64, nrhs);
    DevBuf r64b, partb, normb;
    if ((rc = r64b.alloc(sizeof(cplx<double>) * (size_t)N * nrhs, st))) return rc;
    if ((rc = partb.alloc(sizeof(double) * 2 * (size_t)Gr * nrhs, st))) return rc;
    if ((rc = normb.alloc(sizeof(double) * 2 * (size_t)nrhs, st))) return rc;
    cplx<double> *r64 = r64b.as<cplx<double>>();
    double *rr2 = normb.as<double>(), *bb2 = rr2 + nrhs;
    H3D_CUDA_TRY(cudaMemsetAsync(u, 0, sizeof(cplx<double>) * (size_t)N * nrhs, st));
    if ((rc = residual_f64(op64, b, u, r64, rr2, bb2, nrhs, adj, partb.as<double>(), Gr, st))) return rc;
    long long extra_launches = 2;
    double sw_sec = 0.0;
    int sw_n = 0, sw_variant = -1;
    long long cg_launches = 0;

    std::vector<double> h_rr(nrhs), h_bb(nrhs);
    auto fetch_norms = [&]() -> int {
        H3D_CUDA_TRY(cudaMemcpyAsync(h_rr.data(), rr2, sizeof(double) * nrhs, cudaMemcpyDeviceToHost, st));
        H3D_CUDA_TRY(cudaMemcpyAsync(h_bb.data(), bb2, sizeof(double) * nrhs, cudaMemcpyDeviceToHost, st));
        H3D_CUDA_TRY(cudaStreamSynchronize(st));
        return H3D_OK;
    };
    if ((rc = fetch_norms())) return rc;
    const std::vector<double> bnorm2 = h_bb;

    HostState hs;
    if ((rc = hs.init(nrhs))) return rc;
    int hist_pos = 0;
    int total_iters_max = 0, outer = 0;
    std::vector<int> total_iters(nrhs, 0);
    double last_prec = 0.0;
    bool nonfinite = false;
    std::vector<int> done(nrhs, 0);
    for (int q = 0; q < nrhs; ++q) done[q] = bnorm2[q] < zero_tol2;

    auto true_ok = [&](int q) { return h_bb[q] > 0 ? std::sqrt(h_rr[q] / bnorm2[q]) <= o.tol : true; };

    if (o.precision == H3D_PREC_FP64) {
        CgRun<double> cg;
        cg.op = op64;
        cg.N = N;
        cg.nrhs = nrhs;
        cg.adj = adj;
        cg.w = o.w;
        cg.order = o.order;
        std::memcpy(cg.block, o.block, sizeof cg.block);
        cg.maxit = o.maxit;
        cg.method = o.method;
        cg.verbose = o.verbose;
        if ((rc = cg.alloc(st))) return rc;
        std::vector<double> tolp(nrhs, o.tol);
        H3D_CUDA_TRY(cudaMemcpyAsync(cg.s.tolp, tolp.data(), sizeof(double) * nrhs, cudaMemcpyHostToDevice, st));
        if ((rc = cg.setup(b, bb2, zero_tol2, st))) return rc;
        for (;;) {
            if ((rc = cg_drive(cg, hs, o, res_hist, res_hist_len, &hist_pos, st))) return rc;
            ++outer;
            if ((rc = residual_f64(op64, b, cg.x, r64, rr2, nullptr, nrhs, adj, partb.as<double>(), Gr, st))) return rc;
            extra_launches += 2;
            if ((rc = fetch_norms())) return rc;
            if (o.stop_rule != H3D_STOP_TRUE_RESIDUAL) break;
            bool again = false;
            for (int q = 0; q < nrhs; ++q) {
                if (done[q] || hs.status[q] || hs.iters[q] >= o.maxit) continue;
                const double tr = std::sqrt(h_rr[q] / bnorm2[q]);
                if (tr <= o.tol) continue;
                // Not there yet on the true residual: tighten this column's preconditioned
                // tolerance in proportion and continue the same Krylov sequence.
                tolp[q] = std::max(hs.ratio[q] * (o.tol / tr) * 0.5, 1e-15);
                again = true;
            }
            if (!again || outer > o.max_outer) break;
            std::vector<int> act(nrhs, 0);
            for (int q = 0; q < nrhs; ++q)
                act[q] = (!done[q] && !hs.status[q] && hs.iters[q] < o.maxit &&
                          std::sqrt(h_rr[q] / bnorm2[q]) > o.tol);
            H3D_CUDA_TRY(cudaMemcpyAsync(cg.s.tolp, tolp.data(), sizeof(double) * nrhs, cudaMemcpyHostToDevice, st));
            H3D_CUDA_TRY(cudaMemcpyAsync(cg.s.active, act.data(), sizeof(int) * nrhs, cudaMemcpyHostToDevice, st));
            H3D_CUDA_TRY(cudaStreamSynchronize(st));
        }
        H3D_CUDA_TRY(cudaMemcpyAsync(u, cg.x, sizeof(cplx<double>) * (size_t)N * nrhs, cudaMemcpyDeviceToDevice, st));
        for (int q = 0; q < nrhs; ++q) {
            total_iters[q] = hs.iters[q];
            last_prec = std::max(last_prec, hs.ratio[q]);
            nonfinite |= hs.status[q] != 0;
        }
        sw_sec = cg.sweep_seconds;
        sw_n = cg.sweep_samples;
        sw_variant = cg.shape;
        cg_launches = cg.launches;
    } else {
        // Mixed precision: complex64 CGMN on the scaled FP64 residual, FP64 update and residual.
        DevBuf wn32b, rhs32b;
        if ((rc = wn32b.alloc(sizeof(float) * (size_t)N * (wn_im ? 2 : 1), st))) return rc;
        float *wn32 = wn32b.as<float>();
        if ((rc = cast<double, float>(wn_re, wn32, N, st))) return rc;
        if (wn_im && (rc = cast<double, float>(wn_im, wn32 + N, N, st))) return rc;
        extra_launches += wn_im ? 2 : 1;
        Op<float> op32;
        if ((rc = make_op_f32(g, wn32, wn_im ? wn32 + N : nullptr, &op32))) return rc;
        if ((rc = rhs32b.alloc(sizeof(cplx<float>) * (size_t)N * nrhs, st))) return rc;
        cplx<float> *rhs32 = rhs32b.as<cplx<float>>();
        CgRun<float> cg;
        cg.op = op32;
        cg.N = N;
        cg.nrhs = nrhs;
        cg.adj = adj;
        cg.w = (float)o.w;
        cg.order = o.order;
        std::memcpy(cg.block, o.block, sizeof cg.block);
        cg.maxit = o.maxit;
        cg.method = o.method;
        cg.verbose = o.verbose;
        if ((rc = cg.alloc(st))) return rc;
        DevBuf actb;
        if ((rc = actb.alloc(sizeof(int) * nrhs, st))) return rc;
        int *outer_active = actb.as<int>();
        std::vector<double> tolp(nrhs, o.inner_tol);
        H3D_CUDA_TRY(cudaMemcpyAsync(cg.s.tolp, tolp.data(), sizeof(double) * nrhs, cudaMemcpyHostToDevice, st));
        for (outer = 0; outer < o.max_outer; ++outer) {
            std::vector<int> act(nrhs, 0);
            bool any = false;
            for (int q = 0; q < nrhs; ++q) {
                act[q] = !done[q] && !true_ok(q) && total_iters[q] < o.maxit;
                any |= act[q] != 0;
            }
            if (!any) break;
            H3D_CUDA_TRY(cudaMemcpyAsync(outer_active, act.data(), sizeof(int) * nrhs, cudaMemcpyHostToDevice, st));
            if ((rc = scale_to_c64(r64, rhs32, N, nrhs, rr2, outer_active, st))) return rc;
            if ((rc = cg.setup(rhs32, nullptr, 0.0, st))) return rc;
            // only the columns still above tolerance iterate
            H3D_CUDA_TRY(cudaMemcpyAsync(cg.s.active, act.data(), sizeof(int) * nrhs, cudaMemcpyHostToDevice, st));
            if ((rc = cg_drive(cg, hs, o, res_hist, res_hist_len, &hist_pos, st))) return rc;
            if ((rc = add_scaled_c64(u, cg.x, N, nrhs, rr2, outer_active, st))) return rc;
            for (int q = 0; q < nrhs; ++q) {
                if (!act[q]) continue;
                total_iters[q] += hs.iters[q];
                last_prec = hs.ratio[q];
                nonfinite |= hs.status[q] != 0;
            }
            if ((rc = residual_f64(op64, b, u, r64, rr2, nullptr, nrhs, adj, partb.as<double>(), Gr, st))) return rc;
            extra_launches += 4;  // scale, add, residual (2)
            if ((rc = fetch_norms())) return rc;
            if (nonfinite) break;
        }
        sw_sec = cg.sweep_seconds;
        sw_n = cg.sweep_samples;
        sw_variant = cg.shape;
        cg_launches = cg.launches;
    }
    bool all_ok = !nonfinite;
    double worst = 0.0;
    for (int q = 0; q < nrhs; ++q) {
        total_iters_max = std::max(total_iters_max, total_iters[q]);
        if (done[q]) {
            H3D_CUDA_TRY(cudaMemsetAsync(u + (size_t)q * N, 0, sizeof(cplx<double>) * (size_t)N, st));
            continue;
        }
        const double tr = std::sqrt(h_rr[q] / bnorm2[q]);
        worst = std::max(worst, tr);
        if (o.stop_rule == H3D_STOP_TRUE_RESIDUAL ? !(tr <= o.tol) : false) all_ok = false;
    }
    H3D_CUDA_TRY(cudaStreamSynchronize(st));
    if (info) {
        info->iters = total_iters_max;
        info->outer = outer;
        info->converged = all_ok ? 1 : 0;
        info->nrhs = nrhs;
        info->rel_res_true = worst;
        info->rel_res_prec = last_prec;
        info->seconds = timer.seconds();
        info->sweep_seconds = sw_sec;
        info->sweep_samples = sw_n;
        info->sweep_variant = sw_variant;
        info->kernel_launches = extra_launches + cg_launches;
    }
    if (nonfinite) {
        set_error("non-finite value in the CGMN iteration");
        return H3D_ERR_NONFINITE;
    }
    if (!all_ok) {
        set_error("not converged: max true relative residual %.3e after %d iterations", worst, total_iters_max);
        return H3D_ERR_NOT_CONVERGED;
    }
    return H3D_OK;
}

// Run f on an internal non-blocking stream ordered after the caller's stream.
template <typename F>
static int on_internal_stream(cudaStream_t user, F f)
{
    cudaStream_t st = nullptr;
    cudaEvent_t ev = nullptr;
    H3D_CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    H3D_CUDA_TRY(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    H3D_CUDA_TRY(cudaEventRecord(ev, user));
    H3D_CUDA_TRY(cudaStreamWaitEvent(st, ev, 0));
    int rc = f(st);
    cudaError_t e1 = cudaEventRecord(ev, st);
    cudaError_t e2 = cudaStreamWaitEvent(user, ev, 0);
    cudaError_t e3 = cudaStreamSynchronize(st);
    cudaEventDestroy(ev);
    cudaStreamDestroy(st);
    if (rc) return rc;
    if (e1 != cudaSuccess) return cuda_fail(e1, "cudaEventRecord");
    if (e2 != cudaSuccess) return cuda_fail(e2, "cudaStreamWaitEvent");
    if (e3 != cudaSuccess) return cuda_fail(e3, "cudaStreamSynchronize");
    return H3D_OK;
}

static int check_opts(const h3d_solve_opts *o)
{
    if (!o) return H3D_OK;
    if (!(o->tol > 0) || o->maxit < 1 || !(o->w > 0 && o->w < 2) ||
        (o->precision != H3D_PREC_FP64 && o->precision != H3D_PREC_MIXED) || o->order < 0 ||
        o->order > 3 || (o->method != H3D_METHOD_CGMN && o->method != H3D_METHOD_CRMN) || (o->precision == H3D_PREC_MIXED && !(o->inner_tol > 0 && o->inner_tol < 1))) {
        set_error("invalid solver options");
        return H3D_ERR_BAD_ARG;
    }
    return H3D_OK;
}

}  // namespace h3d

using namespace h3d;

extern "C" {

int h3d_residual(const h3d_grid *g, const double *wn_re, const double *wn_im, const void *b,
                 const void *x, void *r, double *rr2, double *bb2, int nrhs, int mode, void *stream)
{
    if (!wn_re || !b || !x || !r || nrhs < 1 || (mode != H3D_FORWARD && mode != H3D_ADJOINT)) {
        set_error("h3d_residual: bad argument");
        return H3D_ERR_BAD_ARG;
    }
    Op<double> op;
    int rc = make_op_f64(g, wn_re, wn_im, &op);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const int G = mvp_residual_parts(op, nrhs);
    DevBuf part, norms;
    if ((rc = part.alloc(sizeof(double) * 2 * (size_t)G * nrhs, st))) return rc;
    if ((rc = norms.alloc(sizeof(double) * 2 * (size_t)nrhs, st))) return rc;
    double *n1 = norms.as<double>();
    if ((rc = residual_f64(op, (const cplx<double> *)b, (const cplx<double> *)x, (cplx<double> *)r,
                           n1, n1 + nrhs, nrhs, mode == H3D_ADJOINT, part.as<double>(), G, st)))
        return rc;
    if (rr2) H3D_CUDA_TRY(cudaMemcpyAsync(rr2, n1, sizeof(double) * nrhs, cudaMemcpyDeviceToDevice, st));
    if (bb2) H3D_CUDA_TRY(cudaMemcpyAsync(bb2, n1 + nrhs, sizeof(double) * nrhs, cudaMemcpyDeviceToDevice, st));
    return H3D_OK;
}

int h3d_solve(const h3d_grid *g, const double *wn_re, const double *wn_im, const void *b,
              void *u, int nrhs, int mode, const h3d_solve_opts *opts, h3d_solve_info *info,
              double *res_hist, int res_hist_len, void *stream)
{
    if (!wn_re || !b || !u || nrhs < 1 || (mode != H3D_FORWARD && mode != H3D_ADJOINT)) {
        set_error("h3d_solve: bad argument");
        return H3D_ERR_BAD_ARG;
    }
    int rc = check_grid(g);
    if (rc) return rc;
    if ((rc = check_opts(opts))) return rc;
    h3d_solve_opts o;
    h3d_default_opts(&o);
    if (opts) o = *opts;
    return on_internal_stream((cudaStream_t)stream, [&](cudaStream_t st) {
        return solve_impl(g, wn_re, wn_im, (const cplx<double> *)b, (cplx<double> *)u, nrhs, mode, o,
                          info, res_hist, res_hist_len, st);
    });
}

int h3d_solve_batch(const h3d_problem *probs, int nprob, const h3d_solve_opts *opts,
                    h3d_solve_info *infos, void *stream)
{
    if (!probs || nprob < 1) {
        set_error("h3d_solve_batch: bad argument");
        return H3D_ERR_BAD_ARG;
    }
    int worst = H3D_OK;
    for (int q = 0; q < nprob; ++q) {
        const h3d_problem &p = probs[q];
        int rc = h3d_solve(&p.grid, p.wn_re, p.wn_im, p.b, p.u, p.nrhs, p.mode, opts,
                           infos ? &infos[q] : nullptr, nullptr, 0, stream);
        if (rc && rc != H3D_ERR_NOT_CONVERGED) return rc;
        if (rc) worst = rc;
    }
    return worst;
}

int h3d_solve_host(const h3d_grid *g, const double *wn_re, const double *wn_im,
                   const void *b_host, void *u_host, int nrhs, int mode,
                   const h3d_solve_opts *opts, h3d_solve_info *info)
{
    int rc = check_grid(g);
    if (rc) return rc;
    if (!wn_re || !b_host || !u_host || nrhs < 1) {
        set_error("h3d_solve_host: bad argument");
        return H3D_ERR_BAD_ARG;
    }
    const long long N = (long long)g->n[0] * g->n[1] * g->n[2];
    return on_internal_stream(nullptr, [&](cudaStream_t st) -> int {
        DevBuf dw, db, du;
        int r;
        const size_t wb = sizeof(double) * (size_t)N;
        const size_t vb = sizeof(cplx<double>) * (size_t)N * nrhs;
        if ((r = dw.alloc(wb * (wn_im ? 2 : 1), st)) || (r = db.alloc(vb, st)) || (r = du.alloc(vb, st)))
            return r;
        H3D_CUDA_TRY(cudaMemcpyAsync(dw.p, wn_re, wb, cudaMemcpyHostToDevice, st));
        if (wn_im) H3D_CUDA_TRY(cudaMemcpyAsync(dw.as<double>() + N, wn_im, wb, cudaMemcpyHostToDevice, st));
        H3D_CUDA_TRY(cudaMemcpyAsync(db.p, b_host, vb, cudaMemcpyHostToDevice, st));
        r = h3d_solve(g, dw.as<double>(), wn_im ? dw.as<double>() + N : nullptr, db.p, du.p, nrhs, mode,
                      opts, info, nullptr, 0, st);
        if (r && r != H3D_ERR_NOT_CONVERGED) return r;
        H3D_CUDA_TRY(cudaMemcpyAsync(u_host, du.p, vb, cudaMemcpyDeviceToHost, st));
        H3D_CUDA_TRY(cudaStreamSynchronize(st));
        if (info) {
            // the copies are part of the call
        }
        return r;
    });
}

}  // extern "C"
