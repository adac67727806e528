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
//
// With the BLOCK8 order (12^3 blocks, stored coefficients in device memory) one CGMN
// instance iterates every column of a table of problems at once: the problems' columns
// sit one after another in each CG vector (problem-major), the vector kernels follow a
// per-column offset and length, and one batched sweep launch per block parity covers all
// problems (h3d_b8batch.cu).  Problems may differ in grid, PML, wavenumber and mode.
#include <algorithm>
#include <chrono>
#include <type_traits>
#include <map>
#include <mutex>
#include <tuple>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "h3d_b8.cuh"
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
    long long N = 0;   // column length (batched: the longest column)
    long long L = 0;   // elements of each CG vector (N nrhs, or the batch's total)
    int nrhs = 0;      // columns
    B8Batch<T> *b8 = nullptr;           // batched BLOCK8 sweeps (null: sweeps of op)
    std::vector<long long> coloff, collen;  // batched: column map (host copy)
    std::vector<int> colprob;               // batched: problem of each column
    bool b8_tuned = false;
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
    DevBuf vecs, scal, ints, parts, norms, coefs, cmap;
    cudaGraphExec_t exec = nullptr;
    int graph_iters = 0;
    // Timing of the last double sweep of every replayed block: two timing events recorded
    // as event nodes of the graph, read after the block completes.
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    bool timed_pending = false;
    double sweep_seconds = 0.0;
    int sweep_samples = 0;
    double pending_bytes = 0.0;  // algorithmic bytes of the timed sweep of the running block
    double sweep_bytes = 0.0;
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
            sweep_bytes += pending_bytes;
            ++sweep_samples;
        }
        timed_pending = false;
    }

    int alloc(cudaStream_t st)
    {
        if (!b8) L = N * nrhs;
        const size_t vb = sizeof(cplx<T>) * (size_t)L;
        int rc;
        const bool cr = method == H3D_METHOD_CRMN;
        if ((rc = vecs.alloc((cr ? 5 : 4) * vb, st))) return rc;
        x = vecs.as<cplx<T>>();
        r = x + L;
        p = r + L;
        y = p + L;
        ap = cr ? y + L : nullptr;
        s.G = reduction_blocks(N);
        if (b8) {
            if ((rc = cmap.alloc(sizeof(long long) * 2 * (size_t)nrhs, st))) return rc;
            std::vector<long long> h(coloff);
            h.insert(h.end(), collen.begin(), collen.end());
            // pageable source: staged before the call returns
            H3D_CUDA_TRY(cudaMemcpyAsync(cmap.p, h.data(), sizeof(long long) * h.size(), cudaMemcpyHostToDevice, st));
            s.coloff = cmap.as<long long>();
            s.collen = s.coloff + nrhs;
        }
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
        if (b8) return H3D_OK;  // the batch holds its own coefficients and row norms
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

    // One double sweep of v with right-hand side b (null = 0) over the active columns.
    int sweep(cplx<T> *v, const cplx<T> *b, const int *act, cudaStream_t st)
    {
        if (b8) return b8->dsweep(v, b, w, act, st);
        return launch_sweep<T>(op, v, b, nrhs, w, adj, order, block, act, st, rinv, shape, cf());
    }

    // Algorithmic bytes of one double sweep over the columns flagged in act (host flags):
    // 2 (read + write) complex values of x per active column and point, plus one read of
    // the wavenumber per point of every problem with an active column, in each direction.
    double dsweep_bytes(const std::vector<int> &act) const
    {
        const double sc = sizeof(cplx<T>);
        if (!b8) {
            long long na = 0;
            for (int c = 0; c < nrhs; ++c) na += act[c] != 0;
            const double sw = sizeof(T) * (op.wni ? 2 : 1);
            return na ? 2.0 * (double)N * (2.0 * sc * na + sw) : 0.0;
        }
        double bytes = 0.0;
        std::vector<char> seen(b8->items.size(), 0);
        for (int c = 0; c < nrhs; ++c) {
            if (!act[c]) continue;
            bytes += 2.0 * (double)collen[c] * 2.0 * sc;
            const int q = colprob[c];
            if (!seen[q]) {
                seen[q] = 1;
                bytes += 2.0 * (double)collen[c] * sizeof(T) * (b8->items[q].op.wni ? 2 : 1);
            }
        }
        return bytes;
    }

    int sweep_launches() const
    {
        if (b8) return b8->launches();
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
        if (b8) {
            if (b8_tuned) return H3D_OK;
            b8_tuned = true;
            const int rc = b8->tune(y, L, st);
            launches += 5LL * sweep_launches();  // upper bound: at most the configurations the columns fill
            shape = b8->cfg;
            return rc;
        }
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
        if ((rc = zero_vec<T>(y, L, 1, st))) return rc;
        if ((rc = sweep(y, b, nullptr, st))) return rc;
        launches += sweep_launches() + 2;
        if ((rc = cg_init<T>(y, x, r, p, N, nrhs, s, bnorm2_orig, zero_tol2, maxit, st))) return rc;
        if (method != H3D_METHOD_CRMN) return H3D_OK;
        // CRMN.m:54-56, 66-69 with the zero start of linearsolve: r = b~ (y holds it too),
        // Ar = A r, p = r, Ap = Ar, gamma; then the first x, r update and stop test
        // (CRMN.m:79-92).  Every later iteration starts at Ar = A r (CRMN.m:94), so a
        // right-hand side stopped by the test resumes exactly where CRMN.m would continue.
        if ((rc = zero_vec<T>(ap, L, 1, st))) return rc;
        if ((rc = sweep(y, nullptr, s.active, st))) return rc;
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
            if ((rc = sweep(y, nullptr, s.active, st))) return rc;
            if (timed) H3D_CUDA_TRY(cudaEventRecordWithFlags(ev1, st, cudaEventRecordExternal));
            if ((rc = cr_ar_dot<T>(r, y, N, nrhs, s, st))) return rc;
            if ((rc = cr_update_p<T>(p, ap, r, y, N, nrhs, s, false, st))) return rc;
            return cr_update_xr<T>(x, r, p, ap, y, N, nrhs, s, maxit, st);
        }
        if (timed) H3D_CUDA_TRY(cudaEventRecordWithFlags(ev0, st, cudaEventRecordExternal));
        if ((rc = sweep(y, nullptr, s.active, st))) return rc;
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
        H3D_CUDA_TRY(cudaMallocHost(&h_ints, sizeof(int) * (3 * nrhs + 1)));
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
        if (cg.b8) H3D_CUDA_TRY(cudaMemcpyAsync(h_ints + 3 * n, cg.b8->err, sizeof(int), cudaMemcpyDeviceToHost, st));
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
        if (cg.b8 && h_ints[3 * n]) {
            set_error("a bounded wait of the batched BLOCK8 sweep expired (device status %d)", h_ints[3 * n]);
            return H3D_ERR_TIMEOUT;
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
        cg.pending_bytes = cg.dsweep_bytes(hs.active);
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
// One problem of a solve call: grid, FP64 wavenumber, complex128 b and u (device), columns.
struct SolveProb {
    h3d_grid g;
    const double *wn_re, *wn_im;
    const cplx<double> *b;
    cplx<double> *u;
    int nrhs, mode;
};

// Whether the problems run as one batched BLOCK8 solve: the order is BLOCK8 with the default
// 12^3 blocks and the stored coefficients of every problem take at most half of the free
// device memory.
static bool use_batched_block8(const std::vector<SolveProb> &P, const h3d_solve_opts &o)
{
    if (o.order != H3D_ORDER_BLOCK8) return false;
    const int32_t *bk = o.block;
    if (!(bk[0] <= 0 || (bk[0] == 12 && bk[1] == 12 && bk[2] == 12))) return false;
    size_t need = 0;
    const size_t cs = o.precision == H3D_PREC_FP64 ? 16 : 8;
    for (const SolveProb &p : P) {
        const size_t nb = (size_t)((p.g.n[0] + 11) / 12) * ((p.g.n[1] + 11) / 12) * ((p.g.n[2] + 11) / 12) * 27 * 64;
        need += nb * (27 * cs + cs / 2) + (size_t)p.g.n[0] * p.g.n[1] * p.g.n[2] * (cs / 2);
    }
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
        (void)cudaGetLastError();
        return false;
    }
    return need <= fr / 2;
}

// Core solve of one or more problems on an internal stream.  With several problems the
// order must be the batched BLOCK8 one (use_batched_block8).  infos: one entry per problem
// (or null); the wall time is that of the whole call.
static int solve_impl(const std::vector<SolveProb> &P, const h3d_solve_opts &o, h3d_solve_info *infos,
                      double *res_hist, int res_hist_len, cudaStream_t st)
{
    Timer timer;
    int rc;
    const int np = (int)P.size();
    const bool batched = use_batched_block8(P, o);
    if (np > 1 && !batched) {
        set_error("internal: several problems need the batched BLOCK8 solver");
        return H3D_ERR_BAD_ARG;
    }
    std::vector<Op<double>> op64(np);
    std::vector<long long> col0(np), Np(np);
    std::vector<int> c0(np), Gr(np);
    std::vector<size_t> poff(np);
    long long L = 0, Nmax = 0;
    int C = 0;
    size_t ptot = 0;
    for (int q = 0; q < np; ++q) {
        if ((rc = make_op_f64(&P[q].g, P[q].wn_re, P[q].wn_im, &op64[q]))) return rc;
        Np[q] = op64[q].N;
        col0[q] = L;
        c0[q] = C;
        L += Np[q] * P[q].nrhs;
        C += P[q].nrhs;
        Nmax = std::max(Nmax, Np[q]);
        Gr[q] = mvp_residual_parts(op64[q], P[q].nrhs);
        poff[q] = ptot;
        ptot += 2 * (size_t)Gr[q] * P[q].nrhs;
    }
    const double zero_tol2 = 1e-24;  // (1e-12)^2, opAbstractMatrix.m:118
    std::vector<int> colp(C);        // problem of each column
    for (int q = 0; q < np; ++q)
        for (int j = 0; j < P[q].nrhs; ++j) colp[c0[q] + j] = q;

    // FP64 residual machinery: r64 = b - A u per problem (columns in the batch layout),
    // per-column norms.
    DevBuf r64b, partb, normb;
    if ((rc = r64b.alloc(sizeof(cplx<double>) * (size_t)L, st))) return rc;
    if ((rc = partb.alloc(sizeof(double) * ptot, st))) return rc;
    if ((rc = normb.alloc(sizeof(double) * 2 * (size_t)C, st))) return rc;
    cplx<double> *r64 = r64b.as<cplx<double>>();
    double *rr2 = normb.as<double>(), *bb2 = rr2 + C;
    long long extra_launches = 0;
    // r = b - A u for every problem; u_of(q) gives problem q's current solution columns
    auto residual_all = [&](auto u_of, bool with_b) -> int {
        for (int q = 0; q < np; ++q) {
            int r = residual_f64(op64[q], P[q].b, u_of(q), r64 + col0[q], rr2 + c0[q], with_b ? bb2 + c0[q] : nullptr,
                                 P[q].nrhs, P[q].mode == H3D_ADJOINT, partb.as<double>() + poff[q], Gr[q], st);
            if (r) return r;
        }
        extra_launches += 2 * np;
        return H3D_OK;
    };
    for (int q = 0; q < np; ++q)
        H3D_CUDA_TRY(cudaMemsetAsync(P[q].u, 0, sizeof(cplx<double>) * (size_t)Np[q] * P[q].nrhs, st));
    if ((rc = residual_all([&](int q) { return (const cplx<double> *)P[q].u; }, true))) return rc;
    double sw_sec = 0.0, sw_bytes = 0.0;
    int sw_n = 0, sw_variant = -1;
    long long cg_launches = 0;

    std::vector<double> h_rr(C), h_bb(C);
    auto fetch_norms = [&]() -> int {
        H3D_CUDA_TRY(cudaMemcpyAsync(h_rr.data(), rr2, sizeof(double) * C, cudaMemcpyDeviceToHost, st));
        H3D_CUDA_TRY(cudaMemcpyAsync(h_bb.data(), bb2, sizeof(double) * C, cudaMemcpyDeviceToHost, st));
        H3D_CUDA_TRY(cudaStreamSynchronize(st));
        return H3D_OK;
    };
    if ((rc = fetch_norms())) return rc;
    const std::vector<double> bnorm2 = h_bb;

    HostState hs;
    if ((rc = hs.init(C))) return rc;
    int hist_pos = 0;
    int outer = 0;
    std::vector<int> total_iters(C, 0);
    std::vector<double> last_prec(C, 0.0);
    bool nonfinite = false;
    std::vector<int> done(C, 0);
    for (int c = 0; c < C; ++c) done[c] = bnorm2[c] < zero_tol2;

    auto true_ok = [&](int c) { return h_bb[c] > 0 ? std::sqrt(h_rr[c] / bnorm2[c]) <= o.tol : true; };
    // the batch's CGMN instance over all columns
    auto configure = [&](auto &cg, auto &batch, const auto &ops) -> int {
        using TT = std::decay_t<decltype(cg.w)>;
        cg.N = batched ? Nmax : Np[0];
        cg.nrhs = C;
        cg.w = (TT)o.w;
        cg.order = o.order;
        std::memcpy(cg.block, o.block, sizeof cg.block);
        cg.maxit = o.maxit;
        cg.method = o.method;
        cg.verbose = o.verbose;
        if (batched) {
            for (int q = 0; q < np; ++q) batch.add(ops[q], P[q].mode == H3D_ADJOINT, col0[q], c0[q], P[q].nrhs);
            batch.verbose = o.verbose;
            int r = batch.setup(st);
            if (r) return r;
            cg.b8 = &batch;
            cg.L = L;
            cg.coloff.resize(C);
            cg.collen.resize(C);
            cg.colprob = colp;
            for (int c = 0; c < C; ++c) {
                const int q = colp[c];
                cg.coloff[c] = col0[q] + (long long)(c - c0[q]) * Np[q];
                cg.collen[c] = Np[q];
            }
        } else {
            cg.op = ops[0];
            cg.adj = P[0].mode == H3D_ADJOINT;
        }
        return cg.alloc(st);
    };

    if (o.precision == H3D_PREC_FP64) {
        CgRun<double> cg;
        B8Batch<double> batch;
        if ((rc = configure(cg, batch, op64))) return rc;
        // the right-hand sides in the batch layout (one problem: b itself)
        DevBuf bcat;
        const cplx<double> *bb = P[0].b;
        if (np > 1) {
            if ((rc = bcat.alloc(sizeof(cplx<double>) * (size_t)L, st))) return rc;
            for (int q = 0; q < np; ++q)
                H3D_CUDA_TRY(cudaMemcpyAsync(bcat.as<cplx<double>>() + col0[q], P[q].b,
                                             sizeof(cplx<double>) * (size_t)Np[q] * P[q].nrhs, cudaMemcpyDeviceToDevice, st));
            bb = bcat.as<cplx<double>>();
        }
        std::vector<double> tolp(C, o.tol);
        H3D_CUDA_TRY(cudaMemcpyAsync(cg.s.tolp, tolp.data(), sizeof(double) * C, cudaMemcpyHostToDevice, st));
        if ((rc = cg.setup(bb, bb2, zero_tol2, st))) return rc;
        for (;;) {
            if ((rc = cg_drive(cg, hs, o, res_hist, res_hist_len, &hist_pos, st))) return rc;
            ++outer;
            if ((rc = residual_all([&](int q) { return (const cplx<double> *)(cg.x + col0[q]); }, false))) return rc;
            if ((rc = fetch_norms())) return rc;
            if (o.stop_rule != H3D_STOP_TRUE_RESIDUAL) break;
            bool again = false;
            for (int c = 0; c < C; ++c) {
                if (done[c] || hs.status[c] || hs.iters[c] >= o.maxit) continue;
                const double tr = std::sqrt(h_rr[c] / bnorm2[c]);
                if (tr <= o.tol) continue;
                // Not there yet on the true residual: tighten this column's preconditioned
                // tolerance in proportion and continue the same Krylov sequence.
                tolp[c] = std::max(hs.ratio[c] * (o.tol / tr) * 0.5, 1e-15);
                again = true;
            }
            if (!again || outer > o.max_outer) break;
            std::vector<int> act(C, 0);
            for (int c = 0; c < C; ++c)
                act[c] = (!done[c] && !hs.status[c] && hs.iters[c] < o.maxit && std::sqrt(h_rr[c] / bnorm2[c]) > o.tol);
            H3D_CUDA_TRY(cudaMemcpyAsync(cg.s.tolp, tolp.data(), sizeof(double) * C, cudaMemcpyHostToDevice, st));
            H3D_CUDA_TRY(cudaMemcpyAsync(cg.s.active, act.data(), sizeof(int) * C, cudaMemcpyHostToDevice, st));
            H3D_CUDA_TRY(cudaStreamSynchronize(st));
        }
        for (int q = 0; q < np; ++q)
            H3D_CUDA_TRY(cudaMemcpyAsync(P[q].u, cg.x + col0[q], sizeof(cplx<double>) * (size_t)Np[q] * P[q].nrhs,
                                         cudaMemcpyDeviceToDevice, st));
        for (int c = 0; c < C; ++c) {
            total_iters[c] = hs.iters[c];
            last_prec[c] = hs.ratio[c];
            nonfinite |= hs.status[c] != 0;
        }
        sw_sec = cg.sweep_seconds;
        sw_bytes = cg.sweep_bytes;
        sw_n = cg.sweep_samples;
        sw_variant = cg.shape;
        cg_launches = cg.launches;
    } else {
        // Mixed precision: complex64 CGMN on the scaled FP64 residual, FP64 update and residual.
        long long wtot = 0;
        for (int q = 0; q < np; ++q) wtot += Np[q] * (P[q].wn_im ? 2 : 1);
        DevBuf wn32b, rhs32b;
        if ((rc = wn32b.alloc(sizeof(float) * (size_t)wtot, st))) return rc;
        std::vector<Op<float>> op32(np);
        long long wo = 0;
        for (int q = 0; q < np; ++q) {
            float *w32 = wn32b.as<float>() + wo;
            if ((rc = cast<double, float>(P[q].wn_re, w32, Np[q], st))) return rc;
            if (P[q].wn_im && (rc = cast<double, float>(P[q].wn_im, w32 + Np[q], Np[q], st))) return rc;
            extra_launches += P[q].wn_im ? 2 : 1;
            if ((rc = make_op_f32(&P[q].g, w32, P[q].wn_im ? w32 + Np[q] : nullptr, &op32[q]))) return rc;
            wo += Np[q] * (P[q].wn_im ? 2 : 1);
        }
        if ((rc = rhs32b.alloc(sizeof(cplx<float>) * (size_t)L, st))) return rc;
        cplx<float> *rhs32 = rhs32b.as<cplx<float>>();
        CgRun<float> cg;
        B8Batch<float> batch;
        if ((rc = configure(cg, batch, op32))) return rc;
        DevBuf actb;
        if ((rc = actb.alloc(sizeof(int) * C, st))) return rc;
        int *outer_active = actb.as<int>();
        std::vector<double> tolp(C, o.inner_tol);
        H3D_CUDA_TRY(cudaMemcpyAsync(cg.s.tolp, tolp.data(), sizeof(double) * C, cudaMemcpyHostToDevice, st));
        // Later refinement steps only have to close the gap the earlier ones left: on config 1 the
        // first step (to 1e-4) takes 651 iterations and leaves a true residual of 1.1e-3, the
        // second, to 1e-4 again, 2285; aiming it at half the remaining factor (tol / residual,
        // tolerance 4.4e-4) takes 1920 and still lands at 7.2e-7.
        constexpr double kInnerSafety = 0.5, kInnerCeil = 0.1;
        for (outer = 0; outer < o.max_outer; ++outer) {
            std::vector<int> act(C, 0);
            bool any = false;
            for (int c = 0; c < C; ++c) {
                act[c] = !done[c] && !true_ok(c) && total_iters[c] < o.maxit;
                any |= act[c] != 0;
            }
            if (!any) break;
            H3D_CUDA_TRY(cudaMemcpyAsync(outer_active, act.data(), sizeof(int) * C, cudaMemcpyHostToDevice, st));
            if (outer > 0) {
                // the relative tolerance of a later step follows the column's current true
                // residual: never tighter than inner_tol, and at least a tenfold reduction
                for (int c = 0; c < C; ++c) {
                    if (!act[c]) continue;
                    const double tr = std::sqrt(h_rr[c] / bnorm2[c]);
                    tolp[c] = std::min(kInnerCeil, std::max(o.inner_tol, kInnerSafety * o.tol / tr));
                }
                H3D_CUDA_TRY(cudaMemcpyAsync(cg.s.tolp, tolp.data(), sizeof(double) * C, cudaMemcpyHostToDevice, st));
            }
            for (int q = 0; q < np; ++q)
                if ((rc = scale_to_c64(r64 + col0[q], rhs32 + col0[q], Np[q], P[q].nrhs, rr2 + c0[q], outer_active + c0[q], st)))
                    return rc;
            if ((rc = cg.setup(rhs32, nullptr, 0.0, st))) return rc;
            // only the columns still above tolerance iterate
            H3D_CUDA_TRY(cudaMemcpyAsync(cg.s.active, act.data(), sizeof(int) * C, cudaMemcpyHostToDevice, st));
            if ((rc = cg_drive(cg, hs, o, res_hist, res_hist_len, &hist_pos, st))) return rc;
            for (int q = 0; q < np; ++q)
                if ((rc = add_scaled_c64(P[q].u, cg.x + col0[q], Np[q], P[q].nrhs, rr2 + c0[q], outer_active + c0[q], st)))
                    return rc;
            for (int c = 0; c < C; ++c) {
                if (!act[c]) continue;
                total_iters[c] += hs.iters[c];
                last_prec[c] = hs.ratio[c];
                nonfinite |= hs.status[c] != 0;
            }
            if ((rc = residual_all([&](int q) { return (const cplx<double> *)P[q].u; }, false))) return rc;
            extra_launches += 2 * np;  // scale, add
            if ((rc = fetch_norms())) return rc;
            if (o.verbose) {
                double wt = 0.0;
                int it = 0;
                for (int c = 0; c < C; ++c)
                    if (act[c]) {
                        wt = std::max(wt, std::sqrt(h_rr[c] / bnorm2[c]));
                        it = std::max(it, hs.iters[c]);
                    }
                fprintf(stderr, "[h3d] refinement step %d: %d inner iterations, max true residual %.3e\n", outer, it, wt);
            }
            if (nonfinite) break;
        }
        sw_sec = cg.sweep_seconds;
        sw_bytes = cg.sweep_bytes;
        sw_n = cg.sweep_samples;
        sw_variant = cg.shape;
        cg_launches = cg.launches;
    }
    bool all_ok = !nonfinite;
    std::vector<double> worst(np, 0.0), prec(np, 0.0);
    std::vector<int> iters_max(np, 0);
    std::vector<bool> ok(np, !nonfinite);
    for (int c = 0; c < C; ++c) {
        const int q = colp[c];
        iters_max[q] = std::max(iters_max[q], total_iters[c]);
        prec[q] = std::max(prec[q], last_prec[c]);
        if (done[c]) {
            H3D_CUDA_TRY(cudaMemsetAsync(P[q].u + (size_t)(c - c0[q]) * Np[q], 0, sizeof(cplx<double>) * (size_t)Np[q], st));
            continue;
        }
        const double tr = std::sqrt(h_rr[c] / bnorm2[c]);
        worst[q] = std::max(worst[q], tr);
        if (o.stop_rule == H3D_STOP_TRUE_RESIDUAL ? !(tr <= o.tol) : false) {
            all_ok = false;
            ok[q] = false;
        }
    }
    H3D_CUDA_TRY(cudaStreamSynchronize(st));
    const double secs = timer.seconds();
    for (int q = 0; infos && q < np; ++q) {
        h3d_solve_info &in = infos[q];
        in.iters = iters_max[q];
        in.outer = outer;
        in.converged = ok[q] ? 1 : 0;
        in.nrhs = P[q].nrhs;
        in.rel_res_true = worst[q];
        in.rel_res_prec = prec[q];
        in.seconds = secs;
        // the batch's sweep timing and launch count go to the first problem's entry only, so
        // that sums over the entries count them once
        in.sweep_seconds = q == 0 ? sw_sec : 0.0;
        in.sweep_bytes = q == 0 ? sw_bytes : 0.0;
        in.sweep_samples = q == 0 ? sw_n : 0;
        in.sweep_variant = sw_variant;
        in.kernel_launches = q == 0 ? extra_launches + cg_launches : 0;
    }
    if (nonfinite) {
        set_error("non-finite value in the CGMN iteration");
        return H3D_ERR_NONFINITE;
    }
    if (!all_ok) {
        double w = 0.0;
        int it = 0;
        for (int q = 0; q < np; ++q) {
            w = std::max(w, worst[q]);
            it = std::max(it, iters_max[q]);
        }
        set_error("not converged: max true relative residual %.3e after %d iterations", w, it);
        return H3D_ERR_NOT_CONVERGED;
    }
    return H3D_OK;
}

// The calling thread's internal non-blocking stream and event on the current device, created
// on first use and kept for the thread's lifetime (solves of the FWI layer come in long runs).
struct InternalStream {
    int dev = -1;
    cudaStream_t st = nullptr;
    cudaEvent_t ev = nullptr;
    ~InternalStream() { release(); }
    void release()
    {
        if (ev) cudaEventDestroy(ev);
        if (st) cudaStreamDestroy(st);
        ev = nullptr;
        st = nullptr;
    }
    int get(cudaStream_t *s, cudaEvent_t *e)
    {
        int d = 0;
        H3D_CUDA_TRY(cudaGetDevice(&d));
        if (d != dev || !st) {
            release();
            H3D_CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
            H3D_CUDA_TRY(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
            dev = d;
        }
        *s = st;
        *e = ev;
        return H3D_OK;
    }
};
static thread_local InternalStream g_internal;

// Run f on the internal stream, ordered after the caller's stream and before its later work.
template <typename F>
static int on_internal_stream(cudaStream_t user, F f)
{
    cudaStream_t st = nullptr;
    cudaEvent_t ev = nullptr;
    int rc = g_internal.get(&st, &ev);
    if (rc) return rc;
    H3D_CUDA_TRY(cudaEventRecord(ev, user));
    H3D_CUDA_TRY(cudaStreamWaitEvent(st, ev, 0));
    rc = f(st);
    cudaError_t e1 = cudaEventRecord(ev, st);
    cudaError_t e2 = cudaStreamWaitEvent(user, ev, 0);
    cudaError_t e3 = cudaStreamSynchronize(st);
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
    std::vector<SolveProb> P{{*g, wn_re, wn_im, (const cplx<double> *)b, (cplx<double> *)u, nrhs, mode}};
    return on_internal_stream((cudaStream_t)stream,
                              [&](cudaStream_t st) { return solve_impl(P, o, info, res_hist, res_hist_len, st); });
}

int h3d_solve_batch(const h3d_problem *probs, int nprob, const h3d_solve_opts *opts,
                    h3d_solve_info *infos, void *stream)
{
    if (!probs || nprob < 1) {
        set_error("h3d_solve_batch: bad argument");
        return H3D_ERR_BAD_ARG;
    }
    int rc;
    if ((rc = check_opts(opts))) return rc;
    h3d_solve_opts o;
    h3d_default_opts(&o);
    if (opts) o = *opts;
    std::vector<SolveProb> P;
    for (int q = 0; q < nprob; ++q) {
        const h3d_problem &p = probs[q];
        if ((rc = check_grid(&p.grid))) return rc;
        if (!p.wn_re || !p.b || !p.u || p.nrhs < 1 || (p.mode != H3D_FORWARD && p.mode != H3D_ADJOINT)) {
            set_error("h3d_solve_batch: bad argument in problem %d", q);
            return H3D_ERR_BAD_ARG;
        }
        P.push_back({p.grid, p.wn_re, p.wn_im, (const cplx<double> *)p.b, (cplx<double> *)p.u, p.nrhs, p.mode});
    }
    return on_internal_stream((cudaStream_t)stream, [&](cudaStream_t st) -> int {
        // all problems in one batched BLOCK8 solve when the order and memory allow it,
        // otherwise one solve after another
        if (nprob > 1 && use_batched_block8(P, o)) return solve_impl(P, o, infos, nullptr, 0, st);
        int worst = H3D_OK;
        for (int q = 0; q < nprob; ++q) {
            std::vector<SolveProb> one{P[q]};
            int r = solve_impl(one, o, infos ? &infos[q] : nullptr, nullptr, 0, st);
            if (r && r != H3D_ERR_NOT_CONVERGED) return r;
            if (r) worst = r;
        }
        return worst;
    });
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
