// FGMRES preconditioned by the ML_GMRES multigrid V-cycle: the 3D applications' default
// Helmholtz solver (linearsolve.m:139-141 with SOLVE_FGMRES, discrete_helmholtz.m:349-350 with
// PREC_MLGMRES).
//
//   FGMRES        FGMRES.m:33-129: restarted flexible GMRES; classical Gram-Schmidt, the
//                 (k+1) x k least-squares problem solved after every step, the quasi-residual
//                 norm(beta e1 - H y) / normr0 as the inner stopping test, the true residual
//                 b - A x after every cycle as the outer one
//   ML_GMRES      ML_GMRES.m:36-72: smoother = FGMRES, 3 cycles of 5 steps to 1e-6, no
//                 preconditioner; coarse solver = FGMRES, 3 x 5 to 0.5 (opts.k overrides)
//   V-cycle       opMultigrid.m with recursive_v_cycle, GMG_V.m: smooth from zero, residual,
//                 restrict, coarse solve (preconditioned by the next level's V-cycle; on the
//                 last level by an unpreconditioned coarse-solver FGMRES), prolongate and add,
//                 smooth again from there
//
// GB300 layout of the work.  Every vector of every level stays on the device.  Each FGMRES
// instance (the outer solve, the smoother and coarse solver of every level, the last level's
// inner solver) owns its Krylov basis, a partial-sum buffer and a small state block
// (FgState) in device memory.  An Arnoldi step is three launches: the matvec, the k inner
// products V^H w (per-CTA partial sums), and the orthogonalisation w -= V h fused with the final
// sum of those partials and with ||w||^2 partials, whose last CTA applies the previous Givens
// rotations to the new Hessenberg column, forms the next rotation and updates the rotated
// right-hand side and the quasi-residual.  The basis is kept unnormalised with a scale per
// vector in the unpreconditioned instances; the preconditioned ones (whose basis vectors feed
// the V-cycle) add a fourth launch, the scaling V(:,k+1) = w / ||w||.  The Givens update gives
// the least-squares residual norm of FGMRES.m:111-113 without a host round trip; the solution y
// is back-substituted once per cycle, in the update of x.  Every kernel after the matvec reads
// a flag of the state block (the step runs / the cycle runs) and returns at once when it is
// clear, so the host enqueues a whole unpreconditioned cycle without waiting: it
// synchronises once per cycle there, and before each step of a preconditioned instance (to
// decide whether the expensive preconditioner runs at all).  Sums are deterministic: fixed
// per-thread and per-warp sums in the field's precision, then per-CTA partials and their
// totals in FP64 in a fixed order.
//
// The mixed precision of the Python front end carries over: the outer FGMRES in complex128,
// the V-cycle (all levels, smoothers and coarse solves) in complex64 with FP64 inner products.
#include <chrono>
#include <cmath>
#include <functional>

#include "h3d_kernels.cuh"
#include "h3d_vec.cuh"

namespace h3d {
namespace {

constexpr int kMaxM = 16;       // steps per cycle the state block holds
constexpr int kMaxLevels = 8;
constexpr int kThr = 256;

struct FgHead {                 // the part of the state the host reads
    int live;                   // the cycle loop goes on (FGMRES.m:88 and :125)
    int go;                     // the next Arnoldi step runs (FGMRES.m:97)
    int k;                      // steps done in the current cycle
    int it;                     // it_counter (FGMRES.m:74)
    int nhst;                   // quasi-residuals recorded (the leading 1 not counted)
    int conv;                   // stopped on the tolerance (quasi- or true residual)
    double normr0, beta, hst, rn;
};

struct FgState {
    FgHead hd;
    double hn;                  // ||w|| of the current step = H(k+1,k)
    double rhn, rbeta;          // 1 / hn and 1 / beta (0 when the norm is 0)
    double rnormr0;             // 1 / normr0
    double sv[kMaxM];           // basis vector j = sv[j] x stored vector j (1 when stored normalised)
    int ticket;                 // CTAs of the current orthogonalisation launch that have finished
    double gres;                // |g(k+1)|: the current quasi-residual norm (before / normr0)
    double cs[kMaxM];           // Givens rotations: cosines (real) ...
    cplx<double> sn[kMaxM];     // ... and sines
    cplx<double> g[kMaxM + 1];  // rotated beta e1
    cplx<double> R[kMaxM * kMaxM];  // rotated Hessenberg, column j at R + j * kMaxM
    cplx<double> h[kMaxM];      // V^H w of the current step
    cplx<double> y[kMaxM];      // least-squares solution of the current cycle
};

__device__ __forceinline__ bool closed(const int *gate) { return gate && *gate == 0; }

// Block-wide sum of two per-thread values kept in the field's precision T: warp shuffles in T,
// the eight per-warp results added in FP64 by thread 0 in a fixed order (valid there).  GB300
// executes FP64 at a small fraction of its FP32 rate, so the complex64 cycle's vector kernels
// form products and per-thread sums in FP32 (as a complex64 BLAS would) and leave FP64 to the
// few values per CTA; the complex128 instances stay FP64 throughout.
template <typename T>
__device__ __forceinline__ double2 block_sum_t(T a, T b)
{
    __shared__ double sa[kThr / 32], sb[kThr / 32];
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        b += __shfl_down_sync(0xffffffffu, b, o);
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) {
        sa[wid] = (double)a;
        sb[wid] = (double)b;
    }
    __syncthreads();
    double x = 0.0, y = 0.0;
    if (threadIdx.x == 0)
        for (int q = 0; q < kThr / 32; ++q) {
            x += sa[q];
            y += sb[q];
        }
    __syncthreads();
    return make_double2(x, y);
}

// ---- element kernels ----------------------------------------------------------------------

// r = b (x = 0 when given); per-CTA partials of ||r||^2.
template <typename T>
__global__ void __launch_bounds__(kThr) fg_copy_kernel(const cplx<T> *__restrict__ b, cplx<T> *__restrict__ r,
                                                       cplx<T> *__restrict__ x, long long n, double *part)
{
    T s = 0;
    for (long long e = blockIdx.x * (long long)kThr + threadIdx.x; e < n; e += (long long)gridDim.x * kThr) {
        const cplx<T> v = b[e];
        r[e] = v;
        if (x) x[e] = mk<T>(0, 0);
        s = fma(v.re, v.re, fma(v.im, v.im, s));
    }
    const double2 t = block_sum_t<T>(s, T(0));
    if (threadIdx.x == 0) part[blockIdx.x] = t.x;
}

// r = b - ax (r may alias ax); per-CTA partials of ||r||^2 when part is given.
template <typename T>
__global__ void __launch_bounds__(kThr) fg_sub_kernel(const cplx<T> *__restrict__ b, const cplx<T> *ax, cplx<T> *r,
                                                      long long n, double *part, const int *gate)
{
    if (closed(gate)) return;
    T s = 0;
    for (long long e = blockIdx.x * (long long)kThr + threadIdx.x; e < n; e += (long long)gridDim.x * kThr) {
        const cplx<T> v = b[e] - ax[e];
        r[e] = v;
        s = fma(v.re, v.re, fma(v.im, v.im, s));
    }
    if (!part) return;
    const double2 t = block_sum_t<T>(s, T(0));
    if (threadIdx.x == 0) part[blockIdx.x] = t.x;
}

// dst = src * (*rcp): V(:,k) = w / ||w|| with the reciprocal formed once per step.
template <typename T>
__global__ void __launch_bounds__(kThr) fg_scale_kernel(const cplx<T> *__restrict__ src, cplx<T> *__restrict__ dst,
                                                        long long n, const double *rcp, const int *gate)
{
    if (closed(gate)) return;
    const T d = (T)*rcp;
    for (long long e = blockIdx.x * (long long)kThr + threadIdx.x; e < n; e += (long long)gridDim.x * kThr) {
        const cplx<T> v = src[e];
        dst[e] = mk<T>(v.re * d, v.im * d);
    }
}

// Element loops take kU elements per thread per pass (stride apart, each coalesced across the
// warp) so that kU x (vectors) independent loads are in flight before the arithmetic.
constexpr int kU = 4;

// Per-CTA partials of h_j = V_j^H w, j < nv <= MV: part[j * gridDim.x + cta].
// Stored vector 0 is u0, vector j >= 1 is V + j n (the unpreconditioned instances keep vector 0
// in their residual buffer).
template <typename T, int MV>
__global__ void __launch_bounds__(kThr) fg_dots_kernel(const cplx<T> *__restrict__ u0, const cplx<T> *__restrict__ V,
                                                       int nv, const cplx<T> *__restrict__ w, long long n,
                                                       double2 *__restrict__ part, const int *gate)
{
    if (closed(gate)) return;
    cplx<T> acc[MV];
#pragma unroll
    for (int j = 0; j < MV; ++j) acc[j] = mk<T>(0, 0);
    const long long stride = (long long)gridDim.x * kThr;
    long long e = blockIdx.x * (long long)kThr + threadIdx.x;
    for (; e + (kU - 1) * stride < n; e += kU * stride) {
        cplx<T> wv[kU];
#pragma unroll
        for (int u = 0; u < kU; ++u) wv[u] = w[e + u * stride];
#pragma unroll
        for (int j = 0; j < MV; ++j) {
            if (j < nv) {
                const cplx<T> *vj = j == 0 ? u0 : V + (long long)j * n;
                cplx<T> v[kU];
#pragma unroll
                for (int u = 0; u < kU; ++u) v[u] = vj[e + u * stride];
#pragma unroll
                for (int u = 0; u < kU; ++u) cmac_cb(acc[j], wv[u], v[u]);  // conj(v) * w
            }
        }
    }
    for (; e < n; e += stride) {
        const cplx<T> wv = w[e];
#pragma unroll
        for (int j = 0; j < MV; ++j)
            if (j < nv) cmac_cb(acc[j], wv, (j == 0 ? u0 : V + (long long)j * n)[e]);
    }
#pragma unroll
    for (int j = 0; j < MV; ++j) {
        if (j < nv) {
            const double2 t = block_sum_t<T>(acc[j].re, acc[j].im);
            if (threadIdx.x == 0) part[(long long)j * gridDim.x + blockIdx.x] = t;
        }
    }
}

// Sum of per-CTA partials written by other CTAs of the same launch (read through L2).
__device__ double sum_parts_cg(const double *part, int nparts)
{
    double s = 0.0;
    for (int p = threadIdx.x; p < nparts; p += kThr) s += __ldcg(part + p);
    return block_sum_t<double>(s, 0.0).x;
}

// Step j of the cycle (0-based): H(1:j+1, j+1) = h, H(j+2, j+1) = ||w||; Givens rotations
// replace the least-squares solve of FGMRES.m:111 (same solution and residual norm; y itself
// is back-substituted once per cycle, by fg_xupd_kernel).  With H(j+2, j+1) = ||w|| real the
// new rotation needs only reciprocal square roots (FP64 divisions and square roots are long
// dependent sequences on this GPU): c = |a| / r, s = (a / |a|) ||w|| / r, r = sqrt(|a|^2 +
// ||w||^2), and the quasi-residual |g(j+2)| = |s| |g(j+1)| follows without a square root.
// Run by every thread of the CTA that finishes the orthogonalisation last (fg_orth_kernel); the
// state it reads is copied to shared memory by all its threads at once.
// hist (optional): the quasi-residual history, hist[nhst] written after each step.
// lazy: the next basis vector is kept as w itself with scale 1 / ||w||.
__device__ void givens_step(FgState *st, const double *part, int nparts, int j, int m, double tol, double *hist,
                            int lazy)
{
    __shared__ cplx<double> ssn[kMaxM], sc[kMaxM + 1];
    __shared__ double scs[kMaxM];
    if (threadIdx.x < j) {
        scs[threadIdx.x] = st->cs[threadIdx.x];
        ssn[threadIdx.x] = st->sn[threadIdx.x];
    }
    if (threadIdx.x <= j) {
        // written by CTA 0 of the same launch: read through L2
        const double2 v = __ldcg(reinterpret_cast<const double2 *>(st->h + threadIdx.x));
        sc[threadIdx.x] = mk<double>(v.x, v.y);
    }
    const double w2 = sum_parts_cg(part, nparts);  // ||w||^2 (synchronises the block)
    if (threadIdx.x != 0) return;
    const cplx<double> gj = st->g[j];
    const double gres = st->gres;
    FgHead &h = st->hd;
    const double rnormr0 = st->rnormr0;
    const double rhn = w2 > 0.0 ? rsqrt(w2) : 0.0;
    const double hn = w2 * rhn;
    cplx<double> *c = sc;
    // rotations 0..j-1 on the column (c[i + 1] is the unrotated h[i + 1] for i + 1 <= j)
    for (int i = 0; i < j; ++i) {
        const double ci = scs[i];
        const cplx<double> si = ssn[i];
        const cplx<double> t = ci * c[i] + si * c[i + 1];
        c[i + 1] = ci * c[i + 1] - cconj(si) * c[i];
        c[i] = t;
    }
    const cplx<double> a = c[j];
    const double na2 = cabs2(a);
    double cj, sabs;
    cplx<double> sj, rjj;
    if (w2 == 0.0) {
        cj = 1.0;
        sj = mk<double>(0, 0);
        sabs = 0.0;
        rjj = a;
    } else if (na2 == 0.0) {
        cj = 0.0;
        sj = mk<double>(1.0, 0.0);
        sabs = 1.0;
        rjj = mk<double>(hn, 0.0);
    } else {
        const double r2 = na2 + w2, rr = rsqrt(r2), rna = rsqrt(na2);
        const cplx<double> ph = rna * a;
        cj = na2 * rna * rr;
        sabs = hn * rr;
        sj = sabs * ph;
        rjj = (r2 * rr) * ph;
    }
    c[j] = rjj;
    st->cs[j] = cj;
    st->sn[j] = sj;
    for (int i = 0; i <= j; ++i) st->R[j * kMaxM + i] = c[i];
    st->g[j + 1] = mk<double>(0, 0) - cconj(sj) * gj;
    st->g[j] = cj * gj;
    const double gnew = sabs * gres;
    st->gres = gnew;
    const double q = gnew * rnormr0;
    h.hst = q;
    st->hn = hn;
    st->rhn = rhn;
    if (j + 1 < kMaxM) st->sv[j + 1] = lazy ? rhn : 1.0;
    const int nh = h.nhst + 1;
    h.nhst = nh;
    if (hist) hist[nh] = q;
    h.it += 1;
    h.k = j + 1;
    h.go = (q > tol && j + 1 < m) ? 1 : 0;
}

// a -= v * h
template <typename T>
__device__ __forceinline__ void csub_mul(cplx<T> &a, cplx<T> v, cplx<T> h)
{
    a.re -= v.re * h.re;
    a.re += v.im * h.im;
    a.im -= v.re * h.im;
    a.im -= v.im * h.re;
}

// wout = sv[k] win - sum_j V_j h_j, k = nv - 1, with h summed here from the dots' partials (every
// CTA in the same fixed order, so all agree; CTA 0 stores h in the state) and scaled by the
// stored vectors' factors: the basis vector j is sv[j] times stored vector j, win = A (stored
// vector k).  Per-CTA partials of ||wout||^2.  wout may be win.  nv <= MV.
// The CTA that finishes last (a ticket counter in the state: every CTA publishes its partial,
// fences, then takes a ticket; no CTA waits for another) runs the step's Givens update
// (givens_step) for step j = nv - 1 and resets the counter.
template <typename T, int MV>
__global__ void __launch_bounds__(kThr) fg_orth_kernel(const cplx<T> *__restrict__ u0, const cplx<T> *__restrict__ V,
                                                       int nv, const cplx<T> *win, cplx<T> *wout, long long n,
                                                       const double2 *__restrict__ dpart, int nparts, FgState *st,
                                                       double *part, int m, double tol, double *hist, int lazy,
                                                       const int *gate)
{
    if (closed(gate)) return;
    __shared__ cplx<T> sh[kMaxM];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int j = wid; j < nv; j += kThr / 32) {
        double re = 0.0, im = 0.0;
        for (int p = lane; p < nparts; p += 32) {
            const double2 v = dpart[(long long)j * nparts + p];
            re += v.x;
            im += v.y;
        }
        for (int o = 16; o > 0; o >>= 1) {
            re += __shfl_down_sync(0xffffffffu, re, o);
            im += __shfl_down_sync(0xffffffffu, im, o);
        }
        if (lane == 0) {
            const double f = st->sv[j] * st->sv[nv - 1];
            const cplx<double> hj = mk<double>(f * re, f * im);      // H(j+1, k+1)
            sh[j] = mk<T>((T)(st->sv[j] * hj.re), (T)(st->sv[j] * hj.im));  // applied to stored vector j
            if (blockIdx.x == 0) st->h[j] = hj;
        }
    }
    __syncthreads();
    const T sk = (T)st->sv[nv - 1];
    T s = 0;
    const long long stride = (long long)gridDim.x * kThr;
    long long e = blockIdx.x * (long long)kThr + threadIdx.x;
    for (; e + (kU - 1) * stride < n; e += kU * stride) {
        cplx<T> a[kU];
#pragma unroll
        for (int u = 0; u < kU; ++u) {
            const cplx<T> t = win[e + u * stride];
            a[u] = mk<T>(sk * t.re, sk * t.im);
        }
#pragma unroll
        for (int j = 0; j < MV; ++j) {
            if (j < nv) {
                const cplx<T> *vj = j == 0 ? u0 : V + (long long)j * n;
                cplx<T> v[kU];
#pragma unroll
                for (int u = 0; u < kU; ++u) v[u] = vj[e + u * stride];
                const cplx<T> hj = sh[j];
#pragma unroll
                for (int u = 0; u < kU; ++u) csub_mul(a[u], v[u], hj);
            }
        }
#pragma unroll
        for (int u = 0; u < kU; ++u) {
            wout[e + u * stride] = a[u];
            s = fma(a[u].re, a[u].re, fma(a[u].im, a[u].im, s));
        }
    }
    for (; e < n; e += stride) {
        const cplx<T> t = win[e];
        cplx<T> a = mk<T>(sk * t.re, sk * t.im);
#pragma unroll
        for (int j = 0; j < MV; ++j)
            if (j < nv) csub_mul(a, (j == 0 ? u0 : V + (long long)j * n)[e], sh[j]);
        wout[e] = a;
        s = fma(a.re, a.re, fma(a.im, a.im, s));
    }
    const double2 t = block_sum_t<T>(s, T(0));
    __shared__ int last;
    if (threadIdx.x == 0) {
        part[blockIdx.x] = t.x;
        __threadfence();
        last = atomicAdd(&st->ticket, 1) == (int)gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    givens_step(st, part, gridDim.x, nv - 1, m, tol, hist, lazy);
    if (threadIdx.x == 0) st->ticket = 0;
}

// x += sum_{j < k} B_j y_j over the steps of the cycle (FGMRES.m:117-121).  y = R \ g, the
// least-squares solution of FGMRES.m:111 after the cycle's last step, is back-substituted here
// (thread 0 of every CTA, from the rotated Hessenberg matrix) rather than after every step;
// CTA 0 stores it in the state.
// Stored vector 0 is u0, vector j >= 1 is B + j n; with scaled != 0 the basis vector j is sv[j]
// times the stored one.
template <typename T>
__global__ void __launch_bounds__(kThr) fg_xupd_kernel(cplx<T> *__restrict__ x, const cplx<T> *__restrict__ u0,
                                                       const cplx<T> *__restrict__ B, long long n, FgState *st,
                                                       int scaled, const int *gate)
{
    if (closed(gate)) return;
    __shared__ cplx<double> sR[kMaxM * kMaxM], sg[kMaxM], sy[kMaxM];
    __shared__ cplx<T> syt[kMaxM];
    const int kk = st->hd.k;
    for (int q = threadIdx.x; q < kk * kMaxM; q += kThr) sR[q] = st->R[q];
    if (threadIdx.x < kk) sg[threadIdx.x] = st->g[threadIdx.x];
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int i = kk - 1; i >= 0; --i) {
            cplx<double> t = sg[i];
            for (int l = i + 1; l < kk; ++l) t = t - sR[l * kMaxM + i] * sy[l];
            const cplx<double> d = sR[i * kMaxM + i];
            const double dd = cabs2(d);
            sy[i] = dd == 0.0 ? mk<double>(0, 0) : (1.0 / dd) * (t * cconj(d));
        }
        for (int i = 0; i < kk; ++i) {
            const double f = scaled ? st->sv[i] : 1.0;
            syt[i] = mk<T>((T)(f * sy[i].re), (T)(f * sy[i].im));
            if (blockIdx.x == 0) st->y[i] = sy[i];
        }
    }
    __syncthreads();
    const long long stride = (long long)gridDim.x * kThr;
    long long e = blockIdx.x * (long long)kThr + threadIdx.x;
    for (; e + (kU - 1) * stride < n; e += kU * stride) {
        cplx<T> a[kU];
#pragma unroll
        for (int u = 0; u < kU; ++u) a[u] = mk<T>(0, 0);
        for (int j = 0; j < kk; ++j) {
            const cplx<T> *bj = j == 0 ? u0 : B + (long long)j * n;
            cplx<T> v[kU];
#pragma unroll
            for (int u = 0; u < kU; ++u) v[u] = bj[e + u * stride];
            const cplx<T> yj = syt[j];
#pragma unroll
            for (int u = 0; u < kU; ++u) cmac(a[u], v[u], yj);
        }
#pragma unroll
        for (int u = 0; u < kU; ++u) x[e + u * stride] = x[e + u * stride] + a[u];
    }
    for (; e < n; e += stride) {
        cplx<T> a = mk<T>(0, 0);
        for (int j = 0; j < kk; ++j) cmac(a, (j == 0 ? u0 : B + (long long)j * n)[e], syt[j]);
        x[e] = x[e] + a;
    }
}

// complex128 <-> complex64 copies of a field (the mixed-precision preconditioner's edges)
template <typename S, typename D>
__global__ void __launch_bounds__(kThr) fg_cast_kernel(const cplx<S> *__restrict__ a, cplx<D> *__restrict__ b,
                                                       long long n)
{
    for (long long e = blockIdx.x * (long long)kThr + threadIdx.x; e < n; e += (long long)gridDim.x * kThr)
        b[e] = mk<D>((D)a[e].re, (D)a[e].im);
}

// ---- single-CTA state updates ---------------------------------------------------------------

__device__ double sum_parts(const double *part, int nparts)
{
    double s = 0.0;
    for (int p = threadIdx.x; p < nparts; p += kThr) s += part[p];
    return block_sum_t<double>(s, 0.0).x;
}

__device__ __forceinline__ bool cycles_left(int it, int m, long long maxit)
{
    return (long long)(it / m) < maxit;  // floor(it_counter / maxinnerit) < maxit
}

// INIT (first = 1): normr0 = beta = ||r||, hst = 1, it = 1 (FGMRES.m:62-76).
// END OF CYCLE (first = 0, runs while live): the true residual's norm decides the break of
// FGMRES.m:125, then the loop condition of FGMRES.m:88.  Either way the next cycle starts
// from beta = ||r|| (FGMRES.m:92).
// lazy: the cycle keeps its basis unnormalised (vector 0 = r itself, scale 1 / beta).
__global__ void __launch_bounds__(kThr) fg_norm_kernel(FgState *st, const double *part, int nparts, int first,
                                                       double tol, int m, long long maxit, int lazy)
{
    if (!first && st->hd.live == 0) return;
    const double nr = sqrt(sum_parts(part, nparts));
    if (threadIdx.x != 0) return;
    FgHead &h = st->hd;
    if (first) {
        h.normr0 = nr;
        h.hst = 1.0;
        h.it = 1;
        h.nhst = 0;
        h.conv = nr == 0.0 ? 1 : 0;
        h.rn = nr;
        h.live = (nr != 0.0 && h.hst > tol && cycles_left(h.it, m, maxit)) ? 1 : 0;
    } else {
        h.rn = nr;
        if (nr / h.normr0 < tol) {
            h.live = 0;
            h.conv = 1;
        } else {
            if (h.hst <= tol) h.conv = 1;  // (a NaN quasi-residual stops the loop unconverged)
            h.live = (h.hst > tol && cycles_left(h.it, m, maxit)) ? 1 : 0;
        }
    }
    h.beta = nr;
    st->rbeta = nr != 0.0 ? 1.0 / nr : 0.0;
    st->gres = nr;
    st->sv[0] = lazy ? st->rbeta : 1.0;
    if (first) {
        st->rnormr0 = nr != 0.0 ? 1.0 / nr : 0.0;
        st->ticket = 0;
    }
    h.k = 0;
    h.go = h.live;
    st->g[0] = mk<double>(nr, 0.0);
}

// ---- host side -------------------------------------------------------------------------------

int device_sms()
{
    static int sms = 0;
    if (sms == 0) {
        int dev = 0, v = 0;
        if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && v > 0)
            sms = v;
        else {
            cudaGetLastError();
            sms = 148;
        }
    }
    return sms;
}

// CTAs of the reduction kernels (and entries of the partial-sum buffers): one pass of kU
// elements per thread on the coarse levels (latency-bound there: more CTAs in flight), at most
// four CTAs per SM.
int parts_for(long long n)
{
    const long long p = (n + kU * kThr - 1) / (kU * kThr);
    const long long cap = 4LL * device_sms();
    return (int)(p < 1 ? 1 : (p > cap ? cap : p));
}

// Sub-allocations of one device arena, 256-byte aligned.
struct Arena {
    size_t used = 0;
    char *base = nullptr;
    template <typename U>
    U *take(size_t count)
    {
        const size_t off = (used + 255) & ~(size_t)255;
        used = off + sizeof(U) * count;
        return base ? reinterpret_cast<U *>(base + off) : nullptr;
    }
};

template <typename T>
struct Fg {                     // one FGMRES instance
    long long n = 0;
    int m = 0;
    bool pre = false;
    int nparts = 1;
    cplx<T> *V = nullptr, *Z = nullptr, *w = nullptr, *r = nullptr;
    double2 *dpart = nullptr;
    double *part = nullptr;
    FgState *st = nullptr;
    long long nhist = 0;        // history entries to keep (the outer solve), else 0
    double *hist = nullptr;
    void carve(Arena &a)
    {
        hist = nhist ? a.take<double>(nhist) : nullptr;
        V = a.take<cplx<T>>((size_t)m * n);
        Z = pre ? a.take<cplx<T>>((size_t)m * n) : nullptr;
        w = a.take<cplx<T>>(n);
        r = a.take<cplx<T>>(n);
        dpart = a.take<double2>((size_t)kMaxM * nparts);
        part = a.take<double>(nparts);
        st = a.take<FgState>(1);
    }
};

template <typename T>
using Pre = std::function<int(const cplx<T> *, cplx<T> *)>;

struct Run {                    // per-call context
    cudaStream_t s = nullptr;
    bool adj = false;
    int64_t launches = 0, syncs = 0;
    FgHead *hh = nullptr;       // pinned copy of a state head

    int fetch(const FgState *st)
    {
        H3D_CUDA_TRY(cudaMemcpyAsync(hh, &st->hd, sizeof(FgHead), cudaMemcpyDeviceToHost, s));
        H3D_CUDA_TRY(cudaStreamSynchronize(s));
        ++syncs;
        return H3D_OK;
    }
    unsigned blocks(long long n) const
    {
        const long long b = (n + kThr - 1) / kThr, cap = 8LL * device_sms();
        return (unsigned)(b < 1 ? 1 : (b > cap ? cap : b));
    }
};

#define H3D_ML_LAUNCH(...)                   \
    do {                                     \
        __VA_ARGS__;                         \
        ++R.launches;                        \
        H3D_CUDA_TRY(cudaGetLastError());    \
    } while (0)

// FGMRES.m on one instance: x (in/out; zero_x = the initial guess is zero, FGMRES.m:65-67).
// pre: the flexible preconditioner z = P v (null = identity, the basis itself updates x).
// last_fetch: read the state head back at the end (into R.hh).
template <typename T>
int fgmres(Run &R, Fg<T> &I, const Op<T> &op, const cplx<T> *b, cplx<T> *x, bool zero_x, double tol,
           long long maxit, const Pre<T> *pre, bool last_fetch)
{
    const long long n = I.n;
    const int m = I.m;
    const unsigned nb = (unsigned)I.nparts;
    int rc;
    if (zero_x) {
        H3D_ML_LAUNCH((fg_copy_kernel<T><<<nb, kThr, 0, R.s>>>(b, I.r, x, n, I.part)));
    } else {
        if ((rc = launch_mvp<T>(op, x, I.w, 1, R.adj, false, R.s))) return rc;
        ++R.launches;
        H3D_ML_LAUNCH((fg_sub_kernel<T><<<nb, kThr, 0, R.s>>>(b, I.w, I.r, n, I.part, nullptr)));
    }
    // Unpreconditioned instances keep their basis unnormalised (each stored vector with its scale
    // in the state): no separate scaling pass per step; vector 0 is the residual buffer itself.
    const int lazy = pre ? 0 : 1;
    H3D_ML_LAUNCH((fg_norm_kernel<<<1, kThr, 0, R.s>>>(I.st, I.part, I.nparts, 1, tol, m, maxit, lazy)));
    int *live = &I.st->hd.live, *go = &I.st->hd.go;
    const cplx<T> *u0 = lazy ? I.r : I.V;
    cplx<T> *basis = pre ? I.Z : I.V;
    for (long long c = 0; c < maxit; ++c) {
        if (pre || c > 0) {
            if ((rc = R.fetch(I.st))) return rc;
            if (!R.hh->live) break;
        }
        if (!lazy) H3D_ML_LAUNCH((fg_scale_kernel<T><<<nb, kThr, 0, R.s>>>(I.r, I.V, n, &I.st->rbeta, live)));
        for (int j = 0; j < m; ++j) {
            const cplx<T> *vj = j == 0 ? u0 : I.V + (long long)j * n;
            if (pre) {
                if (j > 0) {
                    if ((rc = R.fetch(I.st))) return rc;
                    if (!R.hh->go) break;
                }
                cplx<T> *zj = I.Z + (long long)j * n;
                if ((rc = (*pre)(vj, zj))) return rc;
                vj = zj;
            }
            if ((rc = launch_mvp<T>(op, vj, I.w, 1, R.adj, false, R.s))) return rc;
            ++R.launches;
            // the orthogonalised vector: straight into the next basis slot (lazy), else into w
            cplx<T> *wout = (lazy && j + 1 < m) ? I.V + (long long)(j + 1) * n : I.w;
            if (j < 4) {
                H3D_ML_LAUNCH((fg_dots_kernel<T, 4><<<nb, kThr, 0, R.s>>>(u0, I.V, j + 1, I.w, n, I.dpart, go)));
                H3D_ML_LAUNCH((fg_orth_kernel<T, 4><<<nb, kThr, 0, R.s>>>(u0, I.V, j + 1, I.w, wout, n, I.dpart,
                                                                          I.nparts, I.st, I.part, m, tol, I.hist,
                                                                          lazy, go)));
            } else if (j < 8) {
                H3D_ML_LAUNCH((fg_dots_kernel<T, 8><<<nb, kThr, 0, R.s>>>(u0, I.V, j + 1, I.w, n, I.dpart, go)));
                H3D_ML_LAUNCH((fg_orth_kernel<T, 8><<<nb, kThr, 0, R.s>>>(u0, I.V, j + 1, I.w, wout, n, I.dpart,
                                                                          I.nparts, I.st, I.part, m, tol, I.hist,
                                                                          lazy, go)));
            } else {
                H3D_ML_LAUNCH((fg_dots_kernel<T, kMaxM><<<nb, kThr, 0, R.s>>>(u0, I.V, j + 1, I.w, n, I.dpart, go)));
                H3D_ML_LAUNCH((fg_orth_kernel<T, kMaxM><<<nb, kThr, 0, R.s>>>(u0, I.V, j + 1, I.w, wout, n, I.dpart,
                                                                              I.nparts, I.st, I.part, m, tol, I.hist,
                                                                          lazy, go)));
            }
            if (!lazy && j + 1 < m)
                H3D_ML_LAUNCH((fg_scale_kernel<T><<<nb, kThr, 0, R.s>>>(I.w, I.V + (long long)(j + 1) * n, n,
                                                                        &I.st->rhn, go)));
        }
        H3D_ML_LAUNCH(
            (fg_xupd_kernel<T><<<nb, kThr, 0, R.s>>>(x, pre ? I.Z : u0, basis, n, I.st, lazy, live)));
        if ((rc = launch_mvp<T>(op, x, I.w, 1, R.adj, false, R.s))) return rc;
        ++R.launches;
        H3D_ML_LAUNCH((fg_sub_kernel<T><<<nb, kThr, 0, R.s>>>(b, I.w, I.r, n, I.part, live)));
        H3D_ML_LAUNCH((fg_norm_kernel<<<1, kThr, 0, R.s>>>(I.st, I.part, I.nparts, 0, tol, m, maxit, lazy)));
    }
    if (last_fetch) return R.fetch(I.st);
    return H3D_OK;
}

// The V-cycle hierarchy in one precision.
template <typename T>
struct Cycle {
    int nl = 0;
    Op<T> op[kMaxLevels];
    long long n[kMaxLevels] = {};
    const h3d_ml_transfer *Rt = nullptr, *Pt = nullptr;
    Fg<T> smooth[kMaxLevels], coarse[kMaxLevels], bottom;
    cplx<T> *res[kMaxLevels] = {}, *rc[kMaxLevels] = {}, *xc[kMaxLevels] = {};
    cplx<T> *t1 = nullptr, *t2 = nullptr;
    long long t1n = 0, t2n = 0;
    double stol = 1e-6, ctol = 0.5;
    int sk = 3, ck = 3;

    void size(const int k[4], long long tmp1, long long tmp2)
    {
        t1n = tmp1;
        t2n = tmp2;
        sk = k[0];
        ck = k[2];
        for (int i = 0; i < nl; ++i) {
            if (i < nl - 1) {
                smooth[i].n = n[i];
                smooth[i].m = k[1];
                smooth[i].nparts = parts_for(n[i]);
            }
            if (i >= 1) {
                coarse[i].n = n[i];
                coarse[i].m = k[3];
                coarse[i].pre = true;
                coarse[i].nparts = parts_for(n[i]);
            }
        }
        bottom.n = n[nl - 1];
        bottom.m = k[3];
        bottom.nparts = parts_for(n[nl - 1]);
    }
    void carve(Arena &a)
    {
        for (int i = 0; i < nl; ++i) {
            if (i < nl - 1) {
                smooth[i].carve(a);
                res[i] = a.take<cplx<T>>(n[i]);
            }
            if (i >= 1) {
                coarse[i].carve(a);
                rc[i] = a.take<cplx<T>>(n[i]);
                xc[i] = a.take<cplx<T>>(n[i]);
            }
        }
        bottom.carve(a);
        t1 = a.take<cplx<T>>(t1n);
        t2 = a.take<cplx<T>>(t2n);
    }

    int transfer(Run &R, const h3d_ml_transfer &t, const cplx<T> *x, cplx<T> *y, bool accum)
    {
        int d[3] = {t.n_in[0], t.n_in[1], t.n_in[2]};
        int rcode;
        if ((rcode = launch_axis<T>(t.rowptr[0], t.col[0], t.val[0], t.n_out[0], 0, d, x, t1, 1, 1.0, false, R.s)))
            return rcode;
        d[0] = t.n_out[0];
        if ((rcode = launch_axis<T>(t.rowptr[1], t.col[1], t.val[1], t.n_out[1], 1, d, t1, t2, 1, 1.0, false, R.s)))
            return rcode;
        d[1] = t.n_out[1];
        if ((rcode = launch_axis<T>(t.rowptr[2], t.col[2], t.val[2], t.n_out[2], 2, d, t2, y, 1, t.scale, accum,
                                    R.s)))
            return rcode;
        R.launches += 3;
        return H3D_OK;
    }

    // x = V-cycle(i) b (GMG_V.m; x is overwritten)
    int vcycle(Run &R, int i, const cplx<T> *b, cplx<T> *x)
    {
        int rcode;
        if ((rcode = fgmres<T>(R, smooth[i], op[i], b, x, true, stol, sk, nullptr, false))) return rcode;
        if ((rcode = launch_mvp<T>(op[i], x, res[i], 1, R.adj, false, R.s))) return rcode;
        ++R.launches;
        const unsigned nb = (unsigned)smooth[i].nparts;
        H3D_ML_LAUNCH((fg_sub_kernel<T><<<nb, kThr, 0, R.s>>>(b, res[i], res[i], n[i], nullptr, nullptr)));
        if ((rcode = transfer(R, Rt[i], res[i], rc[i + 1], false))) return rcode;
        Pre<T> pre;
        if (i + 1 == nl - 1)
            pre = [this, &R](const cplx<T> *v, cplx<T> *z) {
                return fgmres<T>(R, bottom, op[nl - 1], v, z, true, ctol, ck, nullptr, false);
            };
        else
            pre = [this, &R, i](const cplx<T> *v, cplx<T> *z) { return vcycle(R, i + 1, v, z); };
        if ((rcode = fgmres<T>(R, coarse[i + 1], op[i + 1], rc[i + 1], xc[i + 1], true, ctol, ck, &pre, false)))
            return rcode;
        if ((rcode = transfer(R, Pt[i], xc[i + 1], x, true))) return rcode;
        return fgmres<T>(R, smooth[i], op[i], b, x, false, stol, sk, nullptr, false);
    }
};

long long npts(const h3d_grid &g) { return (long long)g.n[0] * g.n[1] * g.n[2]; }

bool same3(const int32_t *a, const int32_t *b) { return a[0] == b[0] && a[1] == b[1] && a[2] == b[2]; }

}  // namespace
}  // namespace h3d

using namespace h3d;

extern "C" void h3d_ml_default_opts(h3d_ml_opts *o)
{
    if (!o) return;
    o->tol = 1e-6;
    o->maxit = 10000;
    o->maxinnerit = 5;
    o->precond = H3D_ML_PREC_MLGMRES;
    o->precision = H3D_PREC_FP64;
    o->k[0] = 3;
    o->k[1] = 5;
    o->k[2] = 3;
    o->k[3] = 5;
    o->smooth_tol = 1e-6;
    o->coarse_tol = 0.5;
}

extern "C" int h3d_mlgmres_solve(const h3d_ml_level *levels, int nlevels, const h3d_ml_transfer *restrict_ops,
                                 const h3d_ml_transfer *prolong_ops, const void *b, void *x, int mode,
                                 const h3d_ml_opts *opts, double *hst, int hst_cap, h3d_ml_info *info, void *stream)
{
    const auto t0 = std::chrono::steady_clock::now();
    h3d_ml_opts o;
    h3d_ml_default_opts(&o);
    if (opts) o = *opts;
    const bool ml = o.precond == H3D_ML_PREC_MLGMRES;
    if (!levels || !b || !x || nlevels < 1 || nlevels > kMaxLevels || (mode != H3D_FORWARD && mode != H3D_ADJOINT) ||
        (o.precond != H3D_ML_PREC_NONE && !ml) || (o.precision != H3D_PREC_FP64 && o.precision != H3D_PREC_MIXED) ||
        !(o.tol >= 0.0) || o.maxit < 1 || o.maxinnerit < 1 || o.maxinnerit > kMaxM) {
        set_error("h3d_mlgmres_solve: bad argument");
        return H3D_ERR_BAD_ARG;
    }
    if (ml) {
        if (nlevels < 2 || !restrict_ops || !prolong_ops || o.k[0] < 1 || o.k[1] < 1 || o.k[1] > kMaxM || o.k[2] < 1 ||
            o.k[3] < 1 || o.k[3] > kMaxM || !(o.smooth_tol >= 0.0) || !(o.coarse_tol >= 0.0)) {
            set_error("h3d_mlgmres_solve: the multigrid preconditioner needs 2 or more levels, their transfers, "
                      "and 1-%d steps per smoother / coarse cycle", kMaxM);
            return H3D_ERR_BAD_ARG;
        }
        for (int i = 0; i < nlevels; ++i)
            if (!levels[i].wn || (o.precision == H3D_PREC_MIXED && !levels[i].wn32)) {
                set_error("h3d_mlgmres_solve: level %d has no wavenumber of the precision asked for", i);
                return H3D_ERR_BAD_ARG;
            }
        for (int i = 0; i + 1 < nlevels; ++i) {
            const h3d_ml_transfer &r = restrict_ops[i], &p = prolong_ops[i];
            if (!same3(r.n_in, levels[i].grid.n) || !same3(r.n_out, levels[i + 1].grid.n) ||
                !same3(p.n_in, levels[i + 1].grid.n) || !same3(p.n_out, levels[i].grid.n)) {
                set_error("h3d_mlgmres_solve: transfer %d does not connect the grids of levels %d and %d", i, i,
                          i + 1);
                return H3D_ERR_BAD_ARG;
            }
            for (int a = 0; a < 3; ++a)
                if (!r.rowptr[a] || !r.col[a] || !r.val[a] || !p.rowptr[a] || !p.col[a] || !p.val[a]) {
                    set_error("h3d_mlgmres_solve: transfer %d has a null axis operator", i);
                    return H3D_ERR_BAD_ARG;
                }
        }
    } else if (!levels[0].wn) {
        set_error("h3d_mlgmres_solve: level 0 has no wavenumber");
        return H3D_ERR_BAD_ARG;
    }
    const long long cap_needed = 1 + (long long)o.maxit * o.maxinnerit;
    if (hst && hst_cap < cap_needed) {
        set_error("h3d_mlgmres_solve: hst holds %d values, the solve may record %lld", hst_cap, cap_needed);
        return H3D_ERR_BAD_ARG;
    }
    const int nl = ml ? nlevels : 1;
    for (int i = 0; i < nl; ++i) {
        const int rc = check_grid(&levels[i].grid);
        if (rc) return rc;
    }

    Run R;
    R.s = (cudaStream_t)stream;
    R.adj = mode == H3D_ADJOINT;
    static thread_local FgHead *pinned = nullptr;
    if (!pinned) H3D_CUDA_TRY(cudaMallocHost(&pinned, sizeof(FgHead)));
    R.hh = pinned;

    // operators and sizes
    Cycle<double> c64;
    Cycle<float> c32;
    const bool mixed = o.precision == H3D_PREC_MIXED;
    Op<double> op0;
    int rc = make_op_f64(&levels[0].grid, levels[0].wn, nullptr, &op0);
    if (rc) return rc;
    const long long n0 = npts(levels[0].grid);
    long long tmp1 = 1, tmp2 = 1;
    if (ml) {
        for (int i = 0; i + 1 < nl; ++i) {
            const h3d_ml_transfer *ts[2] = {&restrict_ops[i], &prolong_ops[i]};
            for (const h3d_ml_transfer *t : ts) {
                const long long a = (long long)t->n_out[0] * t->n_in[1] * t->n_in[2];
                const long long bq = (long long)t->n_out[0] * t->n_out[1] * t->n_in[2];
                tmp1 = a > tmp1 ? a : tmp1;
                tmp2 = bq > tmp2 ? bq : tmp2;
            }
        }
        auto setup = [&](auto &cy, auto make) -> int {
            cy.nl = nl;
            cy.Rt = restrict_ops;
            cy.Pt = prolong_ops;
            cy.stol = o.smooth_tol;
            cy.ctol = o.coarse_tol;
            for (int i = 0; i < nl; ++i) {
                cy.n[i] = npts(levels[i].grid);
                const int r2 = make(i, &cy.op[i]);
                if (r2) return r2;
            }
            cy.size(o.k, tmp1, tmp2);
            return H3D_OK;
        };
        if (mixed)
            rc = setup(c32, [&](int i, Op<float> *op) { return make_op_f32(&levels[i].grid, levels[i].wn32, nullptr, op); });
        else
            rc = setup(c64, [&](int i, Op<double> *op) { return make_op_f64(&levels[i].grid, levels[i].wn, nullptr, op); });
        if (rc) return rc;
    }
    Fg<double> outer;
    outer.n = n0;
    outer.m = o.maxinnerit;
    outer.pre = ml;
    outer.nparts = parts_for(n0);
    outer.nhist = hst ? cap_needed : 0;

    // one arena for every vector of the call
    Arena a;
    auto carve_all = [&](Arena &ar, cplx<float> **b32, cplx<float> **x32) {
        outer.carve(ar);
        if (ml) {
            if (mixed) {
                c32.carve(ar);
                *b32 = ar.take<cplx<float>>(n0);
                *x32 = ar.take<cplx<float>>(n0);
            } else
                c64.carve(ar);
        }
    };
    cplx<float> *b32 = nullptr, *x32 = nullptr;
    carve_all(a, &b32, &x32);
    DevBuf arena;
    if ((rc = arena.alloc(a.used, R.s))) return rc;
    Arena a2;
    a2.base = arena.as<char>();
    carve_all(a2, &b32, &x32);

    Pre<double> pre;
    if (ml && mixed)
        pre = [&](const cplx<double> *v, cplx<double> *z) -> int {
            const unsigned nb = R.blocks(n0);
            H3D_ML_LAUNCH((fg_cast_kernel<double, float><<<nb, kThr, 0, R.s>>>(v, b32, n0)));
            const int r2 = c32.vcycle(R, 0, b32, x32);
            if (r2) return r2;
            H3D_ML_LAUNCH((fg_cast_kernel<float, double><<<nb, kThr, 0, R.s>>>(x32, z, n0)));
            return H3D_OK;
        };
    else if (ml)
        pre = [&](const cplx<double> *v, cplx<double> *z) -> int { return c64.vcycle(R, 0, v, z); };

    rc = fgmres<double>(R, outer, op0, (const cplx<double> *)b, (cplx<double> *)x, false, o.tol, o.maxit,
                        ml ? &pre : nullptr, true);
    if (rc) return rc;
    if (hst) {
        hst[0] = 1.0;
        if (R.hh->nhst > 0)
            H3D_CUDA_TRY(cudaMemcpyAsync(hst + 1, outer.hist + 1, sizeof(double) * R.hh->nhst, cudaMemcpyDeviceToHost,
                                         R.s));
    }
    H3D_CUDA_TRY(cudaStreamSynchronize(R.s));
    if (info) {
        info->iters = R.hh->nhst;
        info->converged = R.hh->conv;
        info->rel_res = R.hh->hst;
        info->kernel_launches = R.launches;
        info->host_syncs = R.syncs;
        info->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    if (!std::isfinite(R.hh->hst) || !std::isfinite(R.hh->rn)) {
        set_error("h3d_mlgmres_solve: non-finite residual (NaN or Inf in b, x or the wavenumbers)");
        return H3D_ERR_NONFINITE;
    }
    return H3D_OK;
}
