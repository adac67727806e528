// CGMN vector kernels: masked per-RHS updates with deterministic two-stage FP64 reductions
// (block partials in a fixed grid, then one block per RHS sums them in a fixed order).
//
// One CGMN iteration on A = I - Q, Q y = DSWP(y, 0)  (CGMN.m:66-90, linearsolve.m:150-152):
//   y  = p;  DSWP(y, 0) in place                       (sweep kernels)
//   Ap = p - y;  pAp = <p, Ap>                         cg_ap_dot      (CGMN.m:67-68)
//   alpha = ||r||^2 / pAp                              (inside cg_update_xr, first stage)
//   x += alpha p;  r -= alpha Ap;  ||r||^2             cg_update_xr   (CGMN.m:69-75)
//   stop test, beta = (||r|| / ||r_old||)^2            (second stage)  (CGMN.m:76-83)
//   p = r + beta p;  y = p                             cg_update_p    (CGMN.m:85)
#include "h3d_krylov.cuh"

namespace h3d {

int reduction_blocks(long long N)
{
    long long g = (N + (long long)kVecUnroll * kVecThreads - 1) / ((long long)kVecUnroll * kVecThreads);
    if (g > 608) g = 608;  // four 256-thread blocks per SM
    if (g < 1) g = 1;
    return (int)g;
}

// Block-wide sum of two doubles; result valid in thread 0.
__device__ __forceinline__ double2 block_sum2(double a, double b)
{
    __shared__ double sa[32], sb[32];
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        b += __shfl_down_sync(0xffffffffu, b, o);
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) {
        sa[wid] = a;
        sb[wid] = b;
    }
    __syncthreads();
    const int nw = (blockDim.x + 31) >> 5;
    if (wid == 0) {
        a = lane < nw ? sa[lane] : 0.0;
        b = lane < nw ? sb[lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) {
            a += __shfl_down_sync(0xffffffffu, a, o);
            b += __shfl_down_sync(0xffffffffu, b, o);
        }
    }
    __syncthreads();
    return make_double2(a, b);
}

// Sum the G partial pairs of RHS s in a fixed order (every thread of the block returns it).
__device__ __forceinline__ double2 sum_partials(const double *part, int G, int s)
{
    double a = 0.0, b = 0.0;
    for (int q = threadIdx.x; q < G; q += blockDim.x) {
        a += part[2 * ((long long)s * G + q)];
        b += part[2 * ((long long)s * G + q) + 1];
    }
    double2 t = block_sum2(a, b);
    __shared__ double2 bc;
    if (threadIdx.x == 0) bc = t;
    __syncthreads();
    return bc;
}

template <typename T>
__global__ void k_init(const cplx<T> *__restrict__ bt, cplx<T> *__restrict__ x,
                       cplx<T> *__restrict__ r, cplx<T> *__restrict__ p, ColMap cm, double *part,
                       int G)
{
    const int s = blockIdx.y;
    const long long off = cm.o(s), N = cm.n(s);
    double acc = 0.0;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < N;
         q += (long long)G * blockDim.x) {
        const cplx<T> v = bt[off + q];
        x[off + q] = mk<T>(T(0), T(0));
        r[off + q] = v;
        p[off + q] = v;
        acc += (double)v.re * v.re + (double)v.im * v.im;
    }
    const double2 t = block_sum2(acc, 0.0);
    if (threadIdx.x == 0) {
        part[2 * ((long long)s * G + blockIdx.x)] = t.x;
        part[2 * ((long long)s * G + blockIdx.x) + 1] = 0.0;
    }
}

__global__ void k_init_state(CgState st, const double *bnorm2_orig, double zero_tol2, int nrhs)
{
    const int s = blockIdx.x;
    const double2 t = sum_partials(st.part, st.G, s);
    if (threadIdx.x == 0) {
        st.rr[s] = t.x;
        st.bb[s] = t.x;
        st.ratio[s] = 1.0;
        st.iters[s] = 0;
        st.upd[s] = 0;
        st.status[s] = 0;
        // opAbstractMatrix.m:118: a right-hand side of norm < 1e-12 is answered with 0
        const bool zero = bnorm2_orig ? (bnorm2_orig[s] < zero_tol2) : (t.x <= 0.0);
        st.active[s] = (zero || t.x <= 0.0) ? 0 : 1;
        if (!isfinite(t.x)) {
            st.active[s] = 0;
            st.status[s] = H3D_ERR_NONFINITE;
        }
    }
}

template <typename T>
int cg_init(const cplx<T> *bt, cplx<T> *x, cplx<T> *r, cplx<T> *p, long long N, int nrhs,
            const CgState &s, const double *bnorm2_orig, double zero_tol2, int maxit,
            cudaStream_t st)
{
    (void)maxit;
    k_init<T><<<dim3(s.G, nrhs), kVecThreads, 0, st>>>(bt, x, r, p, ColMap{s.coloff, s.collen, N}, s.part, s.G);
    k_init_state<<<nrhs, kVecThreads, 0, st>>>(s, bnorm2_orig, zero_tol2, nrhs);
    H3D_CUDA_TRY(cudaGetLastError());
    return H3D_OK;
}

// Ap = p - y (written over y), partial <p, Ap> (complex).
template <typename T>
__global__ void k_ap_dot(const cplx<T> *__restrict__ p, cplx<T> *__restrict__ y, ColMap cm,
                         const int *__restrict__ active, double *part, int G)
{
    const int s = blockIdx.y;
    if (!active[s]) return;
    const long long N = cm.n(s);
    const cplx<T> *ps = p + cm.o(s);
    cplx<T> *ys = y + cm.o(s);
    double are = 0.0, aim = 0.0;
    auto body = [&](const cplx<T> pv, const cplx<T> yv, long long q) {
        const cplx<T> ap = pv - yv;
        ys[q] = ap;
        are += (double)pv.re * ap.re + (double)pv.im * ap.im;
        aim += (double)pv.re * ap.im - (double)pv.im * ap.re;
    };
    const long long stride = (long long)G * blockDim.x;
    long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    for (; q + (kVecUnroll - 1) * stride < N; q += kVecUnroll * stride) {
        cplx<T> pv[kVecUnroll], yv[kVecUnroll];
#pragma unroll
        for (int u = 0; u < kVecUnroll; ++u) {
            pv[u] = ps[q + u * stride];
            yv[u] = ys[q + u * stride];
        }
        // the step's kVecUnroll products summed in T, then added to the FP64 accumulators
        T sre = T(0), sim = T(0);
#pragma unroll
        for (int u = 0; u < kVecUnroll; ++u) {
            const cplx<T> ap = pv[u] - yv[u];
            ys[q + u * stride] = ap;
            sre = fma(pv[u].re, ap.re, fma(pv[u].im, ap.im, sre));
            sim = fma(pv[u].re, ap.im, fma(-pv[u].im, ap.re, sim));
        }
        are += (double)sre;
        aim += (double)sim;
    }
    for (; q < N; q += stride) body(ps[q], ys[q], q);
    const double2 t = block_sum2(are, aim);
    if (threadIdx.x == 0) {
        part[2 * ((long long)s * G + blockIdx.x)] = t.x;
        part[2 * ((long long)s * G + blockIdx.x) + 1] = t.y;
    }
}

// alpha = ||r||^2 / pAp (complex, as CGMN.m:68-69 where pAp = sum(conj(p).*Ap)).
__global__ void k_alpha(CgState st)
{
    const int s = blockIdx.x;
    if (!st.active[s]) return;
    const double2 pap = sum_partials(st.part, st.G, s);
    if (threadIdx.x == 0) {
        const double d = pap.x * pap.x + pap.y * pap.y;
        const double rr = st.rr[s];
        st.alpha[2 * s] = rr * pap.x / d;
        st.alpha[2 * s + 1] = -rr * pap.y / d;
        if (!(d > 0.0) || !isfinite(d)) {
            st.alpha[2 * s] = 0.0;
            st.alpha[2 * s + 1] = 0.0;
            st.status[s] = H3D_ERR_NONFINITE;
        }
    }
}

template <typename T>
int cg_ap_dot(const cplx<T> *p, cplx<T> *y, long long N, int nrhs, const CgState &s,
              cudaStream_t st)
{
    k_ap_dot<T><<<dim3(s.G, nrhs), kVecThreads, 0, st>>>(p, y, ColMap{s.coloff, s.collen, N}, s.active,
                                                         s.part, s.G);
    k_alpha<<<nrhs, kVecThreads, 0, st>>>(s);
    H3D_CUDA_TRY(cudaGetLastError());
    return H3D_OK;
}

// x += alpha p; r -= alpha Ap; partial ||r||^2.
template <typename T>
__global__ void k_update_xr(cplx<T> *__restrict__ x, cplx<T> *__restrict__ r,
                            const cplx<T> *__restrict__ p, const cplx<T> *__restrict__ ap,
                            ColMap cm, const int *__restrict__ active,
                            const double *__restrict__ alpha, double *part, int G)
{
    const int s = blockIdx.y;
    if (!active[s]) return;
    const long long off = cm.o(s), N = cm.n(s);
    cplx<T> *xs = x + off, *rs = r + off;
    const cplx<T> *ps = p + off, *as = ap + off;
    const cplx<T> a = mk<T>((T)alpha[2 * s], (T)alpha[2 * s + 1]);
    double acc = 0.0;
    auto body = [&](const cplx<T> pv, const cplx<T> av, cplx<T> xv, cplx<T> rv, long long q) {
        xv = xv + pv * a;
        rv = rv - av * a;
        xs[q] = xv;
        rs[q] = rv;
        acc += (double)rv.re * rv.re + (double)rv.im * rv.im;
    };
    const long long stride = (long long)G * blockDim.x;
    long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    for (; q + (kVecUnroll - 1) * stride < N; q += kVecUnroll * stride) {
        cplx<T> pv[kVecUnroll], av[kVecUnroll], xv[kVecUnroll], rv[kVecUnroll];
#pragma unroll
        for (int u = 0; u < kVecUnroll; ++u) {
            pv[u] = ps[q + u * stride];
            av[u] = as[q + u * stride];
            xv[u] = xs[q + u * stride];
            rv[u] = rs[q + u * stride];
        }
        T sr = T(0);  // the step's squared norms summed in T, then added in FP64
#pragma unroll
        for (int u = 0; u < kVecUnroll; ++u) {
            const cplx<T> xn = xv[u] + pv[u] * a, rn = rv[u] - av[u] * a;
            xs[q + u * stride] = xn;
            rs[q + u * stride] = rn;
            sr = fma(rn.re, rn.re, fma(rn.im, rn.im, sr));
        }
        acc += (double)sr;
    }
    for (; q < N; q += stride) body(ps[q], as[q], xs[q], rs[q], q);
    const double2 t = block_sum2(acc, 0.0);
    if (threadIdx.x == 0) {
        part[2 * ((long long)s * G + blockIdx.x)] = t.x;
        part[2 * ((long long)s * G + blockIdx.x) + 1] = 0.0;
    }
}

// Stop test and beta (CGMN.m:74-83), per RHS instead of the max over columns.
__global__ void k_beta(CgState st, int maxit)
{
    const int s = blockIdx.x;
    const int was = st.active[s];
    if (threadIdx.x == 0) st.upd[s] = was;
    if (!was) return;
    const double2 t = sum_partials(st.part, st.G, s);
    if (threadIdx.x == 0) {
        const double rn = t.x, ro = st.rr[s];
        const double ratio = sqrt(rn / st.bb[s]);
        const int it = st.iters[s] + 1;
        st.iters[s] = it;
        st.ratio[s] = ratio;
        st.beta[s] = rn / ro;
        st.rr[s] = rn;
        if (!isfinite(rn) || st.status[s]) {
            st.status[s] = H3D_ERR_NONFINITE;
            st.active[s] = 0;
            st.upd[s] = 0;
        } else if (ratio <= st.tolp[s] || it >= maxit) {
            st.active[s] = 0;
        }
    }
}

template <typename T>
int cg_update_xr(cplx<T> *x, cplx<T> *r, const cplx<T> *p, const cplx<T> *ap, long long N,
                 int nrhs, const CgState &s, int maxit, cudaStream_t st)
{
    k_update_xr<T><<<dim3(s.G, nrhs), kVecThreads, 0, st>>>(x, r, p, ap, ColMap{s.coloff, s.collen, N},
                                                            s.active, s.alpha, s.part, s.G);
    k_beta<<<nrhs, kVecThreads, 0, st>>>(s, maxit);
    H3D_CUDA_TRY(cudaGetLastError());
    return H3D_OK;
}

// p = r + beta p; y = p (the copy the next sweep works on).
template <typename T>
__global__ void k_update_p(cplx<T> *__restrict__ p, const cplx<T> *__restrict__ r,
                           cplx<T> *__restrict__ y, ColMap cm, const int *__restrict__ upd,
                           const double *__restrict__ beta, int G)
{
    const int s = blockIdx.y;
    if (!upd[s]) return;
    const long long off = cm.o(s), N = cm.n(s);
    cplx<T> *ps = p + off, *ys = y + off;
    const cplx<T> *rs = r + off;
    const T b = (T)beta[s];
    const long long stride = (long long)G * blockDim.x;
    long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    for (; q + (kVecUnroll - 1) * stride < N; q += kVecUnroll * stride) {
        cplx<T> rv[kVecUnroll], pv[kVecUnroll];
#pragma unroll
        for (int u = 0; u < kVecUnroll; ++u) {
            rv[u] = rs[q + u * stride];
            pv[u] = ps[q + u * stride];
        }
#pragma unroll
        for (int u = 0; u < kVecUnroll; ++u) {
            const cplx<T> v = rv[u] + b * pv[u];
            ps[q + u * stride] = v;
            ys[q + u * stride] = v;
        }
    }
    for (; q < N; q += stride) {
        const cplx<T> v = rs[q] + b * ps[q];
        ps[q] = v;
        ys[q] = v;
    }
}

template <typename T>
int cg_update_p(cplx<T> *p, const cplx<T> *r, cplx<T> *y, long long N, int nrhs,
                const CgState &s, cudaStream_t st)
{
    k_update_p<T><<<dim3(s.G, nrhs), kVecThreads, 0, st>>>(p, r, y, ColMap{s.coloff, s.collen, N}, s.upd,
                                                           s.beta, s.G);
    H3D_CUDA_TRY(cudaGetLastError());
    return H3D_OK;
}

// ---- CRMN ------------------------------------------------------------------------------
// x += gamma p; r -= gamma Ap; y = r; partial ||r||^2 (CRMN.m:79-81).
template <typename T>
__global__ void k_cr_update_xr(cplx<T> *__restrict__ x, cplx<T> *__restrict__ r,
                               const cplx<T> *__restrict__ p, const cplx<T> *__restrict__ ap,
                               cplx<T> *__restrict__ y, ColMap cm, const int *__restrict__ active,
                               const double *__restrict__ gamma, double *part, int G)
{
    const int s = blockIdx.y;
    if (!active[s]) return;
    const long long off = cm.o(s), N = cm.n(s);
    cplx<T> *xs = x + off, *rs = r + off, *ys = y + off;
    const cplx<T> *ps = p + off, *as = ap + off;
    const cplx<T> g = mk<T>((T)gamma[2 * s], (T)gamma[2 * s + 1]);
    double acc = 0.0;
    auto body = [&](const cplx<T> pv, const cplx<T> av, cplx<T> xv, cplx<T> rv, long long q) {
        xv = xv + pv * g;
        rv = rv - av * g;
        xs[q] = xv;
        rs[q] = rv;
        ys[q] = rv;
        acc += (double)rv.re * rv.re + (double)rv.im * rv.im;
    };
    const long long stride = (long long)G * blockDim.x;
    long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    for (; q + (kVecUnroll - 1) * stride < N; q += kVecUnroll * stride) {
        cplx<T> pv[kVecUnroll], av[kVecUnroll], xv[kVecUnroll], rv[kVecUnroll];
#pragma unroll
        for (int u = 0; u < kVecUnroll; ++u) {
            pv[u] = ps[q + u * stride];
            av[u] = as[q + u * stride];
            xv[u] = xs[q + u * stride];
            rv[u] = rs[q + u * stride];
        }
#pragma unroll
        for (int u = 0; u < kVecUnroll; ++u) body(pv[u], av[u], xv[u], rv[u], q + u * stride);
    }
    for (; q < N; q += stride) body(ps[q], as[q], xs[q], rs[q], q);
    const double2 t = block_sum2(acc, 0.0);
    if (threadIdx.x == 0) {
        part[2 * ((long long)s * G + blockIdx.x)] = t.x;
        part[2 * ((long long)s * G + blockIdx.x) + 1] = 0.0;
    }
}

template <typename T>
int cr_update_xr(cplx<T> *x, cplx<T> *r, const cplx<T> *p, const cplx<T> *ap, cplx<T> *y,
                 long long N, int nrhs, const CgState &s, int maxit, cudaStream_t st)
{
    k_cr_update_xr<T><<<dim3(s.G, nrhs), kVecThreads, 0, st>>>(x, r, p, ap, y, ColMap{s.coloff, s.collen, N},
                                                               s.active, s.alpha, s.part, s.G);
    k_beta<<<nrhs, kVecThreads, 0, st>>>(s, maxit);  // ||r||, iteration count, stop test
    H3D_CUDA_TRY(cudaGetLastError());
    return H3D_OK;
}

// Ar = r - y over y and partial <r, Ar> (CRMN.m:94-97): the CGMN kernel with p -> r.
template <typename T>
int cr_ar_dot(const cplx<T> *r, cplx<T> *y, long long N, int nrhs, const CgState &s, cudaStream_t st)
{
    k_ap_dot<T><<<dim3(s.G, nrhs), kVecThreads, 0, st>>>(r, y, ColMap{s.coloff, s.collen, N}, s.active,
                                                         s.part, s.G);
    H3D_CUDA_TRY(cudaGetLastError());
    return H3D_OK;
}

// beta = rAr_new / rAr_old (complex; 0 on the first call); rAr_old = rAr_new (CRMN.m:96-102).
__global__ void k_cr_beta(CgState st, int first)
{
    const int s = blockIdx.x;
    if (!st.active[s]) return;
    const double2 rar = sum_partials(st.part, st.G, s);
    if (threadIdx.x == 0) {
        double br = 0.0, bi = 0.0;
        if (!first) {
            const double orr = st.rar[2 * s], oi = st.rar[2 * s + 1];
            const double d = orr * orr + oi * oi;
            br = (rar.x * orr + rar.y * oi) / d;
            bi = (rar.y * orr - rar.x * oi) / d;
            if (!(d > 0.0) || !isfinite(br) || !isfinite(bi)) {
                br = bi = 0.0;
                st.status[s] = H3D_ERR_NONFINITE;
            }
        }
        st.cbeta[2 * s] = br;
        st.cbeta[2 * s + 1] = bi;
        st.rar[2 * s] = rar.x;
        st.rar[2 * s + 1] = rar.y;
    }
}

// p = r + beta p; Ap = Ar + beta Ap; partial ||Ap||^2 (CRMN.m:103-105).
template <typename T>
__global__ void k_cr_update_p(cplx<T> *__restrict__ p, cplx<T> *__restrict__ ap,
                              const cplx<T> *__restrict__ r, const cplx<T> *__restrict__ ar, ColMap cm,
                              const int *__restrict__ active, const double *__restrict__ cbeta,
                              double *part, int G)
{
    const int s = blockIdx.y;
    if (!active[s]) return;
    const long long off = cm.o(s), N = cm.n(s);
    cplx<T> *ps = p + off, *aps = ap + off;
    const cplx<T> *rs = r + off, *ars = ar + off;
    const cplx<T> b = mk<T>((T)cbeta[2 * s], (T)cbeta[2 * s + 1]);
    double acc = 0.0;
    auto body = [&](const cplx<T> rv, const cplx<T> arv, const cplx<T> pv, const cplx<T> apv, long long q) {
        const cplx<T> pn = rv + pv * b;
        const cplx<T> an = arv + apv * b;
        ps[q] = pn;
        aps[q] = an;
        acc += (double)an.re * an.re + (double)an.im * an.im;
    };
    const long long stride = (long long)G * blockDim.x;
    long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    for (; q + (kVecUnroll - 1) * stride < N; q += kVecUnroll * stride) {
        cplx<T> rv[kVecUnroll], arv[kVecUnroll], pv[kVecUnroll], apv[kVecUnroll];
#pragma unroll
        for (int u = 0; u < kVecUnroll; ++u) {
            rv[u] = rs[q + u * stride];
            arv[u] = ars[q + u * stride];
            pv[u] = ps[q + u * stride];
            apv[u] = aps[q + u * stride];
        }
#pragma unroll
        for (int u = 0; u < kVecUnroll; ++u) body(rv[u], arv[u], pv[u], apv[u], q + u * stride);
    }
    for (; q < N; q += stride) body(rs[q], ars[q], ps[q], aps[q], q);
    const double2 t = block_sum2(acc, 0.0);
    if (threadIdx.x == 0) {
        part[2 * ((long long)s * G + blockIdx.x)] = t.x;
        part[2 * ((long long)s * G + blockIdx.x) + 1] = 0.0;
    }
}

// gamma = rAr / ||Ap||^2 (complex over real, CRMN.m:73-77).
__global__ void k_cr_gamma(CgState st)
{
    const int s = blockIdx.x;
    if (!st.active[s]) return;
    const double2 n = sum_partials(st.part, st.G, s);
    if (threadIdx.x == 0) {
        st.nap2[s] = n.x;
        double gr = st.rar[2 * s] / n.x, gi = st.rar[2 * s + 1] / n.x;
        if (!(n.x > 0.0) || !isfinite(gr) || !isfinite(gi)) {
            gr = gi = 0.0;
            st.status[s] = H3D_ERR_NONFINITE;
        }
        st.alpha[2 * s] = gr;
        st.alpha[2 * s + 1] = gi;
    }
}

template <typename T>
int cr_update_p(cplx<T> *p, cplx<T> *ap, const cplx<T> *r, const cplx<T> *ar, long long N, int nrhs,
                const CgState &s, bool first, cudaStream_t st)
{
    k_cr_beta<<<nrhs, kVecThreads, 0, st>>>(s, first ? 1 : 0);
    k_cr_update_p<T><<<dim3(s.G, nrhs), kVecThreads, 0, st>>>(p, ap, r, ar, ColMap{s.coloff, s.collen, N},
                                                              s.active, s.cbeta, s.part, s.G);
    k_cr_gamma<<<nrhs, kVecThreads, 0, st>>>(s);
    H3D_CUDA_TRY(cudaGetLastError());
    return H3D_OK;
}

template <typename T>
__global__ void k_copy_active(const cplx<T> *__restrict__ src, cplx<T> *__restrict__ dst,
                              long long N, const int *__restrict__ active, int G)
{
    const int s = blockIdx.y;
    if (active && !active[s]) return;
    const long long off = (long long)s * N;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < N;
         q += (long long)G * blockDim.x)
        dst[off + q] = src[off + q];
}

template <typename T>
int copy_active(const cplx<T> *src, cplx<T> *dst, long long N, int nrhs, const int *active,
                cudaStream_t st)
{
    const int G = reduction_blocks(N);
    k_copy_active<T><<<dim3(G, nrhs), kVecThreads, 0, st>>>(src, dst, N, active, G);
    H3D_CUDA_TRY(cudaGetLastError());
    return H3D_OK;
}

template <typename T>
int zero_vec(cplx<T> *v, long long N, int nrhs, cudaStream_t st)
{
    H3D_CUDA_TRY(cudaMemsetAsync(v, 0, sizeof(cplx<T>) * (size_t)N * nrhs, st));
    return H3D_OK;
}

__global__ void k_scale_to_c64(const cplx<double> *__restrict__ src, cplx<float> *__restrict__ dst,
                               long long N, const double *__restrict__ norm2,
                               const int *__restrict__ active, int G)
{
    const int s = blockIdx.y;
    const long long off = (long long)s * N;
    const bool on = !active || active[s];
    const double sc = (on && norm2[s] > 0.0) ? 1.0 / sqrt(norm2[s]) : 0.0;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < N;
         q += (long long)G * blockDim.x) {
        const cplx<double> v = src[off + q];
        dst[off + q] = mk<float>((float)(v.re * sc), (float)(v.im * sc));
    }
}

int scale_to_c64(const cplx<double> *src, cplx<float> *dst, long long N, int nrhs,
                 const double *norm2, const int *active, cudaStream_t st)
{
    const int G = reduction_blocks(N);
    k_scale_to_c64<<<dim3(G, nrhs), kVecThreads, 0, st>>>(src, dst, N, norm2, active, G);
    H3D_CUDA_TRY(cudaGetLastError());
    return H3D_OK;
}

__global__ void k_add_scaled_c64(cplx<double> *__restrict__ u, const cplx<float> *__restrict__ e,
                                 long long N, const double *__restrict__ norm2,
                                 const int *__restrict__ active, int G)
{
    const int s = blockIdx.y;
    if (active && !active[s]) return;
    const long long off = (long long)s * N;
    const double sc = sqrt(norm2[s]);
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < N;
         q += (long long)G * blockDim.x) {
        const cplx<float> v = e[off + q];
        cplx<double> o = u[off + q];
        o.re += sc * (double)v.re;
        o.im += sc * (double)v.im;
        u[off + q] = o;
    }
}

int add_scaled_c64(cplx<double> *u, const cplx<float> *e, long long N, int nrhs,
                   const double *norm2, const int *active, cudaStream_t st)
{
    const int G = reduction_blocks(N);
    k_add_scaled_c64<<<dim3(G, nrhs), kVecThreads, 0, st>>>(u, e, N, norm2, active, G);
    H3D_CUDA_TRY(cudaGetLastError());
    return H3D_OK;
}

#define H3D_INST(T)                                                                                   \
    template int cg_init<T>(const cplx<T> *, cplx<T> *, cplx<T> *, cplx<T> *, long long, int,         \
                            const CgState &, const double *, double, int, cudaStream_t);               \
    template int cg_ap_dot<T>(const cplx<T> *, cplx<T> *, long long, int, const CgState &,             \
                              cudaStream_t);                                                           \
    template int cg_update_xr<T>(cplx<T> *, cplx<T> *, const cplx<T> *, const cplx<T> *, long long,   \
                                 int, const CgState &, int, cudaStream_t);                             \
    template int cg_update_p<T>(cplx<T> *, const cplx<T> *, cplx<T> *, long long, int,                 \
                                const CgState &, cudaStream_t);                                        \
    template int cr_update_xr<T>(cplx<T> *, cplx<T> *, const cplx<T> *, const cplx<T> *, cplx<T> *,    \
                                 long long, int, const CgState &, int, cudaStream_t);                  \
    template int cr_ar_dot<T>(const cplx<T> *, cplx<T> *, long long, int, const CgState &, cudaStream_t); \
    template int cr_update_p<T>(cplx<T> *, cplx<T> *, const cplx<T> *, const cplx<T> *, long long, int, \
                                const CgState &, bool, cudaStream_t);                                  \
    template int copy_active<T>(const cplx<T> *, cplx<T> *, long long, int, const int *, cudaStream_t); \
    template int zero_vec<T>(cplx<T> *, long long, int, cudaStream_t);
H3D_INST(double)
H3D_INST(float)
#undef H3D_INST

}  // namespace h3d
