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
    long long g = (N + 4LL * kVecThreads - 1) / (4LL * kVecThreads);
    if (g > 304) g = 304;
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
                       cplx<T> *__restrict__ r, cplx<T> *__restrict__ p, long long N, double *part,
                       int G)
{
    const int s = blockIdx.y;
    const long long off = (long long)s * N;
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
    k_init<T><<<dim3(s.G, nrhs), kVecThreads, 0, st>>>(bt, x, r, p, N, s.part, s.G);
    k_init_state<<<nrhs, kVecThreads, 0, st>>>(s, bnorm2_orig, zero_tol2, nrhs);
    H3D_CUDA_TRY(cudaGetLastError());
    return H3D_OK;
}

// Ap = p - y (written over y), partial <p, Ap> (complex).
template <typename T>
__global__ void k_ap_dot(const cplx<T> *__restrict__ p, cplx<T> *__restrict__ y, long long N,
                         const int *__restrict__ active, double *part, int G)
{
    const int s = blockIdx.y;
    if (!active[s]) return;
    const long long off = (long long)s * N;
    double are = 0.0, aim = 0.0;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < N;
         q += (long long)G * blockDim.x) {
        const cplx<T> pv = p[off + q], yv = y[off + q];
        const cplx<T> ap = pv - yv;
        y[off + q] = ap;
        are += (double)pv.re * ap.re + (double)pv.im * ap.im;
        aim += (double)pv.re * ap.im - (double)pv.im * ap.re;
    }
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
    k_ap_dot<T><<<dim3(s.G, nrhs), kVecThreads, 0, st>>>(p, y, N, s.active, s.part, s.G);
    k_alpha<<<nrhs, kVecThreads, 0, st>>>(s);
    H3D_CUDA_TRY(cudaGetLastError());
    return H3D_OK;
}

// x += alpha p; r -= alpha Ap; partial ||r||^2.
template <typename T>
__global__ void k_update_xr(cplx<T> *__restrict__ x, cplx<T> *__restrict__ r,
                            const cplx<T> *__restrict__ p, const cplx<T> *__restrict__ ap,
                            long long N, const int *__restrict__ active,
                            const double *__restrict__ alpha, double *part, int G)
{
    const int s = blockIdx.y;
    if (!active[s]) return;
    const long long off = (long long)s * N;
    const cplx<T> a = mk<T>((T)alpha[2 * s], (T)alpha[2 * s + 1]);
    double acc = 0.0;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < N;
         q += (long long)G * blockDim.x) {
        const cplx<T> pv = p[off + q], av = ap[off + q];
        cplx<T> xv = x[off + q], rv = r[off + q];
        xv = xv + pv * a;
        rv = rv - av * a;
        x[off + q] = xv;
        r[off + q] = rv;
        acc += (double)rv.re * rv.re + (double)rv.im * rv.im;
    }
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
    k_update_xr<T><<<dim3(s.G, nrhs), kVecThreads, 0, st>>>(x, r, p, ap, N, s.active, s.alpha,
                                                            s.part, s.G);
    k_beta<<<nrhs, kVecThreads, 0, st>>>(s, maxit);
    H3D_CUDA_TRY(cudaGetLastError());
    return H3D_OK;
}

// p = r + beta p; y = p (the copy the next sweep works on).
template <typename T>
__global__ void k_update_p(cplx<T> *__restrict__ p, const cplx<T> *__restrict__ r,
                           cplx<T> *__restrict__ y, long long N, const int *__restrict__ upd,
                           const double *__restrict__ beta, int G)
{
    const int s = blockIdx.y;
    if (!upd[s]) return;
    const long long off = (long long)s * N;
    const T b = (T)beta[s];
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < N;
         q += (long long)G * blockDim.x) {
        const cplx<T> v = r[off + q] + b * p[off + q];
        p[off + q] = v;
        y[off + q] = v;
    }
}

template <typename T>
int cg_update_p(cplx<T> *p, const cplx<T> *r, cplx<T> *y, long long N, int nrhs,
                const CgState &s, cudaStream_t st)
{
    k_update_p<T><<<dim3(s.G, nrhs), kVecThreads, 0, st>>>(p, r, y, N, s.upd, s.beta, s.G);
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
    template int copy_active<T>(const cplx<T> *, cplx<T> *, long long, int, const int *, cudaStream_t); \
    template int zero_vec<T>(cplx<T> *, long long, int, cudaStream_t);
H3D_INST(double)
H3D_INST(float)
#undef H3D_INST

}  // namespace h3d
