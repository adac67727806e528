// CGMN building blocks (tools/solvers/Krylov/CGMN.m:48-90 on the Kaczmarz-preconditioned
// system of linearsolve.m:148-156): per-right-hand-side vector updates with masks and
// deterministic FP64 reductions.  Storage precision T is double (plain FP64 path) or float
// (complex64 inner solves of the mixed-precision path); inner products, norms and the
// CG scalars are always accumulated and kept in double.
#pragma once

#include "h3d_internal.cuh"

namespace h3d {

// Per-RHS scalar state of one CGMN instance (device arrays, nrhs entries each).
struct CgState {
    double *rr;       // ||r||^2 (current)
    double *bb;       // ||b~||^2 (preconditioned right-hand side)
    double *ratio;    // ||r|| / ||b~|| after the last iteration
    double *tolp;     // per-RHS tolerance on ratio
    double *alpha;    // complex alpha (re, im) pairs
    double *beta;     // real beta
    int *active;      // 1 while iterating
    int *upd;         // 1 if the RHS took part in the current iteration
    int *iters;       // iterations done
    int *status;      // 0 ok, H3D_ERR_NONFINITE on NaN/Inf
    double *part;     // reduction partials: nrhs x G x 2
    int G;            // reduction blocks per RHS
    // Column map of a batch of problems of uneven size (null: column s of N elements at s N):
    // column s spans [coloff[s], coloff[s] + collen[s]) of every vector.
    const long long *coloff = nullptr, *collen = nullptr;
    // CRMN only (null for CGMN): complex <r, A r> (re, im) pairs, complex beta pairs,
    // ||A p||^2; alpha holds gamma.
    double *rar = nullptr, *cbeta = nullptr, *nap2 = nullptr;
};

// Where column s of the CG vectors lives (see CgState::coloff).
struct ColMap {
    const long long *off, *len;
    long long N;
    __device__ __forceinline__ long long o(int s) const { return off ? off[s] : (long long)s * N; }
    __device__ __forceinline__ long long n(int s) const { return len ? len[s] : N; }
};

constexpr int kVecThreads = 256;
constexpr int kVecUnroll = 4;  // independent elements per thread and loop step

template <typename T>
int cg_init(const cplx<T> *bt, cplx<T> *x, cplx<T> *r, cplx<T> *p, long long N, int nrhs,
            const CgState &s, const double *bnorm2_orig, double zero_tol2, int maxit,
            cudaStream_t st);
template <typename T>
int cg_ap_dot(const cplx<T> *p, cplx<T> *y, long long N, int nrhs, const CgState &s,
              cudaStream_t st);
template <typename T>
int cg_update_xr(cplx<T> *x, cplx<T> *r, const cplx<T> *p, const cplx<T> *ap, long long N,
                 int nrhs, const CgState &s, int maxit, cudaStream_t st);
template <typename T>
int cg_update_p(cplx<T> *p, const cplx<T> *r, cplx<T> *y, long long N, int nrhs,
                const CgState &s, cudaStream_t st);
// CRMN building blocks (CRMN.m:54-105), on the same masks and reductions.
//   cr_update_xr: x += gamma p; r -= gamma Ap; y = r (the next sweep's input); ||r||^2 and
//                 the stop test (CRMN.m:79-92)
//   cr_ar_dot:    Ar = r - y over y, <r, Ar>                        (CRMN.m:94-97)
//   cr_update_p:  beta = rAr / rAr_old (0 when first); p = r + beta p; Ap = Ar + beta Ap;
//                 ||Ap||^2; gamma = rAr / ||Ap||^2                   (CRMN.m:73-77, 98-105)
template <typename T>
int cr_update_xr(cplx<T> *x, cplx<T> *r, const cplx<T> *p, const cplx<T> *ap, cplx<T> *y,
                 long long N, int nrhs, const CgState &s, int maxit, cudaStream_t st);
template <typename T>
int cr_ar_dot(const cplx<T> *r, cplx<T> *y, long long N, int nrhs, const CgState &s, cudaStream_t st);
template <typename T>
int cr_update_p(cplx<T> *p, cplx<T> *ap, const cplx<T> *r, const cplx<T> *ar, long long N,
                int nrhs, const CgState &s, bool first, cudaStream_t st);

template <typename T>
int copy_active(const cplx<T> *src, cplx<T> *dst, long long N, int nrhs, const int *active,
                cudaStream_t st);
template <typename T>
int zero_vec(cplx<T> *v, long long N, int nrhs, cudaStream_t st);

// Mixed precision glue.
// dst32[s] = (complex64)(src64[s] * scale[s])   with scale[s] = 1/||src64[s]|| (0 if inactive)
int scale_to_c64(const cplx<double> *src, cplx<float> *dst, long long N, int nrhs,
                 const double *norm2, const int *active, cudaStream_t st);
// u64[s] += sqrt(norm2[s]) * (complex128) e32[s]   for active s
int add_scaled_c64(cplx<double> *u, const cplx<float> *e, long long N, int nrhs,
                   const double *norm2, const int *active, cudaStream_t st);

// FP64 residual r = b - A x with per-RHS ||r||^2 and ||b||^2 (h3d_solver.cu).
int residual_f64(const Op<double> &op, const cplx<double> *b, const cplx<double> *x,
                 cplx<double> *r, double *rr2, double *bb2, int nrhs, bool adj, double *part,
                 int G, cudaStream_t st);

int reduction_blocks(long long N);

}  // namespace h3d
