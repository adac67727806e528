/*
 * h3d -- GB300-native 3D frequency-domain Helmholtz hot path (27-point stencil with PML).
 *
 * Plain C ABI: plain pointers and sizes, no C++ or framework types.  Complex
 * device vectors are interleaved (re, im) pairs of double (H3D_C128) or float
 * (H3D_C64), column-major over the grid (x fastest, idx = i + j*nx + k*nx*ny)
 * with right-hand side s at offset s*N.  Wavenumber arrays hold N real values
 * (plus an optional imaginary plane for complex frequencies).
 *
 * Entry points and the reference interface each one replaces
 * (paths inside the reference project SLIM-release-apps):
 *
 *   h3d_mvp            Helm3dmvp_{forw,adj}[_wnc|_deriv]_mex
 *                      (tools/algorithms/3DFreqModeling/Helm3dmvp_mex.c:58-107,
 *                       dispatch helm3d_operto27_mvp.m:22-42)
 *   h3d_kacz_sweep     Helm3d_kacz_sweep{,_wnc,_adj}_mex
 *                      (tools/algorithms/3DFreqModeling/Helm3dkaczswp_mex.c:123-199,
 *                       dispatch helm3d_operto27_kaczswp.m:20-30)
 *   h3d_mex_mvp,       the same two gateways with MATLAB's host-side argument list
 *   h3d_mex_kacz_sweep (separate real/imag double planes, n and npml as doubles);
 *                      used by the drop-in MEX gateway
 *   h3d_solve          H\b and H'\b through linearsolve + CGMN with the Kaczmarz
 *                      preconditioner (tools/solvers/Krylov/linearsolve.m:148-168,
 *                      CGMN.m:36-94, opAbstractMatrix.m:117-125)
 *   h3d_solve_batch    many (problem, right-hand side) solves of uneven size in one launch
 *                      sequence (the (src,freq) loop of PDEfunc.m:254-347 batched: one CGMN
 *                      iteration over every column, one BLOCK8 launch per block parity over
 *                      every problem)
 *   h3d_mex_solve      the same solve with MATLAB's host arrays (the h3d_solve_mex gateway,
 *                      a drop-in for linearsolve(H,b,x0,mode,lsopts) on a Helmholtz operator)
 *   h3d_fwi_grad       PDEfunc OBJ (f and g) for one frequency and a batch of sources, host
 *                      buffers (PDEfunc.m:254-394)
 *   h3d_grad_accum     T_adj(z,u) = conj(u).*(dH'*z) summed over sources and cropped to the
 *                      physical grid (discrete_helmholtz.m:288, PDEfunc.m:386,394)
 *   h3d_src_inject,    sinc-Kaiser source injection Ps and receiver sampling Pr
 *   h3d_rec_sample,    (opInterp.m:34-58, opSincInterp.m:26-70, DataGrid.m:22-44)
 *   h3d_rec_spread
 *   h3d_axis_apply     grid transfers of the ML_GMRES multigrid preconditioner
 *                      (construct_multigrid.m:45-51, fine2coarse.m:40-55: Kronecker
 *                       products of 1D interpolation operators, one axis per call)
 *   h3d_mlgmres_solve  linearsolve with SOLVE_FGMRES and PREC_MLGMRES (FGMRES.m, ML_GMRES.m,
 *                      opMultigrid.m): the 3D applications' default solver; _model and the
 *                      h3d_mex_mlgmres host entry build the hierarchy from the physical model
 *                      (construct_multigrid.m)
 *   h3d_band_coefs     the band-storage (mat_free = false) operator: helmholtz_3d.m:35-190
 *                      (27 x N bands of H) and conj(Htransp(H)) (opBandStorage.m:127-129)
 *   h3d_band_mvp       Hmvp_MT_mex (Hmvp_MT_mex.c:53-73, via Hmvp.m / opBandStorage.multiply)
 *   h3d_band_sweep     sweep_MT_mex (sweep_MT_mex.c:55-97, via opBandStorage.kacz_sweep)
 *   h3d_mex_band_mvp,  host entries of the drop-in Hmvp_MT_mex / sweep_MT_mex gateways
 *   h3d_mex_band_sweep (Hmvp_MT_mex.c:76-141, sweep_MT_mex.c:100-188; ibin/install_MEX:75-86)
 *
 * Every call is asynchronous on the given CUDA stream (NULL = legacy default
 * stream) unless documented otherwise; all pointers are device pointers unless
 * the function name says "mex"/"host".  The library keeps no state between calls
 * except cached device properties and the kernels' constant tables.
 */
#ifndef H3D_H
#define H3D_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define H3D_API_VERSION 1

/* Status codes.  The reference reports errors with mexErrMsgIdAndTxt
 * (Helm3dmvp_mex.c:75-85, Helm3dkaczswp_mex.c:143-164); h3d_status_id() maps a
 * code to the matching reference error identifier. */
typedef enum {
    H3D_OK = 0,
    H3D_ERR_NSIZE = 1,          /* n must be a 3-length vector of positive sizes */
    H3D_ERR_XSIZE = 2,          /* x must have nx*ny*nz rows */
    H3D_ERR_BSIZE = 3,          /* b must have nx*ny*nz rows */
    H3D_ERR_BAD_ARG = 4,        /* other invalid argument (NULL pointer, bad mode, w out of (0,2), ...) */
    H3D_ERR_NOT_CONVERGED = 5,  /* solver hit maxit before the tolerance */
    H3D_ERR_TIMEOUT = 6,        /* a bounded device-side wait expired */
    H3D_ERR_CUDA = 7,           /* CUDA runtime error (message via h3d_last_error) */
    H3D_ERR_NO_MEMORY = 8,
    H3D_ERR_NONFINITE = 9       /* NaN/Inf met in the iteration */
} h3d_status;

typedef enum { H3D_C128 = 0, H3D_C64 = 1 } h3d_dtype;
typedef enum { H3D_FORWARD = 1, H3D_ADJOINT = 2 } h3d_mode;

/* Kaczmarz row orderings of one double sweep.
 *  LEX       the reference's lexicographic order (k, j, i ascending, then descending):
 *            bit-compatible with Helm3d_kacz_sweep_mex.  Executed as hyperplane
 *            wavefronts t = i + 3j + 9k (no two rows on a plane share a neighbour,
 *            and every pair of rows that does is ordered as in the reference).
 *  COLOUR27  27 colour classes q = (i%3) + 3(j%3) + 9(k%3), ascending then descending.
 *  BLOCK     blocks of block[0..2] points visited by the block wavefront
 *            T = I + 2J + 4K, COLOUR27 order inside each block.
 *  BLOCK8    blocks of block[0..2] points (12x12x12 or 24x12x12; 0 = tuned) in eight
 *            parity classes p = I%2 + 2(J%2) + 4(K%2), ascending then descending,
 *            COLOUR27 order inside each block; each block is processed in shared
 *            memory, eight launches per pass.
 * All four give a symmetric double sweep, hence a Hermitian positive
 * semi-definite I - Q for CGMN; they differ in the iterates, not the solution. */
typedef enum { H3D_ORDER_LEX = 0, H3D_ORDER_COLOUR27 = 1, H3D_ORDER_BLOCK = 2, H3D_ORDER_BLOCK8 = 3 } h3d_order;

typedef enum { H3D_PREC_FP64 = 0, H3D_PREC_MIXED = 1 } h3d_precision;

/* Krylov method on (I - Q) u = DSWP(0, b): CGMN (CGMN.m, the default of LinSolveOpts) or
 * CRMN (CRMN.m, LinSolveOpts.SOLVE_CRMN); both dispatched by linearsolve.m:51-64. */
typedef enum { H3D_METHOD_CGMN = 0, H3D_METHOD_CRMN = 1 } h3d_method;

/* Stopping rules.  PRECONDITIONED is CGMN.m:79 (max over columns of the
 * preconditioned residual ratio <= tol); TRUE_RESIDUAL requires
 * ||b - H u||_2 / ||b||_2 <= tol for every right-hand side. */
typedef enum { H3D_STOP_PRECONDITIONED = 0, H3D_STOP_TRUE_RESIDUAL = 1 } h3d_stop_rule;

typedef struct h3d_grid {
    int32_t n[3];     /* nx, ny, nz including the PML */
    double h[3];      /* grid spacing hx, hy, hz */
    int32_t npml[6];  /* lo_x, hi_x, lo_y, hi_y, lo_z, hi_z: the reference's 2x3 npml, column-major */
} h3d_grid;

typedef struct h3d_solve_opts {
    double tol;             /* default 1e-6 (LinSolveOpts.m:56) */
    int32_t maxit;          /* default 10000 (LinSolveOpts.m:57); inner iterations cap */
    double w;               /* relaxation, default 1.5 (linearsolve.m:150) */
    int32_t precision;      /* h3d_precision */
    int32_t order;          /* h3d_order, default BLOCK8 */
    int32_t stop_rule;      /* h3d_stop_rule */
    int32_t check_every;    /* iterations between host-visible convergence checks (graph length) */
    double inner_tol;       /* MIXED: relative tolerance of the first complex64 inner solve; a
                               later one aims at half the reduction still needed (tol over the
                               current true residual), between inner_tol and 0.1 */
    int32_t max_outer;      /* MIXED: maximum refinement steps */
    int32_t block[3];       /* BLOCK / BLOCK8 orders: block size (0 = choose automatically) */
    int32_t use_graphs;     /* capture the iteration in a CUDA graph (1) or launch eagerly (0) */
    int32_t verbose;        /* print progress to stderr */
    int32_t method;         /* h3d_method, default CGMN */
} h3d_solve_opts;

typedef struct h3d_solve_info {
    int32_t iters;          /* CGMN iterations (max over right-hand sides; summed over refinement steps) */
    int32_t outer;          /* refinement steps (MIXED) or true-residual restarts */
    int32_t converged;      /* 1 if every right-hand side met the stopping rule */
    int32_t nrhs;
    double rel_res_true;    /* max over RHS of ||b - H u|| / ||b|| (FP64), or -1 if not computed */
    double rel_res_prec;    /* max over RHS of the last preconditioned residual ratio */
    double seconds;         /* wall time of the call (host clock, after stream sync) */
    double sweep_seconds;   /* sum of the sampled double-sweep device times (CUDA events) */
    int32_t sweep_samples;  /* number of double sweeps timed (one per replayed iteration block) */
    int32_t sweep_variant;  /* kernel configuration the tuner chose: COLOUR27 tile shape 0-3 or
                               4 = stored row coefficients; BLOCK / BLOCK8 configuration */
    int64_t kernel_launches;/* device kernels this call executed (graph replays included) */
    double sweep_bytes;     /* algorithmic bytes of the timed double sweeps (sweep_seconds):
                               per sweep, x read and written once per active right-hand side
                               and the wavenumber read once per problem with an active one */
} h3d_solve_info;

/* One problem of a batched solve: its own grid, wavenumber and right-hand sides. */
typedef struct h3d_problem {
    h3d_grid grid;
    const double *wn_re;    /* device, N values */
    const double *wn_im;    /* device or NULL */
    const void *b;          /* device, complex128 interleaved, N x nrhs */
    void *u;                /* device, complex128 interleaved, N x nrhs (output) */
    int32_t nrhs;
    int32_t mode;           /* h3d_mode */
} h3d_problem;

/* ---- library ----------------------------------------------------------------------- */
int h3d_version(void);
const char *h3d_status_id(int status);      /* reference-style error identifier */
const char *h3d_last_error(void);           /* message of the last failing call on this thread */
void h3d_default_opts(h3d_solve_opts *opts);

/* ---- operator application ------------------------------------------------------------ */
/* y = H x (mode FORWARD), H^H x (ADJOINT); deriv != 0 applies dH (the mass term only,
 * Helm3d_27pt.h:202-206) with wn holding dwn.  wn_re/wn_im are double for H3D_C128 and
 * float for H3D_C64; wn_im may be NULL.  x and y: N x nrhs, must not overlap. */
int h3d_mvp(const h3d_grid *g, const void *wn_re, const void *wn_im, const void *x, void *y,
            int nrhs, int mode, int deriv, int dtype, void *stream);

/* One forward + backward Kaczmarz sweep with relaxation w on x (in place), right-hand
 * side b (NULL = 0).  Same element types as h3d_mvp.  block: BLOCK / BLOCK8 block size
 * (NULL or 0 = default).  COLOUR27 and BLOCK8 with 12x12x12 blocks run on stored row
 * coefficients (about 27 N complex values of temporary device memory) whenever they fit;
 * block[0] == -1 selects the kernels that form the coefficients themselves (COLOUR27: the
 * shared-memory tile kernel; BLOCK8: 12x12x12 blocks).  BLOCK8 on stored coefficients reads
 * the kernel's status word back (H3D_ERR_TIMEOUT if a bounded wait expired), so that call
 * synchronises the stream; it runs the largest right-hand-side group the columns fill, or the
 * configuration whose index the environment variable H3D_BLOCK8_CONFIG holds. */
int h3d_kacz_sweep(const h3d_grid *g, const void *wn_re, const void *wn_im, double w, void *x,
                   const void *b, int nrhs, int mode, int order, const int32_t *block, int dtype,
                   void *stream);

/* r = b - H x (FP64 residual for iterative refinement), and per-RHS ||r||^2, ||b||^2
 * written to device arrays rr2/bb2 (nrhs doubles each; either may be NULL). */
int h3d_residual(const h3d_grid *g, const double *wn_re, const double *wn_im, const void *b,
                 const void *x, void *r, double *rr2, double *bb2, int nrhs, int mode,
                 void *stream);

/* Same result as h3d_residual, for callers that cannot allocate device memory: code whose
 * device memory is owned by its own allocator or fixed budget (a library-side allocation
 * would fail there or break the caller's accounting).  No counterpart in the reference.
 * All scratch (the PML tables and the per-block partial sums) lives in one fixed device
 * array of H3D_NOALLOC_SCRATCH_BYTES that every GPU loading the library holds until the
 * process exits; grids and nrhs needing more are rejected with H3D_ERR_BAD_ARG, before any
 * launch.  The scratch holds one partial sum per 32x8-column block, z chunk and right-hand
 * side, and the z split follows the current device's occupancy, so the largest problem
 * accepted depends on the device.  The
 * first call on a device looks up that array's address (once per device, with the device
 * current); make the first call before any stream capture.  Every call reuses the same
 * array, so calls that overlap on the GPU (other streams, other threads) race: serialise
 * them.  Each call rewrites all the scratch it reads, so no state carries over. */
#define H3D_NOALLOC_SCRATCH_BYTES (4u << 20)
int h3d_residual_noalloc(const h3d_grid *g, const double *wn_re, const double *wn_im,
                         const void *b, const void *x, void *r, double *rr2, double *bb2,
                         int nrhs, int mode, void *stream);

/* ---- diagnostics ------------------------------------------------------------------------ */
/* Checks the bounded waits of the BLOCK8 sweep kernel on this GPU (no counterpart in the
 * reference).  Runs one double sweep on an internal 24^3 problem in which the kernel's first
 * colour step announces a coefficient copy on its mbarrier but never issues it, with every
 * wait limited to limit_ms (0 < limit_ms <= 1000): each CTA gives up after the limit, records
 * the expired wait in the sweep's status word and returns.  Returns H3D_ERR_TIMEOUT when that
 * status came back (the expected result; the context stays usable), H3D_OK if no wait
 * expired, or another status if the call itself failed.  Synchronous. */
int h3d_check_wait_timeout(double limit_ms);

/* ---- MATLAB-layout host entry points (what the drop-in MEX gateway calls) ----------- */
/* Arguments exactly as the reference gateways receive them: wn (N, re/im planes; im may
 * be NULL), h[3], n[3] and npml[6] as doubles, x split into re/im planes (im may be
 * NULL), nrhs columns.  Outputs are split planes of N*nrhs doubles.  Synchronous. */
int h3d_mex_mvp(const double *wn_re, const double *wn_im, const double *h, const double *n,
                size_t n_len, const double *npml, const double *x_re, const double *x_im,
                size_t x_rows, double *y_re, double *y_im, int mode, int deriv);
int h3d_mex_kacz_sweep(const double *wn_re, const double *wn_im, const double *h,
                       const double *n, size_t n_len, const double *npml, double w,
                       const double *x_re, const double *x_im, size_t x_rows, size_t nrhs,
                       const double *b_re, const double *b_im, size_t b_rows, double *y_re,
                       double *y_im, int mode, int order);

/* ---- solvers -------------------------------------------------------------------------- */
/* u = H \ b (mode FORWARD) or H^H \ b (ADJOINT), complex128 interleaved device vectors,
 * N x nrhs.  Right-hand sides with ||b|| < 1e-12 return u = 0 (opAbstractMatrix.m:118).
 * iters_per_rhs (device or NULL, nrhs ints) receives each column's iteration count;
 * res_hist (host or NULL) receives up to res_hist_len preconditioned residual ratios
 * (max over columns) sampled every check_every iterations. */
int h3d_solve(const h3d_grid *g, const double *wn_re, const double *wn_im, const void *b,
              void *u, int nrhs, int mode, const h3d_solve_opts *opts, h3d_solve_info *info,
              double *res_hist, int res_hist_len, void *stream);

/* Solve every problem of the table; infos (host, nprob entries) may be NULL (a batched solve
 * reports its sweep timing, sweep bytes and kernel launches in the first entry and zero in the
 * others).  With the BLOCK8
 * order (12^3 blocks) and room for every problem's stored coefficients in device memory, all
 * problems run as one batched solve: their columns iterate together (each with its own
 * convergence mask), and every sweep launch covers all problems; problems may differ in grid,
 * PML, wavenumber and mode.  Otherwise the problems are solved one after another.  The wall
 * time in each info is that of the whole call. */
int h3d_solve_batch(const h3d_problem *probs, int nprob, const h3d_solve_opts *opts,
                    h3d_solve_info *infos, void *stream);

/* Same as h3d_solve with host (pinned or pageable) b/u and wavenumber: the
 * host->device copies, the solve and the device->host copy of u all happen
 * inside the call.  Synchronous. */
int h3d_solve_host(const h3d_grid *g, const double *wn_re, const double *wn_im,
                   const void *b_host, void *u_host, int nrhs, int mode,
                   const h3d_solve_opts *opts, h3d_solve_info *info);

/* H \ b (mode FORWARD) or H^H \ b (ADJOINT) with MATLAB's host arrays: what linearsolve.m:148-168
 * with CGMN.m:36-94 computes for a Helmholtz operator, in one call (no per-iteration host round
 * trip), behind the h3d_solve_mex gateway.  wn (N, re/im planes; im may be NULL), h[3], n[3]
 * and npml[6] as doubles, b split planes N x nrhs (im may be NULL), u split planes N x nrhs
 * (output).  opts NULL = h3d_default_opts.  b_rows != nx*ny*nz gives H3D_ERR_BSIZE.
 * H3D_ERR_NOT_CONVERGED still returns the last iterate in u.  Synchronous. */
int h3d_mex_solve(const double *wn_re, const double *wn_im, const double *h, const double *n, size_t n_len,
                  const double *npml, const double *b_re, const double *b_im, size_t b_rows, size_t nrhs,
                  double *u_re, double *u_im, int mode, const h3d_solve_opts *opts, h3d_solve_info *info);

/* ---- FWI pieces ----------------------------------------------------------------------- */
/* PDEfunc OBJ for one frequency and a batch of sources with host buffers (PDEfunc.m:254-394,
 * the gradient of discrete_helmholtz.m:288): U = H \ Ps (a_s) for all sources as one batched
 * solve, D = Pr U, f = 1/2 ||D - Dobs||_F^2 (LS_misfit.m:21-26), V = H^H \ (-Pr^T (D - Dobs)),
 * g = sum_s Re(conj(U_s) .* (dH^H V_s)) cropped to the physical grid.  wn, dwn: N doubles, the
 * wavenumber of this frequency on the computational grid and its derivative with respect to
 * the model parameter (param2wavenum.m:20-49); src_pts (nsrc x 3) and rec_pts (nrec x 3):
 * computational-grid coordinates in grid units, 0-based (as h3d_sinc_weights); src_amp: nsrc
 * complex (re, im) pairs, the source weights w(f) Q_s prod(d)/prod(dt); dobs: nrec x nsrc complex
 * pairs, column s at s*nrec; f: one double; g_phys: the physical grid's doubles (overwritten).
 * opts NULL = h3d_default_opts; info (may be NULL) sums the two solves.  Synchronous. */
int h3d_fwi_grad(const h3d_grid *g, const double *wn, const double *dwn, const double *src_pts, int nsrc,
                 const double *src_amp, const double *rec_pts, int nrec, const double *dobs,
                 const h3d_solve_opts *opts, double *f, double *g_phys, h3d_solve_info *info);

/* g_phys[p] += scale * sum_s Re( conj(u_s[i]) * dH^H z_s [i] ) for the physical points i
 * (the PML is cropped, cut_pml=true: discrete_helmholtz.m:231-232).  dwn is the
 * derivative of the wavenumber (device, N doubles); g_phys has (nx-lo_x-hi_x) *
 * (ny-...) * (nz-...) doubles. */
int h3d_grad_accum(const h3d_grid *g, const double *dwn, const void *u, const void *z,
                   int nrhs, double scale, double *g_phys, void *stream);

/* Separable sinc x Kaiser(r=4, beta=6.31) weights: for point p (coords in grid units
 * of the computational grid, 0-based, nsrc points), w[p][a][0..8] are the weights of
 * grid indices base[p][a] + 0..8 along axis a (weights outside the grid are zero). */
int h3d_sinc_weights(const h3d_grid *g, const double *pts, int npts, int32_t *base,
                     double *w);

/* b_s += scale_s * Ps(point s)   (complex scale per source; pts: host weights from
 * h3d_sinc_weights copied to device). */
int h3d_src_inject(const h3d_grid *g, const int32_t *base, const double *w, const double *scale,
                   void *b, int nsrc, void *stream);

/* d[r + s*nrec] = (Pr u_s)[r]   (receiver sampling, complex128). */
int h3d_rec_sample(const h3d_grid *g, const int32_t *base, const double *w, int nrec,
                   const void *u, int nrhs, void *d, void *stream);

/* b_s = scale * Pr^T d_s   (adjoint source; b is overwritten). */
int h3d_rec_spread(const h3d_grid *g, const int32_t *base, const double *w, int nrec,
                   const void *d, int nrhs, double scale, void *b, void *stream);

/* ---- multigrid grid transfer -------------------------------------------------------- */
/* y = A x along one axis of a complex 3D field: A is n_out x dims_in[axis] in CSR form
 * (rowptr[n_out + 1], col, val in double; device pointers; every col < dims_in[axis]),
 * x has dims_in (x fastest) and y the same dims with dims[axis] = n_out, nrhs fields each
 * (dtype C128 or C64; the sums are formed in double). */
int h3d_axis_apply(const int32_t *rowptr, const int32_t *col, const double *val, int n_out, int axis,
                   const int32_t dims_in[3], const void *x, void *y, int nrhs, int dtype, void *stream);

/* ---- FGMRES with the ML_GMRES multigrid preconditioner -------------------------------- */
/* One level of the hierarchy (construct_multigrid.m:10-60): its computational grid and real
 * wavenumber on the device, in double and (for a complex64 cycle) rounded to float. */
typedef struct h3d_ml_level {
    h3d_grid grid;
    const double *wn;       /* device, N values */
    const float *wn32;      /* device, N values; may be NULL when precision is FP64 */
} h3d_ml_level;

/* A grid transfer between neighbouring levels: scale * (A_z (x) A_y (x) A_x) on fields with
 * x fastest, each A_a an n_out[a] x n_in[a] CSR matrix on the device (h3d_axis_apply's
 * layout).  Restriction maps level i to i+1, prolongation level i+1 to i. */
typedef struct h3d_ml_transfer {
    const int32_t *rowptr[3];
    const int32_t *col[3];
    const double *val[3];
    int32_t n_in[3];
    int32_t n_out[3];
    double scale;
} h3d_ml_transfer;

typedef enum { H3D_ML_PREC_NONE = 0, H3D_ML_PREC_MLGMRES = 1 } h3d_ml_prec;

typedef struct h3d_ml_opts {
    double tol;             /* outer FGMRES relative tolerance (default 1e-6) */
    int32_t maxit;          /* outer restart cycles (default 10000) */
    int32_t maxinnerit;     /* outer steps per cycle (default 5), at most 16 */
    int32_t precond;        /* h3d_ml_prec (default MLGMRES) */
    int32_t precision;      /* h3d_precision: FP64, or MIXED = complex64 V-cycle (default FP64) */
    int32_t k[4];           /* ML_GMRES.m:36-47 opts.k: smoother cycles and steps, coarse
                               solver cycles and steps (default 3, 5, 3, 5; steps <= 16) */
    double smooth_tol;      /* smoother tolerance (ML_GMRES.m:56, default 1e-6) */
    double coarse_tol;      /* coarse solver tolerance (ML_GMRES.m:40, default 0.5) */
} h3d_ml_opts;

typedef struct h3d_ml_info {
    int32_t iters;          /* outer FGMRES steps (quasi-residuals recorded after the leading 1) */
    int32_t converged;      /* quasi-residual or true residual reached tol */
    double rel_res;         /* last outer quasi-residual ratio */
    double seconds;         /* wall time of the call (host clock, after stream sync) */
    int64_t kernel_launches;/* device kernels the call launched */
    int64_t host_syncs;     /* stream synchronisations the control flow needed */
} h3d_ml_info;

void h3d_ml_default_opts(h3d_ml_opts *opts);

/* Units of a velocity model (param2wavenum.m): m/s, s^2/m^2, s^2/km^2. */
typedef enum { H3D_UNIT_M_PER_S = 0, H3D_UNIT_S2_PER_M2 = 1, H3D_UNIT_S2_PER_KM2 = 2 } h3d_unit;

/* x = H \ b (mode FORWARD) or H^H \ b (ADJOINT) by FGMRES (FGMRES.m:33-129) preconditioned by
 * the recursive ML_GMRES V-cycle over `nlevels` levels (ML_GMRES.m:36-72, opMultigrid.m;
 * linearsolve.m:139-141 with discrete_helmholtz.m:349-350), or by nothing (PREC_NONE: plain
 * restarted FGMRES = GMRES(m) on level 0).  restrict_ops / prolong_ops: nlevels - 1 transfers
 * each.  b, x: device, complex128, level-0 size; x is the initial guess (all zeros = none) and
 * is overwritten.  hst (optional, hst_cap doubles): the quasi-residual history, leading 1
 * included; the call fails with H3D_ERR_BAD_ARG if it would overflow.  The control flow runs
 * on the host; the Arnoldi steps, Givens rotations and stopping tests on the device, so that
 * the host waits only before a step that applies the preconditioner and at the end of an
 * unpreconditioned cycle.  A non-finite residual (NaN or Inf in the data) returns
 * H3D_ERR_NONFINITE after the loop stops.  Synchronises `stream` before returning. */
int h3d_mlgmres_solve(const h3d_ml_level *levels, int nlevels, const h3d_ml_transfer *restrict_ops,
                      const h3d_ml_transfer *prolong_ops, const void *b, void *x, int mode,
                      const h3d_ml_opts *opts, double *hst, int hst_cap, h3d_ml_info *info,
                      void *stream);

/* The same solve from the physical model: the hierarchy of construct_multigrid.m:10-60 built by
 * the library (level i: the model coarsened i times by opLInterp1D's 4-point Lagrange
 * interpolation to ceil(n/2) points per axis, spacing 2^i h, ceil(npml/2^i) PML points with the
 * model edge-replicated into them, param2wavenum; transfers: LinInterp1D between the
 * computational grids, restriction = prolongation^T / 8), then h3d_mlgmres_solve.  v_phys:
 * host, n_phys[0] x n_phys[1] x n_phys[2], x fastest, in `unit` (h3d_unit); every axis of a
 * level that is coarsened needs 4 or more points.  b, x: device, complex128, on the level-0
 * PML grid (n_phys + 2 npml per axis).  Synchronises `stream`. */
int h3d_mlgmres_solve_model(const double *v_phys, const int32_t n_phys[3], const double h[3], int npml,
                            double freq, int unit, int nlevels, const void *b, void *x, int mode,
                            const h3d_ml_opts *opts, double *hst, int hst_cap, h3d_ml_info *info,
                            void *stream);

/* Host entry of the h3d_mlgmres_mex gateway: MATLAB's split-complex host arrays (b, u:
 * b_rows x nrhs, column-major; b_im may be NULL), n_phys as three doubles, npml a
 * non-negative integer.  Each column is an independent FGMRES solve from zero (the
 * hierarchy is built once).  b_rows != prod(n_phys + 2 npml) gives H3D_ERR_BSIZE, a bad n
 * H3D_ERR_NSIZE.  info: iters / rel_res the maximum over columns, converged all of them,
 * seconds / launches / waits summed.  Synchronous. */
int h3d_mex_mlgmres(const double *v_phys, const double *n_phys, size_t n_len, const double *h,
                    double npml, double freq, int unit, int nlevels, const double *b_re,
                    const double *b_im, size_t b_rows, size_t nrhs, double *u_re, double *u_im,
                    int mode, const h3d_ml_opts *opts, h3d_ml_info *info);

/* Host-only pieces of the hierarchy (no device call), exported for callers that build their
 * own levels and for tests: dense nout x nin row-major interpolation weights from the
 * ascending nodes xin to the ascending points xout, kind 0 = linear (LinInterp1D.m via
 * nearestnbr1d.m), 1 = 4-point Lagrange (opLInterp1D.m getLA; nin >= 4; points outside the
 * nodes give zero rows); and the model coarsening (x fastest; every axis of n >= 4 points)
 * as the separable product of the Lagrange weights on linspace(0, 1, n) nodes. */
int h3d_ml_interp_weights(int kind, const double *xin, int nin, const double *xout, int nout, double *A);
int h3d_ml_coarsen_model(const double *v, const int32_t n[3], const int32_t n_sub[3], double *v_sub);
/* The levels h3d_mlgmres_solve_model builds, on the host: grids[i] (n with PML, spacing, PML
 * widths) and the FP64 wavenumbers of levels 0..nlevels-1 one after the other in wn (wn_cap
 * values; too small gives H3D_ERR_BAD_ARG with the size needed in the message). */
int h3d_ml_levels_host(const double *v_phys, const int32_t n_phys[3], const double h[3], int npml, double freq,
                       int unit, int nlevels, h3d_grid *grids, double *wn, size_t wn_cap);

/* ---- band storage (the reference's mat_free = false path) ---------------------------- */
/* A band matrix holds ndiags couplings per row: coef[k + ndiags*i] = A(i, i + offsets[k])
 * (the reference's ndiags x N column-major array; complex interleaved, device memory).
 *
 * h3d_band_coefs: the 27 x N band matrix of the operator the matrix-free entry points
 * apply (mode FORWARD: H as helmholtz_3d.m:35-190 builds it, couplings to points outside
 * the grid zero; mode ADJOINT: the band storage of H^H that opBandStorage.m:127-129 forms
 * as conj(Htransp(H)), band k holding offset -offsets[k] of the forward bands).  wn as for
 * h3d_mvp; offsets_out: 27 host int64.  The bands are those of the matrix-free operator;
 * helmholtz_3d.m builds the same matrix for equal PML widths on the two sides of each axis,
 * and a different one for unequal widths (create_pml.m reads the 2x3 npml rows the other way
 * round and its profile differs from the matrix-free PML functions there). */
int h3d_band_coefs(const h3d_grid *g, const void *wn_re, const void *wn_im, int mode, void *coef,
                   int64_t offsets_out[27], int dtype, void *stream);

/* y = A x for A in band storage with 1 <= ndiags <= 64 and any offsets (host int64);
 * couplings with i + offsets[k] outside [0, n) are skipped (Hmvp_MT_mex.c:66-71).
 * x, y: n x nrhs, must not overlap. */
int h3d_band_mvp(const void *coef, const int64_t *offsets, int ndiags, int64_t n, const void *x,
                 void *y, int nrhs, int dtype, void *stream);

/* One forward + backward Kaczmarz sweep on band storage (sweep_MT_mex.c:55-97) with
 * relaxation w, on x in place, right-hand side b (NULL = 0).  The 27 offsets (host int64)
 * must be the 27-point neighbourhood of grid g (every axis >= 3 points) in any order, and
 * couplings across a face of the grid must be zero (as h3d_band_coefs and helmholtz_3d.m
 * produce them): the rows then run as parallel hyperplanes with the sequential result.
 * row_norms: squared row norms (double for C128, float for C64), or NULL for the sum of
 * |A(i,k)|^2 over all 27 bands (opBandStorage.m:139-144). */
int h3d_band_sweep(const h3d_grid *g, const void *coef, const int64_t *offsets, const void *row_norms,
                   double w, void *x, const void *b, int nrhs, int dtype, void *stream);

/* Host entries of the band gateways: MATLAB's split-complex host arrays (coef ndiags x n
 * column-major, offsets as doubles, x / b / y n x nrhs), synchronous.  Checks as the
 * reference: x_rows != n and rn_rows != n give H3D_ERR_XSIZE (reported with the reference's
 * HMvp_MT_mex:NumElements identifier by the gateway).  The sweep takes the 27 bands of a
 * grid stencil (the grid is read off the offsets) with the row norms given, and returns the
 * swept copy of x in y. */
int h3d_mex_band_mvp(const double *coef_re, const double *coef_im, size_t ndiags, size_t n,
                     const double *offsets, const double *x_re, const double *x_im, size_t x_rows,
                     size_t nrhs, double *y_re, double *y_im);
int h3d_mex_band_sweep(const double *coef_re, const double *coef_im, size_t ndiags, size_t n,
                       const double *offsets, const double *x_re, const double *x_im, size_t x_rows,
                       size_t nrhs, const double *b_re, const double *b_im, size_t b_rows, double w,
                       const double *row_norms, size_t rn_rows, double *y_re, double *y_im);

#ifdef __cplusplus
}
#endif

#endif /* H3D_H */
