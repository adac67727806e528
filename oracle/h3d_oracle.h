/*
 * CPU oracle for the 27-point Helmholtz hot path (TEST INFRASTRUCTURE ONLY).
 *
 * A plain-C restatement of the reference's stencil kernels
 * (tools/algorithms/3DFreqModeling/Helm3d_27pt.h, Helm3dmvp_mex.c,
 * Helm3dkaczswp_mex.c).  It is the checker for the CUDA library and the CPU
 * baseline ("port") timed beside it.  Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg may load it; the product never does.
 *
 * Layout everywhere (as in the reference): column-major grid, x fastest,
 * idx = i + j*nx + k*nx*ny, separate real and imaginary planes, right-hand
 * side s at offset s*N.
 */
#ifndef H3D_ORACLE_H
#define H3D_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int n[3];      /* nx, ny, nz including PML */
    double h[3];   /* hx, hy, hz */
    int npml[6];   /* lo_x, hi_x, lo_y, hi_y, lo_z, hi_z (column-major 2x3 of the reference) */
} h3do_grid;

/* Sweep row orderings. */
enum {
    H3DO_ORDER_LEX = 0,      /* reference order: k, j, i ascending then descending */
    H3DO_ORDER_COLOUR27 = 1, /* 27 colours q = i%3 + 3(j%3) + 9(k%3), q ascending then descending */
    H3DO_ORDER_BLOCK = 2,    /* block-lexicographic wavefront, 27 colours inside each block */
    H3DO_ORDER_BLOCK8 = 3    /* blocks in 8 parity classes, 27 colours inside each block */
};

/* PML functions xi_lo / xi_hi of one axis at 0-based index idx in [-1, n]. */
void h3do_pml_axis(int n, int npml_lo, int npml_hi, double *lo_re, double *lo_im,
                   double *hi_re, double *hi_im);

/* The 27 coefficients of row (i,j,k) (0-based); adj/deriv select the variant. */
void h3do_row_coefs(const h3do_grid *g, const double *wnr, const double *wni, int i, int j,
                    int k, int adj, int deriv, double *cre, double *cim);

/* y = H x, H^H x, dH x or dH^H x for nrhs columns.  wni may be NULL (real wn).
 * xi may be NULL (real x).  Returns 0 on success. */
int h3do_mvp(const h3do_grid *g, const double *wnr, const double *wni, const double *xr,
             const double *xi, double *yr, double *yi, int nrhs, int adj, int deriv,
             int nthreads);

/* One forward + backward Kaczmarz sweep, in place on (xr, xi), nrhs columns.
 * br/bi may be NULL (b = 0).  blk = block dims for H3DO_ORDER_BLOCK and H3DO_ORDER_BLOCK8. */
int h3do_sweep(const h3do_grid *g, const double *wnr, const double *wni, double w, double *xr,
               double *xi, const double *br, const double *bi, int nrhs, int adj, int order,
               const int *blk, int nthreads);

#ifdef __cplusplus
}
#endif
#endif
