/*
 * CPU oracle for the 27-point Helmholtz hot path (TEST INFRASTRUCTURE ONLY).
 *
 * Restates, in plain C99, the arithmetic of the reference's matrix-free stencil
 * code.  Every function names the reference lines it follows.  Reference files:
 *   H27  = tools/algorithms/3DFreqModeling/Helm3d_27pt.h
 *   MVP  = tools/algorithms/3DFreqModeling/Helm3dmvp_mex.c
 *   SWP  = tools/algorithms/3DFreqModeling/Helm3dkaczswp_mex.c
 *
 * Structure differs from the reference on purpose: PML values are tabulated
 * once per axis instead of being recomputed per row, and the 27 coefficients
 * are produced from an offset-class rule rather than 27 hand-written lines.
 * The floating-point operations per coefficient, their association order and
 * the per-row accumulation order (t = 0..26, x fastest) follow the reference,
 * so results agree with the compiled reference to rounding (usually bitwise).
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it.
 */
#include "h3d_oracle.h"

#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef double complex cplx;

/* ---- stencil weights: H27:194-200 ------------------------------------------------- */
static const double W1 = 1.8395262e-5;
static const double W2 = 0.296692333333333;
static const double W3 = 0.027476150000000;
static const double WM1 = 0.49649658;
static const double WM2 = 0.075168750000000;
static const double WM3 = 0.004373916666667;
static const double WM4 = 5.690375e-07;

/* Grid-dependent constants: H27:639-671. */
typedef struct {
    double wn_c, wn_x, wn_y, wn_z;      /* centre: wn coefficient and per-axis PML sums */
    double pml_x, pml_y, pml_z;         /* face terms */
    double xz, xy, yz;                  /* cross terms */
    double w3a2;                        /* corner term */
} consts_t;

static consts_t make_consts(const double h[3])
{
    const double hx2 = h[0] * h[0], hy2 = h[1] * h[1], hz2 = h[2] * h[2];
    const double hxy = hx2 + hy2, hxz = hx2 + hz2, hyz = hy2 + hz2;
    const double hxyz = hx2 + hy2 + hz2;
    const double w3a = W3 * 3 / (4 * hxyz);
    consts_t c;
    c.w3a2 = 2 * w3a;
    c.wn_c = -(W1 + 3 * W2 + 16 * w3a * hxyz / 3 + WM1 - 1);
    c.wn_x = (W1 / hx2 + W2 / hx2 + W2 / hxz + W2 / hxy + 8 * w3a);
    c.wn_y = (W1 / hy2 + W2 / hy2 + W2 / hyz + W2 / hxy + 8 * w3a);
    c.wn_z = (W1 / hz2 + W2 / hz2 + W2 / hxz + W2 / hyz + 8 * w3a);
    c.pml_x = -(W1 / hx2 + W2 / hx2 + W2 / hxz + W2 / hxy + 8 * w3a);
    c.pml_y = -(W1 / hy2 + W2 / hy2 + W2 / hyz + W2 / hxy + 8 * w3a);
    c.pml_z = -(W1 / hz2 + W2 / hz2 + W2 / hxz + W2 / hyz + 8 * w3a);
    c.xz = W2 / (2 * hxz);
    c.xy = W2 / (2 * hxy);
    c.yz = W2 / (2 * hyz);
    return c;
}

/* ---- PML: H27:326-390 (1-based argument x in the reference) ----------------------- */
static double gam_lo(double x, double n, double nlo)
{
    return cos(M_PI * ((x - 1) * n / (2 * (n + 1) * nlo)));
}

static double gam_hi(double x, double n, double nhi)
{
    return cos(M_PI * ((1 - (x - 1) / (n + 1)) * n / (2 * nhi)));
}

/* pml_func_lower (H27:346-367).  The interior test uses the LOW width for both
 * sides (x <= n+2-npml_lo), exactly as the reference does. */
static cplx xi_lower(double x, double n, double nlo, double nhi)
{
    double g, g1;
    if (x <= nlo) {
        g1 = (x == nlo) ? 0 : gam_lo(x + 1, n, nlo);
        g = gam_lo(x, n, nlo);
    } else if (x <= n + 2 - nlo) {
        g = 0;
        g1 = (x == n + 2 - nlo) ? gam_hi(x + 1, n, nhi) : 0;
    } else {
        g = gam_hi(x, n, nhi);
        g1 = gam_hi(x + 1, n, nhi);
    }
    return (2.0 + 0.0 * I) / ((2.0 - g1 * (g1 + g)) + (3.0 * g1 + g) * I);
}

/* pml_func_upper (H27:369-390). */
static cplx xi_upper(double x, double n, double nlo, double nhi)
{
    double g2, g1;
    if (x <= nlo) {
        g1 = (x == nlo) ? 0 : gam_lo(x + 1, n, nlo);
        g2 = (x >= nlo - 1) ? 0 : gam_lo(x + 2, n, nlo);
    } else if (x <= n + 2 - nlo) {
        g2 = (x >= n + 1 - nlo) ? gam_hi(x + 2, n, nhi) : 0;
        g1 = (x == n + 2 - nlo) ? gam_hi(x + 1, n, nhi) : 0;
    } else {
        g2 = gam_hi(x + 2, n, nhi);
        g1 = gam_hi(x + 1, n, nhi);
    }
    return (2.0 + 0.0 * I) / ((2.0 - g1 * (g1 + g2)) + (3.0 * g1 + g2) * I);
}

/* Per-axis tables over 0-based index idx in [-1, n] stored at [idx+1].
 * Row idx uses xi_lower(idx+1), xi_upper(idx+1) (H27:406-408, 425-427, 467-469);
 * the adjoint windows read the neighbours idx-1 / idx+1 (H27:397-402, 437-442). */
typedef struct {
    cplx *lo, *hi, *sum;
} axis_t;

static void axis_make(axis_t *a, int n, int nlo, int nhi)
{
    a->lo = (cplx *)malloc(sizeof(cplx) * (size_t)(n + 2));
    a->hi = (cplx *)malloc(sizeof(cplx) * (size_t)(n + 2));
    a->sum = (cplx *)malloc(sizeof(cplx) * (size_t)(n + 2));
    for (int idx = -1; idx <= n; ++idx) {
        a->lo[idx + 1] = xi_lower(idx + 1, n, nlo, nhi);
        a->hi[idx + 1] = xi_upper(idx + 1, n, nlo, nhi);
        a->sum[idx + 1] = a->lo[idx + 1] + a->hi[idx + 1];
    }
}

static void axis_free(axis_t *a)
{
    free(a->lo);
    free(a->hi);
    free(a->sum);
}

void h3do_pml_axis(int n, int npml_lo, int npml_hi, double *lo_re, double *lo_im,
                   double *hi_re, double *hi_im)
{
    axis_t a;
    axis_make(&a, n, npml_lo, npml_hi);
    for (int t = 0; t < n + 2; ++t) {
        lo_re[t] = creal(a.lo[t]);
        lo_im[t] = cimag(a.lo[t]);
        hi_re[t] = creal(a.hi[t]);
        hi_im[t] = cimag(a.hi[t]);
    }
    axis_free(&a);
}

/* ---- coefficient rule ---------------------------------------------------------------
 * Offsets d = (dx,dy,dz) in {-1,0,1}^3, t = (dx+1) + 3(dy+1) + 9(dz+1) (H27:163-189).
 * The PML part of the FORWARD coefficient of a row (H27:680-714) depends only on
 * the number of non-zero offset components:
 *   0 (centre)  wn_x*Sx + wn_y*Sy + wn_z*Sz
 *   1 (face a)  pml_a*A_a + cross(a,b1)*S_b1 + cross(a,b2)*S_b2
 *   2 (edge ab) -cross(a,b)*(A_a + A_b) + w3a2*S_c          (c = the zero axis)
 *   3 (corner)  -w3a2*(A_x + A_y + A_z)
 * with A_a the directional PML value of axis a (xi_lo for d_a=-1, xi_hi for +1)
 * and S_a = xi_lo + xi_hi.  The ADJOINT coefficient at offset t (H27:718-809) is
 * the conjugate of the forward coefficient of row (c+t) at offset -t, with the
 * wavenumber taken at the centre c; the directional values are therefore
 * xi_hi(c_a-1) for d_a=-1 and xi_lo(c_a+1) for d_a=+1.
 */
static cplx pml_term(const consts_t *c, int dx, int dy, int dz, const cplx A[3], const cplx S[3])
{
    const int nzc = (dx != 0) + (dy != 0) + (dz != 0);
    if (nzc == 0) return c->wn_x * S[0] + c->wn_y * S[1] + c->wn_z * S[2];
    if (nzc == 3) return -c->w3a2 * (A[0] + A[1] + A[2]);
    if (nzc == 1) {
        if (dx) return c->pml_x * A[0] + c->xz * S[2] + c->xy * S[1];
        if (dy) return c->pml_y * A[1] + c->yz * S[2] + c->xy * S[0];
        return c->pml_z * A[2] + c->yz * S[1] + c->xz * S[0];
    }
    if (!dz) return -c->xy * (A[0] + A[1]) + c->w3a2 * S[2];
    if (!dy) return -c->xz * (A[2] + A[0]) + c->w3a2 * S[1];
    return -c->yz * (A[2] + A[1]) + c->w3a2 * S[0];
}

static double wm_of(int dx, int dy, int dz)
{
    switch ((dx != 0) + (dy != 0) + (dz != 0)) {
    case 1: return WM2;
    case 2: return WM3;
    case 3: return WM4;
    default: return 0.0;
    }
}

typedef struct {
    h3do_grid g;
    consts_t c;
    axis_t ax[3];
    size_t N;
} op_t;

static void op_make(op_t *op, const h3do_grid *g)
{
    op->g = *g;
    op->c = make_consts(g->h);
    for (int a = 0; a < 3; ++a) axis_make(&op->ax[a], g->n[a], g->npml[2 * a], g->npml[2 * a + 1]);
    op->N = (size_t)g->n[0] * g->n[1] * g->n[2];
}

static void op_free(op_t *op)
{
    for (int a = 0; a < 3; ++a) axis_free(&op->ax[a]);
}

static inline cplx wn_at(const double *wnr, const double *wni, size_t idx)
{
    return wni ? wnr[idx] + wni[idx] * I : wnr[idx] + 0.0 * I;
}

/* The 27 coefficients of row (i,j,k): H27:676-825.  Forward coefficients are
 * zeroed where the neighbour is outside the grid (the *_BDRY masks,
 * H27:263-289); adjoint coefficients are not masked (only x is). */
static void coefs(const op_t *op, const double *wnr, const double *wni, int i, int j, int k,
                  int adj, int deriv, cplx coef[27])
{
    const int nx = op->g.n[0], ny = op->g.n[1], nz = op->g.n[2];
    const int pos[3] = {i, j, k};
    const int nn[3] = {nx, ny, nz};
    const size_t sx = 1, sy = (size_t)nx, sz = (size_t)nx * ny;
    const size_t ctr = (size_t)i + sy * j + sz * k;
    cplx S[3];
    for (int a = 0; a < 3; ++a) S[a] = op->ax[a].sum[pos[a] + 1];
    const cplx wc = wn_at(wnr, wni, ctr);
    for (int dz = -1; dz <= 1; ++dz)
        for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) {
                const int t = (dx + 1) + 3 * (dy + 1) + 9 * (dz + 1);
                const int d[3] = {dx, dy, dz};
                int inside = 1;
                for (int a = 0; a < 3; ++a)
                    if (pos[a] + d[a] < 0 || pos[a] + d[a] >= nn[a]) inside = 0;
                const int centre = (t == 13);
                cplx A[3];
                if (!adj) {
                    for (int a = 0; a < 3; ++a)
                        A[a] = d[a] < 0 ? op->ax[a].lo[pos[a] + 1] : op->ax[a].hi[pos[a] + 1];
                    if (!inside) {
                        coef[t] = 0;
                        continue;
                    }
                    cplx wv = wn_at(wnr, wni, ctr + sx * dx + sy * dy + sz * dz);
                    cplx wt = centre ? op->c.wn_c * wv : -wm_of(dx, dy, dz) * wv;
                    if (deriv)
                        coef[t] = wt;
                    else
                        coef[t] = wt + 1.0 * pml_term(&op->c, dx, dy, dz, A, S);
                } else {
                    /* neighbour's xi seen from the centre: xi_hi(c-1) for d=-1, xi_lo(c+1) for d=+1 */
                    for (int a = 0; a < 3; ++a)
                        A[a] = d[a] < 0 ? op->ax[a].hi[pos[a] - 1 + 1] : op->ax[a].lo[pos[a] + 1 + 1];
                    cplx v = centre ? op->c.wn_c * wc : -wm_of(dx, dy, dz) * wc;
                    if (!deriv) v += pml_term(&op->c, -dx, -dy, -dz, A, S);
                    coef[t] = conj(v);
                }
            }
}

void h3do_row_coefs(const h3do_grid *g, const double *wnr, const double *wni, int i, int j,
                    int k, int adj, int deriv, double *cre, double *cim)
{
    op_t op;
    op_make(&op, g);
    cplx c[27];
    coefs(&op, wnr, wni, i, j, k, adj, deriv, c);
    for (int t = 0; t < 27; ++t) {
        cre[t] = creal(c[t]);
        cim[t] = cimag(c[t]);
    }
    op_free(&op);
}

/* Gather the 27-point x neighbourhood with zeros outside the grid: H27:483-520. */
static void gather(const op_t *op, const double *xr, const double *xi, int i, int j, int k,
                   cplx xv[27])
{
    const int nx = op->g.n[0], ny = op->g.n[1], nz = op->g.n[2];
    for (int dz = -1; dz <= 1; ++dz)
        for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) {
                const int t = (dx + 1) + 3 * (dy + 1) + 9 * (dz + 1);
                const int ii = i + dx, jj = j + dy, kk = k + dz;
                if (ii < 0 || ii >= nx || jj < 0 || jj >= ny || kk < 0 || kk >= nz) {
                    xv[t] = 0;
                } else {
                    size_t q = (size_t)ii + (size_t)nx * jj + (size_t)nx * ny * kk;
                    xv[t] = xr[q] + (xi ? xi[q] : 0.0) * I;
                }
            }
}

/* ---- matvec: do_Hmvp, H27:827-875 ------------------------------------------------ */
int h3do_mvp(const h3do_grid *g, const double *wnr, const double *wni, const double *xr,
             const double *xi, double *yr, double *yi, int nrhs, int adj, int deriv,
             int nthreads)
{
    if (!g || g->n[0] < 1 || g->n[1] < 1 || g->n[2] < 1 || nrhs < 1) return 1;
    op_t op;
    op_make(&op, g);
    const int nx = g->n[0], ny = g->n[1], nz = g->n[2];
    const size_t N = op.N;
    if (nthreads < 1) nthreads = 1;
    for (int s = 0; s < nrhs; ++s) {
        const double *xrs = xr + s * N, *xis = xi ? xi + s * N : NULL;
        double *yrs = yr + s * N, *yis = yi + s * N;
#pragma omp parallel for schedule(static) num_threads(nthreads)
        for (int k = 0; k < nz; ++k) {
            cplx c[27], xv[27];
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i) {
                    coefs(&op, wnr, wni, i, j, k, adj, deriv, c);
                    gather(&op, xrs, xis, i, j, k, xv);
                    cplx acc = 0.0 + 0.0 * I;
                    for (int t = 0; t < 27; ++t) acc += c[t] * xv[t];
                    size_t q = (size_t)i + (size_t)nx * j + (size_t)nx * ny * k;
                    yrs[q] = creal(acc);
                    yis[q] = cimag(acc);
                }
        }
    }
    op_free(&op);
    return 0;
}

/* ---- Kaczmarz row projection: the body of do_sweep, SWP:93-118 ------------------- */
static void project_row(const op_t *op, const double *wnr, const double *wni, double w,
                        double *xr, double *xi, const double *br, const double *bi, int i,
                        int j, int k, int adj)
{
    const int nx = op->g.n[0], ny = op->g.n[1], nz = op->g.n[2];
    cplx c[27], xv[27];
    coefs(op, wnr, wni, i, j, k, adj, 0, c);
    gather(op, xr, xi, i, j, k, xv);
    cplx atx = 0.0 + 0.0 * I;
    double nrm = 0;
    for (int t = 0; t < 27; ++t) {
        atx += c[t] * xv[t];
        nrm += creal(conj(c[t]) * c[t]);
    }
    const size_t q0 = (size_t)i + (size_t)nx * j + (size_t)nx * ny * k;
    cplx b = br ? br[q0] + (bi ? bi[q0] : 0.0) * I : 0.0 + 0.0 * I;
    cplx d = w * (b - atx) / nrm;
    for (int dz = -1; dz <= 1; ++dz)
        for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) {
                const int t = (dx + 1) + 3 * (dy + 1) + 9 * (dz + 1);
                const int ii = i + dx, jj = j + dy, kk = k + dz;
                if (ii < 0 || ii >= nx || jj < 0 || jj >= ny || kk < 0 || kk >= nz) continue;
                cplx u = d * conj(c[t]);
                size_t q = (size_t)ii + (size_t)nx * jj + (size_t)nx * ny * kk;
                xr[q] += creal(u);
                xi[q] += cimag(u);
            }
}

/* Rows of one colour q = (i%3) + 3(j%3) + 9(k%3) are pairwise independent
 * (their 3x3x3 footprints are disjoint), so any order within a colour gives
 * the same result; the oracle walks them lexicographically. */
static void colour_pass(const op_t *op, const double *wnr, const double *wni, double w,
                        double *xr, double *xi, const double *br, const double *bi, int adj,
                        int q, const int lo[3], const int hi[3], int par)
{
    const int a = q % 3, b = (q / 3) % 3, cz = q / 9;
    int k0 = lo[2] + ((cz - lo[2] % 3) + 3) % 3;
    int j0 = lo[1] + ((b - lo[1] % 3) + 3) % 3;
    int i0 = lo[0] + ((a - lo[0] % 3) + 3) % 3;
    if (par) {
#pragma omp parallel for schedule(static)
        for (int k = k0; k < hi[2]; k += 3)
            for (int j = j0; j < hi[1]; j += 3)
                for (int i = i0; i < hi[0]; i += 3)
                    project_row(op, wnr, wni, w, xr, xi, br, bi, i, j, k, adj);
    } else {
        for (int k = k0; k < hi[2]; k += 3)
            for (int j = j0; j < hi[1]; j += 3)
                for (int i = i0; i < hi[0]; i += 3)
                    project_row(op, wnr, wni, w, xr, xi, br, bi, i, j, k, adj);
    }
}

static void sweep_one(const op_t *op, const double *wnr, const double *wni, double w, double *xr,
                      double *xi, const double *br, const double *bi, int adj, int order,
                      const int *blk, int par)
{
    const int nx = op->g.n[0], ny = op->g.n[1], nz = op->g.n[2];
    if (order == H3DO_ORDER_LEX) {
        /* xyzloop_updown, H27:63-106 */
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i)
                    project_row(op, wnr, wni, w, xr, xi, br, bi, i, j, k, adj);
        for (int k = nz - 1; k >= 0; --k)
            for (int j = ny - 1; j >= 0; --j)
                for (int i = nx - 1; i >= 0; --i)
                    project_row(op, wnr, wni, w, xr, xi, br, bi, i, j, k, adj);
        return;
    }
    if (order == H3DO_ORDER_COLOUR27) {
        const int lo[3] = {0, 0, 0}, hi[3] = {nx, ny, nz};
        for (int q = 0; q < 27; ++q) colour_pass(op, wnr, wni, w, xr, xi, br, bi, adj, q, lo, hi, par);
        for (int q = 26; q >= 0; --q) colour_pass(op, wnr, wni, w, xr, xi, br, bi, adj, q, lo, hi, par);
        return;
    }
    const int bx = blk[0], by = blk[1], bz = blk[2];
    const int NI = (nx + bx - 1) / bx, NJ = (ny + by - 1) / by, NK = (nz + bz - 1) / bz;
    if (order == H3DO_ORDER_BLOCK8) {
        /* Blocks coloured by parity p = I%2 + 2(J%2) + 4(K%2), p ascending; two blocks
         * of one parity are a whole block apart in some axis (blk >= 2), so their rows
         * share no column and the order among them is immaterial.  27 colours inside a
         * block.  The second pass reverses both levels. */
        for (int pass = 0; pass < 2; ++pass)
            for (int pp = 0; pp < 8; ++pp) {
                const int p = pass == 0 ? pp : 7 - pp;
                for (int bk = p >> 2; bk < NK; bk += 2)
                    for (int bj = (p >> 1) & 1; bj < NJ; bj += 2)
                        for (int bi_ = p & 1; bi_ < NI; bi_ += 2) {
                            const int lo[3] = {bi_ * bx, bj * by, bk * bz};
                            const int hi[3] = {lo[0] + bx < nx ? lo[0] + bx : nx,
                                               lo[1] + by < ny ? lo[1] + by : ny,
                                               lo[2] + bz < nz ? lo[2] + bz : nz};
                            for (int qq = 0; qq < 27; ++qq) {
                                const int q = pass == 0 ? qq : 26 - qq;
                                colour_pass(op, wnr, wni, w, xr, xi, br, bi, adj, q, lo, hi, 0);
                            }
                        }
            }
        return;
    }
    /* Block wavefront: blocks (I,J,K) of size blk, visited by T = I + 2J + 4K.
     * Adjacent blocks always differ in T and blocks sharing a T are never
     * adjacent, so the order among same-T blocks is immaterial. */
    const int Tmax = (NI - 1) + 2 * (NJ - 1) + 4 * (NK - 1);
    for (int pass = 0; pass < 2; ++pass) {
        for (int tt = 0; tt <= Tmax; ++tt) {
            const int T = pass == 0 ? tt : Tmax - tt;
            for (int bk = 0; bk < NK; ++bk)
                for (int bj = 0; bj < NJ; ++bj) {
                    const int bi_ = T - 2 * bj - 4 * bk;
                    if (bi_ < 0 || bi_ >= NI) continue;
                    const int lo[3] = {bi_ * bx, bj * by, bk * bz};
                    const int hi[3] = {lo[0] + bx < nx ? lo[0] + bx : nx,
                                       lo[1] + by < ny ? lo[1] + by : ny,
                                       lo[2] + bz < nz ? lo[2] + bz : nz};
                    for (int qq = 0; qq < 27; ++qq) {
                        const int q = pass == 0 ? qq : 26 - qq;
                        colour_pass(op, wnr, wni, w, xr, xi, br, bi, adj, q, lo, hi, 0);
                    }
                }
        }
    }
}

/* ---- do_sweep: SWP:60-120 (OpenMP across right-hand sides, as SWP:90) ----------- */
int h3do_sweep(const h3do_grid *g, const double *wnr, const double *wni, double w, double *xr,
               double *xi, const double *br, const double *bi, int nrhs, int adj, int order,
               const int *blk, int nthreads)
{
    if (!g || nrhs < 1) return 1;
    if ((order == H3DO_ORDER_BLOCK || order == H3DO_ORDER_BLOCK8) && (!blk || blk[0] < 2 || blk[1] < 2 || blk[2] < 2)) return 2;
    op_t op;
    op_make(&op, g);
    const size_t N = op.N;
    if (nthreads < 1) nthreads = 1;
    const int par_rows = (nrhs == 1 && order == H3DO_ORDER_COLOUR27 && nthreads > 1);
#ifdef _OPENMP
    if (par_rows) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel for schedule(static) num_threads(nthreads) if (!par_rows && nrhs > 1)
    for (int s = 0; s < nrhs; ++s)
        sweep_one(&op, wnr, wni, w, xr + s * N, xi + s * N, br ? br + s * N : NULL,
                  br && bi ? bi + s * N : NULL, adj, order, blk, par_rows);
    op_free(&op);
    return 0;
}
