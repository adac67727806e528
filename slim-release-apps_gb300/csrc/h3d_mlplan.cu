// The multigrid hierarchy built from the physical model (construct_multigrid.m:10-60 with a
// coarsening factor of 2) and the one-call solve on it:
//
//   level i+1     the physical model of level i interpolated to ceil(n / 2) points per axis by
//                 4-point Lagrange interpolation (opLInterp1D.m getLA) between linspace(0, 1, n)
//                 nodes; spacing 2^(i+1) h; ceil(npml / 2^(i+1)) PML points, the model
//                 edge-replicated into them; the wavenumber param2wavenum.m forms from it
//   transfers     prolongation P = linear interpolation between the computational grids
//                 (LinInterp1D.m on linspace(0, 1, n) nodes, PML included), restriction
//                 R = P^T / 8, each a Kronecker product of three axis operators
//
// Host code only (set-up work, O(N) per level); h3d_mlgmres_solve_model uploads the levels
// and transfers and runs h3d_mlgmres_solve.  Fields are x fastest, as everywhere in the
// library.
#include <algorithm>
#include <array>
#include <cmath>
#include <utility>
#include <vector>

#include "h3d_internal.cuh"
#include "h3d_vec.cuh"

using namespace h3d;

namespace {

std::vector<double> linspace01(int m)
{
    std::vector<double> y((size_t)m);
    if (m == 1) {
        y[0] = 0.0;
        return y;
    }
    const double step = 1.0 / (double)(m - 1);
    for (int i = 0; i < m; ++i) y[(size_t)i] = (double)i * step;
    y[(size_t)m - 1] = 1.0;
    return y;
}

// LinInterp1D.m via nearestnbr1d.m: dense nout x nin (row-major) linear interpolation from the
// ascending nodes xin to the ascending points xout.
void linear_weights(const std::vector<double> &xin, const std::vector<double> &xout, std::vector<double> &A)
{
    const int nin = (int)xin.size(), nout = (int)xout.size();
    A.assign((size_t)nout * nin, 0.0);
    for (int o = 0; o < nout; ++o) {
        const double X = xout[(size_t)o];
        // nearest node, ties to the lower one
        const int idx = (int)(std::lower_bound(xin.begin(), xin.end(), X) - xin.begin());
        const int lo = std::min(std::max(idx - 1, 0), nin - 1), hi = std::min(std::max(idx, 0), nin - 1);
        int I = std::fabs(X - xin[(size_t)lo]) <= std::fabs(X - xin[(size_t)hi]) ? lo : hi;
        if (xin[(size_t)I] > X) I -= 1;
        if (I < 0) I = 0;
        const double nxt = I + 1 < nin ? xin[(size_t)std::min(I + 1, nin - 1)] : 1e12;
        const double wb = (X - xin[(size_t)I]) / (nxt - xin[(size_t)I]);
        const double wa = (nxt - X) / (nxt - xin[(size_t)I]);
        A[(size_t)o * nin + I] += wa;
        A[(size_t)o * nin + std::min(I + 1, nin - 1)] += wb;
    }
}

// opLInterp1D.m getLA: dense n2 x n1 (row-major) 4-point Lagrange interpolation from the nodes
// x1 (n1 >= 4) to the points x2; rows of points outside [x1[0], x1[n1-1]] are zero.  The node
// window slides monotonically with the points.
void cubic_weights(const std::vector<double> &x1, const std::vector<double> &x2, std::vector<double> &A)
{
    const int n1 = (int)x1.size(), n2 = (int)x2.size();
    A.assign((size_t)n2 * n1, 0.0);
    int b = 1, c = 2;
    for (int k = 0; k < n2; ++k) {
        const double X = x2[(size_t)k];
        if (!(X >= x1[0] && X <= x1[(size_t)n1 - 1])) continue;
        if (X < x1[(size_t)b]) {
            while (X < x1[(size_t)b] && b > 1) --b;
            c = b + 1;
        } else if (X > x1[(size_t)c]) {
            while (X > x1[(size_t)c] && c < n1 - 2) ++c;
            b = c - 1;
        }
        const int nodes[4] = {b - 1, b, c, c + 1};
        for (int pi = 0; pi < 4; ++pi) {
            const int p = nodes[pi];
            double num = 1.0, den = 1.0;
            for (int qi = 0; qi < 4; ++qi) {
                if (qi == pi) continue;
                num *= X - x1[(size_t)nodes[qi]];
                den *= x1[(size_t)p] - x1[(size_t)nodes[qi]];
            }
            A[(size_t)k * n1 + p] += num / den;
        }
    }
}

// out(a,b,c) = sum_ijk Ax(a,i) Ay(b,j) Az(c,k) v(i,j,k), one axis at a time (x, then y, then z),
// each sum over the nonzero weights of its row in increasing index order.  v and out x fastest.
void coarsen(const std::vector<double> &v, const int32_t n[3], const int32_t ns[3], std::vector<double> &out)
{
    // nonzeros of each output row of the three axis operators
    std::vector<std::vector<std::pair<long long, double>>> rows[3];
    for (int a = 0; a < 3; ++a) {
        std::vector<double> A;
        cubic_weights(linspace01(n[a]), linspace01(ns[a]), A);
        rows[a].resize((size_t)ns[a]);
        for (int o = 0; o < ns[a]; ++o)
            for (int i = 0; i < n[a]; ++i) {
                const double w = A[(size_t)o * n[a] + i];
                if (w != 0.0) rows[a][(size_t)o].push_back({i, w});
            }
    }
    const long long nx = n[0], ny = n[1], nz = n[2], mx = ns[0], my = ns[1], mz = ns[2];
    std::vector<double> t1((size_t)(mx * ny * nz), 0.0), t2((size_t)(mx * my * nz), 0.0);
    for (long long k = 0; k < nz; ++k)
        for (long long j = 0; j < ny; ++j)
            for (long long a = 0; a < mx; ++a) {
                double s = 0.0;
                for (const auto &q : rows[0][(size_t)a]) s += q.second * v[(size_t)(q.first + nx * (j + ny * k))];
                t1[(size_t)(a + mx * (j + ny * k))] = s;
            }
    for (long long k = 0; k < nz; ++k)
        for (long long b = 0; b < my; ++b)
            for (long long a = 0; a < mx; ++a) {
                double s = 0.0;
                for (const auto &q : rows[1][(size_t)b]) s += q.second * t1[(size_t)(a + mx * (q.first + ny * k))];
                t2[(size_t)(a + mx * (b + my * k))] = s;
            }
    out.assign((size_t)(mx * my * mz), 0.0);
    for (long long c = 0; c < mz; ++c)
        for (long long b = 0; b < my; ++b)
            for (long long a = 0; a < mx; ++a) {
                double s = 0.0;
                for (const auto &q : rows[2][(size_t)c]) s += q.second * t2[(size_t)(a + mx * (b + my * q.first))];
                out[(size_t)(a + mx * (b + my * c))] = s;
            }
}

// param2wavenum.m on the model edge-replicated into npml points on every face.
int wavenumber(const std::vector<double> &v, const int32_t n[3], int npml, double freq, int unit,
               std::vector<double> &wn, int32_t nt[3])
{
    for (int a = 0; a < 3; ++a) nt[a] = n[a] + 2 * npml;
    const double kPi = 3.141592653589793;
    const double c = (2.0 * kPi * freq) * (2.0 * kPi * freq);
    const long long NX = nt[0], NY = nt[1], NZ = nt[2];
    wn.assign((size_t)(NX * NY * NZ), 0.0);
    for (long long k = 0; k < NZ; ++k) {
        const long long kk = std::min<long long>(std::max<long long>(k - npml, 0), n[2] - 1);
        for (long long j = 0; j < NY; ++j) {
            const long long jj = std::min<long long>(std::max<long long>(j - npml, 0), n[1] - 1);
            for (long long i = 0; i < NX; ++i) {
                const long long ii = std::min<long long>(std::max<long long>(i - npml, 0), n[0] - 1);
                const double x = v[(size_t)(ii + (long long)n[0] * (jj + (long long)n[1] * kk))];
                double w;
                if (unit == H3D_UNIT_M_PER_S) w = c * std::pow(x, -2.0);
                else if (unit == H3D_UNIT_S2_PER_M2) w = c * x;
                else w = 1e-6 * c * x;
                wn[(size_t)(i + NX * (j + NY * k))] = w;
            }
        }
    }
    return H3D_OK;
}

struct Csr {
    std::vector<int32_t> rowptr, col;
    std::vector<double> val;
};

// CSR of a dense row-major matrix (or of its transpose), exact zeros left out.
Csr to_csr(const std::vector<double> &A, int rows, int cols, bool transpose)
{
    Csr c;
    const int R = transpose ? cols : rows, Cn = transpose ? rows : cols;
    c.rowptr.assign((size_t)R + 1, 0);
    for (int r = 0; r < R; ++r) {
        for (int q = 0; q < Cn; ++q) {
            const double a = transpose ? A[(size_t)q * cols + r] : A[(size_t)r * cols + q];
            if (a != 0.0) {
                c.col.push_back(q);
                c.val.push_back(a);
            }
        }
        c.rowptr[(size_t)r + 1] = (int32_t)c.col.size();
    }
    return c;
}

int check_unit(int unit)
{
    if (unit != H3D_UNIT_M_PER_S && unit != H3D_UNIT_S2_PER_M2 && unit != H3D_UNIT_S2_PER_KM2) {
        set_error("unknown model unit %d", unit);
        return H3D_ERR_BAD_ARG;
    }
    return H3D_OK;
}

// The hierarchy of one model on the device: levels (grid, FP64 and float wavenumbers) and the
// transfers, in one device arena.
struct MlPlan {
    int nlevels = 0;
    std::vector<h3d_ml_level> lv;
    std::vector<h3d_ml_transfer> Rt, Pt;
    DevBuf dev;
};

// Levels on the host: each level's grid (PML included) and FP64 wavenumber.
int ml_levels_host(const double *v_phys, const int32_t n_phys[3], const double h[3], int npml, double freq, int unit,
                   int nlevels, std::vector<h3d_grid> &grids, std::vector<std::vector<double>> &wn)
{
    if (!v_phys || !n_phys || !h || npml < 0 || !(freq > 0.0) || nlevels < 1 || nlevels > 8) {
        set_error("multigrid set-up: bad argument");
        return H3D_ERR_BAD_ARG;
    }
    int rc = check_unit(unit);
    if (rc) return rc;
    // the physical models of all levels
    std::vector<std::vector<double>> vm((size_t)nlevels);
    std::vector<std::array<int32_t, 3>> nm((size_t)nlevels);
    for (int a = 0; a < 3; ++a) {
        if (n_phys[a] < 1) {
            set_error("multigrid set-up: bad model size");
            return H3D_ERR_NSIZE;
        }
        nm[0][a] = n_phys[a];
    }
    const long long N0 = (long long)n_phys[0] * n_phys[1] * n_phys[2];
    vm[0].assign(v_phys, v_phys + N0);
    for (int i = 1; i < nlevels; ++i) {
        int32_t ns[3];
        for (int a = 0; a < 3; ++a) {
            if (nm[(size_t)i - 1][a] < 4) {
                set_error("multigrid set-up: level %d has an axis of fewer than 4 points; use fewer levels", i - 1);
                return H3D_ERR_BAD_ARG;
            }
            ns[a] = (nm[(size_t)i - 1][a] + 1) / 2;
            nm[(size_t)i][a] = ns[a];
        }
        coarsen(vm[(size_t)i - 1], nm[(size_t)i - 1].data(), ns, vm[(size_t)i]);
    }
    // wavenumbers and grids
    wn.assign((size_t)nlevels, std::vector<double>());
    grids.assign((size_t)nlevels, h3d_grid{});
    for (int i = 0; i < nlevels; ++i) {
        const double s = std::ldexp(1.0, i);
        const int p = (int)std::ceil((double)npml / s);
        int32_t nt[3];
        wavenumber(vm[(size_t)i], nm[(size_t)i].data(), p, freq, unit, wn[(size_t)i], nt);
        h3d_grid &g = grids[(size_t)i];
        for (int a = 0; a < 3; ++a) {
            g.n[a] = nt[a];
            g.h[a] = h[a] * s;
        }
        for (int a = 0; a < 6; ++a) g.npml[a] = p;
        if ((rc = check_grid(&g))) return rc;
    }
    return H3D_OK;
}

int ml_plan_build(const double *v_phys, const int32_t n_phys[3], const double h[3], int npml, double freq, int unit,
                  int nlevels, cudaStream_t st, MlPlan &plan)
{
    std::vector<h3d_grid> grids;
    std::vector<std::vector<double>> wn;
    int rc = ml_levels_host(v_phys, n_phys, h, npml, freq, unit, nlevels, grids, wn);
    if (rc) return rc;
    plan.nlevels = nlevels;
    plan.lv.assign((size_t)nlevels, h3d_ml_level{});
    std::vector<h3d_ml_level> &lv = plan.lv;
    for (int i = 0; i < nlevels; ++i) lv[(size_t)i].grid = grids[(size_t)i];
    // transfers between neighbouring computational grids
    std::vector<Csr> Pc((size_t)3 * (nlevels - 1)), Rc((size_t)3 * (nlevels - 1));
    for (int i = 0; i + 1 < nlevels; ++i)
        for (int a = 0; a < 3; ++a) {
            const int nf = lv[(size_t)i].grid.n[a], nc = lv[(size_t)i + 1].grid.n[a];
            std::vector<double> L;
            linear_weights(linspace01(nc), linspace01(nf), L);  // nf x nc: coarse -> fine
            Pc[(size_t)3 * i + a] = to_csr(L, nf, nc, false);
            Rc[(size_t)3 * i + a] = to_csr(L, nf, nc, true);
        }
    // one device arena for the set-up data, filled by one copy
    size_t bytes = 0;
    auto up = [&](size_t nbytes) {
        const size_t off = (bytes + 255) & ~(size_t)255;
        bytes = off + nbytes;
        return off;
    };
    std::vector<size_t> o_wn((size_t)nlevels), o_w32((size_t)nlevels);
    for (int i = 0; i < nlevels; ++i) {
        o_wn[(size_t)i] = up(sizeof(double) * wn[(size_t)i].size());
        o_w32[(size_t)i] = up(sizeof(float) * wn[(size_t)i].size());
    }
    struct Off {
        size_t rp, col, val;
    };
    std::vector<Off> oP(Pc.size()), oR(Rc.size());
    for (size_t q = 0; q < Pc.size(); ++q) {
        oP[q] = {up(sizeof(int32_t) * Pc[q].rowptr.size()), up(sizeof(int32_t) * std::max<size_t>(1, Pc[q].col.size())),
                 up(sizeof(double) * std::max<size_t>(1, Pc[q].val.size()))};
        oR[q] = {up(sizeof(int32_t) * Rc[q].rowptr.size()), up(sizeof(int32_t) * std::max<size_t>(1, Rc[q].col.size())),
                 up(sizeof(double) * std::max<size_t>(1, Rc[q].val.size()))};
    }
    std::vector<char> host(bytes, 0);
    for (int i = 0; i < nlevels; ++i) {
        const std::vector<double> &w = wn[(size_t)i];
        std::copy(w.begin(), w.end(), reinterpret_cast<double *>(host.data() + o_wn[(size_t)i]));
        float *f = reinterpret_cast<float *>(host.data() + o_w32[(size_t)i]);
        for (size_t q = 0; q < w.size(); ++q) f[q] = (float)w[q];
    }
    auto put = [&](const Csr &c, const Off &o) {
        std::copy(c.rowptr.begin(), c.rowptr.end(), reinterpret_cast<int32_t *>(host.data() + o.rp));
        std::copy(c.col.begin(), c.col.end(), reinterpret_cast<int32_t *>(host.data() + o.col));
        std::copy(c.val.begin(), c.val.end(), reinterpret_cast<double *>(host.data() + o.val));
    };
    for (size_t q = 0; q < Pc.size(); ++q) {
        put(Pc[q], oP[q]);
        put(Rc[q], oR[q]);
    }
    if ((rc = plan.dev.alloc(bytes, st))) return rc;
    char *base = plan.dev.as<char>();
    // (pageable source: the copy has read it when the call returns)
    H3D_CUDA_TRY(cudaMemcpyAsync(base, host.data(), bytes, cudaMemcpyHostToDevice, st));
    for (int i = 0; i < nlevels; ++i) {
        lv[(size_t)i].wn = reinterpret_cast<const double *>(base + o_wn[(size_t)i]);
        lv[(size_t)i].wn32 = reinterpret_cast<const float *>(base + o_w32[(size_t)i]);
    }
    plan.Rt.assign((size_t)std::max(1, nlevels - 1), h3d_ml_transfer{});
    plan.Pt.assign((size_t)std::max(1, nlevels - 1), h3d_ml_transfer{});
    for (int i = 0; i + 1 < nlevels; ++i) {
        h3d_ml_transfer &r = plan.Rt[(size_t)i], &p = plan.Pt[(size_t)i];
        for (int a = 0; a < 3; ++a) {
            const size_t q = (size_t)3 * i + a;
            p.rowptr[a] = reinterpret_cast<const int32_t *>(base + oP[q].rp);
            p.col[a] = reinterpret_cast<const int32_t *>(base + oP[q].col);
            p.val[a] = reinterpret_cast<const double *>(base + oP[q].val);
            r.rowptr[a] = reinterpret_cast<const int32_t *>(base + oR[q].rp);
            r.col[a] = reinterpret_cast<const int32_t *>(base + oR[q].col);
            r.val[a] = reinterpret_cast<const double *>(base + oR[q].val);
            p.n_in[a] = lv[(size_t)i + 1].grid.n[a];
            p.n_out[a] = lv[(size_t)i].grid.n[a];
            r.n_in[a] = lv[(size_t)i].grid.n[a];
            r.n_out[a] = lv[(size_t)i + 1].grid.n[a];
        }
        p.scale = 1.0;
        r.scale = 1.0 / 8.0;
    }
    return H3D_OK;
}

int ml_plan_solve(MlPlan &plan, const void *b, void *x, int mode, const h3d_ml_opts *opts, double *hst, int hst_cap,
                  h3d_ml_info *info, cudaStream_t st)
{
    return h3d_mlgmres_solve(plan.lv.data(), plan.nlevels, plan.Rt.data(), plan.Pt.data(), b, x, mode, opts, hst,
                             hst_cap, info, st);
}

}  // namespace

extern "C" {

int h3d_ml_interp_weights(int kind, const double *xin, int nin, const double *xout, int nout, double *A)
{
    if (!xin || !xout || !A || nin < 1 || nout < 1 || (kind != 0 && kind != 1) || (kind == 1 && nin < 4)) {
        set_error("h3d_ml_interp_weights: bad argument (cubic weights need 4 or more nodes)");
        return H3D_ERR_BAD_ARG;
    }
    for (int i = 1; i < nin; ++i)
        if (!(xin[i] > xin[i - 1])) {
            set_error("h3d_ml_interp_weights: nodes must ascend");
            return H3D_ERR_BAD_ARG;
        }
    for (int i = 1; i < nout; ++i)
        if (!(xout[i] >= xout[i - 1])) {
            set_error("h3d_ml_interp_weights: points must ascend");
            return H3D_ERR_BAD_ARG;
        }
    std::vector<double> xi(xin, xin + nin), xo(xout, xout + nout), W;
    if (kind == 0) linear_weights(xi, xo, W);
    else cubic_weights(xi, xo, W);
    std::copy(W.begin(), W.end(), A);
    return H3D_OK;
}

int h3d_ml_levels_host(const double *v_phys, const int32_t n_phys[3], const double h[3], int npml, double freq,
                       int unit, int nlevels, h3d_grid *grids, double *wn, size_t wn_cap)
{
    if (!grids || !wn) {
        set_error("h3d_ml_levels_host: bad argument");
        return H3D_ERR_BAD_ARG;
    }
    std::vector<h3d_grid> g;
    std::vector<std::vector<double>> w;
    int rc = ml_levels_host(v_phys, n_phys, h, npml, freq, unit, nlevels, g, w);
    if (rc) return rc;
    size_t need = 0;
    for (const auto &x : w) need += x.size();
    if (wn_cap < need) {
        set_error("h3d_ml_levels_host: wn holds %zu values, the levels need %zu", wn_cap, need);
        return H3D_ERR_BAD_ARG;
    }
    size_t off = 0;
    for (int i = 0; i < nlevels; ++i) {
        grids[i] = g[(size_t)i];
        std::copy(w[(size_t)i].begin(), w[(size_t)i].end(), wn + off);
        off += w[(size_t)i].size();
    }
    return H3D_OK;
}

int h3d_ml_coarsen_model(const double *v, const int32_t n[3], const int32_t n_sub[3], double *v_sub)
{
    if (!v || !n || !n_sub || !v_sub) {
        set_error("h3d_ml_coarsen_model: bad argument");
        return H3D_ERR_BAD_ARG;
    }
    for (int a = 0; a < 3; ++a)
        if (n[a] < 4 || n_sub[a] < 1) {
            set_error("h3d_ml_coarsen_model: every axis needs 4 or more points");
            return H3D_ERR_BAD_ARG;
        }
    const long long N = (long long)n[0] * n[1] * n[2];
    std::vector<double> in(v, v + N), out;
    coarsen(in, n, n_sub, out);
    std::copy(out.begin(), out.end(), v_sub);
    return H3D_OK;
}

int h3d_mlgmres_solve_model(const double *v_phys, const int32_t n_phys[3], const double h[3], int npml, double freq,
                            int unit, int nlevels, const void *b, void *x, int mode, const h3d_ml_opts *opts,
                            double *hst, int hst_cap, h3d_ml_info *info, void *stream)
{
    if (!b || !x) {
        set_error("h3d_mlgmres_solve_model: bad argument");
        return H3D_ERR_BAD_ARG;
    }
    cudaStream_t st = (cudaStream_t)stream;
    MlPlan plan;
    int rc = ml_plan_build(v_phys, n_phys, h, npml, freq, unit, nlevels, st, plan);
    if (rc) return rc;
    return ml_plan_solve(plan, b, x, mode, opts, hst, hst_cap, info, st);  // synchronises st
}

int h3d_mex_mlgmres(const double *v_phys, const double *n_phys, size_t n_len, const double *h, double npml,
                    double freq, int unit, int nlevels, const double *b_re, const double *b_im, size_t b_rows,
                    size_t nrhs, double *u_re, double *u_im, int mode, const h3d_ml_opts *opts, h3d_ml_info *info)
{
    if (!n_phys || n_len != 3) {
        set_error("n must be a 3-length vector");
        return H3D_ERR_NSIZE;
    }
    int32_t n[3];
    for (int a = 0; a < 3; ++a) {
        if (!(n_phys[a] >= 1) || n_phys[a] > 2147483647.0 || n_phys[a] != std::floor(n_phys[a])) {
            set_error("n must hold three positive integer sizes");
            return H3D_ERR_NSIZE;
        }
        n[a] = (int32_t)n_phys[a];
    }
    if (!(npml >= 0) || npml != std::floor(npml) || npml > 1e6) {
        set_error("npml must be a non-negative integer");
        return H3D_ERR_BAD_ARG;
    }
    const int p = (int)npml;
    const long long N = (long long)(n[0] + 2 * p) * (n[1] + 2 * p) * (n[2] + 2 * p);
    if ((long long)b_rows != N) {
        set_error("b must have (nx+2npml)*(ny+2npml)*(nz+2npml) rows");
        return H3D_ERR_BSIZE;
    }
    if (!v_phys || !h || !b_re || !u_re || !u_im || nrhs < 1 || nrhs > 2147483647u ||
        (mode != H3D_FORWARD && mode != H3D_ADJOINT)) {
        set_error("h3d_mex_mlgmres: bad argument");
        return H3D_ERR_BAD_ARG;
    }
    cudaStream_t st = nullptr;
    H3D_CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    h3d_ml_info tot{};
    tot.converged = 1;
    int rc;
    {
        MlPlan plan;
        DevBuf dpl, db, dx;
        const size_t pb = (size_t)N * sizeof(double);
        rc = ml_plan_build(v_phys, n, h, p, freq, unit, nlevels, st, plan);
        if (!rc) rc = dpl.alloc(2 * pb, st);
        if (!rc) rc = db.alloc(2 * pb, st);
        if (!rc) rc = dx.alloc(2 * pb, st);
        double *pre = dpl.as<double>(), *pim = pre + N;
        for (size_t c = 0; !rc && c < nrhs; ++c) {
            // each column an independent FGMRES solve from x = 0
            cudaError_t e = cudaMemcpyAsync(pre, b_re + c * N, pb, cudaMemcpyHostToDevice, st);
            if (e == cudaSuccess) {
                e = b_im ? cudaMemcpyAsync(pim, b_im + c * N, pb, cudaMemcpyHostToDevice, st)
                         : cudaMemsetAsync(pim, 0, pb, st);
            }
            if (e == cudaSuccess) e = cudaMemsetAsync(dx.p, 0, 2 * pb, st);
            if (e != cudaSuccess) {
                rc = cuda_fail(e, "h3d_mex_mlgmres copy");
                break;
            }
            if ((rc = interleave<double>(pre, pim, db.as<cplx<double>>(), N, st))) break;
            h3d_ml_info ci{};
            if ((rc = ml_plan_solve(plan, db.p, dx.p, mode, opts, nullptr, 0, &ci, st))) break;
            if ((rc = deinterleave<double>(dx.as<cplx<double>>(), pre, pim, N, st))) break;
            e = cudaMemcpyAsync(u_re + c * N, pre, pb, cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess) e = cudaMemcpyAsync(u_im + c * N, pim, pb, cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(st);
            if (e != cudaSuccess) {
                rc = cuda_fail(e, "h3d_mex_mlgmres copy");
                break;
            }
            tot.iters = std::max(tot.iters, ci.iters);
            tot.converged = tot.converged && ci.converged;
            tot.rel_res = std::max(tot.rel_res, ci.rel_res);
            tot.seconds += ci.seconds;
            tot.kernel_launches += ci.kernel_launches;
            tot.host_syncs += ci.host_syncs;
        }
    }
    cudaError_t e = cudaStreamSynchronize(st);
    cudaStreamDestroy(st);
    if (rc) return rc;
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamSynchronize");
    if (info) *info = tot;
    return H3D_OK;
}

}  // extern "C"
