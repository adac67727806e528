// Host-side set-up shared by every entry point: argument checks, the stencil constants
// (Helm3d_27pt.h:639-671), the PML tables (Helm3d_27pt.h:326-390) and a small per-device
// cache of those tables, plus error reporting.
#include <cmath>
#include <complex>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "h3d_internal.cuh"
#include "h3d_kernels.cuh"

namespace h3d {

static thread_local char g_last_error[512] = "";

void set_error(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof g_last_error, fmt, ap);
    va_end(ap);
}

int cuda_fail(cudaError_t e, const char *what)
{
    set_error("CUDA error %d (%s) in %s", (int)e, cudaGetErrorString(e), what);
    return e == cudaErrorMemoryAllocation ? H3D_ERR_NO_MEMORY : H3D_ERR_CUDA;
}

const char *last_error() { return g_last_error; }

int check_grid(const h3d_grid *g)
{
    if (!g) {
        set_error("grid is NULL");
        return H3D_ERR_BAD_ARG;
    }
    for (int a = 0; a < 3; ++a) {
        if (g->n[a] < 1) {
            set_error("n must be a 3-length vector of positive sizes");
            return H3D_ERR_NSIZE;
        }
        if (!(g->h[a] > 0) || !std::isfinite(g->h[a])) {
            set_error("h must hold three positive spacings");
            return H3D_ERR_BAD_ARG;
        }
    }
    for (int a = 0; a < 6; ++a)
        if (g->npml[a] < 0) {
            set_error("npml entries must be non-negative");
            return H3D_ERR_BAD_ARG;
        }
    const long long N = (long long)g->n[0] * g->n[1] * g->n[2];
    if (N > (1LL << 40)) {
        set_error("grid too large");
        return H3D_ERR_NSIZE;
    }
    return H3D_OK;
}

// ---- PML functions: the reference's pml_func_lower / pml_func_upper with 1-based x ----
static double gam_lo(double x, double n, double nlo) { return std::cos(M_PI * ((x - 1) * n / (2 * (n + 1) * nlo))); }
static double gam_hi(double x, double n, double nhi) { return std::cos(M_PI * ((1 - (x - 1) / (n + 1)) * n / (2 * nhi))); }

// As in the reference, the interior test of both functions uses the low-side width.
static std::complex<double> xi_lower(double x, double n, double nlo, double nhi)
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
    return std::complex<double>(2.0, 0.0) / std::complex<double>(2.0 - g1 * (g1 + g), 3.0 * g1 + g);
}

static std::complex<double> xi_upper(double x, double n, double nlo, double nhi)
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
    return std::complex<double>(2.0, 0.0) / std::complex<double>(2.0 - g1 * (g1 + g2), 3.0 * g1 + g2);
}

// Table layout: for axis a, [lo(n_a+2) | hi(n_a+2) | sum(n_a+2)] consecutively.
static void fill_tables(const h3d_grid *g, std::vector<std::complex<double>> &tab, int lo[3], int hi[3], int sum[3])
{
    tab.clear();
    for (int a = 0; a < 3; ++a) {
        const int n = g->n[a];
        const double nlo = g->npml[2 * a], nhi = g->npml[2 * a + 1];
        lo[a] = (int)tab.size();
        hi[a] = lo[a] + n + 2;
        sum[a] = hi[a] + n + 2;
        tab.resize(tab.size() + 3 * (size_t)(n + 2));
        for (int idx = -1; idx <= n; ++idx) {
            const std::complex<double> l = xi_lower(idx + 1, n, nlo, nhi);
            const std::complex<double> h = xi_upper(idx + 1, n, nlo, nhi);
            tab[lo[a] + idx + 1] = l;
            tab[hi[a] + idx + 1] = h;
            tab[sum[a] + idx + 1] = l + h;
        }
    }
}

struct TabEntry {
    void *dev = nullptr;
    int lo[3], hi[3], sum[3];
};

using TabKey = std::tuple<int, int, int, int, int, int, int, int, int, int, int>;
static std::mutex g_tab_mutex;
static std::map<TabKey, TabEntry> g_tab_cache;

template <typename T>
static int get_tables(const h3d_grid *g, TabEntry *out)
{
    int dev = 0;
    H3D_CUDA_TRY(cudaGetDevice(&dev));
    TabKey key{dev, (int)sizeof(T), g->n[0], g->n[1], g->n[2], g->npml[0], g->npml[1], g->npml[2],
               g->npml[3], g->npml[4], g->npml[5]};
    std::lock_guard<std::mutex> lk(g_tab_mutex);
    auto it = g_tab_cache.find(key);
    if (it != g_tab_cache.end()) {
        *out = it->second;
        return H3D_OK;
    }
    std::vector<std::complex<double>> tab;
    TabEntry e;
    fill_tables(g, tab, e.lo, e.hi, e.sum);
    std::vector<cplx<T>> host(tab.size());
    for (size_t q = 0; q < tab.size(); ++q) host[q] = mk<T>((T)tab[q].real(), (T)tab[q].imag());
    H3D_CUDA_TRY(cudaMalloc(&e.dev, host.size() * sizeof(cplx<T>)));
    H3D_CUDA_TRY(cudaMemcpy(e.dev, host.data(), host.size() * sizeof(cplx<T>), cudaMemcpyHostToDevice));
    g_tab_cache[key] = e;
    *out = e;
    return H3D_OK;
}

template <typename T>
static int make_op(const h3d_grid *g, const T *wn, const T *wni, Op<T> *op)
{
    int rc = check_grid(g);
    if (rc) return rc;
    mvp_prime_occupancy();
    TabEntry e;
    rc = get_tables<T>(g, &e);
    if (rc) return rc;
    Op<T> o{};
    o.nx = g->n[0];
    o.ny = g->n[1];
    o.nz = g->n[2];
    o.sy = o.nx;
    o.sz = (long long)o.nx * o.ny;
    o.N = o.sz * o.nz;
    o.wn = wn;
    o.wni = wni;
    o.tab = (const cplx<T> *)e.dev;
    for (int a = 0; a < 3; ++a) {
        o.lo[a] = e.lo[a];
        o.hi[a] = e.hi[a];
        o.sum[a] = e.sum[a];
    }
    // Helm3d_27pt.h:644-665, in FP64, then rounded to T.
    const double hx2 = g->h[0] * g->h[0], hy2 = g->h[1] * g->h[1], hz2 = g->h[2] * g->h[2];
    const double hxy = hx2 + hy2, hxz = hx2 + hz2, hyz = hy2 + hz2, hxyz = hx2 + hy2 + hz2;
    const double w3a = kW3 * 3 / (4 * hxyz);
    o.w3a2 = (T)(2 * w3a);
    o.wn_c = (T)(-(kW1 + 3 * kW2 + 16 * w3a * hxyz / 3 + kWM1 - 1));
    o.wn_x = (T)(kW1 / hx2 + kW2 / hx2 + kW2 / hxz + kW2 / hxy + 8 * w3a);
    o.wn_y = (T)(kW1 / hy2 + kW2 / hy2 + kW2 / hyz + kW2 / hxy + 8 * w3a);
    o.wn_z = (T)(kW1 / hz2 + kW2 / hz2 + kW2 / hxz + kW2 / hyz + 8 * w3a);
    o.pml_x = (T)(-(kW1 / hx2 + kW2 / hx2 + kW2 / hxz + kW2 / hxy + 8 * w3a));
    o.pml_y = (T)(-(kW1 / hy2 + kW2 / hy2 + kW2 / hyz + kW2 / hxy + 8 * w3a));
    o.pml_z = (T)(-(kW1 / hz2 + kW2 / hz2 + kW2 / hxz + kW2 / hyz + 8 * w3a));
    o.xz = (T)(kW2 / (2 * hxz));
    o.xy = (T)(kW2 / (2 * hxy));
    o.yz = (T)(kW2 / (2 * hyz));
    // Interior class constants: the PML terms with every xi_lo = xi_hi = 1 (so each
    // per-axis sum is 2), in the offset classes [centre, face x/y/z, edge xy/xz/yz, corner].
    o.kint[0] = (T)(2 * ((double)o.wn_x + (double)o.wn_y + (double)o.wn_z));
    o.kint[1] = (T)((double)o.pml_x + 2 * (double)o.xz + 2 * (double)o.xy);
    o.kint[2] = (T)((double)o.pml_y + 2 * (double)o.yz + 2 * (double)o.xy);
    o.kint[3] = (T)((double)o.pml_z + 2 * (double)o.yz + 2 * (double)o.xz);
    o.kint[4] = (T)(-2 * (double)o.xy + 2 * (double)o.w3a2);
    o.kint[5] = (T)(-2 * (double)o.xz + 2 * (double)o.w3a2);
    o.kint[6] = (T)(-2 * (double)o.yz + 2 * (double)o.w3a2);
    o.kint[7] = (T)(-3 * (double)o.w3a2);
    o.kxy[0] = (T)((double)o.pml_x + 2 * (double)o.xy);
    o.kxy[1] = (T)((double)o.pml_y + 2 * (double)o.xy);
    o.kxy[2] = (T)(-2 * (double)o.xy);
    o.kxy[3] = (T)(2 * ((double)o.wn_x + (double)o.wn_y));
    o.kxy[4] = (T)(-(double)o.xz + 2 * (double)o.w3a2);
    o.kxy[5] = (T)(-(double)o.yz + 2 * (double)o.w3a2);
    o.kxy[6] = (T)(-2 * (double)o.w3a2);
    o.kxy[7] = (T)(2 * ((double)o.xz + (double)o.yz));
    // Row ranges whose PML values are exactly 1 (and whose neighbours are all inside the
    // grid), from the same FP64 tables the kernels use.
    {
        std::vector<std::complex<double>> tab;
        int lo[3], hi[3], sum[3];
        fill_tables(g, tab, lo, hi, sum);
        const std::complex<double> one(1.0, 0.0), two(2.0, 0.0);
        for (int a = 0; a < 3; ++a) {
            const int n = g->n[a];
            auto fwd = [&](int i) { return tab[lo[a] + i + 1] == one && tab[hi[a] + i + 1] == one; };
            auto adj = [&](int i) {
                return tab[hi[a] + i] == one && tab[lo[a] + i + 2] == one && tab[sum[a] + i + 1] == two;
            };
            for (int pass = 0; pass < 2; ++pass) {
                int first = -1, last = -2;
                for (int i = 1; i < n - 1; ++i)
                    if (pass == 0 ? fwd(i) : adj(i)) {
                        if (first < 0) first = i;
                        last = i;
                    }
                bool contiguous = first >= 0;
                for (int i = first; contiguous && i <= last; ++i) contiguous = pass == 0 ? fwd(i) : adj(i);
                const int l = contiguous ? first : 0, h = contiguous ? last + 1 : 0;
                if (pass == 0) {
                    o.int_lo_f[a] = l;
                    o.int_hi_f[a] = h;
                } else {
                    o.int_lo_a[a] = l;
                    o.int_hi_a[a] = h;
                }
            }
        }
    }
    *op = o;
    return H3D_OK;
}

int make_op_f64(const h3d_grid *g, const double *wn, const double *wni, Op<double> *op)
{
    return make_op<double>(g, wn, wni, op);
}

// FP64 operator whose PML tables live at a caller-chosen device address (no allocation,
// no table cache): the host tables are returned in *host_tab for the caller to copy to
// dev_tab.  Used by the entry point that must not allocate device memory.
int make_op_f64_at(const h3d_grid *g, const double *wn, const double *wni, const void *dev_tab,
                   std::vector<cplx<double>> *host_tab, Op<double> *op)
{
    int rc = check_grid(g);
    if (rc) return rc;
    mvp_prime_occupancy();
    std::vector<std::complex<double>> tab;
    Op<double> o{};
    fill_tables(g, tab, o.lo, o.hi, o.sum);
    host_tab->resize(tab.size());
    for (size_t q = 0; q < tab.size(); ++q) (*host_tab)[q] = mk<double>(tab[q].real(), tab[q].imag());
    o.nx = g->n[0];
    o.ny = g->n[1];
    o.nz = g->n[2];
    o.sy = o.nx;
    o.sz = (long long)o.nx * o.ny;
    o.N = o.sz * o.nz;
    o.wn = wn;
    o.wni = wni;
    o.tab = (const cplx<double> *)dev_tab;
    const double hx2 = g->h[0] * g->h[0], hy2 = g->h[1] * g->h[1], hz2 = g->h[2] * g->h[2];
    const double hxy = hx2 + hy2, hxz = hx2 + hz2, hyz = hy2 + hz2, hxyz = hx2 + hy2 + hz2;
    const double w3a = kW3 * 3 / (4 * hxyz);
    o.w3a2 = 2 * w3a;
    o.wn_c = -(kW1 + 3 * kW2 + 16 * w3a * hxyz / 3 + kWM1 - 1);
    o.wn_x = kW1 / hx2 + kW2 / hx2 + kW2 / hxz + kW2 / hxy + 8 * w3a;
    o.wn_y = kW1 / hy2 + kW2 / hy2 + kW2 / hyz + kW2 / hxy + 8 * w3a;
    o.wn_z = kW1 / hz2 + kW2 / hz2 + kW2 / hxz + kW2 / hyz + 8 * w3a;
    o.pml_x = -o.wn_x;
    o.pml_y = -o.wn_y;
    o.pml_z = -o.wn_z;
    o.xz = kW2 / (2 * hxz);
    o.xy = kW2 / (2 * hxy);
    o.yz = kW2 / (2 * hyz);
    // The residual kernel uses only the general coefficient form: no interior fast path.
    for (int a = 0; a < 3; ++a) {
        o.int_lo_f[a] = o.int_hi_f[a] = o.int_lo_a[a] = o.int_hi_a[a] = 0;
    }
    *op = o;
    return H3D_OK;
}

int make_op_f32(const h3d_grid *g, const float *wn, const float *wni, Op<float> *op)
{
    return make_op<float>(g, wn, wni, op);
}

}  // namespace h3d
