// Internal device-side building blocks of the h3d library: complex arithmetic, the
// operator descriptor, and the 27-point coefficient rule of the Operto-style stencil
// with PML (tools/algorithms/3DFreqModeling/Helm3d_27pt.h in the reference).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "h3d.h"

namespace h3d {

// ---------------------------------------------------------------------------------------
// Complex numbers stored interleaved (re, im); 8- or 16-byte aligned for vector loads.
template <typename T>
struct alignas(2 * sizeof(T)) cplx {
    T re, im;
};

template <typename T>
__host__ __device__ __forceinline__ cplx<T> mk(T r, T i) { return cplx<T>{r, i}; }
template <typename T>
__host__ __device__ __forceinline__ cplx<T> operator+(cplx<T> a, cplx<T> b) { return {a.re + b.re, a.im + b.im}; }
template <typename T>
__host__ __device__ __forceinline__ cplx<T> operator-(cplx<T> a, cplx<T> b) { return {a.re - b.re, a.im - b.im}; }
template <typename T>
__host__ __device__ __forceinline__ cplx<T> operator*(cplx<T> a, cplx<T> b)
{
    return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
template <typename T>
__host__ __device__ __forceinline__ cplx<T> operator*(T s, cplx<T> a) { return {s * a.re, s * a.im}; }
template <typename T>
__host__ __device__ __forceinline__ cplx<T> cconj(cplx<T> a) { return {a.re, -a.im}; }
template <typename T>
__host__ __device__ __forceinline__ T cabs2(cplx<T> a) { return a.re * a.re + a.im * a.im; }
// acc += a * b as four chained multiply-adds (written one product per statement so that
// each contracts into one FMA; `acc += p - q` would cost a multiply, an FMA and an add)
template <typename T>
__host__ __device__ __forceinline__ void cmac(cplx<T> &acc, cplx<T> a, cplx<T> b)
{
    acc.re += a.re * b.re;
    acc.re -= a.im * b.im;
    acc.im += a.re * b.im;
    acc.im += a.im * b.re;
}
// acc += a * conj(b)
template <typename T>
__host__ __device__ __forceinline__ void cmac_cb(cplx<T> &acc, cplx<T> a, cplx<T> b)
{
    acc.re += a.re * b.re;
    acc.re += a.im * b.im;
    acc.im += a.im * b.re;
    acc.im -= a.re * b.im;
}

// ---------------------------------------------------------------------------------------
// Packed complex64 arithmetic.  sm_100-class GPUs execute an FP32 add / multiply / FMA on
// a register pair as one instruction (add.f32x2, fma.rn.f32x2), each component rounded
// exactly like the scalar operation, and take a scalar register or constant as a
// broadcast operand.  A complex value times a real scalar is then one instruction.  The
// packed forms pay off in issue-bound kernels (the matvec); the latency-bound Kaczmarz
// sweeps measured slower with them and keep the scalar forms.  PK selects the packed form
// (complex64 on sm_100+ only; complex128 is always scalar).
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 1000
#define H3D_F32X2 1
#else
#define H3D_F32X2 0
#endif

template <typename T>
__device__ __forceinline__ float2 f2_of(cplx<T> a) { return make_float2(a.re, a.im); }

// acc += s * v (s real)
template <bool PK = false, typename T>
__device__ __forceinline__ void fma_rc(cplx<T> &acc, T s, cplx<T> v)
{
#if H3D_F32X2
    if constexpr (PK && sizeof(T) == 4) {
        const float2 r = __ffma2_rn(make_float2(s, s), f2_of(v), f2_of(acc));
        acc = cplx<T>{r.x, r.y};
        return;
    }
#endif
    acc.re += s * v.re;
    acc.im += s * v.im;
}
// a + b
template <bool PK = false, typename T>
__device__ __forceinline__ cplx<T> cadd(cplx<T> a, cplx<T> b)
{
#if H3D_F32X2
    if constexpr (PK && sizeof(T) == 4) {
        const float2 r = __fadd2_rn(f2_of(a), f2_of(b));
        return cplx<T>{r.x, r.y};
    }
#endif
    return a + b;
}
// s * v (s real)
template <bool PK = false, typename T>
__device__ __forceinline__ cplx<T> cscale(T s, cplx<T> v)
{
#if H3D_F32X2
    if constexpr (PK && sizeof(T) == 4) {
        const float2 r = __fmul2_rn(make_float2(s, s), f2_of(v));
        return cplx<T>{r.x, r.y};
    }
#endif
    return s * v;
}

// A running sum of complex products.  Complex128: one accumulator, chained FMAs (cmac).
// Complex64: two partial sums P += a.re * b and Q += a.im * b (two independent FMA chains,
// or one packed instruction each), the product sum being (P.re - Q.im, P.im + Q.re).
template <typename T>
struct CSum {
    cplx<T> p, q;
};
template <typename T>
__device__ __forceinline__ CSum<T> csum_init(cplx<T> v0) { return CSum<T>{v0, mk<T>(T(0), T(0))}; }
template <bool PK = false, typename T>
__device__ __forceinline__ void csum_mac(CSum<T> &s, cplx<T> a, cplx<T> b)
{
    if constexpr (sizeof(T) == 4) {
        fma_rc<PK>(s.p, a.re, b);
        fma_rc<PK>(s.q, a.im, b);
    } else {
        cmac(s.p, a, b);
    }
}
// s += conj(a) * b
template <bool PK = false, typename T>
__device__ __forceinline__ void csum_mac_ca(CSum<T> &s, cplx<T> a, cplx<T> b)
{
    if constexpr (sizeof(T) == 4) {
        fma_rc<PK>(s.p, a.re, b);
        fma_rc<PK>(s.q, -a.im, b);
    } else {
        cmac(s.p, cconj(a), b);
    }
}
template <typename T>
__device__ __forceinline__ cplx<T> csum_value(const CSum<T> &s)
{
    if constexpr (sizeof(T) == 4) return mk<T>(s.p.re - s.q.im, s.p.im + s.q.re);
    else return s.p;
}
// acc += d * conj(c), the Kaczmarz scatter: c.re (d.re, d.im) + c.im (d.im, -d.re), with the
// pairs (d.re, d.im) and (d.im, -d.re) formed once per row
template <typename T>
struct Scat {
    cplx<T> d1, d2;
};
template <typename T>
__device__ __forceinline__ Scat<T> scat_of(cplx<T> d) { return Scat<T>{d, mk<T>(d.im, -d.re)}; }
template <typename T>
__device__ __forceinline__ void scat_mac(cplx<T> &o, const Scat<T> &s, cplx<T> c)
{
    fma_rc(o, c.re, s.d1);
    fma_rc(o, c.im, s.d2);
}

// Stencil weights W1..W3, WM1..WM4 (Helm3d_27pt.h:194-200).
constexpr double kW1 = 1.8395262e-5;
constexpr double kW2 = 0.296692333333333;
constexpr double kW3 = 0.027476150000000;
constexpr double kWM1 = 0.49649658;
constexpr double kWM2 = 0.075168750000000;
constexpr double kWM3 = 0.004373916666667;
constexpr double kWM4 = 5.690375e-07;

// ---------------------------------------------------------------------------------------
// Operator descriptor.  PML tables hold, per axis a, three arrays of n_a + 2 complex
// values indexed by (idx + 1) for 0-based idx in [-1, n_a]:  xi_lo(idx), xi_hi(idx)
// and their sum (pml_func_lower/upper of Helm3d_27pt.h:346-390 at 1-based idx+1).
template <typename T>
struct Op {
    int nx, ny, nz;
    long long N;                 // nx*ny*nz
    long long sy, sz;            // strides of j and k (nx, nx*ny)
    const T *wn;                 // wavenumber, real part (N)
    const T *wni;                // imaginary part or nullptr
    const cplx<T> *tab;          // PML tables
    int lo[3], hi[3], sum[3];    // offsets of the three arrays of each axis inside tab
    T wn_c, wn_x, wn_y, wn_z;    // centre coefficient and per-axis PML-sum coefficients
    T pml_x, pml_y, pml_z;       // face coefficients
    T xz, xy, yz;                // cross coefficients
    T w3a2;                      // corner coefficient
    // Interior (all xi = 1): PML part of the coefficient per offset class
    // [centre, face x, face y, face z, edge xy, edge xz, edge yz, corner].
    T kint[8];
    // Rows whose x and y PML values are all 1 but whose z values are not: the x/y brackets
    // fold into one real-weighted sum.  [in-plane: fx, fy, corners, centre; plane above or
    // below: fx, fy, corners, centre].
    T kxy[8];
    // Row index ranges [lo, hi) per axis whose PML values are all 1, for the forward
    // rows (xi_lo(i) = xi_hi(i) = 1) and the adjoint rows (xi_hi(i-1) = xi_lo(i+1) = 1
    // and xi_lo(i) + xi_hi(i) = 2).
    int int_lo_f[3], int_hi_f[3], int_lo_a[3], int_hi_a[3];
};

// Enumerate the 27 stencil offsets: t = (dx+1) + 3(dy+1) + 9(dz+1) (Helm3d_27pt.h:163-189).
#define H3D_FOR_27(M)                                                                          \
    M(0, -1, -1, -1) M(1, 0, -1, -1) M(2, 1, -1, -1) M(3, -1, 0, -1) M(4, 0, 0, -1)          \
    M(5, 1, 0, -1) M(6, -1, 1, -1) M(7, 0, 1, -1) M(8, 1, 1, -1) M(9, -1, -1, 0)             \
    M(10, 0, -1, 0) M(11, 1, -1, 0) M(12, -1, 0, 0) M(13, 0, 0, 0) M(14, 1, 0, 0)            \
    M(15, -1, 1, 0) M(16, 0, 1, 0) M(17, 1, 1, 0) M(18, -1, -1, 1) M(19, 0, -1, 1)           \
    M(20, 1, -1, 1) M(21, -1, 0, 1) M(22, 0, 0, 1) M(23, 1, 0, 1) M(24, -1, 1, 1)            \
    M(25, 0, 1, 1) M(26, 1, 1, 1)

// PML part of the coefficient at offset (DX,DY,DZ) given the directional values A*
// (xi_lo for a -1 offset, xi_hi for +1, seen from the row that owns the coefficient)
// and the per-axis sums S*.  One closed form per offset class replaces the 26 written-out
// lines of Helm3d_27pt.h:680-714 (forward) and :755-809 (adjoint, which uses the same
// expressions evaluated at the neighbouring row).
template <int DX, int DY, int DZ, typename T>
__device__ __forceinline__ cplx<T> pml_term(const Op<T> &op, cplx<T> Ax, cplx<T> Ay, cplx<T> Az,
                                            cplx<T> Sx, cplx<T> Sy, cplx<T> Sz)
{
    constexpr int nzc = (DX != 0) + (DY != 0) + (DZ != 0);
    if constexpr (nzc == 0) {
        return op.wn_x * Sx + op.wn_y * Sy + op.wn_z * Sz;
    } else if constexpr (nzc == 3) {
        return (-op.w3a2) * (Ax + Ay + Az);
    } else if constexpr (nzc == 1) {
        if constexpr (DX != 0) return op.pml_x * Ax + op.xz * Sz + op.xy * Sy;
        else if constexpr (DY != 0) return op.pml_y * Ay + op.yz * Sz + op.xy * Sx;
        else return op.pml_z * Az + op.yz * Sy + op.xz * Sx;
    } else {
        if constexpr (DZ == 0) return (-op.xy) * (Ax + Ay) + op.w3a2 * Sz;
        else if constexpr (DY == 0) return (-op.xz) * (Az + Ax) + op.w3a2 * Sy;
        else return (-op.yz) * (Az + Ay) + op.w3a2 * Sx;
    }
}

template <int DX, int DY, int DZ>
struct WM {
    static constexpr int nzc = (DX != 0) + (DY != 0) + (DZ != 0);
    static constexpr double value = nzc == 1 ? kWM2 : (nzc == 2 ? kWM3 : kWM4);
};

template <typename T, bool WNC>
__device__ __forceinline__ cplx<T> load_wn(const Op<T> &op, long long idx)
{
    if constexpr (WNC) return mk<T>(op.wn[idx], op.wni[idx]);
    else return mk<T>(op.wn[idx], T(0));
}

// Bitmask of the 27 neighbours of (i,j,k) that lie inside the grid.
__device__ __forceinline__ uint32_t inside_mask(int i, int j, int k, int nx, int ny, int nz)
{
    const bool xl = i > 0, xr = i < nx - 1, yl = j > 0, yr = j < ny - 1, zl = k > 0, zr = k < nz - 1;
    uint32_t m = 0;
#define H3D_MASK_BIT(t, dx, dy, dz)                                                            \
    if ((dx < 0 ? xl : (dx > 0 ? xr : true)) && (dy < 0 ? yl : (dy > 0 ? yr : true)) &&      \
        (dz < 0 ? zl : (dz > 0 ? zr : true)))                                                  \
        m |= (1u << t);
    H3D_FOR_27(H3D_MASK_BIT)
#undef H3D_MASK_BIT
    return m;
}

// The 27 coefficients of row (i,j,k).
//  forward (Helm3d_27pt.h:678-714): c_t = -WM_t wn[nbr] + pml_term(t) at the row, zero where
//    the neighbour is outside the grid;
//  adjoint (Helm3d_27pt.h:716-822): c_t = conj(-WM_t wn[row] + pml_term(t) evaluated at the
//    neighbour row), not masked;
//  DERIV (Helm3d_27pt.h:202-206, 754): the PML part is dropped.
// PML values one row needs: the per-axis sums S and the directional values A for the
// -1 and +1 offsets (forward: xi_lo(c), xi_hi(c); adjoint: xi_hi(c-1), xi_lo(c+1), the
// windows of pml_adj_info, Helm3d_27pt.h:252-260, 394-465).
template <typename T>
struct RowPml {
    cplx<T> Sx, Sy, Sz, Axm, Axp, Aym, Ayp, Azm, Azp;
};

template <typename T, bool ADJ>
__device__ __forceinline__ RowPml<T> load_row_pml(const Op<T> &op, int i, int j, int k)
{
    const cplx<T> *t = op.tab;
    RowPml<T> p;
    p.Sx = t[op.sum[0] + i + 1];
    p.Sy = t[op.sum[1] + j + 1];
    p.Sz = t[op.sum[2] + k + 1];
    if constexpr (!ADJ) {
        p.Axm = t[op.lo[0] + i + 1]; p.Axp = t[op.hi[0] + i + 1];
        p.Aym = t[op.lo[1] + j + 1]; p.Ayp = t[op.hi[1] + j + 1];
        p.Azm = t[op.lo[2] + k + 1]; p.Azp = t[op.hi[2] + k + 1];
    } else {
        p.Axm = t[op.hi[0] + i]; p.Axp = t[op.lo[0] + i + 2];
        p.Aym = t[op.hi[1] + j]; p.Ayp = t[op.lo[1] + j + 2];
        p.Azm = t[op.hi[2] + k]; p.Azp = t[op.lo[2] + k + 2];
    }
    return p;
}

// Coefficient of one offset (T = 0..26 fixed at compile time).
template <int TT, int DX, int DY, int DZ, typename T, bool ADJ, bool DERIV, bool WNC, typename WnF>
__device__ __forceinline__ cplx<T> coef_at(const Op<T> &op, const RowPml<T> &p, uint32_t inmask,
                                           WnF wnf)
{
    const cplx<T> Ax = DX < 0 ? p.Axm : p.Axp, Ay = DY < 0 ? p.Aym : p.Ayp, Az = DZ < 0 ? p.Azm : p.Azp;
    cplx<T> v;
    if constexpr (!ADJ) {
        if (inmask & (1u << TT)) {
            const cplx<T> wv = wnf(DX, DY, DZ);
            v = (TT == 13) ? op.wn_c * wv : T(-WM<DX, DY, DZ>::value) * wv;
            if constexpr (!DERIV) v = v + pml_term<DX, DY, DZ, T>(op, Ax, Ay, Az, p.Sx, p.Sy, p.Sz);
        } else {
            v = mk<T>(T(0), T(0));
        }
    } else {
        const cplx<T> wc = wnf(0, 0, 0);
        v = (TT == 13) ? op.wn_c * wc : T(-WM<DX, DY, DZ>::value) * wc;
        if constexpr (!DERIV) v = v + pml_term<DX, DY, DZ, T>(op, Ax, Ay, Az, p.Sx, p.Sy, p.Sz);
        v = cconj(v);
    }
    return v;
}

// The wavenumber of neighbour (dx,dy,dz) comes from a caller-supplied accessor
// wnf(dx, dy, dz) -> cplx<T> (global memory or a shared-memory tile).
template <typename T, bool ADJ, bool DERIV, bool WNC, typename WnF>
__device__ __forceinline__ void row_coefs_with(const Op<T> &op, int i, int j, int k,
                                               uint32_t inmask, WnF wnf, cplx<T> c[27])
{
    RowPml<T> p{};
    if constexpr (!DERIV) p = load_row_pml<T, ADJ>(op, i, j, k);
#define H3D_COEF2(t, dx, dy, dz) c[t] = coef_at<t, dx, dy, dz, T, ADJ, DERIV, WNC>(op, p, inmask, wnf);
    H3D_FOR_27(H3D_COEF2)
#undef H3D_COEF2
}

// Real coefficients of a row whose PML values are all xi_lo = xi_hi = 1 (the interior):
// c_t = K_t - WM_t * wn_t with the class constants K_t of Op::kint (forward: wn of the
// neighbour; adjoint: wn of the centre, and conj is the identity for real values).
template <typename T, bool ADJ, typename WnR>
__device__ __forceinline__ void row_coefs_interior(const Op<T> &op, WnR wnr, T c[27])
{
    const T wc = wnr(0, 0, 0);
#define H3D_COEF_INT(t, dx, dy, dz)                                                            \
    {                                                                                          \
        constexpr int nzc = (dx != 0) + (dy != 0) + (dz != 0);                                 \
        constexpr int cls = nzc == 0 ? 0 : nzc == 3 ? 7                                        \
                          : nzc == 1 ? (dx ? 1 : dy ? 2 : 3) : (!dz ? 4 : !dy ? 5 : 6);        \
        const T wv = ADJ ? wc : ((t == 13) ? wc : wnr(dx, dy, dz));                            \
        c[t] = (t == 13) ? (op.wn_c * wv + op.kint[0]) : (op.kint[cls] - T(WM<dx, dy, dz>::value) * wv); \
    }
    H3D_FOR_27(H3D_COEF_INT)
#undef H3D_COEF_INT
}

// One interior coefficient (see row_coefs_interior).
template <int TT, int DX, int DY, int DZ, typename T, bool ADJ, typename WnR>
__device__ __forceinline__ T coef_int(const Op<T> &op, WnR wnr)
{
    constexpr int nzc = (DX != 0) + (DY != 0) + (DZ != 0);
    constexpr int cls = nzc == 0 ? 0 : nzc == 3 ? 7 : nzc == 1 ? (DX ? 1 : DY ? 2 : 3) : (!DZ ? 4 : !DY ? 5 : 6);
    const T wv = ADJ ? wnr(0, 0, 0) : wnr(DX, DY, DZ);
    if constexpr (TT == 13) return op.wn_c * wv + op.kint[0];
    else return op.kint[cls] - T(WM<DX, DY, DZ>::value) * wv;
}

template <typename T, bool ADJ, bool DERIV, bool WNC>
__device__ __forceinline__ void row_coefs(const Op<T> &op, int i, int j, int k, uint32_t inmask,
                                          cplx<T> c[27])
{
    const long long ctr = i + op.sy * j + op.sz * k;
    row_coefs_with<T, ADJ, DERIV, WNC>(op, i, j, k, inmask,
                                       [&](int dx, int dy, int dz) {
                                           return load_wn<T, WNC>(op, ctr + dx + op.sy * dy + op.sz * dz);
                                       },
                                       c);
}

// ---------------------------------------------------------------------------------------
// Host-side helpers (h3d_host.cpp).
struct DeviceTables;

int make_op_f64(const h3d_grid *g, const double *wn, const double *wni, Op<double> *op);
int make_op_f32(const h3d_grid *g, const float *wn, const float *wni, Op<float> *op);
int make_op_f64_at(const h3d_grid *g, const double *wn, const double *wni, const void *dev_tab,
                   std::vector<cplx<double>> *host_tab, Op<double> *op);
int check_grid(const h3d_grid *g);
void set_error(const char *fmt, ...);
int cuda_fail(cudaError_t e, const char *what);

#define H3D_CUDA_TRY(expr)                                                                     \
    do {                                                                                       \
        cudaError_t _e = (expr);                                                               \
        if (_e != cudaSuccess) return ::h3d::cuda_fail(_e, #expr);                             \
    } while (0)

}  // namespace h3d
