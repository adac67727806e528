// Plane-sum form of one row of the 27-point operator, shared by the matvec and the
// sweep gather.  The coefficients of Helm3d_27pt.h:676-825 regroup per z-plane: from the
// 3 x 3 in-plane neighbourhood a thread forms the centre, the x- and y-face values and the
// corner pairs split by the sign of dx and of dy; a row then combines planes k-1, k, k+1
// into 9 complex PML factors (xi per direction, S per axis) times real-weighted brackets
// of those sums, plus the wavenumber (mass) part.
#pragma once

#include "h3d_internal.cuh"

namespace h3d {

// Plane partial sums of one thread.  W* are the mass sums: forward, weighted by the
// neighbour's wavenumber; adjoint, unweighted (the centre wavenumber multiplies later).
template <typename T>
struct PlaneSums {
    cplx<T> m, fxm, fxp, fym, fyp, cxm, cxp, cym, cyp;  // cxm = corners with dx = -1, ...
    cplx<T> wm, wfx, wfy, wc4;
};

template <typename T, bool WNC>
__device__ __forceinline__ cplx<T> wmul(cplx<T> w, cplx<T> v)
{
    if constexpr (WNC) return w * v;
    else return cscale<true>(w.re, v);
}

template <typename T, bool ADJ, bool WNC, int PITCH>
__device__ __forceinline__ PlaneSums<T> plane_sums(const cplx<T> *sxp, const T *swr, const T *swi, int l)
{
    // l = index of the thread's centre in the staged plane, PITCH = its row pitch
    auto X = [&](int dx, int dy) { return sxp[l + dx + PITCH * dy]; };
    auto W = [&](int dx, int dy) {
        const int q = l + dx + PITCH * dy;
        return mk<T>(swr[q], WNC ? swi[q] : T(0));
    };
    PlaneSums<T> p;
    const cplx<T> mm = X(-1, -1), mp = X(-1, 1), pm = X(1, -1), pp = X(1, 1);
    p.m = X(0, 0);
    p.fxm = X(-1, 0);
    p.fxp = X(1, 0);
    p.fym = X(0, -1);
    p.fyp = X(0, 1);
    p.cxm = cadd<true>(mm, mp);
    p.cxp = cadd<true>(pm, pp);
    p.cym = cadd<true>(mm, pm);
    p.cyp = cadd<true>(mp, pp);
    if constexpr (!ADJ) {
        p.wm = wmul<T, WNC>(W(0, 0), p.m);
        if constexpr (WNC) {
            p.wfx = wmul<T, WNC>(W(-1, 0), p.fxm) + wmul<T, WNC>(W(1, 0), p.fxp);
            p.wfy = wmul<T, WNC>(W(0, -1), p.fym) + wmul<T, WNC>(W(0, 1), p.fyp);
            p.wc4 = wmul<T, WNC>(W(-1, -1), mm) + wmul<T, WNC>(W(-1, 1), mp) + wmul<T, WNC>(W(1, -1), pm) +
                    wmul<T, WNC>(W(1, 1), pp);
        } else {
            // real wavenumber: products then accumulated one FMA each
            p.wfx = cscale<true>(W(-1, 0).re, p.fxm);
            fma_rc<true>(p.wfx, W(1, 0).re, p.fxp);
            p.wfy = cscale<true>(W(0, -1).re, p.fym);
            fma_rc<true>(p.wfy, W(0, 1).re, p.fyp);
            p.wc4 = cscale<true>(W(-1, -1).re, mm);
            fma_rc<true>(p.wc4, W(-1, 1).re, mp);
            fma_rc<true>(p.wc4, W(1, -1).re, pm);
            fma_rc<true>(p.wc4, W(1, 1).re, pp);
        }
    } else {
        p.wm = p.m;
        p.wfx = cadd<true>(p.fxm, p.fxp);
        p.wfy = cadd<true>(p.fym, p.fyp);
        p.wc4 = cadd<true>(p.cxm, p.cxp);
    }
    return p;
}

template <typename T>
__device__ __forceinline__ cplx<T> rc(T a, cplx<T> v) { return mk<T>(a * v.re, a * v.im); }

// Brackets of one pending row: the mass part and the real-weighted sums multiplying each
// of the 9 complex PML factors (xi per direction and axis, S per axis).  Planes are
// added one at a time in the role they play for the row: L (k-1), C (k) or U (k+1).
template <typename T>
struct RowAcc {
    cplx<T> mass, bxm, bxp, bym, byp, bzm, bzp, bsx, bsy, bsz;
};

template <typename T>
__device__ __forceinline__ void acc_zero(RowAcc<T> &a)
{
    const cplx<T> z = mk<T>(T(0), T(0));
    a.mass = a.bxm = a.bxp = a.bym = a.byp = a.bzm = a.bzp = a.bsx = a.bsy = a.bsz = z;
}

// acc = s v (SET: the bracket's first term for this row) or acc += s v.  Every bracket is
// set by the first plane that touches it -- role 0 for all but bsz (role 1) and bzp
// (role 2) -- so a finished row's accumulators need no clearing before they serve the next
// row.  s v equals 0 + s v exactly, so the values do not change.
template <bool SET, typename T>
__device__ __forceinline__ void put_rc(cplx<T> &acc, T s, cplx<T> v)
{
    if constexpr (SET) acc = cscale<true>(s, v);
    else fma_rc<true>(acc, s, v);
}

// ROLE: 0 = the plane below the row (k-1), 1 = the row's plane, 2 = the plane above.
template <int ROLE, typename T, bool DERIV>
__device__ __forceinline__ void acc_plane(RowAcc<T> &a, const PlaneSums<T> &P, const Op<T> &op)
{
    constexpr bool F = ROLE == 0;  // first plane of the row
    const T w3 = op.w3a2;
    if constexpr (ROLE == 1) {
        fma_rc<true>(a.mass, op.wn_c, P.wm);
        fma_rc<true>(a.mass, T(-kWM2), cadd<true>(P.wfx, P.wfy));
        fma_rc<true>(a.mass, T(-kWM3), P.wc4);
    } else {
        put_rc<F>(a.mass, T(-kWM2), P.wm);
        fma_rc<true>(a.mass, T(-kWM3), cadd<true>(P.wfx, P.wfy));
        fma_rc<true>(a.mass, T(-kWM4), P.wc4);
    }
    if constexpr (!DERIV) {
        const cplx<T> fx = cadd<true>(P.fxm, P.fxp), fy = cadd<true>(P.fym, P.fyp), c4 = cadd<true>(P.cxm, P.cxp);
        if constexpr (ROLE == 1) {
            fma_rc<true>(a.bxm, op.pml_x, P.fxm); fma_rc<true>(a.bxm, -op.xy, P.cxm);
            fma_rc<true>(a.bxp, op.pml_x, P.fxp); fma_rc<true>(a.bxp, -op.xy, P.cxp);
            fma_rc<true>(a.bym, op.pml_y, P.fym); fma_rc<true>(a.bym, -op.xy, P.cym);
            fma_rc<true>(a.byp, op.pml_y, P.fyp); fma_rc<true>(a.byp, -op.xy, P.cyp);
            fma_rc<true>(a.bsx, op.wn_x, P.m); fma_rc<true>(a.bsx, op.xy, fy);
            fma_rc<true>(a.bsy, op.wn_y, P.m); fma_rc<true>(a.bsy, op.xy, fx);
            put_rc<true>(a.bsz, op.wn_z, P.m); fma_rc<true>(a.bsz, op.xz, fx); fma_rc<true>(a.bsz, op.yz, fy); fma_rc<true>(a.bsz, w3, c4);
        } else {
            put_rc<F>(a.bxm, -op.xz, P.fxm); fma_rc<true>(a.bxm, -w3, P.cxm);
            put_rc<F>(a.bxp, -op.xz, P.fxp); fma_rc<true>(a.bxp, -w3, P.cxp);
            put_rc<F>(a.bym, -op.yz, P.fym); fma_rc<true>(a.bym, -w3, P.cym);
            put_rc<F>(a.byp, -op.yz, P.fyp); fma_rc<true>(a.byp, -w3, P.cyp);
            put_rc<F>(a.bsx, op.xz, P.m); fma_rc<true>(a.bsx, w3, fy);
            put_rc<F>(a.bsy, op.yz, P.m); fma_rc<true>(a.bsy, w3, fx);
            cplx<T> &bz = ROLE == 0 ? a.bzm : a.bzp;
            put_rc<true>(bz, op.pml_z, P.m); fma_rc<true>(bz, -op.xz, fx); fma_rc<true>(bz, -op.yz, fy); fma_rc<true>(bz, -w3, c4);
        }
    }
}

// y = (adjoint: conj(wn_centre) *) mass + sum over the 9 factors of factor * bracket
// (adjoint: the conjugated, neighbour-shifted factors).
template <typename T, bool ADJ, bool DERIV, bool WNC>
__device__ __forceinline__ cplx<T> acc_finish(const RowAcc<T> &a, const RowPml<T> &p, cplx<T> wc)
{
    cplx<T> y = a.mass;
    if constexpr (ADJ) y = WNC ? cconj(wc) * y : cscale<true>(wc.re, y);
    if constexpr (!DERIV) {
        CSum<T> s = csum_init(y);
        auto mac = [&](cplx<T> f, cplx<T> br) {
            if constexpr (ADJ) csum_mac_ca<true>(s, f, br);
            else csum_mac<true>(s, f, br);
        };
        mac(p.Axm, a.bxm);
        mac(p.Axp, a.bxp);
        mac(p.Aym, a.bym);
        mac(p.Ayp, a.byp);
        mac(p.Azm, a.bzm);
        mac(p.Azp, a.bzp);
        mac(p.Sx, a.bsx);
        mac(p.Sy, a.bsy);
        mac(p.Sz, a.bsz);
        y = csum_value(s);
    }
    return y;
}

// Rows whose x and y PML values are all 1 (A = 1, S = 2): the x/y brackets fold into one
// real-weighted sum r (kept in a.bsx) with the constants Op::kxy; ZI: the row's z values
// are 1 as well, and every bracket folds into r with the interior class constants Op::kint.
// The mass part is accumulated as in acc_plane.
template <int ROLE, typename T, bool ZI>
__device__ __forceinline__ void acc_plane_xy(RowAcc<T> &a, const PlaneSums<T> &P, const Op<T> &op)
{
    constexpr bool F = ROLE == 0;  // first plane of the row
    if constexpr (ROLE == 1) {
        fma_rc<true>(a.mass, op.wn_c, P.wm);
        fma_rc<true>(a.mass, T(-kWM2), cadd<true>(P.wfx, P.wfy));
        fma_rc<true>(a.mass, T(-kWM3), P.wc4);
    } else {
        put_rc<F>(a.mass, T(-kWM2), P.wm);
        fma_rc<true>(a.mass, T(-kWM3), cadd<true>(P.wfx, P.wfy));
        fma_rc<true>(a.mass, T(-kWM4), P.wc4);
    }
    const cplx<T> fx = cadd<true>(P.fxm, P.fxp), fy = cadd<true>(P.fym, P.fyp), c4 = cadd<true>(P.cxm, P.cxp);
    cplx<T> &r = a.bsx;
    if constexpr (ZI) {
        if constexpr (ROLE == 1) {
            fma_rc<true>(r, op.kint[1], fx); fma_rc<true>(r, op.kint[2], fy); fma_rc<true>(r, op.kint[4], c4); fma_rc<true>(r, op.kint[0], P.m);
        } else {
            put_rc<F>(r, op.kint[5], fx); fma_rc<true>(r, op.kint[6], fy); fma_rc<true>(r, op.kint[7], c4); fma_rc<true>(r, op.kint[3], P.m);
        }
    } else {
        const T w3 = op.w3a2;
        if constexpr (ROLE == 1) {
            fma_rc<true>(r, op.kxy[0], fx); fma_rc<true>(r, op.kxy[1], fy); fma_rc<true>(r, op.kxy[2], c4); fma_rc<true>(r, op.kxy[3], P.m);
            put_rc<true>(a.bsz, op.wn_z, P.m); fma_rc<true>(a.bsz, op.xz, fx); fma_rc<true>(a.bsz, op.yz, fy); fma_rc<true>(a.bsz, w3, c4);
        } else {
            put_rc<F>(r, op.kxy[4], fx); fma_rc<true>(r, op.kxy[5], fy); fma_rc<true>(r, op.kxy[6], c4); fma_rc<true>(r, op.kxy[7], P.m);
            cplx<T> &bz = ROLE == 0 ? a.bzm : a.bzp;
            put_rc<true>(bz, op.pml_z, P.m); fma_rc<true>(bz, -op.xz, fx); fma_rc<true>(bz, -op.yz, fy); fma_rc<true>(bz, -w3, c4);
        }
    }
}

// Row value from the folded accumulators (ZI: no z brackets left).
template <typename T, bool ADJ, bool ZI>
__device__ __forceinline__ cplx<T> acc_finish_xy(const RowAcc<T> &a, const RowPml<T> &p, cplx<T> wc)
{
    cplx<T> y = a.mass;
    if constexpr (ADJ) y = cscale<true>(wc.re, y);
    y = cadd<true>(y, a.bsx);
    if constexpr (!ZI) {
        CSum<T> s = csum_init(y);
        auto mac = [&](cplx<T> f, cplx<T> br) {
            if constexpr (ADJ) csum_mac_ca<true>(s, f, br);
            else csum_mac<true>(s, f, br);
        };
        mac(p.Azm, a.bzm);
        mac(p.Azp, a.bzp);
        mac(p.Sz, a.bsz);
        y = csum_value(s);
    }
    return y;
}

}  // namespace h3d
