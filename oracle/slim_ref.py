"""numpy restatement of the reference's MATLAB layers on the Helmholtz path (TEST INFRASTRUCTURE).

MATLAB and GNU Octave are not available, so these functions restate, line by line in
numpy, the MATLAB code that sits above the C stencil kernels; the kernels themselves
come from the C oracle (oracle/h3d_oracle.c).  Only tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg use this module.

Reference files (paths inside SLIM-release-apps):
  CGMN        tools/solvers/Krylov/CGMN.m
  linearsolve tools/solvers/Krylov/linearsolve.m
  divide      tools/algorithms/CommonFreqModeling/opAbstractMatrix.m
  p2w         tools/algorithms/CommonFreqModeling/param2wavenum.m
  dh          tools/algorithms/CommonFreqModeling/discrete_helmholtz.m
  ext         tools/operators/misc/opExtension.m
  sinc        tools/operators/misc/opSincInterp.m, opInterp.m
  kaiser      tools/functions/misc/kaiser_window.m, sinc.m
  wavelet     tools/algorithms/CommonFreqModeling/fwi_wavelet.m
  misfit      tools/algorithms/CommonFreqModeling/LS_misfit.m
  PDEfunc     tools/algorithms/CommonFreqModeling/PDEfunc.m
  dist        tools/algorithms/CommonFreqModeling/PDEfunc_dist.m, misfit_setup.m
"""
from __future__ import annotations

import numpy as np
import scipy.special

from . import h3d_oracle as O


# ---- CGMN.m:36-94 ---------------------------------------------------------------------------
def cgmn(A, b, x, tol=1e-6, maxit=None, out_freq=0):
    """Block CG with per-column alpha/beta; stops when max_j ||r_j||/||b_j|| <= tol
    (CGMN.m:79).  ``A`` maps (N, P) arrays to (N, P) arrays."""
    b = np.asarray(b, dtype=np.complex128)
    if b.ndim == 1:
        b = b[:, None]
        x = np.asarray(x, dtype=np.complex128).reshape(-1, 1)
        squeeze = True
    else:
        squeeze = False
    if maxit is None:
        maxit = b.shape[0]
    k = 0
    r = b - A(x)                                                   # :49
    p = r.copy()                                                   # :50
    norm = lambda y: np.sqrt(np.sum(np.abs(y) ** 2, axis=0))       # :52
    normb = norm(b)
    normr = norm(r)
    hst = [float(np.max(normr / normb))]                           # :62
    while True:
        Ap = A(p)                                                  # :67
        pAp = np.sum(np.conj(p) * Ap, axis=0)                      # :68
        alpha = normr ** 2 / pAp                                   # :69
        x = x + p * alpha                                          # :71
        r = r - Ap * alpha                                         # :72
        normr_old = normr
        normr = norm(r)                                            # :75
        hst.append(float(np.max(normr / normb)))                   # :76
        k += 1
        if k >= maxit or hst[-1] <= tol:                           # :79
            break
        beta = (normr / normr_old) ** 2                            # :83
        p = r + p * beta                                           # :85
        if out_freq > 0 and (k - 1) % out_freq == 0:
            print(f"k {k} res {hst[-1]:.3e}")
    return (x[:, 0] if squeeze else x), np.array(hst)


# ---- CRMN.m:38-107 --------------------------------------------------------------------------
def crmn(A, b, x=None, tol=1e-6, maxit=None):
    """Conjugate residual with per-column gamma/beta; stops when max_j ||r_j||/||b_j|| <= tol
    (CRMN.m:90).  ``A`` maps (N, P) arrays to (N, P) arrays; x None means a zero start
    (CRMN.m:47-49: r = b without a product; linearsolve passes zeros, CRMN.m:51)."""
    b = np.asarray(b, dtype=np.complex128)
    squeeze = b.ndim == 1
    if squeeze:
        b = b[:, None]
    if maxit is None:
        maxit = b.shape[0]
    if x is None:
        r = b.copy()                                               # :48
        x = np.zeros_like(b)
    else:
        x = np.asarray(x, dtype=np.complex128).reshape(b.shape)
        r = b - A(x)                                               # :51
    Ar = A(r)                                                      # :54
    p, Ap = r.copy(), Ar.copy()                                    # :55-56
    norm = lambda y: np.sqrt(np.sum(np.abs(y) ** 2, axis=0))       # :61-63
    inner = lambda u, v: np.sum(np.conj(u) * v, axis=0)            # :60-64
    nb, nr, nAp = norm(b), norm(r), norm(Ap)                       # :66-68
    rAr = inner(r, Ar)                                             # :69
    hst = [float(np.max(nr / nb))]                                 # :70
    k = 0
    while True:
        gamma = rAr / nAp ** 2                                     # :73-77
        x = x + p * gamma                                          # :79
        r = r - Ap * gamma                                         # :80
        nr = norm(r)                                               # :81
        hst.append(float(np.max(nr / nb)))                         # :82-84
        k += 1
        if k >= maxit or hst[-1] <= tol:                           # :90-92
            break
        Ar = A(r)                                                  # :94
        old = rAr
        rAr = inner(r, Ar)                                         # :97
        beta = rAr / old                                           # :98-102
        p = r + p * beta                                           # :103
        Ap = Ar + Ap * beta                                        # :104
        nAp = norm(Ap)                                             # :105
    return (x[:, 0] if squeeze else x), np.array(hst)


# ---- linearsolve.m:148-156 with PREC_KACZSWP, solver CGMN -------------------------------------
def linearsolve_cgmn(g, wn, b, mode=1, tol=1e-6, maxit=10000, order=O.ORDER_LEX, blk=None,
                     w=1.5, nthreads=None):
    """u solving H u = b (mode 1) or H^H u = b (else) by CGMN on (I - Q) u = DSWP(0, b)."""
    adj = mode != 1
    b = np.asarray(b, dtype=np.complex128)
    zb = np.zeros_like(b)                                          # :150
    bt = O.sweep(g, wn, w, zb, b, adj=adj, order=order, blk=blk, nthreads=nthreads)  # :151

    def A(y):                                                      # :152 opDirac - opFunction_swp
        return y - O.sweep(g, wn, w, y, None, adj=adj, order=order, blk=blk, nthreads=nthreads)

    x0 = np.zeros_like(b)                                          # :117-119
    return cgmn(A, bt, x0, tol=tol, maxit=maxit)


def linearsolve_crmn(g, wn, b, mode=1, tol=1e-6, maxit=10000, order=O.ORDER_LEX, blk=None,
                     w=1.5, nthreads=None):
    """linearsolve.m:148-156 with SOLVE_CRMN: CRMN on (I - Q) u = DSWP(0, b), zero start."""
    adj = mode != 1
    b = np.asarray(b, dtype=np.complex128)
    bt = O.sweep(g, wn, w, np.zeros_like(b), b, adj=adj, order=order, blk=blk, nthreads=nthreads)

    def A(y):
        return y - O.sweep(g, wn, w, y, None, adj=adj, order=order, blk=blk, nthreads=nthreads)

    return crmn(A, bt, np.zeros_like(b), tol=tol, maxit=maxit)


def divide(g, wn, b, mode=1, **kw):
    """opAbstractMatrix.divide (opAbstractMatrix.m:117-125): zero if norm(b) < 1e-12."""
    b = np.asarray(b, dtype=np.complex128)
    nb = np.linalg.norm(b, 2) if b.ndim == 1 else np.linalg.norm(b, 2)
    if nb < 1e-12:
        return np.zeros_like(b), np.array([0.0])
    return linearsolve_cgmn(g, wn, b, mode=mode, **kw)


def cgmn_solve(g, wn, b, tol=1e-6, maxit=10000, mode=1, order=O.ORDER_LEX, blk=None):
    return divide(g, wn, b, mode=mode, tol=tol, maxit=maxit, order=order, blk=blk)[0]


def true_residual(g, wn, b, u, mode=1):
    r = b - O.mvp(g, wn, u, adj=(mode != 1))
    return np.linalg.norm(r) / np.linalg.norm(b)


# ---- param2wavenum.m:20-49 ------------------------------------------------------------------
def param2wavenum(v, freq, unit):
    c = (2 * np.pi * freq) ** 2
    v = np.asarray(v, dtype=np.float64)
    if unit == "m/s":
        return c * v ** -2, -2 * c * v ** -3, 6 * c * v ** -4
    if unit == "s2/m2":
        return c * v, c * np.ones_like(v), np.zeros_like(v)
    if unit == "s2/km2":
        return 1e-6 * c * v, 1e-6 * c * np.ones_like(v), np.zeros_like(v)
    raise ValueError(f"Unknown unit - {unit}")


# ---- opExtension.m:85-101 (modes 0 and 1) and the 3D Kronecker products of dh:214-220 ---------
def ext1d(x, nb, mode, adjoint, axis):
    lo, hi = nb
    if not adjoint:
        if mode == 0:
            pad = [(0, 0)] * x.ndim
            pad[axis] = (lo, hi)
            return np.pad(x, pad)
        pad = [(0, 0)] * x.ndim
        pad[axis] = (lo, hi)
        return np.pad(x, pad, mode="edge")
    n = x.shape[axis]
    sl = [slice(None)] * x.ndim
    sl[axis] = slice(lo, n - hi)
    y = x[tuple(sl)].copy()
    if mode == 1:
        s_lo = [slice(None)] * x.ndim
        s_lo[axis] = slice(0, lo)
        s_hi = [slice(None)] * x.ndim
        s_hi[axis] = slice(n - hi, n)
        f = [slice(None)] * x.ndim
        f[axis] = slice(0, 1)
        l = [slice(None)] * x.ndim
        l[axis] = slice(-1, None)
        y[tuple(f)] += np.sum(x[tuple(s_lo)], axis=axis, keepdims=True)
        y[tuple(l)] += np.sum(x[tuple(s_hi)], axis=axis, keepdims=True)
    return y


def extend3d(v_phys, npml6, mode=1, adjoint=False):
    a = v_phys
    for ax in range(3):
        a = ext1d(a, (npml6[2 * ax], npml6[2 * ax + 1]), mode, adjoint, ax)
    return a


# ---- sinc interpolation: opSincInterp.m:26-70, kaiser_window.m, sinc.m, opInterp.m:108 ---------
def sinc_interp_matrix(xin, xout, r=4):
    xin = np.asarray(xin, dtype=np.float64)
    xout = np.asarray(xout, dtype=np.float64)
    if xout.size > 1:
        dx = xout[1] - xout[0]
        xin = xin / dx
        xout = xout / dx
    XOUT, XIN = np.meshgrid(xout, xin, indexing="ij")
    D = XOUT - XIN
    with np.errstate(invalid="ignore", divide="ignore"):
        s = np.where(D != 0, np.sin(np.pi * D) / (np.pi * np.where(D != 0, D, 1.0)), 1.0)
    if r > 0:
        r_b = [1.24, 2.94, 4.53, 6.31, 7.91, 9.42, 10.95, 12.53, 14.09, 14.18]
        b = r_b[r - 1]
        win = np.zeros_like(D)
        m = np.abs(D) <= r
        win[m] = scipy.special.i0(b * np.sqrt(1 - (D[m] / r) ** 2)) / scipy.special.i0(b)
        return win * s
    return s


def comp_axes(model_o, model_d, n_total, npml6):
    """odn2grid of the computational grid: ot = o - npml_lo * d (dh:210)."""
    return [model_o[a] - npml6[2 * a] * model_d[a] + np.arange(n_total[a]) * model_d[a] for a in range(3)]


def point_weights(axes, pt):
    """The column of Ps for one source point (opInterp with the point as the input grid)."""
    return [sinc_interp_matrix([pt[a]], axes[a])[:, 0] for a in range(3)]


def inject(n_total, axes, pts, amps):
    """sum_s amps[s] * kron(wz, wy, wx) as an (N, nsrc) array (one column per source)."""
    N = int(np.prod(n_total))
    out = np.zeros((N, len(pts)), dtype=np.complex128)
    for s, pt in enumerate(pts):
        wx, wy, wz = point_weights(axes, pt)
        out[:, s] = amps[s] * np.einsum("k,j,i->kji", wz, wy, wx).reshape(-1)
    return out


def sample(n_total, axes, rec_pts, U):
    """Pr U: receivers r = sum over the grid of the separable weights times U."""
    U = np.asarray(U).reshape(int(np.prod(n_total)), -1)
    out = np.zeros((len(rec_pts), U.shape[1]), dtype=np.complex128)
    for r, pt in enumerate(rec_pts):
        wx, wy, wz = point_weights(axes, pt)
        w = np.einsum("k,j,i->kji", wz, wy, wx).reshape(-1)
        out[r] = w @ U
    return out


def spread(n_total, axes, rec_pts, D):
    """Pr^T D."""
    N = int(np.prod(n_total))
    D = np.asarray(D).reshape(len(rec_pts), -1)
    out = np.zeros((N, D.shape[1]), dtype=np.complex128)
    for r, pt in enumerate(rec_pts):
        wx, wy, wz = point_weights(axes, pt)
        w = np.einsum("k,j,i->kji", wz, wy, wx).reshape(-1)
        out += np.outer(w, D[r])
    return out


# ---- fwi_wavelet.m:44-56, LS_misfit.m:21-26 --------------------------------------------------
def fwi_wavelet(f, t0, f0):
    f = np.asarray(f, dtype=np.float64)
    w = np.exp(-1j * 2 * np.pi * f * t0)
    if f0:
        w = f ** 2 * np.exp(-(f / f0) ** 2) * w
    return w


def ls_misfit(x, y):
    r = x - y
    return 0.5 * np.linalg.norm(r) ** 2, r


# ---- PDEfunc.m OBJ / FORW_MODEL for 3D (numcompsrc = 1, PDEfunc.m:157) ------------------------
def pdefunc(func, v_phys, model, src_pts, src_amp, rec_pts, freqs, Dobs=None, tol=1e-6,
            maxit=10000, order=O.ORDER_LEX, nthreads=None):
    """func in {"forw_model", "obj"}.  ``model``: dict(o, d, n, npml6, unit, f0, t0).
    Returns D (nrec x nsrc*nfreq) for forw_model, (f, g) for obj with g on the physical grid.
    Source amplitudes Q are the per-source scalars ``src_amp`` (Q = diag(src_amp) on a
    source grid that lists the points)."""
    d = model["d"]
    dt = model.get("dt", d)          # params.dt: model.d unless pdefunopts.helm_dt (PDEfunc.m:88-90)
    if tuple(dt) != tuple(d):
        raise NotImplementedError("a Helmholtz grid spacing other than the model's is not restated")
    npml6 = model["npml6"]
    unit = model.get("unit", "m/s")
    n_phys = tuple(model["n"])
    v_pml = extend3d(np.asarray(v_phys).reshape(n_phys, order="F"), npml6, mode=1)   # dh:240
    n_total = v_pml.shape
    axes = comp_axes(model["o"], d, n_total, npml6)
    g = O.make_grid(n_total, d, npml6)
    w = fwi_wavelet(freqs, model.get("t0", 0.0), model["f0"])                        # :214
    nsrc = len(src_pts)
    out = np.zeros((len(rec_pts), nsrc * len(freqs)), dtype=np.complex128)
    f = 0.0
    grad = np.zeros(n_phys, dtype=np.float64)
    col = 0
    for k, fr in enumerate(freqs):
        wn, dwn, _ = param2wavenum(v_pml.reshape(-1, order="F"), fr, unit)           # dh:244,256
        for s in range(nsrc):                                                        # :324
            q = inject(n_total, axes, [src_pts[s]], [w[k] * src_amp[s]])[:, 0]       # :335
            q = q * np.prod(d) / np.prod(dt)                                         # :339
            U = divide(g, wn, q, mode=1, tol=tol, maxit=maxit, order=order,
                       nthreads=nthreads)[0]                                         # :347
            dpred = sample(n_total, axes, rec_pts, U)[:, 0]
            if func == "forw_model":
                out[:, col] = dpred                                                  # :423
            else:
                phi, dphi = ls_misfit(dpred, Dobs[:, col])                           # :389
                f += phi
                rhs = -spread(n_total, axes, rec_pts, dphi)[:, 0]
                V = divide(g, wn, rhs, mode=2, tol=tol, maxit=maxit, order=order,
                           nthreads=nthreads)[0]                                     # :393
                # T(U)'*V = conj(U) .* (dH' * V)  (dh:288), real part, to_phys = crop (dh:232)
                dHV = O.mvp(g, dwn, V, adj=True, deriv=True, nthreads=nthreads)
                tu = np.real(np.conj(U) * dHV).reshape(n_total, order="F")
                grad += extend3d(tu, npml6, mode=0, adjoint=True)                    # :394
            col += 1
    if func == "forw_model":
        return out
    return f, grad.reshape(-1, order="F")
