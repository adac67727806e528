"""ctypes wrapper of the C oracle ``oracle/h3d_oracle.c`` (TEST INFRASTRUCTURE ONLY).

Builds ``oracle/_build/libh3d_oracle.so`` with ``make -C oracle oracle`` on first
use.  All arrays follow the reference layout: column-major, x fastest,
``idx = i + j*nx + k*nx*ny``, right-hand side ``s`` at offset ``s*N``.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libh3d_oracle.so")

ORDER_LEX, ORDER_COLOUR27, ORDER_BLOCK, ORDER_BLOCK8 = 0, 1, 2, 3

_lock = threading.Lock()
_lib = None


class Grid(C.Structure):
    _fields_ = [("n", C.c_int * 3), ("h", C.c_double * 3), ("npml", C.c_int * 6)]


def make_grid(n, h, npml) -> Grid:
    """``npml``: scalar, 3 values (same both sides) or 6 values lo_x,hi_x,lo_y,hi_y,lo_z,hi_z."""
    npml = np.asarray(npml, dtype=np.int64).ravel()
    if npml.size == 1:
        npml = np.repeat(npml, 6)
    elif npml.size == 3:
        npml = np.repeat(npml, 2)
    g = Grid()
    for a in range(3):
        g.n[a] = int(n[a])
        g.h[a] = float(h[a])
    for a in range(6):
        g.npml[a] = int(npml[a])
    return g


def build() -> str:
    subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)
    return LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                build()
            L = C.CDLL(LIB_PATH)
            dp = C.POINTER(C.c_double)
            L.h3do_mvp.argtypes = [C.POINTER(Grid), dp, dp, dp, dp, dp, dp, C.c_int, C.c_int,
                                   C.c_int, C.c_int]
            L.h3do_sweep.argtypes = [C.POINTER(Grid), dp, dp, C.c_double, dp, dp, dp, dp,
                                     C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int), C.c_int]
            L.h3do_row_coefs.argtypes = [C.POINTER(Grid), dp, dp, C.c_int, C.c_int, C.c_int,
                                         C.c_int, C.c_int, dp, dp]
            L.h3do_pml_axis.argtypes = [C.c_int, C.c_int, C.c_int, dp, dp, dp, dp]
            _lib = L
    return _lib


def _dp(a):
    if a is None:
        return C.POINTER(C.c_double)()
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _split(a):
    a = np.asarray(a)
    re = np.ascontiguousarray(np.real(a).reshape(-1, order="F"), dtype=np.float64)
    im = (np.ascontiguousarray(np.imag(a).reshape(-1, order="F"), dtype=np.float64)
          if np.iscomplexobj(a) else None)
    return re, im


def mvp(g: Grid, wn, x, adj=False, deriv=False, nthreads=None):
    """y = H x / H^H x / dH x / dH^H x for x of shape (N,) or (N, P)."""
    N = g.n[0] * g.n[1] * g.n[2]
    x = np.asarray(x)
    P = 1 if x.ndim == 1 else x.shape[1]
    wr, wi = _split(wn)
    xr, xi = _split(x.reshape(N, P, order="F"))
    yr = np.zeros(N * P)
    yi = np.zeros(N * P)
    nt = nthreads or os.cpu_count() or 1
    rc = lib().h3do_mvp(C.byref(g), _dp(wr), _dp(wi), _dp(xr), _dp(xi), _dp(yr), _dp(yi), P,
                        int(adj), int(deriv), nt)
    if rc:
        raise ValueError(f"h3do_mvp failed ({rc})")
    y = (yr + 1j * yi).reshape(N, P, order="F")
    return y[:, 0] if x.ndim == 1 else y


def sweep(g: Grid, wn, w, x, b=None, adj=False, order=ORDER_LEX, blk=None, nthreads=None):
    """Forward + backward Kaczmarz sweep applied to a copy of x (SWP:60-120)."""
    N = g.n[0] * g.n[1] * g.n[2]
    x = np.asarray(x)
    P = 1 if x.ndim == 1 else x.shape[1]
    wr, wi = _split(wn)
    xc = np.asarray(x, dtype=np.complex128).reshape(N, P, order="F")
    xr = np.ascontiguousarray(xc.real.reshape(-1, order="F"))
    xi = np.ascontiguousarray(xc.imag.reshape(-1, order="F"))
    if b is not None:
        bc = np.asarray(b, dtype=np.complex128).reshape(N, P, order="F")
        br = np.ascontiguousarray(bc.real.reshape(-1, order="F"))
        bi = np.ascontiguousarray(bc.imag.reshape(-1, order="F"))
    else:
        br = bi = None
    blk_arr = (C.c_int * 3)(*(blk if blk is not None else (0, 0, 0)))
    nt = nthreads or os.cpu_count() or 1
    rc = lib().h3do_sweep(C.byref(g), _dp(wr), _dp(wi), float(w), _dp(xr), _dp(xi), _dp(br),
                          _dp(bi), P, int(adj), int(order), blk_arr, nt)
    if rc:
        raise ValueError(f"h3do_sweep failed ({rc})")
    y = (xr + 1j * xi).reshape(N, P, order="F")
    return y[:, 0] if x.ndim == 1 else y


def row_coefs(g: Grid, wn, i, j, k, adj=False, deriv=False):
    wr, wi = _split(wn)
    cr = np.zeros(27)
    ci = np.zeros(27)
    lib().h3do_row_coefs(C.byref(g), _dp(wr), _dp(wi), i, j, k, int(adj), int(deriv), _dp(cr),
                         _dp(ci))
    return cr + 1j * ci


def pml_axis(n, nlo, nhi):
    """xi_lo, xi_hi over 0-based index -1..n (length n+2)."""
    arrs = [np.zeros(n + 2) for _ in range(4)]
    lib().h3do_pml_axis(n, nlo, nhi, *[_dp(a) for a in arrs])
    return arrs[0] + 1j * arrs[1], arrs[2] + 1j * arrs[3]
