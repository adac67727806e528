"""ctypes binding of libh3d.so (the C ABI of include/h3d.h).

The library must have been built (``h3d.build.build()``); importing this module
does not fall back to anything else: a missing library raises ``ImportError``.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from . import build as _build

_lock = threading.Lock()
_lib = None

OK = 0
ERR_NSIZE, ERR_XSIZE, ERR_BSIZE, ERR_BAD_ARG, ERR_NOT_CONVERGED, ERR_TIMEOUT, ERR_CUDA, \
    ERR_NO_MEMORY, ERR_NONFINITE = range(1, 10)
C128, C64 = 0, 1
FORWARD, ADJOINT = 1, 2
ORDER_LEX, ORDER_COLOUR27, ORDER_BLOCK, ORDER_BLOCK8 = 0, 1, 2, 3
METHOD_CGMN, METHOD_CRMN = 0, 1
PREC_FP64, PREC_MIXED = 0, 1
STOP_PRECONDITIONED, STOP_TRUE_RESIDUAL = 0, 1


class Grid(C.Structure):
    _fields_ = [("n", C.c_int32 * 3), ("h", C.c_double * 3), ("npml", C.c_int32 * 6)]


class SolveOpts(C.Structure):
    _fields_ = [
        ("tol", C.c_double), ("maxit", C.c_int32), ("w", C.c_double), ("precision", C.c_int32),
        ("order", C.c_int32), ("stop_rule", C.c_int32), ("check_every", C.c_int32),
        ("inner_tol", C.c_double), ("max_outer", C.c_int32), ("block", C.c_int32 * 3),
        ("use_graphs", C.c_int32), ("verbose", C.c_int32), ("method", C.c_int32),
    ]


class SolveInfo(C.Structure):
    _fields_ = [
        ("iters", C.c_int32), ("outer", C.c_int32), ("converged", C.c_int32), ("nrhs", C.c_int32),
        ("rel_res_true", C.c_double), ("rel_res_prec", C.c_double), ("seconds", C.c_double),
        ("sweep_seconds", C.c_double), ("sweep_samples", C.c_int32), ("sweep_variant", C.c_int32),
        ("kernel_launches", C.c_int64), ("sweep_bytes", C.c_double),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Problem(C.Structure):
    _fields_ = [
        ("grid", Grid), ("wn_re", C.c_void_p), ("wn_im", C.c_void_p), ("b", C.c_void_p),
        ("u", C.c_void_p), ("nrhs", C.c_int32), ("mode", C.c_int32),
    ]


class MLLevel(C.Structure):
    _fields_ = [("grid", Grid), ("wn", C.c_void_p), ("wn32", C.c_void_p)]


class MLTransfer(C.Structure):
    _fields_ = [
        ("rowptr", C.c_void_p * 3), ("col", C.c_void_p * 3), ("val", C.c_void_p * 3),
        ("n_in", C.c_int32 * 3), ("n_out", C.c_int32 * 3), ("scale", C.c_double),
    ]


class MLOpts(C.Structure):
    _fields_ = [
        ("tol", C.c_double), ("maxit", C.c_int32), ("maxinnerit", C.c_int32), ("precond", C.c_int32),
        ("precision", C.c_int32), ("k", C.c_int32 * 4), ("smooth_tol", C.c_double),
        ("coarse_tol", C.c_double),
    ]


class MLInfo(C.Structure):
    _fields_ = [
        ("iters", C.c_int32), ("converged", C.c_int32), ("rel_res", C.c_double), ("seconds", C.c_double),
        ("kernel_launches", C.c_int64), ("host_syncs", C.c_int64),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


ML_PREC_NONE, ML_PREC_MLGMRES = 0, 1
UNIT_M_PER_S, UNIT_S2_PER_M2, UNIT_S2_PER_KM2 = 0, 1, 2
UNITS = {"m/s": UNIT_M_PER_S, "s2/m2": UNIT_S2_PER_M2, "s2/km2": UNIT_S2_PER_KM2}


class H3DError(RuntimeError):
    """A non-zero status from the C ABI; ``.status`` and ``.ident`` as the reference's IDs."""

    def __init__(self, status: int, where: str, msg: str, ident: str):
        super().__init__(f"{where}: status {status} ({ident}): {msg}")
        self.status = status
        self.ident = ident


vp = C.c_void_p
dp = C.POINTER(C.c_double)

_SIGS = {
    "h3d_version": (C.c_int, []),
    "h3d_status_id": (C.c_char_p, [C.c_int]),
    "h3d_last_error": (C.c_char_p, []),
    "h3d_default_opts": (None, [C.POINTER(SolveOpts)]),
    "h3d_mvp": (C.c_int, [C.POINTER(Grid), vp, vp, vp, vp, C.c_int, C.c_int, C.c_int, C.c_int, vp]),
    "h3d_kacz_sweep": (C.c_int, [C.POINTER(Grid), vp, vp, C.c_double, vp, vp, C.c_int, C.c_int,
                                 C.c_int, C.POINTER(C.c_int32), C.c_int, vp]),
    "h3d_residual": (C.c_int, [C.POINTER(Grid), vp, vp, vp, vp, vp, vp, vp, C.c_int, C.c_int, vp]),
    "h3d_residual_noalloc": (C.c_int, [C.POINTER(Grid), vp, vp, vp, vp, vp, vp, vp, C.c_int, C.c_int,
                                       vp]),
    "h3d_check_wait_timeout": (C.c_int, [C.c_double]),
    "h3d_mex_mvp": (C.c_int, [dp, dp, dp, dp, C.c_size_t, dp, dp, dp, C.c_size_t, dp, dp, C.c_int,
                              C.c_int]),
    "h3d_mex_kacz_sweep": (C.c_int, [dp, dp, dp, dp, C.c_size_t, dp, C.c_double, dp, dp,
                                     C.c_size_t, C.c_size_t, dp, dp, C.c_size_t, dp, dp, C.c_int,
                                     C.c_int]),
    "h3d_solve": (C.c_int, [C.POINTER(Grid), vp, vp, vp, vp, C.c_int, C.c_int,
                            C.POINTER(SolveOpts), C.POINTER(SolveInfo), dp, C.c_int, vp]),
    "h3d_solve_batch": (C.c_int, [C.POINTER(Problem), C.c_int, C.POINTER(SolveOpts),
                                  C.POINTER(SolveInfo), vp]),
    "h3d_solve_host": (C.c_int, [C.POINTER(Grid), vp, vp, vp, vp, C.c_int, C.c_int,
                                 C.POINTER(SolveOpts), C.POINTER(SolveInfo)]),
    "h3d_mex_solve": (C.c_int, [dp, dp, dp, dp, C.c_size_t, dp, dp, dp, C.c_size_t, C.c_size_t, dp, dp, C.c_int,
                                C.POINTER(SolveOpts), C.POINTER(SolveInfo)]),
    "h3d_fwi_grad": (C.c_int, [C.POINTER(Grid), dp, dp, dp, C.c_int, dp, dp, C.c_int, dp, C.POINTER(SolveOpts),
                               dp, dp, C.POINTER(SolveInfo)]),
    "h3d_grad_accum": (C.c_int, [C.POINTER(Grid), vp, vp, vp, C.c_int, C.c_double, vp, vp]),
    "h3d_sinc_weights": (C.c_int, [C.POINTER(Grid), dp, C.c_int, C.POINTER(C.c_int32), dp]),
    "h3d_src_inject": (C.c_int, [C.POINTER(Grid), vp, vp, vp, vp, C.c_int, vp]),
    "h3d_rec_sample": (C.c_int, [C.POINTER(Grid), vp, vp, C.c_int, vp, C.c_int, vp, vp]),
    "h3d_rec_spread": (C.c_int, [C.POINTER(Grid), vp, vp, C.c_int, vp, C.c_int, C.c_double, vp,
                                 vp]),
    "h3d_axis_apply": (C.c_int, [vp, vp, vp, C.c_int, C.c_int, C.POINTER(C.c_int32), vp, vp, C.c_int,
                                 C.c_int, vp]),
    "h3d_ml_default_opts": (None, [C.POINTER(MLOpts)]),
    "h3d_ml_interp_weights": (C.c_int, [C.c_int, dp, C.c_int, dp, C.c_int, dp]),
    "h3d_ml_coarsen_model": (C.c_int, [dp, C.POINTER(C.c_int32), C.POINTER(C.c_int32), dp]),
    "h3d_ml_levels_host": (C.c_int, [dp, C.POINTER(C.c_int32), dp, C.c_int, C.c_double, C.c_int, C.c_int,
                                     C.POINTER(Grid), dp, C.c_size_t]),
    "h3d_mlgmres_solve_model": (C.c_int, [dp, C.POINTER(C.c_int32), dp, C.c_int, C.c_double, C.c_int, C.c_int, vp,
                                          vp, C.c_int, C.POINTER(MLOpts), dp, C.c_int, C.POINTER(MLInfo), vp]),
    "h3d_mex_mlgmres": (C.c_int, [dp, dp, C.c_size_t, dp, C.c_double, C.c_double, C.c_int, C.c_int, dp, dp,
                                  C.c_size_t, C.c_size_t, dp, dp, C.c_int, C.POINTER(MLOpts), C.POINTER(MLInfo)]),
    "h3d_mlgmres_solve": (C.c_int, [C.POINTER(MLLevel), C.c_int, C.POINTER(MLTransfer), C.POINTER(MLTransfer),
                                    vp, vp, C.c_int, C.POINTER(MLOpts), dp, C.c_int, C.POINTER(MLInfo), vp]),
    "h3d_band_coefs": (C.c_int, [C.POINTER(Grid), vp, vp, C.c_int, vp, C.POINTER(C.c_int64), C.c_int, vp]),
    "h3d_band_mvp": (C.c_int, [vp, C.POINTER(C.c_int64), C.c_int, C.c_int64, vp, vp, C.c_int, C.c_int, vp]),
    "h3d_band_sweep": (C.c_int, [C.POINTER(Grid), vp, C.POINTER(C.c_int64), vp, C.c_double, vp, vp, C.c_int,
                                 C.c_int, vp]),
    "h3d_mex_band_mvp": (C.c_int, [dp, dp, C.c_size_t, C.c_size_t, dp, dp, dp, C.c_size_t, C.c_size_t, dp,
                                   dp]),
    "h3d_mex_band_sweep": (C.c_int, [dp, dp, C.c_size_t, C.c_size_t, dp, dp, dp, C.c_size_t, C.c_size_t, dp,
                                     dp, C.c_size_t, C.c_double, dp, C.c_size_t, dp, dp]),
}

EXPORTED = sorted(_SIGS)


def lib_path() -> str:
    return _build.LIB


def load(path: str | None = None):
    """Load libh3d.so and bind every exported symbol (raises if any is missing)."""
    global _lib
    with _lock:
        if _lib is not None and path is None:
            return _lib
        p = path or lib_path()
        if not os.path.exists(p):
            raise ImportError(f"libh3d.so not built at {p}: run h3d.build.build()")
        L = C.CDLL(p)
        missing = [name for name in _SIGS if not hasattr(L, name)]
        if missing:
            raise ImportError(f"{p} lacks exported symbols: {missing}")
        for name, (res, args) in _SIGS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        if path is None:
            _lib = L
        return L


def check(status: int, where: str):
    if status != OK:
        L = load()
        raise H3DError(status, where, L.h3d_last_error().decode(errors="replace"),
                       L.h3d_status_id(status).decode())


def make_grid(n, h, npml) -> Grid:
    """``npml``: scalar, 3 values (same on both sides), 6 values (lo_x, hi_x, lo_y, hi_y,
    lo_z, hi_z) or the reference's 2x3 matrix (rows lo/hi, columns x/y/z)."""
    import numpy as np

    p = np.asarray(npml)
    if p.shape == (2, 3):
        p = p.T.reshape(-1)          # column-major 2x3 -> lo_x, hi_x, lo_y, hi_y, lo_z, hi_z
    p = p.astype(np.int64).ravel()
    if p.size == 1:
        p = np.repeat(p, 6)
    elif p.size == 3:
        p = np.repeat(p, 2)
    if p.size != 6:
        raise ValueError("npml must have 1, 3 or 6 entries or be 2x3")
    g = Grid()
    for a in range(3):
        g.n[a] = int(n[a])
        g.h[a] = float(h[a])
    for a in range(6):
        g.npml[a] = int(p[a])
    return g


def default_opts(**kw) -> SolveOpts:
    o = SolveOpts()
    load().h3d_default_opts(C.byref(o))
    for k, v in kw.items():
        if k == "block":
            for a in range(3):
                o.block[a] = int(v[a])
        else:
            setattr(o, k, v)
    return o
