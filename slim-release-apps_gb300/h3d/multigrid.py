"""FGMRES with the three-level ML_GMRES multigrid preconditioner on the GPU.

The reference's 3D applications solve the Helmholtz system with FGMRES (tol 1e-6, restart
after 5 steps) preconditioned by ML_GMRES (fwi_exp.m:58-62, discrete_helmholtz.m:344-360):

  levels       construct_multigrid.m:10-60  level i+1: physical model coarsened by 4-point
               Lagrange interpolation (opLInterp1D) to ceil(n/2) points, spacing 2^i dt,
               ceil(npml/2^i) PML points, edge-replicated into the PML, param2wavenum
  transfers    prolongation P = linear interpolation between the computational grids
               (LinInterp1D on linspace(0,1,n) nodes), restriction R = P^T / 8
  V-cycle      GMG_V.m: FGMRES smoothing (3 restarts x 5 steps, no preconditioner),
               residual, restriction, coarse solve, prolongation, smoothing again
  coarse solve FGMRES (3 x 5 steps, tol 0.5) preconditioned by the next level's V-cycle;
               on the last level by an unpreconditioned FGMRES of the same settings
               (ML_GMRES.m:36-72, opMultigrid.m construct with recursive_v_cycle)
  outer        FGMRES.m, preconditioned by the level-0 V-cycle

The solve itself is one library call (h3d_mlgmres_solve): the FGMRES control flow in C++,
every Arnoldi step, Givens rotation and stopping test on the device, the library's 27-point
matvec and its axis kernel for the grid transfers.  The interpolation weights and the model
coarsening are the library's host code (h3d_ml_interp_weights, h3d_ml_coarsen_model); this
module assembles the levels from them, or solve_model hands the physical model to the library
(h3d_mlgmres_solve_model).
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np
import torch

from . import _lib as L
from . import ops


# ---- interpolation weights and model coarsening (the library's host code) -----------------------
def _weights(kind, xin, xout):
    xin = np.ascontiguousarray(xin, float)
    xout = np.ascontiguousarray(xout, float)
    A = np.zeros((len(xout), len(xin)))
    rc = L.load().h3d_ml_interp_weights(kind, xin.ctypes.data_as(L.dp), len(xin), xout.ctypes.data_as(L.dp),
                                        len(xout), A.ctypes.data_as(L.dp))
    L.check(rc, "h3d_ml_interp_weights")
    return A


def linear_weights(xin, xout):
    """LinInterp1D.m: the len(xout) x len(xin) linear interpolation (dense)."""
    return _weights(0, np.sort(np.asarray(xin, float)), np.sort(np.asarray(xout, float)))


def cubic_weights(x1, x2):
    """opLInterp1D.m getLA: len(x2) x len(x1) 4-point Lagrange interpolation (zero rows
    for points outside the node range)."""
    return _weights(1, x1, x2)


def _coarsen_model(v, n_sub):
    """Physical model on n_sub points per axis by separable cubic interpolation."""
    v = np.asarray(v, float)
    n = (C.c_int32 * 3)(*v.shape)
    ns = (C.c_int32 * 3)(*(int(x) for x in n_sub))
    src = np.ascontiguousarray(v.reshape(-1, order="F"))
    out = np.zeros(int(np.prod(n_sub)))
    rc = L.load().h3d_ml_coarsen_model(src.ctypes.data_as(L.dp), n, ns, out.ctypes.data_as(L.dp))
    L.check(rc, "h3d_ml_coarsen_model")
    return out.reshape(tuple(int(x) for x in n_sub), order="F")


def _extend(v, npml):
    return np.pad(v, [(npml, npml)] * 3, mode="edge")


def _wavenumber(v, freq, unit):
    c = (2 * np.pi * freq) ** 2
    if unit == "m/s":
        return c * v ** -2.0
    if unit == "s2/m2":
        return c * v
    if unit == "s2/km2":
        return 1e-6 * c * v
    raise ValueError(f"Unknown unit - {unit}")


# ---- device pieces ---------------------------------------------------------------------------
class _AxisOp:
    """A dense host matrix along one axis, kept on the device in CSR form."""

    def __init__(self, A, dev):
        A = np.asarray(A, float)
        rows, cols = np.nonzero(A)
        self.n_out, self.n_in = A.shape
        rowptr = np.zeros(self.n_out + 1, np.int32)
        np.add.at(rowptr, rows + 1, 1)
        rowptr = np.cumsum(rowptr).astype(np.int32)
        self.rowptr = torch.as_tensor(rowptr, device=dev)
        self.col = torch.as_tensor(cols.astype(np.int32), device=dev)
        self.val = torch.as_tensor(A[rows, cols], device=dev)


class Transfer:
    """Separable operator A_z (x) A_y (x) A_x on column-major fields (optionally scaled)."""

    def __init__(self, Ax, Ay, Az, dev, scale=1.0):
        self.ops = [_AxisOp(A, dev) for A in (Ax, Ay, Az)]
        self.scale = scale
        self.n_in = tuple(o.n_in for o in self.ops)
        self.n_out = tuple(o.n_out for o in self.ops)

    def __call__(self, x: torch.Tensor) -> torch.Tensor:
        lib = L.load()
        dims = list(self.n_in)
        cur = x.contiguous()
        dt = L.C128 if cur.dtype == torch.complex128 else L.C64
        st = torch.cuda.current_stream().cuda_stream
        for axis, op in enumerate(self.ops):
            out_dims = list(dims)
            out_dims[axis] = op.n_out
            out = torch.empty(int(np.prod(out_dims)), dtype=cur.dtype, device=cur.device)
            d_in = (C.c_int32 * 3)(*dims)
            L.check(lib.h3d_axis_apply(C.c_void_p(op.rowptr.data_ptr()), C.c_void_p(op.col.data_ptr()),
                                       C.c_void_p(op.val.data_ptr()), op.n_out, axis, d_in,
                                       C.c_void_p(cur.data_ptr()), C.c_void_p(out.data_ptr()), 1, dt,
                                       C.c_void_p(st)), "h3d_axis_apply")
            cur, dims = out, out_dims
        return cur * self.scale if self.scale != 1.0 else cur


class Level:
    """One discretisation level: computational grid (PML included) and wavenumber."""

    def __init__(self, v_phys, dt, npml, freq, unit, dev):
        self.v_phys = np.asarray(v_phys, float)
        self.dt = tuple(float(x) for x in dt)
        self.npml = int(npml)
        self.nt = tuple(int(n + 2 * self.npml) for n in self.v_phys.shape)
        wn = _wavenumber(_extend(self.v_phys, self.npml), freq, unit)
        self.wn = torch.as_tensor(wn.reshape(-1, order="F").copy(), device=dev)
        self.wn32 = self.wn.float()
        self.grid = L.make_grid(self.nt, self.dt, (self.npml,) * 6)

    def A(self, x: torch.Tensor, mode: int = 1) -> torch.Tensor:
        """H x (mode 1) or H^H x in the precision of x (complex128 or complex64)."""
        return ops.mvp(self.grid, self.wn if x.dtype == torch.complex128 else self.wn32, x, mode)


def build_levels(v_phys, dt, npml, freq, unit="m/s", nlevels=3, device=None):
    """Levels, restrictions and prolongations (construct_multigrid.m:10-60)."""
    dev = torch.device(device or "cuda")
    lv = [Level(v_phys, dt, npml, freq, unit, dev)]
    R, P = [], []
    v = np.asarray(v_phys, float)
    g = lambda m: np.linspace(0.0, 1.0, int(m))
    for i in range(1, nlevels):
        n_sub = tuple(math.ceil(n / 2) for n in v.shape)
        v = _coarsen_model(v, n_sub)
        coarse = Level(v, tuple(d * 2 ** i for d in dt), math.ceil(npml / 2 ** i), freq, unit, dev)
        fine = lv[-1]
        Ls = [linear_weights(g(coarse.nt[a]), g(fine.nt[a])) for a in range(3)]  # coarse -> fine
        P.append(Transfer(*Ls, dev))
        R.append(Transfer(*(Lm.T for Lm in Ls), dev, scale=1.0 / 8.0))
        lv.append(coarse)
    return lv, R, P


# ---- FGMRES + ML_GMRES (h3d_mlgmres_solve) -------------------------------------------------
def _level_structs(levels, R, P):
    lv = (L.MLLevel * len(levels))()
    for i, l in enumerate(levels):
        lv[i].grid = l.grid
        lv[i].wn = l.wn.data_ptr()
        lv[i].wn32 = l.wn32.data_ptr()

    def tr(t):
        s = L.MLTransfer()
        for a, op in enumerate(t.ops):
            s.rowptr[a] = op.rowptr.data_ptr()
            s.col[a] = op.col.data_ptr()
            s.val[a] = op.val.data_ptr()
            s.n_in[a] = op.n_in
            s.n_out[a] = op.n_out
        s.scale = float(t.scale)
        return s

    n = max(1, len(R))
    Rs = (L.MLTransfer * n)(*[tr(t) for t in R])
    Ps = (L.MLTransfer * n)(*[tr(t) for t in P])
    return lv, Rs, Ps


def solve(levels, R, P, b: torch.Tensor, tol=1e-6, maxit=10000, maxinnerit=5, mode=1, precision="fp64",
          precond="mlgmres", x0: torch.Tensor | None = None, k=(3, 5, 3, 5), coarse_tol=0.5):
    """u = H \\ b by FGMRES + ML_GMRES, as linearsolve with SOLVE_FGMRES and PREC_MLGMRES
    (h3d_mlgmres_solve: the Arnoldi steps, Givens rotations and stopping tests on the device).

    precision "fp64": everything in complex128 (the reference's arithmetic).  "mixed": the
    outer FGMRES (its matvecs, Krylov basis and stopping test) stays complex128 and the
    V-cycle runs in complex64 -- FGMRES allows a preconditioner that changes between
    applications, so the inexact single-precision cycle only affects the iteration count.
    precond "none": plain restarted FGMRES on level 0 (GMRES(maxinnerit)).  k: ML_GMRES.m's
    opts.k (smoother cycles and steps, coarse-solver cycles and steps).
    Returns (u, info) with the outer iteration count and the quasi-residual history."""
    if precision not in ("fp64", "mixed"):
        raise ValueError(f"precision must be 'fp64' or 'mixed', not {precision!r}")
    if precond not in ("mlgmres", "none"):
        raise ValueError(f"precond must be 'mlgmres' or 'none', not {precond!r}")
    lib = L.load()
    b = b.to(torch.complex128).contiguous()
    u = torch.zeros_like(b) if x0 is None else x0.to(torch.complex128).clone().contiguous()
    lv, Rs, Ps = _level_structs(levels, R, P)
    o = L.MLOpts()
    lib.h3d_ml_default_opts(C.byref(o))
    o.tol = float(tol)
    o.maxit = int(min(maxit, 2 ** 31 - 1))
    o.maxinnerit = int(maxinnerit)
    o.precond = L.ML_PREC_MLGMRES if precond == "mlgmres" else L.ML_PREC_NONE
    o.precision = L.PREC_FP64 if precision == "fp64" else L.PREC_MIXED
    for i in range(4):
        o.k[i] = int(k[i])
    o.coarse_tol = float(coarse_tol)
    hst = np.zeros(1 + o.maxit * o.maxinnerit)
    info = L.MLInfo()
    st = torch.cuda.current_stream(b.device).cuda_stream
    rc = lib.h3d_mlgmres_solve(lv, len(levels), Rs, Ps, C.c_void_p(b.data_ptr()), C.c_void_p(u.data_ptr()),
                               ops._mode(mode), C.byref(o), hst.ctypes.data_as(L.dp), int(hst.size),
                               C.byref(info), C.c_void_p(st))
    L.check(rc, "h3d_mlgmres_solve")
    d = info.as_dict()
    d["hst"] = hst[: info.iters + 1].tolist()
    return u, d


def solve_model(v_phys, dt, npml, freq, b: torch.Tensor, unit="m/s", nlevels=3, tol=1e-6, maxit=10000,
                maxinnerit=5, mode=1, precision="fp64", k=(3, 5, 3, 5), coarse_tol=0.5):
    """The same solve with the hierarchy built by the library from the physical model
    (h3d_mlgmres_solve_model: construct_multigrid.m in C++, one call).  v_phys: (nx, ny, nz)
    array; b on the level-0 PML grid."""
    if precision not in ("fp64", "mixed"):
        raise ValueError(f"precision must be 'fp64' or 'mixed', not {precision!r}")
    lib = L.load()
    v = np.asarray(v_phys, float)
    src = np.ascontiguousarray(v.reshape(-1, order="F"))
    n = (C.c_int32 * 3)(*v.shape)
    h = np.ascontiguousarray(np.broadcast_to(np.asarray(dt, float), (3,)))
    b = b.to(torch.complex128).contiguous()
    u = torch.zeros_like(b)
    o = L.MLOpts()
    lib.h3d_ml_default_opts(C.byref(o))
    o.tol = float(tol)
    o.maxit = int(min(maxit, 2 ** 31 - 1))
    o.maxinnerit = int(maxinnerit)
    o.precision = L.PREC_FP64 if precision == "fp64" else L.PREC_MIXED
    for i in range(4):
        o.k[i] = int(k[i])
    o.coarse_tol = float(coarse_tol)
    hst = np.zeros(1 + o.maxit * o.maxinnerit)
    info = L.MLInfo()
    st = torch.cuda.current_stream(b.device).cuda_stream
    rc = lib.h3d_mlgmres_solve_model(src.ctypes.data_as(L.dp), n, h.ctypes.data_as(L.dp), int(npml), float(freq),
                                     L.UNITS[unit], int(nlevels), C.c_void_p(b.data_ptr()), C.c_void_p(u.data_ptr()),
                                     ops._mode(mode), C.byref(o), hst.ctypes.data_as(L.dp), int(hst.size),
                                     C.byref(info), C.c_void_p(st))
    L.check(rc, "h3d_mlgmres_solve_model")
    d = info.as_dict()
    d["hst"] = hst[: info.iters + 1].tolist()
    return u, d
