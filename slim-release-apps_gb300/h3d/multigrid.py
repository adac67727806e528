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

Matrix-vector products are the library's 27-point kernels (h3d_mvp), the grid transfers
its axis kernel (h3d_axis_apply); vectors live on the device, the small Hessenberg
least-squares problems on the host.  Model coarsening and interpolation weights are set-up
work on the host.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np
import torch

from . import _lib as L
from . import ops


# ---- interpolation weights (host) -------------------------------------------------------------
def _nearest(xin, xout):
    """Index of the nearest input node per output node, ties to the lower node
    (nearestnbr1d.m); both grids ascending."""
    idx = np.searchsorted(xin, xout, side="left")
    lo = np.clip(idx - 1, 0, len(xin) - 1)
    hi = np.clip(idx, 0, len(xin) - 1)
    return np.where(np.abs(xout - xin[lo]) <= np.abs(xout - xin[hi]), lo, hi)


def linear_weights(xin, xout):
    """LinInterp1D.m: CSR (rowptr, col, val) of the len(xout) x len(xin) linear interpolation."""
    xin = np.sort(np.asarray(xin, float))
    xout = np.sort(np.asarray(xout, float))
    nin, nout = len(xin), len(xout)
    I = _nearest(xin, xout)
    I = np.where(xin[I] > xout, I - 1, I)
    nxt = np.where(I + 1 < nin, xin[np.minimum(I + 1, nin - 1)], 1e12)
    wb = (xout - xin[I]) / (nxt - xin[I])
    wa = (nxt - xout) / (nxt - xin[I])
    dense = np.zeros((nout, nin))
    np.add.at(dense, (np.arange(nout), I), wa)
    np.add.at(dense, (np.arange(nout), np.minimum(I + 1, nin - 1)), wb)
    return dense


def cubic_weights(x1, x2):
    """opLInterp1D.m getLA: len(x2) x len(x1) 4-point Lagrange interpolation (zero rows
    for points outside the node range); the node window slides monotonically as there."""
    x1 = np.asarray(x1, float)
    x2 = np.asarray(x2, float)
    n1 = len(x1)
    A = np.zeros((len(x2), n1))
    b, c = 1, 2
    for k in np.nonzero((x2 >= x1[0]) & (x2 <= x1[-1]))[0]:
        X = x2[k]
        if X < x1[b]:
            while X < x1[b] and b > 1:
                b -= 1
            c = b + 1
        elif X > x1[c]:
            while X > x1[c] and c < n1 - 2:
                c += 1
            b = c - 1
        nodes = (b - 1, b, c, c + 1)
        for p in nodes:
            others = [q for q in nodes if q != p]
            A[k, p] += np.prod([X - x1[q] for q in others]) / np.prod([x1[p] - x1[q] for q in others])
    return A


def _coarsen_model(v, n_sub):
    """Physical model on ceil(n/2) points per axis by separable cubic interpolation."""
    g = lambda m: np.linspace(0.0, 1.0, int(m))
    Ax, Ay, Az = (cubic_weights(g(v.shape[a]), g(n_sub[a])) for a in range(3))
    t = np.tensordot(Ax, v, axes=(1, 0))                        # (a, j, k)
    t = np.tensordot(Ay, t, axes=(1, 1)).transpose(1, 0, 2)     # (a, b, k)
    return np.tensordot(t, Az, axes=(2, 1))                     # (a, b, c)


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


# ---- FGMRES.m --------------------------------------------------------------------------------
def fgmres(A, b: torch.Tensor, x: torch.Tensor | None, tol=1e-6, maxit=math.inf, maxinnerit=10,
           precond=None):
    """Flexible GMRES restarted every maxinnerit steps (FGMRES.m:27-129).  Returns
    (x, res, hst): the solution, true residual norms after each restart and the relative
    quasi-residual history."""
    if x is None or not bool(torch.any(x != 0)):
        r = b.clone()
        x = torch.zeros_like(b)
    else:
        r = b - A(x)
    it = 1
    normr0 = float(torch.linalg.vector_norm(r))
    hst, res = [1.0], []
    m = maxinnerit
    if normr0 == 0.0:
        return x, res, hst
    while hst[-1] > tol and math.floor(it / m) < maxit:
        beta = float(torch.linalg.vector_norm(r))
        V = torch.empty((m, b.numel()), dtype=b.dtype, device=b.device)
        Z = None if precond is None else torch.empty_like(V)
        H = np.zeros((m + 1, m), complex)
        y = np.zeros(m, complex)
        V[0] = r / beta
        k = 1
        while k <= m and hst[-1] > tol:
            if precond is None:
                w = A(V[k - 1])
            else:
                Z[k - 1] = precond(V[k - 1])
                w = A(Z[k - 1])
            h = torch.mv(V[:k].conj(), w)                   # V(:,1:k)' w
            w = w - torch.mv(V[:k].T, h)
            hn = torch.linalg.vector_norm(w)
            hh = torch.cat([h, hn.to(h.dtype).reshape(1)]).cpu().numpy()
            H[:k, k - 1] = hh[:k]
            H[k, k - 1] = hh[k]
            if k < m:
                V[k] = w / hn
            e = np.zeros(k + 1, complex)
            e[0] = beta
            y[:k] = np.linalg.lstsq(H[:k + 1, :k], e, rcond=None)[0]
            hst.append(float(np.linalg.norm(e - H[:k + 1, :k] @ y[:k]) / normr0))
            k += 1
            it += 1
        yk = torch.as_tensor(y[:k - 1], device=b.device, dtype=b.dtype)
        x = x + torch.mv((V if precond is None else Z)[:k - 1].T, yk)
        r = b - A(x)
        rn = float(torch.linalg.vector_norm(r))
        if rn / normr0 < tol:
            break
        res.append(rn)
    return x, res, hst


SMOOTH = dict(tol=1e-6, maxit=3, maxinnerit=5)
COARSE = dict(tol=5e-1, maxit=3, maxinnerit=5)


class MLGMRES:
    """The recursive three-level V-cycle (opMultigrid with recursive_v_cycle)."""

    def __init__(self, levels, R, P):
        self.L, self.R, self.P = levels, R, P

    def _smooth(self, i, b, x, mode):
        return fgmres(lambda v: self.L[i].A(v, mode), b, x, **SMOOTH)[0]

    def _coarse(self, i, b, mode):
        Ai = lambda u: self.L[i].A(u, mode)
        if i == len(self.L) - 1:
            pre = lambda v: fgmres(Ai, v, None, **COARSE)[0]
        else:
            pre = lambda v: self.vcycle(i, v, mode)
        return fgmres(Ai, b, None, precond=pre, **COARSE)[0]

    def vcycle(self, i, b, mode=1):
        x = self._smooth(i, b, None, mode)
        r = b - self.L[i].A(x, mode)
        xc = self._coarse(i + 1, self.R[i](r), mode)
        x = x + self.P[i](xc)
        return self._smooth(i, b, x, mode)

    def __call__(self, b, mode=1):
        return self.vcycle(0, b, mode)


def solve(levels, R, P, b: torch.Tensor, tol=1e-6, maxit=10000, maxinnerit=5, mode=1, precision="fp64"):
    """u = H \\ b by FGMRES + ML_GMRES, as linearsolve with SOLVE_FGMRES and PREC_MLGMRES.

    precision "fp64": everything in complex128 (the reference's arithmetic).  "mixed": the
    outer FGMRES (its matvecs, Krylov basis and stopping test) stays complex128 and the
    V-cycle runs in complex64 -- FGMRES allows a preconditioner that changes between
    applications, so the inexact single-precision cycle only affects the iteration count.
    Returns (u, info) with the outer iteration count and the quasi-residual history."""
    T = MLGMRES(levels, R, P)
    A0 = lambda v: levels[0].A(v, mode)
    if precision == "fp64":
        pre = lambda v: T(v, mode)
    elif precision == "mixed":
        pre = lambda v: T(v.to(torch.complex64), mode).to(torch.complex128)
    else:
        raise ValueError(f"precision must be 'fp64' or 'mixed', not {precision!r}")
    u, res, hst = fgmres(A0, b.to(torch.complex128), None, tol=tol, maxit=maxit, maxinnerit=maxinnerit,
                         precond=pre)
    return u, {"iters": len(hst) - 1, "hst": hst, "res": res}
