"""numpy restatement of FGMRES and the ML_GMRES multigrid preconditioner (TEST INFRASTRUCTURE).

The default solver of the reference's 3D applications (fwi_exp.m:58-62: FGMRES, tol 1e-6,
restart 5, preconditioner LinSolveOpts.PREC_MLGMRES).  Operators are the C oracle's
matvecs; everything above them follows these reference files (paths inside
SLIM-release-apps):

  FGMRES      tools/solvers/Krylov/FGMRES.m
  linearsolve tools/solvers/Krylov/linearsolve.m
  ML_GMRES    tools/solvers/Multigrid/ML_GMRES.m
  construct   tools/solvers/Multigrid/construct_multigrid.m
  opMG        tools/solvers/Multigrid/opMultigrid.m
  GMG_V       tools/solvers/Multigrid/GMG_V.m
  f2c         tools/functions/misc/fine2coarse.m
  lin1d       tools/functions/misc/LinInterp1D.m, nearestnbr1d.m
  cub1d       tools/operators/misc/opLInterp1D.m (getLA)
  dh          tools/algorithms/CommonFreqModeling/discrete_helmholtz.m

Only tests/ use this module.
"""
from __future__ import annotations

import math

import numpy as np
import scipy.sparse as sp

from . import h3d_oracle as O
from . import slim_ref


# ---- 1D interpolation matrices -------------------------------------------------------------
def nearest_neighbour_1d(xin, xout):
    """nearestnbr1d.m: index (0-based) of the input node nearest to each output node,
    ties to the lower one; both grids ascending."""
    xin = np.asarray(xin, float)
    xout = np.asarray(xout, float)
    I = np.zeros(len(xout), dtype=np.int64)
    istart = 0
    xend = xin[1] if len(xin) > 1 else np.inf
    for i, xo in enumerate(xout):
        while xo > xend:
            istart += 1
            xend = np.inf if istart == len(xin) - 1 else xin[istart + 1]
        I[i] = istart if abs(xo - xin[istart]) <= abs(xo - xend) else istart + 1
    return I


def lin_interp_1d(xin, xout):
    """LinInterp1D.m:1-25: sparse (len(xout) x len(xin)) linear interpolation."""
    xin = np.sort(np.asarray(xin, float))
    xout = np.sort(np.asarray(xout, float))
    nin, nout = len(xin), len(xout)
    I = nearest_neighbour_1d(xin, xout)
    I = np.where(xin[I] > xout, I - 1, I)                           # :19
    xe = np.concatenate([xin, [1e12]])                               # :20
    b = (xout - xe[I]) / (xe[I + 1] - xe[I])                          # :21
    a = (xe[I + 1] - xout) / (xe[I + 1] - xe[I])                      # :22
    rows = np.arange(nout)
    A = sp.csr_matrix((a, (rows, I)), shape=(nout, nin))
    A = A + sp.csr_matrix((b, (rows, np.minimum(I + 1, nin - 1))), shape=(nout, nin))
    return A.tocsr()


def cubic_interp_1d(x1, x2):
    """opLInterp1D.m getLA: 4-point Lagrange interpolation from nodes x1 to points x2
    (rows of points outside [x1[0], x1[-1]] are zero)."""
    x1 = np.asarray(x1, float)
    x2 = np.asarray(x2, float)
    n1, n2 = len(x1), len(x2)
    ik = np.nonzero((x2 >= x1[0]) & (x2 <= x1[-1]))[0]
    rows, cols, vals = [], [], []
    a, b, c, d = 0, 1, 2, 3                                           # 1-based 1,2,3,4
    for k in ik:
        if x2[k] < x1[b]:
            while x2[k] < x1[b] and b - 1 > 0:
                b -= 1
            a, c, d = b - 1, b + 1, b + 2
        elif x2[k] > x1[c]:
            while x2[k] > x1[c] and c + 1 < n1 - 1:
                c += 1
            a, b, d = c - 2, c - 1, c + 1
        X = x2[k]
        for j, (p, q1, q2, q3) in enumerate(((a, b, c, d), (b, a, c, d), (c, b, a, d), (d, b, c, a))):
            num = (X - x1[q1]) * (X - x1[q2]) * (X - x1[q3])
            den = (x1[p] - x1[q1]) * (x1[p] - x1[q2]) * (x1[p] - x1[q3])
            rows.append(k)
            cols.append(p)
            vals.append(num / den)
    return sp.csr_matrix((vals, (rows, cols)), shape=(n2, n1))


# ---- separable 3D operators on column-major (x fastest) vectors -----------------------------
class Sep3:
    """opKron(A3, A2, A1) (f2c.m:44-55): A1 along x, A2 along y, A3 along z."""

    def __init__(self, A1, A2, A3):
        self.A = (A1, A2, A3)
        self.n_in = tuple(a.shape[1] for a in self.A)
        self.n_out = tuple(a.shape[0] for a in self.A)

    def T(self):
        return Sep3(*(a.T.tocsr() for a in self.A))

    def __mul__(self, x):
        x = np.asarray(x)
        nx, ny, nz = self.n_in
        t = x.reshape(nz, ny, nx)                                    # [k, j, i]
        t = np.einsum("ai,kji->kja", self.A[0].toarray(), t)
        t = np.einsum("bj,kja->kba", self.A[1].toarray(), t)
        t = np.einsum("ck,kba->cba", self.A[2].toarray(), t)
        return t.reshape(-1)


def fine2coarse(n, d=None, d_sub=None, kind="cubic", n_sub=None):
    """fine2coarse.m: (f2c, c2f, n_sub) for 3D grids.  Either d, d_sub (n_sub = ceil(n d /
    d_sub)) or n_sub directly; kind 'cubic' (opLInterp1D) or 'linear' (LinInterp1D, f2c is
    then c2f')."""
    n = np.asarray(n, int)
    if n_sub is None:
        n_sub = np.ceil(n * np.asarray(d, float) / np.asarray(d_sub, float) - 1e-12).astype(int)
    n_sub = np.asarray(n_sub, int)
    basis = cubic_interp_1d if kind == "cubic" else lin_interp_1d
    grid = lambda m: np.linspace(0.0, 1.0, int(m))
    c2f = Sep3(*(basis(grid(n_sub[a]), grid(n[a])) for a in range(3)))
    f2c = c2f.T() if kind == "linear" else Sep3(*(basis(grid(n[a]), grid(n_sub[a])) for a in range(3)))
    return f2c, c2f, tuple(int(v) for v in n_sub)


# ---- levels --------------------------------------------------------------------------------
class Level:
    """One discretisation: grid (with PML), wavenumber, matvec."""

    def __init__(self, v_phys, dt, npml, freq, unit):
        self.v_phys = np.asarray(v_phys, float)
        self.dt = tuple(float(x) for x in dt)
        self.npml = int(npml)
        n = self.v_phys.shape
        self.nt = tuple(int(n[a] + 2 * self.npml) for a in range(3))    # dh:203-211
        vpml = slim_ref.extend3d(self.v_phys, (self.npml,) * 6, mode=1)  # dh:240
        self.wn = slim_ref.param2wavenum(vpml.reshape(-1, order="F"), freq, unit)[0]
        self.g = O.make_grid(self.nt, self.dt, self.npml)

    @property
    def N(self):
        return int(np.prod(self.nt))

    def A(self, x, mode=1):
        return O.mvp(self.g, self.wn, x, adj=(mode != 1), nthreads=1)


def build_levels(v_phys, dt, npml, freq, unit, nlevels=3):
    """construct_multigrid.m:10-60 with coarse_factor 2: level i+1 coarsens the physical
    model of level i by cubic interpolation to ceil(n / 2) points (spacing 2^i dt) with
    ceil(pml / 2^i) PML points; restriction (1/8) c2f' and prolongation c2f are the linear
    interpolations between the computational grids (PML included)."""
    levels = [Level(v_phys, dt, npml, freq, unit)]
    R, P = [], []
    v = np.asarray(v_phys, float)
    for i in range(1, nlevels):
        dti = np.asarray(dt, float) * 2 ** i                           # :27
        pml_i = math.ceil(npml / 2 ** i)                               # :29
        to_coarse, _, n_c = fine2coarse(v.shape, dti / 2, dti, "cubic")  # :39
        vc = (to_coarse * v.reshape(-1, order="F")).reshape(n_c, order="F")
        lv = Level(vc, dti, pml_i, freq, unit)                          # :42
        f2c, c2f, _ = fine2coarse(levels[-1].nt, kind="linear", n_sub=lv.nt)  # :45
        R.append((f2c, 1.0 / 8.0))                                      # :48 weighted restriction
        P.append(c2f)                                                   # :51
        levels.append(lv)
        v = vc
    return levels, R, P


# ---- FGMRES.m:27-129 -----------------------------------------------------------------------
def fgmres(A, b, x, tol=1e-6, maxit=np.inf, maxinnerit=10, precond=None):
    """Flexible GMRES with restarts every maxinnerit steps.  A, precond: callables on
    vectors (precond None = identity, the opDirac branch).  Returns (x, res, hst)."""
    b = np.asarray(b, complex)
    x = np.zeros_like(b) if x is None else np.asarray(x, complex).copy()
    if np.count_nonzero(x):                                            # :58-63
        r = b - A(x)
    else:
        r = b.copy()
        x = np.zeros_like(b)
    it = 1                                                              # :66
    normr0 = np.linalg.norm(r)
    hst = [1.0]
    res = []
    m = maxinnerit
    while hst[-1] > tol and math.floor(it / m) < maxit:                # :83
        beta = np.linalg.norm(r)
        V = np.zeros((b.size, m), complex)
        Z = [] if precond is None else np.zeros((b.size, m), complex)
        H = np.zeros((m + 1, m), complex)
        y = np.zeros(m, complex)
        V[:, 0] = r / beta
        k = 1
        while k <= m and hst[-1] > tol:                                 # :88
            if precond is None:
                w = A(V[:, k - 1])
            else:
                Z[:, k - 1] = precond(V[:, k - 1])
                w = A(Z[:, k - 1])
            H[:k, k - 1] = V[:, :k].conj().T @ w                        # :97
            w = w - V[:, :k] @ H[:k, k - 1]
            H[k, k - 1] = np.linalg.norm(w)
            if k < m:
                V[:, k] = w / H[k, k - 1]
            e = np.zeros(k + 1, complex)
            e[0] = beta
            y[:k] = np.linalg.lstsq(H[:k + 1, :k], e, rcond=None)[0]   # :106
            hst.append(float(np.linalg.norm(e - H[:k + 1, :k] @ y[:k]) / normr0))
            k += 1
            it += 1
        if precond is None:                                             # :114-118
            x = x + V[:, :k - 1] @ y[:k - 1]
        else:
            x = x + Z[:, :k - 1] @ y[:k - 1]
        r = b - A(x)                                                    # :119
        if np.linalg.norm(r) / normr0 < tol:                            # :124
            break
        res.append(float(np.linalg.norm(r)))
    return x, np.array(res), np.array(hst)


# ---- ML_GMRES.m:36-72, opMultigrid.m recursive V-cycle, GMG_V.m ------------------------------
SMOOTH = dict(tol=1e-6, maxit=3, maxinnerit=5)       # ML_GMRES.m:38-39,53-58 (ks_outer 3, ks_inner 5)
COARSE = dict(tol=5e-1, maxit=3, maxinnerit=5)       # ML_GMRES.m:40-42,60-65 (coarsetol 0.5)


class MLGMRES:
    """The three-level recursive V-cycle preconditioner (opMultigrid with recursive_v_cycle)."""

    def __init__(self, levels, R, P):
        self.L, self.R, self.P = levels, R, P

    def smooth(self, i, b, x, mode):
        """LinearSolver(H_i, smoother): FGMRES, identity preconditioner, 3 x 5 steps."""
        return fgmres(lambda v: self.L[i].A(v, mode), b, x, **SMOOTH)[0]

    def coarse_solve(self, i, b, mode):
        """The coarse solve of level i-1's cycle: FGMRES on level i preconditioned by the
        V-cycle of level i (or, on the last level, by an unpreconditioned FGMRES)."""
        if i == len(self.L) - 1:
            pre = lambda v: fgmres(lambda u: self.L[i].A(u, mode), v, None, **COARSE)[0]
        else:
            pre = lambda v: self.vcycle(i, v, mode)
        return fgmres(lambda u: self.L[i].A(u, mode), b, None, precond=pre, **COARSE)[0]

    def vcycle(self, i, b, mode):
        """GMG_V.m:10-40 on level i with x0 = 0 and maxit 1."""
        x = self.smooth(i, b, None, mode)                               # :29
        r = b - self.L[i].A(x, mode)                                    # :30
        f2c, c = self.R[i]
        xc = c * (f2c * r)                                              # :31
        xc = self.coarse_solve(i + 1, xc, mode)                         # :32
        x = x + self.P[i] * xc                                          # :33
        return self.smooth(i, b, x, mode)                               # :34

    def __call__(self, b, mode=1):
        return self.vcycle(0, b, mode)


def ml_gmres_solve(levels, R, P, b, tol=1e-6, maxit=10000, maxinnerit=5, mode=1):
    """linearsolve(H, b, 0, mode, FGMRES + PREC_MLGMRES) as fwi_exp.m:58-62 configures it."""
    T = MLGMRES(levels, R, P)
    L0 = levels[0]
    return fgmres(lambda v: L0.A(v, mode), b, None, tol=tol, maxit=maxit, maxinnerit=maxinnerit,
                  precond=lambda v: T(v, mode))
