"""Adjoint-state FWI objective and gradient on the GPU (the PDEfunc OBJ / FORW_MODEL path).

Mirrors ``[f,g] = PDEfunc(PDEopts.OBJ, v, Q, [], Dobs, model, params)`` and
``D = PDEfunc(PDEopts.FORW_MODEL, ...)`` for 3D grids
(tools/algorithms/CommonFreqModeling/PDEfunc.m:254-394):

  per frequency k:  wn, dwn = param2wavenum(Pext v, f_k, unit)          (discrete_helmholtz.m:240-257)
  per source s:     q   = Ps (w(f_k) Q_s) prod(d)/prod(dt)               (PDEfunc.m:330-339)
                    U   = H \\ q                                          (PDEfunc.m:347)
                    phi, dphi = LS_misfit(Pr U, D_obs)                    (PDEfunc.m:389, LS_misfit.m:23-25)
                    V   = H' \\ (-Pr' dphi)                               (PDEfunc.m:393)
                    g  += crop( Re(conj(U) .* (dH' V)) )                  (PDEfunc.m:394, discrete_helmholtz.m:288)

The sources of one frequency are right-hand sides of one problem, and (CGMN solver, wavefields
within the HBM budget) the problems of all frequencies are solved as one batch
(h3d_solve_batch: every sweep launch covers all frequencies); the gradient accumulation over
a source batch is one fused kernel (h3d_grad_accum).  Forward wavefields are kept for the
gradient while they fit an HBM budget and recomputed otherwise.  Everything runs through
libh3d.so's C ABI.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib as L
from . import solver as S


def param2wavenum(v: torch.Tensor, freq: float, unit: str):
    """(wn, dwn) = ((2 pi f)^2 * m, derivative) as in param2wavenum.m:20-49."""
    c = (2.0 * np.pi * freq) ** 2
    if unit == "m/s":
        return c * v.pow(-2), -2.0 * c * v.pow(-3)
    if unit == "s2/m2":
        return c * v, torch.full_like(v, c)
    if unit == "s2/km2":
        return 1e-6 * c * v, torch.full_like(v, 1e-6 * c)
    raise ValueError(f"Unknown unit - {unit}")


def extend_edges(v: torch.Tensor, npml6) -> torch.Tensor:
    """opExtension mode 1 in 3D (edge replication), v indexed (x, y, z)."""
    lx, hx, ly, hy, lz, hz = (int(p) for p in npml6)
    t = v.permute(2, 1, 0)[None, None]                         # (1,1,z,y,x)
    t = torch.nn.functional.pad(t, (lx, hx, ly, hy, lz, hz), mode="replicate")
    return t[0, 0].permute(2, 1, 0).contiguous()


def fwi_wavelet(freqs, t0: float, f0: float):
    f = np.asarray(freqs, dtype=np.float64)
    w = np.exp(-1j * 2 * np.pi * f * t0)
    if f0:
        w = f ** 2 * np.exp(-(f / f0) ** 2) * w
    return w


def _flat(v3: torch.Tensor) -> torch.Tensor:
    """(x,y,z) array -> x-fastest flat vector (column-major, the reference layout)."""
    return v3.permute(2, 1, 0).contiguous().reshape(-1)


def _unflat(v: torch.Tensor, n) -> torch.Tensor:
    return v.reshape(n[2], n[1], n[0]).permute(2, 1, 0)


@dataclass
class Geometry:
    """Physical grid and acquisition: origin o, spacing d (m), interior size n, PML widths."""
    o: tuple
    d: tuple
    n: tuple
    npml6: tuple
    src_xyz: np.ndarray             # (nsrc, 3) physical coordinates (m)
    rec_xyz: np.ndarray             # (nrec, 3)
    freqs: np.ndarray
    f0: float = 8.0
    t0: float = 0.0
    unit: str = "m/s"
    src_amp: np.ndarray | None = None   # per-source complex amplitude (Q); ones by default

    @property
    def dt(self):
        """Spacing of the computational grid: params.dt, which PDEfunc.m:88 sets to model.d
        (a Helmholtz grid coarser or finer than the model, pdefunopts.helm_dt, is not built)."""
        return tuple(float(x) for x in self.d)

    @property
    def n_total(self):
        p = self.npml6
        return (self.n[0] + p[0] + p[1], self.n[1] + p[2] + p[3], self.n[2] + p[4] + p[5])

    def grid(self) -> L.Grid:
        return L.make_grid(self.n_total, self.d, self.npml6)

    def to_index(self, xyz: np.ndarray) -> np.ndarray:
        """Physical coordinates -> computational-grid index units (ot = o - npml_lo d)."""
        xyz = np.asarray(xyz, dtype=np.float64).reshape(-1, 3)
        ot = np.array([self.o[a] - self.npml6[2 * a] * self.d[a] for a in range(3)])
        return (xyz - ot) / np.asarray(self.d, dtype=np.float64)


class _Interp:
    """Device-resident separable sinc-Kaiser weights of a point set (h3d_sinc_weights)."""

    def __init__(self, g: L.Grid, pts_idx: np.ndarray, dev):
        n = pts_idx.shape[0]
        base = np.zeros((n, 3), np.int32)
        w = np.zeros((n, 3, 9))
        pts = np.ascontiguousarray(pts_idx, dtype=np.float64)
        rc = L.load().h3d_sinc_weights(C.byref(g), pts.ctypes.data_as(C.POINTER(C.c_double)), n,
                                       base.ctypes.data_as(C.POINTER(C.c_int32)),
                                       w.ctypes.data_as(C.POINTER(C.c_double)))
        L.check(rc, "h3d_sinc_weights")
        self.n = n
        self.base = torch.as_tensor(base, device=dev)
        self.w = torch.as_tensor(w, device=dev)


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


@dataclass
class FWIConfig:
    tol: float = 1e-6
    maxit: int = 10000
    precision: str = "mixed"
    order: str = "block8"
    hbm_budget_bytes: float = 40e9        # keep forward wavefields up to this size
    src_batch: int = 0                    # 0 = all sources of a frequency in one batch
    extra: dict = field(default_factory=dict)
    # "cgmn": the Kaczmarz-preconditioned CGMN solver (batched over sources);
    # "mlgmres": FGMRES + ML_GMRES multigrid (h3d.multigrid), one source at a time --
    # the reference's default for its 3D applications (fwi_exp.m:58-62).  Needs the same
    # PML width on all six faces.
    solver: str = "cgmn"


class FWIProblem:
    """PDEfunc-style forward modelling, objective and gradient on one GPU."""

    def __init__(self, geom: Geometry, cfg: FWIConfig | None = None, device="cuda:0"):
        self.geom = geom
        self.cfg = cfg or FWIConfig()
        self.dev = torch.device(device)
        self.g = geom.grid()
        self.N = int(np.prod(geom.n_total))
        self.src = _Interp(self.g, geom.to_index(geom.src_xyz), self.dev)
        self.rec = _Interp(self.g, geom.to_index(geom.rec_xyz), self.dev)
        self.nsrc, self.nrec = self.src.n, self.rec.n
        amp = geom.src_amp if geom.src_amp is not None else np.ones(self.nsrc)
        self.src_amp = np.asarray(amp, dtype=np.complex128)
        self.wavelet = fwi_wavelet(geom.freqs, geom.t0, geom.f0)
        self.last_infos: list = []

    # -- pieces -------------------------------------------------------------------------------
    def _opts(self):
        c = self.cfg
        return S.make_opts(tol=c.tol, maxit=c.maxit, precision=c.precision, order=c.order, **c.extra)

    def _wavenumbers(self, v_phys: torch.Tensor, freq: float):
        v = extend_edges(v_phys.to(self.dev, torch.float64), self.geom.npml6)
        wn, dwn = param2wavenum(v, freq, self.geom.unit)
        return _flat(wn), _flat(dwn)

    def _sources(self, k: int, srcs) -> torch.Tensor:
        """Q_k for the listed sources: (len(srcs), N) complex128."""
        ns = len(srcs)
        b = torch.zeros(ns, self.N, dtype=torch.complex128, device=self.dev)
        # PDEfunc.m:339: wavefield amplitudes independent of the grid spacing
        scale = self.wavelet[k] * self.src_amp[srcs] * (np.prod(self.geom.d) / np.prod(self.geom.dt))
        sc = torch.as_tensor(np.stack([scale.real, scale.imag], 1), device=self.dev).contiguous()
        base = self.src.base[srcs].contiguous()
        w = self.src.w[srcs].contiguous()
        rc = L.load().h3d_src_inject(C.byref(self.g), C.c_void_p(base.data_ptr()),
                                     C.c_void_p(w.data_ptr()), C.c_void_p(sc.data_ptr()),
                                     C.c_void_p(b.data_ptr()), ns, _stream())
        L.check(rc, "h3d_src_inject")
        return b

    def _sample(self, U: torch.Tensor) -> torch.Tensor:
        P = U.shape[0]
        d = torch.empty(P, self.nrec, dtype=torch.complex128, device=self.dev)
        rc = L.load().h3d_rec_sample(C.byref(self.g), C.c_void_p(self.rec.base.data_ptr()),
                                     C.c_void_p(self.rec.w.data_ptr()), self.nrec,
                                     C.c_void_p(U.data_ptr()), P, C.c_void_p(d.data_ptr()), _stream())
        L.check(rc, "h3d_rec_sample")
        return d

    def _spread(self, D: torch.Tensor, scale: float) -> torch.Tensor:
        P = D.shape[0]
        D = D.contiguous()
        b = torch.empty(P, self.N, dtype=torch.complex128, device=self.dev)
        rc = L.load().h3d_rec_spread(C.byref(self.g), C.c_void_p(self.rec.base.data_ptr()),
                                     C.c_void_p(self.rec.w.data_ptr()), self.nrec,
                                     C.c_void_p(D.data_ptr()), P, float(scale),
                                     C.c_void_p(b.data_ptr()), _stream())
        L.check(rc, "h3d_rec_spread")
        return b

    def _grad_accum(self, dwn, U, V, gphys: torch.Tensor, scale=1.0):
        rc = L.load().h3d_grad_accum(C.byref(self.g), C.c_void_p(dwn.data_ptr()),
                                     C.c_void_p(U.data_ptr()), C.c_void_p(V.data_ptr()), U.shape[0],
                                     float(scale), C.c_void_p(gphys.data_ptr()), _stream())
        L.check(rc, "h3d_grad_accum")

    def _batches(self):
        bs = self.cfg.src_batch or self.nsrc
        return [list(range(s, min(s + bs, self.nsrc))) for s in range(0, self.nsrc, bs)]

    def _levels(self, v_phys: torch.Tensor, freq: float):
        """Multigrid levels of one frequency (solver "mlgmres"), else None."""
        if self.cfg.solver == "cgmn":
            return None
        if self.cfg.solver != "mlgmres":
            raise ValueError(f"unknown solver {self.cfg.solver!r}")
        from . import multigrid as MG

        npml = set(int(p) for p in self.geom.npml6)
        if len(npml) != 1:
            raise ValueError("the multigrid solver needs the same PML width on all faces")
        v = v_phys.detach().to(torch.float64).cpu().numpy().reshape(self.geom.n)
        return MG.build_levels(v, self.geom.d, npml.pop(), freq, self.geom.unit, device=self.dev)

    def _solve_many(self, jobs):
        """Solve every (wn, b, mode) of ``jobs``: one batched call over all of them (the CGMN
        solver: frequencies and source batches iterate together, one sweep launch per block
        parity covering every problem); returns the solutions in order."""
        if self.cfg.solver != "cgmn" or len(jobs) == 1:
            return [self._solve(wn, b, mode) for wn, b, mode in jobs]
        probs = [S.Problem(self.g, wn, b, mode) for wn, b, mode in jobs]
        us, infos = S.solve_batch(probs, opts=self._opts())
        self.last_infos.extend(infos)
        return us

    def _solve(self, wn, b, mode, ml=None):
        if ml is None:
            u, info = S.solve(self.g, wn, b, mode=mode, opts=self._opts())
            self.last_infos.append(info)
            return u
        from . import multigrid as MG

        lv, R, P = ml
        prec = "fp64" if str(self.cfg.precision).lower().startswith("fp") else "mixed"
        out = torch.empty_like(b)
        iters = []
        for s in range(b.shape[0]):
            if float(b[s].abs().max()) == 0.0:        # opAbstractMatrix.m:118
                out[s].zero_()
                continue
            out[s], info = MG.solve(lv, R, P, b[s], tol=self.cfg.tol, maxit=self.cfg.maxit, mode=mode,
                                    precision=prec)
            iters.append(info["iters"])
        self.last_infos.append({"iters": max(iters) if iters else 0, "solver": "mlgmres"})
        return out

    # -- PDEfunc FORW_MODEL ----------------------------------------------------------------------
    def forward_model(self, v_phys: torch.Tensor, return_fields: bool = False):
        """D (nrec x nsrc*nfreq), column = src + nsrc*freq (PDEfunc.m:341,423)."""
        cols, fields = [], []
        for k, fr in enumerate(self.geom.freqs):
            wn, _ = self._wavenumbers(v_phys, float(fr))
            ml = self._levels(v_phys, float(fr))
            for srcs in self._batches():
                U = self._solve(wn, self._sources(k, srcs), 1, ml)
                cols.append(self._sample(U))
                if return_fields:
                    fields.append(U)
        D = torch.cat(cols, 0).T.contiguous()
        return (D, fields) if return_fields else D

    # -- PDEfunc OBJ -----------------------------------------------------------------------------
    def wavefield_bytes(self) -> float:
        return 16.0 * self.N * self.nsrc * len(self.geom.freqs)

    def _units(self):
        """(frequency index, source list) of every batch, in the reference's column order."""
        return [(k, srcs) for k in range(len(self.geom.freqs)) for srcs in self._batches()]

    def misfit_forward(self, v_phys: torch.Tensor, Dobs: torch.Tensor, keep: bool):
        """f and the data residuals; keeps the forward wavefields when ``keep``.  With the CGMN
        solver and the wavefields kept, every frequency's forward solves run as one batch."""
        f = 0.0
        resid, fields = [], []
        units = self._units()
        if keep and self.cfg.solver == "cgmn":
            wns = [self._wavenumbers(v_phys, float(fr))[0] for fr in self.geom.freqs]
            Us = self._solve_many([(wns[k], self._sources(k, srcs), 1) for k, srcs in units])
        else:
            Us = None
        col = 0
        for q, (k, srcs) in enumerate(units):
            if Us is not None:
                U = Us[q]
            else:
                fr = float(self.geom.freqs[k])
                wn, _ = self._wavenumbers(v_phys, fr)
                U = self._solve(wn, self._sources(k, srcs), 1, self._levels(v_phys, fr))
            dpred = self._sample(U)
            dobs = Dobs[:, col:col + len(srcs)].T.to(torch.complex128)
            r = dpred - dobs                                     # LS_misfit.m:23
            f += 0.5 * float(torch.sum(r.real ** 2 + r.imag ** 2))   # LS_misfit.m:24
            resid.append(r)
            fields.append(U if keep else None)
            col += len(srcs)
        return f, resid, fields

    def gradient(self, v_phys: torch.Tensor, resid, fields):
        """g (physical grid, x-fastest flat) from the residuals; recomputes U where not kept.
        With the CGMN solver and the forward wavefields kept, every frequency's adjoint solves
        run as one batch."""
        n = self.geom.n
        g = torch.zeros(int(np.prod(n)), dtype=torch.float64, device=self.dev)
        units = self._units()
        if all(U is not None for U in fields) and self.cfg.solver == "cgmn":
            wd = [self._wavenumbers(v_phys, float(fr)) for fr in self.geom.freqs]
            Vs = self._solve_many([(wd[k][0], self._spread(resid[q], -1.0), 2)       # H' \ (-Pr' dphi)
                                   for q, (k, _) in enumerate(units)])
            for q, (k, _) in enumerate(units):
                self._grad_accum(wd[k][1], fields[q], Vs[q], g)
            return g
        for q, (k, srcs) in enumerate(units):
            fr = float(self.geom.freqs[k])
            wn, dwn = self._wavenumbers(v_phys, fr)
            ml = self._levels(v_phys, fr)
            U = fields[q]
            if U is None:
                U = self._solve(wn, self._sources(k, srcs), 1, ml)   # recompute above the budget
            V = self._solve(wn, self._spread(resid[q], -1.0), 2, ml)   # H' \ (-Pr' dphi)
            self._grad_accum(dwn, U, V, g)
        return g

    def objective_pairs(self, v_phys: torch.Tensor, Dobs: torch.Tensor, k: int, srcs):
        """PDEfunc OBJ restricted to the sources ``srcs`` at frequency index ``k``: (f, g) with g
        on the physical grid as a (nx, ny, nz) tensor.  Dobs holds every pair's column
        (src + nsrc * freq, PDEfunc.m:341); the (src, freq) subsets of PDEfunc_dist.m:120-164
        summed over all pairs give objective()."""
        srcs = [int(s) for s in srcs]
        fr = float(self.geom.freqs[k])
        wn, dwn = self._wavenumbers(v_phys, fr)
        ml = self._levels(v_phys, fr)
        U = self._solve(wn, self._sources(k, srcs), 1, ml)
        cols = [s + self.nsrc * k for s in srcs]
        dobs = Dobs[:, cols].T.to(self.dev, torch.complex128)
        r = self._sample(U) - dobs                                   # LS_misfit.m:23
        f = 0.5 * float(torch.sum(r.real ** 2 + r.imag ** 2))       # LS_misfit.m:24
        g = torch.zeros(int(np.prod(self.geom.n)), dtype=torch.float64, device=self.dev)
        V = self._solve(wn, self._spread(r, -1.0), 2, ml)            # H' \ (-Pr' dphi)
        self._grad_accum(dwn, U, V, g)
        return f, _unflat(g, self.geom.n)

    def objective(self, v_phys: torch.Tensor, Dobs: torch.Tensor):
        """(f, g) as PDEfunc OBJ (no 1/#pairs scaling; misfit_setup applies that)."""
        keep = self.wavefield_bytes() <= self.cfg.hbm_budget_bytes
        f, resid, fields = self.misfit_forward(v_phys, Dobs, keep)
        g = self.gradient(v_phys, resid, fields)
        return f, _unflat(g, self.geom.n)

    # -- PDEfunc JACOB_FORW / JACOB_ADJ / HESS_GN (PDEfunc.m:426-443) ------------------------------
    def _born_source(self, dwn, dm_pml, U):
        """-T(U) dm = -dH diag(dm) U with the forward derivative stencil (discrete_helmholtz.m:287)."""
        from . import ops

        return -ops.mvp(self.g, dwn, (dm_pml[None, :] * U).contiguous(), 1, deriv=True)

    def jacob_forw(self, v_phys: torch.Tensor, dm_phys: torch.Tensor) -> torch.Tensor:
        """Born data J dm: dU = H \\ (-T(U) dm), D = Pr dU (PDEfunc.m:426-429); dm is extended
        into the PML like the model (to_comp = Pext, discrete_helmholtz.m:230)."""
        dm_pml = _flat(extend_edges(dm_phys.to(self.dev, torch.float64), self.geom.npml6)).to(torch.complex128)
        cols = []
        for k, fr in enumerate(self.geom.freqs):
            wn, dwn = self._wavenumbers(v_phys, float(fr))
            for srcs in self._batches():
                U = self._solve(wn, self._sources(k, srcs), 1)
                dU = self._solve(wn, self._born_source(dwn, dm_pml, U), 1)
                cols.append(self._sample(dU))
        return torch.cat(cols, 0).T.contiguous()

    def jacob_adj(self, v_phys: torch.Tensor, dD: torch.Tensor) -> torch.Tensor:
        """Migration J' dD: V = H' \\ (-Pr' dD), g += crop(Re(conj(U) .* (dH' V))) (PDEfunc.m:431-433)."""
        g = torch.zeros(int(np.prod(self.geom.n)), dtype=torch.float64, device=self.dev)
        col = 0
        for k, fr in enumerate(self.geom.freqs):
            wn, dwn = self._wavenumbers(v_phys, float(fr))
            for srcs in self._batches():
                U = self._solve(wn, self._sources(k, srcs), 1)
                d = dD[:, col:col + len(srcs)].T.to(torch.complex128)
                V = self._solve(wn, self._spread(d, -1.0), 2)
                self._grad_accum(dwn, U, V, g)
                col += len(srcs)
        return _unflat(g, self.geom.n)

    def hess_gn(self, v_phys: torch.Tensor, dm_phys: torch.Tensor) -> torch.Tensor:
        """Gauss-Newton Hessian times dm: per (src,freq) dU = H \\ (-T(U) dm),
        dU2 = H' \\ (-Pr' Pr dU), g += crop(Re(conj(U) .* (dH' dU2))) (PDEfunc.m:438-442)."""
        dm_pml = _flat(extend_edges(dm_phys.to(self.dev, torch.float64), self.geom.npml6)).to(torch.complex128)
        g = torch.zeros(int(np.prod(self.geom.n)), dtype=torch.float64, device=self.dev)
        for k, fr in enumerate(self.geom.freqs):
            wn, dwn = self._wavenumbers(v_phys, float(fr))
            for srcs in self._batches():
                U = self._solve(wn, self._sources(k, srcs), 1)
                dU = self._solve(wn, self._born_source(dwn, dm_pml, U), 1)
                V = self._solve(wn, self._spread(self._sample(dU), -1.0), 2)
                self._grad_accum(dwn, U, V, g)
        return _unflat(g, self.geom.n)


class FWIObjective(torch.autograd.Function):
    """f(m) with the adjoint-state gradient as its backward.

    forward: forward solves + misfit (wavefields kept within the HBM budget);
    backward: adjoint solves and the fused gradient accumulation, recomputing the
    forward wavefields when they were not kept.
    """

    @staticmethod
    def forward(ctx, m: torch.Tensor, problem: FWIProblem, Dobs: torch.Tensor):
        keep = problem.wavefield_bytes() <= problem.cfg.hbm_budget_bytes
        f, resid, fields = problem.misfit_forward(m.detach(), Dobs, keep)
        ctx.problem = problem
        ctx.resid = resid
        ctx.fields = fields
        ctx.save_for_backward(m)
        return torch.tensor(f, dtype=torch.float64, device=m.device)

    @staticmethod
    def backward(ctx, gf):
        (m,) = ctx.saved_tensors
        g = ctx.problem.gradient(m.detach(), ctx.resid, ctx.fields)
        ctx.resid = ctx.fields = None
        return gf * _unflat(g, ctx.problem.geom.n).to(m.dtype), None, None


def fwi_objective(m: torch.Tensor, problem: FWIProblem, Dobs: torch.Tensor) -> torch.Tensor:
    return FWIObjective.apply(m, problem, Dobs)
