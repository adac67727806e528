"""Band-storage operator: the reference's ``mat_free = false`` path.

``BandOp`` mirrors ``opBandStorage`` (tools/algorithms/3DFreqModeling/opBandStorage.m):
a matrix held as ``ndiags`` couplings per row (``coef[i, k] = A(i, i + offsets[k])``, the
reference's ``ndiags x N`` column-major array seen row by row), with

* ``BandOp.helmholtz(grid, wn)`` -- the 27-band Helmholtz matrix of ``helmholtz_3d.m``
  (and, for the adjoint, the ``conj(Htransp(H))`` bands of ``opBandStorage.m:127-129``),
  formed on the GPU by the same coefficient rule as the matrix-free kernels;
* ``multiply`` / ``__matmul__`` -- ``Hmvp_MT_mex`` (``opBandStorage.multiply``, :254-272);
* ``kacz_sweep`` -- ``sweep_MT_mex`` (``opBandStorage.kacz_sweep``, :170-205);
* ``solve`` -- ``opBandStorage.linsolve`` with CGMN and the Kaczmarz preconditioner
  (:212-252, CGMN.m:36-94): CG on ``(I - DSWP(., 0)) u = DSWP(0, b)``.

All arithmetic runs in libh3d.so through the C ABI (h3d_band_coefs / h3d_band_mvp /
h3d_band_sweep) on the current CUDA stream; the CG recurrence of ``solve`` is torch vector
algebra in the precision of the bands.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib as L
from .ops import _cdtype, _grid, _mode, _ptr, _stream, _wn_planes


class BandOp:
    """A square band matrix on the GPU: ``coef`` (N, ndiags) complex, ``offsets`` (ndiags,)
    int64.  ``grid`` (optional) is the grid the bands couple, needed by ``kacz_sweep``."""

    def __init__(self, coef: torch.Tensor, offsets, grid=None, row_norms_sq: torch.Tensor | None = None):
        if not coef.is_cuda or not torch.is_complex(coef) or coef.dim() != 2:
            raise ValueError("coef must be a CUDA complex tensor of shape (N, ndiags)")
        self.coef = coef.contiguous()
        self.offsets = np.ascontiguousarray(np.asarray(offsets, dtype=np.int64))
        if self.offsets.shape != (self.coef.shape[1],):
            raise ValueError("one offset per band")
        self.grid = _grid(grid) if grid is not None else None
        self.N = self.coef.shape[0]
        self.dtype = self.coef.dtype
        # opBandStorage.m:139-144: squared row norms over all bands, kept for the sweeps
        self.row_norms_sq = (row_norms_sq if row_norms_sq is not None
                             else (self.coef.abs() ** 2).sum(dim=1).contiguous())

    @classmethod
    def helmholtz(cls, grid, wn: torch.Tensor, mode=1, dtype=torch.complex128) -> "BandOp":
        """The 27-band matrix of H (mode 1) or of H^H (else) for wavenumber ``wn``."""
        g = _grid(grid)
        N = g.n[0] * g.n[1] * g.n[2]
        dt, rdt = _cdtype(torch.empty(0, dtype=dtype))
        wr, wi = _wn_planes(wn.reshape(-1), rdt)
        if wr.numel() != N:
            raise ValueError("wn must have nx*ny*nz elements")
        coef = torch.empty(N, 27, dtype=dtype, device=wr.device)
        off = (C.c_int64 * 27)()
        rc = L.load().h3d_band_coefs(C.byref(g), _ptr(wr), _ptr(wi), _mode(mode), _ptr(coef), off, dt,
                                     _stream())
        L.check(rc, "h3d_band_coefs")
        return cls(coef, np.array(off[:], dtype=np.int64), grid=g)

    def _xin(self, x: torch.Tensor):
        if not x.is_cuda:
            raise ValueError("x must be a CUDA tensor")
        if x.shape[-1] != self.N:
            raise L.H3DError(L.ERR_XSIZE, "h3d_band", "x must have N elements per column",
                             "SLIM_release_apps:tools:algorithms:ThreeDFreqModeling:HMvp_MT_mex:NumElements")
        x = x.to(self.dtype).contiguous()
        P = 1 if x.dim() == 1 else int(np.prod(x.shape[:-1]))
        return x, P

    def multiply(self, x: torch.Tensor) -> torch.Tensor:
        """y = A x (``Hmvp_MT_mex``); ``x`` of shape (N,) or (P, N)."""
        x, P = self._xin(x)
        y = torch.empty_like(x)
        dt, _ = _cdtype(self.coef)
        off = self.offsets.ctypes.data_as(C.POINTER(C.c_int64))
        rc = L.load().h3d_band_mvp(_ptr(self.coef), off, self.coef.shape[1], self.N, _ptr(x), _ptr(y), P, dt,
                                   _stream())
        L.check(rc, "h3d_band_mvp")
        return y

    __matmul__ = multiply

    def kacz_sweep(self, w: float, x: torch.Tensor, b: torch.Tensor | None = None, nsweeps: int = 1) -> torch.Tensor:
        """``nsweeps`` forward + backward Kaczmarz sweeps from ``x`` (a new tensor is
        returned, as ``sweep_MT_mex`` returns a swept copy)."""
        if self.grid is None:
            raise ValueError("kacz_sweep needs the grid the bands couple")
        x, P = self._xin(x)
        x = x.clone()
        if b is not None:
            b, Pb = self._xin(b)
            if Pb != P:
                raise L.H3DError(L.ERR_BSIZE, "h3d_band_sweep", "b must have as many columns as x",
                                 "SLIM_release_apps:tools:algorithms:ThreeDFreqModeling:HMvp_MT_mex:NumElements")
        dt, rdt = _cdtype(self.coef)
        rn = self.row_norms_sq.to(rdt).contiguous()
        off = self.offsets.ctypes.data_as(C.POINTER(C.c_int64))
        for _ in range(int(nsweeps)):
            rc = L.load().h3d_band_sweep(C.byref(self.grid), _ptr(self.coef), off, _ptr(rn), float(w), _ptr(x),
                                         _ptr(b), P, dt, _stream())
            L.check(rc, "h3d_band_sweep")
        return x

    def solve(self, b: torch.Tensor, tol: float = 1e-6, maxit: int = 10000, w: float = 1.5):
        """u with A u = b by CGMN (``opBandStorage.linsolve`` with SOLVE_CGMN and
        PREC_KACZSWP, zero start; columns with ||b|| < 1e-12 give 0, :225-230).  Returns
        (u, residual history of the preconditioned system, max over columns)."""
        b, P = self._xin(b)
        B = b.reshape(P, self.N)
        u = torch.zeros_like(B)
        keep = torch.linalg.vector_norm(B, dim=1) > 1e-12
        if not bool(keep.any()):
            return u.reshape(b.shape), np.array([0.0])
        Bk = B[keep]
        bt = self.kacz_sweep(w, torch.zeros_like(Bk), Bk)                 # DSWP(0, b)

        def A(y):                                                          # I - DSWP(., 0)
            return y - self.kacz_sweep(w, y, None)

        x, hst = _cgmn(A, bt, tol, maxit)
        u[keep] = x
        return u.reshape(b.shape), hst


def _cgmn(A, b: torch.Tensor, tol: float, maxit: int):
    """CGMN.m:36-94 on the rows of ``b`` (each a column of the reference's N x P block):
    per-column alpha and beta, stop when max_j ||r_j|| / ||b_j|| <= tol or after maxit."""
    x = torch.zeros_like(b)
    r = b.clone()
    p = r.clone()
    normb = torch.linalg.vector_norm(b, dim=1)
    normr = torch.linalg.vector_norm(r, dim=1)
    hst = [float((normr / normb).max())]
    k = 0
    while True:
        Ap = A(p)
        pAp = (p.conj() * Ap).sum(dim=1)
        alpha = (normr ** 2) / pAp
        x = x + p * alpha[:, None]
        r = r - Ap * alpha[:, None]
        normr_old = normr
        normr = torch.linalg.vector_norm(r, dim=1)
        hst.append(float((normr / normb).max()))
        k += 1
        if k >= maxit or hst[-1] <= tol:
            break
        beta = (normr / normr_old) ** 2
        p = r + p * beta[:, None]
    return x, np.array(hst)
