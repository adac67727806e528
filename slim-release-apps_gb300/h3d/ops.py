"""Torch-tensor front end of the operator entry points (matvec, Kaczmarz sweep, residual).

Every function calls straight into libh3d.so through the C ABI on the current CUDA
stream; tensors must live on a CUDA device.  Right-hand sides are stacked along the
leading dimension: ``x`` has shape ``(N,)`` or ``(P, N)``, each row one column of the
reference's column-major ``N x P`` matrix (x fastest inside a row).

Mirrors ``helm3d_operto27_mvp(wn,h,nt,npml,x,n_threads,mode,deriv_mode)``
(tools/algorithms/3DFreqModeling/helm3d_operto27_mvp.m:22-42) and
``helm3d_operto27_kaczswp(wn,h,nt,npml,w,x,b,nsweeps,mode)``
(helm3d_operto27_kaczswp.m:20-30): ``mode == 1`` is the forward operator, anything
else its adjoint; a complex ``wn`` selects the complex-wavenumber kernels.
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib as L


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else C.c_void_p()


def _grid(grid):
    return grid if isinstance(grid, L.Grid) else L.make_grid(*grid)


def _mode(mode) -> int:
    if isinstance(mode, str):
        return L.FORWARD if mode.lower().startswith("f") else L.ADJOINT
    return L.FORWARD if int(mode) == 1 else L.ADJOINT


def _wn_planes(wn: torch.Tensor, real_dtype):
    if not wn.is_cuda:
        raise ValueError("wn must be a CUDA tensor")
    if torch.is_complex(wn):
        return wn.real.to(real_dtype).contiguous(), wn.imag.to(real_dtype).contiguous()
    return wn.to(real_dtype).contiguous(), None


def _cdtype(x: torch.Tensor):
    if x.dtype == torch.complex128:
        return L.C128, torch.float64
    if x.dtype == torch.complex64:
        return L.C64, torch.float32
    raise TypeError("x must be complex64 or complex128")


def _rhs(x: torch.Tensor, N: int):
    if not x.is_cuda:
        raise ValueError("x must be a CUDA tensor")
    if x.shape[-1] != N:
        raise L.H3DError(L.ERR_XSIZE, "h3d", "x must have nx*ny*nz elements",
                         "SLIM_release_apps:tools:algorithms:ThreeDFreqModeling:Helm3dkaczswp_mex:Xsize")
    P = 1 if x.dim() == 1 else int(torch.tensor(x.shape[:-1]).prod())
    return x.contiguous(), P


def grid_points(grid) -> int:
    g = _grid(grid)
    return g.n[0] * g.n[1] * g.n[2]


def mvp(grid, wn: torch.Tensor, x: torch.Tensor, mode=1, deriv: bool = False) -> torch.Tensor:
    """y = H x, H^H x, dH x or dH^H x (dtype of x selects FP64 or complex64 arithmetic)."""
    g = _grid(grid)
    N = g.n[0] * g.n[1] * g.n[2]
    if not torch.is_complex(x):
        x = x.to(torch.complex128)
    dt, rdt = _cdtype(x)
    x, P = _rhs(x, N)
    wr, wi = _wn_planes(wn, rdt)
    y = torch.empty_like(x)
    rc = L.load().h3d_mvp(C.byref(g), _ptr(wr), _ptr(wi), _ptr(x), _ptr(y), P, _mode(mode),
                          int(bool(deriv)), dt, _stream())
    L.check(rc, "h3d_mvp")
    return y


def kacz_sweep(grid, wn: torch.Tensor, w: float, x: torch.Tensor, b: torch.Tensor | None = None,
               mode=1, order: int = L.ORDER_LEX, block=None, nsweeps: int = 1) -> torch.Tensor:
    """``nsweeps`` double Kaczmarz sweeps applied to a copy of x (b = None means b = 0)."""
    g = _grid(grid)
    N = g.n[0] * g.n[1] * g.n[2]
    if not torch.is_complex(x):
        x = x.to(torch.complex128)
    dt, rdt = _cdtype(x)
    y, P = _rhs(x.clone(), N)
    if b is not None:
        b = b.to(x.dtype)
        b, Pb = _rhs(b, N)
        if Pb != P:
            raise L.H3DError(L.ERR_BSIZE, "h3d", "b must match x",
                             "SLIM_release_apps:tools:algorithms:ThreeDFreqModeling:Helm3dkaczswp_mex:Bsize")
    wr, wi = _wn_planes(wn, rdt)
    blk = (C.c_int32 * 3)(*(block or (0, 0, 0)))
    for _ in range(nsweeps):
        rc = L.load().h3d_kacz_sweep(C.byref(g), _ptr(wr), _ptr(wi), float(w), _ptr(y), _ptr(b), P,
                                     _mode(mode), int(order), blk, dt, _stream())
        L.check(rc, "h3d_kacz_sweep")
    return y


def residual(grid, wn: torch.Tensor, b: torch.Tensor, x: torch.Tensor, mode=1):
    """r = b - H x in FP64; returns (r, ||r||^2 per RHS, ||b||^2 per RHS)."""
    g = _grid(grid)
    N = g.n[0] * g.n[1] * g.n[2]
    x, P = _rhs(x.to(torch.complex128), N)
    b, _ = _rhs(b.to(torch.complex128), N)
    wr, wi = _wn_planes(wn, torch.float64)
    r = torch.empty_like(x)
    rr = torch.empty(P, dtype=torch.float64, device=x.device)
    bb = torch.empty(P, dtype=torch.float64, device=x.device)
    rc = L.load().h3d_residual(C.byref(g), _ptr(wr), _ptr(wi), _ptr(b), _ptr(x), _ptr(r), _ptr(rr),
                               _ptr(bb), P, _mode(mode), _stream())
    L.check(rc, "h3d_residual")
    return r, rr, bb
