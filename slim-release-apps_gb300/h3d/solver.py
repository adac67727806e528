"""Solver front end: ``H \\ b`` and ``H' \\ b`` through the C ABI (h3d_solve / h3d_solve_batch).

Mirrors the reference's solve path
``opAbstractMatrix.divide -> linearsolve(op,b,x0,mode,lsopts) -> CGMN(A,b,x,par)``
(tools/algorithms/CommonFreqModeling/opAbstractMatrix.m:117-125,
tools/solvers/Krylov/linearsolve.m:148-168, CGMN.m:36-94) with the Kaczmarz
preconditioner (w = 1.5, one double sweep) and a zero start.  ``LinSolveOpts``
fields map to keyword arguments: ``tol`` (1e-6), ``maxit`` (10000).

Additions of this library (all default to the behaviour named in the docstrings):
``precision`` ("fp64" or "mixed": complex64 inner solves under FP64 refinement),
``order`` (sweep row order), ``stop`` ("true": ||b - H u|| / ||b|| <= tol per column,
or "preconditioned": the reference test of CGMN.m:79).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import torch

from . import _lib as L

_ORDERS = {"lex": L.ORDER_LEX, "colour27": L.ORDER_COLOUR27, "color27": L.ORDER_COLOUR27,
           "block": L.ORDER_BLOCK, "block8": L.ORDER_BLOCK8}


def _grid(grid):
    return grid if isinstance(grid, L.Grid) else L.make_grid(*grid)


def _mode(mode) -> int:
    if isinstance(mode, str):
        return L.FORWARD if mode.lower().startswith("f") else L.ADJOINT
    return L.FORWARD if int(mode) == 1 else L.ADJOINT


def make_opts(tol=1e-6, maxit=10000, precision="fp64", order="block8", stop="true",
              inner_tol=None, max_outer=None, check_every=None, block=None, w=1.5,
              use_graphs=True, verbose=False, method="cgmn") -> L.SolveOpts:
    o = L.default_opts()
    o.tol = float(tol)
    o.maxit = int(maxit)
    o.w = float(w)
    o.precision = L.PREC_MIXED if str(precision).lower().startswith("mix") else L.PREC_FP64
    o.order = _ORDERS[order] if isinstance(order, str) else int(order)
    o.stop_rule = L.STOP_TRUE_RESIDUAL if str(stop).lower().startswith("t") else L.STOP_PRECONDITIONED
    if inner_tol is not None:
        o.inner_tol = float(inner_tol)
    if max_outer is not None:
        o.max_outer = int(max_outer)
    if check_every is not None:
        o.check_every = int(check_every)
    if block is not None:
        for a in range(3):
            o.block[a] = int(block[a])
    o.use_graphs = 1 if use_graphs else 0
    o.verbose = 1 if verbose else 0
    o.method = {"cgmn": L.METHOD_CGMN, "crmn": L.METHOD_CRMN}[method] if isinstance(method, str) else int(method)
    return o


def _rhs(b: torch.Tensor, N: int):
    if not b.is_cuda:
        raise ValueError("b must be a CUDA tensor")
    if b.shape[-1] != N:
        raise L.H3DError(L.ERR_BSIZE, "h3d_solve", "b must have nx*ny*nz elements",
                         "SLIM_release_apps:tools:algorithms:ThreeDFreqModeling:Helm3dkaczswp_mex:Bsize")
    b = b.to(torch.complex128).contiguous()
    P = 1 if b.dim() == 1 else b.numel() // N
    return b, P


def solve(grid, wn: torch.Tensor, b: torch.Tensor, mode=1, opts: L.SolveOpts | None = None,
          raise_not_converged: bool = True, history: int = 0, **kw):
    """u = H \\ b (mode 1) or H' \\ b.  ``b``: complex tensor (N,) or (P, N) on the GPU.
    Returns ``(u, info)`` with info the fields of h3d_solve_info as a dict (plus
    ``history`` when requested)."""
    g = _grid(grid)
    N = g.n[0] * g.n[1] * g.n[2]
    o = opts if opts is not None else make_opts(**kw)
    b, P = _rhs(b, N)
    if torch.is_complex(wn):
        wr, wi = wn.real.to(torch.float64).contiguous(), wn.imag.to(torch.float64).contiguous()
    else:
        wr, wi = wn.to(torch.float64).contiguous(), None
    u = torch.empty_like(b)
    info = L.SolveInfo()
    hist = (C.c_double * max(history, 1))()
    rc = L.load().h3d_solve(C.byref(g), C.c_void_p(wr.data_ptr()),
                            C.c_void_p(wi.data_ptr()) if wi is not None else C.c_void_p(),
                            C.c_void_p(b.data_ptr()), C.c_void_p(u.data_ptr()), P, _mode(mode),
                            C.byref(o), C.byref(info), hist if history else None, history,
                            C.c_void_p(torch.cuda.current_stream().cuda_stream))
    d = info.as_dict()
    if history:
        d["history"] = [hist[i] for i in range(history)]
    if rc == L.ERR_NOT_CONVERGED and not raise_not_converged:
        return u, d
    L.check(rc, "h3d_solve")
    return u, d


@dataclass
class Problem:
    """One problem of a batched solve (its own grid, wavenumber and right-hand sides)."""
    grid: object
    wn: torch.Tensor
    b: torch.Tensor
    mode: int = 1


def solve_batch(problems, opts: L.SolveOpts | None = None, raise_not_converged: bool = True, **kw):
    """Solve a list of Problems of uneven size; returns (list of u, list of info dicts).  With the
    BLOCK8 order all problems iterate together (h3d_solve_batch)."""
    o = opts if opts is not None else make_opts(**kw)
    arr = (L.Problem * len(problems))()
    keep, outs = [], []
    for q, p in enumerate(problems):
        g = _grid(p.grid)
        N = g.n[0] * g.n[1] * g.n[2]
        b, P = _rhs(p.b, N)
        wr = p.wn.real.to(torch.float64).contiguous() if torch.is_complex(p.wn) else p.wn.to(torch.float64).contiguous()
        wi = p.wn.imag.to(torch.float64).contiguous() if torch.is_complex(p.wn) else None
        u = torch.empty_like(b)
        keep += [b, wr, wi]
        outs.append(u)
        arr[q].grid = g
        arr[q].wn_re = wr.data_ptr()
        arr[q].wn_im = wi.data_ptr() if wi is not None else None
        arr[q].b = b.data_ptr()
        arr[q].u = u.data_ptr()
        arr[q].nrhs = P
        arr[q].mode = _mode(p.mode)
    infos = (L.SolveInfo * len(problems))()
    rc = L.load().h3d_solve_batch(arr, len(problems), C.byref(o), infos,
                                  C.c_void_p(torch.cuda.current_stream().cuda_stream))
    if not (rc == L.ERR_NOT_CONVERGED and not raise_not_converged):
        L.check(rc, "h3d_solve_batch")
    return outs, [i.as_dict() for i in infos]
