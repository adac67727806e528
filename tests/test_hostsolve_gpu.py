"""Entry points above sweep granularity, with host buffers (GPU).

* h3d_solve_mex (the drop-in gateway for linearsolve / CGMN on a Helmholtz operator, hosted
  by the stub MEX API): forward and adjoint, one and two right-hand sides, FP64 and mixed
  precision; against the oracle's CGMN solution and its matvec (true residual).
* h3d_fwi_grad (PDEfunc OBJ for one frequency and a source batch through ctypes): f and the
  gradient against the oracle's PDEfunc restatement (oracle/slim_ref.pdefunc) and against the
  library's own FWI layer.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import h3d_oracle as O
from oracle import slim_ref

pytestmark = pytest.mark.gpu


def _problem(n=(18, 17, 16), npml=4, f=5.0, seed=3, P=2):
    rng = np.random.default_rng(seed)
    N = int(np.prod(n))
    wn = (2 * np.pi * f) ** 2 / (1500.0 + 1500.0 * rng.random(N)) ** 2
    B = rng.standard_normal((N, P)) + 1j * rng.standard_normal((N, P))
    return n, (25.0, 20.0, 25.0), npml, wn, B


@pytest.mark.parametrize("mode,precision", [(1, 0), (2, 0), (1, 1)])
def test_solve_gateway_matches_oracle(cuda, mode, precision):
    from h3d import build
    from oracle import mexharness as M

    gw = M.MexFunction(build.build_mex()["h3d_solve_mex"])
    n, h, npml, wn, B = _problem(seed=3 + mode)
    g = O.make_grid(n, h, npml)
    npml23 = np.full((2, 3), float(npml))
    U = gw(wn, np.array(h), np.array(n, float), npml23, B, float(mode), 1e-8, 20000.0, float(precision))
    assert U.shape == B.shape
    for s in range(B.shape[1]):
        assert slim_ref.true_residual(g, wn, B[:, s], U[:, s], mode=mode) <= 1e-8
        xref = slim_ref.cgmn_solve(g, wn, B[:, s], tol=1e-11, maxit=20000, mode=mode, order=O.ORDER_COLOUR27)
        assert np.linalg.norm(U[:, s] - xref) / np.linalg.norm(xref) <= 1e-6


def test_solve_gateway_reference_stopping_rule(cuda):
    """stop = 0: CGMN.m:79's preconditioned residual test; the result is then the reference
    solve's up to the row order (true residual of the order of the tolerance)."""
    from h3d import build
    from oracle import mexharness as M

    gw = M.MexFunction(build.build_mex()["h3d_solve_mex"])
    n, h, npml, wn, B = _problem(P=1, seed=9)
    g = O.make_grid(n, h, npml)
    U = gw(wn, np.array(h), np.array(n, float), np.full((2, 3), float(npml)), B, 1.0, 1e-6, 5000.0, 0.0, 0.0)
    xref, hst = slim_ref.linearsolve_cgmn(g, wn, B[:, 0], tol=1e-6, maxit=5000, order=O.ORDER_LEX)
    tr = slim_ref.true_residual(g, wn, B[:, 0], U[:, 0])
    assert tr <= 50 * slim_ref.true_residual(g, wn, B[:, 0], xref)
    assert np.linalg.norm(U[:, 0] - xref) / np.linalg.norm(xref) <= 1e-3


def _fwi_case():
    from h3d import fwi

    n, d, npml = (14, 13, 10), (25.0, 25.0, 25.0), (4, 4, 4, 4, 4, 4)
    rng = np.random.default_rng(19)
    src = np.array([[120.0 + 7.3, 130.0 - 4.1, 50.0], [210.0, 90.0 + 11.0, 50.0]])
    rec = np.array([[x, y, 25.0] for x in (60.0, 160.0, 260.0) for y in (70.0, 230.0)])
    geom = fwi.Geometry(o=(0.0, 0.0, 0.0), d=d, n=n, npml6=npml, src_xyz=src, rec_xyz=rec,
                        freqs=np.array([5.0]), f0=8.0, t0=0.0, unit="s2/m2", src_amp=np.array([1.0, 0.7 - 0.2j]))
    z = np.arange(n[2]) * d[2]
    vel = np.broadcast_to(1500.0 + 1500.0 * z / z[-1], n).copy() * (1.0 + 0.03 * rng.standard_normal(n))
    D = rng.standard_normal((len(rec), 2)) * 1e-4 + 1j * rng.standard_normal((len(rec), 2)) * 1e-4
    return geom, vel ** -2, D


def test_fwi_grad_entry_matches_oracle_and_fwi_layer(cuda):
    import torch
    from h3d import _lib as L
    from h3d import fwi, solver

    geom, m0, D = _fwi_case()
    prob = fwi.FWIProblem(geom, fwi.FWIConfig(tol=1e-10, precision="fp64"))
    mt = torch.as_tensor(m0, device=cuda)
    wn, dwn = prob._wavenumbers(mt, 5.0)
    wn, dwn = wn.cpu().numpy(), dwn.cpu().numpy()
    sp = np.ascontiguousarray(geom.to_index(geom.src_xyz))
    rp = np.ascontiguousarray(geom.to_index(geom.rec_xyz))
    amp = prob.wavelet[0] * prob.src_amp * (np.prod(geom.d) / np.prod(geom.dt))
    amp2 = np.ascontiguousarray(np.stack([amp.real, amp.imag], 1))
    dob = np.ascontiguousarray(np.stack([D.T.real, D.T.imag], -1))      # column s at s * nrec
    gph = np.zeros(int(np.prod(geom.n)))
    f = C.c_double()
    opts = solver.make_opts(tol=1e-10, precision="fp64")
    info = L.SolveInfo()
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    rc = L.load().h3d_fwi_grad(C.byref(prob.g), dp(wn), dp(dwn), dp(sp), len(sp), dp(amp2), dp(rp), len(rp), dp(dob),
                               C.byref(opts), C.byref(f), dp(gph), C.byref(info))
    L.check(rc, "h3d_fwi_grad")
    assert info.converged == 1
    g_lay = prob.objective_pairs(mt, torch.as_tensor(D, device=cuda), 0, [0, 1])
    g_l = g_lay[1].permute(2, 1, 0).reshape(-1).cpu().numpy()
    assert abs(f.value - g_lay[0]) <= 1e-9 * abs(g_lay[0])
    assert np.max(np.abs(gph - g_l)) <= 1e-8 * np.max(np.abs(g_l))
    mod = {"o": geom.o, "d": geom.d, "n": geom.n, "npml6": geom.npml6, "unit": geom.unit, "f0": geom.f0, "t0": 0.0}
    f_ref, g_ref = slim_ref.pdefunc("obj", np.asarray(m0).reshape(-1, order="F"), mod, geom.src_xyz, geom.src_amp,
                                    geom.rec_xyz, geom.freqs, Dobs=D, tol=1e-10, maxit=20000,
                                    order=O.ORDER_COLOUR27, nthreads=1)
    assert abs(f.value - f_ref) <= 1e-6 * abs(f_ref)
    assert np.max(np.abs(gph - g_ref)) <= 1e-5 * np.max(np.abs(g_ref))
