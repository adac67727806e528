"""FWI objective and gradient on the GPU against the oracle's restatement of PDEfunc.

* forward modelling and (f, g) of PDEfunc OBJ match oracle/slim_ref.pdefunc (numpy
  restatement of PDEfunc.m / discrete_helmholtz.m / opSincInterp.m over the C oracle);
* Taylor test: f(m + h dm) - f(m) - h <g, dm> decays as h^2 over six step sizes (dm is
  zero on the outer layer of the physical grid, so the edge-replicated PML does not see
  it and the reference's cropped gradient, discrete_helmholtz.m:231-232, is exact);
* the torch.autograd.Function gives the same gradient whether the forward wavefields
  are kept or recomputed (HBM budget 0).
"""
import numpy as np
import pytest

from oracle import h3d_oracle as O
from oracle import slim_ref

pytestmark = pytest.mark.gpu


def _geometry(unit="s2/m2", freqs=(4.0, 6.0)):
    from h3d import fwi

    n = (14, 13, 10)
    d = (25.0, 25.0, 25.0)
    npml = (4, 4, 4, 4, 4, 4)
    rng = np.random.default_rng(17)
    src = np.array([[120.0 + 7.3, 130.0 - 4.1, 50.0], [210.0, 90.0 + 11.0, 50.0]])
    rec = np.array([[x, y, 25.0] for x in (60.0, 160.0, 260.0) for y in (70.0, 230.0)])
    geom = fwi.Geometry(o=(0.0, 0.0, 0.0), d=d, n=n, npml6=npml, src_xyz=src, rec_xyz=rec,
                        freqs=np.array(freqs), f0=8.0, t0=0.0, unit=unit,
                        src_amp=np.array([1.0, 0.7 - 0.2j]))
    z = np.arange(n[2]) * d[2]
    vel = np.broadcast_to(1500.0 + 1500.0 * z / z[-1], n).copy()
    vel *= 1.0 + 0.03 * rng.standard_normal(n)
    vtrue = vel.copy()
    vtrue[5:9, 5:8, 4:7] += 120.0
    m0 = vel ** -2 if unit == "s2/m2" else vel
    mt = vtrue ** -2 if unit == "s2/m2" else vtrue
    return geom, m0, mt


def _oracle_model(geom):
    return {"o": geom.o, "d": geom.d, "n": geom.n, "npml6": geom.npml6, "unit": geom.unit,
            "f0": geom.f0, "t0": geom.t0}


def _flatF(a):
    return np.asarray(a).reshape(-1, order="F")


@pytest.mark.parametrize("unit", ["s2/m2", "m/s"])
def test_forward_model_and_gradient_match_oracle(cuda, unit):
    import torch
    from h3d import fwi

    geom, m0, mt = _geometry(unit, freqs=(5.0,))
    prob = fwi.FWIProblem(geom, fwi.FWIConfig(tol=1e-10, precision="fp64"))
    mod = _oracle_model(geom)
    D_ref = slim_ref.pdefunc("forw_model", _flatF(mt), mod, geom.src_xyz, geom.src_amp, geom.rec_xyz,
                             geom.freqs, tol=1e-10, maxit=20000, order=O.ORDER_COLOUR27, nthreads=1)
    D = prob.forward_model(torch.as_tensor(mt, device=cuda)).cpu().numpy()
    assert D.shape == D_ref.shape == (6, 2)
    assert np.max(np.abs(D - D_ref)) <= 1e-6 * np.max(np.abs(D_ref))

    f_ref, g_ref = slim_ref.pdefunc("obj", _flatF(m0), mod, geom.src_xyz, geom.src_amp, geom.rec_xyz,
                                    geom.freqs, Dobs=D_ref, tol=1e-10, maxit=20000,
                                    order=O.ORDER_COLOUR27, nthreads=1)
    f, g = prob.objective(torch.as_tensor(m0, device=cuda), torch.as_tensor(D_ref, device=cuda))
    g = _flatF(g.cpu().numpy())
    assert abs(f - f_ref) <= 1e-6 * abs(f_ref)
    assert np.max(np.abs(g - g_ref)) <= 1e-5 * np.max(np.abs(g_ref))


def test_taylor_second_order(cuda):
    import torch
    from h3d import fwi

    geom, m0, mt = _geometry("s2/m2")
    prob = fwi.FWIProblem(geom, fwi.FWIConfig(tol=1e-11, precision="fp64"))
    Dobs = prob.forward_model(torch.as_tensor(mt, device=cuda))
    rng = np.random.default_rng(3)
    dm = np.zeros(geom.n)
    dm[1:-1, 1:-1, 1:-1] = rng.standard_normal((geom.n[0] - 2, geom.n[1] - 2, geom.n[2] - 2))
    dm *= 0.002 * np.abs(m0).max() / np.abs(dm).max()
    f0, g = prob.objective(torch.as_tensor(m0, device=cuda), Dobs)
    gdm = float(torch.sum(g * torch.as_tensor(dm, device=cuda)))
    hs = [2.0 ** -k for k in range(6)]
    e1, e2 = [], []
    for h in hs:
        fh, _, _ = prob.misfit_forward(torch.as_tensor(m0 + h * dm, device=cuda), Dobs, keep=False)
        e1.append(abs(fh - f0))
        e2.append(abs(fh - f0 - h * gdm))
    e1, e2 = np.array(e1), np.array(e2)
    slope1 = np.polyfit(np.log(hs), np.log(e1), 1)[0]
    slope2 = np.polyfit(np.log(hs), np.log(e2), 1)[0]
    assert abs(slope1 - 1.0) <= 0.25
    assert abs(slope2 - 2.0) <= 0.3
    assert np.all(e2 < e1)


def test_autograd_function_and_recompute(cuda):
    import torch
    from h3d import fwi

    geom, m0, mt = _geometry("s2/m2")
    prob = fwi.FWIProblem(geom, fwi.FWIConfig(tol=1e-10, precision="mixed"))
    Dobs = prob.forward_model(torch.as_tensor(mt, device=cuda))
    f_direct, g_direct = prob.objective(torch.as_tensor(m0, device=cuda), Dobs)
    m = torch.as_tensor(m0, device=cuda).clone().requires_grad_(True)
    f = fwi.fwi_objective(m, prob, Dobs)
    f.backward()
    assert abs(f.item() - f_direct) <= 1e-9 * abs(f_direct)
    torch.testing.assert_close(m.grad, g_direct, rtol=1e-7, atol=1e-12 * g_direct.abs().max().item())
    prob.cfg.hbm_budget_bytes = 0.0        # force the recompute path
    m2 = torch.as_tensor(m0, device=cuda).clone().requires_grad_(True)
    fwi.fwi_objective(m2, prob, Dobs).backward()
    torch.testing.assert_close(m2.grad, m.grad, rtol=1e-6, atol=1e-10 * m.grad.abs().max().item())


def test_jacobian_adjoint_and_gauss_newton(cuda):
    """testJacobian / testGaussNewton of test_ToolsAlgorithms3DFreqModeling.m:167-276:
    Born data against a finite difference of the forward model, the dot test
    <J dm, dD> = <dm, J' dD>, and HESS_GN(dm) = JACOB_ADJ(JACOB_FORW(dm))."""
    import torch
    from h3d import fwi

    geom, m0, _ = _geometry("s2/m2", freqs=(5.0,))
    prob = fwi.FWIProblem(geom, fwi.FWIConfig(tol=1e-11, precision="fp64"))
    rng = np.random.default_rng(8)
    dm = np.zeros(geom.n)
    dm[1:-1, 1:-1, 1:-1] = rng.standard_normal((geom.n[0] - 2, geom.n[1] - 2, geom.n[2] - 2))
    dm *= 1e-3 * np.abs(m0).max() / np.abs(dm).max()
    mt, dmt = torch.as_tensor(m0, device=cuda), torch.as_tensor(dm, device=cuda)
    Jdm = prob.jacob_forw(mt, dmt)
    h = 0.1  # dm is already 1e-3 of m: central differences are accurate to ~1e-8 here
    fd = (prob.forward_model(mt + h * dmt) - prob.forward_model(mt - h * dmt)) / (2 * h)
    assert (fd - Jdm).abs().max().item() <= 1e-5 * Jdm.abs().max().item()
    dD = torch.as_tensor(rng.standard_normal(Jdm.shape) + 1j * rng.standard_normal(Jdm.shape), device=cuda)
    JtdD = prob.jacob_adj(mt, dD)
    lhs = torch.sum(torch.conj(dD) * Jdm).real.item()
    rhs = torch.sum(dmt * JtdD).item()
    assert abs(lhs - rhs) <= 1e-8 * max(abs(lhs), abs(rhs))
    hgn = prob.hess_gn(mt, dmt)
    comp = prob.jacob_adj(mt, prob.jacob_forw(mt, dmt))
    assert (hgn - comp).abs().max().item() <= 1e-9 * comp.abs().max().item()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_gradient_with_multigrid_solver_matches_oracle(cuda, precision):
    """FWIConfig(solver="mlgmres"): forward and adjoint solves by FGMRES + ML_GMRES (the
    reference's default for its 3D applications) give the oracle's (f, g) to solver tolerance."""
    import torch
    from h3d import fwi

    geom, m0, mt = _geometry("s2/m2", freqs=(5.0,))
    mod = _oracle_model(geom)
    D_ref = slim_ref.pdefunc("forw_model", _flatF(mt), mod, geom.src_xyz, geom.src_amp, geom.rec_xyz,
                             geom.freqs, tol=1e-10, maxit=20000, order=O.ORDER_COLOUR27, nthreads=1)
    f_ref, g_ref = slim_ref.pdefunc("obj", _flatF(m0), mod, geom.src_xyz, geom.src_amp, geom.rec_xyz,
                                    geom.freqs, Dobs=D_ref, tol=1e-10, maxit=20000,
                                    order=O.ORDER_COLOUR27, nthreads=1)
    prob = fwi.FWIProblem(geom, fwi.FWIConfig(tol=1e-10, precision=precision, solver="mlgmres"))
    D = prob.forward_model(torch.as_tensor(mt, device=cuda)).cpu().numpy()
    assert np.max(np.abs(D - D_ref)) <= 1e-6 * np.max(np.abs(D_ref))
    f, g = prob.objective(torch.as_tensor(m0, device=cuda), torch.as_tensor(D_ref, device=cuda))
    g = _flatF(g.cpu().numpy())
    assert abs(f - f_ref) <= 1e-6 * abs(f_ref)
    assert np.max(np.abs(g - g_ref)) <= 1e-5 * np.max(np.abs(g_ref))
