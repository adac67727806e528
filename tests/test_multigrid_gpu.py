"""FGMRES + ML_GMRES on the GPU (h3d.multigrid) against the oracle's restatement
(oracle/slim_ml.py): the coarse levels' wavenumbers and the grid transfers (h3d_axis_apply),
then the whole preconditioned solve -- same outer iteration count, same quasi-residual
history and the same solution to rounding (FP64 throughout)."""
import numpy as np
import pytest

from oracle import slim_ml as ML

pytestmark = pytest.mark.gpu


def _model(seed=0):
    rng = np.random.default_rng(seed)
    n, h = (17, 15, 13), 25.0
    z = np.arange(n[2]) * h
    v = np.broadcast_to(1500 + 1000 * z / z[-1], n).copy() * (1 + 0.05 * rng.standard_normal(n))
    return v, (h, h, h), 6, 4.0


def test_levels_and_transfers_match_oracle(cuda):
    import torch
    from h3d import multigrid as MG

    v, dt, npml, f = _model()
    lv_ref, R_ref, P_ref = ML.build_levels(v, dt, npml, f, "m/s")
    lv, R, P = MG.build_levels(v, dt, npml, f, "m/s", device=cuda)
    rng = np.random.default_rng(2)
    for a, b in zip(lv, lv_ref):
        assert a.nt == b.nt
        assert np.max(np.abs(a.wn.cpu().numpy() - b.wn)) <= 1e-12 * np.max(np.abs(b.wn))
    for i in range(2):
        xf = rng.standard_normal(lv_ref[i].N) + 1j * rng.standard_normal(lv_ref[i].N)
        xc = rng.standard_normal(lv_ref[i + 1].N) + 1j * rng.standard_normal(lv_ref[i + 1].N)
        f2c, c = R_ref[i]
        r_ref = c * (f2c * xf)
        p_ref = P_ref[i] * xc
        r = R[i](torch.as_tensor(xf, device=cuda)).cpu().numpy()
        p = P[i](torch.as_tensor(xc, device=cuda)).cpu().numpy()
        assert np.max(np.abs(r - r_ref)) <= 1e-12 * np.max(np.abs(r_ref))
        assert np.max(np.abs(p - p_ref)) <= 1e-12 * np.max(np.abs(p_ref))
        # complex64 fields through the same kernel
        r32 = R[i](torch.as_tensor(xf, device=cuda, dtype=torch.complex64)).cpu().numpy()
        assert np.max(np.abs(r32 - r_ref)) <= 1e-6 * np.max(np.abs(r_ref))


def test_fgmres_ml_gmres_matches_oracle(cuda):
    import torch
    from h3d import multigrid as MG

    v, dt, npml, f = _model()
    lv_ref, R_ref, P_ref = ML.build_levels(v, dt, npml, f, "m/s")
    b = np.zeros(lv_ref[0].N, complex)
    nx, ny, _ = lv_ref[0].nt
    b[nx // 2 + nx * (ny // 2) + nx * ny * 9] = 1.0
    x_ref, _, hst_ref = ML.ml_gmres_solve(lv_ref, R_ref, P_ref, b, tol=1e-6)
    lv, R, P = MG.build_levels(v, dt, npml, f, "m/s", device=cuda)
    u, info = MG.solve(lv, R, P, torch.as_tensor(b, device=cuda), tol=1e-6)
    u = u.cpu().numpy()
    assert info["iters"] == len(hst_ref) - 1
    np.testing.assert_allclose(info["hst"], hst_ref, rtol=1e-6, atol=1e-12)
    assert np.linalg.norm(u - x_ref) <= 1e-8 * np.linalg.norm(x_ref)
    r = b - lv_ref[0].A(u)
    assert np.linalg.norm(r) / np.linalg.norm(b) <= 1e-6


def test_mixed_precision_cycle_converges(cuda):
    """complex64 V-cycle under the complex128 FGMRES: the same true residual, at most a
    few more outer iterations than the FP64 solve."""
    import torch
    from h3d import multigrid as MG

    v, dt, npml, f = _model(seed=3)
    lv, R, P = MG.build_levels(v, dt, npml, f, "m/s", device=cuda)
    b = torch.zeros(int(np.prod(lv[0].nt)), dtype=torch.complex128, device=cuda)
    nx, ny, _ = lv[0].nt
    b[nx // 2 + nx * (ny // 2) + nx * ny * 9] = 1.0
    u64, i64 = MG.solve(lv, R, P, b, tol=1e-6)
    u32, i32 = MG.solve(lv, R, P, b, tol=1e-6, precision="mixed")
    for u in (u64, u32):
        assert float((b - lv[0].A(u)).norm() / b.norm()) <= 1e-6
    assert i32["iters"] <= i64["iters"] + 5
