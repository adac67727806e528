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


@pytest.mark.parametrize("mode", [1, 2])
def test_fgmres_ml_gmres_matches_oracle(cuda, mode):
    """Forward (H) and adjoint (H^H) solves: the outer iteration count, the quasi-residual
    history and the solution of the oracle's restatement."""
    import torch
    from h3d import multigrid as MG

    v, dt, npml, f = _model()
    lv_ref, R_ref, P_ref = ML.build_levels(v, dt, npml, f, "m/s")
    b = np.zeros(lv_ref[0].N, complex)
    nx, ny, _ = lv_ref[0].nt
    b[nx // 2 + nx * (ny // 2) + nx * ny * 9] = 1.0
    x_ref, _, hst_ref = ML.ml_gmres_solve(lv_ref, R_ref, P_ref, b, tol=1e-6, mode=mode)
    lv, R, P = MG.build_levels(v, dt, npml, f, "m/s", device=cuda)
    u, info = MG.solve(lv, R, P, torch.as_tensor(b, device=cuda), tol=1e-6, mode=mode)
    u = u.cpu().numpy()
    assert info["iters"] == len(hst_ref) - 1
    assert info["converged"] == 1
    np.testing.assert_allclose(info["hst"], hst_ref, rtol=1e-6, atol=1e-12)
    assert np.linalg.norm(u - x_ref) <= 1e-8 * np.linalg.norm(x_ref)
    r = b - lv_ref[0].A(u, mode)
    assert np.linalg.norm(r) / np.linalg.norm(b) <= 1e-6


def test_plain_fgmres_restart_cycles_match_scipy_gmres(cuda):
    """Without a preconditioner FGMRES.m is GMRES(m): after c cycles of m steps the library's
    solution (device Arnoldi steps and Givens rotations) equals scipy's GMRES(m) on the
    oracle's operator, and every step is recorded."""
    import torch
    from scipy.sparse.linalg import LinearOperator, gmres
    from h3d import multigrid as MG

    v, dt, npml, f = _model()
    lv_ref, _, _ = ML.build_levels(v, dt, npml, f, "m/s")
    lv, R, P = MG.build_levels(v, dt, npml, f, "m/s", device=cuda)
    N = lv_ref[0].N
    rng = np.random.default_rng(5)
    b = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    A = LinearOperator((N, N), matvec=lambda x: lv_ref[0].A(x), dtype=complex)
    for m, c in ((5, 3), (8, 2), (16, 1)):
        ref, _ = gmres(A, b, rtol=1e-30, atol=0.0, restart=m, maxiter=c)
        u, info = MG.solve(lv, R, P, torch.as_tensor(b, device=cuda), tol=1e-30, maxit=c, maxinnerit=m,
                           precond="none")
        assert info["iters"] == c * m and len(info["hst"]) == c * m + 1
        assert np.all(np.diff(info["hst"]) <= 1e-12)          # GMRES residuals never grow in a cycle
        assert np.linalg.norm(u.cpu().numpy() - ref) <= 1e-9 * np.linalg.norm(ref)


def test_initial_guess_and_zero_rhs(cuda):
    """A nonzero initial guess starts from r = b - H x0 (FGMRES.m:62-64) and the solve reduces
    that residual by tol; b = 0 returns x = 0 at once."""
    import torch
    from h3d import multigrid as MG

    v, dt, npml, f = _model(seed=1)
    lv_ref, _, _ = ML.build_levels(v, dt, npml, f, "m/s")
    lv, R, P = MG.build_levels(v, dt, npml, f, "m/s", device=cuda)
    rng = np.random.default_rng(7)
    N = lv_ref[0].N
    b = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    x0 = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    u, info = MG.solve(lv, R, P, torch.as_tensor(b, device=cuda), tol=1e-6,
                       x0=torch.as_tensor(x0, device=cuda), precision="mixed")
    r0 = np.linalg.norm(b - lv_ref[0].A(x0))
    assert np.linalg.norm(b - lv_ref[0].A(u.cpu().numpy())) <= 1e-6 * r0 * 1.01
    z, info = MG.solve(lv, R, P, torch.zeros(N, dtype=torch.complex128, device=cuda))
    assert info["iters"] == 0 and float(z.abs().max()) == 0.0


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


def test_hierarchy_built_by_the_library_and_mex_gateway(cuda):
    """h3d_mlgmres_solve_model (construct_multigrid in the library's host code) and the
    h3d_mlgmres_mex gateway (MATLAB host arrays, two columns) give the solve on the levels
    assembled here: same outer iterations, same solution to rounding (FP64)."""
    import torch
    from h3d import build
    from h3d import multigrid as MG
    from oracle import mexharness as M

    v, dt, npml, f = _model(seed=4)
    lv, R, P = MG.build_levels(v, dt, npml, f, "m/s", device=cuda)
    N = int(np.prod(lv[0].nt))
    rng = np.random.default_rng(9)
    B = rng.standard_normal((N, 2)) + 1j * rng.standard_normal((N, 2))
    ref = [MG.solve(lv, R, P, torch.as_tensor(B[:, c].copy(), device=cuda), tol=1e-8) for c in range(2)]
    u, info = MG.solve_model(v, dt, npml, f, torch.as_tensor(B[:, 0].copy(), device=cuda), tol=1e-8)
    assert info["iters"] == ref[0][1]["iters"] and info["converged"] == 1
    r0 = ref[0][0].cpu().numpy()
    assert np.linalg.norm(u.cpu().numpy() - r0) <= 1e-10 * np.linalg.norm(r0)
    gw = M.MexFunction(build.build_mex()["h3d_mlgmres_mex"])
    U = gw(np.asarray(v, float).reshape(-1, order="F"), np.asarray(dt, float), np.array(v.shape, float),
           float(npml), f, B, 1.0, 1e-8, 10000.0)
    for c in range(2):
        rc = ref[c][0].cpu().numpy()
        assert np.linalg.norm(U[:, c] - rc) <= 1e-10 * np.linalg.norm(rc)
