"""GPU solver parity: CGMN with the Kaczmarz preconditioner against the numpy/C oracle.

* LEX order + the reference stopping rule reproduces the reference iteration
  (linearsolve.m + CGMN.m): same iteration count and the same iterate to rounding.
* COLOUR27 / BLOCK / BLOCK8 orders and the mixed-precision path converge to the same solution;
  their true residual ||b - H u|| / ||b|| is checked in FP64 by the oracle matvec.
"""
import numpy as np
import pytest

from oracle import h3d_oracle as O
from oracle import slim_ref

pytestmark = pytest.mark.gpu


def _problem(n=(20, 19, 18), npml=4, f=5.0, seed=0):
    rng = np.random.default_rng(seed)
    N = int(np.prod(n))
    v = 1500.0 + 1500.0 * rng.random(N)
    wn = (2 * np.pi * f) ** 2 / v ** 2
    b = np.zeros(N, complex)
    b[n[0] // 2 + n[0] * (n[1] // 2) + n[0] * n[1] * (npml + 2)] = 1.0
    grid = (n, (25.0, 25.0, 25.0), npml)
    return grid, O.make_grid(n, (25.0, 25.0, 25.0), npml), wn, b


def _t(a, dev):
    import torch

    return torch.as_tensor(np.ascontiguousarray(a), device=dev)


@pytest.mark.parametrize("mode", [1, 2])
def test_lex_cgmn_reproduces_reference_iteration(cuda, mode):
    from h3d import solver

    grid, g, wn, b = _problem()
    xref, hst = slim_ref.linearsolve_cgmn(g, wn, b, mode=mode, tol=1e-6, maxit=3000, order=O.ORDER_LEX)
    u, info = solver.solve(grid, _t(wn, cuda), _t(b, cuda), mode=mode, tol=1e-6, maxit=3000,
                           order="lex", stop="preconditioned", precision="fp64", check_every=5)
    assert abs(info["iters"] - (len(hst) - 1)) <= 1
    u = u.cpu().numpy()
    assert np.linalg.norm(u - xref) / np.linalg.norm(xref) <= 1e-7


@pytest.mark.parametrize("order", ["colour27", "block", "block8"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_reordered_and_mixed_solves_converge_to_reference_solution(cuda, order, precision):
    from h3d import solver

    grid, g, wn, b = _problem()
    xref = slim_ref.cgmn_solve(g, wn, b, tol=1e-11, maxit=6000, order=O.ORDER_COLOUR27)
    u, info = solver.solve(grid, _t(wn, cuda), _t(b, cuda), tol=1e-6, order=order,
                           block=(8, 8, 8) if order == "block" else None, precision=precision)
    u = u.cpu().numpy()
    tr = slim_ref.true_residual(g, wn, b, u)
    assert tr <= 1e-6 and info["rel_res_true"] <= 1e-6 and info["converged"] == 1
    assert np.linalg.norm(u - xref) / np.linalg.norm(xref) <= 1e-4


@pytest.mark.parametrize("order", ["colour27", "block8"])
def test_multi_rhs_masks_and_zero_rhs(cuda, order):
    from h3d import solver

    grid, g, wn, b = _problem(seed=2)
    N = b.size
    rng = np.random.default_rng(1)
    B = np.stack([b, np.zeros(N), rng.standard_normal(N) + 1j * rng.standard_normal(N)])
    u, info = solver.solve(grid, _t(wn, cuda), _t(B, cuda), tol=1e-6, precision="fp64", order=order)
    u = u.cpu().numpy()
    assert np.all(u[1] == 0)                       # opAbstractMatrix.m:118
    for s in (0, 2):
        assert slim_ref.true_residual(g, wn, B[s], u[s]) <= 1e-6
    u2, _ = solver.solve(grid, _t(wn, cuda), _t(B[2], cuda), tol=1e-6, precision="fp64", order=order)
    assert np.linalg.norm(u2.cpu().numpy() - u[2]) <= 1e-5 * np.linalg.norm(u[2])


def test_batch_of_uneven_problems(cuda):
    from h3d import solver

    probs, refs = [], []
    for q, n in enumerate([(14, 15, 16), (21, 17, 13)]):
        grid, g, wn, b = _problem(n=n, npml=3, seed=10 + q)
        probs.append(solver.Problem(grid, _t(wn, cuda), _t(b, cuda), mode=1 + q))
        refs.append((g, wn, b, 1 + q))
    us, infos = solver.solve_batch(probs, tol=1e-6, precision="mixed")
    for u, info, (g, wn, b, mode) in zip(us, infos, refs):
        assert slim_ref.true_residual(g, wn, b, u.cpu().numpy(), mode=mode) <= 1e-6
        assert info["converged"] == 1


def test_not_converged_reports_status(cuda):
    from h3d import _lib as L
    from h3d import solver

    grid, g, wn, b = _problem()
    with pytest.raises(L.H3DError) as e:
        solver.solve(grid, _t(wn, cuda), _t(b, cuda), tol=1e-6, maxit=3, precision="fp64")
    assert e.value.status == L.ERR_NOT_CONVERGED
    u, info = solver.solve(grid, _t(wn, cuda), _t(b, cuda), tol=1e-6, maxit=3, precision="fp64",
                           raise_not_converged=False)
    assert info["converged"] == 0 and info["iters"] == 3


@pytest.mark.parametrize("mode", [1, 2])
def test_lex_crmn_reproduces_reference_iteration(cuda, mode):
    """LinSolveOpts.SOLVE_CRMN (CRMN.m through linearsolve.m:51-64) in the reference row order
    and stopping rule: the same iteration count and iterate as the oracle restatement."""
    from h3d import solver

    grid, g, wn, b = _problem()
    xref, hst = slim_ref.linearsolve_crmn(g, wn, b, mode=mode, tol=1e-6, maxit=3000, order=O.ORDER_LEX)
    u, info = solver.solve(grid, _t(wn, cuda), _t(b, cuda), mode=mode, tol=1e-6, maxit=3000,
                           order="lex", stop="preconditioned", precision="fp64", check_every=5,
                           method="crmn")
    assert abs(info["iters"] - (len(hst) - 1)) <= 1
    u = u.cpu().numpy()
    assert np.linalg.norm(u - xref) / np.linalg.norm(xref) <= 1e-7


@pytest.mark.parametrize("order,precision", [("colour27", "fp64"), ("block8", "mixed")])
def test_crmn_converges_on_true_residual(cuda, order, precision):
    from h3d import solver

    grid, g, wn, b = _problem(seed=4)
    N = b.size
    rng = np.random.default_rng(6)
    B = np.stack([b, np.zeros(N), rng.standard_normal(N) + 1j * rng.standard_normal(N)])
    u, info = solver.solve(grid, _t(wn, cuda), _t(B, cuda), tol=1e-6, order=order, precision=precision,
                           method="crmn")
    u = u.cpu().numpy()
    assert info["converged"] == 1 and np.all(u[1] == 0)
    for s in (0, 2):
        assert slim_ref.true_residual(g, wn, B[s], u[s]) <= 1e-6


def test_point_source_matches_analytic_greens_function(cuda):
    """The reference's testAnalytic (tools/algorithms/3DFreqModeling/
    test_ToolsAlgorithms3DFreqModeling.m:50-73) at a smaller size: constant velocity
    2000 m/s, h = 10 m, 8 Hz (25 points per wavelength), 40^3 physical points inside a
    15-point PML, a unit point source at the centre.  Away from the source the wavefield must
    match h^3 exp(i k R) / (4 pi R) to 1% over the physical region (the reference's bound).
    The C oracle's CGMN solution of the same problem measures 0.86%."""
    from h3d import solver

    nphys, npml, h, f, v0 = 40, 15, 10.0, 8.0, 2000.0
    n = (nphys + 2 * npml,) * 3
    N = int(np.prod(n))
    k = 2 * np.pi * f / v0
    wn = np.full(N, k ** 2)
    c = n[0] // 2
    b = np.zeros(N, complex)
    b[c + n[0] * c + n[0] * n[1] * c] = 1.0
    u, info = solver.solve((n, (h, h, h), npml), _t(wn, cuda), _t(b, cuda), tol=1e-8, precision="fp64")
    assert info["converged"] == 1
    U = u.cpu().numpy().reshape(n, order="F")
    ax = np.arange(n[0]) * h
    X, Y, Z = np.meshgrid(ax, ax, ax, indexing="ij")
    R = np.sqrt((X - c * h) ** 2 + (Y - c * h) ** 2 + (Z - c * h) ** 2)
    R[c, c, c] = 1.0
    G = h ** 3 * np.exp(1j * k * R) / (4 * np.pi * R)
    r = U - G
    r[c, c, c] = 0.0                      # the wavefield is not expected to be accurate at the source
    s = slice(npml, npml + nphys)
    assert np.linalg.norm(r[s, s, s]) / np.linalg.norm(U[s, s, s]) < 0.01


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_batched_block8_uneven_problems(cuda, precision):
    """Three problems of different grids, PML widths, modes, wavenumber kinds and column
    counts (9 columns: a full group of eight and a partly filled one) in one batched BLOCK8
    solve: every column reaches the true residual 1e-6 (checked by the oracle's matvec) and
    agrees with the oracle's tight solution; a zero column returns zero."""
    import torch
    from h3d import solver

    specs = [((30, 26, 28), 4, 9, 1, False), ((21, 25, 19), 3, 1, 2, False), ((27, 27, 27), 5, 3, 1, True)]
    probs, refs = [], []
    for q, (n, npml, P, mode, wnc) in enumerate(specs):
        grid, g, wn, b = _problem(n=n, npml=npml, seed=50 + q)
        if wnc:
            wn = wn * (1.0 + 0.02j)
        rng = np.random.default_rng(60 + q)
        B = np.stack([b] + [rng.standard_normal(b.size) + 1j * rng.standard_normal(b.size) for _ in range(P - 1)])
        if P >= 3:
            B[1] = 0.0
        probs.append(solver.Problem(grid, _t(wn, cuda), _t(B, cuda), mode=mode))
        refs.append((g, wn, B, mode))
    us, infos = solver.solve_batch(probs, tol=1e-6, precision=precision)
    for u, info, (g, wn, B, mode) in zip(us, infos, refs):
        assert info["converged"] == 1
        U = u.cpu().numpy()
        for s in range(B.shape[0]):
            if not np.any(B[s]):
                assert np.all(U[s] == 0)
                continue
            assert slim_ref.true_residual(g, wn, B[s], U[s], mode=mode) <= 1e-6
        xref = slim_ref.cgmn_solve(g, wn, B[0], tol=1e-11, maxit=8000, mode=mode, order=O.ORDER_COLOUR27)
        assert np.linalg.norm(U[0] - xref) / np.linalg.norm(xref) <= 1e-4


def test_bounded_wait_expires_with_a_status(cuda):
    """The BLOCK8 kernel's bounded mbarrier waits: a coefficient copy announced but never
    issued makes every wait of the first colour step give up after 2 ms; the call returns
    H3D_ERR_TIMEOUT and the context stays usable (a sweep right after matches the oracle)."""
    import torch
    from h3d import _lib as L
    from h3d import ops

    lib = L.load()
    assert lib.h3d_check_wait_timeout(2.0) == L.ERR_TIMEOUT
    assert b"expired" in lib.h3d_last_error()
    torch.cuda.synchronize()
    n, npml = (26, 25, 27), 4
    grid, g, wn, b = _problem(n=n, npml=npml, seed=70)
    rng = np.random.default_rng(71)
    X = rng.standard_normal(b.size) + 1j * rng.standard_normal(b.size)
    ref = O.sweep(g, wn, 1.5, X, b, order=O.ORDER_BLOCK8, blk=(12, 12, 12), nthreads=2)
    y = ops.kacz_sweep(grid, _t(wn, cuda), 1.5, _t(X, cuda), _t(b, cuda), 1, order=3)
    assert np.linalg.norm(y.cpu().numpy() - ref) / np.linalg.norm(ref) <= 1e-12
