"""The oracle's Krylov restatements on small dense Hermitian positive definite systems
(no GPU): CGMN.m and CRMN.m converge to the direct solution, column by column."""
import numpy as np

from oracle import slim_ref


def _hpd(n=40, seed=0):
    rng = np.random.default_rng(seed)
    M = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    return M.conj().T @ M + n * np.eye(n)


def test_cgmn_and_crmn_solve_hpd_systems():
    A = _hpd()
    rng = np.random.default_rng(1)
    B = rng.standard_normal((40, 3)) + 1j * rng.standard_normal((40, 3))
    ref = np.linalg.solve(A, B)
    op = lambda X: A @ X
    x_cg, h_cg = slim_ref.cgmn(op, B, np.zeros_like(B), tol=1e-12, maxit=200)
    x_cr, h_cr = slim_ref.crmn(op, B, np.zeros_like(B), tol=1e-12, maxit=200)
    x_cr0, h_cr0 = slim_ref.crmn(op, B, None, tol=1e-12, maxit=200)
    for x in (x_cg, x_cr, x_cr0):
        assert np.linalg.norm(x - ref) <= 1e-9 * np.linalg.norm(ref)
    assert h_cg[-1] <= 1e-12 and h_cr[-1] <= 1e-12
    assert np.array_equal(x_cr, x_cr0)      # A 0 = 0 exactly: both starts give the same iterates
    # conjugate residual minimises ||r|| over the Krylov space: its history never increases
    assert np.all(np.diff(h_cr) <= 1e-12)


def test_cgmn_and_crmn_restatements_match_scipy_cg_and_minres():
    """On a Hermitian positive definite system (what I - Q is), CGMN.m's iterates are CG's and
    CRMN.m's are the minimal-residual iterates MINRES also produces: the oracle's
    restatements equal scipy's independent CG / MINRES after the same iteration count."""
    from scipy.sparse.linalg import cg, minres

    rng = np.random.default_rng(0)
    n = 30
    B = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    A = B.conj().T @ B / n + 0.5 * np.eye(n)
    b = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    for k in (3, 7, 12):
        ref, _ = cg(A, b, rtol=1e-30, atol=0.0, maxiter=k)
        x, _ = slim_ref.cgmn(lambda y: A @ y, b, np.zeros(n, complex), tol=1e-30, maxit=k)
        assert np.linalg.norm(x - ref) <= 1e-13 * np.linalg.norm(ref)
        ref, _ = minres(A, b, rtol=1e-30, maxiter=k)
        x, _ = slim_ref.crmn(lambda y: A @ y, b, np.zeros(n, complex), tol=1e-30, maxit=k)
        assert np.linalg.norm(x - ref) <= 1e-13 * np.linalg.norm(ref)
