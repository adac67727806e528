"""The oracle's restatement of FGMRES + ML_GMRES (oracle/slim_ml.py) on CPU.

* opLInterp1D's self-test (opLInterp1D.m test()): cubic Lagrange weights reproduce x^3
  exactly on points inside the node range, and the operator's adjoint passes the dot test;
* LinInterp1D reproduces linear functions, and the multigrid restriction is (1/8) times the
  adjoint of the prolongation (construct_multigrid.m:45-51);
* FGMRES (FGMRES.m) solves a small dense system, with and without a preconditioner;
* FGMRES preconditioned by the three-level ML_GMRES V-cycle solves a small Helmholtz problem
  to the requested true residual.
"""
import numpy as np

from oracle import slim_ml as ML


def test_interpolation_operators():
    rng = np.random.default_rng(0)
    x1 = np.linspace(0, 1, 13)
    x2 = np.linspace(0, 1, 7)
    A = ML.cubic_interp_1d(x1, x2)
    assert np.max(np.abs(A @ x1 ** 3 - x2 ** 3)) <= 1e-12
    f1, f2 = rng.standard_normal(13), rng.standard_normal(7)
    assert abs(1 - (A @ f1) @ f2 / (f1 @ (A.T @ f2))) <= 1e-10
    L = ML.lin_interp_1d(np.linspace(0, 1, 7), np.linspace(0, 1, 13))
    assert np.max(np.abs(L @ (3 * np.linspace(0, 1, 7) + 1) - (3 * np.linspace(0, 1, 13) + 1))) <= 1e-12
    f2c, c2f, nsub = ML.fine2coarse((9, 8, 7), kind="linear", n_sub=(5, 4, 4))
    x = rng.standard_normal(9 * 8 * 7)
    y = rng.standard_normal(5 * 4 * 4)
    assert abs((c2f * y) @ x - y @ (f2c * x)) <= 1e-10 * np.linalg.norm(x) * np.linalg.norm(y)


def test_fgmres_dense():
    rng = np.random.default_rng(1)
    n = 30
    M = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) / np.sqrt(n) + 3 * np.eye(n)
    b = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    ref = np.linalg.solve(M, b)
    x, res, hst = ML.fgmres(lambda v: M @ v, b, None, tol=1e-10, maxit=50, maxinnerit=5)
    assert np.linalg.norm(x - ref) <= 1e-8 * np.linalg.norm(ref)
    D = np.diag(1.0 / np.diag(M))
    x2, _, hst2 = ML.fgmres(lambda v: M @ v, b, None, tol=1e-10, maxit=50, maxinnerit=5, precond=lambda v: D @ v)
    assert np.linalg.norm(x2 - ref) <= 1e-8 * np.linalg.norm(ref)


def test_ml_gmres_solves_small_helmholtz():
    rng = np.random.default_rng(0)
    n, h = (17, 15, 13), 25.0
    z = np.arange(n[2]) * h
    v = np.broadcast_to(1500 + 1000 * z / z[-1], n).copy() * (1 + 0.05 * rng.standard_normal(n))
    levels, R, P = ML.build_levels(v, (h, h, h), 6, 4.0, "m/s")
    assert [l.nt for l in levels] == [(29, 27, 25), (15, 14, 13), (9, 8, 8)]
    b = np.zeros(levels[0].N, complex)
    nx, ny, _ = levels[0].nt
    b[nx // 2 + nx * (ny // 2) + nx * ny * 9] = 1.0
    x, res, hst = ML.ml_gmres_solve(levels, R, P, b, tol=1e-6)
    r = b - levels[0].A(x)
    assert np.linalg.norm(r) / np.linalg.norm(b) <= 1e-6
    assert len(hst) - 1 <= 25


def test_library_interpolation_weights_match_oracle():
    """The library's host-side set-up (h3d.multigrid: cubic model coarsening and linear grid
    transfer weights) against the oracle's restatement, on the grid pairs the levels use."""
    import sys, os
    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "..", "slim-release-apps_gb300"))
    from h3d import multigrid as MG

    g = lambda m: np.linspace(0.0, 1.0, m)
    for n, nc in ((61, 31), (201, 101), (101, 51), (29, 15), (16, 8)):
        A = MG.cubic_weights(g(n), g(nc))
        B = ML.cubic_interp_1d(g(n), g(nc)).toarray()
        assert np.max(np.abs(A - B)) <= 1e-13
        A = MG.linear_weights(g(nc), g(n))
        B = ML.lin_interp_1d(g(nc), g(n)).toarray()
        assert np.max(np.abs(A - B)) <= 1e-13
    rng = np.random.default_rng(4)
    v = rng.random((23, 19, 17)) + 1.0
    f2c, _, ns = ML.fine2coarse(v.shape, (1.0, 1.0, 1.0), (2.0, 2.0, 2.0), "cubic")
    ref = (f2c * v.reshape(-1, order="F")).reshape(ns, order="F")
    assert np.max(np.abs(MG._coarsen_model(v, ns) - ref)) <= 1e-12


def test_fgmres_restart_cycles_match_scipy_gmres():
    """FGMRES.m restarted every m steps is GMRES(m) (identity preconditioner) and, with a
    fixed right preconditioner D, GMRES(m) on A D: the oracle's restatement equals scipy's
    independent GMRES after the same number of restart cycles (the library's device FGMRES
    is held to the same scipy solution on the GPU)."""
    from scipy.sparse.linalg import gmres

    rng = np.random.default_rng(3)
    n = 40
    A = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) / np.sqrt(n) + 2.5 * np.eye(n)
    b = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    D = np.diag(1.0 + rng.random(n))
    for m, c in ((5, 3), (8, 2), (4, 6)):
        ref, _ = gmres(A, b, rtol=1e-30, atol=0.0, restart=m, maxiter=c)
        xo, _, hsto = ML.fgmres(lambda v: A @ v, b, None, tol=1e-30, maxit=c, maxinnerit=m)
        assert np.linalg.norm(xo - ref) <= 1e-12 * np.linalg.norm(ref)
        assert len(hsto) == c * m + 1
        yref, _ = gmres(A @ D, b, rtol=1e-30, atol=0.0, restart=m, maxiter=c)
        xo, _, _ = ML.fgmres(lambda v: A @ v, b, None, tol=1e-30, maxit=c, maxinnerit=m, precond=lambda v: D @ v)
        assert np.linalg.norm(xo - D @ yref) <= 1e-12 * np.linalg.norm(D @ yref)


def test_library_levels_and_transfers_match_oracle():
    """h3d.multigrid.build_levels (built on CPU tensors: the grids, PML widths, spacings and
    wavenumbers of the three levels, and the CSR axis operators of the transfers) against the
    oracle's construct_multigrid restatement, operator by operator."""
    import os
    import sys

    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "..", "slim-release-apps_gb300"))
    import scipy.sparse as sp
    from h3d import multigrid as MG

    rng = np.random.default_rng(0)
    n, h = (17, 15, 13), 25.0
    z = np.arange(n[2]) * h
    v = np.broadcast_to(1500 + 1000 * z / z[-1], n).copy() * (1 + 0.05 * rng.standard_normal(n))
    lv, R, P = MG.build_levels(v, (h, h, h), 6, 4.0, "m/s", device="cpu")
    levels, Ro, Po = ML.build_levels(v, (h, h, h), 6, 4.0, "m/s")
    for a, b in zip(lv, levels):
        assert a.nt == b.nt and a.npml == b.npml and a.dt == b.dt
        assert np.max(np.abs(a.wn.numpy() - b.wn)) <= 1e-15 * np.max(np.abs(b.wn))

    def sparse(tr):
        mats = []
        for op in tr.ops:
            rp, col, val = op.rowptr.numpy(), op.col.numpy(), op.val.numpy()
            mats.append(sp.csr_matrix((val, col, rp), shape=(op.n_out, op.n_in)))
        Ax, Ay, Az = mats
        return tr.scale * sp.kron(Az, sp.kron(Ay, Ax), format="csr")

    def sparse_o(op):
        A1, A2, A3 = (sp.csr_matrix(a) for a in op.A)
        return sp.kron(A3, sp.kron(A2, A1), format="csr")

    for i in range(len(P)):
        assert abs(sparse(P[i]) - sparse_o(Po[i])).max() <= 1e-14
        f2c, s = Ro[i]
        assert abs(sparse(R[i]) - s * sparse_o(f2c)).max() <= 1e-14


def test_library_hierarchy_from_the_model_matches_oracle():
    """h3d_ml_levels_host (what h3d_mlgmres_solve_model and the h3d_mlgmres_mex gateway build):
    level grids, spacings, PML widths and wavenumbers against the oracle's construct_multigrid
    restatement, in each model unit."""
    import ctypes as C
    import os
    import sys

    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "..", "slim-release-apps_gb300"))
    from h3d import _lib as L

    lib = L.load()
    rng = np.random.default_rng(11)
    n, h, npml = (17, 15, 13), (25.0, 20.0, 30.0), 6
    v = 1500.0 + 1000.0 * rng.random(n)
    for unit, vv in (("m/s", v), ("s2/m2", v ** -2.0), ("s2/km2", 1e6 * v ** -2.0)):
        ref, _, _ = ML.build_levels(vv, h, npml, 4.0, unit)
        grids = (L.Grid * 3)()
        wn = np.zeros(sum(lv.N for lv in ref))
        src = np.ascontiguousarray(vv.reshape(-1, order="F"))
        hh = np.asarray(h, float)
        rc = lib.h3d_ml_levels_host(src.ctypes.data_as(L.dp), (C.c_int32 * 3)(*n), hh.ctypes.data_as(L.dp), npml,
                                    4.0, L.UNITS[unit], 3, grids, wn.ctypes.data_as(L.dp), wn.size)
        assert rc == L.OK
        off = 0
        for i, lv in enumerate(ref):
            assert tuple(grids[i].n) == lv.nt
            assert tuple(grids[i].h) == lv.dt
            assert set(grids[i].npml) == {lv.npml}
            w = wn[off:off + lv.N]
            off += lv.N
            assert np.max(np.abs(w - lv.wn)) <= 1e-12 * np.max(np.abs(lv.wn))
    small = np.zeros(10)
    rc = lib.h3d_ml_levels_host(src.ctypes.data_as(L.dp), (C.c_int32 * 3)(*n), hh.ctypes.data_as(L.dp), npml, 4.0,
                                0, 3, grids, small.ctypes.data_as(L.dp), small.size)
    assert rc == L.ERR_BAD_ARG and b"levels need" in lib.h3d_last_error()


def _device_formulation_fgmres(A, b, tol, maxit, m, precond=None):
    """The arithmetic h3d_mlgmres.cu runs, restated step by step on the CPU: classical
    Gram-Schmidt; the new Givens rotation from reciprocal square roots (c = |a| / r,
    s = (a / |a|) ||w|| / r, the quasi-residual carried as |s| times the previous one); an
    unnormalised basis with one scale per vector when there is no preconditioner (vector 0 is
    the residual itself); y back-substituted once per cycle; the stopping flags of the state
    block (a step runs while the quasi-residual exceeds tol, a cycle ends with the true
    residual's break test).  x0 = 0."""
    n = b.size
    lazy = precond is None
    r = b.copy()
    x = np.zeros_like(b)
    normr0 = np.linalg.norm(r)
    hst = [1.0]
    live = normr0 != 0.0 and 1.0 > tol and (1 // m) < maxit
    it = 1
    for _ in range(maxit):
        if not live:
            break
        beta = np.linalg.norm(r)
        U = np.zeros((m + 1, n), complex)
        sv = np.zeros(m + 1)
        Z = np.zeros((m, n), complex)
        cs = np.zeros(m)
        sn = np.zeros(m, complex)
        g = np.zeros(m + 1, complex)
        R = np.zeros((m, m), complex)
        g[0] = beta
        gres = beta
        if lazy:
            U[0], sv[0] = r, 1.0 / beta
        else:
            U[0], sv[0] = r / beta, 1.0
        k = 0
        for j in range(m):
            vj = sv[j] * U[j] if lazy else U[j]
            if precond is not None:
                Z[j] = precond(U[j])
                w_raw = A(Z[j])
            else:
                w_raw = A(U[j])
            raw = U[:j + 1].conj() @ w_raw
            h = sv[:j + 1] * sv[j] * raw if lazy else raw
            w = (sv[j] if lazy else 1.0) * w_raw - (U[:j + 1].T @ ((sv[:j + 1] if lazy else 1.0) * h))
            w2 = float(np.vdot(w, w).real)
            rhn = w2 ** -0.5 if w2 > 0 else 0.0
            hn = w2 * rhn
            c = h.astype(complex).copy()
            for i in range(j):
                t = cs[i] * c[i] + sn[i] * c[i + 1]
                c[i + 1] = cs[i] * c[i + 1] - np.conj(sn[i]) * c[i]
                c[i] = t
            a = c[j]
            na2 = abs(a) ** 2
            if w2 == 0.0:
                cj, sj, sabs, rjj = 1.0, 0.0, 0.0, a
            elif na2 == 0.0:
                cj, sj, sabs, rjj = 0.0, 1.0, 1.0, hn
            else:
                r2 = na2 + w2
                rr, rna = r2 ** -0.5, na2 ** -0.5
                ph = rna * a
                cj, sabs = na2 * rna * rr, hn * rr
                sj, rjj = sabs * ph, (r2 * rr) * ph
            c[j] = rjj
            cs[j], sn[j] = cj, sj
            R[:j + 1, j] = c
            g[j + 1] = -np.conj(sj) * g[j]
            g[j] = cj * g[j]
            gres = sabs * gres
            q = gres / normr0
            hst.append(q)
            it += 1
            k = j + 1
            if j + 1 < m:
                if lazy:
                    U[j + 1], sv[j + 1] = w, rhn
                else:
                    U[j + 1], sv[j + 1] = w * rhn, 1.0
            if not (q > tol and j + 1 < m):
                break
        y = np.zeros(k, complex)
        for i in range(k - 1, -1, -1):
            t = g[i] - R[i, i + 1:k] @ y[i + 1:k]
            d = R[i, i]
            y[i] = 0.0 if abs(d) == 0.0 else t / d
        basis = Z[:k] if precond is not None else (sv[:k, None] * U[:k] if lazy else U[:k])
        x = x + basis.T @ y
        r = b - A(x)
        rn = np.linalg.norm(r)
        if rn / normr0 < tol:
            live = False
        else:
            live = hst[-1] > tol and (it // m) < maxit
    return x, np.array(hst)


def test_device_fgmres_formulation_matches_oracle():
    """The device formulation (reciprocal-square-root Givens rotations, unnormalised basis,
    once-per-cycle back substitution, flag-driven stopping) gives FGMRES.m's iterates: same
    quasi-residual history and solution as the oracle's restatement with numpy lstsq, with and
    without a preconditioner, and through a breakdown (numerical and exact, ||w|| = 0)."""
    rng = np.random.default_rng(21)
    n = 30
    A = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) / np.sqrt(n) + 1.5 * np.eye(n)
    b = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    D = np.diag(1.0 + rng.random(n))
    for m, maxit, tol in ((5, 3, 1e-30), (4, 6, 1e-8), (8, 2, 1e-4)):
        for pre in (None, lambda v: D @ v):
            x_ref, _, h_ref = ML.fgmres(lambda v: A @ v, b, None, tol=tol, maxit=maxit, maxinnerit=m,
                                        precond=pre)
            x, h = _device_formulation_fgmres(lambda v: A @ v, b, tol, maxit, m, precond=pre)
            assert len(h) == len(h_ref)
            np.testing.assert_allclose(h, h_ref, rtol=1e-9, atol=1e-14)
            assert np.linalg.norm(x - x_ref) <= 1e-10 * np.linalg.norm(x_ref)
    # b in a 3-dimensional invariant subspace: ||w|| falls to rounding level at step 3
    Q, _ = np.linalg.qr(rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
    lam = np.concatenate([[2.0, 3.0 + 1j, 0.5 - 2j], 1.0 + rng.random(n - 3)])
    Ab = Q @ np.diag(lam) @ Q.conj().T
    bb = Q[:, :3] @ np.array([1.0, 2.0 - 1j, 0.5])
    x, h = _device_formulation_fgmres(lambda v: Ab @ v, bb, 1e-12, 3, 5)
    assert len(h) <= 5 and h[-1] <= 1e-10
    assert np.linalg.norm(Ab @ x - bb) <= 1e-10 * np.linalg.norm(bb)
    # exact breakdown (the ||w|| = 0 branch): b an eigenvector of a diagonal A
    Ad = np.diag(np.arange(1.0, n + 1.0) * (1.0 + 0.5j))
    e1 = np.zeros(n, complex)
    e1[0] = 2.0
    for pre in (None, lambda v: v):
        x, h = _device_formulation_fgmres(lambda v: Ad @ v, e1, 1e-12, 3, 5, precond=pre)
        with np.errstate(invalid="ignore", divide="ignore"):   # FGMRES.m:103 forms V(:,2) = 0/0, unused
            x_ref, _, h_ref = ML.fgmres(lambda v: Ad @ v, e1, None, tol=1e-12, maxit=3, maxinnerit=5, precond=pre)
        np.testing.assert_allclose(h, h_ref, atol=1e-15)
        assert list(h) == [1.0, 0.0]
        np.testing.assert_allclose(x, x_ref, rtol=1e-15)
