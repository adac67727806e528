"""The C oracle against golden vectors produced by the reference's own MEX code.

The goldens (tests/golden/*.npz, generated by tests/golden/make_golden.py from the
reference gateways compiled unmodified) pin the restatement in oracle/h3d_oracle.c.
Runs on CPU; where the reference checkout and its compiled gateways are present the
restatement is also compared with them directly on fresh random inputs.
"""
import numpy as np
import pytest

from oracle import h3d_oracle as O
from oracle import mexharness as M

MVP = [("forw", 0, 0), ("adj", 1, 0), ("forw_deriv", 0, 1), ("adj_deriv", 1, 1),
       ("forw_wnc", 0, 0), ("adj_wnc", 1, 0)]


def _grid(gs, tag):
    n = gs[f"{tag}/n"].astype(int)
    npml = gs[f"{tag}/npml"]
    return O.make_grid(n, gs[f"{tag}/h"], npml.T.reshape(-1))


@pytest.mark.parametrize("tag", ["g7", "g12"])
@pytest.mark.parametrize("var,adj,deriv", MVP)
def test_mvp_matches_reference_golden(golden_small, tag, var, adj, deriv):
    gs = golden_small
    g = _grid(gs, tag)
    wn = gs[f"{tag}/wnc"] if var.endswith("wnc") else (gs[f"{tag}/dwn"] if deriv else gs[f"{tag}/wn"])
    y = O.mvp(g, wn, gs[f"{tag}/x"], adj=adj, deriv=deriv, nthreads=2)
    ref = gs[f"{tag}/mvp_{var}"]
    assert np.max(np.abs(y - ref)) <= 1e-14 * np.max(np.abs(ref))


@pytest.mark.parametrize("tag", ["g7", "g12"])
def test_sweeps_match_reference_golden(golden_small, tag):
    gs = golden_small
    g = _grid(gs, tag)
    X, B = gs[f"{tag}/X"], gs[f"{tag}/B"]
    cases = [
        ("swp_forw", gs[f"{tag}/wn"], 0, X, B),
        ("swp_adj", gs[f"{tag}/wn"], 1, X, B),
        ("swp_wnc", gs[f"{tag}/wnc"], 0, X, B),
        ("swp_wnc_installed", gs[f"{tag}/wnc"].real.copy(), 0, X, B),
        ("swp_forw_b0", gs[f"{tag}/wn"], 0, X, np.zeros_like(B)),
        ("swp_adj_x0", gs[f"{tag}/wn"], 1, np.zeros_like(X), B),
    ]
    for key, wn, adj, x, b in cases:
        y = O.sweep(g, wn, 1.5, x, b, adj=adj, order=O.ORDER_LEX, nthreads=2)
        ref = gs[f"{tag}/{key}"]
        assert np.max(np.abs(y - ref)) <= 1e-13 * np.max(np.abs(ref)), key


def test_adjoint_dot_product():
    rng = np.random.default_rng(5)
    n = (9, 8, 7)
    g = O.make_grid(n, (20.0, 25.0, 30.0), (2, 3, 1, 2, 2, 2))
    N = int(np.prod(n))
    wn = (2 * np.pi * 5) ** 2 / (1500 + 1000 * rng.random(N)) ** 2
    for deriv in (0, 1):
        x = rng.standard_normal(N) + 1j * rng.standard_normal(N)
        y = rng.standard_normal(N) + 1j * rng.standard_normal(N)
        a = np.vdot(y, O.mvp(g, wn, x, adj=0, deriv=deriv))
        b = np.vdot(O.mvp(g, wn, y, adj=1, deriv=deriv), x)
        assert abs(a - b) <= 1e-13 * abs(a)


@pytest.mark.parametrize("order", [O.ORDER_LEX, O.ORDER_COLOUR27, O.ORDER_BLOCK, O.ORDER_BLOCK8])
def test_double_sweep_symmetric_psd(order):
    """test_DoubleKaczmarzSweep.m:125-199 properties for every ordering: with
    Q y = DSWP(y, 0), the operator I - Q is Hermitian and positive semi-definite."""
    rng = np.random.default_rng(9)
    n = (7, 6, 8)
    g = O.make_grid(n, (25.0, 25.0, 25.0), 2)
    N = int(np.prod(n))
    wn = (2 * np.pi * 4) ** 2 / (1500 + 2000 * rng.random(N)) ** 2
    blk = (3, 3, 4)

    def A(v):
        return v - O.sweep(g, wn, 1.5, v, None, order=order, blk=blk, nthreads=1)

    x = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    y = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    lhs, rhs = np.vdot(y, A(x)), np.vdot(A(y), x)
    assert abs(lhs - rhs) <= 1e-10 * abs(lhs)
    for _ in range(3):
        v = rng.standard_normal(N) + 1j * rng.standard_normal(N)
        assert np.vdot(v, A(v)).real >= -1e-12 * np.vdot(v, v).real


def test_colour_orders_differ_from_lex_but_block_whole_grid_is_colour27():
    rng = np.random.default_rng(3)
    n = (6, 6, 6)
    g = O.make_grid(n, (25.0, 25.0, 25.0), 2)
    N = int(np.prod(n))
    wn = (2 * np.pi * 4) ** 2 / (2000 * np.ones(N)) ** 2
    x = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    c27 = O.sweep(g, wn, 1.5, x, None, order=O.ORDER_COLOUR27, nthreads=1)
    blk = O.sweep(g, wn, 1.5, x, None, order=O.ORDER_BLOCK, blk=(6, 6, 6), nthreads=1)
    blk8 = O.sweep(g, wn, 1.5, x, None, order=O.ORDER_BLOCK8, blk=(6, 6, 6), nthreads=1)
    lex = O.sweep(g, wn, 1.5, x, None, order=O.ORDER_LEX, nthreads=1)
    assert np.allclose(c27, blk, rtol=0, atol=1e-14 * np.abs(c27).max())
    assert np.allclose(c27, blk8, rtol=0, atol=1e-14 * np.abs(c27).max())
    blk8b = O.sweep(g, wn, 1.5, x, None, order=O.ORDER_BLOCK8, blk=(3, 3, 3), nthreads=1)
    assert not np.allclose(c27, blk8b)
    assert not np.allclose(c27, lex)


@pytest.mark.skipif(not M.reference_available(), reason="reference gateways not compiled here")
def test_oracle_bitwise_against_compiled_reference():
    rng = np.random.default_rng(21)
    n = (10, 9, 11)
    npml = np.array([[2, 3, 2], [2, 3, 2]], float)
    g = O.make_grid(n, (20.0, 20.0, 10.0), npml.T.reshape(-1))
    N = int(np.prod(n))
    wn = (2 * np.pi * 3) ** 2 / (1500 + 2000 * rng.random(N)) ** 2
    x = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    hv, nv = np.array([20.0, 20.0, 10.0]), np.array(n, float)
    assert np.array_equal(O.mvp(g, wn, x, adj=1), M.load_reference("Helm3dmvp_adj_mex")(wn, hv, nv, npml, x, 2.0)[:, 0])
    X = rng.standard_normal((N, 2)) + 1j * rng.standard_normal((N, 2))
    B = rng.standard_normal((N, 2)) + 1j * rng.standard_normal((N, 2))
    assert np.array_equal(O.sweep(g, wn, 1.2, X, B), M.load_reference("Helm3d_kacz_sweep_mex")(wn, hv, nv, npml, 1.2, X, B))


def test_config0_golden_input_checksums():
    from h3d import models

    c0 = np.load(__import__("os").path.join(__import__("os").path.dirname(__file__), "golden", "config0_mvp.npz"))
    m = models.config0()
    wn = m.wavenumber()
    np.testing.assert_allclose([wn.sum(), np.linalg.norm(wn), wn.min(), wn.max()], c0["wn_checksum"], rtol=1e-12)


def test_band_oracle_matches_reference_golden(golden_band):
    """oracle/slim_band.py against the committed outputs of the compiled band gateways."""
    from oracle import slim_band as SB

    g = golden_band
    n = tuple(int(v) for v in g["n"])
    H, idx = SB.helmholtz_3d_bands(g["wn"].reshape(n, order="F"), g["h"], g["npml"])
    assert np.array_equal(H, g["H"]) and np.array_equal(idx, g["idx"])
    for tag, A, o in (("forw", g["H"], g["idx"]), ("adj", g["Hadj"], g["idxadj"])):
        y = SB.band_mvp(A, o, g["X"])
        assert np.abs(y - g[f"{tag}/mvp"]).max() <= 4e-16 * np.abs(g[f"{tag}/mvp"]).max()
        assert np.array_equal(SB.band_sweep(A, o, g["X"], g["B"], 1.3, g[f"{tag}/rn"]), g[f"{tag}/swp"])
