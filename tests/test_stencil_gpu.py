"""GPU parity of the stencil kernels against the reference goldens and the C oracle.

All calls go through libh3d.so's C ABI (via h3d.ops / the MEX gateways).
Tolerances: FP64 matvec 1e-13 relative (max-norm), FP64 sweeps 1e-12, complex64
kernels 2e-5 relative to the FP64 result.
"""
import os

import numpy as np
import pytest

from oracle import h3d_oracle as O

pytestmark = pytest.mark.gpu

MVP = [("forw", 1, 0), ("adj", 2, 0), ("forw_deriv", 1, 1), ("adj_deriv", 2, 1),
       ("forw_wnc", 1, 0), ("adj_wnc", 2, 0)]


def _t(a, dev, dtype=None):
    import torch

    return torch.as_tensor(np.ascontiguousarray(a), device=dev, dtype=dtype)


def _rel(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


def _grid_args(gs, tag):
    n = gs[f"{tag}/n"].astype(int)
    return (n, gs[f"{tag}/h"], gs[f"{tag}/npml"])


@pytest.mark.parametrize("tag", ["g7", "g12"])
@pytest.mark.parametrize("var,mode,deriv", MVP)
def test_mvp_fp64_matches_reference(cuda, golden_small, tag, var, mode, deriv):
    import torch
    from h3d import ops

    gs = golden_small
    wn = gs[f"{tag}/wnc"] if var.endswith("wnc") else (gs[f"{tag}/dwn"] if deriv else gs[f"{tag}/wn"])
    y = ops.mvp(_grid_args(gs, tag), _t(wn, cuda), _t(gs[f"{tag}/x"], cuda, torch.complex128), mode, deriv)
    assert _rel(y.cpu().numpy(), gs[f"{tag}/mvp_{var}"]) <= 1e-13


@pytest.mark.parametrize("var,mode,deriv", MVP)
def test_mvp_c64_close_to_fp64(cuda, golden_small, var, mode, deriv):
    import torch
    from h3d import ops

    gs, tag = golden_small, "g12"
    wn = gs[f"{tag}/wnc"] if var.endswith("wnc") else (gs[f"{tag}/dwn"] if deriv else gs[f"{tag}/wn"])
    wt = _t(wn.astype(np.complex64) if np.iscomplexobj(wn) else wn.astype(np.float32), cuda)
    y = ops.mvp(_grid_args(gs, tag), wt, _t(gs[f"{tag}/x"], cuda, torch.complex64), mode, deriv)
    assert y.dtype == torch.complex64
    assert _rel(y.cpu().numpy().astype(np.complex128), gs[f"{tag}/mvp_{var}"]) <= 2e-5


def test_mvp_multi_rhs(cuda, golden_small):
    import torch
    from h3d import ops

    gs, tag = golden_small, "g12"
    X = gs[f"{tag}/X"]  # N x P (column-major in the reference)
    y = ops.mvp(_grid_args(gs, tag), _t(gs[f"{tag}/wn"], cuda), _t(X.T, cuda, torch.complex128), 1, False)
    g = O.make_grid(gs[f"{tag}/n"].astype(int), gs[f"{tag}/h"], gs[f"{tag}/npml"].T.reshape(-1))
    ref = O.mvp(g, gs[f"{tag}/wn"], X)
    assert _rel(y.cpu().numpy().T, ref) <= 1e-13


@pytest.mark.parametrize("tag", ["g7", "g12"])
def test_lex_sweep_matches_reference(cuda, golden_small, tag):
    import torch
    from h3d import ops

    gs = golden_small
    X, B = gs[f"{tag}/X"].T, gs[f"{tag}/B"].T
    cases = [("swp_forw", gs[f"{tag}/wn"], 1, X, B), ("swp_adj", gs[f"{tag}/wn"], 2, X, B),
             ("swp_wnc", gs[f"{tag}/wnc"], 1, X, B),
             ("swp_forw_b0", gs[f"{tag}/wn"], 1, X, None),
             ("swp_adj_x0", gs[f"{tag}/wn"], 2, np.zeros_like(X), B)]
    for key, wn, mode, x, b in cases:
        y = ops.kacz_sweep(_grid_args(gs, tag), _t(wn, cuda), 1.5, _t(x, cuda, torch.complex128),
                           None if b is None else _t(b, cuda, torch.complex128), mode, order=0)
        assert _rel(y.cpu().numpy().T, gs[f"{tag}/{key}"]) <= 1e-12, key


# COLOUR27 twice: on stored row coefficients (block None) and with the shared-memory tile
# kernel (block[0] = -1)
@pytest.mark.parametrize("order,blk", [(1, None), (1, (-1, 0, 0)), (2, (8, 8, 8)), (2, (16, 8, 8))])
@pytest.mark.parametrize("mode", [1, 2])
def test_reordered_sweeps_match_oracle(cuda, golden_small, order, blk, mode):
    import torch
    from h3d import ops

    gs, tag = golden_small, "g12"
    g = O.make_grid(gs[f"{tag}/n"].astype(int), gs[f"{tag}/h"], gs[f"{tag}/npml"].T.reshape(-1))
    X, B, wn = gs[f"{tag}/X"], gs[f"{tag}/B"], gs[f"{tag}/wn"]
    ref = O.sweep(g, wn, 1.5, X, B, adj=(mode == 2), order=order, blk=None if order == 1 else blk, nthreads=2)
    y = ops.kacz_sweep(_grid_args(gs, tag), _t(wn, cuda), 1.5, _t(X.T, cuda, torch.complex128),
                       _t(B.T, cuda, torch.complex128), mode, order=order, block=blk)
    assert _rel(y.cpu().numpy().T, ref) <= 1e-12
    # complex64 kernels: same ordering, single precision
    y32 = ops.kacz_sweep(_grid_args(gs, tag), _t(wn.astype(np.float32), cuda), 1.5,
                         _t(X.T, cuda, torch.complex64), _t(B.T, cuda, torch.complex64), mode,
                         order=order, block=blk)
    assert _rel(y32.cpu().numpy().T.astype(np.complex128), ref) <= 5e-5


# BLOCK8 12^3 on stored coefficients (12, 12, 12) and forming them itself (-1, 0, 0)
@pytest.mark.parametrize("order,blk", [(3, (12, 12, 12)), (3, (-1, 0, 0)), (3, (24, 12, 12)), (1, None),
                                       (1, (-1, 0, 0))])
@pytest.mark.parametrize("mode,wnc", [(1, False), (2, False), (1, True), (2, True)])
def test_block8_and_colour27_sweeps_match_oracle(cuda, order, blk, mode, wnc):
    """BLOCK8 (parity classes of blocks) on a grid of several blocks per axis and COLOUR27
    (stored coefficients / tile kernel), three right-hand sides (a partly filled group of
    two for BLOCK8 12^3), real and complex wavenumber, against the C oracle."""
    import torch
    from h3d import ops

    n, h, npml = (29, 27, 26), (25.0, 22.0, 20.0), (3, 4, 2, 3, 4, 2)
    rng = np.random.default_rng(31)
    N = int(np.prod(n))
    g = O.make_grid(n, h, npml)
    wn = (2 * np.pi * 5.0) ** 2 / (1500.0 + 1500.0 * rng.random(N)) ** 2
    if wnc:
        wn = wn * (1.0 + 0.05j * rng.random(N))
    X = rng.standard_normal((N, 3)) + 1j * rng.standard_normal((N, 3))
    B = rng.standard_normal((N, 3)) + 1j * rng.standard_normal((N, 3))
    oblk = None if order != 3 else ((12, 12, 12) if blk[0] == -1 else blk)
    ref = O.sweep(g, wn, 1.5, X, B, adj=(mode == 2), order=order, blk=oblk, nthreads=2)
    grid = (n, h, npml)
    y = ops.kacz_sweep(grid, _t(wn, cuda), 1.5, _t(X.T, cuda, torch.complex128), _t(B.T, cuda, torch.complex128),
                       mode, order=order, block=blk)
    assert _rel(y.cpu().numpy().T, ref) <= 1e-12
    wn32 = wn.astype(np.complex64) if wnc else wn.astype(np.float32)
    y32 = ops.kacz_sweep(grid, _t(wn32, cuda), 1.5, _t(X.T, cuda, torch.complex64), _t(B.T, cuda, torch.complex64),
                         mode, order=order, block=blk)
    assert _rel(y32.cpu().numpy().T.astype(np.complex128), ref) <= 5e-5


@pytest.mark.parametrize("blk", [(12, 12, 12), (-1, 0, 0)])
@pytest.mark.parametrize("nrhs", [1, 5])
@pytest.mark.parametrize("mode", [1, 2])
def test_block8_rhs_groups_match_oracle(cuda, blk, nrhs, mode):
    """BLOCK8 12^3 kernels by right-hand-side group: one right-hand side per block, and five
    in groups of four (the second group partly filled)."""
    import torch
    from h3d import ops

    n, h, npml = (26, 25, 27), (20.0, 20.0, 20.0), (4, 4, 4, 4, 4, 4)
    rng = np.random.default_rng(41 + nrhs)
    N = int(np.prod(n))
    g = O.make_grid(n, h, npml)
    wn = (2 * np.pi * 5.0) ** 2 / (1500.0 + 1500.0 * rng.random(N)) ** 2
    X = rng.standard_normal((N, nrhs)) + 1j * rng.standard_normal((N, nrhs))
    B = rng.standard_normal((N, nrhs)) + 1j * rng.standard_normal((N, nrhs))
    ref = O.sweep(g, wn, 1.5, X, B, adj=(mode == 2), order=O.ORDER_BLOCK8, blk=(12, 12, 12), nthreads=2)
    grid = (n, h, npml)
    y = ops.kacz_sweep(grid, _t(wn, cuda), 1.5, _t(X.T, cuda, torch.complex128), _t(B.T, cuda, torch.complex128),
                       mode, order=3, block=blk)
    assert _rel(y.cpu().numpy().T, ref) <= 1e-12
    y32 = ops.kacz_sweep(grid, _t(wn.astype(np.float32), cuda), 1.5, _t(X.T, cuda, torch.complex64),
                         _t(B.T, cuda, torch.complex64), mode, order=3, block=blk)
    assert _rel(y32.cpu().numpy().T.astype(np.complex128), ref) <= 5e-5


@pytest.mark.parametrize("mode", [1, 2])
def test_mvp_interior_fast_path_matches_oracle(cuda, mode):
    """A grid wide enough for whole 32 x 8 column blocks inside the x/y interior, where the
    matvec folds the PML brackets (rows inside and outside the z interior), against the C
    oracle: FP64 to 1e-13, complex64 to 2e-5."""
    import torch
    from h3d import ops

    n, h, npml = (100, 42, 30), (20.0, 22.0, 25.0), (4, 4, 4, 4, 4, 4)
    rng = np.random.default_rng(5)
    N = int(np.prod(n))
    g = O.make_grid(n, h, npml)
    wn = (2 * np.pi * 5.0) ** 2 / (1500.0 + 1500.0 * rng.random(N)) ** 2
    X = rng.standard_normal((N, 2)) + 1j * rng.standard_normal((N, 2))
    ref = O.mvp(g, wn, X, adj=(mode == 2))
    y = ops.mvp((n, h, npml), _t(wn, cuda), _t(X.T, cuda, torch.complex128), mode)
    assert _rel(y.cpu().numpy().T, ref) <= 1e-13
    y32 = ops.mvp((n, h, npml), _t(wn.astype(np.float32), cuda), _t(X.T, cuda, torch.complex64), mode)
    assert _rel(y32.cpu().numpy().T.astype(np.complex128), ref) <= 2e-5


def test_config0_matvec_golden(cuda):
    """61^3, PML 10: the forward and adjoint matvecs of a seeded complex128 vector,
    against the reference's own output (sampled entries, norm and a probe product)."""
    import torch
    from h3d import models, ops

    c0 = np.load(os.path.join(os.path.dirname(__file__), "golden", "config0_mvp.npz"))
    m = models.config0()
    N = m.N
    rng = np.random.default_rng(20240)
    x = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    np.testing.assert_allclose([x.real.sum(), x.imag.sum(), np.linalg.norm(x)], c0["x_checksum"], rtol=1e-12)
    srng = np.random.default_rng(7)
    srng.choice(N, size=4096, replace=False)
    probe = srng.standard_normal(N) + 1j * srng.standard_normal(N)
    for tag, mode in (("forw", 1), ("adj", 2)):
        y = ops.mvp((m.n_total, m.h, m.npml6), _t(m.wavenumber(), cuda), _t(x, cuda, torch.complex128),
                    mode).cpu().numpy()
        idx = c0[f"{tag}/idx"]
        ref = c0[f"{tag}/samples"]
        assert np.max(np.abs(y[idx] - ref)) <= 1e-13 * np.max(np.abs(ref))
        assert abs(np.linalg.norm(y) - c0[f"{tag}/norm"]) <= 1e-13 * c0[f"{tag}/norm"]
        pd = np.vdot(probe, y)
        assert abs(pd - c0[f"{tag}/probe_dot"]) <= 1e-12 * abs(c0[f"{tag}/probe_dot"])


def test_config1_adjoint_identity(cuda):
    """Full-size (201 x 201 x 101) property check: <y, H x> = <H^H y, x> for the FP64
    kernels, and the complex64 kernels agree with FP64 to single precision."""
    import torch
    from h3d import models, ops

    m = models.config1()
    grid = (m.n_total, m.h, m.npml6)
    wn = _t(m.wavenumber(), cuda)
    gen = torch.Generator(device=cuda).manual_seed(0)
    x = torch.randn(m.N, dtype=torch.complex128, device=cuda, generator=gen)
    y = torch.randn(m.N, dtype=torch.complex128, device=cuda, generator=gen)
    hx = ops.mvp(grid, wn, x, 1)
    hty = ops.mvp(grid, wn, y, 2)
    a = torch.vdot(y, hx).item()
    b = torch.vdot(hty, x).item()
    assert abs(a - b) <= 1e-12 * abs(a)
    hx32 = ops.mvp(grid, wn.float(), x.to(torch.complex64), 1)
    err = (hx32.to(torch.complex128) - hx).abs().max() / hx.abs().max()
    assert err.item() <= 2e-5


def test_mex_gateways_drop_in(cuda, golden_small):
    """The drop-in gateways (same names and argument lists as the reference binaries)
    reproduce the reference outputs, including its error identifiers."""
    from h3d import build
    from oracle import mexharness as M

    gws = build.build_mex()
    gs, tag = golden_small, "g12"
    n, h, npml = gs[f"{tag}/n"], gs[f"{tag}/h"], gs[f"{tag}/npml"]
    for var, mode, deriv in MVP:
        wn = gs[f"{tag}/wnc"] if var.endswith("wnc") else (gs[f"{tag}/dwn"] if deriv else gs[f"{tag}/wn"])
        f = M.MexFunction(gws[f"Helm3dmvp_{var}_mex"])
        y = f(wn, h, n, npml, gs[f"{tag}/x"], 4.0)[:, 0]
        assert _rel(y, gs[f"{tag}/mvp_{var}"]) <= 1e-13, var
    X, B = gs[f"{tag}/X"], gs[f"{tag}/B"]
    for name, key, wn in (("Helm3d_kacz_sweep_mex", "swp_forw", gs[f"{tag}/wn"]),
                          ("Helm3d_kacz_sweep_adj_mex", "swp_adj", gs[f"{tag}/wn"]),
                          ("Helm3d_kacz_sweep_wnc_mex", "swp_wnc", gs[f"{tag}/wnc"])):
        y = M.MexFunction(gws[name])(wn, h, n, npml, 1.5, X, B)
        assert _rel(y, gs[f"{tag}/{key}"]) <= 1e-12, name
    f = M.MexFunction(gws["Helm3dmvp_forw_mex"])
    with pytest.raises(M.MexError) as e:
        f(gs[f"{tag}/wn"], h, n, npml, gs[f"{tag}/x"][:-1], 4.0)
    assert e.value.ident == "SLIM_release_apps:tools:algorithms:ThreeDFreqModeling:Helm3dkaczswp_mex:Xsize"
    with pytest.raises(M.MexError) as e:
        f(gs[f"{tag}/wn"], h, np.array([[1.0, 2.0], [3.0, 4.0]]), npml, gs[f"{tag}/x"], 4.0)
    assert e.value.ident == "SLIM_release_apps:tools:algorithms:ThreeDFreqModeling:Helm3dmvp_mex:Nsize"
    s = M.MexFunction(gws["Helm3d_kacz_sweep_mex"])
    with pytest.raises(M.MexError) as e:
        s(gs[f"{tag}/wn"], h, n, npml, 1.5, X, B[:-2])
    assert e.value.ident == "SLIM_release_apps:tools:algorithms:ThreeDFreqModeling:Helm3dkaczswp_mex:Bsize"


@pytest.mark.parametrize("dtype,cfg", [("c64", c) for c in range(6)] + [("c128", c) for c in range(3)])
def test_block8_batched_kernel_configurations_match_oracle(cuda, dtype, cfg, monkeypatch):
    """Every compiled configuration of the batched BLOCK8 kernel (right-hand sides per CTA and
    per thread), fixed through H3D_BLOCK8_CONFIG, on nine right-hand sides (full and partly
    filled groups) and both modes, against the C oracle's BLOCK8 sweep."""
    import torch
    from h3d import ops

    monkeypatch.setenv("H3D_BLOCK8_CONFIG", str(cfg))
    n, h, npml = (29, 27, 26), (25.0, 22.0, 20.0), (3, 4, 2, 3, 4, 2)
    rng = np.random.default_rng(90 + cfg)
    N = int(np.prod(n))
    g = O.make_grid(n, h, npml)
    wn = (2 * np.pi * 5.0) ** 2 / (1500.0 + 1500.0 * rng.random(N)) ** 2
    X = rng.standard_normal((N, 9)) + 1j * rng.standard_normal((N, 9))
    B = rng.standard_normal((N, 9)) + 1j * rng.standard_normal((N, 9))
    cdt, rdt = (torch.complex64, np.float32) if dtype == "c64" else (torch.complex128, np.float64)
    for mode in (1, 2):
        ref = O.sweep(g, wn, 1.5, X, B, adj=(mode == 2), order=O.ORDER_BLOCK8, blk=(12, 12, 12), nthreads=4)
        y = ops.kacz_sweep((n, h, npml), _t(wn.astype(rdt), cuda), 1.5, _t(X.T, cuda, cdt), _t(B.T, cuda, cdt),
                           mode, order=3)
        tol = 5e-5 if dtype == "c64" else 1e-12
        assert _rel(y.cpu().numpy().T.astype(np.complex128), ref) <= tol, mode
