"""Band-storage path on the GPU (h3d_band_coefs / h3d_band_mvp / h3d_band_sweep, h3d.band).

Parity against oracle/slim_band.py -- the numpy restatement of helmholtz_3d.m,
Htransp.m, Hmvp_MT_mex.c and sweep_MT_mex.c, itself pinned against the compiled reference
gateways by tests/test_band_cpu.py -- and against the library's matrix-free kernels:
  * the band coefficients equal helmholtz_3d's bands (forward) and conj(Htransp(H))
    (adjoint) to 1e-13 relative (FP64; the two PML evaluations round differently);
  * the band matvec equals the matrix-free matvec and the oracle band matvec, also for a
    generic band matrix whose offsets reach outside [0, N);
  * the band sweep equals sweep_MT_mex's sequential sweep (oracle) and the matrix-free LEX
    sweep, to 1e-12;
  * BandOp.solve (CGMN on the band sweeps) solves H u = b;
  * offsets that are not the grid's 27-point neighbourhood are refused (real buffers are
    passed, so a wrong acceptance could not touch memory outside them).
"""
import ctypes as C

import numpy as np
import pytest

from oracle import slim_band as SB

pytestmark = pytest.mark.gpu


def _rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.abs(a - b).max() / np.abs(b).max()


def _problem(cuda, n=(11, 9, 8), npml=3, seed=5):
    import torch
    from h3d import _lib as L

    rng = np.random.default_rng(seed)
    h = (12.0, 10.0, 11.0)
    wn3 = (2 * np.pi * 5) ** 2 / (1500 + 800 * rng.random(n)) ** 2
    grid = L.make_grid(n, h, npml)
    wn = torch.as_tensor(wn3.reshape(-1, order="F"), device=cuda)
    npml23 = np.full((2, 3), float(npml))
    return rng, grid, wn, wn3, h, npml23


@pytest.mark.parametrize("mode", [1, 2])
def test_band_coefs_match_helmholtz_3d(cuda, mode):
    from h3d.band import BandOp

    rng, grid, wn, wn3, h, npml23 = _problem(cuda)
    H, idx = SB.helmholtz_3d_bands(wn3, h, npml23)
    if mode != 1:
        H, idx = SB.htransp(H, idx)
        H = np.conj(H)
    A = BandOp.helmholtz(grid, wn, mode=mode)
    assert np.array_equal(A.offsets, idx)
    assert _rel(A.coef.cpu().numpy(), H.T) <= 1e-13


@pytest.mark.parametrize("mode", [1, 2])
def test_band_mvp_matches_matrix_free_and_oracle(cuda, mode):
    import torch
    from h3d import ops
    from h3d.band import BandOp

    rng, grid, wn, wn3, h, npml23 = _problem(cuda, seed=6)
    N = wn.numel()
    A = BandOp.helmholtz(grid, wn, mode=mode)
    x = torch.as_tensor(rng.standard_normal((2, N)) + 1j * rng.standard_normal((2, N)), device=cuda)
    y = A @ x
    assert _rel(y.cpu().numpy(), ops.mvp(grid, wn, x, mode).cpu().numpy()) <= 1e-13
    ref = SB.band_mvp(A.coef.cpu().numpy().T, A.offsets, x.cpu().numpy().T)
    assert _rel(y.cpu().numpy().T, ref) <= 1e-14
    y32 = BandOp.helmholtz(grid, wn, mode=mode, dtype=torch.complex64) @ x.to(torch.complex64)
    assert _rel(y32.cpu().numpy().astype(np.complex128), ref.T) <= 2e-6


def test_generic_band_mvp_skips_couplings_outside(cuda):
    """Hmvp_MT_mex semantics for any band matrix: 5 bands whose offsets reach past both ends."""
    import torch
    from h3d.band import BandOp

    rng = np.random.default_rng(7)
    N, offs = 500, np.array([-300, -7, 0, 5, 420], dtype=np.int64)
    coef = rng.standard_normal((N, 5)) + 1j * rng.standard_normal((N, 5))
    A = BandOp(torch.as_tensor(coef, device=cuda), offs)
    x = rng.standard_normal((3, N)) + 1j * rng.standard_normal((3, N))
    y = (A @ torch.as_tensor(x, device=cuda)).cpu().numpy()
    assert _rel(y.T, SB.band_mvp(coef.T, offs, x.T)) <= 1e-14


@pytest.mark.parametrize("mode", [1, 2])
def test_band_sweep_matches_sequential_sweep(cuda, mode):
    import torch
    from h3d import _lib as L
    from h3d import ops
    from h3d.band import BandOp

    rng, grid, wn, wn3, h, npml23 = _problem(cuda, n=(9, 10, 7), seed=8)
    N = wn.numel()
    A = BandOp.helmholtz(grid, wn, mode=mode)
    x = rng.standard_normal((2, N)) + 1j * rng.standard_normal((2, N))
    b = rng.standard_normal((2, N)) + 1j * rng.standard_normal((2, N))
    xs = A.kacz_sweep(1.3, torch.as_tensor(x, device=cuda), torch.as_tensor(b, device=cuda)).cpu().numpy()
    Hc = A.coef.cpu().numpy().T
    ref = SB.band_sweep(Hc, A.offsets, x.T, b.T, 1.3, SB.row_norms_sq(Hc))
    assert _rel(xs.T, ref) <= 1e-12
    if mode == 1:
        # forward: the matrix-free LEX sweep has the same coefficients and row norms
        mf = ops.kacz_sweep(grid, wn, 1.3, torch.as_tensor(x, device=cuda), torch.as_tensor(b, device=cuda),
                            1, order=L.ORDER_LEX).cpu().numpy()
        assert _rel(xs, mf) <= 1e-12
    # complex64 bands and sweeps
    A32 = BandOp.helmholtz(grid, wn, mode=mode, dtype=torch.complex64)
    xs32 = A32.kacz_sweep(1.3, torch.as_tensor(x, device=cuda), torch.as_tensor(b, device=cuda)).cpu().numpy()
    assert _rel(xs32.astype(np.complex128).T, ref) <= 5e-5


def test_band_solve(cuda):
    import torch
    from h3d import ops
    from h3d.band import BandOp

    rng, grid, wn, wn3, h, npml23 = _problem(cuda, n=(14, 13, 12), npml=3, seed=9)
    N = wn.numel()
    b = torch.zeros(2, N, dtype=torch.complex128, device=cuda)
    b[0, N // 2 + 7] = 1.0
    b[1, 3 * N // 5] = 1.0 - 0.5j
    A = BandOp.helmholtz(grid, wn)
    u, hst = A.solve(b, tol=1e-8, maxit=2000)
    assert hst[-1] <= 1e-8
    r = b - ops.mvp(grid, wn, u, 1)
    assert (torch.linalg.vector_norm(r, dim=1) / torch.linalg.vector_norm(b, dim=1)).max().item() <= 1e-5
    # a zero column gives zero (opBandStorage.m:225-230)
    u0, _ = A.solve(torch.zeros(N, dtype=torch.complex128, device=cuda))
    assert float(u0.abs().max()) == 0.0


def test_band_sweep_refuses_foreign_offsets(cuda):
    import torch
    from h3d import _lib as L
    from h3d.band import BandOp

    rng, grid, wn, wn3, h, npml23 = _problem(cuda, seed=10)
    A = BandOp.helmholtz(grid, wn)
    x = torch.zeros(A.N, dtype=torch.complex128, device=cuda)
    bad = A.offsets.copy()
    bad[4] += 1                                     # no longer the 27-point neighbourhood
    rc = L.load().h3d_band_sweep(C.byref(grid), C.c_void_p(A.coef.data_ptr()),
                                 bad.ctypes.data_as(C.POINTER(C.c_int64)), C.c_void_p(), 1.5,
                                 C.c_void_p(x.data_ptr()), C.c_void_p(), 1, L.C128,
                                 C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == L.ERR_BAD_ARG
    assert b"neighbourhood" in L.load().h3d_last_error()


def test_band_gateways_drop_in(cuda):
    """Hmvp_MT_mex / sweep_MT_mex gateways (same names and arguments as the reference
    binaries) against the band oracle, itself pinned to the compiled reference gateways."""
    from h3d import build
    from oracle import mexharness as M

    gws = build.build_mex()
    rng, grid, wn, wn3, h, npml23 = _problem(cuda, n=(9, 8, 10), seed=11)
    H, idx = SB.helmholtz_3d_bands(wn3, h, npml23)
    N = H.shape[1]
    X = rng.standard_normal((N, 2)) + 1j * rng.standard_normal((N, 2))
    B = rng.standard_normal((N, 2)) + 1j * rng.standard_normal((N, 2))
    y = M.MexFunction(gws["Hmvp_MT_mex"])(H, idx.astype(float), X, 2.0)
    assert _rel(y, SB.band_mvp(H, idx, X)) <= 1e-14
    rn = SB.row_norms_sq(H)
    ys = M.MexFunction(gws["sweep_MT_mex"])(H, idx.astype(float), X, B, 1.4, rn)
    assert _rel(ys, SB.band_sweep(H, idx, X, B, 1.4, rn)) <= 1e-12


def test_band_path_against_reference_golden(cuda, golden_band):
    """GPU band coefficients, gateways and BandOp against the committed outputs of the
    compiled Hmvp_MT_mex / sweep_MT_mex (tests/golden/band_small.npz)."""
    import torch
    from h3d import _lib as L
    from h3d import build
    from h3d.band import BandOp
    from oracle import mexharness as M

    g = golden_band
    n = tuple(int(v) for v in g["n"])
    grid = L.make_grid(n, tuple(g["h"]), int(g["npml"][0, 0]))
    wn = torch.as_tensor(g["wn"], device=cuda)
    for mode, key in ((1, "H"), (2, "Hadj")):
        A = BandOp.helmholtz(grid, wn, mode=mode)
        assert _rel(A.coef.cpu().numpy(), g[key].T) <= 1e-13
    gws = build.build_mex()
    for tag, A, o in (("forw", g["H"], g["idx"]), ("adj", g["Hadj"], g["idxadj"])):
        y = M.MexFunction(gws["Hmvp_MT_mex"])(A, o.astype(float), g["X"], 2.0)
        assert _rel(y, g[f"{tag}/mvp"]) <= 1e-14
        ys = M.MexFunction(gws["sweep_MT_mex"])(A, o.astype(float), g["X"], g["B"], 1.3, g[f"{tag}/rn"])
        assert _rel(ys, g[f"{tag}/swp"]) <= 1e-12


def test_band_double_sweep_properties_on_random_bands(cuda):
    """test_DoubleKaczmarzSweep.m:125-228 on the GPU band sweep: for a random row-normalised
    27-point band matrix on a 10 x 11 x 12 grid, I - Q (Q x = DSWP(x, 0)) is Hermitian and
    positive semi-definite, a double sweep reduces the error of an iterate, and the sweep
    equals the sequential sweep of sweep_MT_mex (oracle)."""
    import torch
    from h3d.band import BandOp

    n = (10, 11, 12)
    rng = np.random.default_rng(3)
    nx, ny, nz = n
    N = nx * ny * nz
    H = rng.standard_normal((27, N)) + 1j * rng.standard_normal((27, N))
    i, j, k = np.arange(N) % nx, (np.arange(N) // nx) % ny, np.arange(N) // (nx * ny)
    for t, (dx, dy, dz) in enumerate(SB.OFFS):
        H[t, (i + dx < 0) | (i + dx >= nx) | (j + dy < 0) | (j + dy >= ny) | (k + dz < 0) | (k + dz >= nz)] = 0
    H /= np.sqrt(SB.row_norms_sq(H))[None, :]
    idx = np.array([dx + nx * dy + nx * ny * dz for dx, dy, dz in SB.OFFS], dtype=np.int64)
    from h3d import _lib as L

    A = BandOp(torch.as_tensor(H.T.copy(), device=cuda), idx, grid=L.make_grid(n, (1.0, 1.0, 1.0), 0))
    E = torch.eye(N, dtype=torch.complex128, device=cuda)
    IQ = (E - A.kacz_sweep(1.5, E)).cpu().numpy().T             # columns: (I - Q) e_j
    assert np.abs(IQ - IQ.conj().T).max() <= 1e-10                # Hermitian
    assert np.linalg.eigvalsh((IQ + IQ.conj().T) / 2).min() >= -1e-10
    x = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    ref = SB.band_sweep(H, idx, x[:, None], np.zeros((N, 1)), 1.5, SB.row_norms_sq(H))[:, 0]
    got = A.kacz_sweep(1.5, torch.as_tensor(x, device=cuda)).cpu().numpy()
    assert _rel(got, ref) <= 1e-12
    xs = torch.as_tensor(x, device=cuda)
    b = A @ xs
    x1 = A.kacz_sweep(1.5, torch.zeros_like(xs), b)
    assert float(torch.linalg.vector_norm(xs - x1)) < float(torch.linalg.vector_norm(xs))
