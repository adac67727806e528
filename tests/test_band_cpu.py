"""The band-storage (mat_free = false) oracle pinned against the reference, on CPU.

oracle/slim_band.py restates helmholtz_3d.m / create_pml.m (the 27 x N band matrix),
Htransp.m, Hmvp_MT_mex.c and sweep_MT_mex.c.  Pins:
  * the restated band matrix times a vector equals the compiled matrix-free reference
    matvec (Helm3dmvp_forw_mex / Helm3dmvp_adj_mex) to rounding: the two reference paths
    build the same operator;
  * the restated band matvec and band sweep equal the compiled band gateways
    Hmvp_MT_mex / sweep_MT_mex (the sweep bit for bit);
  * the band sweep of helmholtz_3d's matrix equals the matrix-free Kaczmarz sweep.
"""
import os

import numpy as np
import pytest

from oracle import mexharness as M
from oracle import slim_band as SB

BAND_REF = ("Hmvp_MT_mex", "sweep_MT_mex", "Helm3dmvp_forw_mex", "Helm3dmvp_adj_mex", "Helm3d_kacz_sweep_mex")
pytestmark = pytest.mark.skipif(
    not all(os.path.exists(os.path.join(M.REF_DIR, n + ".so")) for n in BAND_REF),
    reason="reference gateways not compiled here")


def _problem(seed, n=(9, 8, 7), npml=((3, 2, 3), (3, 2, 3))):
    rng = np.random.default_rng(seed)
    h = np.array([10.0, 12.0, 11.0])
    wn = (2 * np.pi * 5) ** 2 / (1500 + 500 * rng.random(n)) ** 2
    return rng, wn, h, np.array(npml, float)


def _rel(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


def test_band_matrix_equals_matrix_free_operator():
    rng, wn, h, npml = _problem(1)
    n = wn.shape
    N = wn.size
    H, idx = SB.helmholtz_3d_bands(wn, h, npml)
    assert H.shape == (27, N)
    x = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    args = (wn.reshape(-1, order="F"), h, np.array(n, float), npml, x, 1.0)
    assert _rel(SB.band_mvp(H, idx, x), M.load_reference("Helm3dmvp_forw_mex")(*args)[:, 0]) <= 1e-13
    Ht, idt = SB.htransp(H, idx)
    assert np.array_equal(idt, -idx)
    assert _rel(SB.band_mvp(np.conj(Ht), idt, x), M.load_reference("Helm3dmvp_adj_mex")(*args)[:, 0]) <= 1e-13


def test_band_oracle_against_compiled_band_gateways():
    rng, wn, h, npml = _problem(2, n=(8, 7, 9))
    N = wn.size
    H, idx = SB.helmholtz_3d_bands(wn, h, npml)
    X = rng.standard_normal((N, 2)) + 1j * rng.standard_normal((N, 2))
    B = rng.standard_normal((N, 2)) + 1j * rng.standard_normal((N, 2))
    ref = M.load_reference("Hmvp_MT_mex")(H, idx.astype(float), X, 2.0)
    assert _rel(SB.band_mvp(H, idx, X), ref) <= 4e-16
    rn = SB.row_norms_sq(H)
    swp = M.load_reference("sweep_MT_mex")(H, idx.astype(float), X, B, 1.3, rn)
    assert np.array_equal(SB.band_sweep(H, idx, X, B, 1.3, rn), swp)


def test_band_sweep_equals_matrix_free_sweep():
    rng, wn, h, npml = _problem(3)
    n = wn.shape
    N = wn.size
    H, idx = SB.helmholtz_3d_bands(wn, h, npml)
    x = rng.standard_normal((N, 1)) + 1j * rng.standard_normal((N, 1))
    b = rng.standard_normal((N, 1)) + 1j * rng.standard_normal((N, 1))
    band = SB.band_sweep(H, idx, x, b, 1.5, SB.row_norms_sq(H))
    mf = M.load_reference("Helm3d_kacz_sweep_mex")(wn.reshape(-1, order="F"), h, np.array(n, float), npml, 1.5, x, b)
    assert _rel(band, mf) <= 1e-13


def test_band_gateways_check_sizes_like_the_reference():
    """The drop-in Hmvp_MT_mex / sweep_MT_mex refuse mismatched sizes with the reference's
    identifier before any device work (Hmvp_MT_mex.c:105-109, sweep_MT_mex.c:134-160)."""
    from h3d import build

    gws = build.build_mex()
    rng, wn, h, npml = _problem(4)
    N = wn.size
    H, idx = SB.helmholtz_3d_bands(wn, h, npml)
    x = rng.standard_normal((N, 1)) + 0j
    ident = "SLIM_release_apps:tools:algorithms:ThreeDFreqModeling:HMvp_MT_mex:NumElements"
    for lib in (gws["Hmvp_MT_mex"], os.path.join(M.REF_DIR, "Hmvp_MT_mex.so")):
        with pytest.raises(M.MexError) as e:
            M.MexFunction(lib)(H, idx.astype(float), x[:-1], 1.0)
        assert e.value.ident == ident
    rn = SB.row_norms_sq(H)
    for lib in (gws["sweep_MT_mex"], os.path.join(M.REF_DIR, "sweep_MT_mex.so")):
        f = M.MexFunction(lib)
        with pytest.raises(M.MexError) as e:
            f(H, idx.astype(float), x[:-1], x, 1.5, rn)
        assert e.value.ident == ident
        with pytest.raises(M.MexError) as e:
            f(H, idx.astype(float), x, x, 1.5, rn[:-1])
        assert e.value.ident == ident


def test_band_sweep_gateway_reads_the_grid_off_the_offsets():
    """h3d_mex_band_sweep refuses, before any device work, bands that are not the 27-point
    stencil of a grid of at least 3 points per axis (host arrays only)."""
    import ctypes as C

    from h3d import _lib as L

    lib = L.load()
    rng, wn, h, npml = _problem(5)
    N = wn.size
    H, idx = SB.helmholtz_3d_bands(wn, h, npml)
    x = np.zeros(N)
    rn = SB.row_norms_sq(H)
    yr, yi = np.zeros(N), np.zeros(N)
    p = lambda a: np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(C.POINTER(C.c_double))
    Hr, Hi = np.asfortranarray(H.real), np.asfortranarray(H.imag)

    def call(off, nd=27):
        return lib.h3d_mex_band_sweep(p(Hr), p(Hi), nd, N, p(off), p(x), None, N, 1, p(x), None, N, 1.5, p(rn), N,
                                      p(yr), p(yi))

    bad = idx.astype(float)
    bad[3] += 0.5                                  # not an integer
    assert call(bad) == L.ERR_BAD_ARG
    bad = idx.astype(float)
    bad[20] = 7.0                                  # not a grid neighbourhood
    assert call(bad) == L.ERR_BAD_ARG and b"neighbourhood" in lib.h3d_last_error()
    assert call(idx.astype(float), nd=26) == L.ERR_BAD_ARG
    # a 2-point axis: its offsets collide with another axis' (refused)
    H2, idx2 = SB.helmholtz_3d_bands(np.ones((5, 2, 6)), h, np.zeros((2, 3)))
    N2 = H2.shape[1]
    x2, rn2 = np.zeros(N2), SB.row_norms_sq(H2)
    rc = lib.h3d_mex_band_sweep(p(H2.real), p(H2.imag), 27, N2, p(idx2.astype(float)), p(x2), None, N2, 1, p(x2),
                                None, N2, 1.5, p(rn2), N2, p(x2), p(x2))
    assert rc == L.ERR_BAD_ARG


def test_band_and_matrix_free_paths_differ_for_unequal_pml_widths():
    """The two reference paths build the same operator only for equal PML widths on the two
    sides of an axis (every workload here).  For unequal widths they differ whichever way
    the 2 x 3 npml rows are read: create_pml.m:47-52 takes np(2,a) as the lower width and
    np(1,a) as the upper one, while the matrix-free PML functions (Helm3d_27pt.h:326-390)
    test the interior against the lower width on both sides.  The library's band
    coefficients follow the matrix-free operator."""
    rng, wn, h, _ = _problem(6, n=(10, 9, 8))
    n = wn.shape
    N = wn.size
    npml = np.array([[3.0, 1.0, 2.0], [1.0, 3.0, 4.0]])
    H, idx = SB.helmholtz_3d_bands(wn, h, npml)
    x = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    y = SB.band_mvp(H, idx, x)
    mv = M.load_reference("Helm3dmvp_forw_mex")
    args = lambda p: (wn.reshape(-1, order="F"), h, np.array(n, float), p, x, 1.0)
    assert _rel(y, mv(*args(npml))[:, 0]) > 1e-3
    assert _rel(y, mv(*args(npml[::-1].copy()))[:, 0]) > 1e-3
    sym = np.array([[2.0, 3.0, 1.0], [2.0, 3.0, 1.0]])
    Hs, idxs = SB.helmholtz_3d_bands(wn, h, sym)
    assert _rel(SB.band_mvp(Hs, idxs, x), mv(*args(sym))[:, 0]) <= 1e-13


def _random_band_27(n, seed):
    """A random complex 27-point band matrix on grid n with unit row norms and no coupling
    across a face of the grid (test_DoubleKaczmarzSweep.m:26-119 builds its operators so)."""
    rng = np.random.default_rng(seed)
    nx, ny, nz = n
    N = nx * ny * nz
    H = rng.standard_normal((27, N)) + 1j * rng.standard_normal((27, N))
    i = np.arange(N) % nx
    j = (np.arange(N) // nx) % ny
    k = np.arange(N) // (nx * ny)
    for t, (dx, dy, dz) in enumerate(SB.OFFS):
        out = ((i + dx < 0) | (i + dx >= nx) | (j + dy < 0) | (j + dy >= ny) | (k + dz < 0) | (k + dz >= nz))
        H[t, out] = 0
    H /= np.sqrt(SB.row_norms_sq(H))[None, :]
    idx = np.array([dx + nx * dy + nx * ny * dz for dx, dy, dz in SB.OFFS], dtype=np.int64)
    return H, idx


def test_double_sweep_properties_on_random_bands():
    """The Kaczmarz-sweep properties of test_DoubleKaczmarzSweep.m:125-228 for the compiled
    sweep_MT_mex on a random row-normalised 27-point band matrix (10 x 11 x 12 grid):
    I - Q is Hermitian and positive semi-definite (Q x = DSWP(x, 0)), and a double sweep
    reduces the error of an iterate.  The oracle's sweep agrees with it."""
    n = (10, 11, 12)
    H, idx = _random_band_27(n, 3)
    N = H.shape[1]
    rn = SB.row_norms_sq(H)
    sw = M.load_reference("sweep_MT_mex")
    off = idx.astype(float)
    rng = np.random.default_rng(4)
    x = rng.standard_normal((N, 1)) + 1j * rng.standard_normal((N, 1))
    y = rng.standard_normal((N, 1)) + 1j * rng.standard_normal((N, 1))
    zero = np.zeros((N, 1), complex)
    IQ = lambda v: v - sw(H, off, v, np.zeros_like(v), 1.5, rn)
    lhs = np.vdot(y, IQ(x))
    rhs = np.vdot(IQ(y), x)
    assert abs(lhs - rhs) <= 1e-10 * abs(lhs)                                   # Hermitian
    assert _rel(SB.band_sweep(H, idx, x, zero, 1.5, rn), sw(H, off, x, zero, 1.5, rn)) <= 1e-14
    E = np.eye(N, dtype=complex)
    A = E - sw(H, off, E, np.zeros_like(E), 1.5, rn)                            # I - Q, dense
    assert np.abs(A - A.conj().T).max() <= 1e-10
    assert np.linalg.eigvalsh((A + A.conj().T) / 2).min() >= -1e-10            # PSD
    # error reduction: b = A* x*, one double sweep from 0 moves towards x*
    Bm = np.zeros((N, N), complex)
    for t in range(27):
        rows = np.arange(N)
        cols = rows + idx[t]
        ok = (cols >= 0) & (cols < N) & (H[t] != 0)
        Bm[rows[ok], cols[ok]] = H[t, ok]
    xs = rng.standard_normal((N, 1)) + 1j * rng.standard_normal((N, 1))
    x1 = sw(H, off, zero, Bm @ xs, 1.5, rn)
    assert np.linalg.norm(xs - x1) < np.linalg.norm(xs)
