"""CPU checks of the C ABI: the library builds, loads without a GPU, and exports every
function include/h3d.h declares; host-only helpers behave as documented."""
import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = open(os.path.join(ROOT, "include", "h3d.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(h3d_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    from h3d import _lib, build

    build.build_lib()
    lib = C.CDLL(build.LIB)
    missing = [s for s in _declared() if not hasattr(lib, s)]
    assert not missing, missing
    assert set(_lib.EXPORTED) >= set(_declared())
    assert lib.h3d_version() == 1


def test_status_ids_match_reference_identifiers():
    from h3d import _lib as L

    lib = L.load()
    assert lib.h3d_status_id(L.ERR_XSIZE).decode().endswith("Helm3dkaczswp_mex:Xsize")
    assert lib.h3d_status_id(L.ERR_BSIZE).decode().endswith("Helm3dkaczswp_mex:Bsize")
    assert lib.h3d_status_id(L.ERR_NSIZE).decode().endswith("Helm3dmvp_mex:Nsize")


def test_default_opts_follow_linsolveopts():
    from h3d import _lib as L

    o = L.default_opts()
    assert o.tol == 1e-6 and o.maxit == 10000 and o.w == 1.5


def test_mex_host_entry_rejects_bad_shapes_without_gpu():
    """Argument checks happen before any device work (Helm3dmvp_mex.c:75-85)."""
    from h3d import _lib as L

    lib = L.load()
    dp = C.POINTER(C.c_double)
    wn = np.ones(8)
    h = np.array([10.0, 10.0, 10.0])
    n = np.array([2.0, 2.0, 2.0])
    npml = np.zeros(6)
    x = np.ones(7)
    y = np.zeros(8)
    p = lambda a: a.ctypes.data_as(dp)
    rc = lib.h3d_mex_mvp(p(wn), None, p(h), p(n), 3, p(npml), p(x), None, 7, p(y), p(y), 1, 0)
    assert rc == L.ERR_XSIZE
    rc = lib.h3d_mex_mvp(p(wn), None, p(h), p(n), 2, p(npml), p(x), None, 8, p(y), p(y), 1, 0)
    assert rc == L.ERR_NSIZE
    rc = lib.h3d_mex_kacz_sweep(p(wn), None, p(h), p(n), 3, p(npml), 1.5, p(wn), None, 8, 1,
                                p(wn), None, 7, p(y), p(y), 1, 0)
    assert rc == L.ERR_BSIZE


def test_sinc_weights_host_match_oracle():
    """h3d_sinc_weights (host) against the restated opSincInterp/kaiser_window."""
    from h3d import _lib as L
    from oracle import slim_ref

    lib = L.load()
    g = L.make_grid((30, 28, 26), (25.0, 25.0, 25.0), 5)
    pts = np.array([[10.3, 11.0, 4.75], [0.4, 27.2, 12.5]])
    base = np.zeros((2, 3), np.int32)
    w = np.zeros((2, 3, 9))
    rc = lib.h3d_sinc_weights(C.byref(g), pts.ctypes.data_as(C.POINTER(C.c_double)), 2,
                              base.ctypes.data_as(C.POINTER(C.c_int32)),
                              w.ctypes.data_as(C.POINTER(C.c_double)))
    assert rc == 0
    for p in range(2):
        for a, n in enumerate((30, 28, 26)):
            axis = np.arange(n, dtype=float)
            full = slim_ref.sinc_interp_matrix([pts[p, a]], axis)[:, 0]
            mine = np.zeros(n)
            for o in range(9):
                idx = base[p, a] + o
                if 0 <= idx < n:
                    mine[idx] = w[p, a, o]
            np.testing.assert_allclose(mine, full, rtol=0, atol=1e-14)


def test_noalloc_residual_size_check_is_host_only():
    """h3d_residual_noalloc refuses a problem beyond its fixed scratch before any launch or
    copy and before it looks at the data pointers (left NULL here); on a host without a GPU
    the occupancy query behind the z split fails and the default split is used."""
    from h3d import _lib as L

    lib = L.load()
    grid = L.make_grid((400, 400, 400), (10.0, 10.0, 10.0), 10)
    rc = lib.h3d_residual_noalloc(C.byref(grid), None, None, None, None, None, None, None, 4096, L.FORWARD, None)
    assert rc == L.ERR_BAD_ARG
    assert b"scratch" in lib.h3d_last_error()
    # a problem that fits is refused by the pointer check instead, still without device work
    small = L.make_grid((16, 16, 16), (10.0, 10.0, 10.0), 2)
    rc = lib.h3d_residual_noalloc(C.byref(small), None, None, None, None, None, None, None, 1, L.FORWARD, None)
    assert rc == L.ERR_BAD_ARG
    assert b"scratch" not in lib.h3d_last_error()


def test_bindings_match_header_arity():
    """Every function include/h3d.h declares is bound in h3d._lib with the same number of
    parameters (a parameter added to the header but not to the binding would shift every
    later argument)."""
    from h3d import _lib

    src = open(os.path.join(ROOT, "include", "h3d.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    decls = re.findall(r"\b(?:int|void|const char \*)\s*\*?\s*(h3d_[a-z0-9_]+)\s*\(([^;]*?)\)\s*;", src, flags=re.S)
    assert sorted(d[0] for d in decls) == _declared()
    for name, args in decls:
        args = args.strip()
        n = 0 if args in ("", "void") else len(args.split(","))
        assert name in _lib._SIGS, name
        assert len(_lib._SIGS[name][1]) == n, (name, n, len(_lib._SIGS[name][1]))


def test_sinc_kaiser_restatement_against_independent_formula():
    """The oracle's opSincInterp / kaiser_window / sinc restatement (the checker of the
    library's source and receiver weights) against the published window evaluated with
    numpy's own sinc and Bessel I0: w(D) = sinc(D) I0(beta sqrt(1 - (D/r)^2)) / I0(beta) for
    |D| <= r, 0 beyond, with beta = 6.31 for r = 4 (opSincInterp.m's table)."""
    from oracle import slim_ref

    r, beta = 4, 6.31
    for frac in (0.0, 0.3, 0.5, 0.77):
        xout = np.arange(-6.0, 7.0)                  # unit output spacing
        got = slim_ref.sinc_interp_matrix([frac], xout, r=r)[:, 0]
        D = xout - frac
        want = np.where(np.abs(D) <= r,
                        np.sinc(D) * np.i0(beta * np.sqrt(np.clip(1 - (D / r) ** 2, 0, None))) / np.i0(beta), 0.0)
        np.testing.assert_allclose(got, want, rtol=0, atol=1e-14)


def test_solve_gateway_and_fwi_grad_refuse_bad_sizes_before_device_work():
    """The h3d_solve_mex gateway reports a b of the wrong height and a bad n with its own
    Bsize / Nsize identifiers, and h3d_fwi_grad refuses missing buffers, before any device
    call (so this runs without a GPU)."""
    from h3d import _lib as L
    from h3d import build
    from oracle import mexharness as M

    gw = M.MexFunction(build.build_mex()["h3d_solve_mex"])
    n = np.array([6.0, 5.0, 4.0])
    wn = np.ones(120)
    with pytest.raises(M.MexError) as e:
        gw(wn, np.ones(3), n, np.ones((2, 3)), np.ones(119), 1.0, 1e-6, 10.0)
    assert e.value.ident == "SLIM_release_apps:tools:algorithms:ThreeDFreqModeling:h3d_solve_mex:Bsize"
    with pytest.raises(M.MexError) as e:
        gw(wn, np.ones(3), np.ones((2, 2)), np.ones((2, 3)), np.ones(120), 1.0, 1e-6, 10.0)
    assert e.value.ident == "SLIM_release_apps:tools:algorithms:ThreeDFreqModeling:h3d_solve_mex:Nsize"
    lib = L.load()
    grid = L.make_grid((6, 5, 4), (10.0, 10.0, 10.0), 1)
    rc = lib.h3d_fwi_grad(C.byref(grid), None, None, None, 1, None, None, 1, None, None, None, None, None)
    assert rc == L.ERR_BAD_ARG


def test_wait_timeout_check_refuses_bad_limits_without_a_gpu():
    """h3d_check_wait_timeout checks its limit before any device call."""
    from h3d import _lib as L

    lib = L.load()
    for bad in (0.0, -1.0, 5000.0, float("nan")):
        assert lib.h3d_check_wait_timeout(bad) == L.ERR_BAD_ARG


def test_mlgmres_refuses_bad_arguments_without_a_gpu():
    """h3d_mlgmres_solve checks levels, transfers, step counts and the history buffer before
    any device call (the level and vector pointers below are never dereferenced)."""
    from h3d import _lib as L

    lib = L.load()
    o = L.MLOpts()
    lib.h3d_ml_default_opts(C.byref(o))
    assert (o.tol, o.maxit, o.maxinnerit, list(o.k), o.smooth_tol, o.coarse_tol) == \
        (1e-6, 10000, 5, [3, 5, 3, 5], 1e-6, 0.5)                 # ML_GMRES.m:36-40,56, FGMRES.m
    g = L.make_grid((8, 8, 8), (10.0, 10.0, 10.0), 2)
    lv = (L.MLLevel * 2)()
    for lvl in lv:
        lvl.grid = g
        lvl.wn = 256
        lvl.wn32 = 256
    tr = (L.MLTransfer * 1)()
    dummy = C.c_void_p(256)

    def call(nl, opts, hst=None, cap=0):
        return lib.h3d_mlgmres_solve(lv, nl, tr, tr, dummy, dummy, L.FORWARD, C.byref(opts), hst, cap, None, None)

    assert call(1, o) == L.ERR_BAD_ARG                 # the V-cycle needs two levels
    assert call(2, o) == L.ERR_BAD_ARG                 # transfers that do not connect the grids
    for field, bad in (("maxinnerit", 17), ("maxinnerit", 0), ("maxit", 0)):
        o2 = L.MLOpts.from_buffer_copy(o)
        setattr(o2, field, bad)
        assert call(2, o2) == L.ERR_BAD_ARG
    o3 = L.MLOpts.from_buffer_copy(o)
    o3.k[1] = 0
    assert call(2, o3) == L.ERR_BAD_ARG
    o4 = L.MLOpts.from_buffer_copy(o)
    o4.precond = L.ML_PREC_NONE
    o4.maxit = 2
    hst = np.zeros(10)
    assert call(1, o4, hst.ctypes.data_as(L.dp), 10) == L.ERR_BAD_ARG   # 1 + 2 x 5 entries needed
    assert b"hst holds 10" in lib.h3d_last_error()


def test_multigrid_host_pieces_and_gateway_refuse_bad_input_without_a_gpu():
    """The hierarchy's host code checks its inputs (cubic weights need 4 nodes, nodes must
    ascend), and the h3d_mlgmres_mex gateway reports a bad n and a b of the wrong height with
    its Nsize / Bsize identifiers before any device call."""
    from h3d import _lib as L
    from h3d import build
    from oracle import mexharness as M

    lib = L.load()
    x3 = np.linspace(0.0, 1.0, 3)
    out = np.zeros(9)
    assert lib.h3d_ml_interp_weights(1, x3.ctypes.data_as(L.dp), 3, x3.ctypes.data_as(L.dp), 3,
                                     out.ctypes.data_as(L.dp)) == L.ERR_BAD_ARG
    down = x3[::-1].copy()
    assert lib.h3d_ml_interp_weights(0, down.ctypes.data_as(L.dp), 3, x3.ctypes.data_as(L.dp), 3,
                                     out.ctypes.data_as(L.dp)) == L.ERR_BAD_ARG
    # partition of unity of both interpolations between linspace nodes
    xi, xo = np.linspace(0.0, 1.0, 9), np.linspace(0.0, 1.0, 5)
    for kind in (0, 1):
        A = np.zeros((5, 9))
        assert lib.h3d_ml_interp_weights(kind, xi.ctypes.data_as(L.dp), 9, xo.ctypes.data_as(L.dp), 5,
                                         A.ctypes.data_as(L.dp)) == L.OK
        np.testing.assert_allclose(A.sum(axis=1), 1.0, atol=1e-14)
        np.testing.assert_allclose(A @ xi, xo, atol=1e-14)           # both reproduce linear functions

    gw = M.MexFunction(build.build_mex()["h3d_mlgmres_mex"])
    v = np.full(6 * 5 * 4, 1500.0)
    h = np.full(3, 20.0)
    with pytest.raises(M.MexError) as e:
        gw(v, h, np.ones((2, 2)), 2.0, 4.0, np.ones(10), 1.0, 1e-6, 10.0)
    assert e.value.ident == "SLIM_release_apps:tools:algorithms:ThreeDFreqModeling:h3d_mlgmres_mex:Nsize"
    with pytest.raises(M.MexError) as e:                              # b must cover the PML grid
        gw(v, h, np.array([6.0, 5.0, 4.0]), 2.0, 4.0, np.ones(6 * 5 * 4), 1.0, 1e-6, 10.0)
    assert e.value.ident == "SLIM_release_apps:tools:algorithms:ThreeDFreqModeling:h3d_mlgmres_mex:Bsize"
