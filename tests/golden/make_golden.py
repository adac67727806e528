"""Generate the golden vectors in tests/golden/ from the reference's own MEX code.

Run in a container that has the reference checkout (the gateways are compiled
unmodified by ``make -C oracle ref``):

    make -C oracle ref && python tests/golden/make_golden.py

What is produced (all from seeded inputs, stored with the inputs):

* ``stencil_small.npz`` -- two small grids (7x6x5 PML 2, and 12x11x10 with
  asymmetric PML and anisotropic spacing); outputs of all six
  ``Helm3dmvp_*_mex`` variants and of ``Helm3d_kacz_sweep{,_adj,_wnc}_mex``
  (3 right-hand sides).  The ``_wnc`` sweep is stored twice: as the reference's
  install script builds it (``-DWNCMPLEX`` typo: imag(wn) ignored) and as the
  intended complex-wavenumber build.
* ``config0_mvp.npz`` -- the 61^3 (PML 10, h = 25 m) forward matvec of a
  seeded complex128 vector on the config-0 velocity model: the full input is
  regenerated from the seed, so the file stores a checksum of the input, the
  output at 4096 seeded sample indices, its 2-norm and its inner product with a
  seeded probe vector.
* ``config0_solve.npz`` -- the config-0 forward solve as the reference runs it
  (linearsolve + CGMN with the compiled ``Helm3d_kacz_sweep_mex``, preconditioned
  tolerance 1e-6): iteration count, residual history, true residual, and the solution
  at 4096 seeded indices with its 2-norm and a seeded probe product; beside it the same
  problem solved to a true residual near 1e-9 by the C oracle ("exact/").
* ``config1_solve.npz`` -- the config-1 forward solve by the C oracle to a true residual
  near 1e-9 (samples, norm, probe product), the FP64 reference of the bench's error figures.
* ``config3_grad.npz`` -- PDEfunc OBJ on a reduced config-3 problem (the 161x161x81
  grid, sources 0 and 1 of the 32, all 400 receivers, 6 Hz, squared slowness at the
  background model, observed data zero), solved in the reference's row order and
  tolerance: f and the gradient at 4096 seeded indices with its norm and probe product.
* ``band_small.npz`` -- the band-storage path on a 7x6x8 grid (PML 2): the 27 x N
  band matrix of helmholtz_3d.m (from oracle/slim_band.py, which MATLAB would be
  needed to run directly; pinned to the compiled matrix-free gateways), its adjoint
  bands, and the outputs of the compiled ``Hmvp_MT_mex`` and ``sweep_MT_mex``
  (forward and adjoint bands, 2 right-hand sides).

``python tests/golden/make_golden.py band`` writes only ``band_small.npz``;
``... config0_solve`` (a few minutes), ``... config1_solve`` (hours: a 4 M-unknown solve to
1e-10, GOLDEN_THREADS threads) and ``... config3_grad`` (about an hour: four single-threaded
solves of 2.1 M unknowns, two processes) write one file each.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "slim-release-apps_gb300"))

from oracle import mexharness as M  # noqa: E402

MVP = ["forw", "adj", "forw_deriv", "adj_deriv", "forw_wnc", "adj_wnc"]


def small_case(tag, n, h, npml23, seed, out):
    rng = np.random.default_rng(seed)
    N = int(np.prod(n))
    v = 1500.0 + 2000.0 * rng.random(N)
    wn = (2 * np.pi * 4.0) ** 2 / v ** 2
    wnc = wn * (1.0 + 0.05j * rng.random(N))
    dwn = -2.0 * (2 * np.pi * 4.0) ** 2 / v ** 3
    x = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    P = 3
    X = rng.standard_normal((N, P)) + 1j * rng.standard_normal((N, P))
    B = rng.standard_normal((N, P)) + 1j * rng.standard_normal((N, P))
    nv = np.array(n, float)
    hv = np.array(h, float)
    npml = np.array(npml23, float)
    out[f"{tag}/n"] = nv
    out[f"{tag}/h"] = hv
    out[f"{tag}/npml"] = npml
    out[f"{tag}/wn"] = wn
    out[f"{tag}/wnc"] = wnc
    out[f"{tag}/dwn"] = dwn
    out[f"{tag}/x"] = x
    out[f"{tag}/X"] = X
    out[f"{tag}/B"] = B
    for var in MVP:
        w = wnc if var.endswith("wnc") else (dwn if "deriv" in var else wn)
        y = M.load_reference(f"Helm3dmvp_{var}_mex")(w, hv, nv, npml, x, 4.0)[:, 0]
        out[f"{tag}/mvp_{var}"] = y
    out[f"{tag}/swp_forw"] = M.load_reference("Helm3d_kacz_sweep_mex")(wn, hv, nv, npml, 1.5, X, B)
    out[f"{tag}/swp_adj"] = M.load_reference("Helm3d_kacz_sweep_adj_mex")(wn, hv, nv, npml, 1.5, X, B)
    out[f"{tag}/swp_wnc_installed"] = M.load_reference("Helm3d_kacz_sweep_wnc_mex")(
        wnc, hv, nv, npml, 1.5, X, B)
    out[f"{tag}/swp_wnc"] = M.load_reference("Helm3d_kacz_sweep_wnc_fixed_mex")(
        wnc, hv, nv, npml, 1.5, X, B)
    # b = 0 sweep (the CGMN operator Q) and x = 0 sweep (the preconditioned RHS)
    out[f"{tag}/swp_forw_b0"] = M.load_reference("Helm3d_kacz_sweep_mex")(
        wn, hv, nv, npml, 1.5, X, np.zeros((N, P)))
    out[f"{tag}/swp_adj_x0"] = M.load_reference("Helm3d_kacz_sweep_adj_mex")(
        wn, hv, nv, npml, 1.5, np.zeros((N, P), complex), B)


def config0_case(out):
    from h3d import models  # the seeded config-0 model generator

    m = models.config0()
    n = m.n_total
    N = int(np.prod(n))
    wn = m.wavenumber()
    rng = np.random.default_rng(20240)
    x = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    y = M.load_reference("Helm3dmvp_forw_mex")(wn, np.array(m.h, float), np.array(n, float),
                                                m.npml23(), x, float(os.cpu_count()))[:, 0]
    yadj = M.load_reference("Helm3dmvp_adj_mex")(wn, np.array(m.h, float), np.array(n, float),
                                                 m.npml23(), x, float(os.cpu_count()))[:, 0]
    srng = np.random.default_rng(7)
    idx = np.sort(srng.choice(N, size=4096, replace=False))
    probe = srng.standard_normal(N) + 1j * srng.standard_normal(N)
    out["n"] = np.array(n, float)
    out["x_checksum"] = np.array([np.sum(x.real), np.sum(x.imag), np.linalg.norm(x)])
    out["wn_checksum"] = np.array([np.sum(wn), np.linalg.norm(wn), wn.min(), wn.max()])
    for tag, val in (("forw", y), ("adj", yadj)):
        out[f"{tag}/idx"] = idx
        out[f"{tag}/samples"] = val[idx]
        out[f"{tag}/norm"] = np.array(np.linalg.norm(val))
        out[f"{tag}/probe_dot"] = np.array(np.vdot(probe, val))


def _samples(val, out, tag, seed=7, count=4096):
    """Seeded sample indices, the samples, the 2-norm and a seeded probe inner product."""
    srng = np.random.default_rng(seed)
    idx = np.sort(srng.choice(val.size, size=min(count, val.size), replace=False))
    probe = srng.standard_normal(val.size) + 1j * srng.standard_normal(val.size)
    out[f"{tag}/idx"] = idx
    out[f"{tag}/samples"] = val[idx]
    out[f"{tag}/norm"] = np.array(np.linalg.norm(val))
    out[f"{tag}/probe_dot"] = np.array(np.vdot(probe, val))


def config0_solve_case(out):
    """The config-0 forward solve exactly as the reference runs it: linearsolve.m:148-156
    (b~ = DSWP(0, b), A = I - DSWP(., 0), w = 1.5, zero start) and the CGMN loop of
    CGMN.m:48-90 (restated in oracle/slim_ref.cgmn), every double sweep by the compiled
    reference gateway Helm3d_kacz_sweep_mex (lexicographic order), stopping at the
    reference's preconditioned residual 1e-6 (CGMN.m:79), at most 2000 iterations."""
    from h3d import models
    from oracle import h3d_oracle as O
    from oracle import slim_ref

    m = models.config0()
    n = m.n_total
    N = int(np.prod(n))
    wn = m.wavenumber()
    b = m.point_source()
    hv, nv, npml = np.array(m.h, float), np.array(n, float), m.npml23()
    swp = M.load_reference("Helm3d_kacz_sweep_mex")
    mvp = M.load_reference("Helm3dmvp_forw_mex")
    zero = np.zeros(N, complex)
    bt = swp(wn, hv, nv, npml, 1.5, zero, b)[:, 0]

    def A(y):
        return y - swp(wn, hv, nv, npml, 1.5, y, np.zeros_like(y))

    x, hst = slim_ref.cgmn(A, bt, zero.copy(), tol=1e-6, maxit=2000)
    r = b - mvp(wn, hv, nv, npml, x, float(os.cpu_count()))[:, 0]
    out["n"] = np.array(n, float)
    out["wn_checksum"] = np.array([np.sum(wn), np.linalg.norm(wn), wn.min(), wn.max()])
    out["src_index"] = np.array(int(np.flatnonzero(b)[0]))
    out["iters"] = np.array(len(hst) - 1)
    out["hist"] = hst
    out["rel_res_true"] = np.array(np.linalg.norm(r) / np.linalg.norm(b))
    _samples(x, out, "u")
    # the same problem solved to a true residual near 1e-9 (C oracle, COLOUR27 row order,
    # preconditioned tolerance 1e-10): the FP64 reference the errors of faster solves are
    # stated against
    g = O.make_grid(n, m.h, m.npml6)
    xe, he = slim_ref.linearsolve_cgmn(g, wn, b, tol=1e-10, maxit=20000, order=O.ORDER_COLOUR27,
                                       nthreads=os.cpu_count())
    out["exact/iters"] = np.array(len(he) - 1)
    out["exact/rel_res_true"] = np.array(slim_ref.true_residual(g, wn, b, xe))
    _samples(xe, out, "exact")


def config1_solve_case(out):
    """The config-1 forward solve (201 x 201 x 101, 20-point PML, 6 Hz, surface point source) by
    the C oracle in FP64 to a true residual near 1e-9 (COLOUR27 row order, preconditioned
    tolerance 1e-10, rows of a colour in parallel): the FP64 reference the bench states the
    error of its wavefields against."""
    from h3d import models
    from oracle import h3d_oracle as O
    from oracle import slim_ref

    m = models.config1()
    wn, b = m.wavenumber(), m.point_source()
    g = O.make_grid(m.n_total, m.h, m.npml6)
    x, hst = slim_ref.linearsolve_cgmn(g, wn, b, tol=1e-10, maxit=40000, order=O.ORDER_COLOUR27,
                                       nthreads=int(os.environ.get("GOLDEN_THREADS", os.cpu_count())))
    out["wn_checksum"] = np.array([np.sum(wn), np.linalg.norm(wn), wn.min(), wn.max()])
    out["src_index"] = np.array(int(np.flatnonzero(b)[0]))
    out["iters"] = np.array(len(hst) - 1)
    out["rel_res_true"] = np.array(slim_ref.true_residual(g, wn, b, x))
    _samples(x, out, "exact")


def _config3_reduced():
    """The reduced config-3 gradient problem: sources 0 and 1 of the 32, all 400 receivers,
    6 Hz only, gradient w.r.t. squared slowness at the background model, observed data 0."""
    from h3d import models

    m = models.config3()
    meta = m.meta
    model = {"o": (0.0, 0.0, 0.0), "d": m.h, "n": m.n_phys, "npml6": m.npml6, "unit": "s2/m2",
             "f0": meta["f0"], "t0": 0.0}
    m0 = (meta["v0"] ** -2.0).reshape(-1, order="F")
    return model, m0, meta["src_xyz"][:2], meta["rec_xyz"], np.array([6.0])


def _config3_worker(s):
    from oracle import h3d_oracle as O
    from oracle import slim_ref

    model, m0, src, rec, freqs = _config3_reduced()
    Dobs = np.zeros((len(rec), 1), complex)
    f, g = slim_ref.pdefunc("obj", m0, model, src[s:s + 1], np.ones(1), rec, freqs, Dobs=Dobs,
                            tol=1e-6, maxit=10000, order=O.ORDER_LEX, nthreads=1)
    return f, g


def config3_grad_case(out):
    """PDEfunc OBJ (oracle/slim_ref.pdefunc over the C oracle, whose lexicographic sweep equals
    the compiled reference gateway bit for bit) on the reduced config-3 problem of
    _config3_reduced(), one source per process; the reference's own solver settings
    (CGMN, tol 1e-6 on the preconditioned residual, one source at a time, PDEfunc.m:157)."""
    import multiprocessing as mp

    model, m0, src, rec, freqs = _config3_reduced()
    with mp.get_context("spawn").Pool(len(src)) as pool:
        res = pool.map(_config3_worker, range(len(src)))
    f = sum(r[0] for r in res)
    g = np.sum([r[1] for r in res], axis=0)
    out["f"] = np.array(f)
    out["f_per_source"] = np.array([r[0] for r in res])
    out["n_phys"] = np.array(model["n"], float)
    out["freqs"] = freqs
    out["m0_checksum"] = np.array([np.sum(m0), np.linalg.norm(m0)])
    _samples(g, out, "g")


def band_case(out):
    from oracle import slim_band as SB

    rng = np.random.default_rng(31)
    n, h = (7, 6, 8), (20.0, 25.0, 15.0)
    npml = np.full((2, 3), 2.0)
    wn3 = (2 * np.pi * 4.0) ** 2 / (1500.0 + 2000.0 * rng.random(n)) ** 2
    H, idx = SB.helmholtz_3d_bands(wn3, h, npml)
    Ha, idxa = SB.htransp(H, idx)
    Ha = np.conj(Ha)
    N = H.shape[1]
    X = rng.standard_normal((N, 2)) + 1j * rng.standard_normal((N, 2))
    B = rng.standard_normal((N, 2)) + 1j * rng.standard_normal((N, 2))
    mv, sw = M.load_reference("Hmvp_MT_mex"), M.load_reference("sweep_MT_mex")
    out["n"], out["h"], out["npml"] = np.array(n, float), np.array(h, float), npml
    out["wn"] = wn3.reshape(-1, order="F")
    out["H"], out["idx"], out["Hadj"], out["idxadj"] = H, idx, Ha, idxa
    out["X"], out["B"] = X, B
    for tag, (A, o) in (("forw", (H, idx)), ("adj", (Ha, idxa))):
        rn = SB.row_norms_sq(A)
        out[f"{tag}/rn"] = rn
        out[f"{tag}/mvp"] = mv(A, o.astype(float), X, 2.0)
        out[f"{tag}/swp"] = sw(A, o.astype(float), X, B, 1.3, rn)


def main():
    if not M.reference_available():
        raise SystemExit("reference gateways missing: run `make -C oracle ref` first")
    if sys.argv[1:] == ["config0_solve"]:
        c0s: dict = {}
        config0_solve_case(c0s)
        np.savez_compressed(os.path.join(HERE, "config0_solve.npz"), **c0s)
        print("wrote config0_solve.npz: iterations", int(c0s["iters"]))
        return
    if sys.argv[1:] == ["config1_solve"]:
        c1: dict = {}
        config1_solve_case(c1)
        np.savez_compressed(os.path.join(HERE, "config1_solve.npz"), **c1)
        print("wrote config1_solve.npz: iterations", int(c1["iters"]))
        return
    if sys.argv[1:] == ["config3_grad"]:
        c3: dict = {}
        config3_grad_case(c3)
        np.savez_compressed(os.path.join(HERE, "config3_grad.npz"), **c3)
        print("wrote config3_grad.npz: f", float(c3["f"]))
        return
    band: dict = {}
    band_case(band)
    np.savez_compressed(os.path.join(HERE, "band_small.npz"), **band)
    if sys.argv[1:] == ["band"]:
        print("wrote band_small.npz")
        return
    small: dict = {}
    small_case("g7", (7, 6, 5), (25.0, 25.0, 25.0), [[2, 2, 2], [2, 2, 2]], 11, small)
    small_case("g12", (12, 11, 10), (25.0, 20.0, 15.0), [[3, 2, 3], [2, 3, 1]], 12, small)
    np.savez_compressed(os.path.join(HERE, "stencil_small.npz"), **small)
    c0: dict = {}
    config0_case(c0)
    np.savez_compressed(os.path.join(HERE, "config0_mvp.npz"), **c0)
    print("wrote", sorted(os.listdir(HERE)))


if __name__ == "__main__":
    main()
