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
* ``band_small.npz`` -- the band-storage path on a 7x6x8 grid (PML 2): the 27 x N
  band matrix of helmholtz_3d.m (from oracle/slim_band.py, which MATLAB would be
  needed to run directly; pinned to the compiled matrix-free gateways), its adjoint
  bands, and the outputs of the compiled ``Hmvp_MT_mex`` and ``sweep_MT_mex``
  (forward and adjoint bands, 2 right-hand sides).

``python tests/golden/make_golden.py band`` writes only ``band_small.npz``.
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
