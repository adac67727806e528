"""Host-side pieces of the FWI layer (h3d.fwi) on CPU tensors, against the oracle:
param2wavenum.m:20-49 (wn, dwn, ddwn for every unit), opExtension.m:85-101 mode 1 (edge
replication of the physical model into the PML; its adjoint passes the dot test) and
fwi_wavelet.m:24-28 (the Ricker-weighted spectrum)."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "..", "slim-release-apps_gb300"))

from oracle import slim_ref  # noqa: E402


@pytest.mark.parametrize("unit", ["m/s", "s2/m2", "s2/km2"])
def test_param2wavenum_matches_oracle(unit):
    import torch
    from h3d import fwi

    rng = np.random.default_rng(0)
    v = 1500.0 + 2000.0 * rng.random(50)
    if unit != "m/s":
        v = v ** -2.0 * (1e6 if unit == "s2/km2" else 1.0)
    mine = fwi.param2wavenum(torch.as_tensor(v), 4.5, unit)
    ref = slim_ref.param2wavenum(v, 4.5, unit)
    for a, b in zip(mine, ref):
        a = a.numpy() if hasattr(a, "numpy") else np.asarray(a)
        np.testing.assert_allclose(a, np.broadcast_to(b, a.shape), rtol=1e-15, atol=0)


def test_edge_extension_matches_oracle_and_adjoint():
    import torch
    from h3d import fwi

    rng = np.random.default_rng(1)
    v = rng.random((7, 5, 6))
    npml6 = (2, 3, 1, 4, 0, 2)
    mine = fwi.extend_edges(torch.as_tensor(v), npml6).numpy()
    ref = slim_ref.extend3d(v, npml6, mode=1)
    assert mine.shape == (12, 10, 8)
    assert np.array_equal(mine, ref)
    y = rng.random(ref.shape)
    lhs = np.sum(ref * y)
    rhs = np.sum(v * slim_ref.extend3d(y, npml6, mode=1, adjoint=True))
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)


def test_wavelet_matches_oracle():
    from h3d import fwi

    f = np.array([3.0, 4.5, 6.0, 12.5])
    for t0, f0 in ((0.0, 8.0), (0.1, 10.0), (0.05, 0.0)):
        np.testing.assert_allclose(fwi.fwi_wavelet(f, t0, f0), slim_ref.fwi_wavelet(f, t0, f0), rtol=1e-15, atol=0)
