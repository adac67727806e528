"""Band-storage (mat_free = false) layer of the 3D Helmholtz modelling, restated in numpy.

TEST INFRASTRUCTURE ONLY: the checker for the library's band-storage entry points
(h3d_band_coefs / h3d_band_mvp / h3d_band_sweep); nothing in the product imports it.

Follows, in the reference project:
  * create_pml.m:33-99          -- 1-D PML functions xi(:,1) (lower) and xi(:,2) (upper)
  * helmholtz_3d.m:35-190       -- the 27 x N band matrix H and the offset vector idx
  * Htransp.m:21-35             -- band storage of the transpose (circular shift per band)
  * Hmvp_MT_mex.c:53-73         -- y = A x on band storage (linear-index bounds)
  * sweep_MT_mex.c:55-97        -- Kaczmarz double sweep on band storage
  * opBandStorage.m:139-144     -- squared row norms, sum over all bands of a column

Band index t = (dx+1) + 3(dy+1) + 9(dz+1) (MMM = 1 ... PPP = 27 in the reference's 1-based
naming, x the first letter); column i of the band matrix is grid row i, x fastest.
"""
from __future__ import annotations

import numpy as np

OFFS = [(dx, dy, dz) for dz in (-1, 0, 1) for dy in (-1, 0, 1) for dx in (-1, 0, 1)]


def create_pml(nx: int, ny: int, nz: int, npml):
    """create_pml.m:33-99.  npml: 2 x 3, row 0 = "top" and row 1 = "bot" widths per axis
    (the reference reads np(1,a) as the upper side and np(2,a) as the lower side)."""
    npml = np.asarray(npml, dtype=np.int64).reshape(2, 3)
    out = []
    for a, n in enumerate((nx, ny, nz)):
        top, bot = int(npml[0, a]), int(npml[1, a])
        s = 1.0 / (n + 1)
        g = np.zeros(n + 2)
        if bot > 0:
            m = np.arange(0, bot)
            g[0:bot] = np.cos((np.pi * m * s) / (2 * (bot / n)))
        if top > 0:
            m = np.arange(n + 2 - top, n + 2)          # 1-based (nx+2-npx_top : nx+1)
            g[n + 2 - top:n + 2] = np.cos((np.pi * (1 - m * s)) / (2 * (top / n)))
        one = 1 + 1j * g
        xi = np.zeros((n, 2), dtype=np.complex128)
        xi[:, 0] = 2.0 / (one[1:n + 1] * (one[1:n + 1] + one[0:n]))
        xi[:, 1] = 2.0 / (one[1:n + 1] * (one[1:n + 1] + one[2:n + 2]))
        out.append(xi)
    return out


def helmholtz_3d_bands(wn: np.ndarray, h, npml):
    """helmholtz_3d.m:35-190 with the wavenumber already formed (param2wavenum.m:20-49 is
    applied by the caller).  wn: (nx, ny, nz) real or complex.  Returns (H, idx) with H of
    shape (27, N) complex and idx the 27 linear offsets."""
    nx, ny, nz = wn.shape
    xix, xiy, xiz = create_pml(nx, ny, nz, npml)
    w = np.zeros((nx + 2, ny + 2, nz + 2), dtype=np.result_type(wn.dtype, np.float64))
    w[1:-1, 1:-1, 1:-1] = wn
    hx2, hy2, hz2 = (float(v) ** 2 for v in h)
    hyz, hxy, hxz, hxyz = hy2 + hz2, hy2 + hx2, hx2 + hz2, hx2 + hy2 + hz2
    w1, w2, w3 = 1.8395262e-5, 0.890077 / 3, 0.1099046 / 4
    wm1, wm2, wm3, wm4 = 0.49649658, 0.4510125 / 6, 0.052487 / 12, 0.45523e-5 / 8
    w3a = (w3 * 3) / (4 * hxyz)
    sh = (nx, ny, nz)
    MNN = np.broadcast_to(xix[:, 0][:, None, None], sh)
    PNN = np.broadcast_to(xix[:, 1][:, None, None], sh)
    NMN = np.broadcast_to(xiy[:, 0][None, :, None], sh)
    NPN = np.broadcast_to(xiy[:, 1][None, :, None], sh)
    NNM = np.broadcast_to(xiz[:, 0][None, None, :], sh)
    NNP = np.broadcast_to(xiz[:, 1][None, None, :], sh)

    def W(dx, dy, dz):
        return w[1 + dx:nx + 1 + dx, 1 + dy:ny + 1 + dy, 1 + dz:nz + 1 + dz]

    def t(dx, dy, dz):
        return (dx + 1) + 3 * (dy + 1) + 9 * (dz + 1)

    H = np.zeros((27, nx, ny, nz), dtype=np.complex128)
    ax = w1 / hx2 + w2 / hx2 + w2 / hxz + w2 / hxy
    ay = w1 / hy2 + w2 / hy2 + w2 / hyz + w2 / hxy
    az = w1 / hz2 + w2 / hz2 + w2 / hxz + w2 / hyz
    H[t(-1, 0, 0)] = -ax * MNN + (w2 / (2 * hxz)) * (NNM + NNP) + (w2 / (2 * hxy)) * (NMN + NPN) - 8 * w3a * MNN - wm2 * W(-1, 0, 0)
    H[t(1, 0, 0)] = -ax * PNN + (w2 / (2 * hxz)) * (NNM + NNP) + (w2 / (2 * hxy)) * (NMN + NPN) - 8 * w3a * PNN - wm2 * W(1, 0, 0)
    H[t(0, -1, 0)] = -ay * NMN + (w2 / (2 * hyz)) * (NNM + NNP) + (w2 / (2 * hxy)) * (MNN + PNN) - 8 * w3a * NMN - wm2 * W(0, -1, 0)
    H[t(0, 1, 0)] = -ay * NPN + (w2 / (2 * hyz)) * (NNM + NNP) + (w2 / (2 * hxy)) * (MNN + PNN) - 8 * w3a * NPN - wm2 * W(0, 1, 0)
    H[t(0, 0, -1)] = -az * NNM + (w2 / (2 * hyz)) * (NMN + NPN) + (w2 / (2 * hxz)) * (MNN + PNN) - 8 * w3a * NNM - wm2 * W(0, 0, -1)
    H[t(0, 0, 1)] = -az * NNP + (w2 / (2 * hyz)) * (NMN + NPN) + (w2 / (2 * hxz)) * (MNN + PNN) - 8 * w3a * NNP - wm2 * W(0, 0, 1)
    # yz edges
    H[t(0, 1, 1)] = -(w2 / (2 * hyz)) * (NNP + NPN) + 2 * w3a * (MNN + PNN) - wm3 * W(0, 1, 1)
    H[t(0, -1, -1)] = -(w2 / (2 * hyz)) * (NNM + NMN) + 2 * w3a * (MNN + PNN) - wm3 * W(0, -1, -1)
    H[t(0, 1, -1)] = -(w2 / (2 * hyz)) * (NPN + NNM) + 2 * w3a * (MNN + PNN) - wm3 * W(0, 1, -1)
    H[t(0, -1, 1)] = -(w2 / (2 * hyz)) * (NMN + NNP) + 2 * w3a * (MNN + PNN) - wm3 * W(0, -1, 1)
    # xz edges
    H[t(1, 0, 1)] = -(w2 / (2 * hxz)) * (NNP + PNN) + 2 * w3a * (NMN + NPN) - wm3 * W(1, 0, 1)
    H[t(-1, 0, -1)] = -(w2 / (2 * hxz)) * (NNM + MNN) + 2 * w3a * (NMN + NPN) - wm3 * W(-1, 0, -1)
    H[t(1, 0, -1)] = -(w2 / (2 * hxz)) * (NNM + PNN) + 2 * w3a * (NMN + NPN) - wm3 * W(1, 0, -1)
    H[t(-1, 0, 1)] = -(w2 / (2 * hxz)) * (NNP + MNN) + 2 * w3a * (NMN + NPN) - wm3 * W(-1, 0, 1)
    # xy edges
    H[t(1, -1, 0)] = -(w2 / (2 * hxy)) * (PNN + NMN) + 2 * w3a * (NNM + NNP) - wm3 * W(1, -1, 0)
    H[t(-1, 1, 0)] = -(w2 / (2 * hxy)) * (MNN + NPN) + 2 * w3a * (NNM + NNP) - wm3 * W(-1, 1, 0)
    H[t(1, 1, 0)] = -(w2 / (2 * hxy)) * (PNN + NPN) + 2 * w3a * (NNM + NNP) - wm3 * W(1, 1, 0)
    H[t(-1, -1, 0)] = -(w2 / (2 * hxy)) * (MNN + NMN) + 2 * w3a * (NNM + NNP) - wm3 * W(-1, -1, 0)
    # corners
    H[t(1, 1, 1)] = -2 * w3a * (NPN + NNP + PNN) - wm4 * W(1, 1, 1)
    H[t(-1, -1, -1)] = -2 * w3a * (NMN + NNM + MNN) - wm4 * W(-1, -1, -1)
    H[t(1, 1, -1)] = -2 * w3a * (NNM + PNN + NPN) - wm4 * W(1, 1, -1)
    H[t(-1, -1, 1)] = -2 * w3a * (NNP + MNN + NMN) - wm4 * W(-1, -1, 1)
    H[t(1, -1, 1)] = -2 * w3a * (PNN + NMN + NNP) - wm4 * W(1, -1, 1)
    H[t(-1, 1, -1)] = -2 * w3a * (MNN + NPN + NNM) - wm4 * W(-1, 1, -1)
    H[t(1, -1, -1)] = -2 * w3a * (PNN + NMN + NNM) - wm4 * W(1, -1, -1)
    H[t(-1, 1, 1)] = -2 * w3a * (MNN + NPN + NNP) - wm4 * W(-1, 1, 1)
    H[t(0, 0, 0)] = (-(w1 + 3 * w2 + (16 * w3a * hxyz) / 3 + wm1 - 1) * W(0, 0, 0)
                     + (ax + 8 * w3a) * (MNN + PNN) + (ay + 8 * w3a) * (NMN + NPN)
                     + (w1 / hz2 + w2 / hz2 + w2 / hyz + w2 / hxz + 8 * w3a) * (NNM + NNP))
    # zero the couplings to points outside the grid (helmholtz_3d.m:158-190)
    for k, (dx, dy, dz) in enumerate(OFFS):
        if dx == -1: H[k, 0, :, :] = 0
        if dx == 1: H[k, nx - 1, :, :] = 0
        if dy == -1: H[k, :, 0, :] = 0
        if dy == 1: H[k, :, ny - 1, :] = 0
        if dz == -1: H[k, :, :, 0] = 0
        if dz == 1: H[k, :, :, nz - 1] = 0
    idx = np.array([dx + nx * dy + nx * ny * dz for dx, dy, dz in OFFS], dtype=np.int64)
    return H.reshape(27, -1, order="F"), idx


def htransp(H: np.ndarray, idx: np.ndarray):
    """Htransp.m:21-35 (short-and-fat branch): band k shifted circularly by idx(k), offset
    negated.  opBandStorage.m:127-129 then conjugates for the adjoint."""
    Ht = np.empty_like(H)
    for k in range(H.shape[0]):
        Ht[k] = np.roll(H[k], int(idx[k]))
    return Ht, -idx


def band_mvp(H: np.ndarray, idx: np.ndarray, x: np.ndarray) -> np.ndarray:
    """Hmvp_MT_mex.c:53-73: y(i) = sum_j H(j,i) x(i + idx(j)) over 0 <= i + idx(j) < N."""
    nd, N = H.shape
    X = x.reshape(N, -1)
    y = np.zeros(X.shape, dtype=np.complex128)
    i = np.arange(N)
    for j in range(nd):
        src = i + int(idx[j])
        ok = (src >= 0) & (src < N)
        y[ok] += H[j, ok][:, None] * X[src[ok]]
    return y.reshape(x.shape)


def row_norms_sq(H: np.ndarray) -> np.ndarray:
    """opBandStorage.m:139-144: sum over all bands of |H(:,i)|^2."""
    return np.sum(np.abs(H) ** 2, axis=0)


def band_sweep(H: np.ndarray, idx: np.ndarray, x: np.ndarray, b: np.ndarray, w: float,
               rn: np.ndarray) -> np.ndarray:
    """sweep_MT_mex.c:55-97: rows 0..N-1 then N-1..0, per right-hand side; small N only."""
    nd, N = H.shape
    X = np.array(x, dtype=np.complex128).reshape(N, -1).copy()
    B = np.asarray(b, dtype=np.complex128).reshape(N, -1)
    for s in range(X.shape[1]):
        xs = X[:, s]
        for m in range(2 * N):
            i = 2 * N - m - 1 if m >= N else m
            atx = 0j
            cols = []
            for j in range(nd):
                q = i + int(idx[j])
                if 0 <= q < N:
                    atx += H[j, i] * xs[q]
                    cols.append((j, q))
            c = complex(w * (B[i, s].real - atx.real) / rn[i], w * (B[i, s].imag - atx.imag) / rn[i])
            for j, q in cols:
                xs[q] += np.conj(H[j, i]) * c
    return X.reshape(np.shape(x))
