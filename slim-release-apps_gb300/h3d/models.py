"""Seeded synthetic velocity models and acquisition geometries for the benchmark workloads.

The reference ships no data for its 3D path, so the workloads are synthetic
stand-ins with the shapes, sizes and value distributions of the five benchmark
configurations:

* ``config0`` -- 61^3 incl. 10-point PML, h = 25 m, 4 Hz, linear 1500->3500 m/s
  depth gradient times (1 + 0.1 g), one unit point source.
* ``config1`` -- 201 x 201 x 101 incl. 20-point PML, h = 20 m, 6 Hz, 8 layered
  velocities 1500->4000 m/s with +-40 m interface relief and a +-5% random field.
* ``config2`` -- config-1 model, 64 sources (8 x 8, z = 2 cells), 3/4/5/6 Hz, Ricker
  spectrum weights with an 8 Hz peak.
* ``config3`` -- 161 x 161 x 81 incl. 15-point PML, h = 25 m, FWI with two Gaussian
  anomalies, 32 jittered sources, 400 receivers, 3 / 4.5 / 6 Hz.
* ``config4`` -- 48 problems with seeded sizes in [64, 192] per axis (10-point PML),
  12.5 Hz, config-0 velocity recipe, 1-16 sources each.

Random fields ("g"): white N(0,1) from ``numpy.random.default_rng(seed)``,
filtered by a Gaussian kernel of standard deviation L/h cells (reflecting
edges, kernel truncated at 4 sigma), rescaled to unit standard deviation and
clipped to [-1, 1].

Grid convention (as the reference, ``Helm3d_27pt.h:21-23``): arrays are indexed
(x, y, z), flattened column-major (x fastest); z grows downward; the PML padding
is filled by edge replication (``opExtension`` mode 1, ``opExtension.m:94-101``).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


def _gauss_kernel(sigma: float) -> np.ndarray:
    r = max(1, int(np.ceil(4.0 * sigma)))
    t = np.arange(-r, r + 1, dtype=np.float64)
    k = np.exp(-0.5 * (t / sigma) ** 2)
    return k / k.sum()


def _filter_axis(a: np.ndarray, k: np.ndarray, axis: int) -> np.ndarray:
    r = (k.size - 1) // 2
    pad = [(0, 0)] * a.ndim
    pad[axis] = (r, r)
    p = np.pad(a, pad, mode="symmetric")
    out = np.zeros_like(a)
    n = a.shape[axis]
    for t in range(k.size):
        sl = [slice(None)] * a.ndim
        sl[axis] = slice(t, t + n)
        out += k[t] * p[tuple(sl)]
    return out


def random_field(shape, corr_len: float, h: float, seed: int) -> np.ndarray:
    """Unit-std Gaussian random field with correlation length ``corr_len`` (m), clipped to [-1,1]."""
    rng = np.random.default_rng(seed)
    g = rng.standard_normal(tuple(shape))
    k = _gauss_kernel(corr_len / h)
    for ax in range(g.ndim):
        g = _filter_axis(g, k, ax)
    g = (g - g.mean()) / g.std()
    return np.clip(g, -1.0, 1.0)


def extend_edges(v: np.ndarray, npml6) -> np.ndarray:
    """Pad a physical (x,y,z) array into the PML by edge replication (opExtension mode 1)."""
    lx, hx, ly, hy, lz, hz = (int(p) for p in npml6)
    return np.pad(v, ((lx, hx), (ly, hy), (lz, hz)), mode="edge")


def ricker_weight(f, f0: float, t0: float = 0.0):
    """Source spectrum w(f) = f^2 exp(-(f/f0)^2) exp(-i 2 pi f t0) (fwi_wavelet.m:51-54)."""
    f = np.asarray(f, dtype=np.float64)
    w = np.exp(-1j * 2 * np.pi * f * t0)
    if f0:
        w = f ** 2 * np.exp(-(f / f0) ** 2) * w
    return w


@dataclass
class Model:
    """A velocity model on the physical grid plus PML widths and spacing."""

    v: np.ndarray                  # physical velocity (m/s), shape (nx, ny, nz)
    h: tuple                       # (hx, hy, hz) in m
    npml6: tuple                   # lo_x, hi_x, lo_y, hi_y, lo_z, hi_z
    freq: float = 0.0              # default frequency (Hz)
    name: str = ""
    sources: np.ndarray = field(default_factory=lambda: np.zeros((0, 3)))  # total-grid index coords
    meta: dict = field(default_factory=dict)

    @property
    def n_phys(self):
        return tuple(int(s) for s in self.v.shape)

    @property
    def n_total(self):
        p = self.npml6
        return (self.v.shape[0] + p[0] + p[1], self.v.shape[1] + p[2] + p[3],
                self.v.shape[2] + p[4] + p[5])

    @property
    def N(self) -> int:
        return int(np.prod(self.n_total))

    def npml23(self) -> np.ndarray:
        """The reference's 2x3 PML matrix (rows lo/hi, columns x/y/z)."""
        p = self.npml6
        return np.array([[p[0], p[2], p[4]], [p[1], p[3], p[5]]], dtype=np.float64)

    def v_total(self) -> np.ndarray:
        return extend_edges(self.v, self.npml6)

    def wavenumber(self, freq: float | None = None) -> np.ndarray:
        """wn = (2 pi f)^2 / v^2 on the PML grid, flattened x-fastest (param2wavenum.m:20-29)."""
        f = self.freq if freq is None else freq
        v = self.v_total()
        return ((2 * np.pi * f) ** 2 * v.astype(np.float64) ** -2).reshape(-1, order="F")

    def point_source(self, idx=None) -> np.ndarray:
        """Unit complex delta at a total-grid index triple (default: the first source)."""
        i, j, k = (int(c) for c in (self.sources[0] if idx is None else idx))
        nx, ny, _ = self.n_total
        b = np.zeros(self.N, dtype=np.complex128)
        b[i + nx * j + nx * ny * k] = 1.0
        return b


def _linear_gradient(n_phys, h, v_top, v_bot):
    nz = n_phys[2]
    z = np.arange(nz) * h
    zmax = (nz - 1) * h
    return np.broadcast_to(v_top + (v_bot - v_top) * z / zmax, n_phys).copy()


def config0(seed: int = 0) -> Model:
    """61^3 incl. 10-pt PML, h=25 m, 4 Hz; v = (1500 + 2000 z/zmax)(1 + 0.1 g), L=150 m."""
    n_phys = (41, 41, 41)
    h = 25.0
    g = random_field(n_phys, 150.0, h, seed)
    v = _linear_gradient(n_phys, h, 1500.0, 3500.0) * (1.0 + 0.1 * g)
    m = Model(v=v, h=(h, h, h), npml6=(10,) * 6, freq=4.0, name="config0")
    m.sources = np.array([[30, 30, 10 + 2]])
    return m


def config1(seed: int = 1) -> Model:
    """201x201x101 incl. 20-pt PML, h=20 m, 6 Hz, 8 layers 1500->4000 m/s, relief, +-5% GRF."""
    n_phys = (161, 161, 61)
    h = 20.0
    rng = np.random.default_rng(seed)
    nlay = 8
    vel = np.linspace(1500.0, 4000.0, nlay)
    zmax = (n_phys[2] - 1) * h
    depths = np.linspace(0.0, zmax, nlay + 1)[1:-1]             # 7 interfaces
    z = np.arange(n_phys[2]) * h
    v = np.full(n_phys, vel[0])
    for q, d in enumerate(depths):
        relief = 40.0 * random_field(n_phys[:2], 400.0, h, int(rng.integers(1 << 30)))
        iface = d + relief                                        # (nx, ny)
        below = z[None, None, :] >= iface[:, :, None]
        v = np.where(below, vel[q + 1], v)
    g = random_field(n_phys, 200.0, h, int(rng.integers(1 << 30)))
    v = v * (1.0 + 0.05 * g)
    m = Model(v=v, h=(h, h, h), npml6=(20,) * 6, freq=6.0, name="config1")
    m.sources = np.array([[100, 100, 20]])
    return m


def config2(seed: int = 1):
    """Config-1 model, 64 sources on an 8x8 surface grid at z = 2 cells, f in {3,4,5,6} Hz."""
    m = config1(seed)
    p = m.npml6
    nxi, nyi, _ = m.n_phys
    xs = p[0] + np.round(np.linspace(0, nxi - 1, 10)[1:-1]).astype(int)
    ys = p[2] + np.round(np.linspace(0, nyi - 1, 10)[1:-1]).astype(int)
    src = np.array([[x, y, p[4] + 2] for y in ys for x in xs])
    m.sources = src
    m.name = "config2"
    freqs = np.array([3.0, 4.0, 5.0, 6.0])
    m.meta.update(freqs=freqs, weights=ricker_weight(freqs, 8.0))
    return m


def config3(seed: int = 3):
    """161x161x81 incl. 15-pt PML, h=25 m; true = gradient + two Gaussian anomalies; v0 = gradient."""
    n_phys = (131, 131, 51)
    h = 25.0
    rng = np.random.default_rng(seed)
    v0 = _linear_gradient(n_phys, h, 1500.0, 3500.0)
    X, Y, Z = np.meshgrid(*(np.arange(s) * h for s in n_phys), indexing="ij")
    vt = v0.copy()
    for amp in (300.0, -250.0):
        c = [rng.uniform(0.3, 0.7) * (s - 1) * h for s in n_phys]
        r2 = (X - c[0]) ** 2 + (Y - c[1]) ** 2 + (Z - c[2]) ** 2
        vt += amp * np.exp(-0.5 * r2 / 150.0 ** 2)
    npml = (15,) * 6
    # 32 sources: jittered 8 x 4 surface grid (physical coordinates, m), depth 2 cells
    gx = (np.arange(8) + 0.5) / 8 * (n_phys[0] - 1) * h
    gy = (np.arange(4) + 0.5) / 4 * (n_phys[1] - 1) * h
    src = np.array([[x + rng.uniform(-0.3, 0.3) * h * 4, y + rng.uniform(-0.3, 0.3) * h * 4, 2 * h]
                    for y in gy for x in gx])
    rx = (np.arange(20) + 0.5) / 20 * (n_phys[0] - 1) * h
    ry = (np.arange(20) + 0.5) / 20 * (n_phys[1] - 1) * h
    rec = np.array([[x, y, 1 * h] for y in ry for x in rx])
    m = Model(v=vt, h=(h, h, h), npml6=npml, freq=3.0, name="config3")
    m.meta.update(v0=v0, src_xyz=src, rec_xyz=rec, freqs=np.array([3.0, 4.5, 6.0]), f0=8.0)
    return m


def config4(seed: int = 4, nprob: int = 48):
    """48 problems: total dims U{64..192} per axis (10-pt PML), h=20 m, 12.5 Hz, 1-16 sources."""
    rng = np.random.default_rng(seed)
    h = 20.0
    f = 1500.0 / (6 * h)
    probs = []
    for p in range(nprob):
        n_tot = rng.integers(64, 193, size=3)
        n_phys = tuple(int(s) - 20 for s in n_tot)
        g = random_field(n_phys, 150.0, h, int(rng.integers(1 << 30)))
        v = _linear_gradient(n_phys, h, 1500.0, 3500.0) * (1.0 + 0.1 * g)
        v = np.maximum(v, 1500.0)
        m = Model(v=v, h=(h, h, h), npml6=(10,) * 6, freq=f, name=f"config4[{p}]")
        ns = int(rng.integers(1, 17))
        xs = rng.integers(10, 10 + n_phys[0], size=ns)
        ys = rng.integers(10, 10 + n_phys[1], size=ns)
        m.sources = np.stack([xs, ys, np.full(ns, 12)], axis=1)
        probs.append(m)
    return probs
