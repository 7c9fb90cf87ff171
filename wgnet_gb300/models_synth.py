"""Seeded synthetic velocity models in the style of OpenFWI's families (the dataset itself is not
used): flat layers, sinusoidally curved interfaces, layered models cut by dipping faults, and
layered backgrounds with elliptical Gaussian inclusions. Velocities in m/s, clipped to
[1500, 4500], increasing with depth in the layered background.
"""

from __future__ import annotations

import numpy as np

VMIN, VMAX = 1500.0, 4500.0
FAMILIES = ("flat", "curved", "fault", "blob")


def _layer_velocities(rng, n):
    return np.sort(rng.uniform(VMIN, VMAX, n))


def _layered(rng, nz, nx, depth_fn):
    """Layers whose k-th interface sits at depth_fn(k, x) (cells)."""
    n = int(rng.integers(3, 6))
    vel = _layer_velocities(rng, n)
    base = np.sort(rng.choice(np.arange(int(0.08 * nz) + 2, nz - 3), n - 1, replace=False)).astype(np.float64)
    z = np.arange(nz, dtype=np.float64)[:, None]
    x = np.arange(nx, dtype=np.float64)[None, :]
    layer = np.zeros((nz, nx), np.int64)
    for k in range(n - 1):
        layer += (z >= depth_fn(k, base[k], x)).astype(np.int64)
    return vel[np.minimum(layer, n - 1)]


def flat(rng, nz, nx):
    return _layered(rng, nz, nx, lambda k, b, x: np.full_like(x, b))


def curved(rng, nz, nx):
    amp = rng.uniform(2.0, 10.0)
    wavelength = rng.uniform(0.5, 2.0) * nx
    phase = rng.uniform(0, 2 * np.pi)
    return _layered(rng, nz, nx, lambda k, b, x: b + amp * np.sin(2 * np.pi * x / wavelength + phase + 0.3 * k))


def fault(rng, nz, nx):
    v = flat(rng, nz, nx)
    for _ in range(int(rng.integers(1, 3))):
        throw = int(rng.integers(3, 16)) * (1 if rng.random() < 0.5 else -1)
        x0 = rng.uniform(0.2, 0.8) * nx
        dip = np.tan(np.deg2rad(rng.uniform(45.0, 80.0))) * (1 if rng.random() < 0.5 else -1)
        z = np.arange(nz)[:, None]
        x = np.arange(nx)[None, :]
        hanging = (x - x0) * dip > z  # one side of the fault plane
        zsrc = np.clip(z - throw, 0, nz - 1)
        shifted = v[zsrc[:, 0]][:, :]
        v = np.where(hanging, shifted, v)
    return v


def blob(rng, nz, nx):
    v = flat(rng, nz, nx)
    z = np.arange(nz, dtype=np.float64)[:, None]
    x = np.arange(nx, dtype=np.float64)[None, :]
    for _ in range(int(rng.integers(1, 5))):
        cz, cx = rng.uniform(0.15, 0.9) * nz, rng.uniform(0.1, 0.9) * nx
        sz, sx = rng.uniform(0.04, 0.15) * nz, rng.uniform(0.04, 0.15) * nx
        ang = rng.uniform(0, np.pi)
        dv = rng.uniform(300.0, 800.0) * (1 if rng.random() < 0.5 else -1)
        u = ((x - cx) * np.cos(ang) + (z - cz) * np.sin(ang)) / sx
        w = ((z - cz) * np.cos(ang) - (x - cx) * np.sin(ang)) / sz
        v = v + dv * np.exp(-0.5 * (u * u + w * w))
    return v


_GEN = {"flat": flat, "curved": curved, "fault": fault, "blob": blob}


def make_model(seed: int, nz: int = 70, nx: int = 70, family: str | None = None) -> np.ndarray:
    rng = np.random.default_rng(seed)
    fam = family or FAMILIES[seed % len(FAMILIES)]
    return np.clip(_GEN[fam](rng, nz, nx), VMIN, VMAX).astype(np.float32)


def make_batch(n: int, seed: int = 0, nz: int = 70, nx: int = 70, families=FAMILIES) -> np.ndarray:
    """`[n, nz, nx]` models, families round-robin, model i seeded with seed * 1_000_003 + i."""
    out = np.empty((n, nz, nx), np.float32)
    for i in range(n):
        out[i] = make_model(seed * 1_000_003 + i, nz, nx, families[i % len(families)])
    return out


def smooth(v: np.ndarray, sigma_cells: float) -> np.ndarray:
    """Separable Gaussian low-pass with reflect padding (the macro-model smoothing of
    python/wgnet/igm.py:52-63), applied to `[..., nz, nx]`."""
    if sigma_cells <= 0:
        return v.astype(np.float32)
    half = int(np.ceil(3.0 * sigma_cells))
    t = np.arange(-half, half + 1, dtype=np.float64)
    k = np.exp(-0.5 * (t / sigma_cells) ** 2)
    k /= k.sum()
    x = np.asarray(v, np.float64)
    pad = [(0, 0)] * (x.ndim - 1) + [(half, half)]
    xp = np.pad(x, pad, mode="reflect")
    x = sum(k[j] * xp[..., j:j + x.shape[-1]] for j in range(len(k)))
    pad = [(0, 0)] * (x.ndim - 2) + [(half, half), (0, 0)]
    xp = np.pad(x, pad, mode="reflect")
    x = sum(k[j] * xp[..., j:j + x.shape[-2], :] for j in range(len(k)))
    return x.astype(np.float32)
