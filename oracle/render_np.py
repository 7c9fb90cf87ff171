"""numpy restatement of the Gaussian renderer (python/wgnet/render.py:34-109) and its analytic
vector-Jacobian product. TEST INFRASTRUCTURE ONLY.

`render(params)` gathers, for every slot, its 25 x 25 window (pixel centres k + 0.5, anchors at
(2i+1, 2j+1)) and accumulates `amp * exp(-(u^2 + v^2) / 2)` with
u = (dx cos + dz sin) / sx, v = (dz cos - dx sin) / sz, as render_residual does with index_add_.
`render_vjp(params, cot)` is the derivative of sum(render(params) * cot) w.r.t. params, written
out by hand (the reference obtains it from autograd).
"""

from __future__ import annotations

import numpy as np

GRID, SIDE, WIN = 70, 35, 12


def _window():
    i = np.arange(SIDE)
    cz, cx = np.meshgrid(2 * i, 2 * i, indexing="ij")
    off = np.arange(-WIN, WIN + 1)
    oz, ox = np.meshgrid(off, off, indexing="ij")
    pz = cz.reshape(-1, 1) + oz.reshape(1, -1)
    px = cx.reshape(-1, 1) + ox.reshape(1, -1)
    valid = (pz >= 0) & (pz < GRID) & (px >= 0) & (px < GRID)
    return pz, px, valid


def _terms(params):
    p = np.asarray(params, np.float64)
    pz, px, valid = _window()
    i = np.arange(SIDE, dtype=np.float64)
    gz, gx = np.meshgrid(2 * i + 1, 2 * i + 1, indexing="ij")
    cx = (gx.reshape(-1) + p[..., 0])[..., None]
    cz = (gz.reshape(-1) + p[..., 1])[..., None]
    isx = np.exp(-p[..., 2])[..., None]
    isz = np.exp(-p[..., 3])[..., None]
    c = np.cos(p[..., 4])[..., None]
    s = np.sin(p[..., 4])[..., None]
    dx = (px + 0.5) - cx
    dz = (pz + 0.5) - cz
    ru = dx * c + dz * s
    rv = dz * c - dx * s
    u, v = ru * isx, rv * isz
    e = np.exp(-0.5 * (u * u + v * v)) * valid
    return p, pz, px, valid, isx, isz, c, s, ru, rv, u, v, e


def render(params) -> np.ndarray:
    """[B, 1225, 6] -> [B, 70, 70] (float64)."""
    p, pz, px, valid, *_, e = _terms(params)
    val = p[..., 5][..., None] * e
    out = np.zeros((p.shape[0], GRID * GRID + 1))
    flat = np.where(valid, pz * GRID + px, GRID * GRID)
    for b in range(p.shape[0]):
        np.add.at(out[b], flat.reshape(-1), val[b].reshape(-1))
    return out[:, : GRID * GRID].reshape(-1, GRID, GRID)


def render_vjp(params, cot) -> np.ndarray:
    """d/dparams of sum(render(params) * cot): [B, 1225, 6] (float64)."""
    p, pz, px, valid, isx, isz, c, s, ru, rv, u, v, e = _terms(params)
    ct = np.asarray(cot, np.float64).reshape(-1, GRID, GRID)
    cw = ct[:, np.clip(pz, 0, GRID - 1), np.clip(px, 0, GRID - 1)] * valid
    w = p[..., 5][..., None]
    ge = cw * w * e
    g = np.zeros(p.shape)
    g[..., 0] = np.sum(-ge * (u * (-c * isx) + v * (s * isz)), -1)
    g[..., 1] = np.sum(-ge * (u * (-s * isx) + v * (-c * isz)), -1)
    g[..., 2] = np.sum(ge * u * u, -1)
    g[..., 3] = np.sum(ge * v * v, -1)
    g[..., 4] = np.sum(-ge * (u * rv * isx - v * ru * isz), -1)
    g[..., 5] = np.sum(cw * e, -1)
    return g
