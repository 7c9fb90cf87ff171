"""Vectorised numpy restatement of the reference's two WGSL compute shaders. TEST INFRASTRUCTURE ONLY.

* `forward`: crates/wave-gauss-rs/src/shaders/splatForward.wgsl:48-121, one whole-grid numpy
  update per time step, all shots at once (receivers before the step, frame cells forced to zero,
  stored term 2 v dt^2 w before the source, bilinear source after the update).
* `adjoint`: crates/wave-gauss-rs/src/shaders/splatAdjoint.wgsl:58-131 with the parity ping-pong of
  psi/zeta, CSR residual injection and the gradient accumulation.
* `evaluate_adjoint`: the host steps of crates/wave-gauss-rs/src/wave_wgpu.rs:848-988.

It is written independently of `wave_oracle.cpp` (array formulation, not loops) and is used to
cross-check that restatement on small grids. `dtype` selects f32 (each numpy op rounds in f32,
matching the shader's per-operation rounding) or f64.
"""

from __future__ import annotations

import numpy as np

FD_PAD = 2


def ricker(samples: int, dt: float, peak_hz: float) -> np.ndarray:
    f = np.float32
    i = np.arange(samples, dtype=np.float32)
    t = i * f(dt) - f(1.5) / f(peak_hz)
    u = f(np.pi) * f(peak_hz) * t
    a = u * u
    return ((f(1) - f(2) * a) * np.exp(-a)).astype(np.float32)


def cpml(n: int, h: float, dt: float, width: int, max_vel: float, freq: float):
    x = np.arange(n, dtype=np.float64)
    start0, start1 = float(FD_PAD + width), float(n - 1 - FD_PAD - width)
    sigma0 = -(3.0 * float(np.float32(max_vel)) * np.log(0.001)) / (2.0 * width * float(np.float32(h)))
    frac = np.clip(np.maximum((start0 - x) / width, (x - start1) / width), 0.0, 1.0)
    sigma = sigma0 * frac * frac
    alpha = np.pi * float(np.float32(freq)) * (1.0 - frac)
    ax = np.exp(-(sigma + alpha) * float(np.float32(dt)))
    b = (sigma / (sigma + alpha)) * (ax - 1.0)
    a = np.where(frac == 0.0, 0.0, ax)
    db = np.zeros(n)
    db[2:n - 2] = ((8.0 / 12.0) * (b[3:n - 1] - b[1:n - 3]) - (1.0 / 12.0) * (b[4:n] - b[0:n - 4])) / float(np.float32(h))
    return a.astype(np.float32), b.astype(np.float32), db.astype(np.float32)


class Geometry:
    """Engine geometry (wave_wgpu.rs:204-270) for visible nx_vis x nz_vis, spacing h."""

    def __init__(self, nx_vis, nz_vis, pml, h, dt, peak_hz, vmin, vmax, sources, nrec=None):
        f = np.float32
        self.nx_vis, self.nz_vis, self.pml = nx_vis, nz_vis, pml
        self.pad = FD_PAD + pml
        self.nx, self.nz = nx_vis + 2 * self.pad, nz_vis + 2 * self.pad
        self.h, self.dt, self.vmin, self.vmax = f(h), f(dt), f(vmin), f(vmax)
        self.prof_x = cpml(self.nx, h, dt, pml, vmax, peak_hz)
        self.prof_z = cpml(self.nz, h, dt, pml, vmax, peak_hz)
        self.shots = len(sources)
        self.nrec = nx_vis if nrec is None else nrec
        self.src = [self.corners(s[0], s[1]) for s in np.asarray(sources, np.float32)]
        self.rec = [self.corners(f(r) * self.h, self.h) for r in range(self.nrec)]

    def corners(self, px, pz):
        f = np.float32
        gx = f(px) / self.h + f(self.pad)
        gz = f(pz) / self.h + f(self.pad)
        x0 = min(max(int(np.floor(gx)), 0) if np.isfinite(gx) else 0, self.nx - 2)
        z0 = min(max(int(np.floor(gz)), 0) if np.isfinite(gz) else 0, self.nz - 2)
        fx, fz = gx - f(x0), gz - f(z0)
        one = f(1)
        return [((z0, x0), (one - fx) * (one - fz)), ((z0, x0 + 1), fx * (one - fz)),
                ((z0 + 1, x0), (one - fx) * fz), ((z0 + 1, x0 + 1), fx * fz)]

    def pad_velocity(self, v_vis):
        v = np.asarray(v_vis, np.float32).reshape(self.nz_vis, self.nx_vis)
        zi = np.clip(np.arange(self.nz) - self.pad, 0, self.nz_vis - 1)
        xi = np.clip(np.arange(self.nx) - self.pad, 0, self.nx_vis - 1)
        vp = v[zi][:, xi]
        mask = ((vp > self.vmin) & (vp < self.vmax)).astype(np.float32)
        return np.clip(vp, self.vmin, self.vmax), mask


def _sh(a, d, axis):
    """a shifted so that out[i] = a[i + d] along `axis` (values outside: 0, never used)."""
    out = np.zeros_like(a)
    n = a.shape[axis]
    src = [slice(None)] * a.ndim
    dst = [slice(None)] * a.ndim
    if d >= 0:
        src[axis], dst[axis] = slice(d, n), slice(0, n - d)
    else:
        src[axis], dst[axis] = slice(0, n + d), slice(-d, n)
    out[tuple(dst)] = a[tuple(src)]
    return out


def forward(geo: Geometry, v_vis, wavelet, dtype=np.float32, store=False):
    """Returns traces [shots, nt, nrec] and (if store) stored [shots, nt, nz, nx]."""
    R = dtype
    nt = len(wavelet)
    nx, nz, S = geo.nx, geo.nz, geo.shots
    vel, _ = geo.pad_velocity(v_vis)
    v = vel.astype(R)
    rh = R(1) / R(geo.h)
    dt2 = R(geo.dt) * R(geo.dt)
    v2dt2 = v * v * dt2
    cur = np.zeros((S, nz, nx), R)
    prev = np.zeros((S, nz, nx), R)
    psi = np.zeros((2, S, nz, nx), R)
    zeta = np.zeros((2, S, nz, nx), R)
    traces = np.zeros((S, nt, geo.nrec), R)
    stored = np.zeros((S, nt, nz, nx), R) if store else None
    inner = np.zeros((nz, nx), bool)
    inner[FD_PAD:nz - FD_PAD, FD_PAD:nx - FD_PAD] = True
    region = geo.pml + 2 * FD_PAD
    xs, zs = np.arange(nx), np.arange(nz)
    in_x = np.broadcast_to(((xs < region) | (xs >= nx - region))[None, :], (nz, nx))
    in_z = np.broadcast_to(((zs < region) | (zs >= nz - region))[:, None], (nz, nx))
    profs = []
    for axis, (a, b, db) in ((2, geo.prof_x), (1, geo.prof_z)):
        shp = (1, 1, nx) if axis == 2 else (1, nz, 1)
        profs.append((axis, a.astype(R).reshape(shp), b.astype(R).reshape(shp), db.astype(R).reshape(shp)))
    c_d2a, c_d2b, c_d2c = R(-2.5), R(1.3333333333333333), R(0.08333333333333333)
    c_d1a, c_d1b = R(0.6666666666666666), R(0.08333333333333333)
    wv = np.asarray(wavelet, np.float32).astype(R)
    for t in range(nt):
        for r, crn in enumerate(geo.rec):
            acc = np.zeros(S, R)
            for (zc, xc), w in crn:
                acc = acc + R(w) * cur[:, zc, xc]
            traces[:, t, r] = acc
        u = cur
        w_acc = np.zeros_like(u)
        psi_next = np.zeros_like(psi)
        for k, (axis, A, B, DB) in enumerate(profs):
            um1, up1, um2, up2 = _sh(u, -1, axis), _sh(u, 1, axis), _sh(u, -2, axis), _sh(u, 2, axis)
            d2 = (c_d2a * u + c_d2b * (up1 + um1) - c_d2c * (up2 + um2)) * rh * rh
            inr = in_x if axis == 2 else in_z
            d1 = (c_d1a * (up1 - um1) - c_d1b * (up2 - um2)) * rh
            ps = psi[k]
            ap1 = _sh(A, 1, axis) * _sh(ps, 1, axis)
            am1 = _sh(A, -1, axis) * _sh(ps, -1, axis)
            ap2 = _sh(A, 2, axis) * _sh(ps, 2, axis)
            am2 = _sh(A, -2, axis) * _sh(ps, -2, axis)
            d1_apsi = (c_d1a * (ap1 - am1) - c_d1b * (ap2 - am2)) * rh
            tmp = (R(1) + B) * d2 + DB * d1 + d1_apsi
            w_pml = w_acc + ((R(1) + B) * tmp + A * zeta[k])
            w_acc = np.where(inr, w_pml, w_acc + d2)
            psi_next[k] = np.where(inr, B * d1 + A * ps, R(0))
            zeta[k] = np.where(inr & inner, B * tmp + A * zeta[k], zeta[k])
        if store:
            stored[:, t] = np.where(inner, R(2) * v * dt2 * w_acc, R(0))
        nxt = v2dt2 * w_acc + R(2) * u - prev
        for s in range(S):
            for (zc, xc), wgt in geo.src[s]:
                if inner[zc, xc]:
                    nxt[s, zc, xc] = nxt[s, zc, xc] + (-v2dt2[zc, xc]) * R(wgt) * wv[t]
        nxt = np.where(inner, nxt, R(0))
        psi_next = np.where(inner, psi_next, R(0))
        prev, cur = cur, nxt
        psi = psi_next
    return (traces, stored) if store else traces


def adjoint(geo: Geometry, v_vis, wavelet, residual, stored, dtype=np.float32):
    """residual [shots, nt, nrec]; stored [shots, nt, nz, nx] -> raw gradient [shots, nz, nx]."""
    R = dtype
    nt = len(wavelet)
    nx, nz, S = geo.nx, geo.nz, geo.shots
    vel, _ = geo.pad_velocity(v_vis)
    v = vel.astype(R)
    rh = R(1) / R(geo.h)
    dt2 = R(geo.dt) * R(geo.dt)
    vv = v * v * dt2
    inner = np.zeros((nz, nx), bool)
    inner[FD_PAD:nz - FD_PAD, FD_PAD:nx - FD_PAD] = True
    region = geo.pml + 3 * FD_PAD
    xs, zs = np.arange(nx), np.arange(nz)
    in_x = np.broadcast_to(((xs < region) | (xs >= nx - region))[None, :], (nz, nx))
    in_z = np.broadcast_to(((zs < region) | (zs >= nz - region))[:, None], (nz, nx))
    lam = [np.zeros((S, nz, nx), R), np.zeros((S, nz, nx), R)]
    lpsi = [np.zeros((2, S, nz, nx), R), np.zeros((2, S, nz, nx), R)]
    lzeta = [np.zeros((2, S, nz, nx), R), np.zeros((2, S, nz, nx), R)]
    grad = np.zeros((S, nz, nx), R)
    D1A, D1B = R(0.6666666666666666), R(-0.08333333333333333)
    D2A, D2B, D2C = R(-2.5), R(1.3333333333333333), R(-0.08333333333333333)
    profs = []
    for axis, (a, b, db) in ((2, geo.prof_x), (1, geo.prof_z)):
        shp = (1, 1, nx) if axis == 2 else (1, nz, 1)
        profs.append((axis, a.astype(R).reshape(shp), b.astype(R).reshape(shp), db.astype(R).reshape(shp)))
    wv = np.asarray(wavelet, np.float32).astype(R)
    res = residual.astype(R)
    st = stored.astype(R)
    for t in range(nt - 1, -1, -1):
        q = (nt - 1 - t) & 1
        cur, prev = lam[q], lam[1 - q]
        psi_rd, zeta_rd = lpsi[q], lzeta[q]
        psi_wr, zeta_wr = lpsi[1 - q], lzeta[1 - q]
        vs = vv * cur
        w = np.zeros_like(cur)
        for k, (axis, A, B, DB) in enumerate(profs):
            inr = (in_x if axis == 2 else in_z) & inner
            vsd = [_sh(vs, d, axis) for d in (-2, -1, 0, 1, 2)]
            Bd = [_sh(B, d, axis) for d in (-2, -1, 0, 1, 2)]
            DBd = [_sh(DB, d, axis) for d in (-2, -1, 0, 1, 2)]
            zd = [_sh(zeta_rd[k], d, axis) for d in (-2, -1, 0, 1, 2)]
            pd = [_sh(psi_rd[k], d, axis) for d in (-2, -1, 0, 1, 2)]
            tt = [(R(1) + Bd[d]) * vsd[d] + Bd[d] * zd[d] for d in range(5)]
            u1 = [DBd[d] * tt[d] + Bd[d] * pd[d] for d in range(5)]
            u2 = [(R(1) + Bd[d]) * tt[d] for d in range(5)]
            d1_u1 = (D1A * (u1[3] - u1[1]) + D1B * (u1[4] - u1[0])) * rh
            d2_u2 = (D2A * u2[2] + D2B * (u2[3] + u2[1]) + D2C * (u2[4] + u2[0])) * rh * rh
            d1_t = (D1A * (tt[3] - tt[1]) + D1B * (tt[4] - tt[0])) * rh
            w_pml = w + (-d1_u1 + d2_u2)
            w_int = w + (D2A * vsd[2] + D2B * (vsd[3] + vsd[1]) + D2C * (vsd[4] + vsd[0])) * rh * rh
            w = np.where(inr, w_pml, w_int)
            psi_wr[k] = np.where(inr, -A * d1_t + A * psi_rd[k], psi_wr[k])
            zeta_wr[k] = np.where(inr, A * vsd[2] + A * zeta_rd[k], zeta_wr[k])
        nxt = w + R(2) * cur - prev
        g = R(0) + cur * st[:, t] * R(1)
        for r, crn in enumerate(geo.rec):
            for (zc, xc), wgt in sorted(crn, key=lambda c: c[0]):
                if wgt != 0:
                    nxt[:, zc, xc] = nxt[:, zc, xc] + R(wgt) * res[:, t, r]
        for s in range(S):
            for (zc, xc), wgt in geo.src[s]:
                if inner[zc, xc]:
                    g[s, zc, xc] = g[s, zc, xc] + cur[s, zc, xc] * (R(-2) * v[zc, xc] * dt2 * R(wgt) * wv[t])
        grad = np.where(inner, grad + g, grad)
        lam[1 - q] = np.where(inner, nxt, prev)
    return grad


def evaluate_adjoint(geo: Geometry, v_vis, wavelet, observed, dtype=np.float32):
    """(loss f64, folded grad [nz_vis, nx_vis]) as wave_wgpu.rs:848-988."""
    R = dtype
    obs = np.asarray(observed, np.float32).reshape(geo.shots, len(wavelet), geo.nrec)
    energy = float(np.sum(obs.astype(np.float64) ** 2))
    scale = R(1.0 / energy)
    tr, st = forward(geo, v_vis, wavelet, dtype, store=True)
    d = tr - obs.astype(R)
    res = d * scale
    loss = float(np.sum((R(0.5) * d * d * scale).astype(np.float64)))
    raw = adjoint(geo, v_vis, wavelet, res, st, dtype)
    _, mask = geo.pad_velocity(v_vis)
    pg = np.zeros((geo.nz, geo.nx), R)
    for s in range(geo.shots):
        pg = pg + raw[s]
    pg = pg * mask.astype(R)
    out = np.zeros((geo.nz_vis, geo.nx_vis), np.float64)
    zi = np.clip(np.arange(geo.nz) - geo.pad, 0, geo.nz_vis - 1)
    xi = np.clip(np.arange(geo.nx) - geo.pad, 0, geo.nx_vis - 1)
    np.add.at(out, (zi[:, None], xi[None, :]), pg.astype(np.float64))
    return loss, out.astype(R), raw
