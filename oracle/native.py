"""ctypes loader for the C++ oracle (`wave_oracle.cpp`). TEST INFRASTRUCTURE ONLY.

Builds `oracle/_build/libwave_oracle.so` with `make` on first use if it is missing.
"""

from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "libwave_oracle.so"


class WgoConfig(ctypes.Structure):
    _fields_ = [
        ("nx_vis", ctypes.c_int), ("nz_vis", ctypes.c_int), ("pml", ctypes.c_int),
        ("shots", ctypes.c_int), ("nt", ctypes.c_int), ("nrec", ctypes.c_int),
        ("h", ctypes.c_float), ("dt", ctypes.c_float), ("peak_hz", ctypes.c_float),
        ("vmin", ctypes.c_float), ("vmax", ctypes.c_float),
    ]


def build() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB_PATH


_LIB = None


def lib() -> ctypes.CDLL:
    global _LIB
    if _LIB is None:
        src = HERE / "wave_oracle.cpp"
        if not LIB_PATH.exists() or LIB_PATH.stat().st_mtime < src.stat().st_mtime:
            build()
        _LIB = ctypes.CDLL(str(LIB_PATH))
    return _LIB


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)


def _p(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def cpu_threads() -> int:
    return max(1, len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1))


@dataclass
class Survey:
    """Geometry and time axis of one engine (the reference's PyWaveEngine arguments)."""

    shots: int = 5
    nt: int = 2001
    dt: float = 0.0005
    peak_hz: float = 15.0
    pml: int = 20
    vmin: float = 1000.0
    vmax: float = 5000.0
    nx_vis: int = 70
    nz_vis: int = 70
    h: float = 10.0
    nrec: int | None = None

    def config(self) -> WgoConfig:
        return WgoConfig(self.nx_vis, self.nz_vis, self.pml, self.shots, self.nt,
                         self.nrec if self.nrec is not None else self.nx_vis,
                         self.h, self.dt, self.peak_hz, self.vmin, self.vmax)

    @property
    def n_receivers(self) -> int:
        return self.nrec if self.nrec is not None else self.nx_vis

    @property
    def pad(self) -> int:
        return 2 + self.pml

    @property
    def nx(self) -> int:
        return self.nx_vis + 2 * self.pad

    @property
    def nz(self) -> int:
        return self.nz_vis + 2 * self.pad

    def default_sources(self) -> np.ndarray:
        """wave_wgpu.rs:204-214: x = linspace(0, (nx_vis-1) h, shots) (centre for one shot), z = h."""
        xmax = np.float32((self.nx_vis - 1) * self.h)
        out = np.zeros((self.shots, 2), np.float32)
        for k in range(self.shots):
            out[k, 0] = xmax * np.float32(0.5) if self.shots == 1 else (xmax * np.float32(k)) / np.float32(self.shots - 1)
            out[k, 1] = np.float32(self.h)
        return out


def ricker(samples: int, dt: float, peak_hz: float) -> np.ndarray:
    out = np.zeros(samples, np.float32)
    assert lib().wgo_ricker(ctypes.c_int(samples), ctypes.c_float(dt), ctypes.c_float(peak_hz), _p(out)) == 0
    return out


def cpml_profiles(n: int, h: float, dt: float, width: int, max_vel: float, freq: float):
    a, b, db = (np.zeros(n, np.float32) for _ in range(3))
    rc = lib().wgo_cpml_profiles(ctypes.c_int(n), ctypes.c_float(h), ctypes.c_float(dt), ctypes.c_int(width),
                                 ctypes.c_float(max_vel), ctypes.c_float(freq), _p(a), _p(b), _p(db))
    assert rc == 0
    return a, b, db


def simulate_shot_cpu(vel_vis: np.ndarray, h: float, dt: float, nt: int, pml: int, vmin: float, vmax: float,
                      peak_hz: float, src_x: float, src_z: float, nx_vis: int = 70, nz_vis: int = 70) -> np.ndarray:
    v = _f32(vel_vis).reshape(-1)
    out = np.zeros((nt, nx_vis), np.float32)
    rc = lib().wgo_simulate_shot_cpu(_p(v), ctypes.c_int(nx_vis), ctypes.c_int(nz_vis), ctypes.c_float(h),
                                     ctypes.c_float(dt), ctypes.c_int(nt), ctypes.c_int(pml), ctypes.c_float(vmin),
                                     ctypes.c_float(vmax), ctypes.c_float(peak_hz), ctypes.c_float(src_x),
                                     ctypes.c_float(src_z), _p(out))
    assert rc == 0
    return out


def geometry(sv: Survey, sources: np.ndarray):
    cfg = sv.config()
    cells = sv.nx * sv.nz
    src_cell = np.zeros(4 * sv.shots, np.int32)
    src_w = np.zeros(4 * sv.shots, np.float32)
    rec_cell = np.zeros(4 * sv.n_receivers, np.int32)
    rec_w = np.zeros(4 * sv.n_receivers, np.float32)
    csr = np.zeros(cells + 1, np.int32)
    n_ent = ctypes.c_int(0)
    s = _f32(sources)
    rc = lib().wgo_geometry(ctypes.byref(cfg), _p(s), None, _p(src_cell), _p(src_w), _p(rec_cell), _p(rec_w),
                            _p(csr), ctypes.byref(n_ent))
    assert rc == 0
    return dict(src_cell=src_cell, src_w=src_w, rec_cell=rec_cell, rec_w=rec_w, csr=csr, n_entries=n_ent.value)


def pad_velocity(sv: Survey, vel_vis: np.ndarray):
    cfg = sv.config()
    padded = np.zeros(sv.nx * sv.nz, np.float32)
    mask = np.zeros(sv.nx * sv.nz, np.float32)
    assert lib().wgo_pad_velocity(ctypes.byref(cfg), _p(_f32(vel_vis).reshape(-1)), _p(padded), _p(mask)) == 0
    return padded.reshape(sv.nz, sv.nx), mask.reshape(sv.nz, sv.nx)


def forward(sv: Survey, vel_vis: np.ndarray, sources: np.ndarray, wavelet: np.ndarray, precision: str = "f32",
            store: bool = False, threads: int | None = None):
    """Engine forward for `[B, nz_vis, nx_vis]` (or one `[nz_vis, nx_vis]`) models in m/s.

    Returns traces `[B, shots, nt, nrec]` (f32 or f64) and, when `store`, the per-step gradient
    terms `2 v dt^2 w` as `[B, shots, nt, nz, nx]` (f32 only)."""
    v = _f32(vel_vis).reshape(-1, sv.nz_vis * sv.nx_vis)
    nb = v.shape[0]
    cfg = sv.config()
    threads = threads or cpu_threads()
    w = _f32(wavelet)
    s = _f32(sources)
    shape = (nb, sv.shots, sv.nt, sv.n_receivers)
    if precision == "f64":
        tr = np.zeros(shape, np.float64)
        rc = lib().wgo_forward_f64(ctypes.byref(cfg), ctypes.c_int(nb), _p(v), _p(s), None, _p(w), _p(tr),
                                   ctypes.c_int(threads))
        assert rc == 0
        return tr
    tr = np.zeros(shape, np.float32)
    st = np.zeros((nb, sv.shots, sv.nt, sv.nz, sv.nx), np.float32) if store else None
    rc = lib().wgo_forward_f32(ctypes.byref(cfg), ctypes.c_int(nb), _p(v), _p(s), None, _p(w), _p(tr), _p(st),
                               ctypes.c_int(threads))
    assert rc == 0
    return (tr, st) if store else tr


def evaluate_adjoint(sv: Survey, vel_vis: np.ndarray, sources: np.ndarray, wavelet: np.ndarray,
                     observed: np.ndarray, precision: str = "f32", raw: bool = False, threads: int | None = None):
    """Engine evaluate_adjoint: `(loss [B] f64, grad [B, nz_vis, nx_vis])` in dJ/d(v in m/s).

    With `raw`, also the per-shot padded gradient `[B, shots, nz, nx]` before shot-sum/mask/fold."""
    v = _f32(vel_vis).reshape(-1, sv.nz_vis * sv.nx_vis)
    nb = v.shape[0]
    obs = _f32(observed).reshape(nb, -1)
    assert obs.shape[1] == sv.shots * sv.nt * sv.n_receivers
    cfg = sv.config()
    threads = threads or cpu_threads()
    loss = np.zeros(nb, np.float64)
    if precision == "f64":
        grad = np.zeros((nb, sv.nz_vis, sv.nx_vis), np.float64)
        rc = lib().wgo_evaluate_adjoint_f64(ctypes.byref(cfg), ctypes.c_int(nb), _p(v), _p(_f32(sources)), None,
                                            _p(_f32(wavelet)), _p(obs), _p(loss), _p(grad), ctypes.c_int(threads))
    else:
        grad = np.zeros((nb, sv.nz_vis, sv.nx_vis), np.float32)
        rg = np.zeros((nb, sv.shots, sv.nz, sv.nx), np.float32) if raw else None
        rc = lib().wgo_evaluate_adjoint_f32(ctypes.byref(cfg), ctypes.c_int(nb), _p(v), _p(_f32(sources)), None,
                                            _p(_f32(wavelet)), _p(obs), _p(loss), _p(grad), _p(rg),
                                            ctypes.c_int(threads))
        if raw:
            if rc != 0:
                raise ValueError(f"oracle evaluate_adjoint failed with status {rc}")
            return loss, grad, rg
    if rc != 0:
        raise ValueError(f"oracle evaluate_adjoint failed with status {rc}")
    return loss, grad


def gradients_parallel(sv: Survey, vel_vis: np.ndarray, sources: np.ndarray, wavelet: np.ndarray,
                       observed: np.ndarray, threads: int | None = None):
    """CPU-baseline driver: one model per worker thread (all of its shots on that thread)."""
    v = _f32(vel_vis).reshape(-1, sv.nz_vis * sv.nx_vis)
    nb = v.shape[0]
    obs = _f32(observed).reshape(nb, -1)
    cfg = sv.config()
    loss = np.zeros(nb, np.float64)
    grad = np.zeros((nb, sv.nz_vis, sv.nx_vis), np.float32)
    rc = lib().wgo_gradients_parallel_f32(ctypes.byref(cfg), ctypes.c_int(nb), _p(v), _p(_f32(sources)), None,
                                          _p(_f32(wavelet)), _p(obs), _p(loss), _p(grad),
                                          ctypes.c_int(threads or cpu_threads()))
    if rc != 0:
        raise ValueError(f"oracle gradients failed with status {rc}")
    return loss, grad
