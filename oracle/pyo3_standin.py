"""The reference's PyO3 module `wave_gauss_rs` (crates/wave-gauss-rs/src/lib.rs:1-146) restated over
the C++ oracle. TEST INFRASTRUCTURE ONLY.

It lets the reference's own Python (python/wgnet/data.py, physics.py, refine.py) run unchanged on a
machine with no Rust toolchain and no graphics stack, so that fixtures generated from that Python
(`tests/golden/make_refpy.py`) pin this repository's Python layer against the reference's. Same
names, argument order, defaults, shapes and errors as lib.rs; the engine arithmetic is the oracle's
f32 restatement of the wgpu engine, which the CUDA engine matches bit for bit.
"""

from __future__ import annotations

import numpy as np

from . import native as o

N = 70


def _vel(a, name: str = "vel_mps") -> np.ndarray:
    if not isinstance(a, np.ndarray) or a.dtype != np.float32 or a.ndim != 1:
        raise TypeError(f"argument '{name}': expected a 1-D numpy.ndarray of float32")
    if a.size != N * N:
        raise ValueError(f"{name} must have {N * N} elements")
    return a.reshape(N, N)


def ricker_wavelet(samples: int, dt: float, peak_hz: float) -> np.ndarray:
    """lib.rs:10-15."""
    return o.ricker(int(samples), float(dt), float(peak_hz))


def simulate_shot_cpu(vel_mps, h, dt, nt, pml, vmin, vmax, peak_hz, src_x, src_z) -> np.ndarray:
    """lib.rs:17-42: f32[nt, 70]."""
    return o.simulate_shot_cpu(_vel(vel_mps), float(h), float(dt), int(nt), int(pml), float(vmin), float(vmax),
                               float(peak_hz), float(src_x), float(src_z))


class PyWaveEngine:
    """lib.rs:44-138 over the oracle's engine restatement."""

    def __init__(self, shots: int = 5, nt: int = 2001, dt: float = 0.0005, peak_hz: float = 15.0, pml: int = 20,
                 vmin: float = 1000.0, vmax: float = 5000.0) -> None:
        if shots < 1 or nt < 1:
            raise ValueError("invalid engine configuration")
        self._sv = o.Survey(shots=int(shots), nt=int(nt), dt=float(dt), peak_hz=float(peak_hz), pml=int(pml),
                            vmin=float(vmin), vmax=float(vmax))
        self._src = self._sv.default_sources()
        self._wav = o.ricker(self._sv.nt, self._sv.dt, self._sv.peak_hz)

    @property
    def shots(self) -> int:
        return self._sv.shots

    @property
    def nt(self) -> int:
        return self._sv.nt

    @property
    def nrec(self) -> int:
        return self._sv.n_receivers

    def sources(self) -> np.ndarray:
        return self._src.copy()

    def set_sources(self, xz) -> None:
        a = np.asarray(xz, dtype=np.float32)
        if a.shape != (self.shots, 2):
            raise ValueError("sources must have shape [shots, 2]")
        self._src = np.ascontiguousarray(a)

    def wavelet(self) -> np.ndarray:
        return self._wav.copy()

    def set_wavelet(self, w) -> None:
        a = np.asarray(w, dtype=np.float32).reshape(-1)
        if a.size != self.nt:
            raise ValueError("wavelet length must equal nt")
        self._wav = np.ascontiguousarray(a)

    def simulate(self, vel_mps) -> np.ndarray:
        return o.forward(self._sv, _vel(vel_mps), self._src, self._wav)[0]

    def evaluate_adjoint(self, vel_mps, observed) -> tuple[float, np.ndarray]:
        obs = np.asarray(observed, dtype=np.float32).reshape(-1)
        if obs.size != self.shots * self.nt * self.nrec:
            raise ValueError("observed length does not match shots * nt * nrec")
        loss, grad = o.evaluate_adjoint(self._sv, _vel(vel_mps), self._src, self._wav, obs)
        if not np.isfinite(loss[0]):
            raise RuntimeError("Observed traces have zero energy")
        return float(loss[0]), grad[0]
