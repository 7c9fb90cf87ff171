"""Drop-in replacement for the reference's PyO3 module `wave_gauss_rs`
(crates/wave-gauss-rs/src/lib.rs:1-146), backed by the CUDA engine.

Same names, signatures, argument checks and return shapes:

* `ricker_wavelet(samples, dt, peak_hz) -> f32[samples]`                      (lib.rs:10-15)
* `simulate_shot_cpu(vel_mps, h, dt, nt, pml, vmin, vmax, peak_hz, src_x, src_z) -> f32[nt, 70]`
  (lib.rs:17-42). The name is kept for compatibility; the shot runs on the GPU with the CPU
  solver's arithmetic (receivers at surface nodes, d2 scaled by rh*rh).
* `PyWaveEngine(shots=5, nt=2001, dt=0.0005, peak_hz=15.0, pml=20, vmin=1000.0, vmax=5000.0)`
  (lib.rs:44-138) with `shots`, `nt`, `nrec`, `sources()`, `set_sources()`, `wavelet()`,
  `set_wavelet()`, `simulate()`, `evaluate_adjoint()`.

Argument errors raise ValueError (the reference's PyValueError); a wrong array dtype raises
TypeError, as PyO3's numpy extraction does.
"""

from __future__ import annotations

import numpy as np

from . import _lib
from ._lib import check, ptr
from .engine import WaveEngine
from .engine import ricker_wavelet as _ricker

N = 70
CELLS = N * N


def _f32_1d(a, name: str) -> np.ndarray:
    if not isinstance(a, np.ndarray) or a.dtype != np.float32 or a.ndim != 1:
        raise TypeError(f"argument '{name}': expected a 1-D numpy.ndarray of float32")
    if not a.flags.c_contiguous:
        raise ValueError(f"{name} must be contiguous")
    return a


def ricker_wavelet(samples: int, dt: float, peak_hz: float) -> np.ndarray:
    return _ricker(samples, dt, peak_hz)


def simulate_shot_cpu(vel_mps: np.ndarray, h: float, dt: float, nt: int, pml: int, vmin: float, vmax: float,
                      peak_hz: float, src_x: float, src_z: float) -> np.ndarray:
    v = _f32_1d(vel_mps, "vel_mps")
    if v.size != CELLS:
        raise ValueError("vel_mps must have 4900 elements")
    out = np.zeros((int(nt), N), np.float32)
    check(_lib.load().wg_simulate_shot(ptr(v), N, N, float(h), float(dt), int(nt), int(pml), float(vmin),
                                       float(vmax), float(peak_hz), float(src_x), float(src_z), ptr(out)),
          "simulate_shot_cpu")
    return out


class PyWaveEngine:
    """Multi-shot forward / exact discrete adjoint engine for a 70 x 70 model (lib.rs:44-138)."""

    def __init__(self, shots: int = 5, nt: int = 2001, dt: float = 0.0005, peak_hz: float = 15.0, pml: int = 20,
                 vmin: float = 1000.0, vmax: float = 5000.0) -> None:
        try:
            self._eng = WaveEngine(shots, nt, dt, peak_hz, pml, vmin, vmax)
        except RuntimeError as exc:  # engine creation failure -> ValueError (lib.rs:55)
            raise ValueError(str(exc)) from exc

    @property
    def shots(self) -> int:
        return self._eng.shots

    @property
    def nt(self) -> int:
        return self._eng.nt

    @property
    def nrec(self) -> int:
        return self._eng.nrec

    @property
    def engine(self) -> WaveEngine:
        """The batched engine underneath (extra: not in the reference)."""
        return self._eng

    def sources(self) -> np.ndarray:
        return self._eng.sources()

    def set_sources(self, sources: np.ndarray) -> None:
        if not isinstance(sources, np.ndarray) or sources.dtype != np.float32 or sources.ndim != 2:
            raise TypeError("argument 'sources': expected a 2-D numpy.ndarray of float32")
        if sources.shape[0] != self.shots or sources.shape[1] != 2:
            raise ValueError("sources must have shape [shots, 2]")
        if not sources.flags.c_contiguous:
            raise ValueError("sources must be contiguous")
        self._eng.set_sources(sources)

    def wavelet(self) -> np.ndarray:
        return self._eng.wavelet()

    def set_wavelet(self, wavelet: np.ndarray) -> None:
        w = _f32_1d(wavelet, "wavelet")
        if w.size != self.nt:
            raise ValueError("wavelet length must equal nt")
        self._eng.set_wavelet(w)

    def simulate(self, vel_mps: np.ndarray) -> np.ndarray:
        v = _f32_1d(vel_mps, "vel_mps")
        if v.size != CELLS:
            raise ValueError("vel_mps must have 4900 elements")
        return self._eng.simulate(v)[0]

    def evaluate_adjoint(self, vel_mps: np.ndarray, observed: np.ndarray) -> tuple[float, np.ndarray]:
        v = _f32_1d(vel_mps, "vel_mps")
        o = _f32_1d(observed, "observed")
        if v.size != CELLS:
            raise ValueError("vel_mps must have 4900 elements")
        if o.size != self.shots * self.nt * self.nrec:
            raise ValueError("observed length does not match shots * nt * nrec")
        loss, grad = self._eng.evaluate_adjoint(v, o)
        return float(np.float32(loss[0])), grad[0]
