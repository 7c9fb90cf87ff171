"""Survey constants and engine factory of the reference's data module (python/wgnet/data.py:20-33,
190-193). The OpenFWI loader and on-disk wave cache of that module are not part of this package;
the synthetic model families used for benchmarks and tests live in `wgnet_gb300.models_synth`."""

from __future__ import annotations

import numpy as np

from .wave_gauss_rs import PyWaveEngine

N = 70
H = 10.0
SHOTS = 5
NT = 2001
DT = 0.0005
PEAK_HZ = 15.0
DECIMATE = 8
NT_DEC = (NT - 1) // DECIMATE + 1  # 251


def make_engine(shots: int = SHOTS, nt: int = NT) -> PyWaveEngine:
    """data.py:32-33: PyWaveEngine(shots, nt, DT, PEAK_HZ, pml=20, vmin=1000, vmax=5000)."""
    return PyWaveEngine(shots, nt, DT, PEAK_HZ, 20, 1000.0, 5000.0)


def source_positions_m(shots: int = SHOTS) -> np.ndarray:
    """`[shots]` source x positions in metres matching the engine's default layout (data.py:190-193)."""
    xmax = (N - 1) * H
    return np.array([xmax / 2.0], np.float32) if shots == 1 else np.linspace(0.0, xmax, shots, dtype=np.float32)
