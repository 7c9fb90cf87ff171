"""numpy restatement of the band schedule (python/wgnet/physics.py:18-57). TEST INFRASTRUCTURE ONLY."""

from __future__ import annotations

import math

import numpy as np


def lowpass_kernel(fmax_hz: float, dt: float) -> np.ndarray:
    """Gaussian low-pass, -3 dB at fmax, truncated at 4 sigma, unit DC gain (physics.py:18-26)."""
    sigma_s = math.sqrt(math.log(2.0) / 2.0) / (math.pi * fmax_hz)
    half = int(math.ceil(4.0 * sigma_s / dt))
    n = np.arange(-half, half + 1)
    h = np.exp(-0.5 * (n * dt / sigma_s) ** 2)
    return (h / h.sum()).astype(np.float32)


def band_wavelet(full: np.ndarray, kernel: np.ndarray) -> np.ndarray:
    """set_band's wavelet (physics.py:43-46): full convolution truncated to nt."""
    return np.convolve(full, kernel, mode="full")[: len(full)].astype(np.float32)


def bandlimit(traces: np.ndarray, kernel: np.ndarray) -> np.ndarray:
    """Causal FIR along the time axis of [..., nt, nrec] (physics.py:48-57), in float64:
    y[t] = sum_k kernel[k] x[t - (K - 1) + k], zero before t = 0."""
    x = np.asarray(traces, np.float64)
    k = np.asarray(kernel, np.float64)
    nt = x.shape[-2]
    y = np.zeros_like(x)
    K = len(k)
    for j in range(K):
        lag = K - 1 - j
        if lag >= nt:
            continue
        y[..., lag:, :] += k[j] * x[..., : nt - lag, :]
    return y
