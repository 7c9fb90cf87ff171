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


def lowpass_decimate_f16(traces: np.ndarray, taps: np.ndarray, center: int, factor: int) -> np.ndarray:
    """Wave-cache writer step (python/wgnet/data.py:163-166 subsamples `[:, ::factor, :]` and casts
    to float16): here a zero-phase FIR first, y[j] = sum_k taps[k] x[j factor + k - center] (zero
    outside [0, nt)), accumulated in f32 over k in increasing order, then rounded to float16
    (round to nearest even). `traces` is [..., nt, nrec]; returns [..., ceil(nt / factor), nrec]."""
    x = np.asarray(traces, np.float32)
    nt = x.shape[-2]
    nt_out = -(-nt // factor)
    acc = np.zeros(x.shape[:-2] + (nt_out, x.shape[-1]), np.float32)
    j = np.arange(nt_out)
    for k, w in enumerate(np.asarray(taps, np.float32)):
        t = j * factor + k - center
        ok = (t >= 0) & (t < nt)
        acc[..., ok, :] = acc[..., ok, :] + w * x[..., t[ok], :]
    return acc.astype(np.float16)
