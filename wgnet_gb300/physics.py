"""Exact wave-equation data misfit with frequency continuation (python/wgnet/physics.py:1-76),
on the CUDA engine.

`WavePhysics` keeps the reference's interface (`set_band`, `bandlimit`, `simulate`,
`loss_and_grad`) but runs each call as one batched launch sequence instead of a Python loop over
models. `WaveLoss` is the same misfit as a `torch.autograd.Function` on CUDA tensors: its forward
runs the forward solve, residual and adjoint (checkpointed), its backward returns the stored
gradient scaled by the incoming cotangent.
"""

from __future__ import annotations

import math

import numpy as np
import torch

from . import _lib
from ._lib import check, ptr
from .data import DT, N, NT, SHOTS, make_engine
from .engine import WaveEngine


def lowpass_kernel(fmax_hz: float, dt: float = DT) -> np.ndarray:
    """Causal Gaussian low-pass with its -3 dB point at `fmax_hz`, truncated at 4 sigma, unit DC gain
    (physics.py:18-26). Applied with a delay of len-1 samples so that filtering the wavelet and
    filtering the data commute exactly with the (linear, time-invariant) wave simulation."""
    sigma_s = math.sqrt(math.log(2.0) / 2.0) / (math.pi * fmax_hz)
    half = int(math.ceil(4.0 * sigma_s / dt))
    n = np.arange(-half, half + 1)
    h = np.exp(-0.5 * (n * dt / sigma_s) ** 2)
    return (h / h.sum()).astype(np.float32)


def bandlimit_torch(traces: torch.Tensor, kernel: torch.Tensor) -> torch.Tensor:
    """Causal FIR of `kernel` along the time axis of CUDA traces `[..., nt, nrec]` (CUDA kernel)."""
    if not traces.is_cuda:
        raise TypeError("traces must be a CUDA tensor")
    x = traces.contiguous().float()
    nt, nrec = x.shape[-2], x.shape[-1]
    series = x.numel() // max(nt * nrec, 1)
    k = kernel.to(device=x.device, dtype=torch.float32).contiguous()
    out = torch.empty_like(x)
    with torch.cuda.device(x.device):
        stream = torch.cuda.current_stream().cuda_stream
        check(_lib.load().wg_bandlimit_dev(ptr(x), ptr(k), int(k.numel()), int(series), int(nt), int(nrec), ptr(out),
                                           stream), "bandlimit")
    return out


class WavePhysics:
    """Normalized data misfit `0.5 ||p - d||^2 / ||d||^2` and its exact gradient, with passbands."""

    def __init__(self, shots: int = SHOTS, nt: int = NT, engine=None) -> None:
        self.engine = engine if engine is not None else make_engine(shots, nt)
        self.shots, self.nt = shots, nt
        self.full_wavelet = self.engine.wavelet().copy()
        self.kernel: np.ndarray | None = None
        self.fmax: float | None = None
        # The reference designs the passband at its module DT because its engine is fixed to that
        # step (physics.py:43, data.py:25); here the engine's own step sets the filter, so a 1 ms
        # engine gets a kernel sampled at 1 ms and the -3 dB point stays at the stated frequency.
        self.dt = float(getattr(self.wave, "dt", DT))

    @property
    def wave(self) -> WaveEngine:
        """The batched CUDA engine behind `self.engine`."""
        return self.engine.engine if hasattr(self.engine, "engine") else self.engine

    def set_band(self, fmax_hz: float | None) -> None:
        """physics.py:37-46. `None` restores the full-band Ricker; otherwise the wavelet is convolved
        with the causal low-pass and truncated to nt."""
        if fmax_hz is None:
            self.kernel, self.fmax = None, None
            self.engine.set_wavelet(self.full_wavelet)
            return
        self.kernel = lowpass_kernel(fmax_hz, self.dt)
        self.fmax = float(fmax_hz)
        w = np.convolve(self.full_wavelet, self.kernel, mode="full")[: self.nt].astype(np.float32)
        self.engine.set_wavelet(np.ascontiguousarray(w))

    def bandlimit(self, traces):
        """physics.py:48-57: the current passband kernel applied causally along time to
        `[..., nt, nrec]` traces (numpy in -> numpy out, CUDA tensor in -> CUDA tensor out)."""
        if self.kernel is None:
            return traces
        if isinstance(traces, torch.Tensor):
            return bandlimit_torch(traces, torch.from_numpy(self.kernel))
        x = torch.from_numpy(np.ascontiguousarray(traces, dtype=np.float32)).cuda()
        return bandlimit_torch(x, torch.from_numpy(self.kernel)).cpu().numpy()

    def simulate(self, fields_km) -> np.ndarray:
        """`[B, 70, 70]` km/s -> `[B, shots, nt, 70]` synthetics with the current passband."""
        if isinstance(fields_km, torch.Tensor) and fields_km.is_cuda:
            return self.wave.simulate_torch((fields_km.float() * 1000.0).contiguous())
        v = np.asarray(fields_km, dtype=np.float32).reshape(-1, N * N) * np.float32(1000.0)
        return self.wave.simulate(v)

    def loss_and_grad(self, fields_km, observed):
        """Per-model normalized misfit and its gradient w.r.t. velocity in km/s (physics.py:66-76).
        numpy inputs give `(f32[B], f32[B, 70, 70])`; CUDA tensors give tensors on the device."""
        if isinstance(fields_km, torch.Tensor) and fields_km.is_cuda:
            loss, grad = self.wave.evaluate_adjoint_torch((fields_km.float() * 1000.0).contiguous(),
                                                          observed.float().contiguous())
            return loss.float(), grad * 1000.0
        v = np.asarray(fields_km, dtype=np.float32).reshape(-1, N * N) * np.float32(1000.0)
        loss, grad = self.wave.evaluate_adjoint(v, np.asarray(observed, dtype=np.float32))
        return loss.astype(np.float32), grad * np.float32(1000.0)


class WaveLoss(torch.autograd.Function):
    """`loss[b] = 0.5 ||p_b - d_b||^2 / ||d_b||^2` of CUDA velocity fields in km/s `[B, nz, nx]`
    against observed `[B, shots, nt, nrec]`, with the exact discrete adjoint as its gradient.

    Usage: `WaveLoss.apply(fields_km, observed, engine)` with a `WaveEngine` (its current wavelet
    sets the passband). The forward pass computes the gradient eagerly (forward, residual,
    checkpointed adjoint); backward scales it by the incoming cotangent."""

    @staticmethod
    def forward(ctx, fields_km: torch.Tensor, observed: torch.Tensor, engine: WaveEngine) -> torch.Tensor:
        loss, grad_mps = engine.evaluate_adjoint_torch((fields_km.detach().float() * 1000.0).contiguous(),
                                                       observed.detach().float().contiguous())
        ctx.save_for_backward(grad_mps)
        return loss.to(fields_km.dtype)

    @staticmethod
    def backward(ctx, gout: torch.Tensor):
        (grad_mps,) = ctx.saved_tensors
        g = grad_mps * 1000.0 * gout.to(grad_mps.dtype).view(-1, 1, 1)
        return g, None, None
