"""Batched forward data generation over several grid sizes: the wave-cache writer
(python/wgnet/data.py:138-179) for thousands of models in one CUDA graph launch.

`GatherGenerator({70: n70, 100: n100, 140: n140})` owns one engine per grid size (square grids of
n x n visible cells, n receivers at every surface cell, the survey's default sources), picks each
engine's forward launch shape with the autotuner, and captures the whole batch into one CUDA graph
(`wg_gen_plan_*`): per grid, velocity padding, the resident forward kernel over every (model,
shot) unit and the zero-phase low-pass + decimation to IEEE half. `run()` replays it; outputs are
`{n: [models, shots, ceil(nt / factor), n]}` float16 CUDA tensors.

The reference subsamples `[:, ::8, :]` without a low-pass and stores float16 (data.py:163-166);
here the decimation is preceded by the reference's own Gaussian low-pass (physics.py:18-26,
computed with numpy as there), centred, with its -3 dB point at 0.4 of the decimated Nyquist
frequency unless `cutoff_hz` says otherwise.
"""

from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import check
from .engine import WaveEngine
from .physics import lowpass_kernel


def lowpass_taps(fmax_hz: float, dt: float) -> np.ndarray:
    """physics.py's lowpass_kernel computed by the library (host code)."""
    lib = _lib.load()
    n = lib.wg_lowpass_taps(float(fmax_hz), float(dt), None, 0)
    if n < 0:
        check(-n, "lowpass_taps")
    out = np.zeros(n, np.float32)
    lib.wg_lowpass_taps(float(fmax_hz), float(dt), out.ctypes.data_as(ctypes.c_void_p), n)
    return out


class GatherGenerator:
    """One CUDA graph that simulates, low-passes and decimates batches of models on several grids."""

    def __init__(self, counts: dict[int, int], shots: int = 5, nt: int = 1000, dt: float = 0.001, h: float = 10.0,
                 peak_hz: float = 15.0, pml: int = 20, vmin: float = 1000.0, vmax: float = 5000.0, factor: int = 4,
                 cutoff_hz: float = 0.0, autotune: bool = True, workspace_bytes: int = 0) -> None:
        import torch

        if not torch.cuda.is_available():
            raise RuntimeError("GatherGenerator needs a CUDA device (there is no CPU path)")
        self._lib = _lib.load()
        self.sizes = sorted(int(n) for n in counts)
        self.counts = {int(n): int(counts[n]) for n in counts}
        self.shots, self.nt, self.factor = int(shots), int(nt), int(factor)
        self.nt_out = (self.nt + self.factor - 1) // self.factor
        self.engines: dict[int, WaveEngine] = {}
        self.shapes: dict[int, tuple[int, int, int]] = {}
        for n in self.sizes:
            eng = WaveEngine(shots, nt, dt, peak_hz, pml, vmin, vmax, nx_vis=n, nz_vis=n, h=h)
            if autotune:
                from .autotune import tune

                tune(eng, which=("forward",))
            self.shapes[n] = eng.launch_shape("forward")
            self.engines[n] = eng
        dev = torch.device("cuda", torch.cuda.current_device())
        self.velocity = {n: torch.full((self.counts[n], n, n), 2000.0, device=dev, dtype=torch.float32)
                         for n in self.sizes}
        self.gathers = {n: torch.empty((self.counts[n], self.shots, self.nt_out, n), device=dev, dtype=torch.float16)
                        for n in self.sizes}
        g = len(self.sizes)
        engines = (ctypes.c_void_p * g)(*[self.engines[n]._h.value for n in self.sizes])
        models = (ctypes.c_int * g)(*[self.counts[n] for n in self.sizes])
        vel = (ctypes.c_void_p * g)(*[self.velocity[n].data_ptr() for n in self.sizes])
        out = (ctypes.c_void_p * g)(*[self.gathers[n].data_ptr() for n in self.sizes])
        # the anti-alias taps come from the reference's own lowpass_kernel (numpy, f64 -> f32)
        if cutoff_hz == 0.0 and self.factor > 1:
            cutoff_hz = round(0.4 * 0.5 / (self.factor * float(dt)), 6)
        taps = lowpass_kernel(cutoff_hz, float(dt)) if cutoff_hz > 0 else np.ones(1, np.float32)
        taps = np.ascontiguousarray(taps, dtype=np.float32)
        plan = ctypes.c_void_p()
        torch.cuda.synchronize()
        check(self._lib.wg_gen_plan_create(engines, models, g, vel, out, self.factor,
                                           taps.ctypes.data_as(ctypes.c_void_p), len(taps), float(cutoff_hz),
                                           int(workspace_bytes), ctypes.byref(plan)), "gen_plan_create")
        self._plan = plan
        k, tb, kl = ctypes.c_int(), ctypes.c_size_t(), ctypes.c_int()
        check(self._lib.wg_gen_plan_info(self._plan, ctypes.byref(k), ctypes.byref(tb), None, 0, ctypes.byref(kl)))
        taps = np.zeros(kl.value, np.float32)
        check(self._lib.wg_gen_plan_info(self._plan, None, None, taps.ctypes.data_as(ctypes.c_void_p), kl.value,
                                          None))
        self.kernels_per_launch, self.trace_bytes, self.taps = k.value, tb.value, taps

    @property
    def models(self) -> int:
        return sum(self.counts.values())

    def load(self, velocity: dict) -> None:
        """Copy `{n: [models, n, n]}` velocities (m/s; numpy or torch) into the plan's input buffers
        on the current stream."""
        import torch

        for n, v in velocity.items():
            t = torch.as_tensor(v, dtype=torch.float32)
            dst = self.velocity[int(n)]
            if tuple(t.shape) != tuple(dst.shape):
                raise ValueError(f"velocity for grid {n} must have shape {tuple(dst.shape)}")
            dst.copy_(t, non_blocking=True)

    def launch(self) -> None:
        """Replay the graph on the current torch stream (asynchronous)."""
        import torch

        check(self._lib.wg_gen_plan_launch(self._plan, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)),
              "gen_plan_launch")

    def run(self, velocity: dict | None = None) -> dict:
        """Load velocities (if given), replay the graph and return the float16 gathers
        `{n: [models, shots, nt_out, n]}` (device tensors owned by the generator, overwritten by the
        next run)."""
        if velocity is not None:
            self.load(velocity)
        self.launch()
        return self.gathers

    def close(self) -> None:
        if getattr(self, "_plan", None):
            self._lib.wg_gen_plan_destroy(self._plan)
            self._plan = None
        for eng in getattr(self, "engines", {}).values():
            eng.close()

    def __del__(self) -> None:
        try:
            self.close()
        except Exception:
            pass


def round_robin_counts(total: int, sizes=(70, 100, 140)) -> dict[int, int]:
    """Split `total` models over grid sizes round-robin by seed (model i gets sizes[i % len])."""
    return {n: (total - i + len(sizes) - 1) // len(sizes) for i, n in enumerate(sizes)}


def synthetic_batch(total: int, seed: int = 0, sizes=(70, 100, 140)) -> dict[int, np.ndarray]:
    """Seeded mixed-family models for `round_robin_counts(total, sizes)`: model i (global index) has
    grid sizes[i % len(sizes)] and family i % 4 of the flat / curved / fault / blob generators."""
    from .models_synth import FAMILIES, make_model

    out = {n: [] for n in sizes}
    for i in range(total):
        n = sizes[i % len(sizes)]
        out[n].append(make_model(seed * 1_000_003 + i, n, n, FAMILIES[(i // len(sizes)) % len(FAMILIES)]))
    return {n: np.stack(v).astype(np.float32) if v else np.zeros((0, n, n), np.float32) for n, v in out.items()}


__all__ = ["GatherGenerator", "lowpass_taps", "round_robin_counts", "synthetic_batch"]
