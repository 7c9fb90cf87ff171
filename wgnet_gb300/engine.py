"""`WaveEngine`: Python handle on the CUDA wave engine (C ABI `wg_engine_*`).

Batched counterpart of the reference's `NativeWaveEngine` (crates/wave-gauss-rs/src/wave_wgpu.rs):
host entry points take numpy arrays, `*_torch` entry points take CUDA tensors and run on the
current torch stream. Velocities are `[B, nz_vis, nx_vis]` in m/s; traces `[B, shots, nt, nrec]`.
"""

from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import WgConfig, check, ptr


def _torch_stream():
    import torch

    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


class WaveEngine:
    """One survey (grid, C-PML, wavelet, stations) on the current CUDA device."""

    def __init__(self, shots: int = 5, nt: int = 2001, dt: float = 0.0005, peak_hz: float = 15.0, pml: int = 20,
                 vmin: float = 1000.0, vmax: float = 5000.0, nx_vis: int = 70, nz_vis: int = 70, h: float = 10.0,
                 nrec: int | None = None, checkpoint_every: int | None = None) -> None:
        self._lib = _lib.load()
        cfg = WgConfig(int(shots), int(nt), float(dt), float(peak_hz), int(pml), float(vmin), float(vmax),
                       int(nx_vis), int(nz_vis), float(h), int(nrec or 0))
        handle = ctypes.c_void_p()
        check(self._lib.wg_engine_create(ctypes.byref(cfg), ctypes.byref(handle)), "engine")
        self._h = handle
        dims = [ctypes.c_int() for _ in range(7)]
        check(self._lib.wg_engine_dims(self._h, *[ctypes.byref(d) for d in dims]))
        self.shots, self.nt, self.nrec, self.nx, self.nz, self.nx_vis, self.nz_vis = (d.value for d in dims)
        self.dt, self.peak_hz, self.pml, self.vmin, self.vmax, self.h = float(dt), float(peak_hz), int(pml), \
            float(vmin), float(vmax), float(h)
        if checkpoint_every is not None:
            self.checkpoint_every = checkpoint_every

    # -- lifetime ----------------------------------------------------------------------------
    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.wg_engine_destroy(self._h)
            self._h = None

    def __del__(self) -> None:
        try:
            self.close()
        except Exception:
            pass

    # -- survey ------------------------------------------------------------------------------
    @property
    def cells_vis(self) -> int:
        return self.nx_vis * self.nz_vis

    def sources(self) -> np.ndarray:
        out = np.zeros((self.shots, 2), np.float32)
        check(self._lib.wg_get_sources(self._h, ptr(out), self.shots))
        return out

    def set_sources(self, xz: np.ndarray) -> None:
        a = np.ascontiguousarray(xz, dtype=np.float32)
        if a.shape != (self.shots, 2):
            raise ValueError("sources must have shape [shots, 2]")
        check(self._lib.wg_set_sources(self._h, ptr(a), self.shots))

    def wavelet(self) -> np.ndarray:
        out = np.zeros(self.nt, np.float32)
        check(self._lib.wg_get_wavelet(self._h, ptr(out), self.nt))
        return out

    def set_wavelet(self, w: np.ndarray) -> None:
        a = np.ascontiguousarray(w, dtype=np.float32).reshape(-1)
        if a.size != self.nt:
            raise ValueError("wavelet length must equal nt")
        check(self._lib.wg_set_wavelet(self._h, ptr(a), self.nt))

    @property
    def checkpoint_every(self) -> int:
        return int(self._lib.wg_get_checkpoint_interval(self._h))

    @checkpoint_every.setter
    def checkpoint_every(self, k: int) -> None:
        check(self._lib.wg_set_checkpoint_interval(self._h, int(k)))

    def set_option(self, key: str, value: int) -> None:
        check(self._lib.wg_set_option(self._h, key.encode(), int(value)))

    def get_option(self, key: str) -> int:
        v = ctypes.c_int()
        check(self._lib.wg_get_option(self._h, key.encode(), ctypes.byref(v)))
        return v.value

    def launch_shape(self, which: str = "forward") -> tuple[int, int, int]:
        w = 0 if which.startswith("f") else 1
        c, t, k = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        check(self._lib.wg_get_launch_shape(self._h, w, ctypes.byref(c), ctypes.byref(t), ctypes.byref(k)))
        return c.value, t.value, k.value

    def set_launch_shape(self, which: str, shape: tuple[int, int, int]) -> None:
        w = 0 if which.startswith("f") else 1
        check(self._lib.wg_set_launch_shape(self._h, w, int(shape[0]), int(shape[1]), int(shape[2])))

    def shape_candidates(self, which: str = "forward") -> list[tuple[int, int, int]]:
        w = 0 if which.startswith("f") else 1
        buf = np.zeros(3 * 64, np.int32)
        n = self._lib.wg_shape_candidates(self._h, w, ptr(buf), 64)
        if n < 0:
            check(-n)
        return [tuple(int(v) for v in buf[3 * i:3 * i + 3]) for i in range(min(n, 64))]

    def profile(self, enable: bool = True) -> None:
        """Start (clearing earlier records) or stop per-kernel event timing."""
        check(self._lib.wg_profile(self._h, int(bool(enable))))

    def profile_read(self) -> dict[str, tuple[float, int]]:
        """{kind: (milliseconds, launches)} since profile(True), for the forward, forward-recompute,
        adjoint and auxiliary kernels; clears the records."""
        ms = np.zeros(4, np.float64)
        n = np.zeros(4, np.int64)
        check(self._lib.wg_profile_read(self._h, ptr(ms), ptr(n), 4))
        return {k: (float(ms[i]), int(n[i])) for i, k in enumerate(("forward", "recompute", "adjoint", "aux"))}

    # -- host (numpy) entry points -----------------------------------------------------------
    def _vel(self, vel_mps) -> np.ndarray:
        v = np.ascontiguousarray(vel_mps, dtype=np.float32)
        if v.size % self.cells_vis:
            raise ValueError(f"velocity size {v.size} is not a multiple of {self.cells_vis}")
        return v.reshape(-1, self.cells_vis)

    def simulate(self, vel_mps) -> np.ndarray:
        v = self._vel(vel_mps)
        out = np.empty((v.shape[0], self.shots, self.nt, self.nrec), np.float32)
        check(self._lib.wg_simulate(self._h, ptr(v), v.shape[0], ptr(out)), "simulate")
        return out

    def evaluate_adjoint(self, vel_mps, observed) -> tuple[np.ndarray, np.ndarray]:
        v = self._vel(vel_mps)
        b = v.shape[0]
        obs = np.ascontiguousarray(observed, dtype=np.float32)
        if obs.size != b * self.shots * self.nt * self.nrec:
            raise ValueError("observed length does not match shots * nt * nrec")
        loss = np.zeros(b, np.float64)
        grad = np.empty((b, self.nz_vis, self.nx_vis), np.float32)
        check(self._lib.wg_evaluate_adjoint(self._h, ptr(v), ptr(obs), b, ptr(loss), ptr(grad)), "evaluate_adjoint")
        return loss, grad

    # -- device (torch) entry points ---------------------------------------------------------
    def _dev(self, t, name: str):
        import torch

        if not isinstance(t, torch.Tensor) or not t.is_cuda:
            raise TypeError(f"{name} must be a CUDA tensor")
        if t.dtype != torch.float32:
            raise TypeError(f"{name} must be float32")
        return t.contiguous()

    def status(self, what: str = "") -> None:
        """Wait for the current torch stream and raise if the engine's last device call set an error
        (zero-energy observed data -> RuntimeError, as the reference's panic; a timed-out kernel
        wait -> RuntimeError)."""
        check(self._lib.wg_engine_status(self._h, _torch_stream()), what)

    def simulate_torch(self, vel_mps, check_status: bool = True):
        """Synthetics of CUDA velocities on the current stream. `check_status` waits for the stream
        and raises on a device error; False leaves the call asynchronous (read it later with
        `status()`)."""
        import torch

        v = self._dev(vel_mps, "vel_mps").reshape(-1, self.cells_vis)
        out = torch.empty((v.shape[0], self.shots, self.nt, self.nrec), device=v.device, dtype=torch.float32)
        with torch.cuda.device(v.device):
            check(self._lib.wg_simulate_dev(self._h, ptr(v), v.shape[0], ptr(out), _torch_stream()), "simulate")
            if check_status:
                self.status("simulate")
        return out

    def evaluate_adjoint_torch(self, vel_mps, observed, check_status: bool = True):
        """Misfit and gradient of CUDA tensors on the current stream; `check_status` as in
        `simulate_torch` (zero-energy observed data raise RuntimeError)."""
        import torch

        v = self._dev(vel_mps, "vel_mps").reshape(-1, self.cells_vis)
        b = v.shape[0]
        obs = self._dev(observed, "observed")
        if obs.numel() != b * self.shots * self.nt * self.nrec:
            raise ValueError("observed length does not match shots * nt * nrec")
        loss = torch.empty(b, device=v.device, dtype=torch.float64)
        grad = torch.empty((b, self.nz_vis, self.nx_vis), device=v.device, dtype=torch.float32)
        with torch.cuda.device(v.device):
            check(self._lib.wg_evaluate_adjoint_dev(self._h, ptr(v), ptr(obs), b, ptr(loss), ptr(grad),
                                                    _torch_stream()), "evaluate_adjoint")
            if check_status:
                self.status("evaluate_adjoint")
        return loss, grad


def ricker_wavelet(samples: int, dt: float, peak_hz: float) -> np.ndarray:
    out = np.zeros(int(samples), np.float32)
    check(_lib.load().wg_ricker_wavelet(int(samples), float(dt), float(peak_hz), ptr(out)))
    return out


def cpml_profiles(n: int, h: float, dt: float, width: int, max_vel: float, freq: float):
    a, b, db = (np.zeros(n, np.float32) for _ in range(3))
    check(_lib.load().wg_cpml_profiles(int(n), float(h), float(dt), int(width), float(max_vel), float(freq),
                                       ptr(a), ptr(b), ptr(db)))
    return a, b, db
