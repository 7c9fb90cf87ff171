"""Launch-shape autotuner for the resident kernels.

For one engine (one grid and survey) it times every compiled CTA/cluster shape that fits the grid
(`WaveEngine.shape_candidates`) on a seeded synthetic batch, with CUDA events around each kernel
launch (`WaveEngine.profile`), and keeps the fastest. Results are cached in a JSON file keyed by
the GPU (name, SM count), the kernel (forward or adjoint) and the survey dimensions, so a shape is
measured once per machine type. The reference has no counterpart: its wgpu dispatches use a fixed
workgroup size (crates/wave-gauss-rs/src/shaders/splatForward.wgsl:48).
"""

from __future__ import annotations

import json
import os
import threading
from pathlib import Path

_CACHE_ENV = "WGNET_GB300_AUTOTUNE_CACHE"
_lock = threading.Lock()


def cache_path() -> Path:
    p = os.environ.get(_CACHE_ENV)
    if p:
        return Path(p)
    return Path.home() / ".cache" / "wgnet_gb300" / "autotune.json"


def device_tag() -> str:
    import torch

    props = torch.cuda.get_device_properties(torch.cuda.current_device())
    return f"{props.name}|sm{props.multi_processor_count}"


def cache_key(device: str, which: str, eng) -> str:
    """The timing of a shape depends on the padded grid, the stations, the shot count and the
    arithmetic (fast kernels exist for some shapes only); nt only scales it."""
    arith = eng.get_option("arith")
    return f"{device}|{which}|{eng.nx}x{eng.nz}|pml{eng.pml}|shots{eng.shots}|nrec{eng.nrec}|arith{arith}"


def load_cache(path: Path | None = None) -> dict:
    path = path or cache_path()
    try:
        with open(path, "r", encoding="utf-8") as f:
            data = json.load(f)
        return data if isinstance(data, dict) else {}
    except (OSError, ValueError):
        return {}


def store_cache(entries: dict, path: Path | None = None) -> None:
    """Merge `entries` into the cache file (atomic replace)."""
    path = path or cache_path()
    with _lock:
        data = load_cache(path)
        data.update(entries)
        path.parent.mkdir(parents=True, exist_ok=True)
        tmp = path.with_suffix(path.suffix + f".{os.getpid()}.tmp")
        with open(tmp, "w", encoding="utf-8") as f:
            json.dump(data, f, indent=1, sort_keys=True)
        os.replace(tmp, path)


def _probe_models(eng, models: int, seed: int):
    import torch

    from .models_synth import make_batch

    v = make_batch(models, seed=seed, nz=eng.nz_vis, nx=eng.nx_vis)
    return torch.from_numpy(v).cuda()


def _time_forward(eng, vel, reps: int) -> float:
    import torch

    eng.simulate_torch(vel)  # warm-up (first launch of this shape)
    torch.cuda.synchronize()
    eng.profile(True)
    for _ in range(reps):
        eng.simulate_torch(vel)
    torch.cuda.synchronize()
    rec = eng.profile_read()
    eng.profile(False)
    ms, n = rec["forward"]
    return ms / max(n, 1)


def _time_adjoint(eng, vel, obs, reps: int) -> float:
    import torch

    eng.evaluate_adjoint_torch(vel, obs)
    torch.cuda.synchronize()
    eng.profile(True)
    for _ in range(reps):
        eng.evaluate_adjoint_torch(vel, obs)
    torch.cuda.synchronize()
    rec = eng.profile_read()
    eng.profile(False)
    ms, _ = rec["adjoint"]
    return ms / reps


def tune(eng, which: tuple[str, ...] = ("forward", "adjoint"), models: int = 64, reps: int = 2, seed: int = 7,
         force: bool = False, path: Path | None = None) -> dict[str, tuple[int, int, int]]:
    """Pick and apply the fastest launch shape for each kernel in `which`; returns {kernel: shape}.

    A cached choice is applied without timing unless `force`. Timing uses `models` synthetic models
    (all shots), so the batch spans several waves of clusters over the SMs.
    """
    device = device_tag()
    cache = {} if force else load_cache(path)
    chosen: dict[str, tuple[int, int, int]] = {}
    new_entries: dict = {}
    vel = obs = None
    for kernel in which:
        cands = eng.shape_candidates(kernel)
        key = cache_key(device, kernel, eng)
        hit = cache.get(key)
        if hit and tuple(hit["shape"]) in cands:
            shape = tuple(int(x) for x in hit["shape"])
            eng.set_launch_shape(kernel, shape)
            chosen[kernel] = shape
            continue
        if not cands:
            continue
        if vel is None:
            vel = _probe_models(eng, models, seed)
        if kernel == "adjoint" and obs is None:
            import torch

            from .models_synth import smooth

            obs = eng.simulate_torch(torch.from_numpy(smooth(vel.cpu().numpy(), 3.0)).cuda())
        original = eng.launch_shape(kernel)
        timings = {}
        for shape in cands:
            eng.set_launch_shape(kernel, shape)
            t = _time_forward(eng, vel, reps) if kernel == "forward" else _time_adjoint(eng, vel, obs, reps)
            timings[shape] = t
        best = min(timings, key=timings.get) if timings else original
        eng.set_launch_shape(kernel, best)
        chosen[kernel] = best
        new_entries[key] = {"shape": list(best), "ms": {",".join(map(str, s)): round(t, 4) for s, t in timings.items()},
                            "models": models}
    if new_entries:
        store_cache(new_entries, path)
    return chosen


def measured(path: Path | None = None) -> dict:
    """The cache contents (for reports)."""
    return load_cache(path)


__all__ = ["tune", "cache_path", "cache_key", "load_cache", "store_cache", "device_tag", "measured"]
