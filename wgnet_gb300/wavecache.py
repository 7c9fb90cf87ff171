"""Resumable on-disk cache of decimated FP16 shot gathers: the wave-cache writer of
python/wgnet/data.py:138-179, for batches of models on several grid sizes, fed by the CUDA
generator (`datagen.GatherGenerator`).

Format (this repository's own; one set of files per grid size n, prefix `<root>/<name>_<n>x<n>`):

* `<prefix>.f16.bin`      raw IEEE half, C order `[models, shots, nt_out, n]` (numpy memmap)
* `<prefix>.progress.json` while writing: {"completed": models done, "sq_sum": sum of squares of the
                           stored values (f64), "shape": [...], "fingerprint": "..."}
* `<prefix>.done.json`     when complete: {"count": models, "rms": RMS of the stored values,
                           "shape": [...], "fingerprint": "..."}; the progress file is removed.

Chunks are written in model order; after each chunk the memmap is flushed and only then the
progress file is replaced (write to a temporary file, then an atomic rename), so an interrupted
run resumes from the last recorded chunk and rewrites anything after it: the finished file is
byte-identical to one written without interruption. A progress or done file whose shape or
fingerprint (the generation parameters) differs from the request is refused rather than resumed.
As in the reference, the RMS of the stored gathers is kept for the network's amplitude scale;
unlike it, the traces are low-passed before decimation (datagen.py) and the time step and
decimation are parameters.
"""

from __future__ import annotations

import json
import os
from pathlib import Path
from typing import Callable

import numpy as np


def _write_json(path: Path, data: dict) -> None:
    tmp = path.with_suffix(path.suffix + ".tmp")
    with open(tmp, "w", encoding="utf-8") as f:
        json.dump(data, f, indent=1)
        f.flush()
        os.fsync(f.fileno())
    os.replace(tmp, path)


def _read_json(path: Path) -> dict | None:
    try:
        with open(path, "r", encoding="utf-8") as f:
            return json.load(f)
    except (OSError, ValueError):
        return None


def cache_paths(prefix: Path) -> tuple[Path, Path, Path]:
    prefix = Path(prefix)
    return (prefix.with_name(prefix.name + ".f16.bin"), prefix.with_name(prefix.name + ".progress.json"),
            prefix.with_name(prefix.name + ".done.json"))


def write_wave_cache(prefix: Path, shape: tuple[int, int, int, int], simulate: Callable[[int, int], np.ndarray],
                     chunk: int = 256, fingerprint: str = "", log: Callable[[str], None] | None = None) -> np.memmap:
    """Fill `<prefix>.f16.bin` of `shape = (models, shots, nt_out, nrec)` with `simulate(i0, i1)`
    (float16 `[i1 - i0, shots, nt_out, nrec]` for models i0..i1), resuming from the progress file,
    and return it opened read-only. A complete cache is opened without simulating."""
    shape = tuple(int(s) for s in shape)
    if len(shape) != 4 or min(shape) < 0:
        raise ValueError("shape must be (models, shots, nt_out, nrec)")
    if chunk < 1:
        raise ValueError("chunk must be >= 1")
    binp, progp, donep = cache_paths(prefix)
    done = _read_json(donep)
    if done is not None and binp.exists():
        if tuple(done.get("shape", ())) != shape or done.get("fingerprint", "") != fingerprint:
            raise ValueError(f"{donep} describes another cache (shape {done.get('shape')}, fingerprint "
                             f"{done.get('fingerprint')!r}): remove it or pick another name")
        return np.memmap(binp, dtype=np.float16, mode="r", shape=shape)
    start, sq_sum = 0, 0.0
    prog = _read_json(progp) if binp.exists() else None
    if prog is not None:
        if tuple(prog.get("shape", ())) != shape or prog.get("fingerprint", "") != fingerprint:
            raise ValueError(f"{progp} belongs to another cache (shape {prog.get('shape')}, fingerprint "
                             f"{prog.get('fingerprint')!r}): remove it or pick another name")
        start, sq_sum = int(prog["completed"]), float(prog["sq_sum"])
    binp.parent.mkdir(parents=True, exist_ok=True)
    mm = np.memmap(binp, dtype=np.float16, mode="r+" if start > 0 else "w+", shape=shape)
    models = shape[0]
    for i0 in range(start, models, chunk):
        i1 = min(i0 + chunk, models)
        g = np.asarray(simulate(i0, i1))
        if g.dtype != np.float16 or g.shape != (i1 - i0,) + shape[1:]:
            raise ValueError(f"simulate({i0}, {i1}) returned {g.dtype} {g.shape}, expected float16 "
                             f"{(i1 - i0,) + shape[1:]}")
        mm[i0:i1] = g
        sq_sum += float(np.square(g, dtype=np.float64).sum())
        mm.flush()
        _write_json(progp, {"completed": i1, "sq_sum": sq_sum, "shape": list(shape), "fingerprint": fingerprint})
        if log:
            log(f"[{binp.name}] {i1}/{models}")
    del mm
    count = models * shape[1] * shape[2] * shape[3]
    _write_json(donep, {"count": models, "rms": float(np.sqrt(sq_sum / max(count, 1))), "shape": list(shape),
                        "fingerprint": fingerprint})
    progp.unlink(missing_ok=True)
    return np.memmap(binp, dtype=np.float16, mode="r", shape=shape)


def cache_rms(prefix: Path) -> float:
    """RMS of a complete cache's stored gathers (the network's amplitude normalisation)."""
    done = _read_json(cache_paths(prefix)[2])
    if done is None:
        raise FileNotFoundError(f"{prefix}: cache not complete")
    return max(float(done["rms"]), 1e-6)


def ensure_wave_cache(root: Path, velocity: dict[int, np.ndarray], name: str = "waves", shots: int = 5,
                      nt: int = 1000, dt: float = 0.001, factor: int = 4, chunk: int = 512,
                      log: Callable[[str], None] | None = None, **engine_kw) -> dict[int, np.memmap]:
    """Simulate (resumably) and open the decimated FP16 gather cache of every grid size:
    `velocity = {n: [models, n, n] m/s}` -> `{n: memmap [models, shots, ceil(nt / factor), n]}`.
    Each chunk of `chunk` models is one replay of the generator's CUDA graph (the last chunk is
    padded with copies of its last model, whose outputs are dropped)."""
    from .datagen import GatherGenerator

    out = {}
    nt_out = (nt + factor - 1) // factor
    for n, vel in sorted(velocity.items()):
        n = int(n)
        vel = np.ascontiguousarray(vel, dtype=np.float32)
        models = vel.shape[0]
        prefix = Path(root) / f"{name}_{n}x{n}"
        fp = (f"n={n} shots={shots} nt={nt} dt={dt} factor={factor} "
              f"{sorted(engine_kw.items())} vel_sum={float(vel.astype(np.float64).sum()):.6e}")
        shape = (models, shots, nt_out, n)
        binp, _, donep = cache_paths(prefix)
        if binp.exists() and donep.exists():
            out[n] = write_wave_cache(prefix, shape, None, chunk, fp, log)
            continue
        m = min(chunk, max(models, 1))
        gen = GatherGenerator({n: m}, shots=shots, nt=nt, dt=dt, factor=factor, **engine_kw)

        def simulate(i0, i1, gen=gen, vel=vel, m=m, n=n):
            v = vel[i0:i1]
            if len(v) < m:
                v = np.concatenate([v, np.repeat(v[-1:], m - len(v), axis=0)])
            g = gen.run({n: v})[n]
            return g[: i1 - i0].cpu().numpy()

        try:
            out[n] = write_wave_cache(prefix, shape, simulate, m, fp, log)
        finally:
            gen.close()
    return out


__all__ = ["write_wave_cache", "ensure_wave_cache", "cache_paths", "cache_rms"]
