"""pytest configuration: the `gpu` marker, repository imports, shared helpers."""

from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built CUDA library")


def pytest_collection_modifyitems(config, items):
    try:
        import torch

        has_gpu = torch.cuda.is_available()
    except Exception:  # pragma: no cover
        has_gpu = False
    if has_gpu:
        return
    skip = pytest.mark.skip(reason="no CUDA GPU in this environment")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


@pytest.fixture(scope="session")
def cuda_lib():
    """The CUDA library, built on first use (GPU tests only)."""
    from wgnet_gb300 import _lib, build

    if not _lib.LIB_PATH.exists():
        build.build()
    return _lib.load()


def rel_l2(a, b) -> float:
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.sqrt(np.sum((a - b) ** 2) / max(np.sum(b * b), 1e-300)))


def layered_model(seed: int, nz: int = 70, nx: int = 70, lo: float = 1500.0, hi: float = 4500.0) -> np.ndarray:
    """3-5 flat layers, velocities uniform in [lo, hi], increasing with depth (seeded)."""
    rng = np.random.default_rng(seed)
    n = int(rng.integers(3, 6))
    vel = np.sort(rng.uniform(lo, hi, n))
    cuts = np.sort(rng.choice(np.arange(5, nz - 3), n - 1, replace=False))
    v = np.empty((nz, nx), np.float32)
    edges = [0, *cuts.tolist(), nz]
    for k in range(n):
        v[edges[k]:edges[k + 1]] = vel[k]
    return v
