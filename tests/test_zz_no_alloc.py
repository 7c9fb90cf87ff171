"""The allocation-free gradient entry point, wg_evaluate_adjoint_noalloc, through the C ABI.

It exists for callers that cannot call cudaMalloc at call time because another allocator owns the
GPU's memory. Its results must equal the regular device entry point's (wg_evaluate_adjoint_dev)
bit for bit, on consecutive calls that reuse the same static scratch array, and sizes beyond the
scratch limit must be refused with a clear error. This file is collected last on purpose.
"""

from __future__ import annotations

import numpy as np
import pytest

from conftest import layered_model

pytestmark = pytest.mark.gpu


def _engine():
    from wgnet_gb300.engine import WaveEngine

    eng = WaveEngine(shots=5, nt=1000, dt=0.001, peak_hz=15.0, pml=20, vmin=1000.0, vmax=5000.0,
                     checkpoint_every=50)
    src = np.stack([np.float32([0, 17, 34, 52, 69]) * np.float32(10.0), np.full(5, 10.0, np.float32)], 1)
    eng.set_sources(src.astype(np.float32))
    return eng


def _call_noalloc(eng, vel, obs, models):
    import torch

    from wgnet_gb300 import _lib

    loss = torch.full((models,), float("nan"), dtype=torch.float64, device="cuda")
    grad = torch.full((models, 70, 70), float("nan"), dtype=torch.float32, device="cuda")
    rc = _lib.load().wg_evaluate_adjoint_noalloc(eng._h, vel.data_ptr(), obs.data_ptr(), models, loss.data_ptr(),
                                                 grad.data_ptr(), torch.cuda.current_stream().cuda_stream)
    return rc, loss, grad


def test_noalloc_matches_the_allocating_entry_point_on_consecutive_calls(cuda_lib):
    import torch

    from wgnet_gb300 import _lib

    eng = _engine()
    cases = []
    for seed in (11, 12):
        true = torch.tensor(layered_model(seed), device="cuda")[None]
        start = torch.tensor(layered_model(seed + 100), device="cuda")[None]
        obs = eng.simulate_torch(true)
        cases.append((start.contiguous(), obs.contiguous()))
    for start, obs in cases + cases[:1]:  # two different calls in a row, then the first again
        rc, loss, grad = _call_noalloc(eng, start, obs, 1)
        _lib.check(rc, "wg_evaluate_adjoint_noalloc")
        _lib.check(_lib.load().wg_engine_status(eng._h, torch.cuda.current_stream().cuda_stream), "status")
        ref_loss, ref_grad = eng.evaluate_adjoint_torch(start, obs)
        torch.cuda.synchronize()
        assert torch.isfinite(grad).all()
        np.testing.assert_array_equal(grad.cpu().numpy(), ref_grad.cpu().numpy())
        np.testing.assert_allclose(loss.cpu().numpy(), ref_loss.cpu().numpy(), rtol=1e-12, atol=0)


def test_noalloc_interval_fallback_matches_store_every_step(cuda_lib):
    """With the engine set to keep every step's gradient term (about 260 MB at this size), the
    scratch array cannot hold the engine's scheme, so the call picks the checkpoint interval with
    the smallest footprint (59 steps here, which does not divide nt = 1000). The gradient must still
    equal the allocating entry point's store-every-step result bit for bit."""
    import torch

    from wgnet_gb300 import _lib

    eng = _engine()
    eng.checkpoint_every = 0
    true = torch.tensor(layered_model(21), device="cuda")[None]
    start = torch.tensor(layered_model(121), device="cuda")[None].contiguous()
    obs = eng.simulate_torch(true).contiguous()
    ref_loss, ref_grad = eng.evaluate_adjoint_torch(start, obs)
    for _ in range(2):
        rc, loss, grad = _call_noalloc(eng, start, obs, 1)
        _lib.check(rc, "wg_evaluate_adjoint_noalloc")
        _lib.check(_lib.load().wg_engine_status(eng._h, torch.cuda.current_stream().cuda_stream), "status")
        np.testing.assert_array_equal(grad.cpu().numpy(), ref_grad.cpu().numpy())
        np.testing.assert_allclose(loss.cpu().numpy(), ref_loss.cpu().numpy(), rtol=1e-12, atol=0)


def test_noalloc_refuses_sizes_beyond_its_scratch(cuda_lib):
    import torch

    from wgnet_gb300 import _lib

    eng = _engine()
    models = 4
    vel = torch.full((models, 70, 70), 2500.0, device="cuda")
    obs = torch.ones((models, 5, 1000, 70), device="cuda")
    rc, _, _ = _call_noalloc(eng, vel, obs, models)
    assert rc == _lib.WG_ERR_ARG
    msg = _lib.last_error()
    assert "MiB" in msg and "maximum" in msg
