"""Band schedule on engines whose step is not the reference's 0.5 ms, and device status on the
device-pointer entry points. GPU tests, through the C ABI.

* `WavePhysics.set_band(f)` designs the causal low-pass at the wrapped engine's own step
  (physics.py:37-46 uses the module's DT because the reference's engine is fixed to it): on a 1 ms
  engine the installed wavelet is exactly `np.convolve(full, lowpass_kernel(f, 1e-3))[:nt]`, and the
  band identity of python/verify.py:76-84 holds (synthetics of the filtered wavelet == bandlimit of
  the full-band synthetics, max relative difference < 2e-3).
* Zero-energy observed data raise the reference's error (`assert!(energy > 0)`,
  crates/wave-gauss-rs/src/wave_wgpu.rs:853) through the device entry points too: `WaveLoss.apply`,
  `evaluate_adjoint_torch` and the allocation-free entry point (status read with
  wg_engine_status), and a later good call on the same engine succeeds (the word is cleared per call).
* A bounded wait that runs out: the streamed kernels' mbarrier wait on a copy that is never issued
  gives up after its poll limit and the kernel records the error instead of hanging; the status
  reads WG_ERR_CUDA, and the same context then computes the same traces and gradient as before.
"""

from __future__ import annotations

import numpy as np
import pytest

from conftest import layered_model
from oracle import physics_np

pytestmark = pytest.mark.gpu


def _engine_1ms(shots=5, nt=1000):
    from wgnet_gb300.engine import WaveEngine

    eng = WaveEngine(shots=shots, nt=nt, dt=0.001, peak_hz=15.0, pml=20, vmin=1000.0, vmax=5000.0)
    cells = np.float32([0, 17, 34, 52, 69][:shots])
    eng.set_sources(np.stack([cells * np.float32(10.0), np.full(shots, 10.0, np.float32)], 1).astype(np.float32))
    return eng


@pytest.mark.parametrize("fmax", [6.0, 9.0, 12.0])
def test_set_band_uses_the_engine_step(cuda_lib, fmax):
    from wgnet_gb300.physics import WavePhysics, lowpass_kernel

    eng = _engine_1ms()
    ph = WavePhysics(shots=eng.shots, nt=eng.nt, engine=eng)
    assert ph.dt == 0.001
    full = ph.full_wavelet.copy()
    ph.set_band(fmax)
    k = lowpass_kernel(fmax, 1e-3)
    np.testing.assert_array_equal(ph.kernel, k)
    np.testing.assert_array_equal(k, physics_np.lowpass_kernel(fmax, 1e-3))
    expect = np.convolve(full, k, mode="full")[: eng.nt].astype(np.float32)
    np.testing.assert_array_equal(eng.wavelet(), expect)
    # The Gaussian's amplitude response is exp(-2 pi^2 sigma^2 f^2) with sigma^2 = ln 2 / (2 pi^2 fmax^2):
    # gain 1/2 (power -6 dB, the "-3 dB" of physics.py:19 in its own words) at f = fmax, when the
    # kernel is sampled at the engine's 1 ms step (at 0.5 ms taps on a 1 ms engine it fell at fmax / 2).
    freqs = np.fft.rfftfreq(8192, d=1e-3)
    gain = np.abs(np.fft.rfft(k.astype(np.float64), 8192))
    f_half = float(np.interp(0.5, gain[::-1], freqs[::-1]))
    assert abs(f_half - fmax) < 0.02 * fmax, f_half
    ph.set_band(None)
    np.testing.assert_array_equal(eng.wavelet(), full)


def test_band_identity_on_a_1ms_engine(cuda_lib):
    import torch

    from wgnet_gb300.physics import WavePhysics

    eng = _engine_1ms(shots=2, nt=600)
    ph = WavePhysics(shots=2, nt=600, engine=eng)
    field = torch.tensor(layered_model(3) / 1000.0, dtype=torch.float32, device="cuda")[None]
    ph.set_band(8.0)
    low = ph.simulate(field)
    ph.set_band(None)
    full = ph.simulate(field)
    ph.set_band(8.0)
    filtered = ph.bandlimit(full)
    rel = float((low - filtered).abs().max() / filtered.abs().max())
    assert rel < 2e-3, rel


def test_zero_energy_raises_through_the_device_entry_points(cuda_lib):
    import torch

    from wgnet_gb300 import _lib
    from wgnet_gb300.physics import WaveLoss

    eng = _engine_1ms(shots=5, nt=300)
    vel = torch.tensor(layered_model(5), device="cuda")[None].contiguous()
    zero = torch.zeros((1, 5, 300, 70), device="cuda")
    with pytest.raises(RuntimeError, match="zero energy"):
        eng.evaluate_adjoint_torch(vel, zero)
    with pytest.raises(RuntimeError, match="zero energy"):
        WaveLoss.apply((vel / 1000.0).requires_grad_(True), zero, eng)
    # the allocation-free entry point: same error from its status
    lib = _lib.load()
    loss = torch.empty(1, dtype=torch.float64, device="cuda")
    grad = torch.empty((1, 70, 70), device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    _lib.check(lib.wg_evaluate_adjoint_noalloc(eng._h, vel.data_ptr(), zero.data_ptr(), 1, loss.data_ptr(),
                                               grad.data_ptr(), stream))
    assert lib.wg_engine_status(eng._h, stream) == _lib.WG_ERR_ENERGY
    assert "zero energy" in _lib.last_error()
    # a good call on the same engine afterwards starts with a clear status
    obs = eng.simulate_torch(vel * 1.05)
    l2, g2 = eng.evaluate_adjoint_torch(vel, obs)
    assert torch.isfinite(l2).all() and torch.isfinite(g2).all()
    _lib.check(lib.wg_evaluate_adjoint_noalloc(eng._h, vel.data_ptr(), obs.data_ptr(), 1, loss.data_ptr(),
                                               grad.data_ptr(), stream))
    assert lib.wg_engine_status(eng._h, stream) == _lib.WG_OK
    np.testing.assert_array_equal(grad.cpu().numpy(), g2.cpu().numpy())


def test_a_bounded_wait_that_runs_out_reports_and_the_context_stays_usable(cuda_lib):
    import torch

    from wgnet_gb300 import _lib

    eng = _engine_1ms(shots=2, nt=200)
    lib = _lib.load()
    stream = torch.cuda.current_stream().cuda_stream
    vel = torch.tensor(layered_model(5), device="cuda")[None].contiguous()
    before = eng.simulate_torch(vel)
    obs = eng.simulate_torch(vel * 1.05)
    loss0, grad0 = eng.evaluate_adjoint_torch(vel, obs)
    assert lib.wg_selftest_wait_timeout(eng._h, 0, stream) == _lib.WG_ERR_ARG
    assert lib.wg_selftest_wait_timeout(eng._h, (1 << 22) + 1, stream) == _lib.WG_ERR_ARG
    _lib.check(lib.wg_selftest_wait_timeout(eng._h, 1 << 14, stream))
    assert lib.wg_engine_status(eng._h, stream) == _lib.WG_ERR_CUDA
    assert "timed out" in _lib.last_error()
    # the context is intact: the next calls clear the word and compute the same results as before
    after = eng.simulate_torch(vel)
    assert lib.wg_engine_status(eng._h, stream) == _lib.WG_OK
    assert torch.equal(after, before)
    loss1, grad1 = eng.evaluate_adjoint_torch(vel, obs)
    assert torch.equal(loss1, loss0) and torch.equal(grad1, grad0)
