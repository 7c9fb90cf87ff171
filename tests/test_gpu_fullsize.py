"""The benchmarked gradient workload at full size: 256 seeded mixed-family 70x70 models x 5 shots,
nt 1000, dt 1 ms, checkpoint every 100 steps (the oracle is too slow for all of it, so the batch is
held to properties that do not depend on its size):

* the host-pointer entry point (the reference-facing call that the end-to-end rate times) returns
  the device entry point's loss and gradient bit for bit;
* checkpoint-and-recompute equals storing every step's gradient term (the reference's scheme);
* a model's gradient does not depend on the batch it is computed in;
* sampled models' traces, losses and gradients equal the oracle's bit for bit.
"""

from __future__ import annotations

import numpy as np
import pytest

from oracle import native as o

pytestmark = pytest.mark.gpu

SHOT_CELLS = [0, 17, 34, 52, 69]


def test_full_gradient_batch(cuda_lib):
    import torch

    from wgnet_gb300.engine import WaveEngine
    from wgnet_gb300.models_synth import make_batch, smooth

    src = np.stack([np.float32(SHOT_CELLS) * np.float32(10.0), np.full(5, 10.0, np.float32)], 1).astype(np.float32)
    eng = WaveEngine(shots=5, nt=1000, dt=0.001, peak_hz=15.0, pml=20, vmin=1000.0, vmax=5000.0,
                     checkpoint_every=100)
    eng.set_sources(src)
    true = make_batch(256, seed=0)
    start = smooth(true, 5.0)
    d_start = torch.from_numpy(start).cuda()
    obs = eng.simulate_torch(torch.from_numpy(true).cuda())
    d_loss, d_grad = eng.evaluate_adjoint_torch(d_start, obs)
    loss, grad = d_loss.cpu().numpy(), d_grad.cpu().numpy()
    h_obs = obs.cpu().numpy()
    assert np.isfinite(grad).all() and (loss > 0).all()

    h_loss, h_grad = eng.evaluate_adjoint(start, h_obs)
    np.testing.assert_array_equal(h_grad, grad)
    np.testing.assert_array_equal(h_loss, loss)

    eng.checkpoint_every = 1000
    s_loss, s_grad = eng.evaluate_adjoint_torch(d_start, obs)
    np.testing.assert_array_equal(s_grad.cpu().numpy(), grad)
    np.testing.assert_array_equal(s_loss.cpu().numpy(), loss)
    eng.checkpoint_every = 100

    for i in (0, 131, 255):
        li, gi = eng.evaluate_adjoint_torch(d_start[i:i + 1], obs[i:i + 1])
        np.testing.assert_array_equal(gi.cpu().numpy()[0], grad[i])
        np.testing.assert_array_equal(li.cpu().numpy()[0], loss[i])

    sv = o.Survey(shots=5, nt=1000, dt=0.001, pml=20)
    wav = eng.wavelet()
    idx = [7, 200]
    np.testing.assert_array_equal(h_obs[idx], o.forward(sv, true[idx], src, wav))
    rl, rg = o.evaluate_adjoint(sv, start[idx], src, wav, h_obs[idx])
    np.testing.assert_array_equal(grad[idx], rg)
    np.testing.assert_allclose(loss[idx], rl, rtol=1e-12)
