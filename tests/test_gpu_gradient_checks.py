"""Checks of the gradient path on the GPU: the adjoint dot-product test
<J dv, r> = <dv, J^T r> (J from central differences of the FP64 oracle forward, J^T from the CUDA
adjoint), and gradients flowing through the Gaussian renderer to offset / scale / angle /
amplitude (WaveLoss + render_residual autograd against FP64 finite differences of the oracle)."""

from __future__ import annotations

import numpy as np
import pytest

from conftest import layered_model
from oracle import native as o
from oracle import render_np

pytestmark = pytest.mark.gpu


def _survey(nt=300):
    sv = o.Survey(shots=5, nt=nt, dt=0.001)
    src = np.stack([np.float32([0, 17, 34, 52, 69]) * np.float32(10.0), np.full(5, 10.0, np.float32)], 1)
    return sv, src.astype(np.float32)


def test_adjoint_dot_product(cuda_lib):
    from wgnet_gb300.engine import WaveEngine

    sv, src = _survey()
    eng = WaveEngine(shots=5, nt=sv.nt, dt=sv.dt, checkpoint_every=37)
    eng.set_sources(src)
    wav = eng.wavelet()
    rng = np.random.default_rng(4)
    v = layered_model(3)
    p = eng.simulate(v)[0]
    r = (0.5 * np.sqrt(np.mean(p.astype(np.float64) ** 2)) * rng.standard_normal(p.shape)).astype(np.float32)
    d = (p - r).astype(np.float32)  # observed data whose residual is r
    r64 = p.astype(np.float64) - d.astype(np.float64)
    energy = float(np.sum(d.astype(np.float64) ** 2))
    _, g = eng.evaluate_adjoint(v, d[None])
    jt_r = g[0].astype(np.float64) * energy  # gradient = J^T r / ||d||^2
    dv = rng.standard_normal(v.shape)
    eps = 1e-2
    fp = o.forward(sv, (v + eps * dv).astype(np.float32), src, wav, precision="f64")[0]
    fm = o.forward(sv, (v - eps * dv).astype(np.float32), src, wav, precision="f64")[0]
    dvv = ((v + eps * dv).astype(np.float32).astype(np.float64) - (v - eps * dv).astype(np.float32).astype(np.float64))
    lhs = float(np.sum((fp - fm) * r64))          # <J (v+ - v-), r>
    rhs = float(np.sum(jt_r * dvv))               # <v+ - v-, J^T r>
    assert abs(lhs - rhs) <= 1e-4 * abs(lhs), (lhs, rhs)


def test_gradients_reach_gaussian_parameters(cuda_lib):
    import torch

    from wgnet_gb300.engine import WaveEngine
    from wgnet_gb300.physics import WaveLoss
    from wgnet_gb300.render import N_SLOTS, render_residual

    sv, src = _survey(nt=250)
    eng = WaveEngine(shots=5, nt=sv.nt, dt=sv.dt, checkpoint_every=50)
    eng.set_sources(src)
    wav = eng.wavelet()
    rng = np.random.default_rng(8)
    dense = (layered_model(5) / 1000.0).astype(np.float32)
    params = np.zeros((1, N_SLOTS, 6), np.float64)
    slots = [300, 612, 877]  # three active slots
    for k in slots:
        params[0, k] = [rng.uniform(-1, 1), rng.uniform(-1, 1), np.log(rng.uniform(1.5, 3.0)),
                        np.log(rng.uniform(1.5, 3.0)), rng.uniform(-1, 1), rng.uniform(-0.4, 0.4)]
    true = dense + render_np.render(params)[0].astype(np.float32) * np.float32(1.2)
    obs = o.forward(sv, (true * 1000.0).astype(np.float32), src, wav)

    p = torch.tensor(params, dtype=torch.float32, device="cuda", requires_grad=True)
    field = torch.tensor(dense, device="cuda")[None] + render_residual(p)
    loss = WaveLoss.apply(field, torch.tensor(obs, device="cuda"), eng)
    loss.sum().backward()
    g = p.grad.double().cpu().numpy()

    def oracle_loss(pp):
        f = dense.astype(np.float64) + render_np.render(pp)[0]
        lo, _ = o.evaluate_adjoint(sv, (f * 1000.0).astype(np.float32), src, wav, obs, precision="f64")
        return float(lo[0])

    for k in slots:
        for j, eps in ((0, 1e-3), (2, 1e-3), (4, 1e-3), (5, 1e-4)):  # offset x, log scale x, angle, amplitude
            pp, pm = params.copy(), params.copy()
            pp[0, k, j] += eps
            pm[0, k, j] -= eps
            fd = (oracle_loss(pp) - oracle_loss(pm)) / (2 * eps)
            assert abs(g[0, k, j] - fd) <= 2e-2 * abs(fd) + 1e-9, (k, j, g[0, k, j], fd)
    inactive = np.setdiff1d(np.arange(N_SLOTS), slots)
    assert np.all(g[0, inactive, :5] == 0.0)  # zero amplitude: only the amplitude gradient lives
