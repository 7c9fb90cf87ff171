"""This repository's Python layer against the reference's own Python, on the GPU.

tests/golden/refpy.npz holds outputs of the reference's python/wgnet/physics.py and refine.py, run
unchanged over the C++ oracle standing in for the PyO3 engine (tests/golden/make_refpy.py). Here the
same inputs go through `wgnet_gb300.physics.WavePhysics` and `wgnet_gb300.refine.refine` on the CUDA
engine, which matches the oracle bit for bit. Checked, following python/verify.py:

* loss_and_grad (2 shots, nt 501): gradients bit-identical to the reference's, losses to f32;
* the adjoint through the renderer against central differences, < 3 % (verify.py:57-74);
* set_band / simulate / bandlimit: the band-limited wavelet to 1e-5 (np.convolve of float32 arrays
  rounds differently on x86, where the fixtures were made, and on other CPUs), the synthetics of
  the same wavelet bit-identical, the filtered data to 1e-6 of its peak (torch's conv1d and the CUDA
  FIR sum in different orders), the band identity < 2e-3 (verify.py:76-84);
* refine() (2 shots, nt 801, 30 solves, bands 10 Hz / full): with the reference's rounding of the
  10 Hz wavelet and band-limited data installed (ours agree with them to 1e-6 of the peak), the same
  number of solves and accept/reject sequence, the first iteration's loss to 1e-5 and the second's
  to 3 %, the later ones and the final misfit within the reference's own noise envelope, and the
  misfit reduced below 0.7x (verify.py:107-117). Later iterations cannot match closely: on this
  small-misfit problem the curvature pairs y = g1 - g0 are small differences of gradients, and the
  Gaussian-parameter gradients are f32 sums over 625-pixel windows whose rounding differs between
  any two implementations at ~1e-4. Measured on the reference itself with these inputs, 1e-4
  relative noise on those gradients moves its losses by 2.4 %, 8 %, 9 % and 8 % at iterations 2,
  4, 6 and the end (and 1e-7 noise on its data by 0.2 %). End to end with this repository's own
  set_band and bandlimit: the same solves and accept/reject sequence, and the misfit below 0.7x.
"""

from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = Path(__file__).resolve().parent / "golden" / "refpy.npz"


@pytest.fixture(scope="module")
def g():
    return np.load(GOLD)


def test_loss_and_grad_equals_the_reference_python(cuda_lib, g):
    from wgnet_gb300.physics import WavePhysics

    ph = WavePhysics(shots=2, nt=501)
    losses, grads = ph.loss_and_grad(g["adj_field"], g["adj_observed"])
    assert grads.dtype == np.float32 and losses.dtype == np.float32
    np.testing.assert_array_equal(grads, g["adj_grads"])
    np.testing.assert_allclose(losses, g["adj_losses"], rtol=1e-6, atol=0)


def test_adjoint_through_the_renderer_against_finite_differences(cuda_lib, g):
    import torch

    from wgnet_gb300.physics import WavePhysics
    from wgnet_gb300.render import render_residual

    ph = WavePhysics(shots=2, nt=501)
    observed = g["adj_observed"]
    base = torch.full((1, 70, 70), 2.5, device="cuda")
    init = torch.tensor(g["adj_init_params"], device="cuda", requires_grad=True)
    field = base + render_residual(init)
    losses, grads = ph.loss_and_grad(field.detach().cpu().numpy(), observed)
    (gp,) = torch.autograd.grad((field * torch.tensor(grads, device="cuda")).sum(), init)
    gen = torch.Generator().manual_seed(3)
    direction = (torch.randn(init.shape, generator=gen) * torch.tensor([0.3, 0.3, 0.1, 0.1, 0.1, 0.1])).cuda()
    eps = 0.02
    with torch.no_grad():
        lp, _ = ph.loss_and_grad((base + render_residual(init + eps * direction)).cpu().numpy(), observed)
        lm, _ = ph.loss_and_grad((base + render_residual(init - eps * direction)).cpu().numpy(), observed)
    fd = float(lp[0] - lm[0]) / (2 * eps)
    adj = float((gp * direction).sum())
    assert abs(fd - adj) / max(abs(fd), 1e-12) < 0.03, (fd, adj)


def test_band_schedule_equals_the_reference_python(cuda_lib, g):
    from wgnet_gb300.physics import WavePhysics

    ph = WavePhysics(shots=2, nt=501)
    ph.set_band(8.0)
    np.testing.assert_array_equal(ph.kernel, g["band_kernel"])
    wav = g["band_wavelet"]
    np.testing.assert_allclose(ph.engine.wavelet(), wav, rtol=0, atol=1e-5 * float(np.abs(wav).max()))
    own = ph.simulate(g["adj_field"])
    ph.engine.set_wavelet(wav)  # the reference's rounding of the same convolution
    low = ph.simulate(g["adj_field"])
    np.testing.assert_array_equal(low, g["band_low"])
    assert float(np.linalg.norm(own - low) / np.linalg.norm(low)) < 1e-5
    ph.set_band(None)
    full = ph.simulate(g["adj_field"])
    np.testing.assert_array_equal(full, g["band_full"])
    ph.set_band(8.0)
    filtered = ph.bandlimit(full)
    peak = float(np.abs(g["band_filtered"]).max())
    assert float(np.abs(filtered - g["band_filtered"]).max()) <= 1e-6 * peak
    assert float(np.abs(low - filtered).max()) / float(np.abs(filtered).max()) < 2e-3


def _refine(g, physics):
    from wgnet_gb300.refine import refine

    return refine(g["ref_base"], g["ref_init"], g["ref_observed"], physics, budget_solves=30, bands_hz=(10.0, None))


def _same_path(res, g):
    hist = res.history
    assert res.solves == int(g["ref_solves"])
    np.testing.assert_allclose(res.initial_loss, float(g["ref_initial_loss"]), rtol=1e-4)
    assert len(hist) == len(g["ref_hist_loss"])
    assert [h["accepted"] for h in hist] == g["ref_hist_accepted"].tolist()
    assert [h["solves"] for h in hist] == g["ref_hist_solves"].tolist()
    assert [-1.0 if h["band_hz"] is None else h["band_hz"] for h in hist] == g["ref_hist_band"].tolist()
    assert res.final_loss < 0.7 * res.initial_loss


def test_refine_follows_the_reference_python(cuda_lib, g):
    import torch

    from wgnet_gb300.physics import WavePhysics

    class RefBand(WavePhysics):
        """The 10 Hz band with the reference's rounding of its wavelet and band-limited data."""

        def set_band(self, fmax_hz):
            super().set_band(fmax_hz)
            if fmax_hz == 10.0:
                self.engine.set_wavelet(g["ref_band10_wavelet"])

        def bandlimit(self, traces):
            if self.fmax == 10.0:
                ours = super().bandlimit(traces)
                ref = torch.tensor(g["ref_band10_observed"], device="cuda").reshape(ours.shape)
                assert float((ours - ref).abs().max()) <= 1e-6 * float(ref.abs().max())
                return ref
            return super().bandlimit(traces)

    res = _refine(g, RefBand(shots=2, nt=801))
    _same_path(res, g)
    losses = np.array([h["loss"] for h in res.history])
    ref = g["ref_hist_loss"]
    np.testing.assert_allclose(losses[0], ref[0], rtol=1e-5)  # steepest descent from the same point
    np.testing.assert_allclose(losses[1], ref[1], rtol=3e-2)  # the first curvature pair
    np.testing.assert_allclose(losses, ref, rtol=0.3)
    np.testing.assert_allclose(res.final_loss, float(g["ref_final_loss"]), rtol=0.1)
    print("\n[refine vs the reference's Python] losses", np.round(losses / ref - 1.0, 4).tolist())


def test_refine_end_to_end_meets_the_reference_criterion(cuda_lib, g):
    from wgnet_gb300.physics import WavePhysics

    _same_path(_refine(g, WavePhysics(shots=2, nt=801)), g)
