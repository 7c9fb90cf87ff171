"""Batched pixel-grid FWI (`wgnet_gb300.fwi`) on CPU with a deterministic stand-in physics whose
per-model misfit does not depend on the batch: every model's result and per-band history equal
those of the reference's sequential procedure (python/wgnet/fwi_eval.py:32-57, restated below as
the checker), bit for bit; a failing objective raises in the caller instead of leaving threads
waiting."""

from __future__ import annotations

import numpy as np
import pytest
from scipy.ndimage import gaussian_filter
from scipy.optimize import minimize

from wgnet_gb300 import fwi as F

N = 8


class StandInPhysics:
    """Misfit sum(w (f - t)^2 + 0.1 (f - t)^4) per model; the target t arrives as the model's
    'observed data', scaled by the band (so set_band and bandlimit matter)."""

    def __init__(self):
        self.band = None
        self.batches = []
        rng = np.random.default_rng(3)
        self.w = rng.uniform(0.5, 2.0, (N, N)).astype(np.float32)

    def set_band(self, band):
        self.band = band

    def bandlimit(self, observed):
        return observed if self.band is None else observed * np.float32(1.0 - 0.01 * self.band)

    def loss_and_grad(self, fields, observed):
        f = np.asarray(fields, np.float32)
        t = np.asarray(observed, np.float32).reshape(f.shape)
        self.batches.append(f.shape[0])
        d = f - t
        loss = (self.w * d * d + np.float32(0.1) * d ** 4).sum(axis=(1, 2), dtype=np.float32)
        grad = np.float32(2.0) * self.w * d + np.float32(0.4) * d ** 3
        return loss.astype(np.float32), grad.astype(np.float32)


def sequential_fwi(start, observed_full, physics, bands, budget, smooth_grad):
    x = start.astype(np.float64).reshape(-1)
    per_band = max(2, budget // len(bands))
    history = []
    for band in bands:
        physics.set_band(band)
        observed = physics.bandlimit(observed_full)
        calls = 0

        def objective(vec):
            nonlocal calls
            calls += 1
            losses, grads = physics.loss_and_grad(vec.reshape(1, N, N).astype(np.float32), observed[None])
            g = gaussian_filter(grads[0], smooth_grad, mode="nearest") if smooth_grad > 0 else grads[0]
            return float(losses[0]), g.reshape(-1).astype(np.float64)

        res = minimize(objective, x, jac=True, method="L-BFGS-B", bounds=[(1.4, 4.6)] * (N * N),
                       options={"maxfun": per_band, "maxiter": per_band, "maxcor": 10})
        x = res.x
        history.append({"band_hz": band, "misfit": float(res.fun), "solves": calls})
    physics.set_band(None)
    return x.reshape(N, N).astype(np.float32), history


@pytest.mark.parametrize("smooth_grad", [1.5, 0.0])
def test_batched_fwi_follows_each_models_sequential_trajectory(smooth_grad):
    rng = np.random.default_rng(11)
    B = 6
    starts = rng.uniform(1.6, 4.4, (B, N, N)).astype(np.float32)
    targets = rng.uniform(1.5, 4.5, (B, N, N)).astype(np.float32)
    observed = targets.reshape(B, 1, 1, N * N)
    bands = [5.0, 9.0, None]
    ph = StandInPhysics()
    finals, hists = F.fwi_batch(starts, observed, ph, bands, budget=30, smooth_grad=smooth_grad)
    assert max(ph.batches) == B and ph.band is None  # batched, and the band reset at the end
    for b in range(B):
        ref_final, ref_hist = sequential_fwi(starts[b], observed[b], StandInPhysics(), bands, 30, smooth_grad)
        np.testing.assert_array_equal(finals[b], ref_final)
        assert hists[b] == ref_hist
    one_final, one_hist = F.fwi(starts[2], observed[2], StandInPhysics(), bands, 30, smooth_grad)
    np.testing.assert_array_equal(one_final, finals[2])
    assert one_hist == hists[2]
    assert F.misfit_full(finals[0], observed[0], ph) < F.misfit_full(starts[0], observed[0], ph)


def test_a_failing_objective_raises_in_the_caller():
    class Failing(StandInPhysics):
        def loss_and_grad(self, fields, observed):
            if len(self.batches) == 3:
                raise FloatingPointError("solver failure")
            return super().loss_and_grad(fields, observed)

    rng = np.random.default_rng(5)
    starts = rng.uniform(1.6, 4.4, (4, N, N)).astype(np.float32)
    observed = rng.uniform(1.5, 4.5, (4, 1, 1, N * N)).astype(np.float32)
    with pytest.raises(RuntimeError, match="batched objective failed"):
        F.fwi_batch(starts, observed, Failing(), [None], budget=20)
    with pytest.raises(ValueError):
        F.fwi_batch(starts[0], observed, StandInPhysics(), [None], budget=20)
