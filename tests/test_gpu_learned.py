"""What the trained update network gains: on held-out seeded models (5-, 3- and 1-shot surveys,
starting models smoothed by 5 cells and by 8 cells, bands 6 / 9 / 12 Hz / full), learned-plus-exact
refinement reaches the velocity MAE that plain projected L-BFGS ends with in at least 2x fewer
wave solves, and ends below plain's MAE. The weights are the committed ones
(wgnet_gb300/weights/update_net.npz, made by `python -m wgnet_gb300.learned` from starts smoothed
by 3 to 8 cells; provenance in update_net.json)."""

from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

WEIGHTS = Path(__file__).resolve().parents[1] / "wgnet_gb300" / "weights" / "update_net.npz"


@pytest.mark.parametrize("sigma", [5.0, 8.0])
@pytest.mark.parametrize("shots", [5, 3, 1])
def test_learned_refinement_needs_half_the_solves(cuda_lib, shots, sigma):
    from wgnet_gb300.learned import evaluate
    from wgnet_gb300.precond import UpdateNet

    net = UpdateNet.load(WEIGHTS)
    r = evaluate(net, n_models=16, seed=4242, shots=shots, budget=80, sigma=sigma)
    assert r["reached_fraction"] >= 0.9
    assert r["solve_ratio_median"] >= 2.0, r
    assert r["mae_learned_km"] < r["mae_plain_km"]
