"""Host-side pieces of the batched refinement (no GPU): the parameter space (dense block, coarse
grid and their bounds), the bilinear upsample and its adjoint, and the oracle's restatement of
refine()'s control flow on a toy quadratic (solve accounting and acceptance)."""

from __future__ import annotations

import numpy as np
import torch

from oracle import refine_np


def test_upsample_matches_align_corners_bilinear_and_its_adjoint():
    import torch.nn.functional as F

    from wgnet_gb300.refine import _upsample_matrix

    U = _upsample_matrix(70, 9, "cpu")
    c = torch.randn(2, 9, 9, dtype=torch.float64)
    ref = F.interpolate(c[:, None], size=(70, 70), mode="bilinear", align_corners=True)[:, 0]
    np.testing.assert_allclose((U @ c @ U.t()).numpy(), ref.numpy(), rtol=0, atol=1e-12)
    g = torch.randn(2, 70, 70, dtype=torch.float64)
    lhs = ((U @ c @ U.t()) * g).sum()
    rhs = (c * (U.t() @ g @ U)).sum()
    assert abs(float(lhs - rhs)) < 1e-9 * abs(float(lhs))


def test_space_layout_projection_and_field():
    from wgnet_gb300.refine import COARSE_MAX_KM, DENSE_BOUNDS_KM, DENSE_SCALE, COARSE_SCALE, Space

    start = torch.full((3, 70, 70), 2.5)
    sp = Space(start, None, 0.05, dense_block=True)
    assert sp.P == 4900 + 81 and sp.K == 0
    assert torch.all(sp.scales[:, :4900] == DENSE_SCALE) and torch.all(sp.scales[:, 4900:] == COARSE_SCALE)
    rows = torch.arange(3)
    torch.testing.assert_close(sp.field(sp.x0, rows), start)
    x = sp.x0.clone()
    x[:, :10] = 9.0
    x[:, 4900:4905] = -5.0
    p = sp.project(x)
    assert float(p[:, :4900].max()) == DENSE_BOUNDS_KM[1] and float(p[:, 4900:].min()) == -COARSE_MAX_KM
    # without the dense block the start is the frozen base and only the coarse grid moves
    sp2 = Space(start, None, 0.05, dense_block=False)
    assert sp2.P == 81
    g = torch.randn(3, 70, 70)
    pg = sp2.param_grad(g, sp2.x0, rows)
    assert pg.shape == (3, 81)


def test_refine_loop_accounting_on_a_quadratic():
    """refine()'s control flow on J(x) = 0.5 |x - 1|^2 (gradient exact, one 'solve' per loss and two
    per loss + gradient): the budget is respected per band and the minimiser is approached."""
    target = np.ones(6)
    state = {"calls": 0}

    def evaluate(vec, need_grad, band):
        state["calls"] += 1
        loss = 0.5 * float(np.sum((vec - target) ** 2))
        return (loss, vec - target, 2) if need_grad else (loss, None, 1)

    x, hist, solves = refine_np.refine_loop(np.zeros(6), np.ones(6), lambda v: np.clip(v, -5, 5), evaluate,
                                            (6.0, None), 30, lambda b: None)
    assert solves <= 30 + 2
    assert np.abs(x - target).max() < 1e-6
    assert all(h[3] for h in hist[:2])
