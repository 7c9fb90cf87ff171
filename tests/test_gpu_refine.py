"""Batched GPU refinement: the FP64 kernels (L-BFGS two-loop direction against the reference's
golden vectors, dot products, misfit), the lockstep batch against the oracle's restatement of
refine()'s control flow driven by the same wave solves, batch == single-model runs, and the
learned-proposal plumbing."""

from __future__ import annotations

import numpy as np
import pytest

from conftest import ROOT
from oracle import refine_np

pytestmark = pytest.mark.gpu

BANDS = (6.0, 9.0, 12.0, None)


def test_lbfgs_direction_kernel_matches_reference_golden(cuda_lib):
    import torch

    from wgnet_gb300.refine import dot, lbfgs_direction

    r = np.load(ROOT / "tests" / "golden" / "refine.npz")
    for c in range(4):
        g = r[f"grad_{c}"]
        s, y = list(r[f"s_{c}"]), list(r[f"y_{c}"])
        m = 8
        P = len(g)
        S = torch.zeros((1, m, P), dtype=torch.float64, device="cuda")
        Y = torch.zeros_like(S)
        rho = torch.zeros((1, m), dtype=torch.float64, device="cuda")
        for j, (a, b) in enumerate(zip(s, y)):
            S[0, j] = torch.from_numpy(a)
            Y[0, j] = torch.from_numpy(b)
            rho[0, j] = 1.0 / float(np.dot(a, b))
        d = lbfgs_direction(torch.from_numpy(g)[None].cuda(), S, Y, rho, torch.tensor([len(s)], device="cuda"))
        np.testing.assert_allclose(d[0].cpu().numpy(), r[f"dir_{c}"], rtol=1e-11, atol=1e-14)
    a = torch.randn((5, 1000), dtype=torch.float64, device="cuda")
    b = torch.randn((5, 1000), dtype=torch.float64, device="cuda")
    np.testing.assert_allclose(dot(a, b).cpu().numpy(), (a * b).sum(1).cpu().numpy(), rtol=1e-12)


def test_misfit_kernel(cuda_lib):
    import ctypes

    import torch

    p = torch.randn((3, 5, 100, 70), device="cuda")
    d = torch.randn((3, 5, 100, 70), device="cuda")
    out = torch.empty(3, dtype=torch.float64, device="cuda")
    assert cuda_lib.wg_misfit_dev(ctypes.c_void_p(p.data_ptr()), ctypes.c_void_p(d.data_ptr()), 3, 35000,
                                  ctypes.c_void_p(out.data_ptr()), None) == 0
    pd, dd = p.double().view(3, -1), d.double().view(3, -1)
    ref = 0.5 * ((pd - dd) ** 2).sum(1) / (dd * dd).sum(1)
    np.testing.assert_allclose(out.cpu().numpy(), ref.cpu().numpy(), rtol=1e-12)


def _setup(n, nt=300, seed=3):
    import torch

    from wgnet_gb300.learned import physics_for, problem

    ph = physics_for((0, 1, 2, 3, 4), nt=nt)
    true, start, obs = problem(n, seed, ph)
    return ph, true, start, obs


def test_lockstep_batch_follows_the_reference_control_flow(cuda_lib):
    import torch

    from wgnet_gb300.refine import Space, refine_batch

    ph, true, start, obs = _setup(1)
    budget = 36
    r = refine_batch(start, obs, ph, budget_solves=budget, bands_hz=BANDS, dense_block=True)
    ours = [(h["band_hz"], h["solves"], h["loss"], h["accepted"]) for h in r["history"][0] if h["kind"] == "lbfgs"]

    sp = Space(start, None, 0.05, True)
    rows = torch.arange(1, device="cuda")
    state = {"obs": obs}

    def set_band(band):
        ph.set_band(band)
        state["obs"] = ph.bandlimit(obs) if band is not None else obs

    def evaluate(vec, need_grad, band):
        import ctypes

        from wgnet_gb300 import _lib

        x = torch.from_numpy(vec)[None].cuda()
        f = sp.field(x, rows)
        if not need_grad:
            pred = ph.simulate(f)
            out = torch.empty(1, dtype=torch.float64, device="cuda")
            _lib.load().wg_misfit_dev(ctypes.c_void_p(pred.data_ptr()), ctypes.c_void_p(state["obs"].data_ptr()), 1,
                                      pred[0].numel(), ctypes.c_void_p(out.data_ptr()), None)
            return float(out[0]), None, 1
        loss, gf = ph.loss_and_grad(f, state["obs"].contiguous())
        return float(loss[0]), sp.param_grad(gf, x, rows)[0].cpu().numpy(), 2

    project = lambda v: sp.project(torch.from_numpy(v)[None].cuda())[0].cpu().numpy()  # noqa: E731
    x, hist, solves = refine_np.refine_loop(sp.x0[0].cpu().numpy(), sp.scales[0].cpu().numpy(), project, evaluate,
                                            BANDS, budget, set_band)
    assert len(ours) == len(hist) and len(hist) > 4
    for a, b in zip(ours, hist):
        assert a[0] == b[0] and a[1] == b[1] and a[3] == b[3], (a, b)
        assert abs(a[2] - b[2]) <= 1e-9 * abs(b[2]), (a, b)
    assert int(r["solves"][0]) == solves
    np.testing.assert_allclose(r["x"][0].cpu().numpy(), x, rtol=0, atol=1e-7)


def test_batch_equals_single_model_runs(cuda_lib):
    from wgnet_gb300.refine import refine_batch

    ph, true, start, obs = _setup(3, seed=9)
    rb = refine_batch(start, obs, ph, budget_solves=24, bands_hz=BANDS, dense_block=True, true_km=true)
    for b in range(3):
        r1 = refine_batch(start[b:b + 1], obs[b:b + 1], ph, budget_solves=24, bands_hz=BANDS, dense_block=True)
        assert int(r1["solves"][0]) == int(rb["solves"][b])
        np.testing.assert_allclose(float(r1["final_loss"][0]), float(rb["final_loss"][b]), rtol=1e-12)
        np.testing.assert_array_equal(r1["final_field_km"][0].cpu().numpy(), rb["final_field_km"][b].cpu().numpy())
    assert all(len([h for h in rb["history"][b] if "mae_km" in h]) == len(rb["history"][b]) for b in range(3))
    assert bool((rb["final_loss"] < rb["initial_loss"]).all())


def test_learned_proposals_are_accepted_only_when_the_misfit_drops(cuda_lib):
    from wgnet_gb300.precond import UpdateNet
    from wgnet_gb300.refine import refine_batch

    ph, true, start, obs = _setup(4, seed=12)
    net = UpdateNet(seed=5)
    r = refine_batch(start, obs, ph, budget_solves=32, bands_hz=BANDS, dense_block=True, proposer=net, true_km=true)
    for b in range(4):
        h = r["history"][b]
        assert int(r["solves"][b]) <= 32 + 2
        for band in BANDS:
            losses = [e["loss"] for e in h if e["band_hz"] == band and e["kind"] in ("lbfgs", "learned")]
            assert all(l1 <= l0 for l0, l1 in zip(losses, losses[1:]))
