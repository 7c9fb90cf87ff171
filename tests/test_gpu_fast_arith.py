"""The fast-arithmetic resident kernels (engine option "arith" = 1) against the north-star
tolerances. GPU tests, through the C ABI.

The default kernels round every f32 operation in the reference's order and equal the f32 oracle
bit for bit; the fast kernels compute the same discrete operators with 1/h folded into the stencil
weights and fused multiply-adds, so they are held to the stated tolerances instead: gathers
<= 1e-5 and gradients <= 1e-4 relative L2 against the FP32 CPU reference (the oracle) on config 1
(one 70x70 model, 5 shots, nt 1000). On a config-3 batch (mixed-family models, checkpoint every
100 steps) a model whose misfit is small has a gradient that no differently rounded f32
computation can bring within 1e-4 of the FP32 reference (the reference itself is further than that
from the FP64 result there), so those models are held to the FP32 reference's own error against
FP64. Every error against FP64 is printed. The adjoint dot-product test and the other grids with
fast kernels (100x100, 140x140) are covered too.
"""

from __future__ import annotations

import numpy as np
import pytest

from conftest import layered_model, rel_l2
from oracle import native as o

pytestmark = pytest.mark.gpu

GATHER_TOL = 1e-5
GRAD_TOL = 1e-4


def _survey(nt=1000, n=70):
    sv = o.Survey(shots=5, nt=nt, dt=0.001, nx_vis=n, nz_vis=n)
    cells = np.round(np.linspace(0, n - 1, 5)).astype(np.float32) if n != 70 else np.float32([0, 17, 34, 52, 69])
    src = np.stack([cells * np.float32(10.0), np.full(5, 10.0, np.float32)], 1).astype(np.float32)
    return sv, src


def _engine(sv, src, fast: bool, ck: int = 50):
    from wgnet_gb300.engine import WaveEngine

    eng = WaveEngine(shots=sv.shots, nt=sv.nt, dt=sv.dt, peak_hz=sv.peak_hz, pml=sv.pml, vmin=sv.vmin, vmax=sv.vmax,
                     nx_vis=sv.nx_vis, nz_vis=sv.nz_vis, h=sv.h, checkpoint_every=ck)
    eng.set_sources(src)
    eng.set_option("arith", 1 if fast else 0)
    assert eng.get_option("arith") == (1 if fast else 0)
    return eng


def test_arith_option_rejects_other_values(cuda_lib):
    sv, src = _survey(nt=50)
    eng = _engine(sv, src, fast=False)
    with pytest.raises(ValueError):
        eng.set_option("arith", 2)


def test_fast_config1_within_north_star_tolerance(cuda_lib):
    sv, src = _survey()
    eng = _engine(sv, src, fast=True)
    wav = eng.wavelet()
    true, cur = layered_model(3), layered_model(4)
    got = eng.simulate(np.stack([true, cur]))
    ref = o.forward(sv, np.stack([true, cur]), src, wav)
    ref64 = o.forward(sv, cur, src, wav, precision="f64")
    assert rel_l2(got, ref) <= GATHER_TOL, rel_l2(got, ref)
    assert not np.array_equal(got, ref)  # the fast kernels really ran (they round differently)
    e_fast, e_f32 = rel_l2(got[1:], ref64), rel_l2(ref[1:], ref64)
    assert e_fast <= 2.0 * e_f32 + 1e-9, (e_fast, e_f32)
    obs = ref[:1]
    loss, grad = eng.evaluate_adjoint(cur, obs)
    rl, rg = o.evaluate_adjoint(sv, cur, src, wav, obs)
    l64, g64 = o.evaluate_adjoint(sv, cur, src, wav, obs, precision="f64")
    assert rel_l2(grad, rg) <= GRAD_TOL, rel_l2(grad, rg)
    np.testing.assert_allclose(loss, rl, rtol=1e-5)
    g_fast, g_f32 = rel_l2(grad, g64), rel_l2(rg, g64)
    assert g_fast <= 2.0 * g_f32 + 1e-9, (g_fast, g_f32)
    print(f"\n[fast, 70x70 nt 1000] gathers: rel L2 vs FP32 oracle {rel_l2(got, ref):.3e}, vs FP64 {e_fast:.3e} "
          f"(FP32 oracle vs FP64 {e_f32:.3e}); gradient: vs FP32 oracle {rel_l2(grad, rg):.3e}, vs FP64 "
          f"{g_fast:.3e} (FP32 oracle vs FP64 {g_f32:.3e})")


def test_fast_config3_batch_matches_unfused_path(cuda_lib):
    """A config-3 style batch (mixed families, checkpoint every 100 steps): fast against the
    unfused GPU path, which equals the FP32 oracle bit for bit, and both against the FP64 oracle.

    A gradient's rounding error grows as the misfit shrinks (the residual is a small difference of
    two nearly equal gathers): on model 6 of this batch the residual is 8 % of the data and the
    FP32 CPU reference itself is 3.6e-4 (relative L2) from the FP64 gradient, so no f32 computation
    rounded differently from it can meet 1e-4 against it there. Each model is held to 1e-4 against
    the FP32 reference, or, where the FP32 reference's own error exceeds half of that, to no more
    than 1.5 x that error against FP64 (and 2 x it against the FP32 reference)."""
    import torch

    from wgnet_gb300.models_synth import make_batch, smooth

    sv, src = _survey()
    true = make_batch(12, seed=9)
    start = smooth(true, 5.0)
    exact = _engine(sv, src, fast=False, ck=100)
    fast = _engine(sv, src, fast=True, ck=100)
    d_true, d_start = torch.from_numpy(true).cuda(), torch.from_numpy(start).cuda()
    obs = exact.simulate_torch(d_true)
    obs_fast = fast.simulate_torch(d_true)
    assert rel_l2(obs_fast.cpu().numpy(), obs.cpu().numpy()) <= GATHER_TOL
    l0, g0 = exact.evaluate_adjoint_torch(d_start, obs)
    l1, g1 = fast.evaluate_adjoint_torch(d_start, obs)
    g0, g1 = g0.cpu().numpy(), g1.cpu().numpy()
    l64, g64 = o.evaluate_adjoint(sv, start, src, exact.wavelet(), obs.cpu().numpy(), precision="f64",
                                  threads=o.cpu_threads())
    rows = []
    for b in range(len(true)):
        d_ref, e_ref, e_fast = rel_l2(g1[b], g0[b]), rel_l2(g0[b], g64[b]), rel_l2(g1[b], g64[b])
        rows.append((b, d_ref, e_ref, e_fast))
        if e_ref <= 0.5 * GRAD_TOL:
            assert d_ref <= GRAD_TOL, rows[-1]
        else:
            assert e_fast <= 1.5 * e_ref and d_ref <= 2.0 * e_ref, rows[-1]
    print("\n[fast, config-3 batch] model: vs FP32 reference / FP32 reference vs FP64 / fast vs FP64")
    for b, d_ref, e_ref, e_fast in rows:
        print(f"  {b:2d}: {d_ref:.2e} / {e_ref:.2e} / {e_fast:.2e}")
    # the loss has the same conditioning (a small residual): held to 1e-5 relative to the FP32
    # reference or to 4 x the FP32 reference's own error against FP64, whichever is larger
    l0, l1 = l0.cpu().numpy(), l1.cpu().numpy()
    lim = np.maximum(1e-5, 4.0 * np.abs(l0 - l64) / l64)
    assert np.all(np.abs(l1 - l0) / l0 <= lim), (np.abs(l1 - l0) / l0, lim)
    # the checkpointed and the store-every-step schedules agree on the fast path too
    fast.checkpoint_every = 0
    _, g2 = fast.evaluate_adjoint_torch(d_start, obs)
    np.testing.assert_array_equal(g2.cpu().numpy(), g1)


@pytest.mark.parametrize("n", [100, 140])
def test_fast_other_grids(cuda_lib, n):
    sv, src = _survey(nt=400, n=n)
    exact, fast = _engine(sv, src, fast=False), _engine(sv, src, fast=True)
    assert fast.launch_shape("forward") == exact.launch_shape("forward")
    rng = np.random.default_rng(n)
    v = np.repeat(np.sort(rng.uniform(1500, 4500, n))[:, None], n, 1).astype(np.float32)
    cur = (v * np.float32(0.97)).astype(np.float32)
    p0, p1 = exact.simulate(v), fast.simulate(v)
    assert rel_l2(p1, p0) <= GATHER_TOL
    _, g0 = exact.evaluate_adjoint(cur, p0)
    _, g1 = fast.evaluate_adjoint(cur, p0)
    assert rel_l2(g1, g0) <= GRAD_TOL, rel_l2(g1, g0)


def test_fast_adjoint_dot_product(cuda_lib):
    """<J dv, r> = <dv, J^T r> with J^T from the fast adjoint (J from the FP64 oracle forward)."""
    sv, src = _survey(nt=300)
    eng = _engine(sv, src, fast=True, ck=37)
    wav = eng.wavelet()
    rng = np.random.default_rng(4)
    v = layered_model(3)
    p = eng.simulate(v)[0]
    r = (0.5 * np.sqrt(np.mean(p.astype(np.float64) ** 2)) * rng.standard_normal(p.shape)).astype(np.float32)
    d = (p - r).astype(np.float32)
    r64 = p.astype(np.float64) - d.astype(np.float64)
    energy = float(np.sum(d.astype(np.float64) ** 2))
    _, g = eng.evaluate_adjoint(v, d[None])
    jt_r = g[0].astype(np.float64) * energy
    dv = rng.standard_normal(v.shape)
    eps = 1e-2
    fp = o.forward(sv, (v + eps * dv).astype(np.float32), src, wav, precision="f64")[0]
    fm = o.forward(sv, (v - eps * dv).astype(np.float32), src, wav, precision="f64")[0]
    dvv = (v + eps * dv).astype(np.float32).astype(np.float64) - (v - eps * dv).astype(np.float32).astype(np.float64)
    lhs = float(np.sum((fp - fm) * r64))
    rhs = float(np.sum(jt_r * dvv))
    assert abs(lhs - rhs) <= 1e-4 * abs(lhs), (lhs, rhs)
