"""Parity of the CUDA path with the oracle. GPU tests: everything runs through the C ABI.

The forward and adjoint kernels follow the reference's f32 operation order with no FMA
contraction, so traces, stored terms and gradients are compared bit for bit with the f32
oracle; losses (f64 reductions in a different order) to 1e-12 relative. The benchmark spec's bounds
(gathers <= 1e-5, gradients <= 1e-4 relative L2 vs the FP32 CPU reference) are asserted as well,
and the error against the FP64 oracle is checked against the FP32 oracle's own.
"""

from __future__ import annotations

import numpy as np
import pytest

from conftest import layered_model, rel_l2
from oracle import native as o

pytestmark = pytest.mark.gpu

GATHER_TOL = 1e-5   # relative L2, north star
GRAD_TOL = 1e-4     # relative L2, north star


def small_case(seed=0, shots=3, nt=150, nxv=20, nzv=16, pml=6):
    rng = np.random.default_rng(seed)
    vel = (2000 + 1500 * rng.random((nzv, nxv))).astype(np.float32)
    vel[0, 0] = 900.0
    vel[3, 4] = 5200.0
    src = np.array([[0.0, 10.0], [95.0, 10.0], [190.0, 12.5], [50.0, 30.0]], np.float32)[:shots]
    sv = o.Survey(shots=shots, nt=nt, dt=0.001, nx_vis=nxv, nz_vis=nzv, pml=pml)
    return sv, vel, src


def make_engine(sv: o.Survey, src, **kw):
    from wgnet_gb300.engine import WaveEngine

    eng = WaveEngine(shots=sv.shots, nt=sv.nt, dt=sv.dt, peak_hz=sv.peak_hz, pml=sv.pml, vmin=sv.vmin, vmax=sv.vmax,
                     nx_vis=sv.nx_vis, nz_vis=sv.nz_vis, h=sv.h, **kw)
    eng.set_sources(src)
    return eng


def survey_70x70():
    """70x70, dt = 1 ms, nt = 1000, sources at cells 0, 17, 34, 52, 69, every surface receiver."""
    sv = o.Survey(shots=5, nt=1000, dt=0.001)
    src = np.stack([np.float32([0, 17, 34, 52, 69]) * np.float32(10.0), np.full(5, 10.0, np.float32)], 1)
    return sv, src.astype(np.float32)


def test_forward_bitexact_small(cuda_lib):
    sv, vel, src = small_case()
    eng = make_engine(sv, src)
    wav = eng.wavelet()
    np.testing.assert_array_equal(wav, o.ricker(sv.nt, sv.dt, sv.peak_hz))
    for shape in eng.shape_candidates("forward"):
        eng.set_launch_shape("forward", shape)
        got = eng.simulate(np.stack([vel, vel * np.float32(1.1)]))
        ref = o.forward(sv, np.stack([vel, vel * np.float32(1.1)]), src, wav)
        np.testing.assert_array_equal(got, ref, err_msg=f"shape {shape}")


def test_forward_bitexact_70x70_nt1000(cuda_lib):
    sv, src = survey_70x70()
    eng = make_engine(sv, src)
    vel = np.stack([layered_model(0), layered_model(1)])
    got = eng.simulate(vel)
    ref = o.forward(sv, vel, src, eng.wavelet())
    np.testing.assert_array_equal(got, ref)
    ref64 = o.forward(sv, vel[:1], src, eng.wavelet(), precision="f64")
    err_gpu, err_cpu = rel_l2(got[:1], ref64), rel_l2(ref[:1], ref64)
    assert rel_l2(got, ref) <= GATHER_TOL
    assert err_gpu <= err_cpu * 1.0000001 + 1e-12
    print(f"\n[70x70 nt 1000 forward] rel L2 vs FP32 oracle {rel_l2(got, ref):.3e}, vs FP64 oracle {err_gpu:.3e}")


def test_simulate_shot_cpu_dropin_bitexact(cuda_lib):
    import wave_gauss_rs

    vel = np.full((70, 70), 2500.0, np.float32)
    vel[35:] = 3200.0
    v = vel.reshape(-1)
    for sx, sz in ((0.0, 10.0), (340.0, 10.0), (123.4, 55.5)):
        got = wave_gauss_rs.simulate_shot_cpu(v, 10.0, 0.0005, 400, 20, 1000.0, 5000.0, 15.0, sx, sz)
        ref = o.simulate_shot_cpu(v, 10.0, 0.0005, 400, 20, 1000.0, 5000.0, 15.0, sx, sz)
        np.testing.assert_array_equal(got, ref)


@pytest.mark.parametrize("k", [0, 7, 25, 50, 149, 150])
def test_adjoint_bitexact_small(cuda_lib, k):
    sv, vel, src = small_case(seed=2)
    eng = make_engine(sv, src, checkpoint_every=k)
    wav = eng.wavelet()
    vels = np.stack([vel, vel * np.float32(0.97)])
    obs = o.forward(sv, vels * np.float32(1.04), src, wav)
    loss, grad = eng.evaluate_adjoint(vels, obs)
    rl, rg = o.evaluate_adjoint(sv, vels, src, wav, obs)
    np.testing.assert_array_equal(grad, rg)
    np.testing.assert_allclose(loss, rl, rtol=1e-12, atol=0)


def test_adjoint_all_shapes_agree(cuda_lib):
    sv, vel, src = small_case(seed=4, nxv=24, nzv=30, nt=120)
    eng = make_engine(sv, src, checkpoint_every=40)
    wav = eng.wavelet()
    obs = o.forward(sv, vel * np.float32(1.03), src, wav)
    rl, rg = o.evaluate_adjoint(sv, vel, src, wav, obs)
    shapes = eng.shape_candidates("adjoint")
    assert shapes
    for shape in shapes:
        eng.set_launch_shape("adjoint", shape)
        _, grad = eng.evaluate_adjoint(vel, obs)
        np.testing.assert_array_equal(grad, rg, err_msg=f"shape {shape}")


def test_adjoint_parity_70x70_nt1000(cuda_lib):
    sv, src = survey_70x70()
    eng = make_engine(sv, src, checkpoint_every=50)
    wav = eng.wavelet()
    true = layered_model(3)
    cur = layered_model(4)
    obs = o.forward(sv, true, src, wav)
    loss, grad = eng.evaluate_adjoint(cur, obs)
    rl, rg = o.evaluate_adjoint(sv, cur, src, wav, obs)
    assert rel_l2(grad, rg) <= GRAD_TOL
    np.testing.assert_array_equal(grad, rg)
    np.testing.assert_allclose(loss, rl, rtol=1e-12)
    l64, g64 = o.evaluate_adjoint(sv, cur, src, wav, obs, precision="f64")
    print(f"\n[70x70 nt 1000 gradient] rel L2 vs FP32 oracle {rel_l2(grad, rg):.3e}, vs FP64 oracle {rel_l2(grad, g64):.3e}; "
          f"loss {loss[0]:.6e} (FP64 {l64[0]:.6e})")


def test_batch_equals_individual_models(cuda_lib):
    sv, vel, src = small_case(seed=6)
    eng = make_engine(sv, src, checkpoint_every=30)
    wav = eng.wavelet()
    vels = np.stack([vel * np.float32(s) for s in (0.9, 1.0, 1.1, 1.2)])
    obs = o.forward(sv, vel[None] * np.float32(1.05), src, wav)
    obs = np.repeat(obs, 4, 0)
    loss_b, grad_b = eng.evaluate_adjoint(vels, obs)
    for i in range(4):
        li, gi = eng.evaluate_adjoint(vels[i], obs[i])
        np.testing.assert_array_equal(gi[0], grad_b[i])
        assert li[0] == loss_b[i]


def test_reference_fd_check_on_gpu(cuda_lib):
    """wave_wgpu.rs:1056-1108: Gaussian bumps, 2 shots, nt = 501, central FD with eps = 1 m/s, < 3 %."""
    from wgnet_gb300.engine import WaveEngine

    eng = WaveEngine(shots=2, nt=501, dt=0.0005, peak_hz=15.0, pml=20, vmin=1000.0, vmax=5000.0)
    x = np.arange(70, dtype=np.float32)
    xx, zz = np.meshgrid(x, x)
    g1 = np.exp(-((xx - 8.0) ** 2 + (zz - 9.0) ** 2) / 50.0)
    g2 = np.exp(-((xx - 56.0) ** 2 + (zz - 10.0) ** 2) / 50.0)
    true = (2500.0 + 320.0 * g1 - 230.0 * g2).astype(np.float32)
    cur = (2500.0 + 180.0 * g1 - 120.0 * g2).astype(np.float32)
    d = (np.exp(-((xx - 7.0) ** 2 + (zz - 7.0) ** 2) / 150.0)
         + 0.3 * np.exp(-((xx - 58.0) ** 2 + (zz - 12.0) ** 2) / 100.0)).astype(np.float32)
    obs = eng.simulate(true)
    _, grad = eng.evaluate_adjoint(cur, obs)
    lp, _ = eng.evaluate_adjoint(cur + d, obs)
    lm, _ = eng.evaluate_adjoint(cur - d, obs)
    fd = (float(np.float32(lp[0])) - float(np.float32(lm[0]))) / 2.0
    adj = float(np.sum(grad[0].astype(np.float64) * d))
    assert abs(fd - adj) / max(abs(fd), 1e-12) < 0.03, (fd, adj)


def test_gpu_gradient_vs_fp64_finite_differences(cuda_lib):
    """FD with eps = 1e-3 m/s on the FP64 oracle vs the GPU adjoint."""
    sv, vel, src = small_case(seed=7, nt=200)
    vel = np.clip(vel, 1500, 4500).astype(np.float32)
    eng = make_engine(sv, src, checkpoint_every=25)
    wav = eng.wavelet()
    obs = o.forward(sv, vel * np.float32(1.03), src, wav)
    _, grad = eng.evaluate_adjoint(vel, obs)
    d = np.random.default_rng(1).standard_normal(vel.shape)
    vp = (vel + 1e-3 * d).astype(np.float32)
    vm = (vel - 1e-3 * d).astype(np.float32)
    lp, _ = o.evaluate_adjoint(sv, vp, src, wav, obs, precision="f64")
    lm, _ = o.evaluate_adjoint(sv, vm, src, wav, obs, precision="f64")
    fd = lp[0] - lm[0]
    adj = float(np.sum(grad[0].astype(np.float64) * (vp.astype(np.float64) - vm.astype(np.float64))))
    assert abs(fd - adj) <= 1e-3 * abs(fd), (fd, adj)


def test_zero_energy_raises(cuda_lib):
    sv, vel, src = small_case()
    eng = make_engine(sv, src)
    with pytest.raises(RuntimeError, match="zero energy"):
        eng.evaluate_adjoint(vel, np.zeros((1, sv.shots, sv.nt, sv.n_receivers), np.float32))


def test_dropin_engine_api(cuda_lib):
    import wave_gauss_rs

    e = wave_gauss_rs.PyWaveEngine(shots=2, nt=300, dt=0.001)
    assert (e.shots, e.nt, e.nrec) == (2, 300, 70)
    np.testing.assert_array_equal(e.sources(), np.float32([[0, 10], [690, 10]]))
    with pytest.raises(ValueError):
        e.set_sources(np.zeros((3, 2), np.float32))
    with pytest.raises(ValueError):
        e.set_wavelet(np.zeros(299, np.float32))
    with pytest.raises(ValueError):
        e.simulate(np.zeros(4899, np.float32))
    with pytest.raises(ValueError):
        e.evaluate_adjoint(np.full(4900, 2000, np.float32), np.ones(10, np.float32))
    v = layered_model(5).reshape(-1)
    tr = e.simulate(v)
    assert tr.shape == (2, 300, 70) and tr.dtype == np.float32
    loss, g = e.evaluate_adjoint(v, (tr * np.float32(1.1)).reshape(-1))
    assert isinstance(loss, float) and g.shape == (70, 70)
    w = e.wavelet()
    e.set_wavelet(w * np.float32(2.0))
    tr2 = e.simulate(v)
    # linear in the wavelet up to f32 rounding (the oracle shows the same last-place deviations)
    np.testing.assert_allclose(tr2, 2 * tr, rtol=1e-4, atol=1e-9)
    sv = o.Survey(shots=2, nt=300, dt=0.001)
    np.testing.assert_array_equal(tr2, o.forward(sv, v.reshape(70, 70), e.sources(), w * np.float32(2.0))[0])
    e.set_sources(np.float32([[100, 20], [300, 30]]))
    np.testing.assert_array_equal(e.sources(), np.float32([[100, 20], [300, 30]]))


def test_renderer_matches_reference_golden(cuda_lib):
    import torch

    from conftest import ROOT
    from wgnet_gb300.render import render_residual

    g = np.load(ROOT / "tests" / "golden" / "render.npz")
    p = torch.tensor(g["params"], dtype=torch.float32, device="cuda", requires_grad=True)
    field = render_residual(p)
    np.testing.assert_allclose(field.detach().cpu().numpy(), g["field"], rtol=0, atol=2e-5 * np.abs(g["field"]).max())
    (grad,) = torch.autograd.grad((field * torch.tensor(g["cot"], dtype=torch.float32, device="cuda")).sum(), p)
    assert rel_l2(grad.cpu().numpy(), g["grad"]) < 1e-5


def test_bandlimit_matches_reference_golden(cuda_lib):
    import torch

    from conftest import ROOT
    from wgnet_gb300.physics import bandlimit_torch, lowpass_kernel

    p = np.load(ROOT / "tests" / "golden" / "physics.npz")
    x = torch.tensor(p["bandlimit_in"], device="cuda")
    for f in (6.0, 12.0):
        y = bandlimit_torch(x, torch.from_numpy(lowpass_kernel(f, 0.001))).cpu().numpy()
        np.testing.assert_allclose(y, p[f"bandlimit_{f}"], rtol=0, atol=1e-6)


def test_waveloss_autograd(cuda_lib):
    import torch

    from wgnet_gb300.physics import WaveLoss

    sv, vel, src = small_case(seed=9)
    eng = make_engine(sv, src, checkpoint_every=50)
    obs = o.forward(sv, vel[None] * np.float32(1.05), src, eng.wavelet())
    f = torch.tensor(vel[None] / 1000.0, device="cuda", requires_grad=True)
    loss = WaveLoss.apply(f, torch.tensor(obs, device="cuda"), eng)
    (3.0 * loss.sum()).backward()
    _, g = eng.evaluate_adjoint((f.detach() * 1000.0).cpu().numpy(), obs)
    np.testing.assert_allclose(f.grad.cpu().numpy(), 3.0 * 1000.0 * g, rtol=1e-6)


def test_every_forward_shape_bitexact_70x70(cuda_lib):
    """Each compiled forward launch shape that fits 70x70 (both kernel generations)."""
    sv = o.Survey(shots=3, nt=260, dt=0.001)
    src = np.float32([[0.0, 10.0], [333.3, 10.0], [685.0, 47.5]])
    eng = make_engine(sv, src)
    wav = eng.wavelet()
    vel = np.stack([layered_model(21), layered_model(22)])
    vel[1, 30:40, 5:60] = 900.0  # clamped patch
    ref = o.forward(sv, vel, src, wav)
    shapes = eng.shape_candidates("forward")
    assert len(shapes) >= 3
    for shape in shapes:
        eng.set_launch_shape("forward", shape)
        np.testing.assert_array_equal(eng.simulate(vel), ref, err_msg=f"shape {shape}")


@pytest.mark.parametrize("k", [0, 37])
def test_gradient_with_every_forward_shape_70x70(cuda_lib, k):
    sv = o.Survey(shots=2, nt=240, dt=0.001)
    src = np.float32([[120.0, 10.0], [545.5, 12.0]])
    eng = make_engine(sv, src, checkpoint_every=k)
    wav = eng.wavelet()
    cur = layered_model(31)
    obs = o.forward(sv, layered_model(32), src, wav)
    rl, rg = o.evaluate_adjoint(sv, cur, src, wav, obs)
    for shape in eng.shape_candidates("forward"):
        eng.set_launch_shape("forward", shape)
        loss, grad = eng.evaluate_adjoint(cur, obs)
        np.testing.assert_array_equal(grad, rg, err_msg=f"shape {shape}")
        np.testing.assert_allclose(loss, rl, rtol=1e-12)


@pytest.mark.parametrize("k", [0, 45])
def test_every_adjoint_shape_bitexact_70x70(cuda_lib, k):
    """Each compiled adjoint launch shape that fits 70x70 (both kernel generations)."""
    sv = o.Survey(shots=3, nt=220, dt=0.001)
    src = np.float32([[0.0, 10.0], [351.5, 25.0], [690.0, 10.0]])
    eng = make_engine(sv, src, checkpoint_every=k)
    wav = eng.wavelet()
    cur = np.stack([layered_model(41), layered_model(42)])
    cur[0, 10:20, 30:50] = 5500.0  # clamped patch: zero gradient there
    obs = o.forward(sv, np.stack([layered_model(43), layered_model(44)]), src, wav)
    rl, rg = o.evaluate_adjoint(sv, cur, src, wav, obs)
    shapes = eng.shape_candidates("adjoint")
    assert len(shapes) >= 3
    for pref in (0, 1):
        eng.set_option("adjoint_prefetch", pref)
        for shape in shapes:
            eng.set_launch_shape("adjoint", shape)
            loss, grad = eng.evaluate_adjoint(cur, obs)
            np.testing.assert_array_equal(grad, rg, err_msg=f"shape {shape} prefetch {pref}")
            np.testing.assert_allclose(loss, rl, rtol=1e-12)


def smooth_model(nz: int, nx: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    zz = np.arange(nz, dtype=np.float32)[:, None]
    xx = np.arange(nx, dtype=np.float32)[None, :]
    v = 1800.0 + 2400.0 * zz / nz + 300.0 * np.sin(xx / 7.0 + rng.random()) * np.cos(zz / 5.0)
    return v.astype(np.float32)


@pytest.mark.parametrize("nxv,nzv", [(100, 100), (140, 140), (70, 50)])
def test_every_shape_gradient_bitexact_other_grids(cuda_lib, nxv, nzv):
    """Each compiled forward and adjoint launch shape that fits the 100x100 and 140x140 grids of
    the data-generation batch and a 70-wide grid whose rows do not split evenly into segments."""
    sv = o.Survey(shots=2, nt=160, dt=0.001, nx_vis=nxv, nz_vis=nzv)
    src = np.float32([[0.0, 10.0], [(nxv - 1) * 5.0 + 2.5, 15.0]])
    eng = make_engine(sv, src, checkpoint_every=50)
    wav = eng.wavelet()
    cur = np.stack([smooth_model(nzv, nxv, 1), smooth_model(nzv, nxv, 2)])
    obs = o.forward(sv, np.stack([smooth_model(nzv, nxv, 3), smooth_model(nzv, nxv, 4)]), src, wav)
    rl, rg = o.evaluate_adjoint(sv, cur, src, wav, obs)
    fshapes, ashapes = eng.shape_candidates("forward"), eng.shape_candidates("adjoint")
    assert fshapes and ashapes
    for shape in ashapes:
        eng.set_launch_shape("adjoint", shape)
        loss, grad = eng.evaluate_adjoint(cur, obs)
        np.testing.assert_array_equal(grad, rg, err_msg=f"adjoint shape {shape}")
        np.testing.assert_allclose(loss, rl, rtol=1e-12)
    for shape in fshapes:
        eng.set_launch_shape("forward", shape)
        loss, grad = eng.evaluate_adjoint(cur, obs)
        np.testing.assert_array_equal(grad, rg, err_msg=f"forward shape {shape}")


def test_non_finite_inputs_follow_the_reference(cuda_lib):
    """Velocities go through Rust's f32::clamp (wave_wgpu.rs:714-734): a NaN cell stays NaN and
    spreads through the wavefield, +-inf cells clamp to vmax / vmin with a zero clamp mask (no
    gradient there); observed data whose energy is NaN fail the reference's `energy > 0` check
    (wave_wgpu.rs:853), like zero energy. Traces and gradients equal the oracle's, NaNs included."""
    sv, vel, src = small_case(seed=8, shots=2, nt=120)
    eng = make_engine(sv, src, checkpoint_every=40)
    wav = eng.wavelet()
    inf = vel.copy()
    inf[5, 7], inf[9, 2] = np.inf, -np.inf
    nan = vel.copy()
    nan[6, 10] = np.nan
    models = np.stack([inf, nan])
    got = eng.simulate(models)
    ref = o.forward(sv, models, src, wav)
    np.testing.assert_array_equal(got, ref)
    assert np.isfinite(got[0]).all() and np.isnan(got[1]).any()
    obs = o.forward(sv, np.stack([vel, vel]) * np.float32(1.02), src, wav)
    loss, grad = eng.evaluate_adjoint(models, obs)
    rl, rg = o.evaluate_adjoint(sv, models, src, wav, obs)
    np.testing.assert_array_equal(grad, rg)
    np.testing.assert_array_equal(loss, rl)
    assert grad[0, 5, 7] == 0.0 and grad[0, 9, 2] == 0.0 and np.isfinite(grad[0]).all()
    bad = obs.copy()
    bad[0, 0, 3, 4] = np.nan
    with pytest.raises(RuntimeError, match="zero energy"):
        eng.evaluate_adjoint(np.stack([vel, vel]), bad)


def test_empty_batch_is_an_argument_error(cuda_lib):
    sv, vel, src = small_case(seed=9, shots=2, nt=60)
    eng = make_engine(sv, src)
    empty = np.zeros((0, sv.nz_vis, sv.nx_vis), np.float32)
    with pytest.raises(ValueError):
        eng.simulate(empty)
    with pytest.raises(ValueError):
        eng.evaluate_adjoint(empty, np.zeros((0, sv.shots, sv.nt, sv.n_receivers), np.float32))


def test_reference_default_engine_through_the_dropin_module(cuda_lib):
    """The reference's own engine configuration: `PyWaveEngine()` with its defaults (5 shots,
    nt 2001, dt 0.5 ms, 15 Hz, pml 20; lib.rs:51-72, data.py:32-33) through the drop-in module,
    with its default sources and every surface receiver: traces, loss and gradient equal the
    oracle's bit for bit."""
    import wave_gauss_rs

    e = wave_gauss_rs.PyWaveEngine()
    assert (e.shots, e.nt, e.nrec) == (5, 2001, 70)
    sv = o.Survey()  # the same defaults
    src = e.sources()
    wav = e.wavelet()
    np.testing.assert_array_equal(wav, o.ricker(sv.nt, sv.dt, sv.peak_hz))
    true = layered_model(21)
    cur = layered_model(22)
    tr = e.simulate(true.reshape(-1))
    ref = o.forward(sv, true, src, wav)[0]
    np.testing.assert_array_equal(tr, ref)
    loss, grad = e.evaluate_adjoint(cur.reshape(-1), tr.reshape(-1))
    rl, rg = o.evaluate_adjoint(sv, cur, src, wav, ref[None])
    np.testing.assert_array_equal(grad, rg[0])
    # the engine returns the loss as f32 (wave_wgpu.rs:965-985: the f64 sum rounded once)
    assert isinstance(loss, float) and loss == float(np.float32(rl[0]))
