"""Batched multi-grid data generation on the GPU: the low-pass + decimation kernel, the captured
generation plan (70x70, 100x100 and 140x140 models in one graph launch) and the autotuner, each
compared bit for bit with the oracle (f32 forward, f32 FIR in the kernel's order, float16 cast)."""

from __future__ import annotations

import ctypes

import numpy as np
import pytest

from oracle import native as o
from oracle import physics_np

pytestmark = pytest.mark.gpu


def _decimate_dev(lib, x, taps, center, factor):
    import torch

    xt = torch.tensor(x, device="cuda")
    kt = torch.tensor(taps, device="cuda")
    series, nt, nrec = int(np.prod(x.shape[:-2])), x.shape[-2], x.shape[-1]
    nt_out = -(-nt // factor)
    out = torch.empty(x.shape[:-2] + (nt_out, nrec), device="cuda", dtype=torch.float16)
    rc = lib.wg_lowpass_decimate_f16_dev(ctypes.c_void_p(xt.data_ptr()), ctypes.c_void_p(kt.data_ptr()), len(taps),
                                         center, factor, series, nt, nrec, ctypes.c_void_p(out.data_ptr()), None)
    assert rc == 0
    torch.cuda.synchronize()
    return out.cpu().numpy()


def test_decimate_kernel_bitexact(cuda_lib):
    rng = np.random.default_rng(5)
    x = (rng.standard_normal((3, 5, 1003, 70)) * 30.0).astype(np.float32)
    x[0, 0, 10, 3] = 7.0e4  # overflows float16 after filtering: inf on both sides
    for taps, center, factor in ((physics_np.lowpass_kernel(50.0, 0.001), 15, 4), (np.float32([1.0]), 0, 1),
                                 (physics_np.lowpass_kernel(12.0, 0.001), 0, 8), (np.float32([0.25, 0.75]), 1, 3)):
        got = _decimate_dev(cuda_lib, x, taps, center, factor)
        ref = physics_np.lowpass_decimate_f16(x, taps, center, factor)
        np.testing.assert_array_equal(got.view(np.uint16), ref.view(np.uint16))


def _oracle_gathers(gen, n, vel, taps):
    eng = gen.engines[n]
    sv = o.Survey(shots=eng.shots, nt=eng.nt, dt=eng.dt, peak_hz=eng.peak_hz, pml=eng.pml, vmin=eng.vmin,
                  vmax=eng.vmax, nx_vis=n, nz_vis=n, h=eng.h)
    tr = o.forward(sv, vel, eng.sources(), eng.wavelet())
    return physics_np.lowpass_decimate_f16(tr, taps, len(taps) // 2, gen.factor)


def test_generation_plan_three_grids_bitexact(cuda_lib):
    import torch

    from wgnet_gb300.datagen import GatherGenerator, synthetic_batch

    batch = synthetic_batch(7, seed=11)  # 70: 3 models, 100: 2, 140: 2
    gen = GatherGenerator({n: len(v) for n, v in batch.items()}, nt=240, autotune=False)
    assert gen.kernels_per_launch == 9  # pad + forward + decimate per grid
    np.testing.assert_array_equal(gen.taps, physics_np.lowpass_kernel(50.0, 0.001))
    # the generation-3 kernels compiled for these widths are the defaults
    assert gen.shapes == {70: (2, 704, 10), 100: (4, 672, 10), 140: (6, 640, 12)}
    out = gen.run(batch)
    torch.cuda.synchronize()
    for n, v in batch.items():
        got = out[n].cpu().numpy()
        assert got.shape == (len(v), 5, 60, n)
        ref = _oracle_gathers(gen, n, v, gen.taps)
        np.testing.assert_array_equal(got.view(np.uint16), ref.view(np.uint16), err_msg=f"grid {n}")
        assert np.abs(got.astype(np.float32)).max() > 0


def test_generation_plan_replays_on_new_inputs(cuda_lib):
    import torch

    from wgnet_gb300.datagen import GatherGenerator, synthetic_batch

    gen = GatherGenerator({70: 2, 140: 1}, shots=3, nt=180, autotune=False, cutoff_hz=30.0)
    first = synthetic_batch(3, seed=2, sizes=(70, 140))
    second = synthetic_batch(3, seed=3, sizes=(70, 140))
    a = {n: t.clone() for n, t in gen.run(first).items()}
    b = gen.run(second)
    torch.cuda.synchronize()
    for n in (70, 140):
        assert not torch.equal(a[n], b[n])
        ref = _oracle_gathers(gen, n, second[n], gen.taps)
        np.testing.assert_array_equal(b[n].cpu().numpy().view(np.uint16), ref.view(np.uint16))
    np.testing.assert_array_equal(gen.taps, physics_np.lowpass_kernel(30.0, 0.001))


def test_generation_plan_chunks_inside_the_graph(cuda_lib):
    import torch

    from wgnet_gb300.datagen import GatherGenerator, synthetic_batch

    batch = synthetic_batch(5, seed=4, sizes=(70,))
    per_model = 5 * 200 * 70 * 4
    gen = GatherGenerator({70: 5}, nt=200, autotune=False, workspace_bytes=2 * per_model)
    assert gen.trace_bytes == 2 * per_model and gen.kernels_per_launch == 9  # 3 chunks of <= 2 models
    out = gen.run(batch)[70]
    torch.cuda.synchronize()
    ref = _oracle_gathers(gen, 70, batch[70], gen.taps)
    np.testing.assert_array_equal(out.cpu().numpy().view(np.uint16), ref.view(np.uint16))


def test_autotuner_on_the_gpu(cuda_lib, tmp_path):
    from wgnet_gb300 import autotune
    from wgnet_gb300.engine import WaveEngine

    eng = WaveEngine(shots=5, nt=120, dt=0.001, nx_vis=100, nz_vis=100)
    path = tmp_path / "tune.json"
    got = autotune.tune(eng, models=8, reps=1, path=path)
    assert got["forward"] in eng.shape_candidates("forward")
    assert got["adjoint"] in eng.shape_candidates("adjoint")
    assert eng.launch_shape("forward") == got["forward"]
    cache = autotune.load_cache(path)
    key = autotune.cache_key(autotune.device_tag(), "forward", eng)
    assert tuple(cache[key]["shape"]) == got["forward"]
    assert len(cache[key]["ms"]) == len(eng.shape_candidates("forward"))


@pytest.mark.parametrize("n", [100, 140])
def test_every_shape_bitexact_on_larger_grids(cuda_lib, n):
    """Forward traces and gradients of every compiled launch shape for the 100x100 and 140x140
    surveys (both kernel generations), against the f32 oracle."""
    from conftest import layered_model
    from wgnet_gb300.engine import WaveEngine

    sv = o.Survey(shots=3, nt=150, dt=0.001, nx_vis=n, nz_vis=n)
    eng = WaveEngine(shots=3, nt=150, dt=0.001, nx_vis=n, nz_vis=n)
    src = eng.sources()
    np.testing.assert_array_equal(src, sv.default_sources())
    vel = np.stack([layered_model(21, n, n), layered_model(22, n, n)])
    vel[1, n // 3:n // 2, n // 4:n // 2] = 5300.0  # clamped block
    obs = o.forward(sv, vel * np.float32(0.97), src, eng.wavelet())
    ref_tr = o.forward(sv, vel, src, eng.wavelet())
    ref_loss, ref_grad = o.evaluate_adjoint(sv, vel, src, eng.wavelet(), obs)
    fshapes, ashapes = eng.shape_candidates("forward"), eng.shape_candidates("adjoint")
    assert any(s[0] >= 4 for s in fshapes) and len(ashapes) >= 1
    for shape in fshapes:
        eng.set_launch_shape("forward", shape)
        np.testing.assert_array_equal(eng.simulate(vel), ref_tr, err_msg=f"forward {shape}")
    eng.set_launch_shape("forward", fshapes[0])
    for shape in ashapes:
        eng.set_launch_shape("adjoint", shape)
        for k in (0, 37):
            eng.checkpoint_every = k
            loss, grad = eng.evaluate_adjoint(vel, obs)
            np.testing.assert_array_equal(grad, ref_grad, err_msg=f"adjoint {shape} k={k}")
            np.testing.assert_allclose(loss, ref_loss, rtol=1e-12)
