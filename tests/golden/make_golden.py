"""Generate golden fixtures by running the reference's own Python code.

Run from the repository root in an environment where the WGNet reference checkout is available:

    python tests/golden/make_golden.py /path/to/WGNet

It imports the reference modules directly from `python/wgnet/` (render.py, physics.py, refine.py).
physics.py and refine.py import `wgnet.data`, which needs the compiled `wave_gauss_rs` extension;
a stub `wgnet.data` providing only the constants they use stands in for it, so only pure
numpy/torch code of the reference runs. Outputs (small .npz files) are written next to this script.
"""

from __future__ import annotations

import importlib.util
import sys
import types
from pathlib import Path

import numpy as np
import torch

HERE = Path(__file__).resolve().parent


def load_reference(ref_root: Path):
    pkg_dir = ref_root / "python" / "wgnet"
    pkg = types.ModuleType("wgnet")
    pkg.__path__ = [str(pkg_dir)]
    sys.modules["wgnet"] = pkg
    data = types.ModuleType("wgnet.data")
    # constants of python/wgnet/data.py:20-29
    data.N, data.H, data.SHOTS, data.NT, data.DT, data.PEAK_HZ = 70, 10.0, 5, 2001, 0.0005, 15.0

    def make_engine(*_a, **_k):
        raise RuntimeError("the wgpu engine is not available")

    data.make_engine = make_engine
    sys.modules["wgnet.data"] = data
    mods = {}
    for name in ("render", "physics", "refine"):
        spec = importlib.util.spec_from_file_location(f"wgnet.{name}", pkg_dir / f"{name}.py")
        mod = importlib.util.module_from_spec(spec)
        sys.modules[f"wgnet.{name}"] = mod
        spec.loader.exec_module(mod)
        mods[name] = mod
    return mods


def random_scene(render, gen: torch.Generator, n_active: int) -> torch.Tensor:
    """Seeded scene in the manner of python/verify.py:34-39."""
    raw = torch.randn(1, render.N_SLOTS, 6, generator=gen) * 0.5
    raw[..., 5] = 0.0
    idx = torch.randperm(render.N_SLOTS, generator=gen)[:n_active]
    raw[0, idx, 5] = torch.randn(n_active, generator=gen) * 1.5
    return render.activate_gaussians(raw)


def make_render(render) -> None:
    gen = torch.Generator().manual_seed(1)
    scenes = [random_scene(render, gen, n) for n in (40, 12, 300)]
    # a dense scene: every slot active with random amplitudes
    raw = torch.randn(1, render.N_SLOTS, 6, generator=gen) * 0.7
    scenes.append(render.activate_gaussians(raw))
    params = torch.cat(scenes, 0).double()
    p = params.clone().requires_grad_(True)
    field = render.render_residual(p)
    cot = torch.randn(field.shape, generator=gen, dtype=torch.float64)
    (g,) = torch.autograd.grad((field * cot).sum(), p)
    raw_act = torch.randn(2, 17, 6, generator=gen) * 2.0
    act = render.activate_gaussians(raw_act)
    wild = torch.randn(2, 17, 6, generator=gen, dtype=torch.float64) * 4.0
    clamped = render.clamp_gaussians(wild)
    anchors = render.slot_anchors()
    flat, centers, valid = render.slot_windows()
    np.savez_compressed(
        HERE / "render.npz",
        params=params.numpy(), field=field.detach().numpy(), cot=cot.numpy(), grad=g.numpy(),
        raw_act=raw_act.numpy(), act=act.numpy(), wild=wild.numpy(), clamped=clamped.numpy(),
        anchors=anchors.numpy(), win_flat=flat.numpy().astype(np.int32), win_valid=valid.numpy().astype(np.uint8),
    )


def make_physics(physics) -> None:
    out = {}
    for dt in (0.0005, 0.001):
        for f in (5.0, 6.0, 8.0, 9.0, 10.0, 12.0, 15.0):
            out[f"lowpass_{dt}_{f}"] = physics.lowpass_kernel(f, dt)
    # bandlimit: WavePhysics.bandlimit with a set kernel, on seeded traces [2, 3, nt, nrec]
    rng = np.random.default_rng(7)
    traces = rng.standard_normal((2, 3, 300, 7)).astype(np.float32)
    wp = physics.WavePhysics.__new__(physics.WavePhysics)
    for f in (6.0, 12.0):
        wp.kernel = physics.lowpass_kernel(f, 0.001)
        out[f"bandlimit_in"] = traces
        out[f"bandlimit_{f}"] = wp.bandlimit(traces)
    # set_band: the wavelet convolution (physics.py:43-46) of a Ricker stand-in
    full = rng.standard_normal(1000).astype(np.float32)
    out["setband_full"] = full
    for f in (6.0, 9.0, 12.0):
        k = physics.lowpass_kernel(f, 0.001)
        out[f"setband_{f}"] = np.convolve(full, k, mode="full")[:1000].astype(np.float32)
    np.savez_compressed(HERE / "physics.npz", **out)


def make_metrics(render) -> None:
    """field_metrics (render.py:140-152) on seeded smooth random fields."""
    gen = torch.Generator().manual_seed(5)
    target = 1.5 + 3.0 * torch.rand(4, 70, 70, generator=gen)
    target = torch.nn.functional.avg_pool2d(target[:, None], 5, stride=1, padding=2)[:, 0]
    pred = target + 0.1 * torch.randn(4, 70, 70, generator=gen)
    m = render.field_metrics(pred, target)
    # The same formula in f64: the reference's float32 window cast to f64 for this call only, so
    # that the fixture pins the metric itself and not float32 rounding (its variance terms cancel).
    window = render._gaussian_window
    render._gaussian_window = lambda *a, **k: window(*a, **k).double()
    try:
        ssim64 = render.ssim(pred.double(), target.double())
    finally:
        render._gaussian_window = window
    np.savez(HERE / "metrics.npz", pred=pred.numpy(), target=target.numpy(), ssim64=ssim64.numpy(),
             **{k: v.numpy() for k, v in m.items()})


def make_refine(refine) -> None:
    rng = np.random.default_rng(11)
    out = {}
    for case, m in enumerate((0, 1, 3, 8)):
        n = 81 + 6 * 5
        grad = rng.standard_normal(n)
        s_hist = [rng.standard_normal(n) * 0.1 for _ in range(m)]
        y_hist = [s + 0.05 * rng.standard_normal(n) for s in s_hist]
        rho = [1.0 / float(np.dot(s, y)) for s, y in zip(s_hist, y_hist)]
        d = refine._lbfgs_direction(grad, s_hist, y_hist, rho)
        out[f"grad_{case}"] = grad
        out[f"s_{case}"] = np.array(s_hist).reshape(m, n)
        out[f"y_{case}"] = np.array(y_hist).reshape(m, n)
        out[f"dir_{case}"] = d
    np.savez_compressed(HERE / "refine.npz", **out)


def main() -> None:
    if len(sys.argv) != 2:
        raise SystemExit("usage: python tests/golden/make_golden.py <path to the WGNet checkout>")
    mods = load_reference(Path(sys.argv[1]))
    torch.manual_seed(0)
    make_render(mods["render"])
    make_physics(mods["physics"])
    make_refine(mods["refine"])
    make_metrics(mods["render"])
    for p in sorted(HERE.glob("*.npz")):
        print(p.name, p.stat().st_size)


if __name__ == "__main__":
    main()
