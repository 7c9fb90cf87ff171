"""Generate fixtures by running the reference's own Python layer (python/wgnet/data.py, physics.py,
render.py, refine.py, fwi_eval.py) unchanged, with `import wave_gauss_rs` resolving to the
oracle-backed restatement of the PyO3 module (oracle/pyo3_standin.py).

    python tests/golden/make_refpy.py /path/to/WGNet

The reference's Python cannot run where the GPU tests run (it is not part of this repository), so
its outputs on fixed inputs are stored here (refpy.npz) and tests/test_gpu_refpy.py runs this
repository's WavePhysics and refine() on the same inputs through the CUDA engine. Cases follow
python/verify.py: the adjoint through the renderer (57-74, 2 shots, nt 501), the band identity
(76-84) and budgeted refinement (107-117, 2 shots, nt 801, 30 solves, bands 10 Hz / full); and
fwi_eval.py's budgeted pixel-grid FWI (32-57, 2 shots, nt 501, 12 solves, bands 8 Hz / full).
"""

from __future__ import annotations

import importlib.util
import sys
import types
from pathlib import Path

import numpy as np
import torch

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]


def load_reference(ref_root: Path) -> dict:
    sys.path.insert(0, str(ROOT))
    from oracle import pyo3_standin

    sys.modules["wave_gauss_rs"] = pyo3_standin
    pkg_dir = ref_root / "python" / "wgnet"
    pkg = types.ModuleType("wgnet")
    pkg.__path__ = [str(pkg_dir)]
    sys.modules["wgnet"] = pkg
    mods = {}
    for name in ("data", "render", "physics", "refine", "igm", "model", "train", "fwi_eval"):
        spec = importlib.util.spec_from_file_location(f"wgnet.{name}", pkg_dir / f"{name}.py")
        mod = importlib.util.module_from_spec(spec)
        sys.modules[f"wgnet.{name}"] = mod
        spec.loader.exec_module(mod)
        mods[name] = mod
    return mods


def random_scene(render, gen: torch.Generator, n_active: int) -> torch.Tensor:
    """A seeded scene in the manner of python/verify.py:34-39."""
    raw = torch.randn(1, render.N_SLOTS, 6, generator=gen) * 0.5
    raw[..., 5] = 0.0
    idx = torch.randperm(render.N_SLOTS, generator=gen)[:n_active]
    raw[0, idx, 5] = torch.randn(n_active, generator=gen) * 1.5
    return render.activate_gaussians(raw)


def main() -> None:
    if len(sys.argv) != 2:
        raise SystemExit("usage: python tests/golden/make_refpy.py <path to the WGNet checkout>")
    m = load_reference(Path(sys.argv[1]))
    render, physics_mod, refine_mod = m["render"], m["physics"], m["refine"]
    out = {}

    # adjoint through the renderer (verify.py:57-74)
    physics = physics_mod.WavePhysics(shots=2, nt=501)
    gen = torch.Generator().manual_seed(2)
    base = torch.full((1, 70, 70), 2.5)
    true_params = random_scene(render, gen, 12)
    init_params = true_params + 0.1 * torch.randn(true_params.shape, generator=gen)
    with torch.no_grad():
        observed = physics.simulate((base + render.render_residual(true_params)).numpy())
        field = (base + render.render_residual(init_params)).numpy()
    losses, grads = physics.loss_and_grad(field, observed)
    out.update(adj_true_params=true_params.numpy(), adj_init_params=init_params.numpy(), adj_observed=observed,
               adj_field=field, adj_losses=losses, adj_grads=grads)

    # band identity (verify.py:76-84), on the same field
    physics.set_band(8.0)
    low = physics.simulate(field)
    out["band_kernel"] = physics.kernel.copy()
    out["band_wavelet"] = physics.engine.wavelet()
    physics.set_band(None)
    full = physics.simulate(field)
    physics.set_band(8.0)
    filtered = physics.bandlimit(full)
    physics.set_band(None)
    out.update(band_low=low, band_full=full, band_filtered=filtered)

    # budgeted refinement (verify.py:107-117)
    physics = physics_mod.WavePhysics(shots=2, nt=801)
    gen = torch.Generator().manual_seed(4)
    base_np = np.full((70, 70), 2.5, np.float32)
    true_params = random_scene(render, gen, 10)
    with torch.no_grad():
        observed = physics.simulate((torch.from_numpy(base_np) + render.render_residual(true_params)).numpy())[0]
    init = true_params.clone()
    init[..., 5] *= 0.5
    res = refine_mod.refine(base_np, init[0].numpy(), observed, physics, budget_solves=30, bands_hz=(10.0, None),
                            device="cpu")
    hist = res.history
    # the 10 Hz band as refine() used it: the wavelet (np.convolve of float32 arrays rounds differently
    # on other CPU architectures, ~1e-6) and the band-limited observed data (torch's conv1d; a FIR
    # summed in another order differs by ~1e-6 of the peak). L-BFGS on this small-misfit problem
    # amplifies such last-bit differences, so the test can install these exact inputs to compare
    # the algorithm itself.
    physics.set_band(10.0)
    out["ref_band10_wavelet"] = physics.engine.wavelet()
    out["ref_band10_observed"] = physics.bandlimit(observed)
    physics.set_band(None)
    out.update(ref_base=base_np, ref_init=init[0].numpy(), ref_observed=observed,
               ref_initial_loss=np.float64(res.initial_loss), ref_final_loss=np.float64(res.final_loss),
               ref_solves=np.int64(res.solves), ref_final_field=res.final_field_km,
               ref_initial_field=res.initial_field_km, ref_gaussians=res.gaussians, ref_coarse=res.coarse_km,
               ref_hist_loss=np.array([h["loss"] for h in hist], np.float64),
               ref_hist_solves=np.array([h["solves"] for h in hist], np.int64),
               ref_hist_accepted=np.array([h["accepted"] for h in hist], bool),
               ref_hist_band=np.array([-1.0 if h["band_hz"] is None else h["band_hz"] for h in hist], np.float64))
    # budgeted pixel-grid FWI (fwi_eval.py:32-57) from a smoothed start
    from scipy.ndimage import gaussian_filter

    physics = physics_mod.WavePhysics(shots=2, nt=501)
    gen = torch.Generator().manual_seed(6)
    with torch.no_grad():
        truth = (torch.full((1, 70, 70), 2.5) + render.render_residual(random_scene(render, gen, 10)))[0].numpy()
    start = gaussian_filter(truth, 4.0, mode="nearest").astype(np.float32)
    observed = physics.simulate(truth[None])[0]
    final, fhist = m["fwi_eval"].fwi(start, observed, physics, [8.0, None], 12, 1.5)
    physics.set_band(8.0)
    out["fwi_band8_wavelet"] = physics.engine.wavelet()
    out["fwi_band8_observed"] = physics.bandlimit(observed)
    physics.set_band(None)
    out.update(fwi_truth=truth, fwi_start=start, fwi_observed=observed, fwi_final=final,
               fwi_hist_misfit=np.array([h["misfit"] for h in fhist], np.float64),
               fwi_hist_solves=np.array([h["solves"] for h in fhist], np.int64))
    np.savez_compressed(HERE / "refpy.npz", **out)
    print(f"fwi: MAE {np.abs(start - truth).mean() * 1000:.1f} -> {np.abs(final - truth).mean() * 1000:.1f} m/s, "
          f"history {fhist}")
    print(f"refine: {res.initial_loss:.4e} -> {res.final_loss:.4e} in {res.solves} solves, "
          f"{len(hist)} iterations; loss_and_grad {losses}")


if __name__ == "__main__":
    main()
