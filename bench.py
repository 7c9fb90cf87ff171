"""Benchmark: forward + exact adjoint gradients of the 4th-order C-PML acoustic solver.

Workload (one "step"): the misfit gradient of a batch of 256 mixed-family 70 x 70 velocity models
(10 m cells, pml 20 -> 114 x 114 padded), 5 surface shots at cells 0/17/34/52/69, 70 receivers,
15 Hz Ricker, dt = 1 ms, nt = 1000, wavefield checkpoints every 100 steps with recomputation
(k = 25 and 50 with --checkpoint).
Observed data come from the true models; the gradient is taken at their 5-cell Gaussian-smoothed
versions. Data are synthetic (seeded), in the shapes and value ranges of the reference's setting.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0). `value` = gradients/s with inputs resident in HBM; `e2e` = the same
through the C ABI's host entry point (host->device copy of velocities and observed data and
device->host copy of losses and gradients inside the timed region).
"""

from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "gradients/s (forward + exact adjoint, 70x70, 5 shots, nt=1000)"
UNIT = "gradients/s"
MODELS = 256
SHOTS = 5
NT = 1000
DT = 0.001
NX = 70
PML = 20
CK = 100
UPDATED_CELLS = (NX + 2 * (PML + 2) - 4) ** 2  # 110 x 110 cells updated per step
FLOPS_PER_CELL_UPDATE = 48.0  # average over interior / one-PML-axis / two-PML-axes cells at pml 20
# DRAM bytes per (unit, step) measured with ncu on the small case (32 models, nt 200: the full
# 256-model launch is too large for a multi-pass capture), scaled by unit-steps to a full launch
MEASURED_TRAFFIC_PER_UNIT_STEP = {"adjoint": (813.12e6 + 9.30e6) / 16000, "recompute": (69.86e6 + 735.81e6) / 16000}
# Counters of the same small-case captures (ncu --set full), per kernel: thread-instructions per
# updated cell and step, issue slots busy, L1/shared throughput, shared-memory bank-conflict share.
NCU_SMALL_CASE = {
    "adjoint": {"thread_instructions_per_cell_update": 106.7, "issue_active_pct": 62.7, "l1_shared_pct": 68.0,
                "bank_conflict_pct_of_shared_wavefronts": 1.7, "warps_active_pct": 34.3},
    "recompute": {"thread_instructions_per_cell_update": 71.7, "issue_active_pct": 64.9, "l1_shared_pct": 52.0,
                  "bank_conflict_pct_of_shared_wavefronts": 2.5, "warps_active_pct": 34.3},
}


def flops_per_cell_update(n_vis: int, pml: int = PML) -> float:
    """Algorithmic flops per updated cell and step of the forward (lib.rs:158-205; add, sub, mul 1,
    FMA 2): 24 in the interior, 54 with one C-PML axis, 84 with two, averaged over the updated
    square grid whose C-PML strips are pml + 2 cells wide on each side (48.0 at 70 x 70, pml 20)."""
    n = n_vis + 2 * (pml + 2) - 4
    p = 2 * (pml + 2)
    return (84.0 * p * p + 54.0 * 2 * p * (n - p) + 24.0 * (n - p) ** 2) / (n * n)


FP32_LANES_PER_SM = 128  # FP32 lanes of a Blackwell SM (two dies x 76 SMs on GB300)


def clocks_sampler(stop: threading.Event, out: list):
    q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")
    try:
        p = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits", "-lms", "200"],
                             stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
    except Exception:
        return
    dev = os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0]
    try:
        while not stop.is_set():
            line = p.stdout.readline()
            if not line:
                break
            out.append([x.strip() for x in line.split(",")])
    finally:
        p.terminate()


def summarize_clocks(rows):
    if not rows:
        return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
    sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
    mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    reasons = sorted({names[i] for r in rows for i in range(4) if len(r) > 5 + i and r[5 + i] == "Active"})
    return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
            "reasons": reasons, "samples": len(rows)}


def workload(models: int, seed: int = 0):
    from wgnet_gb300 import models_synth

    true = models_synth.make_batch(models, seed)
    start = models_synth.smooth(true, 5.0)
    src = np.stack([np.float32([0, 17, 34, 52, 69]) * np.float32(10.0), np.full(5, 10.0, np.float32)], 1)
    return true, start, src.astype(np.float32)


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def cpu_baseline(start, obs, src, cores: int, sample_models: int):
    from oracle import native as o

    sv = o.Survey(shots=SHOTS, nt=NT, dt=DT, pml=PML)
    wav = o.ricker(NT, DT, 15.0)
    m = sample_models
    t0 = time.perf_counter()
    o.gradients_parallel(sv, start[:m], src, wav, obs[:m], threads=cores)
    dt = time.perf_counter() - t0
    return m / dt, dt


# One renderer evaluation (render.py:86-109): 2 subtractions, the rotation (4 mul, 2 add), the
# scales (2 mul), u^2 + v^2 (2 mul, 1 add), the -1/2 (1 mul) and the accumulation (1 mul, 1 add),
# plus one exp (an ex2 on the SFU)
RENDER_FLOPS_PER_EVAL = 17
SFU_EX2_PER_SM_CLOCK = 16


def renderer_rate(sms: int, sm_mhz: float, batch: int = MODELS, reps: int = 20) -> dict:
    """The Gaussian renderer on the gradient workload's batch (`batch` models x 1225 slots, 25 x 25
    windows): forward, and forward + backward, timed with CUDA events. Evaluations are the in-grid
    window pixels (the reference also evaluates the out-of-grid ones, on a spare pixel); each costs
    RENDER_FLOPS_PER_EVAL FP32 operations and one exp, so both the FP32 pipe and the SFU bound it."""
    import torch

    from wgnet_gb300 import _lib
    from wgnet_gb300 import render as R

    gen = torch.Generator().manual_seed(1)
    raw = torch.randn(batch, R.N_SLOTS, 6, generator=gen) * 0.5
    raw[..., 5] = torch.randn(batch, R.N_SLOTS, generator=gen) * 1.5
    params = R.activate_gaussians(raw).cuda().contiguous().requires_grad_(True)
    cot = torch.randn(batch, R.GRID, R.GRID, device="cuda")
    for _ in range(3):
        torch.autograd.grad(R.render_residual(params), params, cot)
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    _lib.launch_count(reset=True)
    with torch.no_grad():
        ev[0].record()
        for _ in range(reps):
            R.render_residual(params)
        ev[1].record()
    for _ in range(reps):
        torch.autograd.grad(R.render_residual(params), params, cot)
    ev[2].record()
    torch.cuda.synchronize()
    launches = _lib.launch_count()
    fwd_ms = ev[0].elapsed_time(ev[1]) / reps
    both_ms = ev[1].elapsed_time(ev[2]) / reps
    evals = float(R.slot_windows()[2].sum()) * batch
    fp32_peak = sms * FP32_LANES_PER_SM * 2 * sm_mhz * 1e6 / 1e12
    sfu_peak = sms * SFU_EX2_PER_SM_CLOCK * sm_mhz * 1e6
    achieved = evals * RENDER_FLOPS_PER_EVAL / (fwd_ms / 1000.0) / 1e12
    return {"batch": batch, "evaluations_per_forward": evals,
            "evaluations_reference_counts": float(batch * R.N_SLOTS * R.WIN_SIDE * R.WIN_SIDE),
            "forward_ms": fwd_ms, "forward_backward_ms": both_ms, "launches_per_rep": launches / (2 * reps),
            "roofline": {"kernel": "render_fwd", "bound": "fp32", "achieved": achieved, "peak": fp32_peak,
                         "unit": "TFLOP/s", "frac": achieved / fp32_peak,
                         "flops_per_evaluation": RENDER_FLOPS_PER_EVAL,
                         "sfu": {"achieved_exp_per_s": evals / (fwd_ms / 1000.0), "peak": sfu_peak,
                                 "frac": evals / (fwd_ms / 1000.0) / sfu_peak,
                                 "peak_source": f"computed: {sms} SMs x {SFU_EX2_PER_SM_CLOCK} ex2 per clock x "
                                                f"{sm_mhz:.0f} MHz"}}}


def learned_refinement_brief(models: int = 32) -> dict:
    """Learned-plus-exact refinement against plain projected L-BFGS, the solve-count half of the
    metric: `models` held-out seeded 70x70 models, 5 shots, budget 160 solves, bands 6 / 9 / 12 Hz /
    full, from a 5-cell and from an 8-cell smoothed start, with the committed update network."""
    from wgnet_gb300.learned import evaluate
    from wgnet_gb300.precond import UpdateNet

    net = UpdateNet.load(Path(__file__).resolve().parent / "wgnet_gb300" / "weights" / "update_net.npz")
    out = {}
    for sigma, seed in ((5.0, 777), (8.0, 888)):
        r = evaluate(net, models, seed=seed, shots=5, budget=160, sigma=sigma)
        out[f"start_smoothed_{int(sigma)}_cells"] = {k: v for k, v in r.items() if k != "per_model"}
    return out


def gradient_config(models: int, nt: int, checkpoint: int, arith: str = "exact") -> dict:
    """The gradient workload's `config`, the same for this repository's arm and the reference arm."""
    return {"workload": f"gradient batch: {models} mixed-family 70x70 models x 5 shots, nt={nt}, dt=1ms, "
                        f"pml 20, checkpoint every {checkpoint} steps", "models_per_step": models,
            "shots": SHOTS, "nt": nt, "checkpoint_every": checkpoint,
            "l2": "inputs larger than L2 (observed 358 MB, checkpoints ~10 GB per step)", "arith": arith,
            "passband": "full band (a 6/9/12/15 Hz passband changes the wavelet and the observed data, not the work of "
                        "a gradient)"}


def run_reference(args):
    """The reference's CPU solver path (C++ restatement of geology-core + the engine's adjoint;
    the Rust crate itself cannot be built here) on all host cores."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    from oracle import native as o

    cores = o.cpu_threads()
    sample = max(cores, 1)
    true, start, src = workload(sample)
    sv = o.Survey(shots=SHOTS, nt=NT, dt=DT, pml=PML)
    wav = o.ricker(NT, DT, 15.0)
    obs = o.forward(sv, true, src, wav, threads=cores)
    for _ in range(args.warmup):
        o.gradients_parallel(sv, start[:sample], src, wav, obs[:sample], threads=cores)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        o.gradients_parallel(sv, start[:sample], src, wav, obs[:sample], threads=cores)
        times.append(time.perf_counter() - t0)
    tot = sum(times)
    value = sample * args.steps / tot
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * tot / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": gradient_config(args.models, NT, args.checkpoint),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"each step {sample} of the batch's {args.models} gradients (the first models of "
                                   f"the same seeded batch), one model per thread; the CPU port keeps every step's "
                                   f"gradient term in memory instead of checkpointing"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


DATAGEN_METRIC = "gathers/s (batched forward data generation, 70/100/140 grids, 5 shots, nt=1000, FP16 x4-decimated)"
DATAGEN_UNIT = "gathers/s"


def run_datagen(args):
    """Batched data generation: `args.models` seeded mixed-family models, grids 70/100/140 round-robin,
    5 shots, nt = 1000, dt = 1 ms, simulated, low-passed and decimated to FP16 [N, 5, 250, n] by one
    CUDA graph launch per step."""
    import torch

    from wgnet_gb300 import _lib
    from wgnet_gb300.datagen import GatherGenerator, round_robin_counts, synthetic_batch

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    total = args.models
    counts = round_robin_counts(total)
    batch = synthetic_batch(total, seed=0)
    gen = GatherGenerator(counts, nt=args.nt)
    gen.run(batch)
    torch.cuda.synchronize()
    for _ in range(args.warmup):
        gen.launch()
    torch.cuda.synchronize()
    stop = threading.Event()
    clk = []
    th = threading.Thread(target=clocks_sampler, args=(stop, clk), daemon=True)
    th.start()
    time.sleep(0.3)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    for _ in range(args.steps):
        gen.launch()
    ev1.record()
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    stop.set()
    th.join(timeout=2)
    value = total * args.steps / (ms / 1000.0)
    # e2e: pinned host velocities -> device, graph, FP16 gathers -> pinned host
    h_in = {n: torch.from_numpy(v).pin_memory() for n, v in batch.items()}
    h_out = {n: torch.empty(g.shape, dtype=g.dtype).pin_memory() for n, g in gen.gathers.items()}

    def host_step():
        gen.load(h_in)
        gen.launch()
        for n, g in gen.gathers.items():
            h_out[n].copy_(g, non_blocking=True)
        torch.cuda.synchronize()

    host_step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        host_step()
    e2e_s = time.perf_counter() - t0
    e2e = total * args.steps / e2e_s
    h2d = sum(t.numel() * 4 for t in h_in.values())
    d2h = sum(t.numel() * 2 for t in h_out.values())
    ok = all(torch.isfinite(h_out[n].float()).all().item() for n in h_out)
    # per-grid forward kernel time, measured eagerly with the engine's event timer on the same batch
    per_grid = {}
    flops = 0.0
    for n, eng in gen.engines.items():
        d = torch.from_numpy(batch[n]).cuda()
        eng.simulate_torch(d)
        torch.cuda.synchronize()
        eng.profile(True)
        eng.simulate_torch(d)
        torch.cuda.synchronize()
        fms, fl = eng.profile_read()["forward"]
        eng.profile(False)
        upd = (eng.nx - 4) * (eng.nz - 4)
        f = counts[n] * SHOTS * args.nt * upd * flops_per_cell_update(n)
        flops += f
        per_grid[str(n)] = {"models": counts[n], "forward_ms": fms, "launches": fl, "launch_shape": gen.shapes[n],
                            "gcell_updates_per_s": counts[n] * SHOTS * args.nt * upd / (fms / 1000.0) / 1e9}
    dom = max(per_grid, key=lambda k: per_grid[k]["forward_ms"])
    dn = int(dom)
    dom_ms = per_grid[dom]["forward_ms"]
    dom_bytes = counts[dn] * SHOTS * (args.nt * dn * 4 + (dn + 44) ** 2 * 4)
    dom_flops = counts[dn] * SHOTS * args.nt * (dn + 40) ** 2 * flops_per_cell_update(dn)
    hbm_peak, peak_kind = measured_peaks()
    props = torch.cuda.get_device_properties(0)
    clocks = summarize_clocks(clk)
    sm_mhz = clocks["sm_mhz"] or 2070.0
    fp32_peak = props.multi_processor_count * FP32_LANES_PER_SM * 2 * sm_mhz * 1e6 / 1e12
    line = {
        "metric": DATAGEN_METRIC, "value": value, "unit": DATAGEN_UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 (FP16 output)", "data": "synthetic (seeded mixed-family models)",
        "config": datagen_config(total, args.nt),
        "launch": {"counts": counts, "kernels_per_graph": gen.kernels_per_launch},
        "e2e": {"value": e2e, "unit": DATAGEN_UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": gen.kernels_per_launch * args.steps, "outputs_finite": ok,
        "per_grid": per_grid,
        # resident forward: the wavefield stays in shared memory, so the FP32 pipe bounds it
        "roofline": {"kernel": f"forward {dom}x{dom}", "bound": "fp32",
                     "achieved": dom_flops / (dom_ms / 1000.0) / 1e12, "peak": fp32_peak, "unit": "TFLOP/s",
                     "frac": dom_flops / (dom_ms / 1000.0) / 1e12 / fp32_peak,
                     "peak_source": f"computed: {props.multi_processor_count} SMs x {FP32_LANES_PER_SM} FP32 lanes x "
                                    f"2 flop x {sm_mhz:.0f} MHz (median SM clock of this run)",
                     "traffic": None, "flops_per_launch": dom_flops, "avg_launch_ms": dom_ms,
                     "hbm": {"achieved": dom_bytes / (dom_ms / 1000.0) / 1e9, "peak": hbm_peak, "unit": "GB/s",
                             "peak_source": peak_kind, "bytes_per_launch": dom_bytes}},
        "fp32_whole_graph_tflops": flops / (ms / args.steps / 1000.0) / 1e12,
        "clocks": clocks,
    }
    if not args.no_cpu_baseline:
        from oracle import native as o

        cores = o.cpu_threads()
        sample = synthetic_batch(48 * max(1, cores // 3), seed=0)  # about 10 s of CPU work
        t0 = time.perf_counter()
        m = 0
        for n, v in sample.items():
            sv = o.Survey(shots=SHOTS, nt=args.nt, dt=DT, pml=PML, nx_vis=n, nz_vis=n)
            o.forward(sv, v, sv.default_sources(), o.ricker(args.nt, DT, 15.0), threads=cores)
            m += len(v)
        secs = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": m / secs, "unit": DATAGEN_UNIT, "cores": cores, "kind": "port",
                                "sample": f"{m} models of the mix ({secs:.1f} s), forward only, one shot per thread"}
    print(json.dumps(line), flush=True)
    gen.close()
    return 0


LARGE_METRIC = "Gcell-updates/s (forward + exact adjoint, 800x300 at 5 m, 40 shots, nt=4000, streamed)"
LARGE_UNIT = "Gcell-updates/s"


def large_workload(nt: int, shots: int = 40):
    """One 800 x 300 model (5 m cells: padded 844 x 344), dt = 0.5 ms, `shots` evenly spaced surface
    shots, 800 receivers; observed data from the true layered/curved/faulted/blob model, gradient
    at its 5-cell smoothed version."""
    from wgnet_gb300 import models_synth

    true = models_synth.make_batch(1, seed=4, nz=300, nx=800, families=("fault",))
    start = models_synth.smooth(true, 5.0)
    return true, start


def large_bytes_per_cell_update(nx: int, nz: int, pml: int, shots: int) -> tuple[float, float]:
    """Algorithmic DRAM bytes per updated cell and step of the streamed forward (with stored
    gradient terms) and adjoint kernels: wavefield reads/writes, stored terms, gradient
    accumulator, velocity (shared by the shots), and 16 B per C-PML axis (psi and zeta)."""
    region = pml + 6
    fx = 2 * (region - 2) / (nx - 4)
    fz = 2 * (region - 2) / (nz - 4)
    pml_b = 16.0 * (fx + fz)
    fwd = 4 + 4 + 4 + 4 / shots + 4 + pml_b          # u, u_prev, u_next, v, stored
    adj = 4 + 8 + 4 + 8 + 4 / shots + pml_b          # lambda, lambda_prev r/w, stored, gacc r/w, v
    return fwd, adj


def measure_large(nt: int, shots: int, steps: int, warmup: int) -> dict:
    """The large survey's gradients on the streamed path: `steps` gradients timed with device-resident
    inputs (CUDA events, clocks sampled), then `steps` through the host C ABI entry point."""
    import torch

    from wgnet_gb300 import _lib
    from wgnet_gb300.engine import WaveEngine

    true, start = large_workload(nt, shots)
    eng = WaveEngine(shots=shots, nt=nt, dt=0.0005, peak_hz=15.0, pml=PML, vmin=1000.0, vmax=5000.0, nx_vis=800,
                     nz_vis=300, h=5.0)
    assert eng.get_option("streamed") == 1
    dev = torch.device("cuda", torch.cuda.current_device())
    d_true = torch.from_numpy(true).to(dev)
    d_obs = eng.simulate_torch(d_true)
    d_start = torch.from_numpy(start).to(dev)
    for _ in range(warmup):
        eng.evaluate_adjoint_torch(d_start, d_obs)
    torch.cuda.synchronize()
    stop = threading.Event()
    clk = []
    th = threading.Thread(target=clocks_sampler, args=(stop, clk), daemon=True)
    th.start()
    time.sleep(0.3)
    eng.profile(True)
    _lib.launch_count(reset=True)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    for _ in range(steps):
        loss, grad = eng.evaluate_adjoint_torch(d_start, d_obs, check_status=False)
    ev1.record()
    torch.cuda.synchronize()
    launches = _lib.launch_count()
    ms = ev0.elapsed_time(ev1)
    eng.status("timed gradients")
    prof = eng.profile_read()
    eng.profile(False)
    stop.set()
    th.join(timeout=2)
    assert torch.isfinite(loss).all() and torch.isfinite(grad).all()
    upd = (eng.nx - 4) * (eng.nz - 4)
    cell_updates = 2.0 * upd * nt * shots  # forward + adjoint per gradient
    value = cell_updates * steps / (ms / 1000.0) / 1e9
    # simulate alone (forward only), one step per launch and temporally blocked (4 steps per launch)
    sim_ms = {}
    for tb in (0, 1):
        eng.set_option("temporal_block", tb)
        eng.simulate_torch(d_true, check_status=False)  # first use allocates the blocked kernels' state
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        eng.simulate_torch(d_true, check_status=False)
        e1.record()
        torch.cuda.synchronize()
        eng.status("simulate")
        sim_ms[tb] = e0.elapsed_time(e1)
    eng.set_option("temporal_block", 0)
    # e2e: host velocity and observed data in, loss and gradient out, through the C ABI host entry
    h_vel = torch.from_numpy(start).pin_memory()
    h_obs = d_obs.cpu().pin_memory()
    h_loss = torch.empty(1, dtype=torch.float64).pin_memory()
    h_grad = torch.empty((1, 300, 800), dtype=torch.float32).pin_memory()
    lib = _lib.load()

    def host_step():
        _lib.check(lib.wg_evaluate_adjoint(eng._h, h_vel.data_ptr(), h_obs.data_ptr(), 1, h_loss.data_ptr(),
                                           h_grad.data_ptr()))

    host_step()
    t0 = time.perf_counter()
    for _ in range(steps):
        host_step()
    e2e_s = time.perf_counter() - t0
    e2e = cell_updates * steps / e2e_s / 1e9
    bf, ba = large_bytes_per_cell_update(eng.nx, eng.nz, PML, shots)
    fms, fn = prof["forward"]
    ams, an = prof["adjoint"]
    per_launch = upd * shots  # cell-updates per step (the adjoint runs one launch per step)
    dms = ams / max(an, 1) / nt
    achieved = per_launch * ba / (dms / 1000.0) / 1e9
    hbm_peak, peak_kind = measured_peaks()
    fwd_step_ms = fms / max(fn, 1) / nt
    eng.close()
    return {
        "metric": LARGE_METRIC, "value": value, "unit": LARGE_UNIT, "n_gpus": 1, "steps": steps,
        "warmup": warmup, "ms_per_step": ms / steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded faulted layered model, smoothed start)",
        "config": large_config(nt, shots),
        "gradients_per_s": steps / (ms / 1000.0),
        "simulate": {f"temporal_block_{tb}": {"ms": t, "gcell_updates_per_s": upd * nt * shots / (t / 1000.0) / 1e9}
                     for tb, t in sim_ms.items()},
        "e2e": {"value": e2e, "unit": LARGE_UNIT, "h2d_bytes_per_step": h_vel.numel() * 4 + h_obs.numel() * 4,
                "d2h_bytes_per_step": 8 + h_grad.numel() * 4},
        "gpu_launches": launches,
        "kernels_ms": {"forward": {"total_ms": fms, "steps": nt * max(fn, 1), "ms_per_step": fwd_step_ms},
                       "adjoint": {"total_ms": ams, "steps": nt * max(an, 1), "ms_per_step": dms}},
        "roofline": {"kernel": "adjoint step", "bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved / hbm_peak, "peak_source": peak_kind, "traffic": None,
                     "bytes_per_cell_update": {"forward_per_step_kernel": bf, "adjoint": ba},
                     "avg_launch_ms": dms, "bytes_per_launch": per_launch * ba,
                     "forward_fp32": {"ms_per_step": fwd_step_ms,
                                      "gcell_updates_per_s": per_launch / (fwd_step_ms / 1000.0) / 1e9}},
        "clocks": summarize_clocks(clk),
    }


def large_config(nt: int, shots: int) -> dict:
    """The large survey's `config`, the same for this repository's arm and the reference arm."""
    return {"workload": f"large survey: 800x300 cells at 5 m (padded 844x344), {shots} shots, 800 receivers, "
                        f"dt=0.5ms, nt={nt}, forward + exact adjoint gradient, streamed path",
            "checkpointing": "every step's gradient term stored in HBM when it fits (auto)",
            "temporal_block": "off (one step per launch); `simulate` also times the engine option",
            "l2": "inputs larger than L2 (wavefields ~93 MB + stored terms ~186 GB per gradient)"}


def run_large(args):
    import torch

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    line = measure_large(args.nt, args.shots, args.steps, args.warmup)
    if not args.no_cpu_baseline:
        true, start = large_workload(args.nt, args.shots)
        v, cores, sample = large_cpu_rate(true, start)
        line["cpu_baseline"] = {"value": v, "unit": LARGE_UNIT, "cores": cores, "kind": "port", "sample": sample}
    print(json.dumps(line), flush=True)
    return 0


def large_cpu_rate(true, start, nt_sample: int = 400):
    """The oracle's forward + adjoint (store-all, f32) of one shot per host thread over a 400-step
    record of the large survey (the rate per cell-update does not depend on the record length),
    repeated until about 10 s of CPU work."""
    from oracle import native as o

    cores = o.cpu_threads()
    sv = o.Survey(shots=cores, nt=nt_sample, dt=0.0005, h=5.0, nx_vis=800, nz_vis=300, pml=PML)
    src = sv.default_sources()
    wav = o.ricker(nt_sample, 0.0005, 15.0)
    obs = o.forward(sv, true, src, wav, threads=cores)
    t0 = time.perf_counter()
    reps = 0
    while reps == 0 or time.perf_counter() - t0 < 10.0:
        o.evaluate_adjoint(sv, start, src, wav, obs, threads=cores)
        reps += 1
    secs = time.perf_counter() - t0
    upd = (sv.nx - 4) * (sv.nz - 4)
    return (2.0 * upd * nt_sample * cores * reps / secs / 1e9, cores,
            f"{reps} x {cores} shots x {nt_sample} steps of the survey ({secs:.1f} s), forward + adjoint, "
            "one shot per thread")


def run_reference_large(args):
    """The reference's CPU solver path (C++ restatement) on a bounded sample of the large survey."""
    true, start = large_workload(args.nt, args.shots)
    times = []
    for i in range(args.warmup + args.steps):
        v, cores, sample = large_cpu_rate(true, start)
        if i >= args.warmup:
            times.append(v)
    value = sum(times) / len(times)
    print(json.dumps({"impl": "reference", "metric": LARGE_METRIC, "value": value, "unit": LARGE_UNIT,
                      "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": None,
                      "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                      "data": "synthetic", "config": large_config(args.nt, args.shots),
                      "cpu_baseline": {"value": value, "unit": LARGE_UNIT, "cores": cores, "kind": "port",
                                       "sample": f"each step {sample}"},
                      "e2e": {"value": value, "unit": LARGE_UNIT, "h2d_bytes_per_step": 0,
                              "d2h_bytes_per_step": 0}}), flush=True)
    return 0


def run_train(args):
    """Learned update network: training throughput (samples/s) of `UpdateNet.train_step` on batches
    of 32 synthetic 70x70 samples, and the tensor-core GEMM of one 64 -> 64 3x3 convolution layer
    (M = 32 x 4900 pixels, N = 64, K = 576) timed alone against the measured bf16 peak."""
    import ctypes

    import torch

    from wgnet_gb300 import _lib
    from wgnet_gb300.models_synth import make_batch, smooth
    from wgnet_gb300.precond import UpdateNet

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    B = 32
    v = make_batch(B, seed=3) / 1000.0
    s0 = smooth(v, 5.0)
    vel = torch.from_numpy(s0.astype(np.float32)).cuda()
    grad = torch.randn((B, 70, 70), device="cuda") * 0.01
    band = torch.tensor([i % 4 for i in range(B)], dtype=torch.int32, device="cuda")
    target = torch.from_numpy((v - s0).astype(np.float32)).cuda()
    net = UpdateNet(seed=0)
    for _ in range(args.warmup):
        net.train_step(vel, grad, band, target, lr=1e-4)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    _lib.launch_count(reset=True)
    ev0.record()
    for _ in range(args.steps):
        net.train_step(vel, grad, band, target, lr=1e-4)
    ev1.record()
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / args.steps
    launches = _lib.launch_count() // max(args.steps, 1)
    # one convolution GEMM alone
    lib = _lib.load()
    M, N, K = B * 4900, 64, 576
    a = torch.randn((M, K), device="cuda").to(torch.bfloat16)
    b = torch.randn((N, K), device="cuda").to(torch.bfloat16)
    d = torch.empty((M, N), device="cuda")
    st = torch.zeros(4, dtype=torch.int32, device="cuda")

    def gemm():
        _lib.check(lib.wg_gemm_bf16_dev(ctypes.c_void_p(a.data_ptr()), ctypes.c_void_p(b.data_ptr()),
                                        ctypes.c_void_p(d.data_ptr()), M, N, K, 1, ctypes.c_void_p(st.data_ptr()),
                                        ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))

    for _ in range(5):
        gemm()
    torch.cuda.synchronize()
    reps = 50
    ev0.record()
    for _ in range(reps):
        gemm()
    ev1.record()
    torch.cuda.synchronize()
    gms = ev0.elapsed_time(ev1) / reps
    tflops = 2.0 * M * N * K / (gms / 1000.0) / 1e12
    # with N = 64 output channels the GEMM reads its im2col operand once: 52 flops per byte, below
    # the ridge point, so the HBM roofline bounds it (algorithmic bytes: A, B read, D written)
    gemm_bytes = M * K * 2 + N * K * 2 + M * N * 4
    hbm_peak, peak_kind = measured_peaks()
    bf16_peak = None
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        bf16_peak = float(json.loads(p.read_text()).get("bf16_tflops", 0.0)) or None
    line = {"metric": "update-network training samples/s (70x70, batch 32)", "value": B / (ms / 1000.0),
            "unit": "samples/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "bf16 weights, f32 accumulate",
            "data": "synthetic", "config": {"workload": "UpdateNet.train_step, batch 32, 447,552 parameters",
                                           "batch": B},
            "gpu_launches": launches,
            "roofline": {"kernel": "gemm_bf16_kernel (conv 64->64, M 156800, N 64, K 576)", "bound": "hbm",
                         "achieved": gemm_bytes / (gms / 1000.0) / 1e9, "peak": hbm_peak, "unit": "GB/s",
                         "frac": gemm_bytes / (gms / 1000.0) / 1e9 / hbm_peak, "peak_source": peak_kind,
                         "traffic": None, "bytes_per_launch": gemm_bytes, "avg_launch_ms": gms},
            "tensor": {"achieved_tflops": tflops, "bf16_peak_tflops": bf16_peak,
                       "frac": (tflops / bf16_peak) if bf16_peak else None,
                       "flops_per_byte": 2.0 * M * N * K / gemm_bytes}}
    print(json.dumps(line), flush=True)
    return 0


def datagen_config(models: int, nt: int) -> dict:
    """The generation workload's `config`, the same for this repository's arm and the reference arm."""
    return {"workload": f"batched generation: {models} models round-robin over 70x70/100x100/140x140, 5 shots, "
                        f"nt={nt}, dt=1ms, low-pass + x4 decimation to FP16, one CUDA graph launch",
            "l2": "inputs and outputs larger than L2 (f32 traces ~8 GB per step)"}


def run_reference_datagen(args):
    """The reference's CPU forward (C++ restatement) on a bounded sample of the generation mix."""
    from oracle import native as o
    from wgnet_gb300.datagen import synthetic_batch

    cores = o.cpu_threads()
    sample = synthetic_batch(3 * max(1, cores // 3), seed=0)
    times = []
    m = sum(len(v) for v in sample.values())
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        for n, v in sample.items():
            sv = o.Survey(shots=SHOTS, nt=args.nt, dt=DT, pml=PML, nx_vis=n, nz_vis=n)
            o.forward(sv, v, sv.default_sources(), o.ricker(args.nt, DT, 15.0), threads=cores)
        if i >= args.warmup:
            times.append(time.perf_counter() - t0)
    value = m * len(times) / sum(times)
    print(json.dumps({"impl": "reference", "metric": DATAGEN_METRIC, "value": value, "unit": DATAGEN_UNIT,
                      "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
                      "ms_per_step": 1000.0 * sum(times) / len(times), "higher_is_better": True, "scaling": "weak",
                      "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                      "config": datagen_config(args.models, args.nt),
                      "cpu_baseline": {"value": value, "unit": DATAGEN_UNIT, "cores": cores, "kind": "port",
                                       "sample": f"each step {m} models of the same mix, forward in f32 without the "
                                                 f"FP16 decimation, one shot per thread"},
                      "e2e": {"value": value, "unit": DATAGEN_UNIT, "h2d_bytes_per_step": 0,
                              "d2h_bytes_per_step": 0}}), flush=True)
    return 0


def fast_arith_rate(args, eng, lib, d_start, d_obs, h_vel, h_obs, h_loss, h_grad, models, dist, dev, world, tune_it):
    """The same gradient batch with the fast-arithmetic forward (engine option arith = 1: fused,
    reassociated stencils; the adjoint keeps the reference order), timed the same way. Its results
    are not bit-identical to the reference: gathers agree to <= 1e-5 and gradients to <= 1e-4
    relative L2 on config 1; on a model with a small misfit the gradient agrees with the FP64
    result as well as the FP32 reference does (tests/test_gpu_fast_arith.py)."""
    import torch

    from wgnet_gb300 import _lib, replicas

    eng.set_option("arith", 1)
    if tune_it:
        from wgnet_gb300.autotune import tune

        tune(eng)
    for _ in range(args.warmup):
        eng.evaluate_adjoint_torch(d_start, d_obs, check_status=False)
    torch.cuda.synchronize()
    replicas.barrier(dist)
    lib.wg_profile(eng._h, 1)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    for _ in range(args.steps):
        eng.evaluate_adjoint_torch(d_start, d_obs, check_status=False)
    ev1.record()
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    eng.status("timed gradients (fast arithmetic)")
    kms = (ctypes.c_double * 4)()
    kn = (ctypes.c_longlong * 4)()
    lib.wg_profile_read(eng._h, kms, kn, 4)
    lib.wg_profile(eng._h, 0)
    ms = replicas.max_over_ranks(ms, dist, dev)
    value = replicas.aggregate_rate(models, args.steps, world, ms)

    def host_step():
        _lib.check(lib.wg_evaluate_adjoint(eng._h, h_vel.data_ptr(), h_obs.data_ptr(), models, h_loss.data_ptr(),
                                           h_grad.data_ptr()))

    host_step()
    replicas.barrier(dist)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        host_step()
    e2e_s = replicas.max_over_ranks(time.perf_counter() - t0, dist, dev)
    eng.set_option("arith", 0)
    names = ["forward", "recompute", "adjoint"]
    return {"value": value, "unit": UNIT, "ms_per_step": ms / args.steps,
            "e2e": {"value": replicas.aggregate_rate(models, args.steps, world, e2e_s * 1000.0), "unit": UNIT},
            "kernels_ms": {names[k]: {"total_ms": kms[k], "launches": int(kn[k])} for k in range(3)},
            "launch_shape": {"forward": eng.launch_shape("forward"), "adjoint": eng.launch_shape("adjoint")},
            "accuracy": "not bit-identical: gathers <= 1e-5, gradients <= 1e-4 rel L2 vs the FP32 reference on "
                        "config 1; small-misfit models as close to FP64 as the FP32 reference"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--models", type=int, default=MODELS)
    ap.add_argument("--checkpoint", type=int, default=CK)
    ap.add_argument("--nt", type=int, default=NT, help="time steps (profiling runs use a short record)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="keep the engine's default launch shapes")
    ap.add_argument("--no-large", action="store_true",
                    help="skip the short measurement of the 800x300 streamed survey in the default run")
    ap.add_argument("--no-learned", action="store_true",
                    help="skip the short learned-versus-plain refinement comparison in the default run")
    ap.add_argument("--no-fast", action="store_true",
                    help="skip the secondary measurement with the fast-arithmetic forward (arith 1)")
    ap.add_argument("--arith", default="exact", choices=["exact", "fast"],
                    help="exact: the reference's f32 operation order (bit-identical results); fast: fused, "
                         "reassociated stencils (within the stated f32 tolerances)")
    ap.add_argument("--workload", default="gradient", choices=["gradient", "datagen", "large", "train"],
                    help="gradient: the 256-model misfit-gradient batch (default); datagen: batched generation; "
                         "large: the 800x300 40-shot survey on the streamed path")
    ap.add_argument("--shots", type=int, default=40, help="shots of the large survey")
    args = ap.parse_args()
    if args.workload == "train":
        return run_train(args)
    if args.workload == "large":
        if args.nt == NT:
            args.nt = 4000
        return run_reference_large(args) if args.impl == "reference" else run_large(args)
    if args.workload == "datagen":
        if args.models == MODELS:
            args.models = 4096
        if args.impl == "reference":
            return run_reference_datagen(args)
        return run_datagen(args)
    if args.impl == "reference":
        return run_reference(args)
    nt = args.nt

    import torch

    from wgnet_gb300 import replicas

    rank, world, local = replicas.env()
    torch.cuda.set_device(local)
    dist = replicas.init("nccl")

    from wgnet_gb300 import _lib
    from wgnet_gb300.engine import WaveEngine

    lib = _lib.load()
    M = args.models
    true, start, src = workload(M, seed=replicas.rank_seed(0, rank))
    eng = WaveEngine(shots=SHOTS, nt=nt, dt=DT, peak_hz=15.0, pml=PML, vmin=1000.0, vmax=5000.0,
                     checkpoint_every=args.checkpoint)
    eng.set_sources(src)
    eng.set_option("arith", 1 if args.arith == "fast" else 0)
    tuned = None
    if not args.no_autotune:
        from wgnet_gb300.autotune import tune

        tuned = tune(eng)  # launch shapes timed per kernel (cached per GPU and survey)
    dev = torch.device("cuda", local)
    d_true = torch.from_numpy(true).to(dev)
    d_obs = eng.simulate_torch(d_true)
    d_start = torch.from_numpy(start).to(dev)
    torch.cuda.synchronize()

    def step():
        # asynchronous on the stream; the device status is read once after the timed region
        return eng.evaluate_adjoint_torch(d_start, d_obs, check_status=False)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()

    # timed region: device-resident inputs
    stop = threading.Event()
    clk = []
    th = threading.Thread(target=clocks_sampler, args=(stop, clk), daemon=True)
    th.start()
    time.sleep(0.3)
    replicas.barrier(dist)
    torch.cuda.synchronize()
    lib.wg_profile(eng._h, 1)
    _lib.launch_count(reset=True)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    for _ in range(args.steps):
        loss, grad = step()
    ev1.record()
    torch.cuda.synchronize()
    launches = _lib.launch_count()
    ms = ev0.elapsed_time(ev1)
    eng.status("timed gradients")
    kms = (ctypes.c_double * 4)()
    kn = (ctypes.c_longlong * 4)()
    lib.wg_profile_read(eng._h, kms, kn, 4)
    lib.wg_profile(eng._h, 0)
    stop.set()
    th.join(timeout=2)
    replicas.barrier(dist)
    ms = replicas.max_over_ranks(ms, dist, dev)
    value = replicas.aggregate_rate(M, args.steps, world, ms)
    ms_step = ms / args.steps
    assert torch.isfinite(loss).all() and torch.isfinite(grad).all()

    # e2e: host pinned buffers through the C ABI's host entry point
    h_vel = torch.from_numpy(start).pin_memory()
    h_obs = d_obs.cpu().pin_memory()
    h_loss = torch.empty(M, dtype=torch.float64).pin_memory()
    h_grad = torch.empty((M, NX, NX), dtype=torch.float32).pin_memory()

    def host_step():
        _lib.check(lib.wg_evaluate_adjoint(eng._h, h_vel.data_ptr(), h_obs.data_ptr(), M, h_loss.data_ptr(),
                                           h_grad.data_ptr()))

    host_step()
    replicas.barrier(dist)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        host_step()
    e2e_s = time.perf_counter() - t0
    replicas.barrier(dist)
    e2e_s = replicas.max_over_ranks(e2e_s, dist, dev)
    e2e = replicas.aggregate_rate(M, args.steps, world, e2e_s * 1000.0)
    h2d = h_vel.numel() * 4 + h_obs.numel() * 4
    d2h = h_loss.numel() * 8 + h_grad.numel() * 4

    # roofline of the dominant kernel (live CUDA-event timings of every launch in the timed region)
    names = ["forward", "recompute", "adjoint", "aux"]
    dom = max(range(3), key=lambda k: kms[k])
    units = M * SHOTS
    seg = args.checkpoint if 0 < args.checkpoint < nt else nt
    steps_per_launch = {0: nt, 1: seg, 2: seg}[dom]
    # algorithmic HBM bytes per launch of the dominant kernel
    if dom == 2:  # adjoint: read stored terms of every updated cell and step, residuals; state in/out
        per = units * steps_per_launch * (UPDATED_CELLS * 4 + 70 * 4)
    elif dom == 1:  # recompute: write stored terms
        per = units * steps_per_launch * UPDATED_CELLS * 4
    else:  # forward: traces
        per = units * nt * 70 * 4
    avg_ms = kms[dom] / max(kn[dom], 1)
    hbm_peak, peak_kind = measured_peaks()
    achieved = per / (avg_ms / 1000.0) / 1e9
    flops_launch = units * steps_per_launch * UPDATED_CELLS * FLOPS_PER_CELL_UPDATE
    fp32_tflops = flops_launch / (avg_ms / 1000.0) / 1e12
    cells_per_s = M * SHOTS * nt * UPDATED_CELLS * 2 / (ms_step / 1000.0)
    clocks = summarize_clocks(clk)
    props = torch.cuda.get_device_properties(dev)
    sm_mhz = clocks["sm_mhz"] or 2070.0
    fp32_peak = props.multi_processor_count * FP32_LANES_PER_SM * 2 * sm_mhz * 1e6 / 1e12
    traffic = MEASURED_TRAFFIC_PER_UNIT_STEP.get(names[dom], 0.0) * units * steps_per_launch or None

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded mixed-family models: flat, curved, faulted, blob inclusions)",
        "config": gradient_config(M, nt, args.checkpoint, args.arith),
        "launch": {"shape": {"forward": eng.launch_shape("forward"), "adjoint": eng.launch_shape("adjoint")},
                   "autotuned": tuned is not None},
        "gcell_updates_per_s": cells_per_s / 1e9,
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": launches,
        "kernels_ms": {names[k]: {"total_ms": kms[k], "launches": int(kn[k])} for k in range(3)},
        # The resident 70x70 kernels keep the wavefield in shared memory: FP32-pipe bound (shared
        # memory the second bound); HBM carries only the stored gradient terms and the gathers.
        "roofline": {"kernel": names[dom], "bound": "fp32", "achieved": fp32_tflops, "peak": fp32_peak,
                     "unit": "TFLOP/s", "frac": fp32_tflops / fp32_peak,
                     "peak_source": f"computed: {props.multi_processor_count} SMs x {FP32_LANES_PER_SM} FP32 lanes x "
                                    f"2 flop x {sm_mhz:.0f} MHz (median SM clock of this run's clocks record)",
                     "flops_per_launch": flops_launch, "flops_per_cell_update": FLOPS_PER_CELL_UPDATE,
                     "avg_launch_ms": avg_ms, "traffic": traffic,
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of a 32-model nt-200 capture, "
                                       "scaled by unit-steps",
                     "hbm": {"achieved": achieved, "peak": hbm_peak, "unit": "GB/s", "frac": achieved / hbm_peak,
                             "peak_source": peak_kind, "bytes_per_launch": per},
                     "ncu_small_case": NCU_SMALL_CASE.get(names[dom])},
    }
    line["clocks"] = clocks
    if rank == 0:
        line["renderer"] = renderer_rate(props.multi_processor_count, sm_mhz)
    if args.arith == "exact" and not args.no_fast:
        line["fast_arith"] = fast_arith_rate(args, eng, lib, d_start, d_obs, h_vel, h_obs, h_loss, h_grad, M, dist,
                                             dev, world, tuned is not None)
    if rank == 0 and not args.no_cpu_baseline:
        from oracle import native as o

        cores = o.cpu_threads()
        n_cpu = min(M, 10 * cores)  # about 10 s of CPU work (one gradient takes ~1 s per core)
        v, secs = cpu_baseline(start, d_obs[:n_cpu].cpu().numpy(), src, cores, n_cpu)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                                "sample": f"{n_cpu} of the {M} gradients ({secs:.1f} s), one model per thread"}
    if not args.no_large and rank == 0 and world == 1:
        # the large streamed survey, briefly: its own line is `--workload large`
        eng.close()
        del d_obs, d_start, d_true, h_obs
        torch.cuda.empty_cache()
        line["large_survey"] = measure_large(4000, 40, steps=2, warmup=1)
    if not args.no_learned and rank == 0 and world == 1:
        line["learned_refinement"] = learned_refinement_brief()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
