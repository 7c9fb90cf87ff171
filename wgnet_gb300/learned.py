"""Learned refinement: trajectory generation with the exact solver, training of the update network,
and the comparison against plain projected L-BFGS.

    python -m wgnet_gb300.learned --train-models 2048 --eval-models 128 --out results/

1. Trajectories: seeded mixed-family 70x70 models (flat, curved, faulted, blob inclusions), start =
   the true model smoothed by a 5-cell Gaussian, observed data simulated from the true model
   (5 shots at cells 0, 17, 34, 52, 69, 70 receivers, 15 Hz Ricker, dt 1 ms, nt 1000). Plain
   refinement (`refine_batch`, dense pixel block + coarse grid, bands 6 / 9 / 12 Hz / full) records
   (field, field gradient, band) at every gradient evaluation; the training target is the
   trajectory's final field minus the recorded field (where plain L-BFGS gets to).
   With `--target true` (default) the target is the true model minus the recorded field instead.
2. Training: `UpdateNet.train_step` (tensor-core kernels) on shuffled batches.
3. Evaluation on held-out seeds with 5-, 3- and 1-shot surveys: plain refinement with the full
   budget, then the learned variant; reported are the wave solves each needs to reach the plain
   method's final velocity MAE (the true model is used only to score).
"""

from __future__ import annotations

import argparse
import json
import time
from pathlib import Path

import numpy as np
import torch

from .models_synth import make_batch, smooth
from .physics import WavePhysics
from .precond import UpdateNet
from .refine import refine_batch

BANDS = (6.0, 9.0, 12.0, None)
SHOT_CELLS = (0, 17, 34, 52, 69)
SUBSETS = {5: (0, 1, 2, 3, 4), 3: (0, 2, 4), 1: (2,)}


def physics_for(shots: tuple[int, ...], nt: int = 1000) -> WavePhysics:
    from .engine import WaveEngine

    eng = WaveEngine(shots=len(shots), nt=nt, dt=0.001, peak_hz=15.0, pml=20, vmin=1000.0, vmax=5000.0)
    src = np.stack([np.float32([SHOT_CELLS[i] for i in shots]) * np.float32(10.0),
                    np.full(len(shots), 10.0, np.float32)], 1).astype(np.float32)
    eng.set_sources(src)
    return WavePhysics(shots=len(shots), nt=nt, engine=eng)


def problem(n: int, seed: int, physics: WavePhysics, sigma: float = 5.0):
    true = make_batch(n, seed=seed) / np.float32(1000.0)
    start = smooth(true, sigma)
    with torch.no_grad():
        physics.set_band(None)
        obs = physics.simulate(torch.from_numpy(true).cuda())
    return torch.from_numpy(true).cuda(), torch.from_numpy(start).cuda(), obs


def trajectories(n_models: int, seed: int, budget: int = 80, chunk: int = 256, nt: int = 1000,
                 target: str = "true", sigmas: tuple[float, ...] = (5.0,)) -> dict:
    """Plain refinement trajectories; returns GPU tensors field, grad, band, target and the MAEs.
    target "true": the true model minus the recorded field (the training models are synthetic, so
    the truth is known); "final": the trajectory's final field minus the recorded field. The
    starting models are the true ones smoothed by `sigmas` cells, taken in turn per chunk."""
    ph = physics_for(SUBSETS[5], nt)
    fields, grads, bands, targets = [], [], [], []
    mae0, mae1 = [], []
    for c0 in range(0, n_models, chunk):
        n = min(chunk, n_models - c0)
        true, start, obs = problem(n, seed * 1_000_003 + c0, ph, sigma=sigmas[(c0 // chunk) % len(sigmas)])
        r = refine_batch(start, obs, ph, budget_solves=budget, bands_hz=BANDS, dense_block=True, record=True)
        final = r["final_field_km"]
        for f, g, b, rows in r["records"]:
            rows = rows.cuda()
            fields.append(f.cuda())
            grads.append(g.cuda())
            bands.append(b.cuda())
            ref = true[rows] if target == "true" else final[rows]
            targets.append(ref - f.cuda())
        mae0.append((start - true).abs().mean(dim=(1, 2)))
        mae1.append((final - true).abs().mean(dim=(1, 2)))
    return {"field": torch.cat(fields), "grad": torch.cat(grads), "band": torch.cat(bands).to(torch.int32),
            "target": torch.cat(targets), "mae_start": torch.cat(mae0), "mae_plain": torch.cat(mae1)}


def train(net: UpdateNet, data: dict, epochs: int = 4, batch: int = 32, lr: float = 1e-3, seed: int = 0,
          log=print) -> list[float]:
    n = data["field"].shape[0]
    g = torch.Generator(device="cpu").manual_seed(seed)
    losses = []
    steps = epochs * (n // batch)
    k = 0
    for ep in range(epochs):
        perm = torch.randperm(n, generator=g).cuda()
        for i in range(n // batch):
            idx = perm[i * batch:(i + 1) * batch]
            rate = lr * 0.5 * (1.0 + np.cos(np.pi * k / max(steps, 1)))
            loss = net.train_step(data["field"][idx], data["grad"][idx], data["band"][idx], data["target"][idx],
                                  lr=float(rate))
            losses.append(loss)
            k += 1
        log(f"epoch {ep}: mean loss {np.mean(losses[-(n // batch):]):.6f}")
    return losses


def mae_curve(history: list, key: str = "mae_km") -> list[tuple[int, float]]:
    return [(h["solves"], h[key]) for h in history if key in h]


def solves_to_reach(curve: list[tuple[int, float]], target: float) -> int | None:
    for s, m in curve:
        if m <= target:
            return s
    return None


def evaluate(net: UpdateNet, n_models: int, seed: int, shots: int, budget: int = 160, nt: int = 1000,
             sigma: float = 5.0) -> dict:
    """Plain and learned refinement of `n_models` held-out seeded models from a `sigma`-cell smoothed
    start (the training trajectories start from a 5-cell smoothing)."""
    ph = physics_for(SUBSETS[shots], nt)
    true, start, obs = problem(n_models, seed, ph, sigma=sigma)
    t0 = time.perf_counter()
    plain = refine_batch(start, obs, ph, budget_solves=budget, bands_hz=BANDS, dense_block=True, true_km=true)
    t_plain = time.perf_counter() - t0
    t0 = time.perf_counter()
    learned = refine_batch(start, obs, ph, budget_solves=budget, bands_hz=BANDS, dense_block=True, true_km=true,
                           proposer=net)
    t_learned = time.perf_counter() - t0
    rows = []
    for b in range(n_models):
        cp = mae_curve(plain["history"][b])
        cl = mae_curve(learned["history"][b])
        target = cp[-1][1]
        sp, sl = solves_to_reach(cp, target), solves_to_reach(cl, target)
        rows.append({"mae_start": cp[0][1], "mae_plain": target, "mae_learned": cl[-1][1], "solves_plain": sp,
                     "solves_learned": sl, "learned_steps": sum(h["kind"] == "learned" for h in learned["history"][b])})
    sp = np.array([r["solves_plain"] for r in rows], float)
    sl = np.array([r["solves_learned"] if r["solves_learned"] is not None else np.nan for r in rows], float)
    reached = np.isfinite(sl)
    return {"shots": shots, "models": n_models, "budget": budget, "start_sigma_cells": sigma,
            "mae_start_km": float(np.mean([r["mae_start"] for r in rows])),
            "mae_plain_km": float(np.mean([r["mae_plain"] for r in rows])),
            "mae_learned_km": float(np.mean([r["mae_learned"] for r in rows])),
            "solves_plain_mean": float(np.mean(sp)), "solves_learned_mean": float(np.nanmean(sl)) if reached.any() else None,
            "reached_fraction": float(reached.mean()),
            "solve_ratio_median": float(np.nanmedian(sp / sl)) if reached.any() else None,
            "seconds_plain": t_plain, "seconds_learned": t_learned, "per_model": rows}


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--train-models", type=int, default=2048)
    ap.add_argument("--eval-models", type=int, default=128)
    ap.add_argument("--traj-budget", type=int, default=80)
    ap.add_argument("--eval-budget", type=int, default=160)
    ap.add_argument("--epochs", type=int, default=4)
    ap.add_argument("--batch", type=int, default=32)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--nt", type=int, default=1000)
    ap.add_argument("--out", default="learned_out")
    ap.add_argument("--weights", default=None, help="skip training: load these weights")
    ap.add_argument("--target", default="true", choices=["true", "final"])
    ap.add_argument("--ood-models", type=int, default=0,
                    help="also evaluate this many held-out models from a more strongly smoothed start")
    ap.add_argument("--ood-sigma", type=float, default=8.0, help="smoothing (cells) of that start")
    ap.add_argument("--train-sigmas", default="5", help="smoothing (cells) of the training starts, comma-separated, "
                                                        "taken in turn per chunk of 256 models")
    args = ap.parse_args(argv)
    out = Path(args.out)
    out.mkdir(parents=True, exist_ok=True)
    logf = open(out / "log.txt", "a")

    def log(msg):
        print(msg, flush=True)
        logf.write(msg + "\n")
        logf.flush()

    report = {"args": {k: v for k, v in vars(args).items() if k != "out"}}
    if args.weights:
        net = UpdateNet.load(args.weights)
    else:
        t0 = time.perf_counter()
        sigmas = tuple(float(v) for v in args.train_sigmas.split(","))
        data = trajectories(args.train_models, seed=1, budget=args.traj_budget, nt=args.nt, target=args.target,
                            sigmas=sigmas)
        torch.cuda.synchronize()
        report["trajectories"] = {"models": args.train_models, "samples": int(data["field"].shape[0]),
                                  "seconds": time.perf_counter() - t0,
                                  "mae_start_km": float(data["mae_start"].mean()),
                                  "mae_plain_km": float(data["mae_plain"].mean())}
        log(json.dumps(report["trajectories"]))
        net = UpdateNet(seed=0)
        t0 = time.perf_counter()
        losses = train(net, data, epochs=args.epochs, batch=args.batch, lr=args.lr, log=log)
        torch.cuda.synchronize()
        report["training"] = {"steps": len(losses), "seconds": time.perf_counter() - t0, "first_loss": losses[0],
                              "last_loss": float(np.mean(losses[-50:])), "parameters": net.parameters}
        log(json.dumps(report["training"]))
        net.save(out / "update_net.npz")
        del data
    report["evaluation"] = {}
    for shots in (5, 3, 1):
        r = evaluate(net, args.eval_models, seed=777, shots=shots, budget=args.eval_budget, nt=args.nt)
        log(json.dumps({k: v for k, v in r.items() if k != "per_model"}))
        report["evaluation"][str(shots)] = r
    if args.ood_models:
        report["evaluation_shifted_start"] = {}
        for shots in (5, 3, 1):
            r = evaluate(net, args.ood_models, seed=888, shots=shots, budget=args.eval_budget, nt=args.nt,
                         sigma=args.ood_sigma)
            log(json.dumps({k: v for k, v in r.items() if k != "per_model"}))
            report["evaluation_shifted_start"][str(shots)] = r
    (out / "report.json").write_text(json.dumps(report, indent=1))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
