"""Budgeted refinement on the GPU, batched over models: refine() (python/wgnet/refine.py:56-169)
for many models in lockstep, with an optional learned proposal step.

The refinable field is `base + dense + upsample(coarse) + render(gaussians)` as in the reference
(coarse 9x9 bilinear, align_corners; the active Gaussian slots), plus an optional dense pixel block
(`dense_block=True`: the 70x70 field itself, bounded to [1.4, 4.6] km/s; `base` is then zero). The
algorithm is the reference's, model by model: projected L-BFGS (8 pairs, two-loop direction in
FP64 on the GPU, `wg_lbfgs_direction_dev`), direction normalized to norm <= 1, Armijo backtracking
(6 trials, c = 1e-4), one solve per loss-only evaluation and two per loss + gradient, the budget
split evenly over the passbands, each band restarted from a fresh gradient and empty memory. The
models run in lockstep: every round, the pending evaluations of all models are one batched wave
solve (simulate or evaluate_adjoint over the models that need it); per-model state never mixes.

Learned variant (`proposer=UpdateNet`): at each iteration, before the L-BFGS step, the network
proposes a dense-block update from (field, field gradient, band), tried at full and then half
length; the exact misfit accepts it if it lowers the loss (then the gradient there is taken and the
curvature pair kept), otherwise the iteration falls back to the L-BFGS step and the network is not
asked again in that band.
"""

from __future__ import annotations

import ctypes
import time
from typing import NamedTuple, Sequence

import numpy as np
import torch

from . import _lib
from ._lib import check
from .render import ACTIVE_AMP_KM, GRID, N_SLOTS, clamp_gaussians, render_residual

COARSE = 9
COARSE_MAX_KM = 1.0
GAUSS_SCALES = (1.0, 1.0, 0.2, 0.2, 0.2, 0.1)
COARSE_SCALE = 0.1
DENSE_SCALE = 1.0
DENSE_BOUNDS_KM = (1.4, 4.6)
LBFGS_PAIRS = 8
LINE_SEARCH_TRIALS = 6
ARMIJO = 1e-4
LEARNED_STEPS = (1.0, 0.5)  # lengths at which a learned proposal is tried


class RefineResult(NamedTuple):
    initial_field_km: np.ndarray
    final_field_km: np.ndarray
    initial_loss: float
    final_loss: float
    solves: int
    seconds: float
    history: list
    gaussians: np.ndarray
    coarse_km: np.ndarray


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def dot(a: torch.Tensor, b: torch.Tensor) -> torch.Tensor:
    """Per-row FP64 dot products of [B, P] tensors (fixed-order block reduction)."""
    a = a.contiguous()
    b = b.contiguous()
    out = torch.empty(a.shape[0], device=a.device, dtype=torch.float64)
    check(_lib.load().wg_dot_f64_dev(_p(a), _p(b), a.shape[0], a.shape[1], _p(out), _stream()), "dot")
    return out


def lbfgs_direction(grad, S, Y, rho, count) -> torch.Tensor:
    """_lbfgs_direction (refine.py:41-53) for each row: grad [B, P], S/Y [B, m, P] oldest first,
    rho [B, m], count [B] int32."""
    grad = grad.contiguous()
    out = torch.empty_like(grad)
    check(_lib.load().wg_lbfgs_direction_dev(_p(grad), _p(S.contiguous()), _p(Y.contiguous()), _p(rho.contiguous()),
                                             _p(count.to(torch.int32).contiguous()), grad.shape[0], S.shape[1],
                                             grad.shape[1], _p(out), _stream()), "lbfgs")
    return out


def _upsample_matrix(n_out: int, n_in: int, device) -> torch.Tensor:
    """Bilinear interpolation weights with align_corners=True: [n_out, n_in] (f64)."""
    u = torch.zeros((n_out, n_in), dtype=torch.float64)
    for i in range(n_out):
        src = i * (n_in - 1) / (n_out - 1)
        i0 = min(int(np.floor(src)), n_in - 1)
        i1 = min(i0 + 1, n_in - 1)
        lam = src - i0
        u[i, i0] += 1.0 - lam
        u[i, i1] += lam
    return u.to(device)


class Space:
    """Parameter layout of a batch: [dense pixels (optional)] [coarse 9x9] [active Gaussians, padded]."""

    def __init__(self, dense_km: torch.Tensor, gaussians: torch.Tensor | None, amp_keep_km: float,
                 dense_block: bool):
        dev = dense_km.device
        self.B = dense_km.shape[0]
        self.dense_block = dense_block
        self.base = torch.zeros_like(dense_km) if dense_block else dense_km.float()
        self.start = dense_km.float()
        if gaussians is None:
            gaussians = torch.zeros((self.B, N_SLOTS, 6), device=dev)
        act = [torch.nonzero(gaussians[b, :, 5].abs() >= amp_keep_km).flatten() for b in range(self.B)]
        self.K = max([len(a) for a in act] + [0])
        self.slot = torch.zeros((self.B, self.K), dtype=torch.long, device=dev)
        self.valid = torch.zeros((self.B, self.K), dtype=torch.bool, device=dev)
        g0 = torch.zeros((self.B, self.K, 6), dtype=torch.float64, device=dev)
        for b, a in enumerate(act):
            self.slot[b, : len(a)] = a
            self.valid[b, : len(a)] = True
            g0[b, : len(a)] = gaussians[b, a].double()
        self.nd = GRID * GRID if dense_block else 0
        self.nc = COARSE * COARSE
        self.P = self.nd + self.nc + 6 * self.K
        sc = [torch.full((self.B, self.nd), DENSE_SCALE, dtype=torch.float64, device=dev),
              torch.full((self.B, self.nc), COARSE_SCALE, dtype=torch.float64, device=dev),
              (torch.tensor(GAUSS_SCALES, dtype=torch.float64, device=dev).expand(self.B, self.K, 6)
               * self.valid.unsqueeze(-1)).reshape(self.B, -1)]
        self.scales = torch.cat(sc, dim=1).contiguous()
        x0 = [self.start.double().reshape(self.B, -1) if dense_block else sc[0],
              torch.zeros((self.B, self.nc), dtype=torch.float64, device=dev), g0.reshape(self.B, -1)]
        self.x0 = torch.cat(x0, dim=1).contiguous()
        self.U = _upsample_matrix(GRID, COARSE, dev)

    def split(self, x):
        d = x[:, : self.nd]
        c = x[:, self.nd: self.nd + self.nc].reshape(x.shape[0], COARSE, COARSE)
        g = x[:, self.nd + self.nc:].reshape(x.shape[0], self.K, 6)
        return d, c, g

    def project(self, x: torch.Tensor, rows=None) -> torch.Tensor:
        out = x.clone()
        d, c, g = self.split(out)
        if self.nd:
            d.clamp_(*DENSE_BOUNDS_KM)
        c.clamp_(-COARSE_MAX_KM, COARSE_MAX_KM)
        if self.K:
            g.copy_(clamp_gaussians(g.float()).double())
        return out

    def _full(self, g, rows):
        full = torch.zeros((len(rows), N_SLOTS, 6), device=g.device)
        valid = self.valid[rows]
        for j in range(self.K):
            v = valid[:, j]
            if v.any():
                r = torch.nonzero(v).flatten()
                full[r, self.slot[rows][r, j]] = g[r, j].float()
        return full

    def field(self, x: torch.Tensor, rows: torch.Tensor) -> torch.Tensor:
        """[len(rows), 70, 70] km/s (f32) of parameter rows x (x is already the subset)."""
        d, c, g = self.split(x)
        f = self.base[rows].clone()
        if self.nd:
            f += d.reshape(-1, GRID, GRID).float()
        f += (self.U @ c @ self.U.t()).float()
        if self.K:
            f += render_residual(self._full(g, rows))
        return f

    def param_grad(self, gfield: torch.Tensor, x: torch.Tensor, rows: torch.Tensor) -> torch.Tensor:
        """Chain rule from dJ/dfield [n, 70, 70] to the parameters, times the scales (refine.py:107)."""
        n = gfield.shape[0]
        parts = []
        if self.nd:
            parts.append(gfield.double().reshape(n, -1))
        parts.append((self.U.t() @ gfield.double() @ self.U).reshape(n, -1))
        if self.K:
            _, _, g = self.split(x)
            full = self._full(g, rows).requires_grad_(True)
            r = render_residual(full)
            (gg,) = torch.autograd.grad((r * gfield.float()).sum(), [full])
            sel = torch.stack([gg[i, self.slot[rows][i]] for i in range(n)]).double()
            parts.append((sel * self.valid[rows].unsqueeze(-1)).reshape(n, -1))
        return torch.cat(parts, dim=1) * self.scales[rows]


class _Evaluator:
    """Batched loss / loss + gradient evaluations with solve accounting (refine.py:96-108)."""

    def __init__(self, physics, space: Space, solves: torch.Tensor):
        self.ph = physics
        self.sp = space
        self.solves = solves
        self.lib = _lib.load()

    def loss(self, x, rows, observed):
        field = self.sp.field(x, rows)
        pred = self.ph.simulate(field)
        obs = observed[rows].contiguous()
        out = torch.empty(len(rows), device=x.device, dtype=torch.float64)
        check(self.lib.wg_misfit_dev(_p(pred), _p(obs), len(rows), pred[0].numel(), _p(out), _stream()), "misfit")
        self.solves[rows] += 1
        return out

    def loss_grad(self, x, rows, observed):
        field = self.sp.field(x, rows)
        loss, gfield = self.ph.loss_and_grad(field, observed[rows].contiguous())
        self.solves[rows] += 2
        return loss.double(), self.sp.param_grad(gfield, x, rows), gfield


def refine_batch(dense_km, observed_full, physics, gaussians=None, budget_solves: int = 160,
                 bands_hz: Sequence = (8.0, 12.0, None), amp_keep_km: float = ACTIVE_AMP_KM,
                 dense_block: bool = False, proposer=None, true_km=None, record: bool = False) -> dict:
    """Refine B models at once. `dense_km [B, 70, 70]` km/s, `gaussians [B, 1225, 6]` activated or
    None, `observed_full [B, shots, nt, nrec]` (CUDA tensors or arrays). Returns a dict with the
    final parameters/fields, losses, solves per model, per-model history (band, solves, loss,
    accepted, kind, and the MAE against `true_km` when given: evaluation only, the optimizer never
    sees it) and, with `record`, the (field, field gradient, band) at every gradient evaluation."""
    from .precond import band_index

    t0 = time.perf_counter()
    dev = torch.device("cuda")
    dense_km = torch.as_tensor(dense_km, dtype=torch.float32).to(dev)
    obs_full = torch.as_tensor(observed_full, dtype=torch.float32).to(dev)
    if gaussians is not None:
        gaussians = torch.as_tensor(gaussians, dtype=torch.float32).to(dev)
    true = torch.as_tensor(true_km, dtype=torch.float32).to(dev) if true_km is not None else None
    if proposer is not None and not dense_block:
        raise ValueError("the learned proposal updates the dense block: use dense_block=True")
    sp = Space(dense_km, gaussians, amp_keep_km, dense_block)
    B, P = sp.B, sp.P
    solves = torch.zeros(B, dtype=torch.long, device=dev)
    ev = _Evaluator(physics, sp, solves)
    allrows = torch.arange(B, device=dev)
    x = sp.project(sp.x0)
    history = [[] for _ in range(B)]
    records = []

    def log(rows, band, loss, accepted, kind, xx=None):
        mae = None
        if true is not None:
            f = sp.field((x if xx is None else xx)[rows], rows)
            mae = (f - true[rows]).abs().mean(dim=(1, 2)).tolist()
        for i, r in enumerate(rows.tolist()):
            h = {"band_hz": band, "solves": int(solves[r]), "loss": float(loss[i]), "accepted": bool(accepted[i]),
                 "kind": kind}
            if mae is not None:
                h["mae_km"] = mae[i]
            history[r].append(h)

    physics.set_band(None)
    initial_loss = ev.loss(x, allrows, obs_full)
    initial_field = sp.field(x, allrows)
    log(allrows, "initial", initial_loss, torch.ones(B, dtype=torch.bool), "initial")
    budget_per_band = budget_solves // len(bands_hz)
    m = LBFGS_PAIRS
    for band in bands_hz:
        physics.set_band(band)
        observed = physics.bandlimit(obs_full) if band is not None else obs_full
        band_budget = solves + budget_per_band
        cur_loss, cur_grad, cur_gf = ev.loss_grad(x, allrows, observed)
        bidx = torch.full((B,), band_index(band), dtype=torch.int32, device=dev)
        if record:
            records.append((sp.field(x, allrows).cpu(), cur_gf.float().cpu(), bidx.cpu(), allrows.cpu()))
        S = torch.zeros((B, m, P), dtype=torch.float64, device=dev)
        Y = torch.zeros_like(S)
        rho = torch.zeros((B, m), dtype=torch.float64, device=dev)
        count = torch.zeros(B, dtype=torch.int32, device=dev)
        running = torch.ones(B, dtype=torch.bool, device=dev)
        learned_ok = torch.full((B,), proposer is not None, dtype=torch.bool, device=dev)

        def push(rows, s, y):
            sy = dot(s, y)
            keep = sy > 1e-12
            for i, r in enumerate(rows.tolist()):
                if not bool(keep[i]):
                    continue
                n = int(count[r])
                if n >= m:
                    S[r, :-1] = S[r, 1:].clone()
                    Y[r, :-1] = Y[r, 1:].clone()
                    rho[r, :-1] = rho[r, 1:].clone()
                    n = m - 1
                S[r, n] = s[i]
                Y[r, n] = y[i]
                rho[r, n] = 1.0 / sy[i]
                count[r] = n + 1

        def take(rows, cand, cl, need_grad_rows):
            """Accept cand for rows; rows in need_grad_rows also get the gradient and a pair."""
            nonlocal cur_loss, cur_grad, cur_gf
            if len(need_grad_rows):
                gi = torch.nonzero(torch.isin(rows, need_grad_rows)).flatten()
                gl, gg, gf = ev.loss_grad(cand[gi], need_grad_rows, observed)
                s = (cand[gi] - x[need_grad_rows]) / torch.where(sp.scales[need_grad_rows] > 0,
                                                                sp.scales[need_grad_rows], 1.0)
                push(need_grad_rows, s, gg - cur_grad[need_grad_rows])
                cl = cl.clone()
                cl[gi] = gl
                cur_grad[need_grad_rows] = gg
                cur_gf[need_grad_rows] = gf
                if record:
                    records.append((sp.field(cand[gi], need_grad_rows).cpu(), gf.float().cpu(),
                                    bidx[need_grad_rows].cpu(), need_grad_rows.cpu()))
            x[rows] = cand
            cur_loss[rows] = cl

        while True:
            running &= (solves + 1 < band_budget)
            if not bool(running.any()):
                break
            rows = torch.nonzero(running).flatten()
            accepted = torch.zeros(B, dtype=torch.bool, device=dev)
            # learned proposal, tried at full length and then at half length
            lp = torch.nonzero(running & learned_ok).flatten()
            if len(lp):
                f = sp.field(x[lp], lp)
                upd = proposer.forward(f, cur_gf[lp].float().contiguous(), bidx[lp]).reshape(len(lp), -1).double()
                trying = torch.ones(len(lp), dtype=torch.bool, device=dev)
                for scale in LEARNED_STEPS:
                    trying &= (solves[lp] + 1 < band_budget[lp])
                    if not bool(trying.any()):
                        break
                    ti = torch.nonzero(trying).flatten()
                    tr = lp[ti]
                    cand = x[tr].clone()
                    cand[:, : sp.nd] += scale * upd[ti]
                    cand = sp.project(cand)
                    cl = ev.loss(cand, tr, observed)
                    ok = cl < cur_loss[tr]
                    if bool(ok.any()):
                        oi = torch.nonzero(ok).flatten()
                        good = tr[oi]
                        with_grad = good[(solves[good] + 2) <= band_budget[good]]
                        take(good, cand[oi], cl[oi], with_grad)
                        accepted[good] = True
                        trying[ti[oi]] = False
                        log(good, band, cur_loss[good], torch.ones(len(good), dtype=torch.bool), "learned")
                learned_ok[lp[trying]] = False
            # L-BFGS step for the running models that did not take a learned step
            rows = torch.nonzero(running & ~accepted).flatten()
            if len(rows):
                g = cur_grad[rows]
                d = lbfgs_direction(g, S[rows], Y[rows], rho[rows], count[rows])
                slope = dot(g, d)
                bad = ~torch.isfinite(slope) | (slope >= 0.0)
                if bool(bad.any()):
                    br = rows[bad]
                    count[br] = 0
                    d[bad] = -g[bad]
                    slope[bad] = -dot(g[bad], g[bad])
                norm = dot(d, d).sqrt()
                big = norm > 1.0
                d[big] = d[big] / norm[big].unsqueeze(1)
                slope[big] = slope[big] / norm[big]
                searching = torch.ones(len(rows), dtype=torch.bool, device=dev)
                step = 1.0
                for _ in range(LINE_SEARCH_TRIALS):
                    searching &= (solves[rows] + 1 < band_budget[rows])
                    if not bool(searching.any()):
                        break
                    si = torch.nonzero(searching).flatten()
                    sr = rows[si]
                    cand = sp.project(x[sr] + step * sp.scales[sr] * d[si])
                    cl = ev.loss(cand, sr, observed)
                    ok = cl <= cur_loss[sr] + ARMIJO * step * slope[si]
                    if bool(ok.any()):
                        oi = torch.nonzero(ok).flatten()
                        good = sr[oi]
                        with_grad = good[(solves[good] + 2) <= band_budget[good]]
                        take(good, cand[oi], cl[oi], with_grad)
                        accepted[good] = True
                        searching[si[oi]] = False
                    step *= 0.5
                log(rows, band, cur_loss[rows], accepted[rows], "lbfgs")
            running &= accepted

    physics.set_band(None)
    final_loss = ev.loss(x, allrows, obs_full)
    final_field = sp.field(x, allrows)
    log(allrows, "final", final_loss, torch.ones(B, dtype=torch.bool), "final")
    _, c, g = sp.split(x)
    return {"x": x, "space": sp, "initial_field_km": initial_field, "final_field_km": final_field,
            "initial_loss": initial_loss, "final_loss": final_loss, "solves": solves.clone(),
            "seconds": time.perf_counter() - t0, "history": history, "coarse_km": c.float(), "gaussians": g.float(),
            "records": records}


def refine(dense_km: np.ndarray, gaussians: np.ndarray, observed_full: np.ndarray, physics, budget_solves: int = 160,
           bands_hz: Sequence = (8.0, 12.0, None), amp_keep_km: float = ACTIVE_AMP_KM, device="cuda",
           dense_block: bool = False) -> RefineResult:
    """refine() with the reference's signature (refine.py:56-65): one model, `dense_km [70, 70]`,
    `gaussians [1225, 6]` activated, `observed_full [shots, nt, 70]`."""
    r = refine_batch(np.asarray(dense_km)[None], np.asarray(observed_full)[None], physics,
                     gaussians=None if gaussians is None else np.asarray(gaussians)[None], budget_solves=budget_solves,
                     bands_hz=bands_hz, amp_keep_km=amp_keep_km, dense_block=dense_block)
    hist = [h for h in r["history"][0] if h["kind"] in ("lbfgs", "learned")]
    sp = r["space"]
    return RefineResult(initial_field_km=r["initial_field_km"][0].cpu().numpy(),
                        final_field_km=r["final_field_km"][0].cpu().numpy(),
                        initial_loss=float(r["initial_loss"][0]), final_loss=float(r["final_loss"][0]),
                        solves=int(r["solves"][0]), seconds=r["seconds"], history=hist,
                        gaussians=r["gaussians"][0][sp.valid[0]].cpu().numpy(),
                        coarse_km=r["coarse_km"][0].cpu().numpy())


__all__ = ["refine", "refine_batch", "RefineResult", "lbfgs_direction", "dot", "Space"]
