"""Restatement of the L-BFGS two-loop recursion of refine() (python/wgnet/refine.py:41-53).
TEST INFRASTRUCTURE ONLY."""

from __future__ import annotations

import numpy as np


def lbfgs_direction(grad, s_hist, y_hist, rho) -> np.ndarray:
    q = np.array(grad, np.float64, copy=True)
    alphas = []
    for s, y, r in zip(reversed(s_hist), reversed(y_hist), reversed(rho)):
        a = r * float(np.dot(s, q))
        alphas.append(a)
        q -= a * y
    if len(s_hist):
        sy, yy = float(np.dot(s_hist[-1], y_hist[-1])), float(np.dot(y_hist[-1], y_hist[-1]))
        q *= sy / max(yy, 1e-30)
    for s, y, r, a in zip(s_hist, y_hist, rho, reversed(alphas)):
        q += s * (a - r * float(np.dot(y, q)))
    return -q


def refine_loop(x0, scales, project, evaluate, bands, budget_solves, set_band):
    """Control flow of refine() (python/wgnet/refine.py:84-158), restated with numpy f64 for one
    model. `evaluate(vec, need_grad, band)` returns (loss, scaled gradient or None) and the number
    of solves it used (1 without, 2 with the gradient); `project(vec)` the projected vector;
    `set_band(band)` switches the passband (None: full band). Returns (x, history, solves) with
    history entries (band, solves, loss, accepted) as in the reference."""
    LBFGS_PAIRS, LINE_SEARCH_TRIALS, ARMIJO = 8, 6, 1e-4
    solves = 0
    history = []

    def ev(vec, need_grad, band):
        nonlocal solves
        loss, grad, used = evaluate(vec, need_grad, band)
        solves += used
        return loss, grad

    x = project(np.asarray(x0, np.float64))
    set_band(None)
    ev(x, False, None)
    per_band = budget_solves // len(bands)
    for band in bands:
        set_band(band)
        band_budget = solves + per_band
        cur_loss, cur_grad = ev(x, True, band)
        s_hist, y_hist, rho = [], [], []
        while solves + 1 < band_budget:
            d = lbfgs_direction(cur_grad, s_hist, y_hist, rho)
            slope = float(np.dot(cur_grad, d))
            if not np.isfinite(slope) or slope >= 0.0:
                s_hist, y_hist, rho = [], [], []
                d = -cur_grad
                slope = -float(np.dot(cur_grad, cur_grad))
            norm = float(np.linalg.norm(d))
            if norm > 1.0:
                d, slope = d / norm, slope / norm
            step, accepted = 1.0, False
            for _ in range(LINE_SEARCH_TRIALS):
                if solves + 1 >= band_budget:
                    break
                cand = project(x + step * scales * d)
                cand_loss, _ = ev(cand, False, band)
                if cand_loss <= cur_loss + ARMIJO * step * slope:
                    if solves + 2 > band_budget:
                        x, cur_loss = cand, cand_loss
                        accepted = True
                        break
                    cand_loss, cand_grad = ev(cand, True, band)
                    s, y = (cand - x) / scales, cand_grad - cur_grad
                    sy = float(np.dot(s, y))
                    if sy > 1e-12:
                        if len(s_hist) >= LBFGS_PAIRS:
                            s_hist.pop(0), y_hist.pop(0), rho.pop(0)
                        s_hist.append(s), y_hist.append(y), rho.append(1.0 / sy)
                    x, cur_loss, cur_grad = cand, cand_loss, cand_grad
                    accepted = True
                    break
                step *= 0.5
            history.append((band, solves, cur_loss, accepted))
            if not accepted:
                break
    set_band(None)
    ev(x, False, None)
    return x, history, solves
