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
