"""Budgeted multiscale full-waveform inversion on the pixel grid (python/wgnet/fwi_eval.py:32-57):
scipy's L-BFGS-B under the velocity bounds [1.4, 4.6] km/s, the budget split evenly over the bands,
passband continuation, and the exact-adjoint gradient smoothed by a Gaussian of `smooth_grad` cells.

`fwi` keeps the reference's signature and result. `fwi_batch` inverts many models at once: each
model's L-BFGS-B runs exactly as in `fwi`, in a thread of its own, and a broker gathers the models'
objective calls into one batched `loss_and_grad` (one launch sequence over every waiting model) per
round. A model's loss and gradient do not depend on the batch they are computed in, so each model
follows the trajectory `fwi` gives it alone, bit for bit.
"""

from __future__ import annotations

import threading

import numpy as np
from scipy.ndimage import gaussian_filter
from scipy.optimize import minimize

V_BOUNDS_KM = (1.4, 4.6)


class _Broker:
    """Objective calls of `n` optimizer threads; the last active thread to arrive evaluates every
    waiting call in one batch. A thread that finishes (or fails) leaves, so the others never wait
    for it."""

    def __init__(self, n: int, evaluate) -> None:
        self._cv = threading.Condition()
        self._evaluate = evaluate
        self._active = n
        self._pending: dict[int, np.ndarray] = {}
        self._results: dict[int, tuple] = {}
        self._error: BaseException | None = None
        self.rounds = 0

    def _run(self) -> None:  # with the lock held
        idx = sorted(self._pending)
        xs = [self._pending.pop(i) for i in idx]
        self.rounds += 1
        try:
            out = self._evaluate(idx, xs)
        except BaseException as exc:  # every waiting thread raises it
            self._error = exc
            out = [None] * len(idx)
        for i, r in zip(idx, out):
            self._results[i] = r
        self._cv.notify_all()

    def call(self, i: int, x: np.ndarray):
        with self._cv:
            if self._error is not None:
                raise RuntimeError("the batched objective failed") from self._error
            self._pending[i] = x
            if len(self._pending) == self._active:
                self._run()
            while i not in self._results:
                self._cv.wait()
            r = self._results.pop(i)
            if self._error is not None:
                raise RuntimeError("the batched objective failed") from self._error
            return r

    def leave(self) -> None:
        with self._cv:
            self._active -= 1
            if self._pending and len(self._pending) == self._active:
                self._run()


def fwi_batch(starts_km, observed_full, physics, bands: list[float | None], budget: int,
              smooth_grad: float = 1.5) -> tuple[list[np.ndarray], list[list[dict]]]:
    """`fwi` for `starts_km [B, n, n]` against `observed_full [B, shots, nt, nrec]` (full band).
    Returns the final models and, per model, the per-band history of misfit and solve counts."""
    starts = np.asarray(starts_km, dtype=np.float32)
    if starts.ndim != 3 or starts.shape[1] != starts.shape[2]:
        raise ValueError("starts_km must be [B, n, n]")
    observed_full = np.asarray(observed_full, dtype=np.float32)
    if observed_full.shape[0] != starts.shape[0]:
        raise ValueError("one observed gather set per starting model")
    B, n = starts.shape[0], starts.shape[-1]
    xs = [starts[b].astype(np.float64).reshape(-1) for b in range(B)]
    per_band = max(2, budget // len(bands))
    histories: list[list[dict]] = [[] for _ in range(B)]
    for band in bands:
        physics.set_band(band)
        observed = physics.bandlimit(observed_full)
        calls = [0] * B

        def evaluate(idx, vecs):
            fields = np.stack([v.reshape(n, n).astype(np.float32) for v in vecs])
            losses, grads = physics.loss_and_grad(fields, observed[idx])
            out = []
            for k in range(len(idx)):
                g = gaussian_filter(grads[k], smooth_grad, mode="nearest") if smooth_grad > 0 else grads[k]
                out.append((float(losses[k]), g.reshape(-1).astype(np.float64)))
            return out

        broker = _Broker(B, evaluate)
        results: list = [None] * B
        errors: list[BaseException] = []

        def run(b: int) -> None:
            def objective(vec: np.ndarray):
                calls[b] += 1
                return broker.call(b, vec)

            try:
                results[b] = minimize(objective, xs[b], jac=True, method="L-BFGS-B", bounds=[V_BOUNDS_KM] * (n * n),
                                      options={"maxfun": per_band, "maxiter": per_band, "maxcor": 10})
            except BaseException as exc:
                errors.append(exc)
            finally:
                broker.leave()

        threads = [threading.Thread(target=run, args=(b,), daemon=True) for b in range(B)]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        if errors:
            physics.set_band(None)
            raise errors[0]
        for b in range(B):
            xs[b] = results[b].x
            histories[b].append({"band_hz": band, "misfit": float(results[b].fun), "solves": calls[b]})
    physics.set_band(None)
    return [x.reshape(n, n).astype(np.float32) for x in xs], histories


def fwi(start_km: np.ndarray, observed_full: np.ndarray, physics, bands: list[float | None], budget: int,
        smooth_grad: float = 1.5) -> tuple[np.ndarray, list[dict]]:
    """fwi_eval.py:32-57: one model's budgeted multiscale FWI. Returns the final model and the
    per-band history of misfit and solve counts."""
    finals, histories = fwi_batch(np.asarray(start_km, np.float32)[None], np.asarray(observed_full)[None], physics,
                                  bands, budget, smooth_grad)
    return finals[0], histories[0]


def misfit_full(model_km: np.ndarray, observed_full: np.ndarray, physics) -> float:
    """fwi_eval.py:60-63: the full-band misfit of one model."""
    physics.set_band(None)
    losses, _ = physics.loss_and_grad(np.asarray(model_km, np.float32)[None], np.asarray(observed_full)[None])
    return float(losses[0])
