"""bench.py's own arithmetic, on CPU: the algorithmic flop and byte counts that the roofline divides
by, the clock record that decides whether a run is kept, and the workload `config` that the two
arms (this repository's and the reference's CPU path) must print identically."""

from __future__ import annotations

import importlib.util
import json
import types
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", ROOT / "bench.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.mark.parametrize("n_vis", [70, 100, 140])
def test_flops_per_cell_update_is_the_average_over_the_updated_grid(bench, n_vis):
    # cell by cell: 24 flops in the interior, 30 more per C-PML axis the cell lies in
    pml = bench.PML
    n = n_vis + 2 * (pml + 2) - 4
    strip = 2 * (pml + 2) // 2
    idx = np.arange(n)
    in_strip = (idx < strip) | (idx >= n - strip)
    per_cell = 24.0 + 30.0 * in_strip[:, None] + 30.0 * in_strip[None, :]
    assert bench.flops_per_cell_update(n_vis) == pytest.approx(per_cell.mean(), rel=1e-12)
    if n_vis == 70:
        assert bench.flops_per_cell_update(70) == 48.0 == bench.FLOPS_PER_CELL_UPDATE
        assert n * n == bench.UPDATED_CELLS


def test_streamed_bytes_per_cell_update(bench):
    fwd, adj = bench.large_bytes_per_cell_update(844, 344, 20, 40)
    # 12 B wavefield + 4 B stored term + 0.1 B velocity + 16 B per C-PML axis on the strip fraction
    assert fwd == pytest.approx(19.273, abs=1e-3)
    assert adj == pytest.approx(27.273, abs=1e-3)
    assert adj - fwd == pytest.approx(8.0)  # the gradient accumulator's read and write


def test_clock_record_summary(bench):
    idle = ["0", "2070", "2070", "900.0", "0x0", "Not Active", "Not Active", "Not Active", "Not Active"]
    capped = ["0", "1980", "2070", "1400.0", "0x4", "Not Active", "Not Active", "Not Active", "Active"]
    hot = ["0", "1500", "2070", "1400.0", "0x40", "Not Active", "Active", "Not Active", "Not Active"]
    s = bench.summarize_clocks([idle, capped, idle])
    assert s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0 and s["samples"] == 3
    assert s["reasons"] == ["sw_power_cap"]  # kept and noted
    assert bench.summarize_clocks([idle, hot])["reasons"] == ["hw_thermal_slowdown"]  # a run to reject
    assert bench.summarize_clocks([])["sm_mhz"] is None


def test_reference_arm_prints_this_arms_config(bench, monkeypatch, capsys):
    """The reference arm's line carries the same `config` as the default gradient run, with its
    per-step sample described in `cpu_baseline.sample` (the solver itself is replaced by a stub:
    this checks the line, not the CPU solver)."""
    import oracle

    calls = []

    def gradients_parallel(sv, start, src, wav, obs, threads):
        calls.append(len(start))
        return np.zeros(len(start)), np.zeros_like(start)

    fake = types.SimpleNamespace(
        cpu_threads=lambda: 4,
        Survey=lambda **kw: types.SimpleNamespace(**kw),
        ricker=lambda nt, dt, f: np.zeros(nt, np.float32),
        forward=lambda sv, true, src, wav, threads: np.zeros((len(true), 5, 1000, 70), np.float32),
        gradients_parallel=gradients_parallel,
    )
    monkeypatch.setattr(oracle, "native", fake, raising=False)
    monkeypatch.setitem(__import__("sys").modules, "oracle.native", fake)
    args = types.SimpleNamespace(gpus=1, steps=2, warmup=1, models=bench.MODELS, checkpoint=bench.CK)
    assert bench.run_reference(args) == 0
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    assert line["config"] == bench.gradient_config(bench.MODELS, bench.NT, bench.CK, "exact")
    assert line["metric"] == bench.METRIC and line["unit"] == bench.UNIT
    assert line["e2e"]["value"] == line["value"] == line["cpu_baseline"]["value"]
    assert calls == [4, 4, 4]  # warm-up + 2 timed steps, one model per host thread
