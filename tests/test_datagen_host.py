"""Host side of batched data generation (no GPU): the library's low-pass taps against the
reference's lowpass_kernel golden vectors, the decimation restatement, the model split and the
autotuner's cache."""

from __future__ import annotations

import json

import numpy as np
import pytest

from conftest import ROOT
from oracle import physics_np

GOLD = ROOT / "tests" / "golden"


@pytest.fixture(scope="module")
def lib():
    from wgnet_gb300 import _lib, build

    if not _lib.LIB_PATH.exists():
        build.build()
    return _lib.load()


def test_library_lowpass_taps_equal_reference_golden(lib):
    from wgnet_gb300.datagen import lowpass_taps

    p = np.load(GOLD / "physics.npz")
    n = 0
    for k in p.files:
        if k.startswith("lowpass_"):
            _, dt, f = k.split("_")
            # the C library's exp may differ from numpy's in the last bit (aarch64 glibc does)
            np.testing.assert_allclose(lowpass_taps(float(f), float(dt)), p[k], rtol=2.5e-7, atol=0, err_msg=k)
            n += 1
    assert n >= 10
    # the anti-alias filter of the x4 decimation at dt = 1 ms: -3 dB at 50 Hz, 4 sigma = 15 samples
    t = lowpass_taps(50.0, 0.001)
    assert len(t) == 31 and abs(float(t.astype(np.float64).sum()) - 1.0) < 1e-6
    np.testing.assert_allclose(t, physics_np.lowpass_kernel(50.0, 0.001), rtol=2.5e-7, atol=0)


def test_lowpass_taps_rejects_bad_arguments(lib):
    from wgnet_gb300.datagen import lowpass_taps

    for f, dt in ((0.0, 0.001), (-5.0, 0.001), (10.0, 0.0), (1e-12, 1.0e-6)):
        with pytest.raises(ValueError):
            lowpass_taps(f, dt)


def test_decimation_restatement_naive_loop():
    rng = np.random.default_rng(3)
    x = rng.standard_normal((3, 2, 37, 5)).astype(np.float32) * np.float32(50.0)
    for taps, center, factor in ((physics_np.lowpass_kernel(50.0, 0.001), 15, 4), (np.float32([1.0]), 0, 1),
                                 (np.float32([0.2, 0.3, 0.5]), 2, 3), (physics_np.lowpass_kernel(20.0, 0.001), 0, 8)):
        got = physics_np.lowpass_decimate_f16(x, taps, center, factor)
        nt_out = -(-37 // factor)
        ref = np.zeros((3, 2, nt_out, 5), np.float32)
        for j in range(nt_out):
            for k in range(len(taps)):
                t = j * factor + k - center
                if 0 <= t < 37:
                    ref[..., j, :] = ref[..., j, :] + np.float32(taps[k]) * x[..., t, :]
        np.testing.assert_array_equal(got, ref.astype(np.float16))
    # factor 1, single unit tap: the plain float16 cast of the reference's cache writer
    np.testing.assert_array_equal(physics_np.lowpass_decimate_f16(x, np.float32([1.0]), 0, 1), x.astype(np.float16))


def test_round_robin_split_and_batch():
    from wgnet_gb300.datagen import round_robin_counts, synthetic_batch

    assert round_robin_counts(4096) == {70: 1366, 100: 1365, 140: 1365}
    assert round_robin_counts(2) == {70: 1, 100: 1, 140: 0}
    b = synthetic_batch(7, seed=1)
    assert {n: v.shape for n, v in b.items()} == {70: (3, 70, 70), 100: (2, 100, 100), 140: (2, 140, 140)}
    for v in b.values():
        assert v.dtype == np.float32 and v.min() >= 1500.0 and v.max() <= 4500.0
    again = synthetic_batch(7, seed=1)
    for n in b:
        np.testing.assert_array_equal(b[n], again[n])


class _FakeEngine:
    nx = nz = 114
    pml = 20
    shots = 5
    nrec = 70
    nz_vis = nx_vis = 70

    def __init__(self, arith: int = 0):
        self.shape = {"forward": (2, 704, 10), "adjoint": (2, 704, 10)}
        self.set_calls = []
        self.arith = arith

    def get_option(self, key):
        assert key == "arith"
        return self.arith

    def shape_candidates(self, which):
        return [(2, 704, 10), (2, 896, 8), (4, 448, 8)]

    def launch_shape(self, which):
        return self.shape[which]

    def set_launch_shape(self, which, shape):
        self.shape[which] = tuple(shape)
        self.set_calls.append((which, tuple(shape)))


def test_autotuner_cache_roundtrip_and_hit(tmp_path, monkeypatch):
    from wgnet_gb300 import autotune

    path = tmp_path / "tune.json"
    monkeypatch.setattr(autotune, "device_tag", lambda: "GB300-test|sm152")
    eng = _FakeEngine()
    key_f = autotune.cache_key("GB300-test|sm152", "forward", eng)
    key_a = autotune.cache_key("GB300-test|sm152", "adjoint", eng)
    assert key_f != key_a and "114x114" in key_f and "nrec70" in key_f
    # the fast-arithmetic kernels exist for some shapes only: their timings are cached apart
    assert autotune.cache_key("GB300-test|sm152", "forward", _FakeEngine(arith=1)) != key_f
    autotune.store_cache({key_f: {"shape": [2, 896, 8]}, key_a: {"shape": [4, 448, 8]}}, path)
    autotune.store_cache({"other": {"shape": [1, 1, 1]}}, path)  # merge, not overwrite
    data = json.loads(path.read_text())
    assert set(data) == {key_f, key_a, "other"}

    def no_timing(*a, **k):
        raise AssertionError("a cached shape must not be re-timed")

    monkeypatch.setattr(autotune, "_time_forward", no_timing)
    monkeypatch.setattr(autotune, "_time_adjoint", no_timing)
    got = autotune.tune(eng, path=path)
    assert got == {"forward": (2, 896, 8), "adjoint": (4, 448, 8)}
    assert eng.shape == got


def test_autotuner_times_every_candidate_and_keeps_fastest(tmp_path, monkeypatch):
    from wgnet_gb300 import autotune

    path = tmp_path / "tune.json"
    monkeypatch.setattr(autotune, "device_tag", lambda: "GB300-test|sm152")
    monkeypatch.setattr(autotune, "_probe_models", lambda eng, models, seed: object())
    fake_ms = {(2, 704, 10): 3.0, (2, 896, 8): 2.5, (4, 448, 8): 4.0}
    monkeypatch.setattr(autotune, "_time_forward", lambda eng, vel, reps: fake_ms[eng.shape["forward"]])
    eng = _FakeEngine()
    got = autotune.tune(eng, which=("forward",), path=path)
    assert got == {"forward": (2, 896, 8)} and eng.shape["forward"] == (2, 896, 8)
    timed = [s for w, s in eng.set_calls if w == "forward"]
    assert set(timed[:3]) == set(fake_ms)
    entry = json.loads(path.read_text())[autotune.cache_key("GB300-test|sm152", "forward", eng)]
    assert entry["shape"] == [2, 896, 8] and len(entry["ms"]) == 3
    # a stale cache entry (shape not compiled for this grid) is re-timed
    autotune.store_cache({autotune.cache_key("GB300-test|sm152", "forward", eng): {"shape": [9, 9, 9]}}, path)
    eng2 = _FakeEngine()
    assert autotune.tune(eng2, which=("forward",), path=path) == {"forward": (2, 896, 8)}
