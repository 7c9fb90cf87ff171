"""The resumable wave-cache writer (python/wgnet/data.py:138-179's role) on CPU, with a deterministic
stand-in simulator: an interrupted run resumes from its progress file and ends byte-identical to
an uninterrupted one, also when the interruption falls between a chunk's data and its progress
record; mismatched caches are refused; a complete cache reopens without simulating."""

from __future__ import annotations

import json

import numpy as np
import pytest

from wgnet_gb300 import wavecache

SHAPE = (11, 3, 20, 7)  # models, shots, nt_out, nrec


def fake_simulate(i0, i1):
    rng = np.random.default_rng(1000 + i0)
    return (rng.standard_normal((i1 - i0,) + SHAPE[1:]) * 0.01).astype(np.float16)


class Boom(RuntimeError):
    pass


def test_uninterrupted_and_resumed_caches_are_identical(tmp_path):
    ref = wavecache.write_wave_cache(tmp_path / "a", SHAPE, fake_simulate, chunk=3, fingerprint="x")
    ref_bytes = (tmp_path / "a.f16.bin").read_bytes()
    assert ref.shape == SHAPE and ref.dtype == np.float16
    calls = []

    def failing(i0, i1):
        calls.append(i0)
        if len(calls) == 3:
            raise Boom("interrupted")
        return fake_simulate(i0, i1)

    with pytest.raises(Boom):
        wavecache.write_wave_cache(tmp_path / "b", SHAPE, failing, chunk=3, fingerprint="x")
    prog = json.loads((tmp_path / "b.progress.json").read_text())
    assert prog["completed"] == 6 and prog["shape"] == list(SHAPE)
    assert not (tmp_path / "b.done.json").exists()
    seen = []

    def resumed(i0, i1):
        seen.append(i0)
        return fake_simulate(i0, i1)

    out = wavecache.write_wave_cache(tmp_path / "b", SHAPE, resumed, chunk=3, fingerprint="x")
    assert seen == [6, 9]  # resumed after the last recorded chunk
    assert (tmp_path / "b.f16.bin").read_bytes() == ref_bytes
    assert not (tmp_path / "b.progress.json").exists()
    done = json.loads((tmp_path / "b.done.json").read_text())
    rms = float(np.sqrt(np.mean(np.asarray(ref, dtype=np.float64) ** 2)))
    assert done["count"] == SHAPE[0] and abs(done["rms"] - rms) <= 1e-12 * rms
    assert abs(wavecache.cache_rms(tmp_path / "b") - rms) <= 1e-12 * rms
    np.testing.assert_array_equal(np.asarray(out), np.asarray(ref))


def test_crash_between_data_and_progress_record(tmp_path, monkeypatch):
    ref = wavecache.write_wave_cache(tmp_path / "a", SHAPE, fake_simulate, chunk=4, fingerprint="")
    real = wavecache._write_json
    count = {"n": 0}

    def flaky(path, data):
        count["n"] += 1
        if count["n"] == 2:  # the second chunk's data is in the file, its record is not
            raise Boom("power cut")
        real(path, data)

    monkeypatch.setattr(wavecache, "_write_json", flaky)
    with pytest.raises(Boom):
        wavecache.write_wave_cache(tmp_path / "b", SHAPE, fake_simulate, chunk=4, fingerprint="")
    monkeypatch.setattr(wavecache, "_write_json", real)
    assert json.loads((tmp_path / "b.progress.json").read_text())["completed"] == 4
    wavecache.write_wave_cache(tmp_path / "b", SHAPE, fake_simulate, chunk=4, fingerprint="")
    assert (tmp_path / "b.f16.bin").read_bytes() == (tmp_path / "a.f16.bin").read_bytes()
    np.testing.assert_array_equal(np.asarray(wavecache.write_wave_cache(tmp_path / "b", SHAPE, None, 4, "")),
                                  np.asarray(ref))


def test_complete_cache_reopens_without_simulating(tmp_path):
    wavecache.write_wave_cache(tmp_path / "c", SHAPE, fake_simulate, chunk=5, fingerprint="f")

    def never(i0, i1):
        raise AssertionError("a complete cache must not be simulated again")

    mm = wavecache.write_wave_cache(tmp_path / "c", SHAPE, never, chunk=5, fingerprint="f")
    assert mm.shape == SHAPE


def test_mismatched_caches_are_refused(tmp_path):
    def failing(i0, i1):
        if i0 >= 3:
            raise Boom()
        return fake_simulate(i0, i1)

    with pytest.raises(Boom):
        wavecache.write_wave_cache(tmp_path / "d", SHAPE, failing, chunk=3, fingerprint="one")
    with pytest.raises(ValueError, match="another cache"):
        wavecache.write_wave_cache(tmp_path / "d", SHAPE, fake_simulate, chunk=3, fingerprint="two")
    with pytest.raises(ValueError, match="another cache"):
        wavecache.write_wave_cache(tmp_path / "d", (12,) + SHAPE[1:], fake_simulate, chunk=3, fingerprint="one")
    wavecache.write_wave_cache(tmp_path / "e", SHAPE, fake_simulate, chunk=3, fingerprint="one")
    with pytest.raises(ValueError, match="another cache"):
        wavecache.write_wave_cache(tmp_path / "e", SHAPE, fake_simulate, chunk=3, fingerprint="two")


def test_bad_simulator_output_and_arguments(tmp_path):
    with pytest.raises(ValueError, match="float16"):
        wavecache.write_wave_cache(tmp_path / "f", SHAPE, lambda a, b: fake_simulate(a, b).astype(np.float32), 4)
    with pytest.raises(ValueError, match="float16"):
        wavecache.write_wave_cache(tmp_path / "g", SHAPE, lambda a, b: fake_simulate(a, b)[:, :2], 4)
    with pytest.raises(ValueError):
        wavecache.write_wave_cache(tmp_path / "h", SHAPE, fake_simulate, chunk=0)
    with pytest.raises(ValueError):
        wavecache.write_wave_cache(tmp_path / "i", (3, 4, 5), fake_simulate, chunk=2)
