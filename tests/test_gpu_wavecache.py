"""The on-disk wave cache fed by the CUDA generator (GPU): per grid size, the cache written in
chunks (graph replays with a padded last chunk) holds exactly the FP16 gathers of one generator run
over all models; an interruption after the first chunk resumes to the same bytes."""

from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


class Stop(RuntimeError):
    pass


def test_wave_cache_matches_one_generator_run_and_resumes(cuda_lib, tmp_path):
    from wgnet_gb300 import wavecache
    from wgnet_gb300.datagen import GatherGenerator, synthetic_batch

    batch = synthetic_batch(8, seed=5, sizes=(70, 100))  # 4 models per grid
    kw = dict(shots=5, nt=200, dt=0.001, factor=4)
    caches = wavecache.ensure_wave_cache(tmp_path / "a", batch, chunk=3, autotune=False, **kw)
    gen = GatherGenerator({n: len(v) for n, v in batch.items()}, autotune=False, **kw)
    ref = {n: g.cpu().numpy() for n, g in gen.run(batch).items()}
    gen.close()
    for n in batch:
        assert caches[n].shape == ref[n].shape == (4, 5, 50, n)
        np.testing.assert_array_equal(np.asarray(caches[n]), ref[n])
        assert np.isfinite(np.asarray(caches[n], dtype=np.float32)).all()
        assert wavecache.cache_rms(tmp_path / "a" / f"waves_{n}x{n}") > 0

    lines = []

    def stop_after_first(msg):
        lines.append(msg)
        if len(lines) == 1:
            raise Stop(msg)

    with pytest.raises(Stop):
        wavecache.ensure_wave_cache(tmp_path / "b", batch, chunk=3, autotune=False, log=stop_after_first, **kw)
    out = wavecache.ensure_wave_cache(tmp_path / "b", batch, chunk=3, autotune=False, **kw)
    for n in batch:
        a = (tmp_path / "a" / f"waves_{n}x{n}.f16.bin").read_bytes()
        b = (tmp_path / "b" / f"waves_{n}x{n}.f16.bin").read_bytes()
        assert a == b
        np.testing.assert_array_equal(np.asarray(out[n]), ref[n])
