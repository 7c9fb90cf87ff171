"""The C-ABI library: it loads, exports every entry point declared in include/wgnet_gb300.h, and
its host-side routines (no GPU needed) equal the oracle's. No kernel is launched here."""

from __future__ import annotations

import ctypes
import re

import numpy as np
import pytest

from conftest import ROOT


@pytest.fixture(scope="module")
def lib():
    from wgnet_gb300 import _lib, build

    if not _lib.LIB_PATH.exists():
        build.build()
    return _lib.load()


def declared_symbols() -> list[str]:
    text = (ROOT / "include" / "wgnet_gb300.h").read_text()
    return sorted(set(re.findall(r"^\s*(?:int|void|const char\*|long long)\s+(wg_\w+)\s*\(", text, re.M)))


def test_header_declares_the_entry_points():
    names = declared_symbols()
    assert len(names) >= 20
    for required in ("wg_engine_create", "wg_simulate", "wg_evaluate_adjoint", "wg_set_sources", "wg_set_wavelet",
                     "wg_simulate_shot", "wg_render_fwd_dev", "wg_render_bwd_dev", "wg_bandlimit_dev"):
        assert required in names


def test_library_exports_every_declared_symbol(lib):
    for name in declared_symbols():
        assert hasattr(lib, name), name
        assert isinstance(getattr(lib, name), ctypes._CFuncPtr)


def test_python_binding_covers_the_header(lib):
    from wgnet_gb300._lib import SIGNATURES

    assert set(declared_symbols()) <= set(SIGNATURES)


def test_host_ricker_and_cpml_equal_oracle(lib):
    from oracle import native as o
    from wgnet_gb300.engine import cpml_profiles, ricker_wavelet

    for nt, dt, f in ((2001, 0.0005, 15.0), (1000, 0.001, 15.0), (4000, 0.0005, 15.0), (37, 0.002, 7.5)):
        np.testing.assert_array_equal(ricker_wavelet(nt, dt, f), o.ricker(nt, dt, f))
    for n, h, dt, w, vmax in ((114, 10.0, 0.001, 20, 5000.0), (844, 5.0, 0.0005, 20, 4500.0), (30, 10.0, 0.001, 4, 3000.0)):
        for a, b in zip(cpml_profiles(n, h, dt, w, vmax, 15.0), o.cpml_profiles(n, h, dt, w, vmax, 15.0)):
            np.testing.assert_array_equal(a, b)


def test_error_reporting_without_gpu(lib):
    from wgnet_gb300 import _lib

    rc = lib.wg_ricker_wavelet(-1, 0.001, 15.0, None)
    assert rc == _lib.WG_ERR_ARG
    assert _lib.last_error() != ""
    with pytest.raises(ValueError):
        _lib.check(rc)
    assert lib.wg_engine_create(None, None) == _lib.WG_ERR_ARG
    rc = lib.wg_bandlimit_dev(None, None, 3, 1, 10, 4, None, None)
    assert rc == _lib.WG_ERR_ARG


def test_drop_in_module_surface():
    import wave_gauss_rs

    assert callable(wave_gauss_rs.ricker_wavelet)
    assert callable(wave_gauss_rs.simulate_shot_cpu)
    assert isinstance(wave_gauss_rs.PyWaveEngine, type)
    for m in ("sources", "set_sources", "wavelet", "set_wavelet", "simulate", "evaluate_adjoint"):
        assert hasattr(wave_gauss_rs.PyWaveEngine, m)
    for p in ("shots", "nt", "nrec"):
        assert isinstance(getattr(wave_gauss_rs.PyWaveEngine, p), property)


def test_drop_in_argument_checks_before_any_gpu_work():
    import wave_gauss_rs

    with pytest.raises(TypeError):
        wave_gauss_rs.simulate_shot_cpu(np.zeros(4900), 10.0, 0.001, 10, 20, 1000.0, 5000.0, 15.0, 0.0, 10.0)
    with pytest.raises(ValueError):
        wave_gauss_rs.simulate_shot_cpu(np.zeros(4899, np.float32), 10.0, 0.001, 10, 20, 1000.0, 5000.0, 15.0, 0.0,
                                        10.0)
    with pytest.raises(ValueError):
        wave_gauss_rs.simulate_shot_cpu(np.zeros((2, 4900), np.float32)[:, 0], 10.0, 0.001, 10, 20, 1000.0, 5000.0,
                                        15.0, 0.0, 10.0)
