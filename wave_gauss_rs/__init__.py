"""`import wave_gauss_rs` for code written against the reference's PyO3 module: re-exports the
CUDA-backed implementation in `wgnet_gb300.wave_gauss_rs`."""

from wgnet_gb300.wave_gauss_rs import CELLS, N, PyWaveEngine, ricker_wavelet, simulate_shot_cpu

__all__ = ["PyWaveEngine", "ricker_wavelet", "simulate_shot_cpu", "N", "CELLS"]
