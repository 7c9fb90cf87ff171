"""wgnet_gb300: GB300-native (sm_103a) physics hot path of WGNet.

The 4th-order C-PML acoustic forward solver and its exact discrete adjoint, the normalized misfit
with its causal low-pass band schedule, and the additive Gaussian renderer, as hand-written CUDA
kernels behind the reference's own Python interfaces:

* `wgnet_gb300.wave_gauss_rs` (also importable as top-level `wave_gauss_rs`): the PyO3 module's
  `ricker_wavelet`, `simulate_shot_cpu`, `PyWaveEngine`;
* `wgnet_gb300.physics`: `WavePhysics`, `lowpass_kernel`, plus `WaveLoss` (autograd);
* `wgnet_gb300.render`: `render_residual` and its helpers;
* `wgnet_gb300.engine.WaveEngine`: the batched engine (numpy and CUDA-tensor entry points).

The CUDA library is built by `python -m wgnet_gb300.build`; nothing here falls back to the CPU.
"""

__version__ = "0.1.0"

__all__ = ["__version__"]
