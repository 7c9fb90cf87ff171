"""CPU oracle for the WGNet physics path. TEST INFRASTRUCTURE ONLY.

Only `tests/`, `__graft_entry__.smoke()` and the CPU-baseline leg of `bench.py` may import this
package, and only as the checker (or the timed CPU baseline) — never as the thing measured or
shipped. The product (`wgnet_gb300`, `wave_gauss_rs`) never imports it.

Contents
--------
* `wave_oracle.cpp` (+ `Makefile`, loaded by `native.py`): C++ restatement of the reference's
  CPU solver (crates/geology-core/src/lib.rs) and of the wgpu engine's forward/adjoint/residual/
  fold semantics (crates/wave-gauss-rs/src/shaders/*.wgsl, src/wave_wgpu.rs), in f32 and f64.
* `wgsl_np.py`: an independent vectorised numpy restatement of the two WGSL shaders, used to
  cross-check the C++ restatement on small cases.
* `physics_np.py`: numpy restatement of `lowpass_kernel` / `set_band` / `bandlimit`
  (python/wgnet/physics.py:18-57).
* `render_np.py`: numpy restatement of the Gaussian renderer forward and its analytic backward
  (python/wgnet/render.py:34-109).
* `refine_np.py`: restatement of the L-BFGS two-loop recursion (python/wgnet/refine.py:41-53).

Parity pinning
--------------
The reference crates cannot be compiled in this environment (no Rust toolchain), and the reference
ships no golden vectors. The forward/adjoint restatement is pinned by the reference's own
known-answer tests (lib.rs:227-251, wave_wgpu.rs:1023-1108), by agreement of two independent
restatements (C++ of the CPU solver vs numpy of the WGSL shaders), and by the adjoint's own
mathematical properties (dot-product test, FP64 finite differences). The Python parts
(renderer, low-pass, L-BFGS direction) are pinned bit-for-bit-tolerance against golden fixtures
generated by importing the reference Python (`tests/golden/make_golden.py`).
"""
