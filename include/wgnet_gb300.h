/*
 * wgnet_gb300 C ABI: the GB300 (sm_103a) wave engine behind WGNet's `wave_gauss_rs` interface.
 *
 * Plain C: opaque handles, plain pointers and sizes, int status codes (0 = success). On failure
 * `wg_last_error()` returns a message for the calling thread. Entry points ending in `_dev` take
 * device pointers and a cudaStream_t (passed as void*; NULL = the CUDA default stream) and are
 * asynchronous on that stream; the others take host pointers, run on the engine's own stream and
 * block until their results are on the host.
 *
 * Each declaration names the reference interface it replaces (file:line in arthifact/WGNet).
 */
#ifndef WGNET_GB300_H
#define WGNET_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. */
#define WG_OK 0
#define WG_ERR_ARG 1          /* bad argument, shape or length (reference: PyValueError) */
#define WG_ERR_CUDA 2         /* CUDA runtime error or no usable GPU */
#define WG_ERR_NONFINITE 3    /* non-finite input */
#define WG_ERR_ENERGY 4       /* observed traces have zero energy (reference: wave_wgpu.rs:853 panic) */
#define WG_ERR_UNSUPPORTED 5  /* grid too large for the resident kernels */
#define WG_ERR_CFL 6
#define WG_ERR_OOM 7          /* device allocation failed */

/* Engine configuration: the arguments of PyWaveEngine(shots, nt, dt, peak_hz, pml, vmin, vmax)
 * (crates/wave-gauss-rs/src/lib.rs:51-57), plus the visible grid and spacing that the reference
 * hard-wires (crates/geology-core/src/lib.rs:5-9: 70 x 70, 10 m). Zero in nx_vis/nz_vis/h/nrec
 * selects the reference's value (70, 70, 10 m, one receiver per surface cell). */
typedef struct wg_config {
  int shots;
  int nt;
  float dt;
  float peak_hz;
  int pml;
  float vmin;
  float vmax;
  int nx_vis;
  int nz_vis;
  float h;
  int nrec;
} wg_config;

typedef struct wg_engine wg_engine;

/* NativeWaveEngine::new (crates/wave-gauss-rs/src/wave_wgpu.rs:144-712): geometry (bilinear
 * source/receiver corners, receiver CSR), C-PML profiles, Ricker wavelet, device statics. */
int wg_engine_create(const wg_config* cfg, wg_engine** out);
void wg_engine_destroy(wg_engine* eng);

/* Read-only properties `shots`, `nt`, `nrec` (lib.rs:59-72) and the padded grid. */
int wg_engine_dims(const wg_engine* eng, int* shots, int* nt, int* nrec, int* nx, int* nz, int* nx_vis,
                   int* nz_vis);

/* PyWaveEngine.sources / set_sources: [shots][2] (x, z) in metres (lib.rs:74-90,
 * wave_wgpu.rs:761-785). `n` must equal shots. */
int wg_get_sources(const wg_engine* eng, float* out, int n);
int wg_set_sources(wg_engine* eng, const float* xz, int n);

/* PyWaveEngine.wavelet / set_wavelet: [nt] (lib.rs:92-106, wave_wgpu.rs:788-795). */
int wg_get_wavelet(const wg_engine* eng, float* out, int n);
int wg_set_wavelet(wg_engine* eng, const float* w, int n);

/* PyWaveEngine.simulate (lib.rs:108-116, wave_wgpu.rs:799-844) for `models` velocity models
 * [models][nz_vis][nx_vis] in m/s -> traces [models][shots][nt][nrec]. */
int wg_simulate(wg_engine* eng, const float* vel_mps, int models, float* traces);
int wg_simulate_dev(wg_engine* eng, const float* d_vel_mps, int models, float* d_traces, void* stream);

/* PyWaveEngine.evaluate_adjoint (lib.rs:118-137, wave_wgpu.rs:848-988) for `models` models:
 * observed [models][shots][nt][nrec]; loss[m] = 0.5 |p - d|^2 / |d|^2 (f64), grad [models][nz_vis]
 * [nx_vis] = dloss/d(v in m/s), zero where v is clamped, folded onto the visible grid. */
int wg_evaluate_adjoint(wg_engine* eng, const float* vel_mps, const float* observed, int models, double* loss,
                        float* grad);
int wg_evaluate_adjoint_dev(wg_engine* eng, const float* d_vel_mps, const float* d_observed, int models,
                            double* d_loss, float* d_grad, void* stream);

/* Device status of the engine's last device-pointer call (wg_simulate_dev,
 * wg_evaluate_adjoint_dev, wg_evaluate_adjoint_noalloc), which clear it when they start: waits for
 * `stream`, then returns WG_OK, WG_ERR_ENERGY (observed traces with zero energy: the reference's
 * `assert!(energy > 0)` panic, wave_wgpu.rs:853) or WG_ERR_CUDA (a kernel's bounded wait timed
 * out), with the message in wg_last_error(). The host-pointer entry points check it themselves. */
int wg_engine_status(wg_engine* eng, void* stream);

/* Self-test of the time-out path that wg_engine_status reports: clears the engine's status word
 * and launches, on `stream`, one CTA whose bounded mbarrier wait (the wait the streamed kernels use
 * for their TMA copies) waits for a copy that is never issued. The wait gives up after `polls`
 * polls (1 .. 2^22; the kernels use 2^22), records the error and the kernel returns: no fault, no
 * hang, the context stays usable. wg_engine_status then returns WG_ERR_CUDA. No reference
 * counterpart. */
int wg_selftest_wait_timeout(wg_engine* eng, long long polls, void* stream);

/* Wavefield checkpoint interval for evaluate_adjoint: snapshots every k steps, segments recomputed
 * in reverse. k >= nt stores the gradient term of every step (the reference's scheme,
 * wave_wgpu.rs:181-182); so does k <= 0 on the resident path, while on the streamed path k <= 0
 * (its default) stores every step when that fits in 70% of the free device memory and otherwise
 * picks the interval that fits. No reference counterpart for k > 0. */
int wg_set_checkpoint_interval(wg_engine* eng, int k);
int wg_get_checkpoint_interval(const wg_engine* eng);

/* Named tuning options: "checkpoint_every" (as wg_set_checkpoint_interval), "adjoint_prefetch"
 * (0/1: the column-pair adjoint fetches the next step's stored terms one step ahead), "streamed"
 * (0/1: wavefields in device memory and one launch per time step instead of the resident
 * kernels; engines whose grid fits no resident kernel start with 1; needs a padded width
 * nx_vis + 2 (pml + 2) divisible by 4), "arith" (0, the default: every f32 operation in the
 * reference's order, unfused, so results equal the reference's bit for bit; 1: the forward
 * kernels compute the same discrete operator with 1/h folded into the stencil weights and fused
 * multiply-adds, faster and equal to f32 accuracy, on the resident kernels of the default 70x70,
 * 100x100 and 140x140 shapes; the adjoint, other shapes and the streamed path keep the unfused
 * arithmetic), "temporal_block" (0/1, default 0; 1: on the streamed path, forward passes that
 * start from the zero state and need no checkpoints (simulate, and the gradient's forward when
 * every step's gradient term is kept) advance each tile 4 steps per launch from a halo of 8 cells
 * held in shared memory, with identical results; slower than the per-step kernels on the 800x300
 * survey, whose per-step forward is not bandwidth-bound). No reference counterpart. */
int wg_set_option(wg_engine* eng, const char* key, int value);
int wg_get_option(const wg_engine* eng, const char* key, int* value);

/* Launch shape of the resident kernels (which = 0 forward, 1 adjoint): CTAs per (model, shot)
 * cluster, threads per CTA, cells-per-thread bound. wg_shape_candidates lists the compiled
 * shapes that fit this engine's grid. No reference counterpart (wgpu dispatches 16x16 tiles). */
int wg_set_launch_shape(wg_engine* eng, int which, int cluster, int threads, int cpt);
int wg_get_launch_shape(const wg_engine* eng, int which, int* cluster, int* threads, int* cpt);
int wg_shape_candidates(const wg_engine* eng, int which, int* out3, int max_shapes);

/* geology_core::simulate_shot_cpu via PyO3 (crates/wave-gauss-rs/src/lib.rs:17-42,
 * crates/geology-core/src/lib.rs:70-221): one shot, receivers at every surface node, d2 scaled by
 * rh*rh precomputed as in the CPU solver. Runs on the GPU; out [nt][nx_vis]. */
int wg_simulate_shot(const float* vel_mps, int nx_vis, int nz_vis, float h, float dt, int nt, int pml, float vmin,
                     float vmax, float peak_hz, float src_x, float src_z, float* out);

/* geology_core::ricker_wavelet (lib.rs:11-21) and cpml_profiles (lib.rs:23-68), host side. */
int wg_ricker_wavelet(int samples, float dt, float peak_hz, float* out);
int wg_cpml_profiles(int n, float h, float dt, int width, float max_vel, float freq, float* a, float* b, float* db);

/* WavePhysics.bandlimit (python/wgnet/physics.py:48-57): causal FIR of `klen` taps along time for
 * `series` blocks of [nt][nrec] traces, zero history before t = 0. Device pointers. */
int wg_bandlimit_dev(const float* d_in, const float* d_kernel, int klen, int series, int nt, int nrec, float* d_out,
                     void* stream);

/* Wave-cache writer step (python/wgnet/data.py:138-179, which decimates by plain subsampling
 * `[:, ::8, :]` and stores float16): zero-phase FIR low-pass (taps d_kernel[0..klen), centre tap
 * `center`) then decimation by `factor`, [series][nt][nrec] f32 -> [series][ceil(nt/factor)][nrec]
 * IEEE half. Device pointers. */
int wg_lowpass_decimate_f16_dev(const float* d_in, const float* d_kernel, int klen, int center, int factor, int series,
                                int nt, int nrec, void* d_out, void* stream);

/* Batched forward data generation (the wave-cache writer, python/wgnet/data.py:138-179, for many
 * models and several grid sizes at once). Group i simulates models[i] models with engines[i]
 * (velocities d_vel[i], [models][nz_vis][nx_vis] m/s, device) and writes low-passed, decimated
 * IEEE-half gathers to d_out[i], [models][shots][ceil(nt/factor)][nrec] (device). The low-pass is
 * the FIR `taps` (host, odd length klen, applied zero-phase about the centre tap) or, when taps is
 * NULL, physics.py's Gaussian lowpass_kernel with its -3 dB point at cutoff_hz (0: 0.4 x the
 * decimated Nyquist frequency; factor 1 with cutoff 0 is a plain cast). The work of all groups is
 * captured into one CUDA graph, one branch per group, at creation: buffers and engine statics are
 * fixed then, and wg_gen_plan_launch replays it on `stream` (NULL = default stream). Engines must
 * outlive the plan and share dt. workspace_bytes bounds the f32 trace workspace (0: 16 GiB);
 * larger batches are processed in chunks inside the graph. */
typedef struct wg_gen_plan wg_gen_plan;
int wg_gen_plan_create(wg_engine* const* engines, const int* models, int groups, const float* const* d_vel,
                       void* const* d_out, int factor, const float* taps, int klen, float cutoff_hz,
                       size_t workspace_bytes, wg_gen_plan** out);
int wg_gen_plan_launch(wg_gen_plan* plan, void* stream);
/* Kernels per launch, trace workspace bytes, and the filter taps (up to taps_cap of *klen). */
int wg_gen_plan_info(const wg_gen_plan* plan, int* kernels, size_t* trace_bytes, float* taps, int taps_cap, int* klen);
void wg_gen_plan_destroy(wg_gen_plan* plan);
/* lowpass_kernel (python/wgnet/physics.py:18-26) on the host, with the C library's exp (which may
 * differ from numpy's in the last bit of a tap): returns the tap count n and writes the taps when
 * out != NULL and cap >= n; negative status on bad arguments. */
int wg_lowpass_taps(double fmax_hz, double dt, float* out, int cap);

/* Tensor-core GEMM used by the learned update network's convolutions (no reference counterpart):
 * d_d[z][m][n] = sum over k in split z of A[m][k] * B[n][k], A [m][k] and B [n][k] row-major IEEE
 * bfloat16 (16-byte aligned), FP32 accumulation and output; k a positive multiple of 64, n a
 * multiple of 4; splits > 1 partitions k and writes one [m][n] partial per split. d_status
 * receives an error code if a pipeline wait times out. */
int wg_gemm_bf16_dev(const void* d_a, const void* d_b, float* d_d, int m, int n, int k, int splits, int* d_status,
                     void* stream);

/* FP64 reductions of the batched refinement (python/wgnet/refine.py:41-53): the L-BFGS two-loop
 * direction dir[b] = -H_b grad[b] from `count[b]` (<= cap) curvature pairs per model stored
 * oldest first in s/y [models][cap][params], rho [models][cap]; and per-model dot products. One
 * block per model, fixed reduction order. Device pointers. */
int wg_lbfgs_direction_dev(const double* d_grad, const double* d_s, const double* d_y, const double* d_rho,
                           const int* d_count, int models, int cap, long params, double* d_dir, void* stream);
int wg_dot_f64_dev(const double* d_a, const double* d_b, int models, long params, double* d_out, void* stream);
/* Per-model misfit 0.5 sum (p - d)^2 / sum d^2 in f64 over per_model values (refine.py:100-104). */
int wg_misfit_dev(const float* d_pred, const float* d_obs, int models, long per_model, double* d_loss, void* stream);

/* Learned update network kernels (no reference counterpart). Activations [B][H][W][C] with
 * channels contiguous; im2col columns [B H W][Kp] bf16 with k = (3 ky + kx) C + c for the 3x3 taps
 * at dilation dil (zero outside the grid and for k >= 9 C); weights [N][Kp] bf16 and their
 * transpose [Kp][N]. All pointers are device pointers; stream NULL = default stream. */
int wg_pc_im2col(const void* d_act_bf16, int batch, int h, int w, int c, int dil, int kp, void* d_col_bf16,
                 void* stream);
/* dact[m][c] (+)= sum over taps of dcol[m'][tap c_count + c] (m' = the pixel whose tap reads m). */
int wg_pc_col2im(const float* d_dcol, int batch, int h, int w, int c, int dil, int kp, float* d_dact, int accumulate,
                 void* stream);
int wg_pc_transpose_bf16(const void* d_in, long rows, int cols, void* d_out, void* stream);
/* out[r][c] = bf16(relu ? max(x[r][c], 0) : x[r][c]) for the first `cols` of rows of ld floats. */
int wg_pc_cast_bf16(const float* d_x, long rows, int ld, int cols, int relu, void* d_out, void* stream);
/* out = a + b (f32) and, if d_out_bf16 != NULL, its bf16 copy. */
int wg_pc_add(const float* d_a, const float* d_b, long n, float* d_out, void* d_out_bf16, void* stream);
/* out = d where the bf16 activation mask > 0, else 0. */
int wg_pc_relu_grad(const float* d_d, const void* d_mask_bf16, long n, float* d_out, void* stream);
/* Input features [B][h][w][8] bf16: v - 3 (km/s), gradient / its per-sample RMS (written to d_rms),
 * one-hot band index (4), depth row / h, 0. */
int wg_pc_features(const float* d_vel_km, const float* d_grad, const int* d_band, int batch, int h, int w,
                   float* d_rms, void* d_out_bf16, void* stream);
/* Mean over m of (scale out[m][0] - target[m])^2 added to *d_loss (f64); d_dout[m][0] = its
 * derivative (other columns untouched). */
int wg_pc_mse(const float* d_out, int ld, const float* d_target, float scale, long m, double* d_loss, float* d_dout,
              void* stream);
/* Adam step on FP32 master weights [n][kp] with the gradient = sum of `splits` partials of its
 * transpose [splits][kp][n]; writes the bf16 weights and their transpose. d_partial NULL: only
 * refresh the bf16 copies. */
int wg_pc_adam(const float* d_partial, int splits, int n, int kp, float* d_w32, float* d_m1, float* d_m2, float lr,
               float b1, float b2, float eps, int step, void* d_w_bf16, void* d_wt_bf16, void* stream);

/* render_residual (python/wgnet/render.py:86-109): activated slot parameters [B][1225][6] ->
 * residual field [B][70][70] in km/s; and its vector-Jacobian product: cotangent [B][70][70] ->
 * parameter gradient [B][1225][6]. Device pointers. */
int wg_render_fwd_dev(const float* d_params, int batch, float* d_field, void* stream);
int wg_render_bwd_dev(const float* d_params, const float* d_cot, int batch, float* d_grad, void* stream);

/* Per-kernel timing with CUDA events on the launching stream. wg_profile(eng, 1) starts
 * recording (and clears earlier records); wg_profile_read fills ms[k] and launches[k] for kinds
 * k = 0 forward (with receivers), 1 forward recompute (stored terms), 2 adjoint, and clears.
 * No reference counterpart (wgpu timestamp_writes are off in the reference). */
int wg_profile(wg_engine* eng, int enable);
int wg_profile_read(wg_engine* eng, double* ms, long long* launches, int kinds);

/* evaluate_adjoint that allocates nothing: no counterpart in the reference. For callers that
 * cannot call cudaMalloc at call time because another allocator owns the GPU's memory (a
 * framework's caching allocator that reserved the device, a service with a fixed memory budget).
 * Same inputs and outputs as wg_evaluate_adjoint_dev (device pointers, caller's stream); all
 * intermediates live in one static 48 MiB device array that the library holds on every GPU that
 * loads it until the process exits. Sizes needing more scratch (33 MiB for one 70x70 5-shot
 * model at nt = 1000 and checkpoint interval 50, so one such model per call) are rejected with
 * WG_ERR_ARG; when the engine's interval does not fit, the interval with the smallest footprint
 * is used (the gradient is the same). The first call on a device after an engine was created
 * there looks up the array's address (make that call before any stream capture); creating an
 * engine drops the cached address, so a cudaDeviceReset followed by a new engine is safe. Calls
 * share the array: calls that overlap on the GPU (other streams, other threads) race and corrupt
 * each other's results. Read the call's device status with wg_engine_status. */
int wg_evaluate_adjoint_noalloc(wg_engine* eng, const float* d_vel_mps, const float* d_observed, int models,
                                double* d_loss, float* d_grad, void* stream);

/* Message of the last failing call on this thread ("" if none). */
const char* wg_last_error(void);

/* Number of kernel launches this library issued on this thread since the last reset. */
long long wg_launch_count(int reset);

#ifdef __cplusplus
}
#endif

#endif /* WGNET_GB300_H */
