// Host-side interface of the resident kernels (wave_kernels.cu) and the auxiliary kernels
// (aux_kernels.cu), used by the engine (engine.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <string>

#include "wave_common.cuh"

namespace wg {

constexpr size_t kMaxSmemPerCta = 227 * 1024;

int fwd_shape_count();
int adj_shape_count();
Shape fwd_shape(int i);
Shape adj_shape(int i);
size_t fwd_smem_bytes(const Shape& s, int nx, int nz, int sw, int nrec);
size_t adj_smem_bytes(const Shape& s, int nx, int nz, int swa, int nrec);
bool fwd_shape_fits(const Shape& s, int nx, int nz, int sw, int nrec);
bool adj_shape_fits(const Shape& s, int nx, int nz, int swa, int nrec);

// Per-shape launchers, specialised in the wave_inst_*.cu files.
template <int C, int NT, int CPT>
cudaError_t fwd_dispatch(bool traces, bool store, const FwdArgs& a, size_t smem, cudaStream_t s);
template <int C, int NT, int CPT>
cudaError_t adj_dispatch(const AdjArgs& a, size_t smem, cudaStream_t s);
template <int NX, int PMLP, int C, int S, int NSEG, int NI>
cudaError_t fwd3_dispatch(bool traces, bool store, const FwdArgs& a, size_t smem, cudaStream_t s);
template <int NX, int PMLP, int C, int S, int NSEG, int NI>
cudaError_t adj3_dispatch(const AdjArgs& a, size_t smem, cudaStream_t s);
// fast-arithmetic forward, compiled for the shapes of WG_G3_FAST_SHAPES (wave_table.cu)
template <int NX, int PMLP, int C, int S, int NSEG, int NI>
cudaError_t fwd3f_dispatch(bool traces, bool store, const FwdArgs& a, size_t smem, cudaStream_t s);

// Forward over units = models * shots. traces: record receivers; store: write 2 v dt^2 w.
cudaError_t launch_fwd(const Shape& s, bool traces, bool store, const FwdArgs& a, cudaStream_t stream);
cudaError_t launch_adj(const Shape& s, const AdjArgs& a, cudaStream_t stream);

// --- auxiliary kernels (aux_kernels.cu) ---

// Edge-replicate [models][nz_vis][nx_vis] velocities onto the padded grid, clamp to [vmin, vmax]
// and build the clamp mask (1 where vmin < v < vmax), as wave_wgpu.rs:714-734.
cudaError_t launch_pad_velocity(const float* vis, int models, int nx_vis, int nz_vis, int pad, float vmin, float vmax,
                                float* padded, float* mask, cudaStream_t s);

// Per-model observed energy sum d^2 in f64 and scale = f32(1 / energy); status on energy <= 0.
cudaError_t launch_energy(const float* observed, int models, size_t per_model, double* energy, float* scale,
                          int* status, cudaStream_t s);

// residual[i] = (pred[i] - obs[i]) * scale[model]; loss[model] = sum 0.5 (p-d)^2 scale (f64).
// pred and residual may alias.
cudaError_t launch_residual(const float* pred, const float* observed, const float* scale, int models,
                            size_t per_model, float* residual, double* loss, cudaStream_t s);

// grad[m][vz][vx] = sum over padded cells folding onto (vz, vx) of
//   (sum_s gacc[m][s][cell]) * mask[m][cell]       (f32 shot-sum, f64 fold), wave_wgpu.rs:974-1005.
cudaError_t launch_fold(const float* gacc, const float* mask, int models, int shots, int nx, int nz, int pad,
                        int nx_vis, int nz_vis, float* grad, cudaStream_t s);

// Causal FIR along time: out[b][t][r] = sum_k ker[k] * in[b][t - (K-1) + k][r] (zero before t=0).
cudaError_t launch_bandlimit(const float* in, const float* ker, int klen, int series, int nt, int nrec, float* out,
                             cudaStream_t s);

// Zero-phase FIR (taps ker[0..klen), centre tap `center`) and decimation by `factor` of
// [series][nt][nrec] traces into FP16 [series][nt_out][nrec].
cudaError_t launch_decimate(const float* in, const float* ker, int klen, int center, int factor, int series, int nt,
                            int nrec, int nt_out, void* out_half, cudaStream_t s);

// Error reporting and launch accounting shared by the C ABI entry points (engine.cu).
int report_error(int code, const char* msg);
void note_launch();

// Read-only view of an engine's device statics and launch settings, for entry points that
// sequence the kernels with their own buffers.
struct EngineView {
  Grid grid;
  Stations stations;
  int shots, nt, nrec, nx, nz, nx_vis, nz_vis, pad, ck_every;
  float vmin, vmax, dt;
  Shape fshape, ashape;
  int* d_status;
  int adj_prefetch;
  int fast;    // fast-arithmetic kernels (engine option "arith")
  int tblock;  // streamed path: temporally blocked forward where it applies (engine option "temporal_block")
};

// Event marks around groups of launches (kind 0 forward, 1 forward recompute, 2 adjoint) for the
// engine's per-kernel timing; no-op without a callback.
struct StreamTimer {
  void* ctx = nullptr;
  void (*fn)(void* ctx, int kind, bool begin, cudaStream_t s) = nullptr;
  void mark(int kind, bool begin, cudaStream_t s) const {
    if (fn) fn(ctx, kind, begin, s);
  }
};

// Streamed path (stream.cu): wavefields in HBM, one persistent TMA-pipelined launch per time step.
struct StreamWork;
StreamWork* stream_work_new();
void stream_work_free(StreamWork* w);
bool stream_supported(const EngineView& v, std::string* why);
int stream_simulate(StreamWork* w, const EngineView& v, const int* h_rec_cell, const float* d_vis, int models,
                    float* d_traces, cudaStream_t st, const StreamTimer& timer);
int stream_gradient(StreamWork* w, const EngineView& v, const int* h_rec_cell, const float* d_vis, const float* d_obs,
                    int models, double* d_loss, float* d_grad, cudaStream_t st, const StreamTimer& timer);

// Launch the bounded-wait self-test (stream.cu): one CTA's wait on an mbarrier nothing completes
// gives up after `polls` polls and records ST_CUDA in *d_status.
int wait_timeout_selftest(int* d_status, long long polls, cudaStream_t st);

// out[i] = in[i] * alpha (unit conversion), n elements.
cudaError_t launch_scale(const float* in, float alpha, size_t n, float* out, cudaStream_t s);

}  // namespace wg
