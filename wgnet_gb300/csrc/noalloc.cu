// wg_evaluate_adjoint_noalloc: the misfit gradient with every intermediate buffer in one static
// device array, so the call itself allocates no device memory.
//
// Who needs it: a caller whose GPU memory is owned by another allocator cannot call cudaMalloc at
// call time. Examples are a training framework whose caching allocator has reserved the device
// (a cudaMalloc then fails or fragments its pool) and a service that fixes its memory budget at
// start-up and forbids allocation afterwards. The engine (created once, ahead of time) supplies
// the survey's statics; the caller passes inputs and outputs; everything in between lives here.
//
// The array is a file-scope __device__ variable of fixed size, so every GPU that loads this
// library holds it until the process exits. Host code may not use the array's name as a device
// address, so the address is fetched once per device with cudaGetSymbolAddress (on the first call
// on that device, with that device current) and passed to the kernels.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <string>

#include "wave_launch.h"
#include "wgnet_gb300.h"

namespace wg {
EngineView engine_view(wg_engine* e, std::unique_lock<std::mutex>& lock);
int engine_device(const wg_engine* e);
}  // namespace wg

namespace {

constexpr size_t kScratchBytes = size_t(48) << 20;  // 48 MiB
constexpr size_t kAlign = 256;
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_addr_mu;
void* g_addr[kMaxDevices] = {};

size_t up(size_t b) { return (b + kAlign - 1) / kAlign * kAlign; }

}  // namespace

namespace wg {
// Called when an engine is created on `dev`: drops the cached scratch address of that device, so
// that after a cudaDeviceReset (which may reload the module and move the array) the next call
// looks it up again instead of launching on a stale address.
void noalloc_forget_device(int dev) {
  if (dev < 0 || dev >= kMaxDevices) return;
  std::lock_guard<std::mutex> lk(g_addr_mu);
  g_addr[dev] = nullptr;
}
}  // namespace wg

namespace {

// Scratch address on the current device (fetched once per device).
int scratch_address(int dev, void** out) {
  if (dev < 0 || dev >= kMaxDevices) return wg::report_error(WG_ERR_CUDA, "device index out of range");
  std::lock_guard<std::mutex> lk(g_addr_mu);
  if (!g_addr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return wg::report_error(WG_ERR_CUDA, (std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e)).c_str());
    g_addr[dev] = p;
  }
  *out = g_addr[dev];
  return WG_OK;
}

struct Carve {
  size_t vpad, mask, traces, energy, scale, ckpt, stored, adj, gacc, total;
};

// Byte offsets of the buffers of one call with checkpoint interval k (k = nt: no checkpoints).
Carve carve(const wg::EngineView& v, int models, int k) {
  const size_t units = static_cast<size_t>(models) * v.shots;
  const size_t cells = static_cast<size_t>(v.nx) * v.nz;
  const int J = (v.nt + k - 1) / k;
  const int seg = std::min(k, v.nt);
  Carve c{};
  size_t o = 0;
  c.vpad = o;
  o += up(models * cells * 4);
  c.mask = o;
  o += up(models * cells * 4);
  c.traces = o;
  o += up(units * v.nt * v.nrec * 4);
  c.energy = o;
  o += up(models * 8);
  c.scale = o;
  o += up(models * 4);
  c.ckpt = o;
  o += up(units * static_cast<size_t>(J - 1) * wg::ckpt_floats(v.nx, v.nz, v.grid.sw) * 4);
  c.stored = o;
  o += up(units * static_cast<size_t>(seg) * cells * 4);
  c.adj = o;
  o += up(units * wg::adjstate_floats(v.nx, v.nz, v.grid.swa) * 4);
  c.gacc = o;
  o += up(units * cells * 4);
  c.total = o;
  return c;
}

#define NA_LAUNCH(expr)                                                                      \
  do {                                                                                       \
    const cudaError_t e_ = (expr);                                                           \
    wg::note_launch();                                                                       \
    if (e_ != cudaSuccess) return wg::report_error(WG_ERR_CUDA, (std::string(#expr) + ": " + cudaGetErrorString(e_)).c_str()); \
  } while (0)

}  // namespace

extern "C" int wg_evaluate_adjoint_noalloc(wg_engine* eng, const float* d_vel_mps, const float* d_observed,
                                           int models, double* d_loss, float* d_grad, void* stream) {
  if (!eng || !d_vel_mps || !d_observed || !d_loss || !d_grad) return wg::report_error(WG_ERR_ARG, "null argument");
  if (models < 1) return wg::report_error(WG_ERR_ARG, "models must be >= 1");
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return wg::report_error(WG_ERR_CUDA, "cudaGetDevice failed");
  if (dev != wg::engine_device(eng))
    return wg::report_error(WG_ERR_ARG, "the engine belongs to another device: make its device current first");
  void* base = nullptr;
  if (int rc = scratch_address(dev, &base)) return rc;
  std::unique_lock<std::mutex> lock;
  const wg::EngineView v = wg::engine_view(eng, lock);
  if (v.ashape.cluster == 0) return wg::report_error(WG_ERR_UNSUPPORTED, "grid does not fit the adjoint kernel");
  // The engine's checkpoint interval if it fits, else the interval with the smallest footprint.
  int k = (v.ck_every > 0 && v.ck_every < v.nt) ? v.ck_every : v.nt;
  Carve c = carve(v, models, k);
  if (c.total > kScratchBytes) {
    for (int kk = 1; kk <= v.nt; ++kk) {
      const Carve t = carve(v, models, kk);
      if (t.total < c.total) {
        c = t;
        k = kk;
      }
    }
  }
  if (c.total > kScratchBytes)
    return wg::report_error(WG_ERR_ARG, ("wg_evaluate_adjoint_noalloc: " + std::to_string(models) +
                                         " model(s) need " + std::to_string(c.total >> 20) +
                                         " MiB of scratch; the maximum is " + std::to_string(kScratchBytes >> 20) +
                                         " MiB (use fewer models per call)").c_str());
  unsigned char* s = static_cast<unsigned char*>(base);
  float* vpad = reinterpret_cast<float*>(s + c.vpad);
  float* mask = reinterpret_cast<float*>(s + c.mask);
  float* traces = reinterpret_cast<float*>(s + c.traces);
  double* energy = reinterpret_cast<double*>(s + c.energy);
  float* scale = reinterpret_cast<float*>(s + c.scale);
  float* ckpt = reinterpret_cast<float*>(s + c.ckpt);
  float* stored = reinterpret_cast<float*>(s + c.stored);
  float* adj = reinterpret_cast<float*>(s + c.adj);
  float* gacc = reinterpret_cast<float*>(s + c.gacc);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int units = models * v.shots;
  const int J = (v.nt + k - 1) / k;
  const int slots = J - 1;
  const size_t per_model = static_cast<size_t>(v.shots) * v.nt * v.nrec;
  const size_t cells = static_cast<size_t>(v.nx) * v.nz;

  // The status word starts clear; the energy kernel (zero-energy observed data) and the kernels'
  // bounded waits set it, and wg_engine_status reads it once the stream has finished this call.
  {
    const cudaError_t e = cudaMemsetAsync(v.d_status, 0, sizeof(int), st);
    if (e != cudaSuccess) return wg::report_error(WG_ERR_CUDA, cudaGetErrorString(e));
  }
  NA_LAUNCH(wg::launch_pad_velocity(d_vel_mps, models, v.nx_vis, v.nz_vis, v.pad, v.vmin, v.vmax, vpad, mask, st));
  NA_LAUNCH(wg::launch_energy(d_observed, models, per_model, energy, scale, v.d_status, st));
  wg::FwdArgs f{};
  f.g = v.grid;
  f.st = v.stations;
  f.vel = vpad;
  f.units = units;
  f.t0 = 0;
  f.t1 = v.nt;
  f.traces = traces;
  f.status = v.d_status;
  f.fast = v.fast;
  if (slots == 0) {
    // one segment: the first pass keeps every step's gradient term
    f.stored = stored;
    NA_LAUNCH(wg::launch_fwd(v.fshape, true, true, f, st));
  } else {
    // As the allocating entry point does: steps [0, (J-1) k] with receivers and checkpoints, then
    // the last segment from its checkpoint with receivers and stored terms, so the reverse sweep
    // starts without a recompute.
    f.ck_out = ckpt;
    f.ck_every = k;
    f.ck_slots = slots;
    f.t1 = (J - 1) * k + 1;
    NA_LAUNCH(wg::launch_fwd(v.fshape, true, false, f, st));
    wg::FwdArgs l = f;
    l.t0 = (J - 1) * k;
    l.t1 = v.nt;
    l.ck_out = nullptr;
    l.ck_in = ckpt;
    l.ck_in_slot = J - 2;
    l.stored = stored;
    NA_LAUNCH(wg::launch_fwd(v.fshape, true, true, l, st));
  }
  NA_LAUNCH(wg::launch_residual(traces, d_observed, scale, models, per_model, traces, d_loss, st));
  // The accumulator's frame cells are never written by the kernels; the array keeps the previous
  // call's contents, so clear it.
  {
    const cudaError_t e = cudaMemsetAsync(gacc, 0, static_cast<size_t>(units) * cells * 4, st);
    if (e != cudaSuccess) return wg::report_error(WG_ERR_CUDA, cudaGetErrorString(e));
  }
  wg::AdjArgs a{};
  a.g = v.grid;
  a.st = v.stations;
  a.vel = vpad;
  a.units = units;
  a.residual = traces;
  a.stored = stored;
  a.state = adj;
  a.gacc = gacc;
  a.status = v.d_status;
  a.prefetch = v.adj_prefetch;
  for (int j = J - 1; j >= 0; --j) {
    const int t0 = j * k, t1 = std::min(t0 + k, v.nt);
    wg::FwdArgs r{};
    r.g = v.grid;
    r.st = v.stations;
    r.vel = vpad;
    r.units = units;
    r.t0 = t0;
    r.t1 = t1;
    r.ck_in = j > 0 ? ckpt : nullptr;
    r.ck_in_slot = j - 1;
    r.ck_slots = slots;
    r.ck_every = k;
    r.stored = stored;
    r.status = v.d_status;
    r.fast = v.fast;
    if (j < J - 1)  // the last segment's terms are already stored by the first pass
      NA_LAUNCH(wg::launch_fwd(v.fshape, false, true, r, st));
    a.t_hi = t1;
    a.t_lo = t0;
    a.first = (j == J - 1) ? 1 : 0;
    NA_LAUNCH(wg::launch_adj(v.ashape, a, st));
  }
  NA_LAUNCH(wg::launch_fold(gacc, mask, models, v.shots, v.nx, v.nz, v.pad, v.nx_vis, v.nz_vis, d_grad, st));
  return WG_OK;
}
