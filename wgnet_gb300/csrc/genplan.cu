// Batched forward data generation: several surveys (one engine per grid size), each with its own
// batch of models, simulated, low-passed and decimated to FP16 gathers by one CUDA graph launch.
//
// The reference writes its wave cache one model at a time (python/wgnet/data.py:138-179:
// `engine.simulate(vel)[:, ::DECIMATE, :]` then `astype(np.float16)`). Here the whole batch is one
// graph: a fork into one branch per survey, and in each branch velocity padding, the resident
// forward kernel over all (model, shot) units of the chunk and the low-pass + decimation kernel,
// then a join. The branches run concurrently, so the small grids fill the SMs that the large
// grids' clusters leave idle at the end of a wave.
//
// Every pointer the kernels use (engine statics, the caller's velocity and output buffers, the
// plan's workspaces) is fixed when the graph is captured: a launch replays the same work on
// whatever the caller's buffers hold at that time. The engines must outlive the plan, and a change
// of an engine's sources or wavelet is not seen by a plan captured before it.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "wave_launch.h"
#include "wgnet_gb300.h"

namespace wg {
EngineView engine_view(wg_engine* e, std::unique_lock<std::mutex>& lock);
int engine_device(const wg_engine* e);
}  // namespace wg

namespace {

struct Buf {
  void* p = nullptr;
  ~Buf() {
    if (p) cudaFree(p);
  }
  int alloc(size_t bytes) {
    if (cudaMalloc(&p, std::max<size_t>(bytes, 16)) != cudaSuccess) {
      cudaGetLastError();
      p = nullptr;
      return wg::report_error(WG_ERR_OOM, ("cudaMalloc(" + std::to_string(bytes) + ") for the generation plan").c_str());
    }
    return WG_OK;
  }
};

struct Group {
  wg::EngineView v{};
  int models = 0, chunk = 0;
  const float* vel = nullptr;  // [models][nz_vis][nx_vis] m/s
  void* out = nullptr;         // [models][shots][nt_out][nrec] half
  Buf vpad, traces;
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
};

}  // namespace

struct wg_gen_plan {
  int device = 0;
  int factor = 1, klen = 0, center = 0, kernels = 0;
  size_t trace_bytes = 0;
  std::vector<float> taps;
  Buf d_taps;
  std::vector<Group> groups;
  cudaStream_t cap = nullptr;
  cudaEvent_t fork = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  ~wg_gen_plan() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    for (auto& g : groups) {
      if (g.done) cudaEventDestroy(g.done);
      if (g.stream) cudaStreamDestroy(g.stream);
    }
    if (fork) cudaEventDestroy(fork);
    if (cap) cudaStreamDestroy(cap);
  }
};

namespace {

#define GP_CK(expr)                                                                                    \
  do {                                                                                                 \
    cudaError_t e_ = (expr);                                                                           \
    if (e_ != cudaSuccess) {                                                                           \
      cudaGetLastError();                                                                              \
      return wg::report_error(WG_ERR_CUDA, (std::string(#expr) + ": " + cudaGetErrorString(e_)).c_str()); \
    }                                                                                                  \
  } while (0)

#define GP_LAUNCH(expr)  \
  do {                   \
    wg::note_launch();   \
    ++p->kernels;        \
    GP_CK(expr);         \
  } while (0)

// lowpass_kernel (python/wgnet/physics.py:18-26): Gaussian with its -3 dB point at fmax, truncated
// at 4 sigma, unit DC gain; f64 arithmetic, f32 taps.
std::vector<float> lowpass_taps(double fmax_hz, double dt) {
  const double sigma = std::sqrt(std::log(2.0) / 2.0) / (3.14159265358979323846 * fmax_hz);
  const int half = static_cast<int>(std::ceil(4.0 * sigma / dt));
  std::vector<double> h(2 * half + 1);
  double sum = 0.0;
  for (int n = -half; n <= half; ++n) {
    const double x = n * dt / sigma;
    h[n + half] = std::exp(-0.5 * (x * x));
    sum += h[n + half];
  }
  std::vector<float> out(h.size());
  for (size_t i = 0; i < h.size(); ++i) out[i] = static_cast<float>(h[i] / sum);
  return out;
}

// Records the work of every group into the capturing stream p->cap (fork/join over the groups'
// streams).
int record(wg_gen_plan* p) {
  GP_CK(cudaEventRecord(p->fork, p->cap));
  for (auto& g : p->groups) {
    if (g.models == 0) continue;
    GP_CK(cudaStreamWaitEvent(g.stream, p->fork, 0));
    const wg::EngineView& v = g.v;
    const int nt_out = (v.nt + p->factor - 1) / p->factor;
    const size_t vis = static_cast<size_t>(v.nx_vis) * v.nz_vis;
    for (int m0 = 0; m0 < g.models; m0 += g.chunk) {
      const int mc = std::min(g.chunk, g.models - m0);
      GP_LAUNCH(wg::launch_pad_velocity(g.vel + m0 * vis, mc, v.nx_vis, v.nz_vis, v.pad, v.vmin, v.vmax,
                                        static_cast<float*>(g.vpad.p), nullptr, g.stream));
      wg::FwdArgs a{};
      a.g = v.grid;
      a.st = v.stations;
      a.vel = static_cast<const float*>(g.vpad.p);
      a.units = mc * v.shots;
      a.t0 = 0;
      a.t1 = v.nt;
      a.traces = static_cast<float*>(g.traces.p);
      a.status = v.d_status;
      a.fast = v.fast;
      GP_LAUNCH(wg::launch_fwd(v.fshape, true, false, a, g.stream));
      auto* out = static_cast<unsigned short*>(g.out) + static_cast<size_t>(m0) * v.shots * nt_out * v.nrec;
      GP_LAUNCH(wg::launch_decimate(static_cast<const float*>(g.traces.p), static_cast<const float*>(p->d_taps.p),
                                    p->klen, p->center, p->factor, mc * v.shots, v.nt, v.nrec, nt_out, out, g.stream));
    }
    GP_CK(cudaEventRecord(g.done, g.stream));
    GP_CK(cudaStreamWaitEvent(p->cap, g.done, 0));
  }
  return WG_OK;
}

int create(wg_engine* const* engines, const int* models, int groups, const float* const* d_vel, void* const* d_out,
           int factor, const float* taps, int klen, float cutoff_hz, size_t budget, wg_gen_plan** out) {
  if (!engines || !models || !d_vel || !d_out || !out || groups < 1 || groups > 64 || factor < 1 || factor > 64 ||
      !(cutoff_hz >= 0.0f) || (taps && (klen < 1 || klen % 2 == 0 || klen > 1 << 16)))
    return wg::report_error(WG_ERR_ARG, "bad argument");
  *out = nullptr;
  auto p = new wg_gen_plan();
  std::unique_ptr<wg_gen_plan> guard(p);
  p->factor = factor;
  GP_CK(cudaGetDevice(&p->device));
  double dt = 0.0;
  size_t per_unit_total = 0;
  p->groups.resize(groups);
  for (int i = 0; i < groups; ++i) {
    if (!engines[i] || models[i] < 0 || (models[i] > 0 && (!d_vel[i] || !d_out[i])))
      return wg::report_error(WG_ERR_ARG, "bad group");
    if (wg::engine_device(engines[i]) != p->device)
      return wg::report_error(WG_ERR_ARG, "every engine must live on the current device");
    Group& g = p->groups[i];
    {
      std::unique_lock<std::mutex> lk;
      g.v = wg::engine_view(engines[i], lk);
    }
    if (i == 0) dt = static_cast<double>(g.v.dt);
    if (static_cast<double>(g.v.dt) != dt) return wg::report_error(WG_ERR_ARG, "every survey must share dt");
    g.models = models[i];
    g.vel = d_vel[i];
    g.out = d_out[i];
    per_unit_total += static_cast<size_t>(g.models) * g.v.shots * g.v.nt * g.v.nrec * 4;
  }
  // Anti-alias filter: the reference's Gaussian low-pass, applied zero-phase. Default cut-off
  // (-3 dB) at 0.4 of the decimated Nyquist frequency; factor 1 with cutoff 0 is a plain cast.
  float fc = cutoff_hz;
  if (fc == 0.0f && factor > 1) fc = static_cast<float>(0.4 * 0.5 / (factor * dt));
  if (taps)
    p->taps.assign(taps, taps + klen);
  else
    p->taps = fc > 0.0f ? lowpass_taps(fc, dt) : std::vector<float>{1.0f};
  p->klen = static_cast<int>(p->taps.size());
  p->center = p->klen / 2;
  // Trace workspace: at most `budget` bytes over all groups (chunks of models otherwise).
  if (budget == 0) budget = size_t(16) << 30;
  const double share = per_unit_total > budget ? static_cast<double>(budget) / per_unit_total : 1.0;
  for (auto& g : p->groups)
    if (g.models > 0) g.chunk = std::max(1, std::min(g.models, static_cast<int>(share * g.models)));
  GP_CK(cudaStreamCreateWithFlags(&p->cap, cudaStreamNonBlocking));
  GP_CK(cudaEventCreateWithFlags(&p->fork, cudaEventDisableTiming));
  for (auto& g : p->groups) {
    GP_CK(cudaStreamCreateWithFlags(&g.stream, cudaStreamNonBlocking));
    GP_CK(cudaEventCreateWithFlags(&g.done, cudaEventDisableTiming));
    if (g.models == 0) continue;
    const size_t cells = static_cast<size_t>(g.v.nx) * g.v.nz;
    int rc = g.vpad.alloc(static_cast<size_t>(g.chunk) * cells * 4);
    if (rc != WG_OK) return rc;
    const size_t tb = static_cast<size_t>(g.chunk) * g.v.shots * g.v.nt * g.v.nrec * 4;
    rc = g.traces.alloc(tb);
    if (rc != WG_OK) return rc;
    p->trace_bytes += tb;
    if ((g.v.nt + factor - 1) / factor > 65535) return wg::report_error(WG_ERR_ARG, "too many output samples");
  }
  {
    int rc = p->d_taps.alloc(p->taps.size() * 4);
    if (rc != WG_OK) return rc;
  }
  GP_CK(cudaMemcpy(p->d_taps.p, p->taps.data(), p->taps.size() * 4, cudaMemcpyHostToDevice));
  GP_CK(cudaStreamBeginCapture(p->cap, cudaStreamCaptureModeRelaxed));
  const int rc = record(p);
  cudaGraph_t graph = nullptr;
  const cudaError_t ec = cudaStreamEndCapture(p->cap, &graph);
  if (rc != WG_OK) {
    if (graph) cudaGraphDestroy(graph);
    return rc;
  }
  if (ec != cudaSuccess) {
    cudaGetLastError();
    return wg::report_error(WG_ERR_CUDA, (std::string("cudaStreamEndCapture: ") + cudaGetErrorString(ec)).c_str());
  }
  p->graph = graph;
  GP_CK(cudaGraphInstantiate(&p->exec, p->graph, 0));
  *out = guard.release();
  return WG_OK;
}

}  // namespace

extern "C" {

int wg_gen_plan_create(wg_engine* const* engines, const int* models, int groups, const float* const* d_vel,
                       void* const* d_out, int factor, const float* taps, int klen, float cutoff_hz,
                       size_t workspace_bytes, wg_gen_plan** out) {
  return create(engines, models, groups, d_vel, d_out, factor, taps, klen, cutoff_hz, workspace_bytes, out);
}

int wg_gen_plan_launch(wg_gen_plan* p, void* stream) {
  if (!p) return wg::report_error(WG_ERR_ARG, "null plan");
  GP_CK(cudaGraphLaunch(p->exec, static_cast<cudaStream_t>(stream)));
  return WG_OK;
}

int wg_gen_plan_info(const wg_gen_plan* p, int* kernels, size_t* trace_bytes, float* taps, int taps_cap, int* klen) {
  if (!p) return wg::report_error(WG_ERR_ARG, "null plan");
  if (kernels) *kernels = p->kernels;
  if (trace_bytes) *trace_bytes = p->trace_bytes;
  if (klen) *klen = p->klen;
  if (taps)
    for (int i = 0; i < std::min(taps_cap, p->klen); ++i) taps[i] = p->taps[i];
  return WG_OK;
}

void wg_gen_plan_destroy(wg_gen_plan* p) { delete p; }

int wg_lowpass_taps(double fmax_hz, double dt, float* out, int cap) {
  if (!(fmax_hz > 0.0) || !(dt > 0.0) || !(4.0 * std::sqrt(std::log(2.0) / 2.0) / (3.14159265358979323846 * fmax_hz) / dt < 1.0e6))
    return -wg::report_error(WG_ERR_ARG, "bad low-pass parameters");
  const std::vector<float> t = lowpass_taps(fmax_hz, dt);
  if (out && cap >= static_cast<int>(t.size()))
    for (size_t i = 0; i < t.size(); ++i) out[i] = t[i];
  return static_cast<int>(t.size());
}

}  // extern "C"
