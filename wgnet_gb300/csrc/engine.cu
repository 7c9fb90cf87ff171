// Host side of the wave engine and the C ABI (include/wgnet_gb300.h).
//
// The engine owns the static data of one survey (C-PML profiles, wavelet, station geometry) on the
// device and a growable workspace, and sequences the kernels of wave_kernels.cu / aux_kernels.cu:
//
//   simulate:          pad -> forward (receivers)
//   evaluate_adjoint:  pad -> energy -> forward (receivers + checkpoints) -> residual/misfit
//                      -> for each segment, last to first: forward recompute (stored terms)
//                         -> adjoint -> shot-sum / mask / fold
//
// mirroring NativeWaveEngine (crates/wave-gauss-rs/src/wave_wgpu.rs:143-989), with every
// (model, shot) of a batch in one launch instead of one dispatch per time step.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "wave_launch.h"
#include "wgnet_gb300.h"

namespace {

thread_local std::string g_err;
thread_local long long g_launches = 0;

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

#define WG_CK(expr)                                                                              \
  do {                                                                                           \
    cudaError_t e_ = (expr);                                                                     \
    if (e_ != cudaSuccess) return fail(WG_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
  } while (0)

#define WG_LAUNCH(expr)                                                                          \
  do {                                                                                           \
    cudaError_t e_ = (expr);                                                                     \
    ++g_launches;                                                                                \
    if (e_ != cudaSuccess) return fail(WG_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
  } while (0)

#define WG_TRY(expr)          \
  do {                        \
    int rc_ = (expr);         \
    if (rc_ != WG_OK) return rc_; \
  } while (0)

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  ~DevBuf() {
    if (p) cudaFree(p);
  }
  int ensure(size_t need) {
    if (need <= bytes) return WG_OK;
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
    cudaError_t e = cudaMalloc(&p, need);
    if (e != cudaSuccess) {
      cudaGetLastError();
      p = nullptr;
      return fail(WG_ERR_OOM, std::string("cudaMalloc(") + std::to_string(need) + "): " + cudaGetErrorString(e));
    }
    bytes = need;
    return WG_OK;
  }
  template <typename T>
  T* as() const {
    return static_cast<T*>(p);
  }
};

constexpr int FD = wg::FD_PAD;

// geology_core::ricker_wavelet (crates/geology-core/src/lib.rs:11-21): delay 1.5 / peak_hz.
void ricker(int samples, float dt, float peak_hz, float* out) {
  const float delay = 1.5f / peak_hz;
  const float pi = 3.14159265358979323846f;
  for (int i = 0; i < samples; ++i) {
    const float t = static_cast<float>(i) * dt - delay;
    const float u = pi * peak_hz * t;
    const float a = u * u;
    out[i] = (1.0f - 2.0f * a) * std::exp(-a);
  }
}

// geology_core::cpml_profiles (lib.rs:23-68): quadratic sigma ramp, linear alpha, f64 inside.
void cpml(int n, float h, float dt, int width, float max_vel, float freq, float* a_out, float* b_out, float* db_out) {
  std::vector<double> a(n), b(n), db(n, 0.0);
  const double w = static_cast<double>(width), hf = static_cast<double>(h), dtf = static_cast<double>(dt);
  const double lo = static_cast<double>(FD + width), hi = static_cast<double>(n - 1 - FD - width);
  const double sigma0 = -(3.0 * static_cast<double>(max_vel) * std::log(0.001)) / (2.0 * w * hf);
  for (int x = 0; x < n; ++x) {
    const double xf = static_cast<double>(x);
    const double frac = std::min(std::max(std::max((lo - xf) / w, (xf - hi) / w), 0.0), 1.0);
    const double sigma = sigma0 * frac * frac;
    const double alpha = 3.14159265358979323846 * static_cast<double>(freq) * (1.0 - frac);
    const double e = std::exp(-(sigma + alpha) * dtf);
    b[x] = (sigma / (sigma + alpha)) * (e - 1.0);
    a[x] = (frac == 0.0) ? 0.0 : e;
  }
  for (int x = 2; x + 2 < n; ++x)
    db[x] = ((8.0 / 12.0) * (b[x + 1] - b[x - 1]) - (1.0 / 12.0) * (b[x + 2] - b[x - 2])) / hf;
  for (int x = 0; x < n; ++x) {
    a_out[x] = static_cast<float>(a[x]);
    b_out[x] = static_cast<float>(b[x]);
    db_out[x] = static_cast<float>(db[x]);
  }
}

// Rust `f32 as usize`: saturating, NaN -> 0.
long to_index(float v) {
  if (!(v > 0.0f)) return 0;
  if (v >= 1.0e9f) return 1000000000L;
  return static_cast<long>(v);
}

}  // namespace

namespace wg {
int report_error(int code, const char* msg) { return fail(code, msg); }
void note_launch() { ++g_launches; }
void noalloc_forget_device(int dev);  // noalloc.cu
}  // namespace wg

struct wg_engine {
  wg_config cfg{};
  int shots = 0, nt = 0, nrec = 0, nx_vis = 0, nz_vis = 0, pad = 0, nx = 0, nz = 0, cells = 0;
  int sw = 0, swa = 0, region = 0, region_adj = 0;
  float h = 0, rh = 0, dt2 = 0, d2a = 0, d2b = 0;
  std::vector<float> prof, sources, receivers, wavelet;
  std::vector<int> src_cell, rec_cell, csr, ent_rec;
  std::vector<float> src_w, rec_w, ent_w;
  int device = 0;
  cudaStream_t stream = nullptr;
  DevBuf d_prof, d_wavelet, d_src_cell, d_src_w, d_rec_cell, d_rec_w, d_csr, d_ent_rec, d_ent_w, d_status;
  wg::Shape fshape{0, 0, 0}, ashape{0, 0, 0};
  int ck_every = 50;
  int adj_prefetch = 1;
  int fast = 0;      // 1: fast-arithmetic resident kernels (option "arith")
  int tblock = 0;    // streamed path: temporally blocked forward (option "temporal_block")
  int streamed = 0;  // 1: wavefields in HBM, one launch per step (grids beyond the resident kernels)
  cudaStream_t copy_stream = nullptr;  // host->device copy of observed data, overlapping the forward
  cudaEvent_t obs_ready = nullptr;
  wg::StreamWork* swork = nullptr;
  // per-kernel timing: (kind, start, stop) events recorded on the launching stream
  bool prof_on = false;
  std::vector<int> prof_kind;
  std::vector<cudaEvent_t> prof_ev;
  size_t prof_used = 0;
  // workspace
  DevBuf w_vis, w_obs, w_vpad, w_mask, w_traces, w_energy, w_scale, w_loss, w_grad, w_ckpt, w_stored, w_adj, w_gacc;
  std::mutex mu;

  wg::Grid grid() const {
    wg::Grid g;
    g.nx = nx;
    g.nz = nz;
    g.pml = cfg.pml;
    g.region = region;
    g.region_adj = region_adj;
    g.sw = sw;
    g.swa = swa;
    g.rh = rh;
    g.dt2 = dt2;
    g.d2a = d2a;
    g.d2b = d2b;
    g.nt = nt;
    g.prof = d_prof.as<float>();
    g.wavelet = d_wavelet.as<float>();
    return g;
  }
  wg::Stations stations() const {
    wg::Stations s;
    s.shots = shots;
    s.nrec = nrec;
    s.src_cell = d_src_cell.as<int>();
    s.src_w = d_src_w.as<float>();
    s.rec_cell = d_rec_cell.as<int>();
    s.rec_w = d_rec_w.as<float>();
    s.csr = d_csr.as<int>();
    s.ent_rec = d_ent_rec.as<int>();
    s.ent_w = d_ent_w.as<float>();
    return s;
  }
};

namespace {

// The engine's device statics and launch settings (the caller holds the engine's lock).
wg::EngineView view_of(const wg_engine* e) {
  wg::EngineView v;
  v.grid = e->grid();
  v.stations = e->stations();
  v.shots = e->shots;
  v.nt = e->nt;
  v.nrec = e->nrec;
  v.nx = e->nx;
  v.nz = e->nz;
  v.nx_vis = e->nx_vis;
  v.nz_vis = e->nz_vis;
  v.pad = e->pad;
  v.ck_every = e->ck_every;
  v.vmin = e->cfg.vmin;
  v.vmax = e->cfg.vmax;
  v.dt = e->cfg.dt;
  v.fshape = e->fshape;
  v.ashape = e->ashape;
  v.d_status = e->d_status.as<int>();
  v.adj_prefetch = e->adj_prefetch;
  v.fast = e->fast;
  v.tblock = e->tblock;
  return v;
}

// Bilinear corners of a station (wave_wgpu.rs:217-230): x0 = min(floor(gx), nx - 2).
void corners(const wg_engine& e, float px, float pz, int* cell, float* w) {
  const float gx = px / e.h + static_cast<float>(e.pad);
  const float gz = pz / e.h + static_cast<float>(e.pad);
  const long x0 = std::min(to_index(std::floor(gx)), static_cast<long>(e.nx - 2));
  const long z0 = std::min(to_index(std::floor(gz)), static_cast<long>(e.nz - 2));
  const float fx = gx - static_cast<float>(x0);
  const float fz = gz - static_cast<float>(z0);
  cell[0] = static_cast<int>(z0 * e.nx + x0);
  cell[1] = static_cast<int>(z0 * e.nx + x0 + 1);
  cell[2] = static_cast<int>((z0 + 1) * e.nx + x0);
  cell[3] = static_cast<int>((z0 + 1) * e.nx + x0 + 1);
  w[0] = (1.0f - fx) * (1.0f - fz);
  w[1] = fx * (1.0f - fz);
  w[2] = (1.0f - fx) * fz;
  w[3] = fx * fz;
}

template <typename T>
int upload(DevBuf& b, const std::vector<T>& v) {
  WG_TRY(b.ensure(std::max<size_t>(v.size(), 1) * sizeof(T)));
  if (!v.empty()) WG_CK(cudaMemcpy(b.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
  return WG_OK;
}

int set_sources_impl(wg_engine* e, const float* xz) {
  e->sources.assign(xz, xz + 2 * e->shots);
  e->src_cell.resize(4 * e->shots);
  e->src_w.resize(4 * e->shots);
  for (int s = 0; s < e->shots; ++s) corners(*e, xz[2 * s], xz[2 * s + 1], &e->src_cell[4 * s], &e->src_w[4 * s]);
  WG_TRY(upload(e->d_src_cell, e->src_cell));
  WG_TRY(upload(e->d_src_w, e->src_w));
  return WG_OK;
}

// Receivers at (k h, h) for k < nrec (wave_wgpu.rs:215) and the per-cell CSR of their corners with
// non-zero weight, ordered by (cell, receiver) (wave_wgpu.rs:232-270).
int set_receivers_impl(wg_engine* e) {
  e->rec_cell.resize(4 * e->nrec);
  e->rec_w.resize(4 * e->nrec);
  e->receivers.resize(2 * e->nrec);
  for (int r = 0; r < e->nrec; ++r) {
    e->receivers[2 * r] = static_cast<float>(r) * e->h;
    e->receivers[2 * r + 1] = e->h;
    corners(*e, e->receivers[2 * r], e->receivers[2 * r + 1], &e->rec_cell[4 * r], &e->rec_w[4 * r]);
  }
  struct Ent {
    int cell, rec;
    float w;
  };
  std::vector<Ent> ents;
  for (int r = 0; r < e->nrec; ++r)
    for (int k = 0; k < 4; ++k)
      if (e->rec_w[4 * r + k] != 0.0f) ents.push_back({e->rec_cell[4 * r + k], r, e->rec_w[4 * r + k]});
  std::stable_sort(ents.begin(), ents.end(),
                   [](const Ent& a, const Ent& b) { return a.cell != b.cell ? a.cell < b.cell : a.rec < b.rec; });
  e->csr.assign(e->cells + 1, 0);
  size_t k = 0;
  for (int c = 0; c <= e->cells; ++c) {
    while (k < ents.size() && ents[k].cell < c) ++k;
    e->csr[c] = static_cast<int>(k);
  }
  e->ent_rec.clear();
  e->ent_w.clear();
  for (const Ent& en : ents) {
    e->ent_rec.push_back(en.rec);
    e->ent_w.push_back(en.w);
  }
  WG_TRY(upload(e->d_rec_cell, e->rec_cell));
  WG_TRY(upload(e->d_rec_w, e->rec_w));
  WG_TRY(upload(e->d_csr, e->csr));
  WG_TRY(upload(e->d_ent_rec, e->ent_rec));
  WG_TRY(upload(e->d_ent_w, e->ent_w));
  return WG_OK;
}

// Compiled shape with this (cluster, threads, cells-per-thread) triple.
bool find_shape(int which, int cluster, int threads, int cpt, wg::Shape* out) {
  const int n = which == 0 ? wg::fwd_shape_count() : wg::adj_shape_count();
  for (int i = 0; i < n; ++i) {
    const wg::Shape k = which == 0 ? wg::fwd_shape(i) : wg::adj_shape(i);
    if (k.cluster == cluster && k.threads == threads && k.cpt == cpt) {
      *out = k;
      return true;
    }
  }
  return false;
}

bool pick_shapes(wg_engine* e) {
  // Preference order; the first compiled shape that fits the grid is the default (the autotuner
  // can choose another among wg_shape_candidates).
  static const int fpref[][3] = {{2, 704, 10}, {4, 672, 10}, {6, 640, 12}, {2, 896, 8}, {4, 480, 14}, {6, 384, 20}, {4, 896, 4}, {4, 448, 8}, {1, 1024, 12},
                                 {2, 1024, 6}, {2, 512, 12}, {2, 1024, 10}, {4, 1024, 8}, {2, 1024, 16},
                                 {4, 512, 16}};
  static const int apref[][3] = {{2, 704, 10}, {4, 672, 10}, {6, 640, 12}, {2, 896, 8}, {4, 480, 14}, {6, 384, 20}, {2, 1024, 6}, {4, 896, 4}, {4, 448, 8},
                                 {2, 512, 12}, {4, 1024, 4}, {4, 1024, 8}, {4, 512, 16}};
  e->fshape = wg::Shape{0, 0, 0};
  e->ashape = wg::Shape{0, 0, 0};
  for (const auto& t : fpref) {
    wg::Shape s;
    if (find_shape(0, t[0], t[1], t[2], &s) && wg::fwd_shape_fits(s, e->nx, e->nz, e->sw, e->nrec)) {
      e->fshape = s;
      break;
    }
  }
  for (const auto& t : apref) {
    wg::Shape s;
    if (find_shape(1, t[0], t[1], t[2], &s) && wg::adj_shape_fits(s, e->nx, e->nz, e->swa, e->nrec)) {
      e->ashape = s;
      break;
    }
  }
  return e->fshape.cluster > 0;
}

int create_impl(const wg_config* c, bool cpu_d2, wg_engine** out) {
  if (!c || !out) return fail(WG_ERR_ARG, "null argument");
  wg_config cfg = *c;
  if (cfg.nx_vis == 0) cfg.nx_vis = 70;
  if (cfg.nz_vis == 0) cfg.nz_vis = 70;
  if (cfg.h == 0.0f) cfg.h = 10.0f;
  if (cfg.nrec == 0) cfg.nrec = cfg.nx_vis;
  if (cfg.shots < 1 || cfg.nt < 1 || cfg.pml < 0 || !(cfg.dt > 0.0f) || !(cfg.h > 0.0f) || cfg.nx_vis < 8 ||
      cfg.nz_vis < 8 || cfg.nrec < 1 || !(cfg.vmin <= cfg.vmax) || !(cfg.peak_hz > 0.0f))
    return fail(WG_ERR_ARG, "invalid engine configuration");
  if (cfg.shots > 1 << 20 || cfg.nrec > 4096) return fail(WG_ERR_ARG, "too many shots or receivers");
  int dev = 0;
  WG_CK(cudaGetDevice(&dev));
  wg::noalloc_forget_device(dev);
  auto e = new wg_engine();
  e->cfg = cfg;
  e->device = dev;
  e->shots = cfg.shots;
  e->nt = cfg.nt;
  e->nrec = cfg.nrec;
  e->nx_vis = cfg.nx_vis;
  e->nz_vis = cfg.nz_vis;
  e->h = cfg.h;
  e->pad = FD + cfg.pml;
  e->nx = cfg.nx_vis + 2 * e->pad;
  e->nz = cfg.nz_vis + 2 * e->pad;
  e->cells = e->nx * e->nz;
  e->region = cfg.pml + 2 * FD;
  e->region_adj = cfg.pml + 3 * FD;
  e->sw = e->region + 2;
  e->swa = e->region_adj + 2;
  e->rh = 1.0f / cfg.h;
  e->dt2 = cfg.dt * cfg.dt;
  if (cpu_d2) {
    e->d2a = e->rh * e->rh;
    e->d2b = 1.0f;
  } else {
    e->d2a = e->rh;
    e->d2b = e->rh;
  }
  e->prof.resize(3 * (e->nx + e->nz));
  float* p = e->prof.data();
  cpml(e->nx, cfg.h, cfg.dt, cfg.pml, cfg.vmax, cfg.peak_hz, p, p + e->nx, p + 2 * e->nx);
  float* q = p + 3 * e->nx;
  cpml(e->nz, cfg.h, cfg.dt, cfg.pml, cfg.vmax, cfg.peak_hz, q, q + e->nz, q + 2 * e->nz);
  e->wavelet.resize(cfg.nt);
  ricker(cfg.nt, cfg.dt, cfg.peak_hz, e->wavelet.data());
  int rc = WG_OK;
  cudaError_t ce = cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking);
  if (ce != cudaSuccess) rc = fail(WG_ERR_CUDA, std::string("cudaStreamCreate: ") + cudaGetErrorString(ce));
  if (rc == WG_OK) rc = upload(e->d_prof, e->prof);
  if (rc == WG_OK) rc = upload(e->d_wavelet, e->wavelet);
  if (rc == WG_OK) rc = e->d_status.ensure(16);
  if (rc == WG_OK) {
    // Default sources: x = linspace(0, (nx_vis - 1) h, shots) (centre for one shot), z = h
    // (wave_wgpu.rs:204-214).
    std::vector<float> src(2 * cfg.shots);
    const float xmax = static_cast<float>(cfg.nx_vis - 1) * cfg.h;
    for (int k = 0; k < cfg.shots; ++k) {
      src[2 * k] = cfg.shots == 1 ? xmax * 0.5f : (xmax * static_cast<float>(k)) / static_cast<float>(cfg.shots - 1);
      src[2 * k + 1] = cfg.h;
    }
    rc = set_sources_impl(e, src.data());
  }
  if (rc == WG_OK) rc = set_receivers_impl(e);
  if (rc == WG_OK && !pick_shapes(e)) {
    // beyond the resident kernels: the streamed path, with checkpointing sized to the free memory
    std::string why;
    if (wg::stream_supported(view_of(e), &why)) {
      e->streamed = 1;
      e->ck_every = 0;
    } else {
      rc = fail(WG_ERR_UNSUPPORTED, "grid " + std::to_string(e->nx) + "x" + std::to_string(e->nz) +
                                        " does not fit the resident kernels and " + why);
    }
  }
  if (rc != WG_OK) {
    if (e->stream) cudaStreamDestroy(e->stream);
    delete e;
    return rc;
  }
  *out = e;
  return WG_OK;
}

// Device entry points run on the caller's stream; NULL is the CUDA default stream (torch's
// default stream has handle 0).
cudaStream_t pick_stream(wg_engine*, void* s) { return static_cast<cudaStream_t>(s); }

// Kernel kinds for per-kernel timing.
enum : int { K_FWD = 0, K_RECOMPUTE = 1, K_ADJ = 2, K_AUX = 3, K_KINDS = 4 };

// Records an event pair around one launch when timing is on.
template <typename F>
cudaError_t timed(wg_engine* e, int kind, cudaStream_t st, F&& launch) {
  if (!e->prof_on) return launch();
  if (e->prof_used + 2 > e->prof_ev.size()) {
    for (int i = 0; i < 64; ++i) {
      cudaEvent_t ev;
      cudaError_t r = cudaEventCreate(&ev);
      if (r != cudaSuccess) return r;
      e->prof_ev.push_back(ev);
    }
  }
  cudaEvent_t a = e->prof_ev[e->prof_used], b = e->prof_ev[e->prof_used + 1];
  e->prof_used += 2;
  e->prof_kind.push_back(kind);
  cudaError_t r = cudaEventRecord(a, st);
  if (r != cudaSuccess) return r;
  r = launch();
  if (r != cudaSuccess) return r;
  return cudaEventRecord(b, st);
}

// Event marks around groups of streamed-path launches (one pair per group, same records as timed()).
void prof_mark(void* ctx, int kind, bool begin, cudaStream_t st) {
  auto* e = static_cast<wg_engine*>(ctx);
  if (!e->prof_on) return;
  if (begin) {
    if (e->prof_used + 2 > e->prof_ev.size()) {
      for (int i = 0; i < 64; ++i) {
        cudaEvent_t ev;
        if (cudaEventCreate(&ev) != cudaSuccess) return;
        e->prof_ev.push_back(ev);
      }
    }
    cudaEventRecord(e->prof_ev[e->prof_used], st);
  } else if (e->prof_used + 2 <= e->prof_ev.size()) {
    cudaEventRecord(e->prof_ev[e->prof_used + 1], st);
    e->prof_used += 2;
    e->prof_kind.push_back(kind);
  }
}

wg::StreamTimer timer_of(wg_engine* e) {
  wg::StreamTimer t;
  t.ctx = e;
  t.fn = prof_mark;
  return t;
}

size_t per_model_grad_bytes(const wg_engine* e, int k, bool store_all) {
  const size_t S = e->shots, cells = e->cells;
  size_t b = 2 * cells * 4 + S * e->nt * e->nrec * 4 + 64;
  const int J = store_all ? 1 : (e->nt + k - 1) / k;
  const int seg = store_all ? e->nt : k;
  b += S * static_cast<size_t>(J - 1) * wg::ckpt_floats(e->nx, e->nz, e->sw) * 4;
  b += S * static_cast<size_t>(seg) * cells * 4;
  b += S * wg::adjstate_floats(e->nx, e->nz, e->swa) * 4;
  b += S * cells * 4;
  return b;
}

int chunk_models(const wg_engine* e, int models, size_t per_model) {
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
    cudaGetLastError();
    free_b = size_t(8) << 30;
  }
  size_t budget = std::min<size_t>(free_b / 10 * 7, size_t(96) << 30);
  long m = static_cast<long>(budget / std::max<size_t>(per_model, 1));
  m = std::max<long>(1, std::min<long>(m, models));
  (void)e;
  return static_cast<int>(m);
}

int simulate_dev_impl(wg_engine* e, const float* d_vis, int models, float* d_traces, cudaStream_t st) {
  if (models < 1) return fail(WG_ERR_ARG, "models must be >= 1");
  if (!d_vis || !d_traces) return fail(WG_ERR_ARG, "null pointer");
  if (e->streamed) {
    if (!e->swork) e->swork = wg::stream_work_new();
    return wg::stream_simulate(e->swork, view_of(e), e->rec_cell.data(), d_vis, models, d_traces, st, timer_of(e));
  }
  const size_t cells = e->cells;
  const int M = chunk_models(e, models, cells * 4 + 64);
  WG_TRY(e->w_vpad.ensure(static_cast<size_t>(M) * cells * 4));
  for (int m0 = 0; m0 < models; m0 += M) {
    const int mc = std::min(M, models - m0);
    WG_LAUNCH(wg::launch_pad_velocity(d_vis + static_cast<size_t>(m0) * e->nx_vis * e->nz_vis, mc, e->nx_vis,
                                      e->nz_vis, e->pad, e->cfg.vmin, e->cfg.vmax, e->w_vpad.as<float>(), nullptr, st));
    wg::FwdArgs a{};
    a.g = e->grid();
    a.st = e->stations();
    a.vel = e->w_vpad.as<float>();
    a.units = mc * e->shots;
    a.t0 = 0;
    a.t1 = e->nt;
    a.traces = d_traces + static_cast<size_t>(m0) * e->shots * e->nt * e->nrec;
    a.status = e->d_status.as<int>();
    a.fast = e->fast;
    WG_LAUNCH(timed(e, K_FWD, st, [&] { return wg::launch_fwd(e->fshape, true, false, a, st); }));
  }
  return WG_OK;
}

// obs_ready (optional): an event the observed data's arrival is recorded on; nothing reads them
// before the first forward pass has been launched, so their host->device copy can overlap it.
int gradient_dev_impl(wg_engine* e, const float* d_vis, const float* d_obs, int models, double* d_loss, float* d_grad,
                      cudaStream_t st, cudaEvent_t obs_ready = nullptr) {
  if (models < 1) return fail(WG_ERR_ARG, "models must be >= 1");
  if (!d_vis || !d_obs || !d_loss || !d_grad) return fail(WG_ERR_ARG, "null pointer");
  if (e->streamed) {
    if (!e->swork) e->swork = wg::stream_work_new();
    return wg::stream_gradient(e->swork, view_of(e), e->rec_cell.data(), d_vis, d_obs, models, d_loss, d_grad, st,
                               timer_of(e));
  }
  if (e->ashape.cluster == 0) return fail(WG_ERR_UNSUPPORTED, "grid does not fit the resident adjoint kernel");
  const bool store_all = e->ck_every <= 0 || e->ck_every >= e->nt;
  const int k = store_all ? e->nt : e->ck_every;
  const int J = store_all ? 1 : (e->nt + k - 1) / k;
  const int slots = J - 1;
  const int seg = store_all ? e->nt : k;
  const size_t S = e->shots, cells = e->cells, tr = static_cast<size_t>(e->nt) * e->nrec;
  const size_t ckf = wg::ckpt_floats(e->nx, e->nz, e->sw);
  const size_t asf = wg::adjstate_floats(e->nx, e->nz, e->swa);
  const int M = chunk_models(e, models, per_model_grad_bytes(e, k, store_all));
  WG_TRY(e->w_vpad.ensure(M * cells * 4));
  WG_TRY(e->w_mask.ensure(M * cells * 4));
  WG_TRY(e->w_traces.ensure(M * S * tr * 4));
  WG_TRY(e->w_energy.ensure(M * 8));
  WG_TRY(e->w_scale.ensure(M * 4));
  if (slots > 0) WG_TRY(e->w_ckpt.ensure(M * S * slots * ckf * 4));
  WG_TRY(e->w_stored.ensure(M * S * seg * cells * 4));
  WG_TRY(e->w_adj.ensure(M * S * asf * 4));
  WG_TRY(e->w_gacc.ensure(M * S * cells * 4));
  for (int m0 = 0; m0 < models; m0 += M) {
    const int mc = std::min(M, models - m0);
    const int units = mc * e->shots;
    const float* obs = d_obs + static_cast<size_t>(m0) * S * tr;
    WG_LAUNCH(wg::launch_pad_velocity(d_vis + static_cast<size_t>(m0) * e->nx_vis * e->nz_vis, mc, e->nx_vis,
                                      e->nz_vis, e->pad, e->cfg.vmin, e->cfg.vmax, e->w_vpad.as<float>(),
                                      e->w_mask.as<float>(), st));
    wg::FwdArgs f{};
    f.g = e->grid();
    f.st = e->stations();
    f.vel = e->w_vpad.as<float>();
    f.units = units;
    f.t0 = 0;
    f.t1 = e->nt;
    f.traces = e->w_traces.as<float>();
    f.status = e->d_status.as<int>();
    f.fast = e->fast;
    if (store_all) {
      f.stored = e->w_stored.as<float>();
      WG_LAUNCH(timed(e, K_FWD, st, [&] { return wg::launch_fwd(e->fshape, true, true, f, st); }));
    } else {
      // Steps [0, (J-1) k] with receivers and checkpoints (the last checkpoint is written at the
      // start of step (J-1) k, which is computed once more below), then the last segment from
      // that checkpoint with receivers and stored terms: the reverse sweep starts without a
      // recompute.
      f.ck_out = e->w_ckpt.as<float>();
      f.ck_every = k;
      f.ck_slots = slots;
      f.t1 = (J - 1) * k + 1;
      WG_LAUNCH(timed(e, K_FWD, st, [&] { return wg::launch_fwd(e->fshape, true, false, f, st); }));
      wg::FwdArgs l = f;
      l.t0 = (J - 1) * k;
      l.t1 = e->nt;
      l.ck_out = nullptr;
      l.ck_in = e->w_ckpt.as<float>();
      l.ck_in_slot = J - 2;
      l.stored = e->w_stored.as<float>();
      WG_LAUNCH(timed(e, K_FWD, st, [&] { return wg::launch_fwd(e->fshape, true, true, l, st); }));
    }
    if (obs_ready && m0 == 0) WG_CK(cudaStreamWaitEvent(st, obs_ready, 0));
    WG_LAUNCH(wg::launch_energy(obs, mc, S * tr, e->w_energy.as<double>(), e->w_scale.as<float>(),
                                e->d_status.as<int>(), st));
    WG_LAUNCH(wg::launch_residual(e->w_traces.as<float>(), obs, e->w_scale.as<float>(), mc, S * tr,
                                  e->w_traces.as<float>(), d_loss + m0, st));
    WG_CK(cudaMemsetAsync(e->w_gacc.p, 0, static_cast<size_t>(units) * cells * 4, st));
    wg::AdjArgs a{};
    a.g = e->grid();
    a.st = e->stations();
    a.vel = e->w_vpad.as<float>();
    a.units = units;
    a.residual = e->w_traces.as<float>();
    a.stored = e->w_stored.as<float>();
    a.state = e->w_adj.as<float>();
    a.gacc = e->w_gacc.as<float>();
    a.status = e->d_status.as<int>();
    a.prefetch = e->adj_prefetch;
    if (store_all) {
      a.t_hi = e->nt;
      a.t_lo = 0;
      a.first = 1;
      WG_LAUNCH(timed(e, K_ADJ, st, [&] { return wg::launch_adj(e->ashape, a, st); }));
    } else {
      for (int j = J - 1; j >= 0; --j) {
        const int t0 = j * k, t1 = std::min(t0 + k, e->nt);
        wg::FwdArgs r{};
        r.g = e->grid();
        r.st = e->stations();
        r.vel = e->w_vpad.as<float>();
        r.units = units;
        r.t0 = t0;
        r.t1 = t1;
        r.ck_in = j > 0 ? e->w_ckpt.as<float>() : nullptr;
        r.ck_in_slot = j - 1;
        r.ck_slots = slots;
        r.ck_every = k;
        r.stored = e->w_stored.as<float>();
        r.status = e->d_status.as<int>();
        r.fast = e->fast;
        if (j < J - 1)  // the last segment's terms are already stored by the first pass
          WG_LAUNCH(timed(e, K_RECOMPUTE, st, [&] { return wg::launch_fwd(e->fshape, false, true, r, st); }));
        a.t_hi = t1;
        a.t_lo = t0;
        a.first = (j == J - 1) ? 1 : 0;
        WG_LAUNCH(timed(e, K_ADJ, st, [&] { return wg::launch_adj(e->ashape, a, st); }));
      }
    }
    WG_LAUNCH(wg::launch_fold(e->w_gacc.as<float>(), e->w_mask.as<float>(), mc, e->shots, e->nx, e->nz, e->pad,
                              e->nx_vis, e->nz_vis, d_grad + static_cast<size_t>(m0) * e->nx_vis * e->nz_vis, st));
  }
  return WG_OK;
}

int read_status(wg_engine* e) {
  int s = 0;
  WG_CK(cudaMemcpy(&s, e->d_status.p, sizeof(int), cudaMemcpyDeviceToHost));
  if (s == wg::ST_ENERGY) return fail(WG_ERR_ENERGY, "Observed traces have zero energy");
  if (s != 0) return fail(s, "device status " + std::to_string(s));
  return WG_OK;
}

}  // namespace

namespace wg {
using ::view_of;

// Snapshot of the engine's statics under its lock; `lock` keeps the engine locked while the caller
// launches with them.
EngineView engine_view(wg_engine* e, std::unique_lock<std::mutex>& lock) {
  lock = std::unique_lock<std::mutex>(e->mu);
  return view_of(e);
}

int engine_device(const wg_engine* e) { return e->device; }

}  // namespace wg

extern "C" {

int wg_engine_create(const wg_config* cfg, wg_engine** out) { return create_impl(cfg, false, out); }

void wg_engine_destroy(wg_engine* eng) {
  if (!eng) return;
  if (eng->stream) {
    cudaStreamSynchronize(eng->stream);
    cudaStreamDestroy(eng->stream);
  }
  for (cudaEvent_t ev : eng->prof_ev) cudaEventDestroy(ev);
  if (eng->obs_ready) cudaEventDestroy(eng->obs_ready);
  if (eng->copy_stream) {
    cudaStreamSynchronize(eng->copy_stream);
    cudaStreamDestroy(eng->copy_stream);
  }
  if (eng->swork) wg::stream_work_free(eng->swork);
  delete eng;
}

int wg_profile(wg_engine* e, int enable) {
  if (!e) return fail(WG_ERR_ARG, "null engine");
  std::lock_guard<std::mutex> lk(e->mu);
  e->prof_on = enable != 0;
  e->prof_used = 0;
  e->prof_kind.clear();
  return WG_OK;
}

int wg_profile_read(wg_engine* e, double* ms, long long* launches, int kinds) {
  if (!e || !ms || !launches || kinds < 1) return fail(WG_ERR_ARG, "bad argument");
  std::lock_guard<std::mutex> lk(e->mu);
  for (int k = 0; k < kinds; ++k) {
    ms[k] = 0.0;
    launches[k] = 0;
  }
  for (size_t i = 0; i < e->prof_kind.size(); ++i) {
    WG_CK(cudaEventSynchronize(e->prof_ev[2 * i + 1]));
    float t = 0.0f;
    WG_CK(cudaEventElapsedTime(&t, e->prof_ev[2 * i], e->prof_ev[2 * i + 1]));
    const int k = e->prof_kind[i];
    if (k < kinds) {
      ms[k] += t;
      launches[k] += 1;
    }
  }
  e->prof_used = 0;
  e->prof_kind.clear();
  return WG_OK;
}

int wg_engine_dims(const wg_engine* e, int* shots, int* nt, int* nrec, int* nx, int* nz, int* nx_vis, int* nz_vis) {
  if (!e) return fail(WG_ERR_ARG, "null engine");
  if (shots) *shots = e->shots;
  if (nt) *nt = e->nt;
  if (nrec) *nrec = e->nrec;
  if (nx) *nx = e->nx;
  if (nz) *nz = e->nz;
  if (nx_vis) *nx_vis = e->nx_vis;
  if (nz_vis) *nz_vis = e->nz_vis;
  return WG_OK;
}

int wg_get_sources(const wg_engine* e, float* out, int n) {
  if (!e || !out) return fail(WG_ERR_ARG, "null argument");
  if (n != e->shots) return fail(WG_ERR_ARG, "sources must have shape [shots, 2]");
  std::memcpy(out, e->sources.data(), sizeof(float) * 2 * e->shots);
  return WG_OK;
}

int wg_set_sources(wg_engine* e, const float* xz, int n) {
  if (!e || !xz) return fail(WG_ERR_ARG, "null argument");
  if (n != e->shots) return fail(WG_ERR_ARG, "sources must have shape [shots, 2]");
  std::lock_guard<std::mutex> lk(e->mu);
  WG_CK(cudaSetDevice(e->device));
  WG_CK(cudaStreamSynchronize(e->stream));
  return set_sources_impl(e, xz);
}

int wg_get_wavelet(const wg_engine* e, float* out, int n) {
  if (!e || !out) return fail(WG_ERR_ARG, "null argument");
  if (n != e->nt) return fail(WG_ERR_ARG, "wavelet length must equal nt");
  std::memcpy(out, e->wavelet.data(), sizeof(float) * e->nt);
  return WG_OK;
}

int wg_set_wavelet(wg_engine* e, const float* w, int n) {
  if (!e || !w) return fail(WG_ERR_ARG, "null argument");
  if (n != e->nt) return fail(WG_ERR_ARG, "wavelet length must equal nt");
  std::lock_guard<std::mutex> lk(e->mu);
  WG_CK(cudaSetDevice(e->device));
  WG_CK(cudaStreamSynchronize(e->stream));
  e->wavelet.assign(w, w + n);
  return upload(e->d_wavelet, e->wavelet);
}

int wg_simulate_dev(wg_engine* e, const float* d_vel, int models, float* d_traces, void* stream) {
  if (!e) return fail(WG_ERR_ARG, "null engine");
  std::lock_guard<std::mutex> lk(e->mu);
  WG_CK(cudaSetDevice(e->device));
  // each call starts with a clear status word; wg_engine_status reads what this call's kernels set
  WG_CK(cudaMemsetAsync(e->d_status.p, 0, sizeof(int), pick_stream(e, stream)));
  return simulate_dev_impl(e, d_vel, models, d_traces, pick_stream(e, stream));
}

int wg_simulate(wg_engine* e, const float* vel, int models, float* traces) {
  if (!e || !vel || !traces) return fail(WG_ERR_ARG, "null argument");
  if (models < 1) return fail(WG_ERR_ARG, "models must be >= 1");
  std::lock_guard<std::mutex> lk(e->mu);
  WG_CK(cudaSetDevice(e->device));
  const size_t nv = static_cast<size_t>(models) * e->nx_vis * e->nz_vis;
  const size_t nt = static_cast<size_t>(models) * e->shots * e->nt * e->nrec;
  WG_TRY(e->w_vis.ensure(nv * 4));
  WG_TRY(e->w_obs.ensure(nt * 4));
  WG_CK(cudaMemsetAsync(e->d_status.p, 0, sizeof(int), e->stream));
  WG_CK(cudaMemcpyAsync(e->w_vis.p, vel, nv * 4, cudaMemcpyHostToDevice, e->stream));
  WG_TRY(simulate_dev_impl(e, e->w_vis.as<float>(), models, e->w_obs.as<float>(), e->stream));
  WG_CK(cudaMemcpyAsync(traces, e->w_obs.p, nt * 4, cudaMemcpyDeviceToHost, e->stream));
  WG_CK(cudaStreamSynchronize(e->stream));
  return read_status(e);
}

int wg_evaluate_adjoint_dev(wg_engine* e, const float* d_vel, const float* d_obs, int models, double* d_loss,
                            float* d_grad, void* stream) {
  if (!e) return fail(WG_ERR_ARG, "null engine");
  std::lock_guard<std::mutex> lk(e->mu);
  WG_CK(cudaSetDevice(e->device));
  WG_CK(cudaMemsetAsync(e->d_status.p, 0, sizeof(int), pick_stream(e, stream)));
  return gradient_dev_impl(e, d_vel, d_obs, models, d_loss, d_grad, pick_stream(e, stream));
}

int wg_engine_status(wg_engine* e, void* stream) {
  if (!e) return fail(WG_ERR_ARG, "null engine");
  std::lock_guard<std::mutex> lk(e->mu);
  WG_CK(cudaSetDevice(e->device));
  cudaStream_t st = pick_stream(e, stream);
  int s = 0;
  WG_CK(cudaMemcpyAsync(&s, e->d_status.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  WG_CK(cudaStreamSynchronize(st));
  if (s == wg::ST_ENERGY) return fail(WG_ERR_ENERGY, "Observed traces have zero energy");
  if (s != 0) return fail(WG_ERR_CUDA, "device status " + std::to_string(s) + " (a pipeline wait timed out)");
  return WG_OK;
}

int wg_selftest_wait_timeout(wg_engine* e, long long polls, void* stream) {
  if (!e) return fail(WG_ERR_ARG, "null engine");
  if (polls < 1 || polls > (1LL << 22)) return fail(WG_ERR_ARG, "polls must be in [1, 2^22]");
  std::lock_guard<std::mutex> lk(e->mu);
  WG_CK(cudaSetDevice(e->device));
  cudaStream_t st = pick_stream(e, stream);
  WG_CK(cudaMemsetAsync(e->d_status.p, 0, sizeof(int), st));
  return wg::wait_timeout_selftest(static_cast<int*>(e->d_status.p), polls, st);
}

int wg_evaluate_adjoint(wg_engine* e, const float* vel, const float* obs, int models, double* loss, float* grad) {
  if (!e || !vel || !obs || !loss || !grad) return fail(WG_ERR_ARG, "null argument");
  if (models < 1) return fail(WG_ERR_ARG, "models must be >= 1");
  std::lock_guard<std::mutex> lk(e->mu);
  WG_CK(cudaSetDevice(e->device));
  const size_t nv = static_cast<size_t>(models) * e->nx_vis * e->nz_vis;
  const size_t no = static_cast<size_t>(models) * e->shots * e->nt * e->nrec;
  WG_TRY(e->w_vis.ensure(nv * 4));
  WG_TRY(e->w_obs.ensure(no * 4));
  WG_TRY(e->w_loss.ensure(static_cast<size_t>(models) * 8));
  WG_TRY(e->w_grad.ensure(nv * 4));
  WG_CK(cudaMemsetAsync(e->d_status.p, 0, sizeof(int), e->stream));
  WG_CK(cudaMemcpyAsync(e->w_vis.p, vel, nv * 4, cudaMemcpyHostToDevice, e->stream));
  // the observed data travel on a second stream while the first forward pass runs
  if (!e->copy_stream) WG_CK(cudaStreamCreateWithFlags(&e->copy_stream, cudaStreamNonBlocking));
  if (!e->obs_ready) WG_CK(cudaEventCreateWithFlags(&e->obs_ready, cudaEventDisableTiming));
  WG_CK(cudaMemcpyAsync(e->w_obs.p, obs, no * 4, cudaMemcpyHostToDevice, e->copy_stream));
  WG_CK(cudaEventRecord(e->obs_ready, e->copy_stream));
  const int rc = e->streamed ? [&] {
    const cudaError_t w = cudaStreamWaitEvent(e->stream, e->obs_ready, 0);
    return w == cudaSuccess ? gradient_dev_impl(e, e->w_vis.as<float>(), e->w_obs.as<float>(), models,
                                                e->w_loss.as<double>(), e->w_grad.as<float>(), e->stream)
                            : fail(WG_ERR_CUDA, cudaGetErrorString(w));
  }()
                             : gradient_dev_impl(e, e->w_vis.as<float>(), e->w_obs.as<float>(), models,
                                                 e->w_loss.as<double>(), e->w_grad.as<float>(), e->stream, e->obs_ready);
  if (rc != WG_OK) {
    cudaStreamSynchronize(e->copy_stream);
    return rc;
  }
  WG_CK(cudaMemcpyAsync(loss, e->w_loss.p, static_cast<size_t>(models) * 8, cudaMemcpyDeviceToHost, e->stream));
  WG_CK(cudaMemcpyAsync(grad, e->w_grad.p, nv * 4, cudaMemcpyDeviceToHost, e->stream));
  WG_CK(cudaStreamSynchronize(e->stream));
  return read_status(e);
}

int wg_set_checkpoint_interval(wg_engine* e, int k) {
  if (!e) return fail(WG_ERR_ARG, "null engine");
  std::lock_guard<std::mutex> lk(e->mu);
  e->ck_every = k;
  return WG_OK;
}

int wg_get_checkpoint_interval(const wg_engine* e) { return e ? e->ck_every : -1; }

int wg_set_option(wg_engine* e, const char* key, int value) {
  if (!e || !key) return fail(WG_ERR_ARG, "null argument");
  std::lock_guard<std::mutex> lk(e->mu);
  const std::string k(key);
  if (k == "checkpoint_every") {
    e->ck_every = value;
  } else if (k == "adjoint_prefetch") {
    e->adj_prefetch = value ? 1 : 0;
  } else if (k == "arith") {
    if (value != 0 && value != 1) return fail(WG_ERR_ARG, "arith must be 0 (reference order) or 1 (fast)");
    e->fast = value;
  } else if (k == "temporal_block") {
    e->tblock = value ? 1 : 0;
  } else if (k == "streamed") {
    if (value) {
      std::string why;
      if (!wg::stream_supported(view_of(e), &why)) return fail(WG_ERR_UNSUPPORTED, why);
    } else if (e->fshape.cluster == 0 || e->ashape.cluster == 0) {
      return fail(WG_ERR_UNSUPPORTED, "grid does not fit the resident kernels");
    }
    e->streamed = value ? 1 : 0;
  } else {
    return fail(WG_ERR_ARG, "unknown option: " + k);
  }
  return WG_OK;
}

int wg_get_option(const wg_engine* e, const char* key, int* value) {
  if (!e || !key || !value) return fail(WG_ERR_ARG, "null argument");
  const std::string k(key);
  if (k == "checkpoint_every") {
    *value = e->ck_every;
  } else if (k == "adjoint_prefetch") {
    *value = e->adj_prefetch;
  } else if (k == "arith") {
    *value = e->fast;
  } else if (k == "temporal_block") {
    *value = e->tblock;
  } else if (k == "streamed") {
    *value = e->streamed;
  } else {
    return fail(WG_ERR_ARG, "unknown option: " + k);
  }
  return WG_OK;
}

int wg_set_launch_shape(wg_engine* e, int which, int cluster, int threads, int cpt) {
  if (!e) return fail(WG_ERR_ARG, "null engine");
  if (which != 0 && which != 1) return fail(WG_ERR_ARG, "which must be 0 (forward) or 1 (adjoint)");
  wg::Shape s;
  if (!find_shape(which, cluster, threads, cpt, &s)) return fail(WG_ERR_ARG, "launch shape not compiled");
  std::lock_guard<std::mutex> lk(e->mu);
  if (which == 0) {
    if (!wg::fwd_shape_fits(s, e->nx, e->nz, e->sw, e->nrec)) return fail(WG_ERR_ARG, "forward shape does not fit this grid");
    e->fshape = s;
  } else {
    if (!wg::adj_shape_fits(s, e->nx, e->nz, e->swa, e->nrec)) return fail(WG_ERR_ARG, "adjoint shape does not fit this grid");
    e->ashape = s;
  }
  return WG_OK;
}

int wg_get_launch_shape(const wg_engine* e, int which, int* cluster, int* threads, int* cpt) {
  if (!e || !cluster || !threads || !cpt) return fail(WG_ERR_ARG, "null argument");
  const wg::Shape s = which == 0 ? e->fshape : e->ashape;
  *cluster = s.cluster;
  *threads = s.threads;
  *cpt = s.cpt;
  return WG_OK;
}

int wg_shape_candidates(const wg_engine* e, int which, int* out3, int max_shapes) {
  if (!e || (!out3 && max_shapes > 0)) return -fail(WG_ERR_ARG, "null argument");
  int n = 0;
  const int total = which == 0 ? wg::fwd_shape_count() : wg::adj_shape_count();
  for (int i = 0; i < total; ++i) {
    const wg::Shape s = which == 0 ? wg::fwd_shape(i) : wg::adj_shape(i);
    const bool fits = which == 0 ? wg::fwd_shape_fits(s, e->nx, e->nz, e->sw, e->nrec)
                                 : wg::adj_shape_fits(s, e->nx, e->nz, e->swa, e->nrec);
    if (!fits) continue;
    if (n < max_shapes) {
      out3[3 * n] = s.cluster;
      out3[3 * n + 1] = s.threads;
      out3[3 * n + 2] = s.cpt;
    }
    ++n;
  }
  return n;
}

int wg_simulate_shot(const float* vel, int nx_vis, int nz_vis, float h, float dt, int nt, int pml, float vmin,
                     float vmax, float peak_hz, float src_x, float src_z, float* out) {
  if (!vel || !out) return fail(WG_ERR_ARG, "null argument");
  wg_config c{};
  c.shots = 1;
  c.nt = nt;
  c.dt = dt;
  c.peak_hz = peak_hz;
  c.pml = pml;
  c.vmin = vmin;
  c.vmax = vmax;
  c.nx_vis = nx_vis;
  c.nz_vis = nz_vis;
  c.h = h;
  c.nrec = nx_vis;
  wg_engine* e = nullptr;
  WG_TRY(create_impl(&c, true, &e));
  const float src[2] = {src_x, src_z};
  int rc = wg_set_sources(e, src, 1);
  if (rc == WG_OK) rc = wg_simulate(e, vel, 1, out);
  wg_engine_destroy(e);
  return rc;
}

int wg_ricker_wavelet(int samples, float dt, float peak_hz, float* out) {
  if (samples < 0 || (!out && samples > 0)) return fail(WG_ERR_ARG, "bad argument");
  ricker(samples, dt, peak_hz, out);
  return WG_OK;
}

int wg_cpml_profiles(int n, float h, float dt, int width, float max_vel, float freq, float* a, float* b, float* db) {
  if (n < 5 || !a || !b || !db) return fail(WG_ERR_ARG, "bad argument");
  cpml(n, h, dt, width, max_vel, freq, a, b, db);
  return WG_OK;
}

int wg_bandlimit_dev(const float* d_in, const float* d_kernel, int klen, int series, int nt, int nrec, float* d_out,
                     void* stream) {
  if (!d_in || !d_kernel || !d_out || klen < 1 || series < 0 || nt < 0 || nrec < 0)
    return fail(WG_ERR_ARG, "bad argument");
  if (series == 0 || nt == 0 || nrec == 0) return WG_OK;
  if (d_in == d_out) return fail(WG_ERR_ARG, "bandlimit cannot run in place");
  WG_LAUNCH(wg::launch_bandlimit(d_in, d_kernel, klen, series, nt, nrec, d_out, static_cast<cudaStream_t>(stream)));
  return WG_OK;
}

int wg_lowpass_decimate_f16_dev(const float* d_in, const float* d_kernel, int klen, int center, int factor, int series,
                                int nt, int nrec, void* d_out, void* stream) {
  if (!d_in || !d_kernel || !d_out || klen < 1 || center < 0 || center >= klen || factor < 1 || series < 0 || nt < 0 ||
      nrec < 0)
    return fail(WG_ERR_ARG, "bad argument");
  const int nt_out = (nt + factor - 1) / factor;
  if (series == 0 || nt_out == 0 || nrec == 0) return WG_OK;
  if (nt_out > 65535) return fail(WG_ERR_ARG, "too many output samples");
  WG_LAUNCH(wg::launch_decimate(d_in, d_kernel, klen, center, factor, series, nt, nrec, nt_out, d_out,
                                static_cast<cudaStream_t>(stream)));
  return WG_OK;
}

const char* wg_last_error(void) { return g_err.c_str(); }

long long wg_launch_count(int reset) {
  const long long n = g_launches;
  if (reset) g_launches = 0;
  return n;
}

}  // extern "C"
