// CPU oracle for the WGNet physics path. TEST INFRASTRUCTURE ONLY.
//
// This file restates, in plain C++, the reference algorithms that the CUDA path must reproduce.
// It is the parity checker and the timed CPU baseline; the product library never links it.
//
//   ricker_wavelet        crates/geology-core/src/lib.rs:11-21
//   cpml_profiles         crates/geology-core/src/lib.rs:23-68 (f64 inside, f32 out)
//   simulate_shot_cpu     crates/geology-core/src/lib.rs:70-221 (node receivers, d2 * rh2)
//   engine geometry       crates/wave-gauss-rs/src/wave_wgpu.rs:204-270 (bilinear corners, CSR)
//   pad_velocity          crates/wave-gauss-rs/src/wave_wgpu.rs:714-734
//   engine forward step   crates/wave-gauss-rs/src/shaders/splatForward.wgsl:48-121 (d2 * rh * rh)
//   residual + misfit     crates/wave-gauss-rs/src/wave_wgpu.rs:13-54, 852-854, 960-965
//   engine adjoint step   crates/wave-gauss-rs/src/shaders/splatAdjoint.wgsl:58-131
//   shot-sum, mask, fold  crates/wave-gauss-rs/src/wave_wgpu.rs:974-987, 993-1005
//
// Every routine is templated on the real type R: R = float reproduces the reference's f32
// arithmetic operation by operation (build with -ffp-contract=off, as Rust never contracts);
// R = double runs the same discrete model (same f32 profiles, wavelet, velocities and weights)
// in double precision and is the FP64 yardstick for error reporting.
//
// Generalisation beyond the reference: the visible grid is nx_vis x nz_vis (the reference fixes
// 70 x 70) and the spacing h is a parameter (the engine fixes H = 10 m). With the defaults the
// behaviour is the reference's.

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <thread>
#include <vector>

extern "C" {
typedef struct {
  int nx_vis, nz_vis;  // visible grid (reference: 70 x 70)
  int pml;             // C-PML width in cells (reference default 20)
  int shots, nt, nrec; // nrec receivers; default layout = every surface cell (nrec = nx_vis)
  float h, dt, peak_hz, vmin, vmax;
} wgo_config;
}

namespace {

constexpr int FD_PAD = 2;

// --------------------------------------------------------------------------------------------
// geology-core building blocks
// --------------------------------------------------------------------------------------------

// lib.rs:11-21. The delay is 1.5 / peak_hz.
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

// lib.rs:23-68. Deepwave-style 4th-order C-PML profiles, computed in f64 and stored in f32.
void cpml(int n, float h, float dt, int width, float max_vel, float freq, float* a_out, float* b_out,
          float* db_out) {
  std::vector<double> a(n, 0.0), b(n, 0.0), db(n, 0.0);
  const double start0 = static_cast<double>(FD_PAD + width);
  const double start1 = static_cast<double>(n - 1 - FD_PAD - width);
  const double width_f = static_cast<double>(width);
  const double h_f = static_cast<double>(h);
  const double dt_f = static_cast<double>(dt);
  const double sigma0 = -(3.0 * static_cast<double>(max_vel) * std::log(0.001)) / (2.0 * width_f * h_f);
  for (int x = 0; x < n; ++x) {
    const double xf = static_cast<double>(x);
    const double f0 = (start0 - xf) / width_f;
    const double f1 = (xf - start1) / width_f;
    const double frac = std::min(std::max(std::max(f0, f1), 0.0), 1.0);
    const double sigma = sigma0 * frac * frac;
    const double alpha = 3.14159265358979323846 * static_cast<double>(freq) * (1.0 - frac);
    const double ax = std::exp(-(sigma + alpha) * dt_f);
    b[x] = (sigma / (sigma + alpha)) * (ax - 1.0);
    a[x] = (frac == 0.0) ? 0.0 : ax;
  }
  for (int x = 2; x < n - 2; ++x)
    db[x] = ((8.0 / 12.0) * (b[x + 1] - b[x - 1]) - (1.0 / 12.0) * (b[x + 2] - b[x - 2])) / h_f;
  for (int i = 0; i < n; ++i) {
    a_out[i] = static_cast<float>(a[i]);
    b_out[i] = static_cast<float>(b[i]);
    db_out[i] = static_cast<float>(db[i]);
  }
}

// Rust's f32::clamp(min, max): NaN stays NaN.
inline float clampf(float v, float lo, float hi) { return v < lo ? lo : (v > hi ? hi : v); }

// Rust `x as usize` for a float: saturating, NaN -> 0.
inline long sat_usize(float x) {
  if (!(x > 0.0f)) return 0;
  if (x >= 1.8e19f) return 0x7fffffffffffffffL;
  return static_cast<long>(x);
}

// --------------------------------------------------------------------------------------------
// engine geometry: wave_wgpu.rs:204-270
// --------------------------------------------------------------------------------------------

struct Geo {
  wgo_config c;
  int pad, nx, nz, cells;
  std::vector<float> ax, bx, dbx, az, bz, dbz;
  std::vector<int> src_cell;   // [shots][4]
  std::vector<float> src_w;    // [shots][4]
  std::vector<int> rec_cell;   // [nrec][4]
  std::vector<float> rec_w;    // [nrec][4]
  std::vector<int> csr;        // [cells + 1]
  std::vector<int> ent_rec;    // receiver of each entry, entries ordered by (cell, receiver)
  std::vector<float> ent_w;
};

void corners(const Geo& g, float px, float pz, int* cell, float* w) {
  const float gx = px / g.c.h + static_cast<float>(g.pad);
  const float gz = pz / g.c.h + static_cast<float>(g.pad);
  const long x0 = std::min(sat_usize(std::floor(gx)), static_cast<long>(g.nx - 2));
  const long z0 = std::min(sat_usize(std::floor(gz)), static_cast<long>(g.nz - 2));
  const float fx = gx - static_cast<float>(x0);
  const float fz = gz - static_cast<float>(z0);
  cell[0] = static_cast<int>(z0 * g.nx + x0);
  cell[1] = static_cast<int>(z0 * g.nx + x0 + 1);
  cell[2] = static_cast<int>((z0 + 1) * g.nx + x0);
  cell[3] = static_cast<int>((z0 + 1) * g.nx + x0 + 1);
  w[0] = (1.0f - fx) * (1.0f - fz);
  w[1] = fx * (1.0f - fz);
  w[2] = (1.0f - fx) * fz;
  w[3] = fx * fz;
}

Geo make_geo(const wgo_config& c, const float* sources, const float* receivers) {
  Geo g;
  g.c = c;
  g.pad = FD_PAD + c.pml;
  g.nx = c.nx_vis + 2 * g.pad;
  g.nz = c.nz_vis + 2 * g.pad;
  g.cells = g.nx * g.nz;
  g.ax.resize(g.nx); g.bx.resize(g.nx); g.dbx.resize(g.nx);
  g.az.resize(g.nz); g.bz.resize(g.nz); g.dbz.resize(g.nz);
  cpml(g.nx, c.h, c.dt, c.pml, c.vmax, c.peak_hz, g.ax.data(), g.bx.data(), g.dbx.data());
  cpml(g.nz, c.h, c.dt, c.pml, c.vmax, c.peak_hz, g.az.data(), g.bz.data(), g.dbz.data());
  g.src_cell.resize(4 * c.shots); g.src_w.resize(4 * c.shots);
  for (int s = 0; s < c.shots; ++s) corners(g, sources[2 * s], sources[2 * s + 1], &g.src_cell[4 * s], &g.src_w[4 * s]);
  g.rec_cell.resize(4 * c.nrec); g.rec_w.resize(4 * c.nrec);
  for (int r = 0; r < c.nrec; ++r) {
    float px, pz;
    if (receivers) { px = receivers[2 * r]; pz = receivers[2 * r + 1]; }
    else { px = static_cast<float>(r) * c.h; pz = c.h; }  // wave_wgpu.rs:215
    corners(g, px, pz, &g.rec_cell[4 * r], &g.rec_w[4 * r]);
  }
  struct E { int cell, rec; float w; };
  std::vector<E> ents;
  for (int r = 0; r < c.nrec; ++r)
    for (int k = 0; k < 4; ++k)
      if (g.rec_w[4 * r + k] != 0.0f) ents.push_back({g.rec_cell[4 * r + k], r, g.rec_w[4 * r + k]});
  std::stable_sort(ents.begin(), ents.end(), [](const E& a, const E& b) {
    return a.cell != b.cell ? a.cell < b.cell : a.rec < b.rec;
  });
  g.csr.assign(g.cells + 1, 0);
  size_t e = 0;
  for (int cell = 0; cell <= g.cells; ++cell) {
    while (e < ents.size() && ents[e].cell < cell) ++e;
    g.csr[cell] = static_cast<int>(e);
  }
  for (const E& en : ents) { g.ent_rec.push_back(en.rec); g.ent_w.push_back(en.w); }
  return g;
}

// wave_wgpu.rs:714-734: edge replication, clamp to [vmin, vmax], clamp mask (strict inequalities).
void pad_velocity(const Geo& g, const float* v_vis, float* padded, float* mask) {
  const int nxv = g.c.nx_vis, nzv = g.c.nz_vis;
  for (int z = 0; z < g.nz; ++z) {
    const int vz = std::min(std::max(z - g.pad, 0), nzv - 1);
    for (int x = 0; x < g.nx; ++x) {
      const int vx = std::min(std::max(x - g.pad, 0), nxv - 1);
      const float v = v_vis[vz * nxv + vx];
      const int idx = z * g.nx + x;
      if (mask) mask[idx] = (v > g.c.vmin && v < g.c.vmax) ? 1.0f : 0.0f;
      padded[idx] = clampf(v, g.c.vmin, g.c.vmax);
    }
  }
}

// --------------------------------------------------------------------------------------------
// engine forward: splatForward.wgsl:48-121, one shot, all nt steps
// --------------------------------------------------------------------------------------------

template <typename R>
void forward_shot(const Geo& g, const float* vel_padded, int s, const float* wavelet, R* traces,
                  R* stored) {
  const int nx = g.nx, nz = g.nz, cells = g.cells, nt = g.c.nt, nrec = g.c.nrec;
  const int region = g.c.pml + 2 * FD_PAD;
  const R rh = R(1) / R(g.c.h);
  const R dt2 = R(g.c.dt) * R(g.c.dt);
  std::vector<R> cur(cells, R(0)), prev(cells, R(0));
  std::vector<R> psi(2 * cells, R(0)), psi_next(2 * cells, R(0)), zeta(2 * cells, R(0));
  std::vector<R> prof[2][3];
  {
    const std::vector<float>* src[2][3] = {{&g.ax, &g.bx, &g.dbx}, {&g.az, &g.bz, &g.dbz}};
    for (int ax = 0; ax < 2; ++ax)
      for (int k = 0; k < 3; ++k) prof[ax][k].assign(src[ax][k]->begin(), src[ax][k]->end());
  }
  const R c_d2a = R(-2.5), c_d2b = R(1.3333333333333333), c_d2c = R(0.08333333333333333);
  const R c_d1a = R(0.6666666666666666), c_d1b = R(0.08333333333333333);
  for (int t = 0; t < nt; ++t) {
    for (int r = 0; r < nrec; ++r) {
      R acc = R(0);
      for (int k = 0; k < 4; ++k) acc += R(g.rec_w[4 * r + k]) * cur[g.rec_cell[4 * r + k]];
      traces[static_cast<size_t>(t) * nrec + r] = acc;
    }
    const R f = R(wavelet[t]);
    for (int z = FD_PAD; z < nz - FD_PAD; ++z) {
      for (int x = FD_PAD; x < nx - FD_PAD; ++x) {
        const int i = z * nx + x;
        const R u = cur[i];
        R w = R(0);
        for (int axis = 0; axis < 2; ++axis) {
          const int stride = axis == 0 ? 1 : nx;
          const int along = axis == 0 ? x : z;
          const int n = axis == 0 ? nx : nz;
          const R* A = prof[axis][0].data();
          const R* B = prof[axis][1].data();
          const R* DB = prof[axis][2].data();
          const R um1 = cur[i - stride], up1 = cur[i + stride];
          const R um2 = cur[i - 2 * stride], up2 = cur[i + 2 * stride];
          const R d2 = (c_d2a * u + c_d2b * (up1 + um1) - c_d2c * (up2 + um2)) * rh * rh;
          const int ai = axis * cells + i;
          if (along < region || along >= n - region) {
            const R d1 = (c_d1a * (up1 - um1) - c_d1b * (up2 - um2)) * rh;
            const R a = A[along], b = B[along];
            const R ap1 = A[along + 1] * psi[ai + stride];
            const R am1 = A[along - 1] * psi[ai - stride];
            const R ap2 = A[along + 2] * psi[ai + 2 * stride];
            const R am2 = A[along - 2] * psi[ai - 2 * stride];
            const R d1_apsi = (c_d1a * (ap1 - am1) - c_d1b * (ap2 - am2)) * rh;
            const R tmp = (R(1) + b) * d2 + DB[along] * d1 + d1_apsi;
            w += (R(1) + b) * tmp + a * zeta[ai];
            psi_next[ai] = b * d1 + a * psi[ai];
            zeta[ai] = b * tmp + a * zeta[ai];
          } else {
            w += d2;
            psi_next[ai] = R(0);
          }
        }
        const R v = R(vel_padded[i]);
        const R v2dt2 = v * v * dt2;
        if (stored) stored[static_cast<size_t>(t) * cells + i] = R(2) * v * dt2 * w;
        R next = v2dt2 * w + R(2) * u - prev[i];
        for (int k = 0; k < 4; ++k)
          if (i == g.src_cell[4 * s + k]) next += -v2dt2 * R(g.src_w[4 * s + k]) * f;
        prev[i] = next;
      }
    }
    std::swap(cur, prev);
    std::swap(psi, psi_next);
  }
}

// --------------------------------------------------------------------------------------------
// engine adjoint: splatAdjoint.wgsl:58-131, one shot, t = nt-1 .. 0
// --------------------------------------------------------------------------------------------

template <typename R>
void adjoint_shot(const Geo& g, const float* vel_padded, int s, const float* wavelet, const R* residual,
                  const R* stored, R* grad) {
  const int nx = g.nx, nz = g.nz, cells = g.cells, nt = g.c.nt, nrec = g.c.nrec;
  const int region_adj = g.c.pml + 3 * FD_PAD;
  const R rh = R(1) / R(g.c.h);
  const R dt2 = R(g.c.dt) * R(g.c.dt);
  std::vector<R> lam[2] = {std::vector<R>(cells, R(0)), std::vector<R>(cells, R(0))};
  std::vector<R> lpsi[2] = {std::vector<R>(2 * cells, R(0)), std::vector<R>(2 * cells, R(0))};
  std::vector<R> lzeta[2] = {std::vector<R>(2 * cells, R(0)), std::vector<R>(2 * cells, R(0))};
  std::vector<R> prof[2][3];
  {
    const std::vector<float>* src[2][3] = {{&g.ax, &g.bx, &g.dbx}, {&g.az, &g.bz, &g.dbz}};
    for (int ax = 0; ax < 2; ++ax)
      for (int k = 0; k < 3; ++k) prof[ax][k].assign(src[ax][k]->begin(), src[ax][k]->end());
  }
  std::vector<R> vv(cells);
  for (int i = 0; i < cells; ++i) vv[i] = R(vel_padded[i]) * R(vel_padded[i]) * dt2;
  const R D1A = R(0.6666666666666666), D1B = R(-0.08333333333333333);
  const R D2A = R(-2.5), D2B = R(1.3333333333333333), D2C = R(-0.08333333333333333);
  std::fill(grad, grad + cells, R(0));
  for (int t = nt - 1; t >= 0; --t) {
    const int q = (nt - 1 - t) & 1;
    const std::vector<R>& cur = lam[q];
    std::vector<R>& prev = lam[1 - q];
    const std::vector<R>& psi_rd = lpsi[q];
    std::vector<R>& psi_wr = lpsi[1 - q];
    const std::vector<R>& zeta_rd = lzeta[q];
    std::vector<R>& zeta_wr = lzeta[1 - q];
    const R f = R(wavelet[t]);
    const R* res_t = residual + static_cast<size_t>(t) * nrec;
    const R* st_t = stored + static_cast<size_t>(t) * cells;
    for (int z = FD_PAD; z < nz - FD_PAD; ++z) {
      for (int x = FD_PAD; x < nx - FD_PAD; ++x) {
        const int i = z * nx + x;
        R w = R(0);
        for (int axis = 0; axis < 2; ++axis) {
          const int stride = axis == 0 ? 1 : nx;
          const int along = axis == 0 ? x : z;
          const int n = axis == 0 ? nx : nz;
          const R* A = prof[axis][0].data();
          const R* B = prof[axis][1].data();
          const R* DB = prof[axis][2].data();
          const R v0 = vv[i] * cur[i];
          const R vp1 = vv[i + stride] * cur[i + stride];
          const R vm1 = vv[i - stride] * cur[i - stride];
          const R vp2 = vv[i + 2 * stride] * cur[i + 2 * stride];
          const R vm2 = vv[i - 2 * stride] * cur[i - 2 * stride];
          if (along < region_adj || along >= n - region_adj) {
            const int base = axis * cells + i;
            R tt[5], u1[5], u2[5];
            const R vs[5] = {vm2, vm1, v0, vp1, vp2};
            for (int d = 0; d < 5; ++d) {
              const int k = along + d - 2;
              const int off = base + (d - 2) * stride;
              const R b = B[k];
              const R term = (R(1) + b) * vs[d] + b * zeta_rd[off];
              tt[d] = term;
              u1[d] = DB[k] * term + b * psi_rd[off];
              u2[d] = (R(1) + b) * term;
            }
            const R d1_u1 = (D1A * (u1[3] - u1[1]) + D1B * (u1[4] - u1[0])) * rh;
            const R d2_u2 = (D2A * u2[2] + D2B * (u2[3] + u2[1]) + D2C * (u2[4] + u2[0])) * rh * rh;
            const R d1_t = (D1A * (tt[3] - tt[1]) + D1B * (tt[4] - tt[0])) * rh;
            w += -d1_u1 + d2_u2;
            const R a = A[along];
            psi_wr[base] = -a * d1_t + a * psi_rd[base];
            zeta_wr[base] = a * v0 + a * zeta_rd[base];
          } else {
            w += (D2A * v0 + D2B * (vp1 + vm1) + D2C * (vp2 + vm2)) * rh * rh;
          }
        }
        R next = w + R(2) * cur[i] - prev[i];
        R gacc = R(0);
        gacc += cur[i] * st_t[i] * R(1);
        for (int e = g.csr[i]; e < g.csr[i + 1]; ++e) next += R(g.ent_w[e]) * res_t[g.ent_rec[e]];
        const R v = R(vel_padded[i]);
        for (int k = 0; k < 4; ++k)
          if (i == g.src_cell[4 * s + k]) gacc += cur[i] * (R(-2) * v * dt2 * R(g.src_w[4 * s + k]) * f);
        grad[i] += gacc;
        prev[i] = next;
      }
    }
  }
}

void parallel_for(int n, int threads, const std::function<void(int)>& fn) {
  if (threads <= 1 || n <= 1) {
    for (int i = 0; i < n; ++i) fn(i);
    return;
  }
  threads = std::min(threads, n);
  std::vector<std::thread> pool;
  std::atomic_int next{0};
  for (int k = 0; k < threads; ++k)
    pool.emplace_back([&]() {
      for (int i = next.fetch_add(1); i < n; i = next.fetch_add(1)) fn(i);
    });
  for (auto& th : pool) th.join();
}

// --------------------------------------------------------------------------------------------
// evaluate_adjoint host steps: wave_wgpu.rs:848-988 (energy in f64, f32 scale, residual in
// place, f64 loss, f32 shot-sum x clamp mask, f64 fold)
// --------------------------------------------------------------------------------------------

template <typename R>
void evaluate_adjoint_model(const Geo& g, const float* v_vis, const float* observed, const float* wavelet,
                            double* loss_out, R* grad_vis, R* raw_grad, int threads) {
  const int S = g.c.shots, nt = g.c.nt, nrec = g.c.nrec, cells = g.cells;
  const size_t tlen = static_cast<size_t>(S) * nt * nrec;
  double energy = 0.0;
  for (size_t i = 0; i < tlen; ++i) energy += static_cast<double>(observed[i]) * static_cast<double>(observed[i]);
  const R scale = static_cast<R>(1.0 / energy);
  std::vector<float> padded(cells), mask(cells);
  pad_velocity(g, v_vis, padded.data(), mask.data());
  std::vector<R> traces(tlen);
  std::vector<R> raw(static_cast<size_t>(S) * cells);
  std::vector<double> shot_loss(S, 0.0);
  parallel_for(S, threads, [&](int s) {
    std::vector<R> stored(static_cast<size_t>(nt) * cells);
    R* tr = traces.data() + static_cast<size_t>(s) * nt * nrec;
    forward_shot<R>(g, padded.data(), s, wavelet, tr, stored.data());
    const float* ob = observed + static_cast<size_t>(s) * nt * nrec;
    double e = 0.0;
    for (size_t i = 0; i < static_cast<size_t>(nt) * nrec; ++i) {
      const R d = tr[i] - R(ob[i]);
      tr[i] = d * scale;
      e += static_cast<double>(R(0.5) * d * d * scale);
    }
    shot_loss[s] = e;
    adjoint_shot<R>(g, padded.data(), s, wavelet, tr, stored.data(), raw.data() + static_cast<size_t>(s) * cells);
  });
  double loss = 0.0;
  for (int s = 0; s < S; ++s) loss += shot_loss[s];
  *loss_out = loss;
  std::vector<R> pg(cells);
  for (int c = 0; c < cells; ++c) {
    R sum = R(0);
    for (int s = 0; s < S; ++s) sum += raw[static_cast<size_t>(s) * cells + c];
    pg[c] = sum * R(mask[c]);
  }
  if (raw_grad) std::copy(raw.begin(), raw.end(), raw_grad);
  const int nxv = g.c.nx_vis, nzv = g.c.nz_vis;
  std::vector<double> acc(static_cast<size_t>(nxv) * nzv, 0.0);
  for (int z = 0; z < g.nz; ++z) {
    const int vz = std::min(std::max(z - g.pad, 0), nzv - 1);
    for (int x = 0; x < g.nx; ++x) {
      const int vx = std::min(std::max(x - g.pad, 0), nxv - 1);
      acc[vz * nxv + vx] += static_cast<double>(pg[z * g.nx + x]);
    }
  }
  for (size_t i = 0; i < acc.size(); ++i) grad_vis[i] = static_cast<R>(acc[i]);
}

bool valid(const wgo_config* c) {
  return c && c->nx_vis > 0 && c->nz_vis > 0 && c->pml >= 0 && c->shots > 0 && c->nt > 0 && c->nrec > 0 &&
         c->h > 0.0f && c->dt > 0.0f;
}

}  // namespace

extern "C" {

int wgo_ricker(int samples, float dt, float peak_hz, float* out) {
  if (samples < 0 || !out) return 1;
  ricker(samples, dt, peak_hz, out);
  return 0;
}

int wgo_cpml_profiles(int n, float h, float dt, int width, float max_vel, float freq, float* a, float* b, float* db) {
  if (n < 5 || !a || !b || !db) return 1;
  cpml(n, h, dt, width, max_vel, freq, a, b, db);
  return 0;
}

// geology-core simulate_shot_cpu (lib.rs:70-221), generalised to nx_vis x nz_vis visible cells.
// Receivers at every surface node (x = pad + r, z = pad + 1), recorded before each step;
// source injected after the update with bilinear weights; d2 uses rh2 = rh * rh.
int wgo_simulate_shot_cpu(const float* v_vis, int nxv, int nzv, float h, float dt, int nt, int pml, float vmin,
                          float vmax, float peak_hz, float src_x, float src_z, float* out) {
  if (!v_vis || !out || nxv <= 0 || nzv <= 0 || nt <= 0 || pml < 0) return 1;
  const int pad = FD_PAD + pml;
  const int nx = nxv + 2 * pad, nz = nzv + 2 * pad, cells = nx * nz;
  const int region = pml + 2 * FD_PAD;
  const float rh = 1.0f / h;
  const float rh2 = rh * rh;
  const float dt2 = dt * dt;
  std::vector<float> vel(cells);
  for (int z = 0; z < nz; ++z) {
    const int vz = std::min(std::max(z - pad, 0), nzv - 1);
    for (int x = 0; x < nx; ++x) {
      const int vx = std::min(std::max(x - pad, 0), nxv - 1);
      vel[z * nx + x] = clampf(v_vis[vz * nxv + vx], vmin, vmax);
    }
  }
  std::vector<float> ax(nx), bx(nx), dbx(nx), az(nz), bz(nz), dbz(nz);
  cpml(nx, h, dt, pml, vmax, peak_hz, ax.data(), bx.data(), dbx.data());
  cpml(nz, h, dt, pml, vmax, peak_hz, az.data(), bz.data(), dbz.data());
  std::vector<float> wavelet(nt);
  ricker(nt, dt, peak_hz, wavelet.data());
  const float gx = src_x / h + static_cast<float>(pad);
  const float gz = src_z / h + static_cast<float>(pad);
  const long x0 = std::min(sat_usize(std::floor(gx)), static_cast<long>(nx - 2));
  const long z0 = std::min(sat_usize(std::floor(gz)), static_cast<long>(nz - 2));
  const float fx = gx - static_cast<float>(x0);
  const float fz = gz - static_cast<float>(z0);
  const long sc[4] = {z0 * nx + x0, z0 * nx + x0 + 1, (z0 + 1) * nx + x0, (z0 + 1) * nx + x0 + 1};
  const float sw[4] = {(1.0f - fx) * (1.0f - fz), fx * (1.0f - fz), (1.0f - fx) * fz, fx * fz};
  const int rec_z = pad + 1;
  std::vector<float> cur(cells, 0.0f), prev(cells, 0.0f), psi_x(cells, 0.0f), psi_x_next(cells, 0.0f),
      psi_z(cells, 0.0f), psi_z_next(cells, 0.0f), zeta_x(cells, 0.0f), zeta_z(cells, 0.0f);
  const float C1 = 0.6666666666666666f, C2 = 0.08333333333333333f;
  const float D0 = -2.5f, D1 = 1.3333333333333333f, D2 = 0.08333333333333333f;
  for (int t = 0; t < nt; ++t) {
    for (int r = 0; r < nxv; ++r) out[static_cast<size_t>(t) * nxv + r] = cur[rec_z * nx + (pad + r)];
    for (int z = FD_PAD; z < nz - FD_PAD; ++z) {
      const bool in_pml_z = z < region || z >= nz - region;
      for (int x = FD_PAD; x < nx - FD_PAD; ++x) {
        const int i = z * nx + x;
        const float u = cur[i];
        float w = 0.0f;
        const float um1x = cur[i - 1], up1x = cur[i + 1], um2x = cur[i - 2], up2x = cur[i + 2];
        const float d2x = (D0 * u + D1 * (up1x + um1x) - D2 * (up2x + um2x)) * rh2;
        if (x < region || x >= nx - region) {
          const float d1x = (C1 * (up1x - um1x) - C2 * (up2x - um2x)) * rh;
          const float a = ax[x], b = bx[x];
          const float ap1 = ax[x + 1] * psi_x[i + 1];
          const float am1 = ax[x - 1] * psi_x[i - 1];
          const float ap2 = ax[x + 2] * psi_x[i + 2];
          const float am2 = ax[x - 2] * psi_x[i - 2];
          const float d1_apsi = (C1 * (ap1 - am1) - C2 * (ap2 - am2)) * rh;
          const float tmp = (1.0f + b) * d2x + dbx[x] * d1x + d1_apsi;
          w += (1.0f + b) * tmp + a * zeta_x[i];
          psi_x_next[i] = b * d1x + a * psi_x[i];
          zeta_x[i] = b * tmp + a * zeta_x[i];
        } else {
          w += d2x;
          psi_x_next[i] = 0.0f;
        }
        const float um1z = cur[i - nx], up1z = cur[i + nx], um2z = cur[i - 2 * nx], up2z = cur[i + 2 * nx];
        const float d2z = (D0 * u + D1 * (up1z + um1z) - D2 * (up2z + um2z)) * rh2;
        if (in_pml_z) {
          const float d1z = (C1 * (up1z - um1z) - C2 * (up2z - um2z)) * rh;
          const float a = az[z], b = bz[z];
          const float ap1 = az[z + 1] * psi_z[i + nx];
          const float am1 = az[z - 1] * psi_z[i - nx];
          const float ap2 = az[z + 2] * psi_z[i + 2 * nx];
          const float am2 = az[z - 2] * psi_z[i - 2 * nx];
          const float d1_apsi = (C1 * (ap1 - am1) - C2 * (ap2 - am2)) * rh;
          const float tmp = (1.0f + b) * d2z + dbz[z] * d1z + d1_apsi;
          w += (1.0f + b) * tmp + a * zeta_z[i];
          psi_z_next[i] = b * d1z + a * psi_z[i];
          zeta_z[i] = b * tmp + a * zeta_z[i];
        } else {
          w += d2z;
          psi_z_next[i] = 0.0f;
        }
        const float v = vel[i];
        prev[i] = v * v * dt2 * w + 2.0f * u - prev[i];
      }
    }
    const float f_t = wavelet[t];
    for (int k = 0; k < 4; ++k)
      if (sw[k] != 0.0f) {
        const float v = vel[sc[k]];
        prev[sc[k]] += -(v * v * dt2) * sw[k] * f_t;
      }
    std::swap(cur, prev);
    std::swap(psi_x, psi_x_next);
    std::swap(psi_z, psi_z_next);
  }
  return 0;
}

// Engine geometry as the GPU receives it (for cross-checks of the product's geometry builder).
int wgo_geometry(const wgo_config* c, const float* sources, const float* receivers, int* src_cell, float* src_w,
                 int* rec_cell, float* rec_w, int* csr, int* n_entries) {
  if (!valid(c) || !sources) return 1;
  Geo g = make_geo(*c, sources, receivers);
  if (src_cell) std::copy(g.src_cell.begin(), g.src_cell.end(), src_cell);
  if (src_w) std::copy(g.src_w.begin(), g.src_w.end(), src_w);
  if (rec_cell) std::copy(g.rec_cell.begin(), g.rec_cell.end(), rec_cell);
  if (rec_w) std::copy(g.rec_w.begin(), g.rec_w.end(), rec_w);
  if (csr) std::copy(g.csr.begin(), g.csr.end(), csr);
  if (n_entries) *n_entries = static_cast<int>(g.ent_rec.size());
  return 0;
}

int wgo_pad_velocity(const wgo_config* c, const float* v_vis, float* padded, float* mask) {
  if (!valid(c) || !v_vis || !padded) return 1;
  float dummy[2] = {0, 0};
  wgo_config cc = *c;
  cc.shots = 1;
  Geo g = make_geo(cc, dummy, nullptr);
  pad_velocity(g, v_vis, padded, mask);
  return 0;
}

// Engine forward for `models` velocity models: traces [models][shots][nt][nrec]; optionally
// the stored gradient terms 2 v dt^2 w of every step [models][shots][nt][cells].
int wgo_forward_f32(const wgo_config* c, int models, const float* v_vis, const float* sources,
                    const float* receivers, const float* wavelet, float* traces, float* stored, int threads) {
  if (!valid(c) || models <= 0 || !v_vis || !sources || !wavelet || !traces) return 1;
  Geo g = make_geo(*c, sources, receivers);
  const size_t vis = static_cast<size_t>(c->nx_vis) * c->nz_vis;
  const size_t tshot = static_cast<size_t>(c->nt) * c->nrec;
  parallel_for(models * c->shots, threads, [&](int u) {
    const int m = u / c->shots, s = u % c->shots;
    std::vector<float> padded(g.cells);
    pad_velocity(g, v_vis + m * vis, padded.data(), nullptr);
    forward_shot<float>(g, padded.data(), s, wavelet, traces + static_cast<size_t>(u) * tshot,
                        stored ? stored + static_cast<size_t>(u) * c->nt * g.cells : nullptr);
  });
  return 0;
}

int wgo_forward_f64(const wgo_config* c, int models, const float* v_vis, const float* sources,
                    const float* receivers, const float* wavelet, double* traces, int threads) {
  if (!valid(c) || models <= 0 || !v_vis || !sources || !wavelet || !traces) return 1;
  Geo g = make_geo(*c, sources, receivers);
  const size_t vis = static_cast<size_t>(c->nx_vis) * c->nz_vis;
  const size_t tshot = static_cast<size_t>(c->nt) * c->nrec;
  parallel_for(models * c->shots, threads, [&](int u) {
    const int m = u / c->shots, s = u % c->shots;
    std::vector<float> padded(g.cells);
    pad_velocity(g, v_vis + m * vis, padded.data(), nullptr);
    forward_shot<double>(g, padded.data(), s, wavelet, traces + static_cast<size_t>(u) * tshot, nullptr);
  });
  return 0;
}

// evaluate_adjoint for `models` models: loss [models] (f64), folded gradient [models][nz_vis][nx_vis]
// in dJ/d(v in m/s); optionally the raw per-shot padded gradient [models][shots][cells].
// Models run one after another; the shots of a model run on up to `threads` threads.
int wgo_evaluate_adjoint_f32(const wgo_config* c, int models, const float* v_vis, const float* sources,
                             const float* receivers, const float* wavelet, const float* observed, double* loss,
                             float* grad, float* raw_grad, int threads) {
  if (!valid(c) || models <= 0 || !v_vis || !sources || !wavelet || !observed || !loss || !grad) return 1;
  Geo g = make_geo(*c, sources, receivers);
  const size_t vis = static_cast<size_t>(c->nx_vis) * c->nz_vis;
  const size_t tmodel = static_cast<size_t>(c->shots) * c->nt * c->nrec;
  for (int m = 0; m < models; ++m) {
    double e = 0.0;
    for (size_t i = 0; i < tmodel; ++i) e += static_cast<double>(observed[m * tmodel + i]) * observed[m * tmodel + i];
    if (!(e > 0.0)) return 2;  // wave_wgpu.rs:853 asserts positive energy
    evaluate_adjoint_model<float>(g, v_vis + m * vis, observed + m * tmodel, wavelet, loss + m, grad + m * vis,
                                  raw_grad ? raw_grad + static_cast<size_t>(m) * c->shots * g.cells : nullptr,
                                  threads);
  }
  return 0;
}

int wgo_evaluate_adjoint_f64(const wgo_config* c, int models, const float* v_vis, const float* sources,
                             const float* receivers, const float* wavelet, const float* observed, double* loss,
                             double* grad, int threads) {
  if (!valid(c) || models <= 0 || !v_vis || !sources || !wavelet || !observed || !loss || !grad) return 1;
  Geo g = make_geo(*c, sources, receivers);
  const size_t vis = static_cast<size_t>(c->nx_vis) * c->nz_vis;
  const size_t tmodel = static_cast<size_t>(c->shots) * c->nt * c->nrec;
  for (int m = 0; m < models; ++m) {
    double e = 0.0;
    for (size_t i = 0; i < tmodel; ++i) e += static_cast<double>(observed[m * tmodel + i]) * observed[m * tmodel + i];
    if (!(e > 0.0)) return 2;
    evaluate_adjoint_model<double>(g, v_vis + m * vis, observed + m * tmodel, wavelet, loss + m, grad + m * vis,
                                   nullptr, threads);
  }
  return 0;
}

// CPU baseline throughput driver: `models` gradients with one (model) per worker thread, all
// shots of a model on that thread (the reference's CPU solver is single-threaded per shot).
int wgo_gradients_parallel_f32(const wgo_config* c, int models, const float* v_vis, const float* sources,
                               const float* receivers, const float* wavelet, const float* observed, double* loss,
                               float* grad, int threads) {
  if (!valid(c) || models <= 0 || !v_vis || !sources || !wavelet || !observed || !loss || !grad) return 1;
  Geo g = make_geo(*c, sources, receivers);
  const size_t vis = static_cast<size_t>(c->nx_vis) * c->nz_vis;
  const size_t tmodel = static_cast<size_t>(c->shots) * c->nt * c->nrec;
  std::atomic_int bad{0};
  parallel_for(models, threads, [&](int m) {
    double e = 0.0;
    for (size_t i = 0; i < tmodel; ++i) e += static_cast<double>(observed[m * tmodel + i]) * observed[m * tmodel + i];
    if (!(e > 0.0)) { bad = 1; return; }
    evaluate_adjoint_model<float>(g, v_vis + m * vis, observed + m * tmodel, wavelet, loss + m, grad + m * vis,
                                  nullptr, 1);
  });
  return bad ? 2 : 0;
}

}  // extern "C"
