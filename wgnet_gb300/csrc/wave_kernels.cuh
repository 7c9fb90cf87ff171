// Kernel templates of the resident time-stepping kernels for the 4th-order C-PML acoustic solver and its exact discrete
// adjoint (the work of splatForward.wgsl / splatAdjoint.wgsl, reorganised for sm_103a).
//
// One cluster of C CTAs owns one (model, shot) unit for all the steps of a launch. The rows of the
// padded grid are split over the CTAs; every wavefield the stencil reads at neighbours lives in
// shared memory (double-buffered, so a step needs one barrier), per-cell private state lives in
// registers, and the two halo rows a CTA needs from its neighbour are pushed into the neighbour's
// shared memory through DSMEM after each update. Global memory sees only the velocity (read
// once), the receiver traces, checkpoints, and the per-step gradient terms of a segment.
//
// Arithmetic: compiled with -fmad=false; every expression follows the reference's operation
// order, so results are bit-identical to the f32 restatement of the reference.
#pragma once
#include <cuda_runtime.h>

#include "wave_device.cuh"
#include "wave_launch.h"

namespace wg {

// ------------------------------------------------------------------------------------------------
// Forward: splatForward.wgsl:48-121 (receivers before the step, frame cells untouched, source
// after the update, stored term 2 v dt^2 w before the source).
// ------------------------------------------------------------------------------------------------
template <int C, int NT, int CPT, bool TRACES, bool STORE>
__global__ void __launch_bounds__(NT, 1) fwd_kernel(const __grid_constant__ FwdArgs p) {
  extern __shared__ __align__(16) float sm[];
  const Grid& g = p.g;
  const int nx = g.nx, nz = g.nz, sw = g.sw, W = nx - 2 * FD_PAD;
  const int region = g.region, nrec = p.st.nrec;
  const float rh = g.rh, dt2 = g.dt2, d2a = g.d2a, d2b = g.d2b;
  const int tid = threadIdx.x;
  const int rank = (C > 1) ? static_cast<int>(cluster_rank()) : 0;
  const int unit = blockIdx.x / C;
  const int shot = unit % p.st.shots;
  const int model = unit / p.st.shots;
  const size_t cells = static_cast<size_t>(nx) * nz;
  const FwdLayout L = fwd_layout(nx, nz, sw, C, nrec);
  const int r0 = split_row(nz, C, rank), r1 = split_row(nz, C, rank + 1);
  const int zl0 = r0 - FD_PAD;
  const int own = (r1 - r0) * W;
  const int bot_off = (C == 1) ? sw : 0;
  const int ustride = L.lr * nx, xstride = L.maxrows * 2 * sw, zstride = L.zs * nx;
  float* U = sm + L.off_u;
  float* APX = sm + L.off_apx;
  float* APZ = sm + L.off_apz;
  float* sAX = sm + L.off_prof;
  float* sBX = sAX + nx;
  float* sDBX = sBX + nx;
  float* sAZ = sDBX + nx;
  float* sBZ = sAZ + nz;
  float* sDBZ = sBZ + nz;
  int* sRecCell = reinterpret_cast<int*>(sm + L.off_rec);
  float* sRecW = sm + L.off_rec + 4 * nrec;
  int* sRecOk = reinterpret_cast<int*>(sm + L.off_rec + 8 * nrec);

  for (int i = tid; i < L.total; i += NT) sm[i] = 0.0f;
  __syncthreads();
  for (int i = tid; i < 3 * (nx + nz); i += NT) sAX[i] = g.prof[i];
  if (TRACES) {
    for (int r = tid; r < nrec; r += NT) {
      const int z0 = p.st.rec_cell[4 * r] / nx;
      const bool ok = (z0 >= r0 || rank == 0) && (z0 < r1 || rank == C - 1);
      sRecOk[r] = ok ? 1 : 0;
      for (int k = 0; k < 4; ++k) {
        const int cell = p.st.rec_cell[4 * r + k];
        sRecCell[4 * r + k] = ok ? (cell / nx - zl0) * nx + cell % nx : 0;
        sRecW[4 * r + k] = p.st.rec_w[4 * r + k];
      }
    }
  }

  // Cells of this thread: j = tid + m * NT over the CTA's rows, row-major over updated columns.
  int xz[CPT];
  float v2[CPT], zx[CPT], zz[CPT];
  float vv[STORE ? CPT : 1];
  unsigned srcmask = 0;
  const int* sc = p.st.src_cell + 4 * shot;
  const float* vel = p.vel + static_cast<size_t>(model) * cells;
#pragma unroll
  for (int m = 0; m < CPT; ++m) {
    const int j = tid + m * NT;
    zx[m] = 0.0f;
    zz[m] = 0.0f;
    xz[m] = 0;
    v2[m] = 0.0f;
    if (STORE) vv[m] = 0.0f;
    if (j < own) {
      const int z = r0 + j / W, x = FD_PAD + j % W;
      xz[m] = x | (z << 16);
      const float v = vel[z * nx + x];
      v2[m] = v * v * dt2;
      if (STORE) vv[m] = v;
      const int cell = z * nx + x;
      if (cell == sc[0] || cell == sc[1] || cell == sc[2] || cell == sc[3]) srcmask |= 1u << m;
    }
  }

  // Initial state: a checkpoint (state at the start of step t0) or zeros.
  const size_t ckf = ckpt_floats(nx, nz, sw);
  if (p.ck_in) {
    const float* ck = p.ck_in + (static_cast<size_t>(unit) * p.ck_slots + p.ck_in_slot) * ckf;
    const float* cU = ck;
    const float* cP = ck + cells;
    const float* cAX = ck + 2 * cells;
    const float* cAZ = cAX + static_cast<size_t>(nz) * 2 * sw;
    const float* cZX = cAZ + static_cast<size_t>(2) * sw * nx;
    const float* cZZ = cZX + static_cast<size_t>(nz) * 2 * sw;
    // U_cur with halo rows (frame rows stay zero).
    const int ra = max(r0 - FD_PAD, FD_PAD), rb = min(r1 + FD_PAD, nz - FD_PAD);
    for (int i = tid; i < (rb - ra) * W; i += NT) {
      const int z = ra + i / W, x = FD_PAD + i % W;
      U[(z - zl0) * nx + x] = cU[z * nx + x];
    }
#pragma unroll
    for (int m = 0; m < CPT; ++m) {
      if (tid + m * NT < own) {
        const int x = xz[m] & 0xffff, z = xz[m] >> 16;
        U[ustride + (z - zl0) * nx + x] = cP[z * nx + x];
        if (x < sw || x >= nx - sw) {
          const int xs = strip_col(x, nx, sw);
          APX[(z - r0) * 2 * sw + xs] = cAX[z * 2 * sw + xs];
          zx[m] = cZX[z * 2 * sw + xs];
        }
        if (z < sw || z >= nz - sw) {
          const int zsc = strip_col(z, nz, sw);
          const int zss = (z < sw) ? z : z - (nz - sw) + bot_off;
          APZ[zss * nx + x] = cAZ[zsc * nx + x];
          zz[m] = cZZ[zsc * nx + x];
        }
      }
    }
  }
  if constexpr (C > 1) cluster_barrier();
  else __syncthreads();

  const int pr_lo = (rank > 0) ? split_row(nz, C, rank - 1) - FD_PAD : 0;  // peer rank-1 zl0
  for (int t = p.t0; t < p.t1; ++t) {
    const int par = (t - p.t0) & 1;
    const float* Uc = U + par * ustride;
    float* Un = U + (1 - par) * ustride;
    const float* APXc = APX + par * xstride;
    float* APXn = APX + (1 - par) * xstride;
    const float* APZc = APZ + par * zstride;
    float* APZn = APZ + (1 - par) * zstride;

    if (TRACES) {
      for (int r = tid; r < nrec; r += NT) {
        if (sRecOk[r]) {
          float acc = 0.0f;
#pragma unroll
          for (int k = 0; k < 4; ++k) acc = acc + sRecW[4 * r + k] * Uc[sRecCell[4 * r + k]];
          p.traces[(static_cast<size_t>(unit) * g.nt + t) * nrec + r] = acc;
        }
      }
    }

    float* ckw = nullptr;
    if (p.ck_out && t > p.t0 && (t % p.ck_every) == 0)
      ckw = p.ck_out + (static_cast<size_t>(unit) * p.ck_slots + (t / p.ck_every - 1)) * ckf;

    const float f = __ldg(&g.wavelet[t]);
    float* st_t = STORE ? p.stored + (static_cast<size_t>(unit) * (p.t1 - p.t0) + (t - p.t0)) * cells : nullptr;

#pragma unroll
    for (int m = 0; m < CPT; ++m) {
      if (tid + m * NT < own) {
        int xzm = xz[m];
        asm volatile("" : "+r"(xzm));  // keep per-cell index math inside the step loop
        const int x = xzm & 0xffff, z = xzm >> 16;
        const int c = (z - zl0) * nx + x;
        const bool sx = (x < sw || x >= nx - sw);
        const bool sz = (z < sw || z >= nz - sw);
        const int ca = (z - r0) * 2 * sw + strip_col(x, nx, sw);
        const int zss = (z < sw) ? z : z - (nz - sw) + bot_off;
        const int cz = zss * nx + x;
        if (ckw) {
          ckw[z * nx + x] = Uc[c];
          ckw[cells + z * nx + x] = Un[c];
          float* cAX = ckw + 2 * cells;
          float* cAZ = cAX + static_cast<size_t>(nz) * 2 * sw;
          float* cZX = cAZ + static_cast<size_t>(2) * sw * nx;
          float* cZZ = cZX + static_cast<size_t>(nz) * 2 * sw;
          if (sx) {
            const int xs = strip_col(x, nx, sw);
            cAX[z * 2 * sw + xs] = APXc[ca];
            cZX[z * 2 * sw + xs] = zx[m];
          }
          if (sz) {
            const int zsc = strip_col(z, nz, sw);
            cAZ[zsc * nx + x] = APZc[cz];
            cZZ[zsc * nx + x] = zz[m];
          }
        }
        const float u = Uc[c];
        float w = 0.0f;
        {  // x axis
          const float um1 = Uc[c - 1], up1 = Uc[c + 1], um2 = Uc[c - 2], up2 = Uc[c + 2];
          const float d2 = (((F_D2A * u + F_D2B * (up1 + um1)) - F_D2C * (up2 + um2)) * d2a) * d2b;
          if (x < region || x >= nx - region) {
            const float d1 = ((F_D1A * (up1 - um1)) - F_D1B * (up2 - um2)) * rh;
            const float a = sAX[x], b = sBX[x], db = sDBX[x];
            const float ap1 = APXc[ca + 1], am1 = APXc[ca - 1], ap2 = APXc[ca + 2], am2 = APXc[ca - 2];
            const float d1_apsi = ((F_D1A * (ap1 - am1)) - F_D1B * (ap2 - am2)) * rh;
            const float opb = 1.0f + b;
            const float tmp = ((opb * d2) + (db * d1)) + d1_apsi;
            w = w + ((opb * tmp) + (a * zx[m]));
            const float psin = (b * d1) + APXc[ca];
            zx[m] = (b * tmp) + (a * zx[m]);
            APXn[ca] = a * psin;
          } else {
            w = w + d2;
          }
        }
        {  // z axis
          const float um1 = Uc[c - nx], up1 = Uc[c + nx], um2 = Uc[c - 2 * nx], up2 = Uc[c + 2 * nx];
          const float d2 = (((F_D2A * u + F_D2B * (up1 + um1)) - F_D2C * (up2 + um2)) * d2a) * d2b;
          if (z < region || z >= nz - region) {
            const float d1 = ((F_D1A * (up1 - um1)) - F_D1B * (up2 - um2)) * rh;
            const float a = sAZ[z], b = sBZ[z], db = sDBZ[z];
            const float ap1 = APZc[cz + nx], am1 = APZc[cz - nx], ap2 = APZc[cz + 2 * nx],
                        am2 = APZc[cz - 2 * nx];
            const float d1_apsi = ((F_D1A * (ap1 - am1)) - F_D1B * (ap2 - am2)) * rh;
            const float opb = 1.0f + b;
            const float tmp = ((opb * d2) + (db * d1)) + d1_apsi;
            w = w + ((opb * tmp) + (a * zz[m]));
            const float psin = (b * d1) + APZc[cz];
            zz[m] = (b * tmp) + (a * zz[m]);
            APZn[cz] = a * psin;
          } else {
            w = w + d2;
          }
        }
        if (STORE) st_t[z * nx + x] = ((2.0f * vv[m]) * dt2) * w;
        float nxt = ((v2[m] * w) + (2.0f * u)) - Un[c];
        if (srcmask & (1u << m)) {
          const int cell = z * nx + x;
#pragma unroll
          for (int k = 0; k < 4; ++k)
            if (cell == sc[k]) nxt = nxt + (((-v2[m]) * p.st.src_w[4 * shot + k]) * f);
        }
        Un[c] = nxt;
        if constexpr (C > 1) {
          if (rank > 0 && z < r0 + FD_PAD) st_peer(&Un[(z - pr_lo) * nx + x], rank - 1, nxt);
          if (rank < C - 1 && z >= r1 - FD_PAD) st_peer(&Un[(z - (r1 - FD_PAD)) * nx + x], rank + 1, nxt);
        }
        (void)sx;
        (void)sz;
      }
    }
    step_barrier<C>();
  }
}

// ------------------------------------------------------------------------------------------------
// Adjoint: splatAdjoint.wgsl:58-131. The per-neighbour terms the shader recomputes for each of
// the five stencil points (term = (1+b) vs + b zeta, u1 = db term + b psi) depend only on the
// neighbour cell, so each cell computes its own once per step into shared memory ("derived"
// arrays VS, TX/U1X, TZ/U1Z) and the stencil reads them; the values are identical.
// ------------------------------------------------------------------------------------------------
template <int C, int NT, int CPT>
__global__ void __launch_bounds__(NT, 1) adj_kernel(const __grid_constant__ AdjArgs p) {
  extern __shared__ __align__(16) float sm[];
  const Grid& g = p.g;
  const int nx = g.nx, nz = g.nz, swa = g.swa, W = nx - 2 * FD_PAD;
  const int region = g.region_adj, nrec = p.st.nrec, nt = g.nt;
  const float rh = g.rh, dt2 = g.dt2;
  const int tid = threadIdx.x;
  const int rank = (C > 1) ? static_cast<int>(cluster_rank()) : 0;
  const int unit = blockIdx.x / C;
  const int shot = unit % p.st.shots;
  const int model = unit / p.st.shots;
  const size_t cells = static_cast<size_t>(nx) * nz;
  const AdjLayout L = adj_layout(nx, nz, swa, C);
  const int r0 = split_row(nz, C, rank), r1 = split_row(nz, C, rank + 1);
  const int zl0 = r0 - FD_PAD;
  const int own = (r1 - r0) * W;
  const int bot_off = (C == 1) ? swa : 0;
  const int vstride = L.lr * nx, xstride = L.maxrows * 2 * swa, zstride = L.zs * nx;
  float* VS = sm + L.off_vs;
  float* TX = sm + L.off_tx;
  float* U1X = sm + L.off_u1x;
  float* TZ = sm + L.off_tz;
  float* U1Z = sm + L.off_u1z;
  float* LPX = sm + L.off_lpx;
  float* LZX = sm + L.off_lzx;
  float* LPZ = sm + L.off_lpz;
  float* LZZ = sm + L.off_lzz;
  float* sAX = sm + L.off_prof;
  float* sBX = sAX + nx;
  float* sDBX = sBX + nx;
  float* sAZ = sDBX + nx;
  float* sBZ = sAZ + nz;
  float* sDBZ = sBZ + nz;

  for (int i = tid; i < L.total; i += NT) sm[i] = 0.0f;
  __syncthreads();
  for (int i = tid; i < 3 * (nx + nz); i += NT) sAX[i] = g.prof[i];

  int xz[CPT];
  float v2[CPT], lc[CPT], lp[CPT], ga[CPT];
  unsigned srcmask = 0, recmask = 0;
  const int* sc = p.st.src_cell + 4 * shot;
  const float* vel = p.vel + static_cast<size_t>(model) * cells;
  const size_t asf = adjstate_floats(nx, nz, swa);
  float* stt = p.state + static_cast<size_t>(unit) * asf;
  float* sLc = stt;
  float* sLp = stt + cells;
  float* sPX = stt + 2 * cells;
  float* sZX = sPX + static_cast<size_t>(nz) * 2 * swa;
  float* sPZ = sZX + static_cast<size_t>(nz) * 2 * swa;
  float* sZZ = sPZ + static_cast<size_t>(2) * swa * nx;
  float* gacc = p.gacc + static_cast<size_t>(unit) * cells;
  __syncthreads();
#pragma unroll
  for (int m = 0; m < CPT; ++m) {
    const int j = tid + m * NT;
    xz[m] = 0;
    v2[m] = 0.0f;
    lc[m] = 0.0f;
    lp[m] = 0.0f;
    ga[m] = 0.0f;
    if (j < own) {
      const int z = r0 + j / W, x = FD_PAD + j % W;
      xz[m] = x | (z << 16);
      const int cell = z * nx + x;
      const float v = vel[cell];
      v2[m] = v * v * dt2;
      if (cell == sc[0] || cell == sc[1] || cell == sc[2] || cell == sc[3]) srcmask |= 1u << m;
      if (p.st.csr[cell] < p.st.csr[cell + 1]) recmask |= 1u << m;
      if (!p.first) {
        lc[m] = sLc[cell];
        lp[m] = sLp[cell];
        ga[m] = gacc[cell];
        if (x < swa || x >= nx - swa) {
          const int xs = strip_col(x, nx, swa);
          LPX[(z - r0) * 2 * swa + xs] = sPX[z * 2 * swa + xs];
          LZX[(z - r0) * 2 * swa + xs] = sZX[z * 2 * swa + xs];
        }
        if (z < swa || z >= nz - swa) {
          const int zsc = strip_col(z, nz, swa);
          const int zss = (z < swa) ? z : z - (nz - swa) + bot_off;
          LPZ[zss * nx + x] = sPZ[zsc * nx + x];
          LZZ[zss * nx + x] = sZZ[zsc * nx + x];
        }
      }
    }
  }
  if constexpr (C > 1) cluster_barrier();
  else __syncthreads();

  const int pr_lo = (rank > 0) ? split_row(nz, C, rank - 1) - FD_PAD : 0;

  // Derived arrays of this thread's cells into buffer `b`.
  auto derive = [&](int b) {
    float* VSb = VS + b * vstride;
    float* TXb = TX + b * xstride;
    float* U1Xb = U1X + b * xstride;
    float* TZb = TZ + b * zstride;
    float* U1Zb = U1Z + b * zstride;
#pragma unroll
    for (int m = 0; m < CPT; ++m) {
      if (tid + m * NT < own) {
        int xzm = xz[m];
        asm volatile("" : "+r"(xzm));
        const int x = xzm & 0xffff, z = xzm >> 16;
        const float vs = v2[m] * lc[m];
        VSb[(z - zl0) * nx + x] = vs;
        if constexpr (C > 1) {
          if (rank > 0 && z < r0 + FD_PAD) st_peer(&VSb[(z - pr_lo) * nx + x], rank - 1, vs);
          if (rank < C - 1 && z >= r1 - FD_PAD) st_peer(&VSb[(z - (r1 - FD_PAD)) * nx + x], rank + 1, vs);
        }
        if (x < swa || x >= nx - swa) {
          const int ca = (z - r0) * 2 * swa + strip_col(x, nx, swa);
          const float bb = sBX[x], db = sDBX[x];
          const float T = ((1.0f + bb) * vs) + (bb * LZX[ca]);
          TXb[ca] = T;
          U1Xb[ca] = (db * T) + (bb * LPX[ca]);
        }
        if (z < swa || z >= nz - swa) {
          const int cz = ((z < swa) ? z : z - (nz - swa) + bot_off) * nx + x;
          const float bb = sBZ[z], db = sDBZ[z];
          const float T = ((1.0f + bb) * vs) + (bb * LZZ[cz]);
          TZb[cz] = T;
          U1Zb[cz] = (db * T) + (bb * LPZ[cz]);
        }
      }
    }
  };

  derive(0);
  step_barrier<C>();

  const int seg = p.t_hi - p.t_lo;
  for (int t = p.t_hi - 1; t >= p.t_lo; --t) {
    const int par = (p.t_hi - 1 - t) & 1;
    const float* VSd = VS + par * vstride;
    const float* TXd = TX + par * xstride;
    const float* U1Xd = U1X + par * xstride;
    const float* TZd = TZ + par * zstride;
    const float* U1Zd = U1Z + par * zstride;
    const float f = __ldg(&g.wavelet[t]);
    const float* st_t = p.stored + (static_cast<size_t>(unit) * seg + (t - p.t_lo)) * cells;
    const float* res_t = p.residual + (static_cast<size_t>(unit) * nt + t) * nrec;
#pragma unroll
    for (int m = 0; m < CPT; ++m) {
      if (tid + m * NT < own) {
        int xzm = xz[m];
        asm volatile("" : "+r"(xzm));
        const int x = xzm & 0xffff, z = xzm >> 16;
        const int cv = (z - zl0) * nx + x;
        const float v0 = VSd[cv];
        float w = 0.0f;
        {  // x axis
          if (x < region || x >= nx - region) {
            const int ca = (z - r0) * 2 * swa + strip_col(x, nx, swa);
            const float t0_ = TXd[ca - 2], t1_ = TXd[ca - 1], t2_ = TXd[ca], t3_ = TXd[ca + 1], t4_ = TXd[ca + 2];
            const float u10 = U1Xd[ca - 2], u11 = U1Xd[ca - 1], u13 = U1Xd[ca + 1], u14 = U1Xd[ca + 2];
            const float u20 = (1.0f + sBX[x - 2]) * t0_;
            const float u21 = (1.0f + sBX[x - 1]) * t1_;
            const float u22 = (1.0f + sBX[x]) * t2_;
            const float u23 = (1.0f + sBX[x + 1]) * t3_;
            const float u24 = (1.0f + sBX[x + 2]) * t4_;
            const float d1_u1 = ((F_D1A * (u13 - u11)) + (A_D1B * (u14 - u10))) * rh;
            const float d2_u2 = ((((F_D2A * u22) + (F_D2B * (u23 + u21))) + (A_D2C * (u24 + u20))) * rh) * rh;
            const float d1_t = ((F_D1A * (t3_ - t1_)) + (A_D1B * (t4_ - t0_))) * rh;
            w = w + ((-d1_u1) + d2_u2);
            const float a = sAX[x];
            LPX[ca] = ((-a) * d1_t) + (a * LPX[ca]);
            LZX[ca] = (a * v0) + (a * LZX[ca]);
          } else {
            const float vp1 = VSd[cv + 1], vm1 = VSd[cv - 1], vp2 = VSd[cv + 2], vm2 = VSd[cv - 2];
            w = w + ((((F_D2A * v0) + (F_D2B * (vp1 + vm1))) + (A_D2C * (vp2 + vm2))) * rh) * rh;
          }
        }
        {  // z axis
          if (z < region || z >= nz - region) {
            const int cz = ((z < swa) ? z : z - (nz - swa) + bot_off) * nx + x;
            const float t0_ = TZd[cz - 2 * nx], t1_ = TZd[cz - nx], t2_ = TZd[cz], t3_ = TZd[cz + nx],
                        t4_ = TZd[cz + 2 * nx];
            const float u10 = U1Zd[cz - 2 * nx], u11 = U1Zd[cz - nx], u13 = U1Zd[cz + nx], u14 = U1Zd[cz + 2 * nx];
            const float u20 = (1.0f + sBZ[z - 2]) * t0_;
            const float u21 = (1.0f + sBZ[z - 1]) * t1_;
            const float u22 = (1.0f + sBZ[z]) * t2_;
            const float u23 = (1.0f + sBZ[z + 1]) * t3_;
            const float u24 = (1.0f + sBZ[z + 2]) * t4_;
            const float d1_u1 = ((F_D1A * (u13 - u11)) + (A_D1B * (u14 - u10))) * rh;
            const float d2_u2 = ((((F_D2A * u22) + (F_D2B * (u23 + u21))) + (A_D2C * (u24 + u20))) * rh) * rh;
            const float d1_t = ((F_D1A * (t3_ - t1_)) + (A_D1B * (t4_ - t0_))) * rh;
            w = w + ((-d1_u1) + d2_u2);
            const float a = sAZ[z];
            LPZ[cz] = ((-a) * d1_t) + (a * LPZ[cz]);
            LZZ[cz] = (a * v0) + (a * LZZ[cz]);
          } else {
            const float vp1 = VSd[cv + nx], vm1 = VSd[cv - nx], vp2 = VSd[cv + 2 * nx], vm2 = VSd[cv - 2 * nx];
            w = w + ((((F_D2A * v0) + (F_D2B * (vp1 + vm1))) + (A_D2C * (vp2 + vm2))) * rh) * rh;
          }
        }
        const int cell = z * nx + x;
        float nxt = (w + (2.0f * lc[m])) - lp[m];
        float gt = 0.0f;
        gt = gt + ((lc[m] * st_t[cell]) * 1.0f);
        if (recmask & (1u << m)) {
          const int e1 = p.st.csr[cell + 1];
          for (int e = p.st.csr[cell]; e < e1; ++e) nxt = nxt + (p.st.ent_w[e] * res_t[p.st.ent_rec[e]]);
        }
        if (srcmask & (1u << m)) {
          const float v = vel[cell];
#pragma unroll
          for (int k = 0; k < 4; ++k)
            if (cell == sc[k]) gt = gt + lc[m] * (((((-2.0f) * v) * dt2) * p.st.src_w[4 * shot + k]) * f);
        }
        ga[m] = ga[m] + gt;
        lp[m] = lc[m];
        lc[m] = nxt;
      }
    }
    if (t > p.t_lo) derive(1 - par);
    step_barrier<C>();
  }

  // Save the state for the next (earlier) segment and the gradient accumulator.
#pragma unroll
  for (int m = 0; m < CPT; ++m) {
    if (tid + m * NT < own) {
      const int x = xz[m] & 0xffff, z = xz[m] >> 16;
      const int cell = z * nx + x;
      sLc[cell] = lc[m];
      sLp[cell] = lp[m];
      gacc[cell] = ga[m];
      if (x < swa || x >= nx - swa) {
        const int xs = strip_col(x, nx, swa);
        sPX[z * 2 * swa + xs] = LPX[(z - r0) * 2 * swa + xs];
        sZX[z * 2 * swa + xs] = LZX[(z - r0) * 2 * swa + xs];
      }
      if (z < swa || z >= nz - swa) {
        const int zsc = strip_col(z, nz, swa);
        const int zss = (z < swa) ? z : z - (nz - swa) + bot_off;
        sPZ[zsc * nx + x] = LPZ[zss * nx + x];
        sZZ[zsc * nx + x] = LZZ[zss * nx + x];
      }
    }
  }
}


template <typename Args>
cudaError_t launch_cluster(void (*kernel)(Args), int C, int NT, int units, size_t smem, cudaStream_t stream,
                           const Args& args) {
  cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  if (e != cudaSuccess) return e;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(units * C);
  cfg.blockDim = dim3(NT);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = C;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, args);
}

template <int C, int NT, int CPT>
cudaError_t fwd_dispatch_impl(bool traces, bool store, const FwdArgs& a, size_t smem, cudaStream_t s) {
  if (traces && store) return launch_cluster(fwd_kernel<C, NT, CPT, true, true>, C, NT, a.units, smem, s, a);
  if (traces) return launch_cluster(fwd_kernel<C, NT, CPT, true, false>, C, NT, a.units, smem, s, a);
  if (store) return launch_cluster(fwd_kernel<C, NT, CPT, false, true>, C, NT, a.units, smem, s, a);
  return cudaErrorInvalidValue;
}


template <int C, int NT, int CPT>
cudaError_t adj_dispatch_impl(const AdjArgs& a, size_t smem, cudaStream_t s) {
  return launch_cluster(adj_kernel<C, NT, CPT>, C, NT, a.units, smem, s, a);
}

}  // namespace wg
