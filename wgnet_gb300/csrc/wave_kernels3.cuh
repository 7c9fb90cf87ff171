// Third-generation resident kernels (forward and adjoint) for grids of compile-time width NX.
//
// Thread mapping: each thread owns a pair of adjacent columns (x, x+1) over a segment of S rows.
// Per segment, one "PML warp" owns the PMLP leftmost and PMLP rightmost column pairs (exactly the
// C-PML region of the adjoint, which contains the forward's) and runs the PML formulas; the
// remaining "interior warps" own the pairs in between and run the interior formulas, so no warp
// diverges on the PML test. With NX known at compile time every shared-memory access of a row is
// a per-thread base register plus an immediate offset.
//
// Values a cell's neighbours read (the wavefield, a*psi, the adjoint's derived terms) are exchanged
// through double-buffered shared memory (one barrier per step); a thread's own leapfrog pair stays
// in registers, and the update writes the new value over the oldest one, alternating the roles of
// the two register arrays every step. Arithmetic follows the reference's operation order (the
// library is built with -fmad=false), so results are bit-identical to the f32 restatement.
#pragma once
#include <cuda_runtime.h>

#include "wave_device.cuh"
#include "wave_kernels.cuh"
#include "wave_kernels3_layout.h"
#include "wave_launch.h"

namespace wg {

// Column layout of a generation-3 kernel.
//
// The PML warp's left pairs sit on lanes [0, PMLP) and its right pairs on lanes [16, 16 + PMLP):
// a 64-bit shared-memory access is served per half-warp, and with the right pairs starting at lane
// PMLP both halves of the row ran into the same banks (the last left pair and the first right pair
// of a 114-wide row, and the packed strips' left and right columns), replaying a wavefront on
// every access of the PML warp. Each half-warp now reads one contiguous run of columns.
template <int NX, int PMLP>
struct Cols3 {
  static_assert(PMLP <= 16, "the PML warp holds at most 16 column pairs per side");
  static constexpr int PCOLS = 2 * PMLP;          // PML columns per side, starting at x = 2
  static constexpr int SW = PCOLS + 4;            // packed strip width per side (reads reach x+3); = g3_sw
  static constexpr int IPAIRS = (NX - 4 - 2 * PCOLS) / 2;
  __device__ static int x_of(int wk, int lane) {
    if (wk == 0) return lane < 16 ? FD_PAD + 2 * lane : (NX - FD_PAD - PCOLS) + 2 * (lane - 16);
    return FD_PAD + PCOLS + 2 * ((wk - 1) * 32 + lane);
  }
  __device__ static bool active(int wk, int lane) {
    if (wk == 0) return (lane & 15) < PMLP;
    return (wk - 1) * 32 + lane < IPAIRS;
  }
  __host__ __device__ static int strip(int x) { return x < SW ? x : x - (NX - 2 * SW); }
};

// Role of warp `warp` within its segment (0: the PML warp). Warp w issues from scheduler w % 4; with
// 2 or 4 warps per segment a fixed role per position would put every PML warp (the heavier work) on
// the same schedulers, so the roles rotate from segment to segment.
template <int NI>
__device__ __forceinline__ int warp_role(int warp) {
  constexpr int W = 1 + NI;
  const int seg = warp / W, j = warp % W;
  if constexpr (4 % W == 0) return (j + (seg * W) / 4) % W;
  return j;
}

// Wavelet ring in shared memory: the sample of step u (counted from the launch's first step, in
// the launch's direction) sits at W[u % G3_WAV_STEPS]. The launch starts with the first
// G3_WAV_STEPS samples; every G3_WAV_STEPS / 2 steps the threads `ltid` < G3_WAV_STEPS / 2 load the
// half G3_WAV_STEPS / 2 .. G3_WAV_STEPS steps ahead, before that step's barrier (the slots they
// overwrite were read in earlier steps). `time(u)` maps a step count to the wavelet index.
template <class TimeOf>
__device__ __forceinline__ void wavelet_ring_fill(float* W, const float* wav, int u0, int u1, int steps, int tid,
                                                  int nthreads, TimeOf time) {
  for (int u = u0 + tid; u < u1 && u < steps; u += nthreads) W[u % G3_WAV_STEPS] = wav[time(u)];
}

// Thread order for the per-step receiver work (trace recording, residual staging): it starts at a
// segment away from the z strips and from the rows sent to the peer CTAs, whose warps have the
// least to do per step.
template <int NSEG, int NI, int C>
__device__ __forceinline__ int light_tid(int tid, int rank) {
  constexpr int SEGT = 32 * (1 + NI), NT = NSEG * SEGT;
  const int ls = (C == 1) ? NSEG / 2 : (rank == 0 ? NSEG / 2 + 1 : 1);
  return (tid - ls * SEGT + NT) % NT;
}

// Fast arithmetic (the forward's FA kernels): the reference's stencils with 1/h and 1/h^2 folded
// into the weights and the products fused (fmaf rounds once). The same discrete operator as the
// reference's operation order, rounded differently: results agree with the unfused kernels to f32
// accuracy, not bit for bit. Weights: k0 = -5/2 / h^2, k1 = 4/3 / h^2, k2 = -1/12 / h^2 (second
// difference), e1 = 2/3 / h, e2 = -1/12 / h (first difference). The adjoint keeps the reference
// order: a fused variant of it measured 1.3 % slower than the unfused one (its longer dependency
// chains cost more than its 11 % fewer instructions save), so it was not kept.
struct FastCoef {
  float k0, k1, k2, k00, e1, e2;
  __device__ __forceinline__ static FastCoef make(float rh) {
    const float rh2 = rh * rh;
    FastCoef c;
    c.k0 = F_D2A * rh2;
    c.k1 = F_D2B * rh2;
    c.k2 = -F_D2C * rh2;
    c.k00 = 2.0f * c.k0;
    c.e1 = F_D1A * rh;
    c.e2 = -F_D1B * rh;
    return c;
  }
  // second difference along one axis from the centre value and the sums of the +-1 and +-2 neighbours
  __device__ __forceinline__ float d2(float u, float s1, float s2) const { return fmaf(k2, s2, fmaf(k1, s1, k0 * u)); }
  // acc + the second difference along one axis
  __device__ __forceinline__ float d2acc(float acc, float u, float s1, float s2) const {
    return fmaf(k2, s2, fmaf(k1, s1, fmaf(k0, u, acc)));
  }
  // both axes' second differences of a cell, s1 / s2 summed over its four neighbours at distance 1 / 2
  __device__ __forceinline__ float lap(float u, float s1, float s2) const { return fmaf(k2, s2, fmaf(k1, s1, k00 * u)); }
  // first difference from (u[+1] - u[-1]) and (u[+2] - u[-2])
  __device__ __forceinline__ float d1(float dd1, float dd2) const { return fmaf(e2, dd2, e1 * dd1); }
};

__device__ __forceinline__ float2 lds2(const float* p) { return *reinterpret_cast<const float2*>(p); }
__device__ __forceinline__ void sts2(float* p, float a, float b) { *reinterpret_cast<float2*>(p) = make_float2(a, b); }

// Store to the peer CTA's copy of a shared array. The address translation is a pure function; the
// store has no memory clobber, so it does not pin this thread's other shared-memory accesses, none
// of which touch the peer's copy. It stays ahead of the step's cluster fence and barrier because
// those are volatile asm too.
__device__ __forceinline__ void st_peer_v2(const float* local_ptr, unsigned peer, float a, float b) {
  unsigned la = static_cast<unsigned>(__cvta_generic_to_shared(local_ptr));
  unsigned ra;
  asm("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(ra) : "r"(la), "r"(peer));
  asm volatile("st.shared::cluster.v2.f32 [%0], {%1, %2};" ::"r"(ra), "f"(a), "f"(b));
}

// ------------------------------------------------------------------------------------------------
// Forward (splatForward.wgsl:48-121)
// ------------------------------------------------------------------------------------------------
// Row layouts (LAY): LAY_RUNTIME, any nz; LAY_EVEN, the rows split evenly into the segments (every
// segment has exactly S rows); LAY_SQUARE, a square grid (nz = NX), so nz and every shared-memory
// offset are compile-time constants (and the rows split evenly when C S NSEG = NX - 4).
enum : int { LAY_RUNTIME = 0, LAY_EVEN = 1, LAY_SQUARE = 2 };

// FA: fast arithmetic (see FastCoef); otherwise the reference's operation order, unfused.
template <int NX, int PMLP, int C, int S, int NSEG, int NI, int LAY, bool TRACES, bool STORE, bool FA = false>
__global__ void __launch_bounds__(NSEG * 32 * (1 + NI), 1) fwd3_kernel(const __grid_constant__ FwdArgs p) {
  using CL = Cols3<NX, PMLP>;
  constexpr int SW = CL::SW;
  constexpr int NT = NSEG * 32 * (1 + NI);
  extern __shared__ __align__(16) float sm[];
  const Grid& g = p.g;
  constexpr bool SQ = LAY == LAY_SQUARE;
  constexpr bool FULL = LAY == LAY_EVEN || (SQ && NX - 2 * FD_PAD == C * S * NSEG);
  const int nz = SQ ? NX : g.nz;
  const int sw = g.sw, region = g.region, nrec = p.st.nrec;
  const float rh = g.rh, dt2 = g.dt2, d2a = g.d2a, d2b = g.d2b;
  const FastCoef fc = FastCoef::make(rh);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int seg = warp / (1 + NI), wk = warp_role<NI>(warp);
  const int rank = (C > 1) ? static_cast<int>(cluster_rank()) : 0;
  const int unit = blockIdx.x / C;
  const int shot = unit % p.st.shots;
  const int model = unit / p.st.shots;
  const size_t cells = static_cast<size_t>(NX) * nz;
  const F3Layout L = f3_layout_rt(NX, PMLP, nz, sw, C, nrec);
  const int r0 = split_row(nz, C, rank), r1 = split_row(nz, C, rank + 1);
  const int zl0 = r0 - FD_PAD;
  const int bot_off = (C == 1) ? sw : 0;
  const int ustride = L.lr * NX, xstride = L.maxrows * 2 * SW, zstride = L.zs * NX;
  float* U = sm + L.off_u;
  float* APX = sm + L.off_apx;
  float* ZX = sm + L.off_zx;
  float* APZ = sm + L.off_apz;
  float* ZZ = sm + L.off_zz;
  float* sAZ = sm + L.off_prof + 3 * NX;
  float* sBZ = sAZ + nz;
  float* sDBZ = sBZ + nz;
  int* sRecCell = reinterpret_cast<int*>(sm + L.off_rec);
  float* sRecW = sm + L.off_rec + 4 * nrec;
  int* sRecOk = reinterpret_cast<int*>(sm + L.off_rec + 8 * nrec);

  for (int i = tid; i < L.total; i += NT) sm[i] = 0.0f;
  __syncthreads();
  for (int i = tid; i < 3 * (NX + nz); i += NT) sm[L.off_prof + i] = g.prof[i];
  if (TRACES) {
    for (int r = tid; r < nrec; r += NT) {
      const int z0 = p.st.rec_cell[4 * r] / NX;
      const bool ok = (z0 >= r0 || rank == 0) && (z0 < r1 || rank == C - 1);
      sRecOk[r] = ok ? 1 : 0;
      for (int k = 0; k < 4; ++k) {
        const int cell = p.st.rec_cell[4 * r + k];
        sRecCell[4 * r + k] = ok ? (cell / NX - zl0) * NX + cell % NX : 0;
        sRecW[4 * r + k] = p.st.rec_w[4 * r + k];
      }
    }
  }

  const bool pml = (wk == 0);
  const int x = CL::x_of(wk, lane);
  const int zb = r0 + seg * S;
  const int ltid = light_tid<NSEG, NI, C>(tid, rank);
  const int nrows = CL::active(wk, lane) ? (FULL ? S : max(0, min(S, r1 - zb))) : 0;
  const bool pusher = (C > 1) && nrows > 0 && ((rank > 0 && zb < r0 + FD_PAD) || (rank < C - 1 && zb + nrows > r1 - FD_PAD));
  const int ubase = (zb - zl0) * NX + x;                 // row 0 of the segment in U
  const int abase = (zb - r0) * 2 * SW + CL::strip(x);   // row 0 in APX / ZX (PML warp)
  const int zsh = (zb < nz / 2) ? 0 : (nz - sw - bot_off);
  const int zbase = (zb - zsh) * NX + x;                 // row 0 in APZ / ZZ (z-strip rows)
  const int gbase = zb * NX + x;                         // row 0 in a global [nz][NX] field

  float ax0 = 0.f, ax1 = 0.f, bx0 = 0.f, bx1 = 0.f, dbx0 = 0.f, dbx1 = 0.f;
  if (pml) {
    ax0 = g.prof[x];
    ax1 = g.prof[x + 1];
    bx0 = g.prof[NX + x];
    bx1 = g.prof[NX + x + 1];
    dbx0 = g.prof[2 * NX + x];
    dbx1 = g.prof[2 * NX + x + 1];
  }
  const float opbx0 = 1.0f + bx0, opbx1 = 1.0f + bx1;

  float uA[S][2], uB[S][2];
  unsigned srcmask = 0;
  const int* sc = p.st.src_cell + 4 * shot;
  const float* vel = p.vel + static_cast<size_t>(model) * cells + gbase;
  // Source corners: cell and the step-invariant factor (-v^2 dt^2) w of the shader's
  // (((-v^2 dt^2) w) f); the wavelet samples come from a ring in shared memory, so the injection
  // reads shared memory only.
  int* sSrcCell = reinterpret_cast<int*>(sm + L.off_src);
  float* sSrcQ = sm + L.off_src + 4;
  float* sW = sm + L.off_src + 8;
  const int wsteps = p.t1 - p.t0;
  auto wtime = [&](int u) { return p.t0 + u; };
  if (tid < 4) {
    const int cell = sc[tid];
    const float v = p.vel[static_cast<size_t>(model) * cells + cell];
    sSrcCell[tid] = cell;
    sSrcQ[tid] = (-(v * v * dt2)) * p.st.src_w[4 * shot + tid];
  }
  wavelet_ring_fill(sW, g.wavelet, 0, G3_WAV_STEPS, wsteps, tid, NT, wtime);
  float* V2o = sm + L.off_v2 + (zb - r0) * NX + x;  // owner-only coefficient rows
  float* C2o = sm + L.off_c2 + (zb - r0) * NX + x;
#pragma unroll
  for (int i = 0; i < S; ++i) {
    uA[i][0] = uA[i][1] = uB[i][0] = uB[i][1] = 0.f;
    if (i < nrows) {
      const float2 v = __ldg(reinterpret_cast<const float2*>(vel + i * NX));
      sts2(V2o + i * NX, v.x * v.x * dt2, v.y * v.y * dt2);
      if (STORE) sts2(C2o + i * NX, (2.0f * v.x) * dt2, (2.0f * v.y) * dt2);
      const int cell = gbase + i * NX;
      if (cell == sc[0] || cell == sc[1] || cell == sc[2] || cell == sc[3]) srcmask |= 1u << (2 * i);
      if (cell + 1 == sc[0] || cell + 1 == sc[1] || cell + 1 == sc[2] || cell + 1 == sc[3])
        srcmask |= 1u << (2 * i + 1);
    }
  }

  const size_t ckf = ckpt_floats(NX, nz, sw);
  if (p.ck_in) {
    const float* ck = p.ck_in + (static_cast<size_t>(unit) * p.ck_slots + p.ck_in_slot) * ckf;
    const float* cU = ck;
    const float* cP = ck + cells;
    const float* cAX = ck + 2 * cells;
    const float* cAZ = cAX + static_cast<size_t>(nz) * 2 * sw;
    const float* cZX = cAZ + static_cast<size_t>(2) * sw * NX;
    const float* cZZ = cZX + static_cast<size_t>(nz) * 2 * sw;
    constexpr int W = NX - 2 * FD_PAD;
    const int ra = max(r0 - FD_PAD, FD_PAD), rb = min(r1 + FD_PAD, nz - FD_PAD);
    for (int i = tid; i < (rb - ra) * W; i += NT) {
      const int z = ra + i / W, xx = FD_PAD + i % W;
      U[(z - zl0) * NX + xx] = cU[z * NX + xx];
    }
#pragma unroll
    for (int i = 0; i < S; ++i) {
      if (i < nrows) {
        const int z = zb + i;
#pragma unroll
        for (int j = 0; j < 2; ++j) {
          const int xx = x + j;
          uA[i][j] = cU[z * NX + xx];
          uB[i][j] = cP[z * NX + xx];
          if (xx < sw || xx >= NX - sw) {
            const int xc = strip_col(xx, NX, sw);
            APX[abase + i * 2 * SW + j] = cAX[z * 2 * sw + xc];
            ZX[abase + i * 2 * SW + j] = cZX[z * 2 * sw + xc];
          }
          if (z < sw || z >= nz - sw) {
            const int zc = strip_col(z, nz, sw);
            APZ[zbase + i * NX + j] = cAZ[zc * NX + xx];
            ZZ[zbase + i * NX + j] = cZZ[zc * NX + xx];
          }
        }
      }
    }
  }
  // rows where any lane of the warp injects the source: warp-uniform branches, per-lane selects
  const unsigned wsrc = __reduce_or_sync(0xffffffffu, srcmask);
  if constexpr (C > 1) cluster_barrier();
  else __syncthreads();

  const int pr_lo = (rank > 0) ? split_row(nz, C, rank - 1) - FD_PAD : 0;

  auto step = [&](int t, float (&uc)[S][2], float (&un)[S][2]) {
    const int par = (t - p.t0) & 1;
    const float* Uc = U + par * ustride + ubase;
    float* Un = U + (1 - par) * ustride + ubase;
    const float* APXc = APX + par * xstride + abase;
    float* APXn = APX + (1 - par) * xstride + abase;
    float* ZXo = ZX + abase;
    const float* APZc = APZ + par * zstride + zbase;
    float* APZn = APZ + (1 - par) * zstride + zbase;
    float* ZZo = ZZ + zbase;

    if (p.ck_out && t > p.t0 && (t % p.ck_every) == 0) {
      float* ck = p.ck_out + (static_cast<size_t>(unit) * p.ck_slots + (t / p.ck_every - 1)) * ckf;
      float* cAX = ck + 2 * cells;
      float* cAZ = cAX + static_cast<size_t>(nz) * 2 * sw;
      float* cZX = cAZ + static_cast<size_t>(2) * sw * NX;
      float* cZZ = cZX + static_cast<size_t>(nz) * 2 * sw;
#pragma unroll
      for (int i = 0; i < S; ++i) {
        if (i < nrows) {
          const int z = zb + i;
#pragma unroll
          for (int j = 0; j < 2; ++j) {
            const int xx = x + j;
            ck[z * NX + xx] = uc[i][j];
            ck[cells + z * NX + xx] = un[i][j];
            if (xx < sw || xx >= NX - sw) {
              const int xc = strip_col(xx, NX, sw);
              cAX[z * 2 * sw + xc] = APXc[i * 2 * SW + j];
              cZX[z * 2 * sw + xc] = ZXo[i * 2 * SW + j];
            }
            if (z < sw || z >= nz - sw) {
              const int zc = strip_col(z, nz, sw);
              cAZ[zc * NX + xx] = APZc[i * NX + j];
              cZZ[zc * NX + xx] = ZZo[i * NX + j];
            }
          }
        }
      }
    }

    const float f = sW[(t - p.t0) % G3_WAV_STEPS];
    float* st = STORE ? p.stored + (static_cast<size_t>(unit) * (p.t1 - p.t0) + (t - p.t0)) * cells + gbase : nullptr;
    // The row updates write only through these restrict-qualified pointers (disjoint arrays), so
    // the compiler may issue a row's loads ahead of the previous row's stores.
    auto rows = [&](float* __restrict__ uw, float* __restrict__ apxn, float* __restrict__ zxo,
                    float* __restrict__ apzn, float* __restrict__ zzo, float* __restrict__ stg) {
#pragma unroll
      for (int i = 0; i < S; ++i) {
        if (i < nrows) {
          const int z = zb + i;
          const float2 A = lds2(Uc + i * NX - 2);
          const float2 B = lds2(Uc + i * NX + 2);
          float zm2[2], zm1[2], zp1[2], zp2[2];
          if (i >= 2) {
            zm2[0] = uc[i - 2][0];
            zm2[1] = uc[i - 2][1];
          } else {
            const float2 q = lds2(Uc + (i - 2) * NX);
            zm2[0] = q.x;
            zm2[1] = q.y;
          }
          if (i >= 1) {
            zm1[0] = uc[i - 1][0];
            zm1[1] = uc[i - 1][1];
          } else {
            const float2 q = lds2(Uc + (i - 1) * NX);
            zm1[0] = q.x;
            zm1[1] = q.y;
          }
          if (i + 1 < S && (FULL || i + 1 < nrows)) {
            zp1[0] = uc[i + 1 < S ? i + 1 : i][0];
            zp1[1] = uc[i + 1 < S ? i + 1 : i][1];
          } else {
            const float2 q = lds2(Uc + (i + 1) * NX);
            zp1[0] = q.x;
            zp1[1] = q.y;
          }
          if (i + 2 < S && (FULL || i + 2 < nrows)) {
            zp2[0] = uc[i + 2 < S ? i + 2 : i][0];
            zp2[1] = uc[i + 2 < S ? i + 2 : i][1];
          } else {
            const float2 q = lds2(Uc + (i + 2) * NX);
            zp2[0] = q.x;
            zp2[1] = q.y;
          }
          const float u0 = uc[i][0], u1 = uc[i][1];
          float n0, n1;
          if constexpr (FA) {
            // the same update, reassociated: 1/h and 1/h^2 folded into the stencil weights, the
            // interior x and z second differences summed before weighting, products fused
            const bool zpml = z < region || z >= nz - region;
            float w0, w1;
            if (pml) {
              const float2 P0 = lds2(APXc + i * 2 * SW - 2);
              const float2 P1 = lds2(APXc + i * 2 * SW);
              const float2 P2 = lds2(APXc + i * 2 * SW + 2);
              const float2 Z = lds2(zxo + i * 2 * SW);
              // cell x: neighbours x-2..x+2 = A.x, A.y, u0, u1, B.x; cell x+1: A.y, u0, u1, B.x, B.y
              const float d2x0 = fc.d2(u0, u1 + A.y, B.x + A.x);
              const float d2x1 = fc.d2(u1, B.x + u0, B.y + A.y);
              const float d10 = fc.d1(u1 - A.y, B.x - A.x);
              const float d11 = fc.d1(B.x - u0, B.y - A.y);
              const float da0 = fc.d1(P1.y - P0.y, P2.x - P0.x);
              const float da1 = fc.d1(P2.x - P1.x, P2.y - P0.y);
              const float tmp0 = fmaf(opbx0, d2x0, fmaf(dbx0, d10, da0));
              const float tmp1 = fmaf(opbx1, d2x1, fmaf(dbx1, d11, da1));
              const float az0 = ax0 * Z.x, az1 = ax1 * Z.y;
              w0 = fmaf(opbx0, tmp0, az0);
              w1 = fmaf(opbx1, tmp1, az1);
              sts2(zxo + i * 2 * SW, fmaf(bx0, tmp0, az0), fmaf(bx1, tmp1, az1));
              sts2(apxn + i * 2 * SW, ax0 * fmaf(bx0, d10, P1.x), ax1 * fmaf(bx1, d11, P1.y));
              if (!zpml) {
                w0 = fc.d2acc(w0, u0, zp1[0] + zm1[0], zp2[0] + zm2[0]);
                w1 = fc.d2acc(w1, u1, zp1[1] + zm1[1], zp2[1] + zm2[1]);
              }
            } else if (!zpml) {  // interior in both axes: one weighted sum of both axes' neighbours
              w0 = fc.lap(u0, (u1 + A.y) + (zp1[0] + zm1[0]), (B.x + A.x) + (zp2[0] + zm2[0]));
              w1 = fc.lap(u1, (B.x + u0) + (zp1[1] + zm1[1]), (B.y + A.y) + (zp2[1] + zm2[1]));
            } else {
              w0 = fc.d2(u0, u1 + A.y, B.x + A.x);
              w1 = fc.d2(u1, B.x + u0, B.y + A.y);
            }
            if (zpml) {
              const float az = sAZ[z], bz = sBZ[z], dbz = sDBZ[z];
              const float opbz = 1.0f + bz;
              const float2 Qm2 = lds2(APZc + (i - 2) * NX);
              const float2 Qm1 = lds2(APZc + (i - 1) * NX);
              const float2 Q0 = lds2(APZc + i * NX);
              const float2 Qp1 = lds2(APZc + (i + 1) * NX);
              const float2 Qp2 = lds2(APZc + (i + 2) * NX);
              const float2 Z = lds2(zzo + i * NX);
              const float d2z0 = fc.d2(u0, zp1[0] + zm1[0], zp2[0] + zm2[0]);
              const float d2z1 = fc.d2(u1, zp1[1] + zm1[1], zp2[1] + zm2[1]);
              const float d10 = fc.d1(zp1[0] - zm1[0], zp2[0] - zm2[0]);
              const float d11 = fc.d1(zp1[1] - zm1[1], zp2[1] - zm2[1]);
              const float da0 = fc.d1(Qp1.x - Qm1.x, Qp2.x - Qm2.x);
              const float da1 = fc.d1(Qp1.y - Qm1.y, Qp2.y - Qm2.y);
              const float tmp0 = fmaf(opbz, d2z0, fmaf(dbz, d10, da0));
              const float tmp1 = fmaf(opbz, d2z1, fmaf(dbz, d11, da1));
              const float az0 = az * Z.x, az1 = az * Z.y;
              w0 = w0 + fmaf(opbz, tmp0, az0);
              w1 = w1 + fmaf(opbz, tmp1, az1);
              sts2(zzo + i * NX, fmaf(bz, tmp0, az0), fmaf(bz, tmp1, az1));
              sts2(apzn + i * NX, az * fmaf(bz, d10, Q0.x), az * fmaf(bz, d11, Q0.y));
            }
            const float2 vv = lds2(V2o + i * NX);
            if (STORE) {
              const float2 cc = lds2(C2o + i * NX);
              *reinterpret_cast<float2*>(stg + i * NX) = make_float2(cc.x * w0, cc.y * w1);
            }
            n0 = fmaf(vv.x, w0, fmaf(2.0f, u0, -un[i][0]));
            n1 = fmaf(vv.y, w1, fmaf(2.0f, u1, -un[i][1]));
          } else {
            const float d2x0 = (((F_D2A * u0 + F_D2B * (u1 + A.y)) - F_D2C * (B.x + A.x)) * d2a) * d2b;
            const float d2x1 = (((F_D2A * u1 + F_D2B * (B.x + u0)) - F_D2C * (B.y + A.y)) * d2a) * d2b;
            float w0, w1;
            if (pml) {
              const float2 P0 = lds2(APXc + i * 2 * SW - 2);
              const float2 P1 = lds2(APXc + i * 2 * SW);
              const float2 P2 = lds2(APXc + i * 2 * SW + 2);
              const float2 Z = lds2(zxo + i * 2 * SW);
              const float d10 = ((F_D1A * (u1 - A.y)) - F_D1B * (B.x - A.x)) * rh;
              const float d11 = ((F_D1A * (B.x - u0)) - F_D1B * (B.y - A.y)) * rh;
              const float da0 = ((F_D1A * (P1.y - P0.y)) - F_D1B * (P2.x - P0.x)) * rh;
              const float da1 = ((F_D1A * (P2.x - P1.x)) - F_D1B * (P2.y - P0.y)) * rh;
              const float tmp0 = ((opbx0 * d2x0) + (dbx0 * d10)) + da0;
              const float tmp1 = ((opbx1 * d2x1) + (dbx1 * d11)) + da1;
              w0 = (opbx0 * tmp0) + (ax0 * Z.x);
              w1 = (opbx1 * tmp1) + (ax1 * Z.y);
              const float psi0 = (bx0 * d10) + P1.x;
              const float psi1 = (bx1 * d11) + P1.y;
              sts2(zxo + i * 2 * SW, (bx0 * tmp0) + (ax0 * Z.x), (bx1 * tmp1) + (ax1 * Z.y));
              sts2(apxn + i * 2 * SW, ax0 * psi0, ax1 * psi1);
            } else {
              w0 = d2x0;
              w1 = d2x1;
            }
            const float d2z0 = (((F_D2A * u0 + F_D2B * (zp1[0] + zm1[0])) - F_D2C * (zp2[0] + zm2[0])) * d2a) * d2b;
            const float d2z1 = (((F_D2A * u1 + F_D2B * (zp1[1] + zm1[1])) - F_D2C * (zp2[1] + zm2[1])) * d2a) * d2b;
            if (z < region || z >= nz - region) {
              const float az = sAZ[z], bz = sBZ[z], dbz = sDBZ[z];
              const float opbz = 1.0f + bz;
              const float2 Qm2 = lds2(APZc + (i - 2) * NX);
              const float2 Qm1 = lds2(APZc + (i - 1) * NX);
              const float2 Q0 = lds2(APZc + i * NX);
              const float2 Qp1 = lds2(APZc + (i + 1) * NX);
              const float2 Qp2 = lds2(APZc + (i + 2) * NX);
              const float2 Z = lds2(zzo + i * NX);
              const float d10 = ((F_D1A * (zp1[0] - zm1[0])) - F_D1B * (zp2[0] - zm2[0])) * rh;
              const float d11 = ((F_D1A * (zp1[1] - zm1[1])) - F_D1B * (zp2[1] - zm2[1])) * rh;
              const float da0 = ((F_D1A * (Qp1.x - Qm1.x)) - F_D1B * (Qp2.x - Qm2.x)) * rh;
              const float da1 = ((F_D1A * (Qp1.y - Qm1.y)) - F_D1B * (Qp2.y - Qm2.y)) * rh;
              const float tmp0 = ((opbz * d2z0) + (dbz * d10)) + da0;
              const float tmp1 = ((opbz * d2z1) + (dbz * d11)) + da1;
              w0 = w0 + ((opbz * tmp0) + (az * Z.x));
              w1 = w1 + ((opbz * tmp1) + (az * Z.y));
              const float psi0 = (bz * d10) + Q0.x;
              const float psi1 = (bz * d11) + Q0.y;
              sts2(zzo + i * NX, (bz * tmp0) + (az * Z.x), (bz * tmp1) + (az * Z.y));
              sts2(apzn + i * NX, az * psi0, az * psi1);
            } else {
              w0 = w0 + d2z0;
              w1 = w1 + d2z1;
            }
            const float2 vv = lds2(V2o + i * NX);
            const float v20 = vv.x, v21 = vv.y;
            if (STORE) {  // written as the row is updated: holding them for after the barrier spilled registers
              const float2 cc = lds2(C2o + i * NX);
              *reinterpret_cast<float2*>(stg + i * NX) = make_float2(cc.x * w0, cc.y * w1);
            }
            n0 = ((v20 * w0) + (2.0f * u0)) - un[i][0];
            n1 = ((v21 * w1) + (2.0f * u1)) - un[i][1];
          }
          if (wsrc & (3u << (2 * i))) {
            const int cell = gbase + i * NX;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
              const int c = sSrcCell[k];
              const float q = sSrcQ[k] * f;
              const float a0 = n0 + q, a1 = n1 + q;
              n0 = (cell == c) ? a0 : n0;
              n1 = (cell + 1 == c) ? a1 : n1;
            }
          }
          un[i][0] = n0;
          un[i][1] = n1;
          sts2(uw + i * NX, n0, n1);
          if constexpr (C > 1) {
            if (rank > 0 && z < r0 + FD_PAD) st_peer_v2(U + (1 - par) * ustride + (z - pr_lo) * NX + x, rank - 1, n0, n1);
            if (rank < C - 1 && z >= r1 - FD_PAD)
              st_peer_v2(U + (1 - par) * ustride + (z - (r1 - FD_PAD)) * NX + x, rank + 1, n0, n1);
          }
        }
      }
    };
    rows(Un, APXn, ZXo, APZn, ZZo, st);
    if (TRACES) {
      // receivers at time t, recorded after this thread's update by the threads with the least
      // work per step: nothing writes buffer `par` before this step's barrier
      const float* Ucb = U + par * ustride;
      for (int r = ltid; r < nrec; r += NT) {
        if (sRecOk[r]) {
          float acc = 0.0f;
#pragma unroll
          for (int k = 0; k < 4; ++k) acc = acc + sRecW[4 * r + k] * Ucb[sRecCell[4 * r + k]];
          p.traces[(static_cast<size_t>(unit) * g.nt + t) * nrec + r] = acc;
        }
      }
    }
    {
      constexpr int H = G3_WAV_STEPS / 2;
      const int u = t - p.t0;
      if (u >= H && u % H == 0) wavelet_ring_fill(sW, g.wavelet, u + H, u + 2 * H, wsteps, ltid, H, wtime);
    }
    if constexpr (C > 1) {
      if (pusher) fence_cluster();
      __syncthreads();
      cluster_arrive_relaxed();
    }
    if constexpr (C > 1) cluster_wait_acquire();
    else __syncthreads();
  };

  int t = p.t0;
  for (; t + 1 < p.t1; t += 2) {
    step(t, uA, uB);
    step(t + 1, uB, uA);
  }
  if (t < p.t1) step(t, uA, uB);
}

// ------------------------------------------------------------------------------------------------
// Adjoint (splatAdjoint.wgsl:58-131)
// ------------------------------------------------------------------------------------------------
// PREF: fetch the next step's stored gradient terms between the barrier's arrive and wait (2 S more
// registers per thread) instead of loading each row's terms when the row is processed.
template <int NX, int PMLP, int C, int S, int NSEG, int NI, int LAY, bool PREF>
__global__ void __launch_bounds__(NSEG * 32 * (1 + NI), 1) adj3_kernel(const __grid_constant__ AdjArgs p) {
  using CL = Cols3<NX, PMLP>;
  constexpr int SW = CL::SW;
  constexpr int NT = NSEG * 32 * (1 + NI);
  extern __shared__ __align__(16) float sm[];
  const Grid& g = p.g;
  constexpr bool SQ = LAY == LAY_SQUARE;
  constexpr bool FULL = LAY == LAY_EVEN || (SQ && NX - 2 * FD_PAD == C * S * NSEG);  // S rows per segment
  const int nz = SQ ? NX : g.nz;                                                     // compile-time if square
  const int swa = g.swa, region = g.region_adj, nrec = p.st.nrec, nt = g.nt;
  const float rh = g.rh, dt2 = g.dt2;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int seg = warp / (1 + NI), wk = warp_role<NI>(warp);
  const int rank = (C > 1) ? static_cast<int>(cluster_rank()) : 0;
  const int unit = blockIdx.x / C;
  const int shot = unit % p.st.shots;
  const int model = unit / p.st.shots;
  const size_t cells = static_cast<size_t>(NX) * nz;
  const A3Layout L = a3_layout_rt(NX, PMLP, nz, swa, C, nrec);
  const int r0 = split_row(nz, C, rank), r1 = split_row(nz, C, rank + 1);
  const int zl0 = r0 - FD_PAD;
  const int bot_off = (C == 1) ? swa : 0;
  const int vstride = L.lr * NX;
  float* sAX = sm + L.off_prof;
  float* sBX = sAX + NX;
  float* sDBX = sBX + NX;
  float* sAZ = sDBX + NX;
  float* sBZ = sAZ + nz;
  float* sDBZ = sBZ + nz;

  for (int i = tid; i < L.total; i += NT) sm[i] = 0.0f;
  __syncthreads();
  for (int i = tid; i < 3 * (NX + nz); i += NT) sAX[i] = g.prof[i];

  const bool pml = (wk == 0);
  const int x = CL::x_of(wk, lane);
  const int zb = r0 + seg * S;
  const int nrows = CL::active(wk, lane) ? (FULL ? S : max(0, min(S, r1 - zb))) : 0;
  const bool pusher = (C > 1) && nrows > 0 && ((rank > 0 && zb < r0 + FD_PAD) || (rank < C - 1 && zb + nrows > r1 - FD_PAD));
  // The PML warp's stencil reaches two columns past its own on the interior side: the pair next to
  // the interior on the left strip reads x + 2, x + 3, the one on the right strip x - 2, x - 1.
  // There b = db = 0 and the adjoint psi, zeta are zero, so the strip terms are T = VS and U1 = 0
  // (T = 1 VS + 0 zeta differs from VS at most in the sign of a zero): those two lanes read VS
  // instead, so only the PML warp derives strip terms for the x strips.
  const bool edge_r = pml && (x + 2 == FD_PAD + CL::PCOLS);
  const bool edge_l = pml && (x == NX - FD_PAD - CL::PCOLS);
  const int vbase = (zb - zl0) * NX + x;
  const int abase = (zb - r0) * 2 * SW + CL::strip(x);
  const int zsh = (zb < nz / 2) ? 0 : (nz - swa - bot_off);
  const int zbase = (zb - zsh) * NX + x;
  const int gbase = zb * NX + x;
  float* LPX = sm + L.off_lpx + abase;
  float* LZX = sm + L.off_lzx + abase;
  float* LPZ = sm + L.off_lpz + zbase;
  float* LZZ = sm + L.off_lzz + zbase;
  float* TXs = sm + L.off_tx + abase;
  float* U1Xs = sm + L.off_u1x + abase;
  float* TZs = sm + L.off_tz + zbase;
  float* U1Zs = sm + L.off_u1z + zbase;
  float* V2o = sm + L.off_v2 + (zb - r0) * NX + x;
  float* GAo = sm + L.off_ga + (zb - r0) * NX + x;

  // per-column constants live in shared memory: (1 + b) in sOPB, a, b, db in the profiles
  float* sOPB = sm + L.off_opb;
  for (int i = tid; i < NX; i += NT) sOPB[i] = 1.0f + g.prof[NX + i];
  // Source corners: cell and the step-invariant factor ((-2 v) dt^2) w of the shader's
  // ((((-2 v) dt^2) w) f) (left to right, so the product with f rounds identically).
  int* sSrcCell = reinterpret_cast<int*>(sm + L.off_src);
  float* sSrcF = sm + L.off_src + 4;
  // wavelet ring, counted from the launch's first (latest) step backwards
  float* sW = sm + L.off_src + 8;
  const int wsteps = p.t_hi - p.t_lo;
  auto wtime = [&](int u) { return p.t_hi - 1 - u; };
  wavelet_ring_fill(sW, g.wavelet, 0, G3_WAV_STEPS, wsteps, tid, NT, wtime);
  if (tid < 4) {
    const int cell = p.st.src_cell[4 * shot + tid];
    sSrcCell[tid] = cell;
    sSrcF[tid] = (((-2.0f) * p.vel[static_cast<size_t>(model) * cells + cell]) * dt2) * p.st.src_w[4 * shot + tid];
  }
  // The receiver CSR of this CTA's rows in shared memory: up to G3_REC_ROWS rows with entries get
  // a slot with their cells' entry offsets (relative to the CTA's first entry e0); rows beyond that
  // read the global CSR. Per step, P[t & 1][e] = w_e * residual(t, receiver_e) (the product of the
  // shader's injection term) is formed one step ahead, from a residual loaded two steps ahead, by
  // one thread per entry, so the injection adds shared-memory values in CSR order.
  int* sRRow = reinterpret_cast<int*>(sm + L.off_rrow);
  int* sROff = reinterpret_cast<int*>(sm + L.off_roff);
  float* sEW = sm + L.off_ew;
  int* sER = reinterpret_cast<int*>(sm + L.off_er);
  float* sP = sm + L.off_res;
  const int crows = r1 - r0;
  const int E0 = p.st.csr[r0 * NX];
  const int ecnt = p.st.csr[r1 * NX] - E0;
  const bool stage = ecnt <= L.pcap && ecnt <= NT;
  const int ltid = light_tid<NSEG, NI, C>(tid, rank);
  const float* resu = p.residual + static_cast<size_t>(unit) * nt * nrec;
  float rnext = 0.0f;
  if (stage && ltid < ecnt) {
    const int rec = p.st.ent_rec[E0 + ltid];
    const float w = p.st.ent_w[E0 + ltid];
    sEW[ltid] = w;
    sER[ltid] = rec;
    sP[((p.t_hi - 1) & 1) * L.pcap + ltid] = w * resu[static_cast<size_t>(p.t_hi - 1) * nrec + rec];
    if (p.t_hi - 2 >= p.t_lo) rnext = resu[static_cast<size_t>(p.t_hi - 2) * nrec + rec];
  }
  if (warp == 0) {
    int used = 0;
    for (int c0 = 0; c0 < crows; c0 += 32) {
      const int r = c0 + lane;
      const bool has = r < crows && p.st.csr[(r0 + r) * NX] < p.st.csr[(r0 + r + 1) * NX];
      const unsigned b = __ballot_sync(0xffffffffu, has);
      const int slot = used + __popc(b & ((1u << lane) - 1u));
      if (r < crows) sRRow[r] = (has && stage && slot < G3_REC_ROWS) ? slot : -1;
      used += __popc(b);
    }
  }

  float lA[S][2], lB[S][2];
  unsigned srcmask = 0, recmask = 0;
  const int* sc = p.st.src_cell + 4 * shot;
  const float* vel = p.vel + static_cast<size_t>(model) * cells + gbase;
  const size_t asf = adjstate_floats(NX, nz, swa);
  float* stt = p.state + static_cast<size_t>(unit) * asf;
  float* sLc = stt;
  float* sLp = stt + cells;
  float* sPX = stt + 2 * cells;
  float* sZX = sPX + static_cast<size_t>(nz) * 2 * swa;
  float* sPZ = sZX + static_cast<size_t>(nz) * 2 * swa;
  float* sZZ = sPZ + static_cast<size_t>(2) * swa * NX;
  float* gacc = p.gacc + static_cast<size_t>(unit) * cells + gbase;
  __syncthreads();
  for (int i = tid; i < crows * (NX + 1); i += NT) {
    const int r = i / (NX + 1), xx = i - r * (NX + 1), slot = sRRow[r];
    if (slot >= 0) sROff[slot * (NX + 4) + xx] = p.st.csr[(r0 + r) * NX + xx] - E0;
  }
  unsigned recslots = 0;  // per own row: 3 bits, the row's slot or 7 (global CSR)
#pragma unroll
  for (int i = 0; i < S; ++i) {
    if (i < nrows) {
      const int slot = sRRow[zb - r0 + i];
      recslots |= static_cast<unsigned>(slot >= 0 ? slot : 7) << (3 * i);
    }
#pragma unroll
    for (int j = 0; j < 2; ++j) lA[i][j] = lB[i][j] = 0.f;
    if (i < nrows) {
      const int z = zb + i;
      {
        const float2 v = __ldg(reinterpret_cast<const float2*>(vel + i * NX));
        sts2(V2o + i * NX, v.x * v.x * dt2, v.y * v.y * dt2);
        sts2(GAo + i * NX, 0.0f, 0.0f);
      }
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        const int cell = gbase + i * NX + j;
        if (cell == sc[0] || cell == sc[1] || cell == sc[2] || cell == sc[3]) srcmask |= 1u << (2 * i + j);
        if (p.st.csr[cell] < p.st.csr[cell + 1]) recmask |= 1u << (2 * i + j);
        if (!p.first) {
          lA[i][j] = sLc[cell];
          lB[i][j] = sLp[cell];
          GAo[i * NX + j] = gacc[i * NX + j];
          const int xx = x + j;
          if (xx < swa || xx >= NX - swa) {
            const int xc = strip_col(xx, NX, swa);
            LPX[i * 2 * SW + j] = sPX[z * 2 * swa + xc];
            LZX[i * 2 * SW + j] = sZX[z * 2 * swa + xc];
          }
          if (z < swa || z >= nz - swa) {
            const int zc = strip_col(z, nz, swa);
            LPZ[i * NX + j] = sPZ[zc * NX + xx];
            LZZ[i * NX + j] = sZZ[zc * NX + xx];
          }
        }
      }
    }
  }
  // rows where any lane of the warp injects a residual or the source: warp-uniform branches
  const unsigned wrec = __reduce_or_sync(0xffffffffu, recmask);
  const unsigned wsrc = __reduce_or_sync(0xffffffffu, srcmask);
  if constexpr (C > 1) cluster_barrier();
  else __syncthreads();

  const int pr_lo = (rank > 0) ? split_row(nz, C, rank - 1) - FD_PAD : 0;

  // VS = v^2 dt^2 lambda of row i into buffer b (and into the peer CTA's halo rows).
  auto put_vs = [&](int b, int i, float l0, float l1) {
    float* VSb = sm + L.off_vs + b * vstride;
    const int z = zb + i;
    const float2 v2 = lds2(V2o + i * NX);
    const float vs0 = v2.x * l0;
    const float vs1 = v2.y * l1;
    sts2(VSb + vbase + i * NX, vs0, vs1);
    if constexpr (C > 1) {
      if (rank > 0 && z < r0 + FD_PAD) st_peer_v2(VSb + (z - pr_lo) * NX + x, rank - 1, vs0, vs1);
      if (rank < C - 1 && z >= r1 - FD_PAD) st_peer_v2(VSb + (z - (r1 - FD_PAD)) * NX + x, rank + 1, vs0, vs1);
    }
  };
  // Strip terms T = (1 + b) VS + b zeta and U1 = db T + b psi of this thread's cells from VS in
  // buffer b, into their single buffers.
  // The strip arrays are written only through the restrict-qualified pointers of `put`, so the
  // compiler may issue every row's loads ahead of the earlier rows' stores; the per-column
  // profile values are loaded once.
  auto derive_strips = [&](int b) {
    const float* VSb = sm + L.off_vs + b * vstride;
    auto put = [&](float* __restrict__ TXb, float* __restrict__ U1Xb, float* __restrict__ TZb,
                   float* __restrict__ U1Zb) {
      const bool xs = pml;
      const float2 o = xs ? lds2(sOPB + x) : make_float2(0.f, 0.f);
      const float2 bx = xs ? lds2(sBX + x) : make_float2(0.f, 0.f);
      const float2 db = xs ? lds2(sDBX + x) : make_float2(0.f, 0.f);
#pragma unroll
      for (int i = 0; i < S; ++i) {
        if (i < nrows) {
          const int z = zb + i;
          const bool zstrip = z < swa || z >= nz - swa;
          if (!(xs || zstrip)) continue;
          const float2 vs = lds2(VSb + vbase + i * NX);
          const float vs0 = vs.x, vs1 = vs.y;
          if (xs) {
            const float2 Z = lds2(LZX + i * 2 * SW);
            const float2 P = lds2(LPX + i * 2 * SW);
            const float T0 = (o.x * vs0) + (bx.x * Z.x);
            const float T1 = (o.y * vs1) + (bx.y * Z.y);
            sts2(TXb + i * 2 * SW, T0, T1);
            sts2(U1Xb + i * 2 * SW, (db.x * T0) + (bx.x * P.x), (db.y * T1) + (bx.y * P.y));
          }
          if (zstrip) {
            const float bz = sBZ[z], dbz = sDBZ[z];
            const float opbz = 1.0f + bz;
            const float2 Z = lds2(LZZ + i * NX);
            const float2 P = lds2(LPZ + i * NX);
            const float T0 = (opbz * vs0) + (bz * Z.x);
            const float T1 = (opbz * vs1) + (bz * Z.y);
            sts2(TZb + i * NX, T0, T1);
            sts2(U1Zb + i * NX, (dbz * T0) + (bz * P.x), (dbz * T1) + (bz * P.y));
          }
        }
      }
    };
    put(TXs, U1Xs, TZs, U1Zs);
  };


#pragma unroll
  for (int i = 0; i < S; ++i)
    if (i < nrows) put_vs(0, i, lA[i][0], lA[i][1]);
  derive_strips(0);  // reads only this thread's own VS cells
  step_barrier<C>();

  const int segn = p.t_hi - p.t_lo;
  // stored gradient terms of the next step to process, loaded one step ahead (PREF)
  float2 stv[PREF ? S : 1];
  if (PREF) {
    const float* st0 = p.stored + (static_cast<size_t>(unit) * segn + (p.t_hi - 1 - p.t_lo)) * cells + gbase;
#pragma unroll
    for (int i = 0; i < S; ++i)
      stv[i] = (i < nrows) ? __ldcs(reinterpret_cast<const float2*>(st0 + i * NX)) : make_float2(0.f, 0.f);
  }
  // One reverse step at time t: `lc` holds lambda at t, `lp` holds the previous one and receives
  // the next.
  auto step = [&](int t, float (&lc)[S][2], float (&lp)[S][2]) {
    const int par = (p.t_hi - 1 - t) & 1;
    const float* VSd = sm + L.off_vs + par * vstride + vbase;
    const float* TXd = TXs;
    const float* U1Xd = U1Xs;
    const float* TZd = TZs;
    const float* U1Zd = U1Zs;
    const float f = sW[(p.t_hi - 1 - t) % G3_WAV_STEPS];
    const float* res_t = p.residual + (static_cast<size_t>(unit) * nt + t) * nrec;
    const float* st_t = p.stored + (static_cast<size_t>(unit) * segn + (t - p.t_lo)) * cells + gbase;
#pragma unroll
    for (int i = 0; i < S; ++i) {
      if (i < nrows) {
        const int z = zb + i;
        const float2 Vb = lds2(VSd + i * NX);  // own v^2 dt^2 lambda
        float w0, w1;
        if (pml) {
          const float2 Ta = lds2(edge_l ? VSd + i * NX - 2 : TXd + i * 2 * SW - 2), Tb = lds2(TXd + i * 2 * SW),
                       Tc = lds2(edge_r ? VSd + i * NX + 2 : TXd + i * 2 * SW + 2);
          float2 Ua = lds2(U1Xd + i * 2 * SW - 2), Uc = lds2(U1Xd + i * 2 * SW + 2);
          const float2 Ub = lds2(U1Xd + i * 2 * SW);
          if (edge_l) Ua = make_float2(0.f, 0.f);
          if (edge_r) Uc = make_float2(0.f, 0.f);
          const float2 Oa = lds2(sOPB + x - 2), Ob = lds2(sOPB + x), Oc = lds2(sOPB + x + 2);
          const float q0 = Oa.x * Ta.x, q1 = Oa.y * Ta.y, q2 = Ob.x * Tb.x, q3 = Ob.y * Tb.y, q4 = Oc.x * Tc.x,
                      q5 = Oc.y * Tc.y;
          // cell x: neighbours x-2..x+2 = (Ta.x, Ta.y, Tb.x, Tb.y, Tc.x)
          const float du0 = ((F_D1A * (Ub.y - Ua.y)) + (A_D1B * (Uc.x - Ua.x))) * rh;
          const float dd0 = ((((F_D2A * q2) + (F_D2B * (q3 + q1))) + (A_D2C * (q4 + q0))) * rh) * rh;
          const float dt0 = ((F_D1A * (Tb.y - Ta.y)) + (A_D1B * (Tc.x - Ta.x))) * rh;
          // cell x+1: neighbours x-1..x+3 = (Ta.y, Tb.x, Tb.y, Tc.x, Tc.y)
          const float du1 = ((F_D1A * (Uc.x - Ub.x)) + (A_D1B * (Uc.y - Ua.y))) * rh;
          const float dd1 = ((((F_D2A * q3) + (F_D2B * (q4 + q2))) + (A_D2C * (q5 + q1))) * rh) * rh;
          const float dt1 = ((F_D1A * (Tc.x - Tb.x)) + (A_D1B * (Tc.y - Ta.y))) * rh;
          w0 = (-du0) + dd0;
          w1 = (-du1) + dd1;
          const float2 P = lds2(LPX + i * 2 * SW);
          const float2 Z = lds2(LZX + i * 2 * SW);
          const float2 a = lds2(sAX + x);
          sts2(LPX + i * 2 * SW, ((-a.x) * dt0) + (a.x * P.x), ((-a.y) * dt1) + (a.y * P.y));
          sts2(LZX + i * 2 * SW, (a.x * Vb.x) + (a.x * Z.x), (a.y * Vb.y) + (a.y * Z.y));
        } else {
          const float2 Va = lds2(VSd + i * NX - 2), Vc = lds2(VSd + i * NX + 2);
          w0 = ((((F_D2A * Vb.x) + (F_D2B * (Vb.y + Va.y))) + (A_D2C * (Vc.x + Va.x))) * rh) * rh;
          w1 = ((((F_D2A * Vb.y) + (F_D2B * (Vc.x + Vb.x))) + (A_D2C * (Vc.y + Va.y))) * rh) * rh;
        }
        if (z < region || z >= nz - region) {
          const float2 Tm2 = lds2(TZd + (i - 2) * NX), Tm1 = lds2(TZd + (i - 1) * NX), T0 = lds2(TZd + i * NX),
                       Tp1 = lds2(TZd + (i + 1) * NX), Tp2 = lds2(TZd + (i + 2) * NX);
          const float2 Um2 = lds2(U1Zd + (i - 2) * NX), Um1 = lds2(U1Zd + (i - 1) * NX),
                       Up1 = lds2(U1Zd + (i + 1) * NX), Up2 = lds2(U1Zd + (i + 2) * NX);
          const float om2 = 1.0f + sBZ[z - 2], om1 = 1.0f + sBZ[z - 1], o0 = 1.0f + sBZ[z], op1 = 1.0f + sBZ[z + 1],
                      op2 = 1.0f + sBZ[z + 2];
          const float du0 = ((F_D1A * (Up1.x - Um1.x)) + (A_D1B * (Up2.x - Um2.x))) * rh;
          const float du1 = ((F_D1A * (Up1.y - Um1.y)) + (A_D1B * (Up2.y - Um2.y))) * rh;
          const float dd0 = ((((F_D2A * (o0 * T0.x)) + (F_D2B * ((op1 * Tp1.x) + (om1 * Tm1.x)))) +
                              (A_D2C * ((op2 * Tp2.x) + (om2 * Tm2.x)))) * rh) * rh;
          const float dd1 = ((((F_D2A * (o0 * T0.y)) + (F_D2B * ((op1 * Tp1.y) + (om1 * Tm1.y)))) +
                              (A_D2C * ((op2 * Tp2.y) + (om2 * Tm2.y)))) * rh) * rh;
          const float dt0 = ((F_D1A * (Tp1.x - Tm1.x)) + (A_D1B * (Tp2.x - Tm2.x))) * rh;
          const float dt1 = ((F_D1A * (Tp1.y - Tm1.y)) + (A_D1B * (Tp2.y - Tm2.y))) * rh;
          w0 = w0 + ((-du0) + dd0);
          w1 = w1 + ((-du1) + dd1);
          const float az = sAZ[z];
          const float2 P = lds2(LPZ + i * NX);
          const float2 Z = lds2(LZZ + i * NX);
          sts2(LPZ + i * NX, ((-az) * dt0) + (az * P.x), ((-az) * dt1) + (az * P.y));
          sts2(LZZ + i * NX, (az * Vb.x) + (az * Z.x), (az * Vb.y) + (az * Z.y));
        } else {
          const float2 Vm2 = lds2(VSd + (i - 2) * NX), Vm1 = lds2(VSd + (i - 1) * NX), Vp1 = lds2(VSd + (i + 1) * NX),
                       Vp2 = lds2(VSd + (i + 2) * NX);
          w0 = w0 + ((((F_D2A * Vb.x) + (F_D2B * (Vp1.x + Vm1.x))) + (A_D2C * (Vp2.x + Vm2.x))) * rh) * rh;
          w1 = w1 + ((((F_D2A * Vb.y) + (F_D2B * (Vp1.y + Vm1.y))) + (A_D2C * (Vp2.y + Vm2.y))) * rh) * rh;
        }
        float n0 = (w0 + (2.0f * lc[i][0])) - lp[i][0];
        float n1 = (w1 + (2.0f * lc[i][1])) - lp[i][1];
        const float2 sv = PREF ? stv[PREF ? i : 0] : __ldcs(reinterpret_cast<const float2*>(st_t + i * NX));
        // the shader starts the per-step gradient at +0; starting from the product itself differs
        // only in the sign of an exact zero
        float g0 = (lc[i][0] * sv.x) * 1.0f;
        float g1 = (lc[i][1] * sv.y) * 1.0f;
        if (wrec & (3u << (2 * i))) {  // cells without entries have empty ranges
          const unsigned slot = (recslots >> (3 * i)) & 7u;
          if (slot < G3_REC_ROWS) {
            const int* o = sROff + slot * (NX + 4) + x;
            const float* P = sP + (t & 1) * L.pcap;
            const int e0 = o[0], e1 = o[1], e2 = o[2];
            for (int e = e0; e < e1; ++e) n0 = n0 + P[e];
            for (int e = e1; e < e2; ++e) n1 = n1 + P[e];
          } else {
            const int cell = gbase + i * NX;
            const int e1 = p.st.csr[cell + 1], e2 = p.st.csr[cell + 2];
            for (int e = p.st.csr[cell]; e < e1; ++e) n0 = n0 + (p.st.ent_w[e] * res_t[p.st.ent_rec[e]]);
            for (int e = e1; e < e2; ++e) n1 = n1 + (p.st.ent_w[e] * res_t[p.st.ent_rec[e]]);
          }
        }
        if (t > p.t_lo) put_vs(1 - par, i, n0, n1);  // VS of the new lambda for step t - 1
        if (wsrc & (3u << (2 * i))) {
          const int cell = gbase + i * NX;
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            const int c = sSrcCell[k];
            const float q = sSrcF[k] * f;
            const float a0 = g0 + lc[i][0] * q, a1 = g1 + lc[i][1] * q;
            g0 = (cell == c) ? a0 : g0;
            g1 = (cell + 1 == c) ? a1 : g1;
          }
        }
        {
          const float2 ga = lds2(GAo + i * NX);
          sts2(GAo + i * NX, ga.x + g0, ga.y + g1);
        }
        lp[i][0] = n0;
        lp[i][1] = n1;
      }
    }
    if (t > p.t_lo) {
      __syncthreads();  // every read of the single-buffered strip terms of step t is done
      derive_strips(1 - par);
      if (stage && ltid < ecnt) sP[((t - 1) & 1) * L.pcap + ltid] = sEW[ltid] * rnext;
      constexpr int H = G3_WAV_STEPS / 2;
      const int u = p.t_hi - 1 - t;
      if (u >= H && u % H == 0) wavelet_ring_fill(sW, g.wavelet, u + H, u + 2 * H, wsteps, ltid, H, wtime);
    }
    if constexpr (C > 1) {
      if (pusher) fence_cluster();
      __syncthreads();
      cluster_arrive_relaxed();
    }
    if (stage && ltid < ecnt && t - 2 >= p.t_lo) rnext = resu[static_cast<size_t>(t - 2) * nrec + sER[ltid]];
    if (PREF && t > p.t_lo) {  // next step's stored terms, fetched while the peers catch up
      const float* stn = p.stored + (static_cast<size_t>(unit) * segn + (t - 1 - p.t_lo)) * cells + gbase;
#pragma unroll
      for (int i = 0; i < S; ++i)
        if (i < nrows) stv[PREF ? i : 0] = __ldcs(reinterpret_cast<const float2*>(stn + i * NX));
    }
    if constexpr (C > 1) cluster_wait_acquire();
    else __syncthreads();
  };

  int t = p.t_hi - 1;
  int flips = 0;
  for (; t - 1 >= p.t_lo; t -= 2) {
    step(t, lA, lB);
    step(t - 1, lB, lA);
  }
  if (t >= p.t_lo) {
    step(t, lA, lB);
    flips = 1;
  }
  // after an odd number of steps lB holds the current lambda and lA the previous one
#pragma unroll
  for (int i = 0; i < S; ++i) {
    if (i < nrows) {
      const int z = zb + i;
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        const int cell = gbase + i * NX + j;
        sLc[cell] = flips ? lB[i][j] : lA[i][j];
        sLp[cell] = flips ? lA[i][j] : lB[i][j];
        gacc[i * NX + j] = GAo[i * NX + j];
        const int xx = x + j;
        if (xx < swa || xx >= NX - swa) {
          const int xc = strip_col(xx, NX, swa);
          sPX[z * 2 * swa + xc] = LPX[i * 2 * SW + j];
          sZX[z * 2 * swa + xc] = LZX[i * 2 * SW + j];
        }
        if (z < swa || z >= nz - swa) {
          const int zc = strip_col(z, nz, swa);
          sPZ[zc * NX + xx] = LPZ[i * NX + j];
          sZZ[zc * NX + xx] = LZZ[i * NX + j];
        }
      }
    }
  }
}

// Every segment of every CTA has exactly S rows when the CTAs' rows split evenly into NSEG segments.
template <int C, int S, int NSEG>
inline bool g3_even(int nz) {
  for (int r = 0; r < C; ++r)
    if (split_row(nz, C, r + 1) - split_row(nz, C, r) != S * NSEG) return false;
  return true;
}

// Layout a launch takes: with one interior warp per segment a square grid takes the compile-time
// layout; with several, the compile-time layout makes the forward spill registers and run slower
// (measured), so evenly split grids take LAY_EVEN.
template <int NX, int C, int S, int NSEG, int NI>
inline int g3_layout(int nz) {
  if (NI == 1) return nz == NX ? LAY_SQUARE : LAY_RUNTIME;
  return g3_even<C, S, NSEG>(nz) ? LAY_EVEN : LAY_RUNTIME;
}

template <int NX, int PMLP, int C, int S, int NSEG, int NI, int LAY, bool FA>
cudaError_t fwd3_launch(bool traces, bool store, const FwdArgs& a, size_t smem, cudaStream_t s) {
  constexpr int NT = NSEG * 32 * (1 + NI);
  if (traces && store)
    return launch_cluster(fwd3_kernel<NX, PMLP, C, S, NSEG, NI, LAY, true, true, FA>, C, NT, a.units, smem, s, a);
  if (traces)
    return launch_cluster(fwd3_kernel<NX, PMLP, C, S, NSEG, NI, LAY, true, false, FA>, C, NT, a.units, smem, s, a);
  if (store)
    return launch_cluster(fwd3_kernel<NX, PMLP, C, S, NSEG, NI, LAY, false, true, FA>, C, NT, a.units, smem, s, a);
  return cudaErrorInvalidValue;
}

// FA: the fast-arithmetic kernels (instantiated in their own translation units).
template <int NX, int PMLP, int C, int S, int NSEG, int NI, bool FA = false>
cudaError_t fwd3_dispatch_impl(bool traces, bool store, const FwdArgs& a, size_t smem, cudaStream_t s) {
  constexpr int LAY_FAST = NI == 1 ? LAY_SQUARE : LAY_EVEN;
  if (g3_layout<NX, C, S, NSEG, NI>(a.g.nz) == LAY_FAST)
    return fwd3_launch<NX, PMLP, C, S, NSEG, NI, LAY_FAST, FA>(traces, store, a, smem, s);
  return fwd3_launch<NX, PMLP, C, S, NSEG, NI, LAY_RUNTIME, FA>(traces, store, a, smem, s);
}

template <int NX, int PMLP, int C, int S, int NSEG, int NI, bool PREF>
cudaError_t adj3_dispatch_impl(const AdjArgs& a, size_t smem, cudaStream_t s) {
  constexpr int NT = NSEG * 32 * (1 + NI);
  constexpr int LAY_FAST = NI == 1 ? LAY_SQUARE : LAY_EVEN;
  if (g3_layout<NX, C, S, NSEG, NI>(a.g.nz) == LAY_FAST)
    return launch_cluster(adj3_kernel<NX, PMLP, C, S, NSEG, NI, LAY_FAST, PREF>, C, NT, a.units, smem, s, a);
  return launch_cluster(adj3_kernel<NX, PMLP, C, S, NSEG, NI, LAY_RUNTIME, PREF>, C, NT, a.units, smem, s, a);
}

// Adjoint launch: the prefetching variant when `pref` is set in the shape.
template <int NX, int PMLP, int C, int S, int NSEG, int NI>
cudaError_t adj3_dispatch_impl_pref(const AdjArgs& a, size_t smem, cudaStream_t s) {
  if (a.prefetch) return adj3_dispatch_impl<NX, PMLP, C, S, NSEG, NI, true>(a, smem, s);
  return adj3_dispatch_impl<NX, PMLP, C, S, NSEG, NI, false>(a, smem, s);
}

}  // namespace wg
