// Second-generation resident kernels: column-pair x segment thread mapping.
//
// Each thread owns two adjacent columns (x, x+1) over a segment of S consecutive rows and keeps
// its cells' wavefield values in registers across time steps, so the z-direction stencil reads its
// own registers and the x-direction stencil needs two 8-byte shared-memory loads per row. Warps are
// class-pure: per segment, one warp owns the 16 leftmost and 16 rightmost column pairs (the C-PML
// columns, widened to 32 per side) and runs the PML formula; the other warps own interior pairs
// and run the interior formula. Applying the PML formula where a = b = db = 0 yields the interior
// result exactly (up to the sign of zero), so widening the PML columns keeps bit-exact parity.
//
// The leapfrog update writes u_next over u_prev in place; the time loop alternates the roles of the
// two register arrays, so no values are moved between steps.
#pragma once
#include <cuda_runtime.h>

#include "wave_device.cuh"
#include "wave_kernels2_layout.h"
#include "wave_kernels.cuh"
#include "wave_launch.h"

namespace wg {

__device__ __forceinline__ void st_peer2(const float* local_ptr, unsigned peer, float a, float b) {
  unsigned la = static_cast<unsigned>(__cvta_generic_to_shared(local_ptr));
  unsigned ra;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(ra) : "r"(la), "r"(peer));
  asm volatile("st.shared::cluster.v2.f32 [%0], {%1, %2};" ::"r"(ra), "f"(a), "f"(b) : "memory");
}

// Column of the first cell of the pair owned by lane `lane` of warp kind `wk` (0 = PML warp).
__device__ __forceinline__ int pair_x(int wk, int lane, int nx) {
  if (wk == 0) return lane < kPmlPairs ? FD_PAD + 2 * lane : (nx - FD_PAD - kPmlCols) + 2 * (lane - kPmlPairs);
  return FD_PAD + kPmlCols + 2 * ((wk - 1) * 32 + lane);
}

__device__ __forceinline__ int swx_col(int x, int nx) { return x < kSwx ? x : x - (nx - 2 * kSwx); }


template <int C, int S, int NSEG, int NI, bool TRACES, bool STORE>
__global__ void __launch_bounds__(NSEG * 32 * (1 + NI), 1) fwd2_kernel(const __grid_constant__ FwdArgs p) {
  constexpr int NT = NSEG * 32 * (1 + NI);
  extern __shared__ __align__(16) float sm[];
  const Grid& g = p.g;
  const int nx = g.nx, nz = g.nz, sw = g.sw;
  const int region = g.region, nrec = p.st.nrec;
  const float rh = g.rh, dt2 = g.dt2, d2a = g.d2a, d2b = g.d2b;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int seg = warp / (1 + NI), wk = warp % (1 + NI);
  const int rank = (C > 1) ? static_cast<int>(cluster_rank()) : 0;
  const int unit = blockIdx.x / C;
  const int shot = unit % p.st.shots;
  const int model = unit / p.st.shots;
  const size_t cells = static_cast<size_t>(nx) * nz;
  const Fwd2Layout L = fwd2_layout(nx, nz, sw, C, nrec);
  const int r0 = split_row(nz, C, rank), r1 = split_row(nz, C, rank + 1);
  const int zl0 = r0 - FD_PAD;
  const int bot_off = (C == 1) ? sw : 0;
  const int ustride = L.lr * nx, xstride = L.maxrows * 2 * kSwx, zstride = L.zs * nx;
  float* U = sm + L.off_u;
  float* APX = sm + L.off_apx;
  float* APZ = sm + L.off_apz;
  float* ZZ = sm + L.off_zz;
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

  const int x = pair_x(wk, lane, nx);
  const bool active = (wk == 0) || (x < nx - FD_PAD - kPmlCols);
  const int zb = r0 + seg * S;                 // first row of the segment
  const int nrows = active ? max(0, min(S, r1 - zb)) : 0;
  const bool pml = (wk == 0);
  const int xs = swx_col(x, nx);               // packed a*psi_x column (PML warp)

  // per-column constants of the pair
  float ax0 = 0.f, ax1 = 0.f, bx0 = 0.f, bx1 = 0.f, dbx0 = 0.f, dbx1 = 0.f;
  if (pml) {
    ax0 = g.prof[x];
    ax1 = g.prof[x + 1];
    bx0 = g.prof[nx + x];
    bx1 = g.prof[nx + x + 1];
    dbx0 = g.prof[2 * nx + x];
    dbx1 = g.prof[2 * nx + x + 1];
  }
  const float opbx0 = 1.0f + bx0, opbx1 = 1.0f + bx1;

  float uA[S][2], uB[S][2], v2[S][2], zx[S][2];
  float c2[STORE ? S : 1][2];
  unsigned srcmask = 0;
  const int* sc = p.st.src_cell + 4 * shot;
  const float* vel = p.vel + static_cast<size_t>(model) * cells;
#pragma unroll
  for (int i = 0; i < S; ++i) {
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      uA[i][j] = 0.f;
      uB[i][j] = 0.f;
      v2[i][j] = 0.f;
      zx[i][j] = 0.f;
      if (STORE) c2[i][j] = 0.f;
    }
    if (i < nrows) {
      const int z = zb + i;
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        const float v = vel[z * nx + x + j];
        v2[i][j] = v * v * dt2;
        if (STORE) c2[i][j] = (2.0f * v) * dt2;
        const int cell = z * nx + x + j;
        if (cell == sc[0] || cell == sc[1] || cell == sc[2] || cell == sc[3]) srcmask |= 1u << (2 * i + j);
      }
    }
  }

  const size_t ckf = ckpt_floats(nx, nz, sw);
  if (p.ck_in) {
    const float* ck = p.ck_in + (static_cast<size_t>(unit) * p.ck_slots + p.ck_in_slot) * ckf;
    const float* cU = ck;
    const float* cP = ck + cells;
    const float* cAX = ck + 2 * cells;
    const float* cAZ = cAX + static_cast<size_t>(nz) * 2 * sw;
    const float* cZX = cAZ + static_cast<size_t>(2) * sw * nx;
    const float* cZZ = cZX + static_cast<size_t>(nz) * 2 * sw;
    // U_cur into shared memory with the halo rows (frame cells stay zero)
    const int W = nx - 2 * FD_PAD;
    const int ra = max(r0 - FD_PAD, FD_PAD), rb = min(r1 + FD_PAD, nz - FD_PAD);
    for (int i = tid; i < (rb - ra) * W; i += NT) {
      const int z = ra + i / W, xx = FD_PAD + i % W;
      U[(z - zl0) * nx + xx] = cU[z * nx + xx];
    }
#pragma unroll
    for (int i = 0; i < S; ++i) {
      if (i < nrows) {
        const int z = zb + i;
#pragma unroll
        for (int j = 0; j < 2; ++j) {
          const int xx = x + j;
          uA[i][j] = cU[z * nx + xx];
          uB[i][j] = cP[z * nx + xx];
          if (xx < sw || xx >= nx - sw) {
            const int xc = strip_col(xx, nx, sw);
            APX[(z - r0) * 2 * kSwx + swx_col(xx, nx)] = cAX[z * 2 * sw + xc];
            zx[i][j] = cZX[z * 2 * sw + xc];
          }
          if (z < sw || z >= nz - sw) {
            const int zc = strip_col(z, nz, sw);
            const int zss = (z < sw) ? z : z - (nz - sw) + bot_off;
            APZ[zss * nx + xx] = cAZ[zc * nx + xx];
            ZZ[zss * nx + xx] = cZZ[zc * nx + xx];
          }
        }
      }
    }
  }
  if constexpr (C > 1) cluster_barrier();
  else __syncthreads();

  const int pr_lo = (rank > 0) ? split_row(nz, C, rank - 1) - FD_PAD : 0;

  // One time step. `uc` holds u_t of this thread's cells, `un` holds u_{t-1} and receives u_{t+1}.
  auto step = [&](int t, float (&uc)[S][2], float (&un)[S][2]) {
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
    if (p.ck_out && t > p.t0 && (t % p.ck_every) == 0) {
      float* ck = p.ck_out + (static_cast<size_t>(unit) * p.ck_slots + (t / p.ck_every - 1)) * ckf;
      float* cAX = ck + 2 * cells;
      float* cAZ = cAX + static_cast<size_t>(nz) * 2 * sw;
      float* cZX = cAZ + static_cast<size_t>(2) * sw * nx;
      float* cZZ = cZX + static_cast<size_t>(nz) * 2 * sw;
#pragma unroll
      for (int i = 0; i < S; ++i) {
        if (i < nrows) {
          const int z = zb + i;
#pragma unroll
          for (int j = 0; j < 2; ++j) {
            const int xx = x + j;
            ck[z * nx + xx] = uc[i][j];
            ck[cells + z * nx + xx] = un[i][j];
            if (xx < sw || xx >= nx - sw) {
              const int xc = strip_col(xx, nx, sw);
              cAX[z * 2 * sw + xc] = APXc[(z - r0) * 2 * kSwx + swx_col(xx, nx)];
              cZX[z * 2 * sw + xc] = zx[i][j];
            }
            if (z < sw || z >= nz - sw) {
              const int zc = strip_col(z, nz, sw);
              const int zss = (z < sw) ? z : z - (nz - sw) + bot_off;
              cAZ[zc * nx + xx] = APZc[zss * nx + xx];
              cZZ[zc * nx + xx] = ZZ[zss * nx + xx];
            }
          }
        }
      }
    }

    const float f = __ldg(&g.wavelet[t]);
    float* st_t = STORE ? p.stored + (static_cast<size_t>(unit) * (p.t1 - p.t0) + (t - p.t0)) * cells : nullptr;
#pragma unroll
    for (int i = 0; i < S; ++i) {
      if (i < nrows) {
        const int z = zb + i;
        const int rowl = (z - zl0) * nx;
        // x neighbours: (x-2, x-1) and (x+2, x+3)
        const float2 A = *reinterpret_cast<const float2*>(&Uc[rowl + x - 2]);
        const float2 B = *reinterpret_cast<const float2*>(&Uc[rowl + x + 2]);
        // z neighbours from registers inside the segment, else shared memory
        float zm2[2], zm1[2], zp1[2], zp2[2];
        if (i >= 2) {
          zm2[0] = uc[i - 2][0];
          zm2[1] = uc[i - 2][1];
        } else {
          const float2 q = *reinterpret_cast<const float2*>(&Uc[rowl - 2 * nx + x]);
          zm2[0] = q.x;
          zm2[1] = q.y;
        }
        if (i >= 1) {
          zm1[0] = uc[i - 1][0];
          zm1[1] = uc[i - 1][1];
        } else {
          const float2 q = *reinterpret_cast<const float2*>(&Uc[rowl - nx + x]);
          zm1[0] = q.x;
          zm1[1] = q.y;
        }
        if (i + 1 < nrows) {
          zp1[0] = uc[i + 1 < S ? i + 1 : i][0];
          zp1[1] = uc[i + 1 < S ? i + 1 : i][1];
        } else {
          const float2 q = *reinterpret_cast<const float2*>(&Uc[rowl + nx + x]);
          zp1[0] = q.x;
          zp1[1] = q.y;
        }
        if (i + 2 < nrows) {
          zp2[0] = uc[i + 2 < S ? i + 2 : i][0];
          zp2[1] = uc[i + 2 < S ? i + 2 : i][1];
        } else {
          const float2 q = *reinterpret_cast<const float2*>(&Uc[rowl + 2 * nx + x]);
          zp2[0] = q.x;
          zp2[1] = q.y;
        }
        const float u0 = uc[i][0], u1 = uc[i][1];
        // x-direction second derivative of both cells
        const float d2x0 = (((F_D2A * u0 + F_D2B * (u1 + A.y)) - F_D2C * (B.x + A.x)) * d2a) * d2b;
        const float d2x1 = (((F_D2A * u1 + F_D2B * (B.x + u0)) - F_D2C * (B.y + A.y)) * d2a) * d2b;
        float w0, w1;
        if (pml) {
          const int ca = (z - r0) * 2 * kSwx + xs;
          const float2 P0 = *reinterpret_cast<const float2*>(&APXc[ca - 2]);
          const float2 P1 = *reinterpret_cast<const float2*>(&APXc[ca]);
          const float2 P2 = *reinterpret_cast<const float2*>(&APXc[ca + 2]);
          const float d10 = ((F_D1A * (u1 - A.y)) - F_D1B * (B.x - A.x)) * rh;
          const float d11 = ((F_D1A * (B.x - u0)) - F_D1B * (B.y - A.y)) * rh;
          const float da0 = ((F_D1A * (P1.y - P0.y)) - F_D1B * (P2.x - P0.x)) * rh;
          const float da1 = ((F_D1A * (P2.x - P1.x)) - F_D1B * (P2.y - P0.y)) * rh;
          const float tmp0 = ((opbx0 * d2x0) + (dbx0 * d10)) + da0;
          const float tmp1 = ((opbx1 * d2x1) + (dbx1 * d11)) + da1;
          w0 = (opbx0 * tmp0) + (ax0 * zx[i][0]);
          w1 = (opbx1 * tmp1) + (ax1 * zx[i][1]);
          const float psi0 = (bx0 * d10) + P1.x;
          const float psi1 = (bx1 * d11) + P1.y;
          zx[i][0] = (bx0 * tmp0) + (ax0 * zx[i][0]);
          zx[i][1] = (bx1 * tmp1) + (ax1 * zx[i][1]);
          *reinterpret_cast<float2*>(&APXn[ca]) = make_float2(ax0 * psi0, ax1 * psi1);
        } else {
          w0 = d2x0;
          w1 = d2x1;
        }
        {  // z direction
          const float d2z0 = (((F_D2A * u0 + F_D2B * (zp1[0] + zm1[0])) - F_D2C * (zp2[0] + zm2[0])) * d2a) * d2b;
          const float d2z1 = (((F_D2A * u1 + F_D2B * (zp1[1] + zm1[1])) - F_D2C * (zp2[1] + zm2[1])) * d2a) * d2b;
          if (z < region || z >= nz - region) {
            const int zss = (z < sw) ? z : z - (nz - sw) + bot_off;
            const int cz = zss * nx + x;
            const float az = sAZ[z], bz = sBZ[z], dbz = sDBZ[z];
            const float opbz = 1.0f + bz;
            const float2 Qm2 = *reinterpret_cast<const float2*>(&APZc[cz - 2 * nx]);
            const float2 Qm1 = *reinterpret_cast<const float2*>(&APZc[cz - nx]);
            const float2 Q0 = *reinterpret_cast<const float2*>(&APZc[cz]);
            const float2 Qp1 = *reinterpret_cast<const float2*>(&APZc[cz + nx]);
            const float2 Qp2 = *reinterpret_cast<const float2*>(&APZc[cz + 2 * nx]);
            const float2 Z = *reinterpret_cast<const float2*>(&ZZ[cz]);
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
            *reinterpret_cast<float2*>(&ZZ[cz]) = make_float2((bz * tmp0) + (az * Z.x), (bz * tmp1) + (az * Z.y));
            *reinterpret_cast<float2*>(&APZn[cz]) = make_float2(az * psi0, az * psi1);
          } else {
            w0 = w0 + d2z0;
            w1 = w1 + d2z1;
          }
        }
        if (STORE) {
          *reinterpret_cast<float2*>(&st_t[z * nx + x]) = make_float2(c2[i][0] * w0, c2[i][1] * w1);
        }
        float n0 = ((v2[i][0] * w0) + (2.0f * u0)) - un[i][0];
        float n1 = ((v2[i][1] * w1) + (2.0f * u1)) - un[i][1];
        if (srcmask & (3u << (2 * i))) {
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            const int cell = z * nx + x;
            const float wk_ = p.st.src_w[4 * shot + k];
            if (cell == sc[k]) n0 = n0 + (((-v2[i][0]) * wk_) * f);
            if (cell + 1 == sc[k]) n1 = n1 + (((-v2[i][1]) * wk_) * f);
          }
        }
        un[i][0] = n0;
        un[i][1] = n1;
        *reinterpret_cast<float2*>(&Un[rowl + x]) = make_float2(n0, n1);
        if constexpr (C > 1) {
          if (rank > 0 && z < r0 + FD_PAD) st_peer2(&Un[(z - pr_lo) * nx + x], rank - 1, n0, n1);
          if (rank < C - 1 && z >= r1 - FD_PAD) st_peer2(&Un[(z - (r1 - FD_PAD)) * nx + x], rank + 1, n0, n1);
        }
      }
    }
    step_barrier<C>();
  };

  int t = p.t0;
  for (; t + 1 < p.t1; t += 2) {
    step(t, uA, uB);
    step(t + 1, uB, uA);
  }
  if (t < p.t1) step(t, uA, uB);
}

template <int C, int S, int NSEG, int NI>
cudaError_t fwd2_dispatch_impl(bool traces, bool store, const FwdArgs& a, size_t smem, cudaStream_t s) {
  constexpr int NT = NSEG * 32 * (1 + NI);
  if (traces && store) return launch_cluster(fwd2_kernel<C, S, NSEG, NI, true, true>, C, NT, a.units, smem, s, a);
  if (traces) return launch_cluster(fwd2_kernel<C, S, NSEG, NI, true, false>, C, NT, a.units, smem, s, a);
  if (store) return launch_cluster(fwd2_kernel<C, S, NSEG, NI, false, true>, C, NT, a.units, smem, s, a);
  return cudaErrorInvalidValue;
}

}  // namespace wg
