// Streamed path for grids too large for the resident kernels (for example 844 x 344 padded cells,
// 800 x 300 visible at 5 m): the wavefields of every (model, shot) unit live in HBM and each time
// step is one persistent launch over all units' tiles.
//
// A tile is 64 x 32 cells (x by z). A CTA walks the tiles of the step (unit-major, so neighbouring
// CTAs share halos in L2) with a two-stage TMA pipeline: while it updates one tile, the next tile's
// wavefield with its halo (72 x 36 floats; the x halo is rounded to 16 bytes) is already being
// copied into shared memory by cp.async.bulk.tensor, completion signalled on an mbarrier. Each
// thread owns a column pair over 4 rows; the vertical neighbours come from its column in shared
// memory, the horizontal ones from float2 loads beside it. Tiles that touch the C-PML read and
// write the packed PML strips (global memory, L1/L2 resident); interior tiles skip them entirely.
//
// Arithmetic follows the reference's operation order (splatForward.wgsl:48-121 and
// splatAdjoint.wgsl:58-131, restated in the resident kernels) with -fmad=false, so traces and
// gradients equal the f32 restatement bit for bit. The PML formulas are applied to every column
// pair that has a cell inside the adjoint's PML region; on cells outside a region the profiles are
// zero and the PML formula reduces exactly to the interior one.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <string>
#include <vector>

#include "wave_launch.h"
#include "wgnet_gb300.h"

namespace wg {
namespace {

constexpr int TX_ = 64, TZ_ = 32;           // tile of cells per CTA iteration
constexpr int HX = 4, HZ = 2;               // halo loaded on each side (x rounded to 16 bytes)
constexpr int BX = TX_ + 2 * HX;            // 72 columns in shared memory
constexpr int BZ = TZ_ + 2 * HZ;            // 36 rows
constexpr int NTH = 256;                    // 32 column pairs x 8 groups of 4 rows
constexpr int RPT = 4;                      // rows per thread
constexpr unsigned kTileBytes = BX * BZ * 4;
constexpr long kWaitLimit = 1L << 22;       // mbarrier polls before giving up

struct SArgs {
  int nx, nz, units, shots, models_unused;
  int tiles_x, tiles_z;
  int ssw;         // packed strip width per side (x strips: columns, z strips: rows)
  int region;      // PML region used for both axes (the adjoint's, pml + 3 FD_PAD)
  int nt, t, seg_t0;
  float rh, dt2, d2a, d2b;
  const float* prof;     // ax bx dbx (nx) | az bz dbz (nz)
  const float* wavelet;
  Stations st;
  const float* vel;      // [models][nz][nx] clamped padded velocity
  int rec_z0, rec_z1;    // rows holding receiver corners
  const int* tile_rec_start;  // [tiles + 1] receivers recorded by each tile (forward)
  const int* tile_rec;
  int* status;
  float* W;              // forward: wavefield ping-pong [2][units][nz][nx]; adjoint: lambda
  float* PX;             // forward a*psi_x ping-pong [2][units][nz][2 ssw]; adjoint psi_x ping-pong
  float* ZX;             // forward zeta_x [units][nz][2 ssw]; adjoint zeta_x ping-pong
  float* PZ;             // forward a*psi_z ping-pong [2][units][2 ssw][nx]; adjoint psi_z ping-pong
  float* ZZ;             // forward zeta_z [units][2 ssw][nx]; adjoint zeta_z ping-pong
  float* traces;         // [units][nt][nrec]
  float* stored;         // [units][seg][nz][nx], step t at t - seg_t0
  int seg;
  const float* residual; // [units][nt][nrec]
  float* gacc;           // [units][nz][nx]
};

__device__ __forceinline__ float2 lds2(const float* p) { return *reinterpret_cast<const float2*>(p); }
__device__ __forceinline__ float2 ldg2(const float* p) { return __ldg(reinterpret_cast<const float2*>(p)); }
__device__ __forceinline__ float2 ld2(const float* p) { return *reinterpret_cast<const float2*>(p); }
__device__ __forceinline__ void st2(float* p, float a, float b) { *reinterpret_cast<float2*>(p) = make_float2(a, b); }

__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// Bounded wait for the phase with parity `parity`; false when `limit` polls are reached.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity, long limit = kWaitLimit) {
  const unsigned a = smem_u32(bar);
  for (long i = 0; i < limit; ++i) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}

// 3-D tiled TMA load of one tile box (x, z, buffer*units + unit) into shared memory.
__device__ __forceinline__ void tma_load(float* dst, const CUtensorMap* map, int x, int z, int u, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(z), "r"(u), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ int xstrip(int x, int nx, int ssw) { return x < ssw ? x : x - (nx - 2 * ssw); }

struct Pipe {
  uint64_t* bar;
  float* stage;  // [2][BZ * BX]
};

// Issue the tile load of job `job` (buffer `buf` of the wavefield) into stage s.
__device__ __forceinline__ void issue(const SArgs& a, const CUtensorMap* map, Pipe& p, int job, int s, int buf) {
  const int tiles = a.tiles_x * a.tiles_z;
  const int unit = job / tiles, tile = job % tiles;
  const int tz = tile / a.tiles_x, tx = tile % a.tiles_x;
  mbar_expect_tx(&p.bar[s], kTileBytes);
  tma_load(p.stage + s * BZ * BX, map, tx * TX_ - HX, tz * TZ_ - HZ, buf * a.units + unit, &p.bar[s]);
}

__device__ __forceinline__ void report(int* status) { atomicCAS(status, 0, ST_CUDA); }

// A tile (with its halo) clear of the PML strips, the grid frame, the receivers' rows and this
// unit's source corners: every pair of every row takes the interior formulas.
__device__ __forceinline__ bool interior_tile(const SArgs& a, int x0, int z0, const int* sc) {
  const int m = a.ssw;
  if (x0 - HX < m || x0 + TX_ + HX > a.nx - m || z0 - HZ < m || z0 + TZ_ + HZ > a.nz - m) return false;
  if (z0 + TZ_ > a.rec_z0 && z0 <= a.rec_z1) return false;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int c = __ldg(&sc[k]);
    const int cz = c / a.nx, cx = c % a.nx;
    if (cz >= z0 && cz < z0 + TZ_ && cx >= x0 && cx < x0 + TX_) return false;
  }
  return true;
}

// ------------------------------------------------------------------------------------------------
// Forward step t: u_next = v^2 dt^2 w + 2 u - u_prev over every unit, receivers read before the
// update, source after it (splatForward.wgsl:48-121).
// ------------------------------------------------------------------------------------------------
struct FwdMaps {
  CUtensorMap u;  // wavefield with halo: 72 x 36 boxes over [2 units][nz][nx]
  CUtensorMap p;  // wavefield without halo (the previous step): 64 x 32 boxes
  CUtensorMap v;  // velocity: 64 x 32 boxes over [models][nz][nx]
};
constexpr int FST = 3;                                        // forward pipeline stages
constexpr int FSTAGE_F = BZ * BX + 2 * TZ_ * TX_;             // floats per stage: U | P | V
constexpr size_t kFwdSmem = FST * FSTAGE_F * 4 + 128 + 16 * FST;

// Issue the three copies of job `job` into stage buffer `st` with barrier `bar`.
__device__ __forceinline__ void issue_fwd(const SArgs& a, const FwdMaps& m, float* st, uint64_t* bar, int job,
                                          int par) {
  const int tiles = a.tiles_x * a.tiles_z;
  const int unit = job / tiles, tile = job % tiles;
  const int tz = tile / a.tiles_x, tx = tile % a.tiles_x;
  mbar_expect_tx(bar, FSTAGE_F * 4);
  tma_load(st, &m.u, tx * TX_ - HX, tz * TZ_ - HZ, par * a.units + unit, bar);
  tma_load(st + BZ * BX, &m.p, tx * TX_, tz * TZ_, (1 - par) * a.units + unit, bar);
  tma_load(st + BZ * BX + TZ_ * TX_, &m.v, tx * TX_, tz * TZ_, unit / a.shots, bar);
}

constexpr int FWD_THREADS = NTH + 32;  // 8 consumer warps + 1 producer warp

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Warp-specialised: warp 8 (one lane) streams the jobs' tiles into FST stages (waiting on each
// stage's "empty" barrier before refilling it), warps 0-7 update the tiles and release each stage
// with one arrival per warp. No CTA-wide barrier per tile: consumer warps run up to FST tiles
// apart. Every wait is bounded; a consumer that gives up records the error and leaves; the
// producer that gives up records it and waits (bounded) for the copies it issued.
template <bool TRACES, bool STORE>
__global__ void __launch_bounds__(FWD_THREADS, 2) fwd_stream_kernel(const __grid_constant__ FwdMaps maps,
                                                                    const __grid_constant__ SArgs a) {
  extern __shared__ __align__(128) float fsm_raw[];
  float* stage = fsm_raw + ((128 - (smem_u32(fsm_raw) & 127)) & 127) / 4;  // [FST][U | P | V]
  uint64_t* full = reinterpret_cast<uint64_t*>(stage + FST * FSTAGE_F);
  uint64_t* empty = full + FST;
  const int tid = threadIdx.x;
  const int tiles = a.tiles_x * a.tiles_z;
  const int jobs = a.units * tiles;
  const int par = a.t & 1;
  const int nx = a.nx, nz = a.nz, ssw = a.ssw, region = a.region;
  const size_t cells = static_cast<size_t>(nx) * nz;
  if (tid == 0) {
    for (int k = 0; k < FST; ++k) {
      mbar_init(&full[k], 1);
      mbar_init(&empty[k], NTH / 32);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (tid >= NTH) {  // producer warp
    if (tid == NTH) {
      int issued = 0;
      for (int job = blockIdx.x; job < jobs; job += gridDim.x, ++issued) {
        const int s = issued % FST;
        if (issued >= FST && !mbar_wait(&empty[s], (issued / FST - 1) & 1)) {
          report(a.status);
          for (int k = 1; k <= FST && issued - k >= 0; ++k)  // the copies still landing
            mbar_wait(&full[(issued - k) % FST], ((issued - k) / FST) & 1);
          return;
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        issue_fwd(a, maps, stage + s * FSTAGE_F, &full[s], job, par);
      }
    }
    return;
  }
  const float f = __ldg(&a.wavelet[a.t]);
  const int pc = tid & 31, grp = tid >> 5;
  int job = blockIdx.x;
  for (int i = 0; job < jobs; ++i, job += gridDim.x) {
    const int s = i % FST;
    if (!mbar_wait(&full[s], (i / FST) & 1)) {
      report(a.status);
      return;
    }
    const int unit = job / tiles, tile = job % tiles;
    const int tzi = tile / a.tiles_x, txi = tile % a.tiles_x;
    const int x0 = txi * TX_, z0 = tzi * TZ_;
    const int shot = unit % a.shots;
    const int x = x0 + 2 * pc;
    const int zr = z0 + RPT * grp;
    const bool xok = x >= FD_PAD && x + 1 < nx - FD_PAD;
    const bool xpml = x < region || x + 1 >= nx - region;
    float* Wn = a.W + (static_cast<size_t>(1 - par) * a.units + unit) * cells;
    const float* Pt = stage + s * FSTAGE_F + BZ * BX;
    const float* Vt = Pt + TZ_ * TX_;
    float2 pv[RPT], vv[RPT];
#pragma unroll
    for (int r = 0; r < RPT; ++r) {
      pv[r] = lds2(Pt + (RPT * grp + r) * TX_ + 2 * pc);
      vv[r] = lds2(Vt + (RPT * grp + r) * TX_ + 2 * pc);
    }
    const float* T = stage + s * FSTAGE_F;

    if (interior_tile(a, x0, z0, a.st.src_cell + 4 * shot)) {
      // interior tile: no frame, PML, receivers or sources
      const int sx = 2 * pc + HX, sz = RPT * grp + HZ;
      float2 col[RPT + 4];
#pragma unroll
      for (int k = 0; k < RPT + 4; ++k) col[k] = lds2(T + (sz - 2 + k) * BX + sx);
      float* stp = STORE ? a.stored + (static_cast<size_t>(unit) * a.seg + (a.t - a.seg_t0)) * cells : nullptr;
#pragma unroll
      for (int r = 0; r < RPT; ++r) {
        const int cell = (zr + r) * nx + x;
        const float2 A = lds2(T + (sz + r) * BX + sx - 2);
        const float2 B = lds2(T + (sz + r) * BX + sx + 2);
        const float u0 = col[r + 2].x, u1 = col[r + 2].y;
        const float2 zm2 = col[r], zm1 = col[r + 1], zp1 = col[r + 3], zp2 = col[r + 4];
        const float d2x0 = (((F_D2A * u0 + F_D2B * (u1 + A.y)) - F_D2C * (B.x + A.x)) * a.d2a) * a.d2b;
        const float d2x1 = (((F_D2A * u1 + F_D2B * (B.x + u0)) - F_D2C * (B.y + A.y)) * a.d2a) * a.d2b;
        const float d2z0 = (((F_D2A * u0 + F_D2B * (zp1.x + zm1.x)) - F_D2C * (zp2.x + zm2.x)) * a.d2a) * a.d2b;
        const float d2z1 = (((F_D2A * u1 + F_D2B * (zp1.y + zm1.y)) - F_D2C * (zp2.y + zm2.y)) * a.d2a) * a.d2b;
        const float w0 = d2x0 + d2z0, w1 = d2x1 + d2z1;
        const float2 v = vv[r];
        const float v20 = (v.x * v.x) * a.dt2, v21 = (v.y * v.y) * a.dt2;
        const float n0 = ((v20 * w0) + (2.0f * u0)) - pv[r].x;
        const float n1 = ((v21 * w1) + (2.0f * u1)) - pv[r].y;
        if (STORE)
          __stcs(reinterpret_cast<float2*>(stp + cell),
                 make_float2(((2.0f * v.x) * a.dt2) * w0, ((2.0f * v.y) * a.dt2) * w1));
        st2(Wn + cell, n0, n1);
      }
      __syncwarp();
      if (pc == 0) mbar_arrive(&empty[s]);
      continue;
    }

    if (TRACES) {
      const int r0 = a.tile_rec_start[tile], r1 = a.tile_rec_start[tile + 1];
      for (int k = r0 + tid; k < r1; k += NTH) {
        const int r = a.tile_rec[k];
        float acc = 0.0f;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          const int cell = a.st.rec_cell[4 * r + c];
          const int cz = cell / nx - (z0 - HZ), cx = cell % nx - (x0 - HX);
          acc = acc + a.st.rec_w[4 * r + c] * T[cz * BX + cx];
        }
        a.traces[(static_cast<size_t>(unit) * a.nt + a.t) * a.st.nrec + r] = acc;
      }
    }

    const int sx = 2 * pc + HX, sz = RPT * grp + HZ;
    float2 col[RPT + 4];
#pragma unroll
    for (int k = 0; k < RPT + 4; ++k) col[k] = lds2(T + (sz - 2 + k) * BX + sx);
    const int* sc = a.st.src_cell + 4 * shot;
    // bit 2 r + j: cell (zr + r, x + j) is a corner of this unit's source
    unsigned srcm = 0;
    {
      const int base = zr * nx + x;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int d = __ldg(&sc[k]) - base;
#pragma unroll
        for (int r = 0; r < RPT; ++r) {
          const unsigned o = static_cast<unsigned>(d - r * nx);
          if (o < 2u) srcm |= 1u << (2 * r + o);
        }
      }
    }
    float* stp = STORE ? a.stored + (static_cast<size_t>(unit) * a.seg + (a.t - a.seg_t0)) * cells : nullptr;
    float ax0 = 0.f, ax1 = 0.f, bx0 = 0.f, bx1 = 0.f, dbx0 = 0.f, dbx1 = 0.f;
    if (xok && xpml) {
      const float2 pa = ldg2(a.prof + x), pb = ldg2(a.prof + nx + x), pd = ldg2(a.prof + 2 * nx + x);
      ax0 = pa.x, ax1 = pa.y, bx0 = pb.x, bx1 = pb.y, dbx0 = pd.x, dbx1 = pd.y;
    }
    const float opbx0 = 1.0f + bx0, opbx1 = 1.0f + bx1;
    const size_t xs_unit = static_cast<size_t>(nz) * 2 * ssw;  // floats per unit of an x strip array
    const size_t zs_unit = static_cast<size_t>(2) * ssw * nx;
    const float* PXc = a.PX + (static_cast<size_t>(par) * a.units + unit) * xs_unit;
    float* PXn = a.PX + (static_cast<size_t>(1 - par) * a.units + unit) * xs_unit;
    float* ZXo = a.ZX + static_cast<size_t>(unit) * xs_unit;
    const float* PZc = a.PZ + (static_cast<size_t>(par) * a.units + unit) * zs_unit;
    float* PZn = a.PZ + (static_cast<size_t>(1 - par) * a.units + unit) * zs_unit;
    float* ZZo = a.ZZ + static_cast<size_t>(unit) * zs_unit;
    const int xc = xstrip(x, nx, ssw);
#pragma unroll
    for (int r = 0; r < RPT; ++r) {
      const int z = zr + r;
      if (!xok || z < FD_PAD || z >= nz - FD_PAD) continue;
      const int cell = z * nx + x;
      const float2 U = col[r + 2];
      const float2 A = lds2(T + (sz + r) * BX + sx - 2);
      const float2 B = lds2(T + (sz + r) * BX + sx + 2);
      const float u0 = U.x, u1 = U.y;
      const float d2x0 = (((F_D2A * u0 + F_D2B * (u1 + A.y)) - F_D2C * (B.x + A.x)) * a.d2a) * a.d2b;
      const float d2x1 = (((F_D2A * u1 + F_D2B * (B.x + u0)) - F_D2C * (B.y + A.y)) * a.d2a) * a.d2b;
      float w0, w1;
      if (xpml) {
        const float* row = PXc + z * 2 * ssw + xc;
        const float2 P0 = ld2(row - 2), P1 = ld2(row), P2 = ld2(row + 2);
        float* zrow = ZXo + z * 2 * ssw + xc;
        const float2 Z = ld2(zrow);
        const float d10 = ((F_D1A * (u1 - A.y)) - F_D1B * (B.x - A.x)) * a.rh;
        const float d11 = ((F_D1A * (B.x - u0)) - F_D1B * (B.y - A.y)) * a.rh;
        const float da0 = ((F_D1A * (P1.y - P0.y)) - F_D1B * (P2.x - P0.x)) * a.rh;
        const float da1 = ((F_D1A * (P2.x - P1.x)) - F_D1B * (P2.y - P0.y)) * a.rh;
        const float tmp0 = ((opbx0 * d2x0) + (dbx0 * d10)) + da0;
        const float tmp1 = ((opbx1 * d2x1) + (dbx1 * d11)) + da1;
        w0 = (opbx0 * tmp0) + (ax0 * Z.x);
        w1 = (opbx1 * tmp1) + (ax1 * Z.y);
        const float psi0 = (bx0 * d10) + P1.x;
        const float psi1 = (bx1 * d11) + P1.y;
        st2(zrow, (bx0 * tmp0) + (ax0 * Z.x), (bx1 * tmp1) + (ax1 * Z.y));
        st2(PXn + z * 2 * ssw + xc, ax0 * psi0, ax1 * psi1);
      } else {
        w0 = d2x0;
        w1 = d2x1;
      }
      const float2 zm2 = col[r], zm1 = col[r + 1], zp1 = col[r + 3], zp2 = col[r + 4];
      const float d2z0 = (((F_D2A * u0 + F_D2B * (zp1.x + zm1.x)) - F_D2C * (zp2.x + zm2.x)) * a.d2a) * a.d2b;
      const float d2z1 = (((F_D2A * u1 + F_D2B * (zp1.y + zm1.y)) - F_D2C * (zp2.y + zm2.y)) * a.d2a) * a.d2b;
      if (z < region || z >= nz - region) {
        const int zc = z < ssw ? z : z - (nz - 2 * ssw);
        const float az = __ldg(&a.prof[3 * nx + z]), bz = __ldg(&a.prof[3 * nx + nz + z]),
                    dbz = __ldg(&a.prof[3 * nx + 2 * nz + z]);
        const float opbz = 1.0f + bz;
        const float* q = PZc + zc * nx + x;
        const float2 Qm2 = ld2(q - 2 * nx), Qm1 = ld2(q - nx), Q0 = ld2(q), Qp1 = ld2(q + nx), Qp2 = ld2(q + 2 * nx);
        float* zz = ZZo + zc * nx + x;
        const float2 Z = ld2(zz);
        const float d10 = ((F_D1A * (zp1.x - zm1.x)) - F_D1B * (zp2.x - zm2.x)) * a.rh;
        const float d11 = ((F_D1A * (zp1.y - zm1.y)) - F_D1B * (zp2.y - zm2.y)) * a.rh;
        const float da0 = ((F_D1A * (Qp1.x - Qm1.x)) - F_D1B * (Qp2.x - Qm2.x)) * a.rh;
        const float da1 = ((F_D1A * (Qp1.y - Qm1.y)) - F_D1B * (Qp2.y - Qm2.y)) * a.rh;
        const float tmp0 = ((opbz * d2z0) + (dbz * d10)) + da0;
        const float tmp1 = ((opbz * d2z1) + (dbz * d11)) + da1;
        w0 = w0 + ((opbz * tmp0) + (az * Z.x));
        w1 = w1 + ((opbz * tmp1) + (az * Z.y));
        const float psi0 = (bz * d10) + Q0.x;
        const float psi1 = (bz * d11) + Q0.y;
        st2(zz, (bz * tmp0) + (az * Z.x), (bz * tmp1) + (az * Z.y));
        st2(PZn + zc * nx + x, az * psi0, az * psi1);
      } else {
        w0 = w0 + d2z0;
        w1 = w1 + d2z1;
      }
      const float2 v = vv[r];
      const float v20 = (v.x * v.x) * a.dt2, v21 = (v.y * v.y) * a.dt2;
      const float2 prev = pv[r];
      float n0 = ((v20 * w0) + (2.0f * u0)) - prev.x;
      float n1 = ((v21 * w1) + (2.0f * u1)) - prev.y;
      if (STORE)
        __stcs(reinterpret_cast<float2*>(stp + cell), make_float2(((2.0f * v.x) * a.dt2) * w0, ((2.0f * v.y) * a.dt2) * w1));
      if (srcm & (3u << (2 * r))) {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          if (cell == sc[k]) n0 = n0 + (((-v20) * a.st.src_w[4 * shot + k]) * f);
          if (cell + 1 == sc[k]) n1 = n1 + (((-v21) * a.st.src_w[4 * shot + k]) * f);
        }
      }
      st2(Wn + cell, n0, n1);
    }
    __syncwarp();
    if (pc == 0) mbar_arrive(&empty[s]);  // this warp is done with the stage
  }
}

// ------------------------------------------------------------------------------------------------
// Temporally blocked forward: TB_T steps per launch. Each job (unit, 64 x 32 tile) takes its tile
// with a halo of 2 TB_T cells per side (the stencil reaches 2 cells per step) into shared memory:
// u(t), u(t-1) and the velocity by TMA (double-buffered: the next job's boxes land while this one
// computes), and, on tiles that reach a C-PML strip, a*psi and zeta of the strip cells. It then
// advances the region TB_T steps in shared memory, the computed region shrinking by 2 cells per
// side per step, and writes back the tile: the halo cells are computed by every tile that holds
// them, with the same operations on the same values, so each cell's value is the per-step kernel's
// bit for bit (sources are injected into halo copies too; receivers are recorded by the tile that
// holds their first corner). Per step the wavefield crosses HBM once per TB_T steps instead of once
// per step. The state is read from one set and written to the other (sets alternate per launch),
// so no CTA overwrites cells a neighbouring CTA still has to read. Off by default (engine option
// "temporal_block"): the per-step forward is latency-bound rather than bandwidth-bound, so the
// saved traffic buys nothing, and the redundant halo updates (31 % of the work) make this kernel
// slower on the 800 x 300 survey.
// ------------------------------------------------------------------------------------------------
constexpr int TB_T = 4;                      // time steps per launch
constexpr int TB_H = 2 * TB_T;               // halo per side
constexpr int TB_RX = TX_ + 2 * TB_H;        // 80 region columns (x offset 64 k - 8: 16-byte aligned)
constexpr int TB_RZ = TZ_ + 2 * TB_H;        // 48 region rows
constexpr int TB_N = TB_RX * TB_RZ;          // cells of a region
constexpr int TB_THREADS = 512;
constexpr int TB_STAGE = 3 * TB_N;           // floats per stage: u(t) | u(t-1) | v
constexpr size_t kTbSmem = static_cast<size_t>(2 * TB_STAGE + 6 * TB_N) * 4 + 2 * 8 + 128;

struct TbArgs {
  SArgs a;         // geometry, stations, profiles, traces, stored terms, status; a.t = first step
  int nsub;        // steps of this launch, 1..TB_T
  int set_in;      // state set read (the other one is written)
  float* W;        // [2 sets][2 levels: u(t), u(t-1)][units][nz][nx]
  float* PX;       // a psi_x [2 sets][units][nz][2 ssw]
  float* ZX;       // zeta_x  [2 sets][units][nz][2 ssw]
  float* PZ;       // a psi_z [2 sets][units][2 ssw][nx]
  float* ZZ;       // zeta_z  [2 sets][units][2 ssw][nx]
};

template <bool TRACES, bool STORE>
__global__ void __launch_bounds__(TB_THREADS, 1) fwd_tb_kernel(const __grid_constant__ CUtensorMap umap,
                                                               const __grid_constant__ CUtensorMap vmap,
                                                               const __grid_constant__ TbArgs p) {
  extern __shared__ __align__(128) float tsm_raw[];
  float* sm = tsm_raw + ((128 - (smem_u32(tsm_raw) & 127)) & 127) / 4;
  float* stages = sm;             // [2][u(t) | u(t-1) | v]
  float* PXA = sm + 2 * TB_STAGE;  // a psi_x, two buffers (neighbours read x +- 2)
  float* PXB = PXA + TB_N;
  float* ZXr = PXB + TB_N;         // zeta_x (owner only, updated in place)
  float* PZA = ZXr + TB_N;         // a psi_z, two buffers
  float* PZB = PZA + TB_N;
  float* ZZr = PZB + TB_N;
  uint64_t* full = reinterpret_cast<uint64_t*>(ZZr + TB_N);
  const SArgs& a = p.a;
  const int tid = threadIdx.x;
  const int tiles = a.tiles_x * a.tiles_z;
  const int jobs = a.units * tiles;
  const int nx = a.nx, nz = a.nz, ssw = a.ssw, region = a.region;
  const size_t cells = static_cast<size_t>(nx) * nz;
  const size_t xs_unit = static_cast<size_t>(nz) * 2 * ssw, zs_unit = static_cast<size_t>(2) * ssw * nx;
  const int set_out = 1 - p.set_in;
  if (tid == 0) {
    mbar_init(&full[0], 1);
    mbar_init(&full[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  auto issue = [&](int job, int s) {
    const int unit = job / tiles, tile = job % tiles;
    const int x = (tile % a.tiles_x) * TX_ - TB_H, z = (tile / a.tiles_x) * TZ_ - TB_H;
    float* st = stages + s * TB_STAGE;
    mbar_expect_tx(&full[s], TB_STAGE * 4);
    tma_load(st, &umap, x, z, (p.set_in * 2 + 0) * a.units + unit, &full[s]);
    tma_load(st + TB_N, &umap, x, z, (p.set_in * 2 + 1) * a.units + unit, &full[s]);
    tma_load(st + 2 * TB_N, &vmap, x, z, unit / a.shots, &full[s]);
  };
  if (tid == 0 && static_cast<int>(blockIdx.x) < jobs) issue(blockIdx.x, 0);
  int i = 0;
  for (int job = blockIdx.x; job < jobs; job += gridDim.x, ++i) {
    const int s = i & 1;
    const bool next = job + static_cast<int>(gridDim.x) < jobs;
    if (tid == 0 && next) {  // the other stage's last job ended with a CTA barrier
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      issue(job + gridDim.x, 1 - s);
    }
    const bool ok = mbar_wait(&full[s], (i >> 1) & 1);
    if (__syncthreads_or(!ok)) {
      if (tid == 0) {
        report(a.status);
        if (next) mbar_wait(&full[1 - s], ((i + 1) >> 1) & 1);  // the copies still landing (bounded)
      }
      return;
    }
    const int unit = job / tiles, tile = job % tiles;
    const int x0 = (tile % a.tiles_x) * TX_, z0 = (tile / a.tiles_x) * TZ_;
    const int rx0 = x0 - TB_H, rz0 = z0 - TB_H;  // region origin in grid coordinates
    const int shot = unit % a.shots;
    float* U = stages + s * TB_STAGE;
    float* UP = U + TB_N;
    const float* V = UP + TB_N;
    const bool pml_tile = rx0 < ssw || rx0 + TB_RX > nx - ssw || rz0 < ssw || rz0 + TB_RZ > nz - ssw;
    if (pml_tile) {
      const float* PXi = p.PX + (static_cast<size_t>(p.set_in) * a.units + unit) * xs_unit;
      const float* ZXi = p.ZX + (static_cast<size_t>(p.set_in) * a.units + unit) * xs_unit;
      const float* PZi = p.PZ + (static_cast<size_t>(p.set_in) * a.units + unit) * zs_unit;
      const float* ZZi = p.ZZ + (static_cast<size_t>(p.set_in) * a.units + unit) * zs_unit;
      for (int c = tid; c < TB_N; c += TB_THREADS) {
        const int z = rz0 + c / TB_RX, x = rx0 + c % TB_RX;
        float px = 0.f, zx = 0.f, pz = 0.f, zz = 0.f;
        if (x >= 0 && x < nx && z >= 0 && z < nz) {
          if (x < ssw || x >= nx - ssw) {
            const int k = z * 2 * ssw + xstrip(x, nx, ssw);
            px = PXi[k];
            zx = ZXi[k];
          }
          if (z < ssw || z >= nz - ssw) {
            const int k = (z < ssw ? z : z - (nz - 2 * ssw)) * nx + x;
            pz = PZi[k];
            zz = ZZi[k];
          }
        }
        // both buffers: a*psi of strip cells outside the C-PML region is never updated
        PXA[c] = px;
        PXB[c] = px;
        ZXr[c] = zx;
        PZA[c] = pz;
        PZB[c] = pz;
        ZZr[c] = zz;
      }
      __syncthreads();
    }
    const int* sc = a.st.src_cell + 4 * shot;
    const float* sw = a.st.src_w + 4 * shot;
    const int sc0 = __ldg(&sc[0]), sc1 = __ldg(&sc[1]), sc2 = __ldg(&sc[2]), sc3 = __ldg(&sc[3]);
    for (int k = 0; k < p.nsub; ++k) {
      const int t = a.t + k;
      const float f = __ldg(&a.wavelet[t]);
      const float* Uc = (k & 1) ? UP : U;  // u(t)
      float* Un = (k & 1) ? U : UP;        // u(t - 1), overwritten by u(t + 1)
      const float* Pc = (k & 1) ? PXB : PXA;
      float* Pn = (k & 1) ? PXA : PXB;
      const float* Qc = (k & 1) ? PZB : PZA;
      float* Qn = (k & 1) ? PZA : PZB;
      if (TRACES) {
        const int r0 = a.tile_rec_start[tile], r1 = a.tile_rec_start[tile + 1];
        for (int q = r0 + tid; q < r1; q += TB_THREADS) {
          const int r = a.tile_rec[q];
          float acc = 0.0f;
#pragma unroll
          for (int cc = 0; cc < 4; ++cc) {
            const int cell = a.st.rec_cell[4 * r + cc];
            acc = acc + a.st.rec_w[4 * r + cc] * Uc[(cell / nx - rz0) * TB_RX + (cell % nx - rx0)];
          }
          a.traces[(static_cast<size_t>(unit) * a.nt + t) * a.st.nrec + r] = acc;
        }
      }
      float* stp = STORE ? a.stored + (static_cast<size_t>(unit) * a.seg + (t - a.seg_t0)) * cells : nullptr;
      const int m = 2 * (k + 1);  // region of step k: 2 (k + 1) cells inside the loaded one
      const int pairs = (TB_RX - 2 * m) / 2, rows = TB_RZ - 2 * m;
      for (int idx = tid; idx < pairs * rows; idx += TB_THREADS) {
        const int lz = m + idx / pairs, lx = m + 2 * (idx % pairs);
        const int z = rz0 + lz, x = rx0 + lx;
        if (z < FD_PAD || z >= nz - FD_PAD || x < FD_PAD || x + 1 >= nx - FD_PAD) continue;
        const int c = lz * TB_RX + lx;
        const int cell = z * nx + x;
        const float2 U0 = lds2(Uc + c);
        const float2 A = lds2(Uc + c - 2);
        const float2 B = lds2(Uc + c + 2);
        const float u0 = U0.x, u1 = U0.y;
        const float d2x0 = (((F_D2A * u0 + F_D2B * (u1 + A.y)) - F_D2C * (B.x + A.x)) * a.d2a) * a.d2b;
        const float d2x1 = (((F_D2A * u1 + F_D2B * (B.x + u0)) - F_D2C * (B.y + A.y)) * a.d2a) * a.d2b;
        float w0, w1;
        if (x < region || x + 1 >= nx - region) {
          const float2 pa = ldg2(a.prof + x), pb = ldg2(a.prof + nx + x), pd = ldg2(a.prof + 2 * nx + x);
          const float ax0 = pa.x, ax1 = pa.y, bx0 = pb.x, bx1 = pb.y, dbx0 = pd.x, dbx1 = pd.y;
          const float opbx0 = 1.0f + bx0, opbx1 = 1.0f + bx1;
          const float2 P0 = lds2(Pc + c - 2), P1 = lds2(Pc + c), P2 = lds2(Pc + c + 2);
          const float2 Z = lds2(ZXr + c);
          const float d10 = ((F_D1A * (u1 - A.y)) - F_D1B * (B.x - A.x)) * a.rh;
          const float d11 = ((F_D1A * (B.x - u0)) - F_D1B * (B.y - A.y)) * a.rh;
          const float da0 = ((F_D1A * (P1.y - P0.y)) - F_D1B * (P2.x - P0.x)) * a.rh;
          const float da1 = ((F_D1A * (P2.x - P1.x)) - F_D1B * (P2.y - P0.y)) * a.rh;
          const float tmp0 = ((opbx0 * d2x0) + (dbx0 * d10)) + da0;
          const float tmp1 = ((opbx1 * d2x1) + (dbx1 * d11)) + da1;
          w0 = (opbx0 * tmp0) + (ax0 * Z.x);
          w1 = (opbx1 * tmp1) + (ax1 * Z.y);
          const float psi0 = (bx0 * d10) + P1.x;
          const float psi1 = (bx1 * d11) + P1.y;
          st2(ZXr + c, (bx0 * tmp0) + (ax0 * Z.x), (bx1 * tmp1) + (ax1 * Z.y));
          st2(Pn + c, ax0 * psi0, ax1 * psi1);
        } else {
          w0 = d2x0;
          w1 = d2x1;
        }
        const float2 zm2 = lds2(Uc + c - 2 * TB_RX), zm1 = lds2(Uc + c - TB_RX), zp1 = lds2(Uc + c + TB_RX),
                     zp2 = lds2(Uc + c + 2 * TB_RX);
        const float d2z0 = (((F_D2A * u0 + F_D2B * (zp1.x + zm1.x)) - F_D2C * (zp2.x + zm2.x)) * a.d2a) * a.d2b;
        const float d2z1 = (((F_D2A * u1 + F_D2B * (zp1.y + zm1.y)) - F_D2C * (zp2.y + zm2.y)) * a.d2a) * a.d2b;
        if (z < region || z >= nz - region) {
          const float az = __ldg(&a.prof[3 * nx + z]), bz = __ldg(&a.prof[3 * nx + nz + z]),
                      dbz = __ldg(&a.prof[3 * nx + 2 * nz + z]);
          const float opbz = 1.0f + bz;
          const float2 Qm2 = lds2(Qc + c - 2 * TB_RX), Qm1 = lds2(Qc + c - TB_RX), Q0 = lds2(Qc + c),
                       Qp1 = lds2(Qc + c + TB_RX), Qp2 = lds2(Qc + c + 2 * TB_RX);
          const float2 Z = lds2(ZZr + c);
          const float d10 = ((F_D1A * (zp1.x - zm1.x)) - F_D1B * (zp2.x - zm2.x)) * a.rh;
          const float d11 = ((F_D1A * (zp1.y - zm1.y)) - F_D1B * (zp2.y - zm2.y)) * a.rh;
          const float da0 = ((F_D1A * (Qp1.x - Qm1.x)) - F_D1B * (Qp2.x - Qm2.x)) * a.rh;
          const float da1 = ((F_D1A * (Qp1.y - Qm1.y)) - F_D1B * (Qp2.y - Qm2.y)) * a.rh;
          const float tmp0 = ((opbz * d2z0) + (dbz * d10)) + da0;
          const float tmp1 = ((opbz * d2z1) + (dbz * d11)) + da1;
          w0 = w0 + ((opbz * tmp0) + (az * Z.x));
          w1 = w1 + ((opbz * tmp1) + (az * Z.y));
          const float psi0 = (bz * d10) + Q0.x;
          const float psi1 = (bz * d11) + Q0.y;
          st2(ZZr + c, (bz * tmp0) + (az * Z.x), (bz * tmp1) + (az * Z.y));
          st2(Qn + c, az * psi0, az * psi1);
        } else {
          w0 = w0 + d2z0;
          w1 = w1 + d2z1;
        }
        const float2 v = lds2(V + c);
        const float v20 = (v.x * v.x) * a.dt2, v21 = (v.y * v.y) * a.dt2;
        const float2 prev = lds2(Un + c);
        float n0 = ((v20 * w0) + (2.0f * u0)) - prev.x;
        float n1 = ((v21 * w1) + (2.0f * u1)) - prev.y;
        if (STORE && lz >= TB_H && lz < TB_H + TZ_ && lx >= TB_H && lx < TB_H + TX_)
          __stcs(reinterpret_cast<float2*>(stp + cell),
                 make_float2(((2.0f * v.x) * a.dt2) * w0, ((2.0f * v.y) * a.dt2) * w1));
        // sources: corners in the halo are injected too, so that halo copies match their owners
        if (cell == sc0 || cell + 1 == sc0 || cell == sc1 || cell + 1 == sc1 || cell == sc2 || cell + 1 == sc2 ||
            cell == sc3 || cell + 1 == sc3) {
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const int scq = q == 0 ? sc0 : q == 1 ? sc1 : q == 2 ? sc2 : sc3;
            if (cell == scq) n0 = n0 + (((-v20) * __ldg(&sw[q])) * f);
            if (cell + 1 == scq) n1 = n1 + (((-v21) * __ldg(&sw[q])) * f);
          }
        }
        st2(Un + c, n0, n1);
      }
      __syncthreads();
    }
    // write back the tile: u(t + nsub), u(t + nsub - 1), and the strip cells' C-PML state
    const int ns = p.nsub;
    const float* Ucur = (ns & 1) ? UP : U;
    const float* Uold = (ns & 1) ? U : UP;
    float* W0 = p.W + (static_cast<size_t>(set_out * 2 + 0) * a.units + unit) * cells;
    float* W1 = p.W + (static_cast<size_t>(set_out * 2 + 1) * a.units + unit) * cells;
    for (int idx = tid; idx < TZ_ * (TX_ / 4); idx += TB_THREADS) {
      const int lz = idx / (TX_ / 4), lx4 = 4 * (idx % (TX_ / 4));
      const int z = z0 + lz, x = x0 + lx4;
      if (z >= nz || x >= nx) continue;  // nx is a multiple of 4
      const int c = (lz + TB_H) * TB_RX + lx4 + TB_H;
      *reinterpret_cast<float4*>(W0 + z * nx + x) = *reinterpret_cast<const float4*>(Ucur + c);
      *reinterpret_cast<float4*>(W1 + z * nx + x) = *reinterpret_cast<const float4*>(Uold + c);
    }
    if (pml_tile) {
      const float* Pcur = (ns & 1) ? PXB : PXA;
      const float* Qcur = (ns & 1) ? PZB : PZA;
      float* PXo = p.PX + (static_cast<size_t>(set_out) * a.units + unit) * xs_unit;
      float* ZXo = p.ZX + (static_cast<size_t>(set_out) * a.units + unit) * xs_unit;
      float* PZo = p.PZ + (static_cast<size_t>(set_out) * a.units + unit) * zs_unit;
      float* ZZo = p.ZZ + (static_cast<size_t>(set_out) * a.units + unit) * zs_unit;
      for (int idx = tid; idx < TZ_ * TX_; idx += TB_THREADS) {
        const int lz = idx / TX_, lx = idx % TX_;
        const int z = z0 + lz, x = x0 + lx;
        if (z >= nz || x >= nx) continue;
        const int c = (lz + TB_H) * TB_RX + lx + TB_H;
        if (x < ssw || x >= nx - ssw) {
          const int k = z * 2 * ssw + xstrip(x, nx, ssw);
          PXo[k] = Pcur[c];
          ZXo[k] = ZXr[c];
        }
        if (z < ssw || z >= nz - ssw) {
          const int k = (z < ssw ? z : z - (nz - 2 * ssw)) * nx + x;
          PZo[k] = Qcur[c];
          ZZo[k] = ZZr[c];
        }
      }
    }
    __syncthreads();  // this stage and the C-PML arrays are free again
  }
}

// ------------------------------------------------------------------------------------------------
// Adjoint step t (reverse time): lambda_next = w + 2 lambda - lambda_prev + injected residuals,
// gradient += lambda * stored term (+ the source-term correction), splatAdjoint.wgsl:58-131.
// Derived terms v^2 dt^2 lambda (VS) and, in the PML strips, T = (1+b) VS + b zeta and
// U1 = db T + b psi are formed once per tile cell (halo included) in shared memory.
// ------------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(NTH) adj_stream_kernel(const __grid_constant__ CUtensorMap map,
                                                         const __grid_constant__ SArgs a) {
  extern __shared__ __align__(128) float dsm_raw[];
  // TMA destinations start on a 128-byte boundary
  float* dsm = dsm_raw + ((128 - (smem_u32(dsm_raw) & 127)) & 127) / 4;
  float* stage = dsm;                      // [2][BZ*BX] lambda tiles (TMA)
  float* VS = dsm + 2 * BZ * BX;           // [BZ*BX]
  float* TXs = VS + BZ * BX;
  float* U1Xs = TXs + BZ * BX;
  float* TZs = U1Xs + BZ * BX;
  float* U1Zs = TZs + BZ * BX;
  uint64_t* bar = reinterpret_cast<uint64_t*>(U1Zs + BZ * BX);
  const int tid = threadIdx.x;
  const int tiles = a.tiles_x * a.tiles_z;
  const int jobs = a.units * tiles;
  const int q = a.t & 1;  // lambda(t) in buffer q; lambda(t-1) is written into buffer 1 - q
  const int nx = a.nx, nz = a.nz, ssw = a.ssw, region = a.region;
  const size_t cells = static_cast<size_t>(nx) * nz;
  const size_t xs_unit = static_cast<size_t>(nz) * 2 * ssw;
  const size_t zs_unit = static_cast<size_t>(2) * ssw * nx;
  Pipe pipe{bar, stage};
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  int job = blockIdx.x;
  if (tid == 0 && job < jobs) issue(a, &map, pipe, job, 0, q);
  const float f = __ldg(&a.wavelet[a.t]);
  const float* sAX = a.prof;
  const float* sBX = a.prof + nx;
  const float* sDBX = a.prof + 2 * nx;
  const float* sAZ = a.prof + 3 * nx;
  const float* sBZ = sAZ + nz;
  const float* sDBZ = sBZ + nz;
  const int pc = tid & 31, grp = tid >> 5;
  constexpr int DER = (BZ * (BX / 2) + NTH - 1) / NTH;  // derive pairs per thread
  for (int i = 0; job < jobs; ++i, job += gridDim.x) {
    const int s = i & 1;
    const int nxt = job + gridDim.x;
    if (tid == 0 && nxt < jobs) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      issue(a, &map, pipe, nxt, s ^ 1, q);
    }
    const int unit = job / tiles, tile = job % tiles;
    const int tzi = tile / a.tiles_x, txi = tile % a.tiles_x;
    const int x0 = txi * TX_, z0 = tzi * TZ_;
    const int model = unit / a.shots, shot = unit % a.shots;
    const float* vel = a.vel + static_cast<size_t>(model) * cells;
    const bool xtile = x0 - 2 < region + 3 || x0 + TX_ + 2 > nx - region - 3;
    const bool ztile = z0 - 2 < region + 2 || z0 + TZ_ + 2 > nz - region - 2;
    const float* LPXc = a.PX + (static_cast<size_t>(q) * a.units + unit) * xs_unit;
    const float* LZXc = a.ZX + (static_cast<size_t>(q) * a.units + unit) * xs_unit;
    const float* LPZc = a.PZ + (static_cast<size_t>(q) * a.units + unit) * zs_unit;
    const float* LZZc = a.ZZ + (static_cast<size_t>(q) * a.units + unit) * zs_unit;
    const int x = x0 + 2 * pc;
    const int zr = z0 + RPT * grp;
    const bool xok = x >= FD_PAD && x + 1 < nx - FD_PAD;
    float* Ln = a.W + (static_cast<size_t>(1 - q) * a.units + unit) * cells;
    const float* st_t = a.stored + (static_cast<size_t>(unit) * a.seg + (a.t - a.seg_t0)) * cells;
    float* gacc = a.gacc + static_cast<size_t>(unit) * cells;
    // inputs that do not depend on the tile copy, requested before it is waited for: the
    // velocity of the derive pairs, and per own cell lambda_prev, the stored term, the gradient
    float2 vd[DER];
#pragma unroll
    for (int d = 0; d < DER; ++d) {
      const int e = tid + d * NTH;
      const int k = e / (BX / 2), j = e % (BX / 2);
      const int z = z0 - HZ + k, xx = x0 - HX + 2 * j;
      const bool in = e < BZ * (BX / 2) && z >= 0 && z < nz && xx >= 0 && xx < nx;
      vd[d] = in ? ldg2(vel + static_cast<size_t>(z) * nx + xx) : make_float2(0.f, 0.f);
    }
    float2 lpv[RPT], stv[RPT], gav[RPT];
#pragma unroll
    for (int r = 0; r < RPT; ++r) {
      const int z = zr + r;
      const bool ok = xok && z >= FD_PAD && z < nz - FD_PAD;
      const int cell = (ok ? z : FD_PAD) * nx + (ok ? x : FD_PAD);
      lpv[r] = ld2(Ln + cell);
      stv[r] = __ldcs(reinterpret_cast<const float2*>(st_t + cell));
      gav[r] = ld2(gacc + cell);
    }
    // a wait that runs out (the copy never completed) ends the kernel in every thread together,
    // after thread 0 has waited, again bounded, for the copy it issued for the next tile
    if (__syncthreads_or(mbar_wait(&bar[s], (i >> 1) & 1) ? 0 : 1)) {
      if (tid == 0) {
        report(a.status);
        if (nxt < jobs) mbar_wait(&bar[s ^ 1], ((i + 1) >> 1) & 1);
      }
      return;
    }
    const float* L = stage + s * BZ * BX;

    if (interior_tile(a, x0, z0, a.st.src_cell + 4 * shot)) {
      // interior tile: VS over the tile and halo, then the interior update
#pragma unroll
      for (int d = 0; d < DER; ++d) {
        const int e = tid + d * NTH;
        if (e >= BZ * (BX / 2)) break;
        const int o = (e / (BX / 2)) * BX + 2 * (e % (BX / 2));
        const float2 l = lds2(L + o);
        st2(VS + o, ((vd[d].x * vd[d].x) * a.dt2) * l.x, ((vd[d].y * vd[d].y) * a.dt2) * l.y);
      }
      __syncthreads();
      const int sx = 2 * pc + HX, sz = RPT * grp + HZ;
      float* Lnf = a.W + (static_cast<size_t>(1 - q) * a.units + unit) * cells;
      float* gf = a.gacc + static_cast<size_t>(unit) * cells;
#pragma unroll
      for (int r = 0; r < RPT; ++r) {
        const int cell = (zr + r) * nx + x;
        const int so = (sz + r) * BX + sx;
        const float2 Vb = lds2(VS + so), Va = lds2(VS + so - 2), Vc = lds2(VS + so + 2);
        const float2 Vm2 = lds2(VS + so - 2 * BX), Vm1 = lds2(VS + so - BX), Vp1 = lds2(VS + so + BX),
                     Vp2 = lds2(VS + so + 2 * BX);
        float w0 = ((((F_D2A * Vb.x) + (F_D2B * (Vb.y + Va.y))) + (A_D2C * (Vc.x + Va.x))) * a.rh) * a.rh;
        float w1 = ((((F_D2A * Vb.y) + (F_D2B * (Vc.x + Vb.x))) + (A_D2C * (Vc.y + Va.y))) * a.rh) * a.rh;
        w0 = w0 + ((((F_D2A * Vb.x) + (F_D2B * (Vp1.x + Vm1.x))) + (A_D2C * (Vp2.x + Vm2.x))) * a.rh) * a.rh;
        w1 = w1 + ((((F_D2A * Vb.y) + (F_D2B * (Vp1.y + Vm1.y))) + (A_D2C * (Vp2.y + Vm2.y))) * a.rh) * a.rh;
        const float2 lc = lds2(L + so);
        const float n0 = (w0 + (2.0f * lc.x)) - lpv[r].x;
        const float n1 = (w1 + (2.0f * lc.y)) - lpv[r].y;
        const float g0 = 0.0f + ((lc.x * stv[r].x) * 1.0f);
        const float g1 = 0.0f + ((lc.y * stv[r].y) * 1.0f);
        st2(gf + cell, gav[r].x + g0, gav[r].y + g1);
        st2(Lnf + cell, n0, n1);
      }
      __syncthreads();  // stage and VS are reused by the next tile
      continue;
    }

    // derived terms over the tile and its halo (pairs of columns x0-4+2j, rows z0-2+k)
#pragma unroll
    for (int d = 0; d < DER; ++d) {
      const int e = tid + d * NTH;
      if (e >= BZ * (BX / 2)) break;
      const int k = e / (BX / 2), j = e % (BX / 2);
      const int z = z0 - HZ + k, x = x0 - HX + 2 * j;
      const int o = k * BX + 2 * j;
      float vs0 = 0.f, vs1 = 0.f;
      const bool in = z >= 0 && z < nz && x >= 0 && x < nx;
      if (in) {
        const float2 v = vd[d];
        const float2 l = lds2(L + o);
        vs0 = ((v.x * v.x) * a.dt2) * l.x;
        vs1 = ((v.y * v.y) * a.dt2) * l.y;
      }
      st2(VS + o, vs0, vs1);
      if (xtile && in && (x < ssw || x >= nx - ssw)) {
        const int xc = xstrip(x, nx, ssw);
        const float2 b = ldg2(sBX + x), db = ldg2(sDBX + x);
        const float2 Z = ld2(LZXc + static_cast<size_t>(z) * 2 * ssw + xc);
        const float2 P = ld2(LPXc + static_cast<size_t>(z) * 2 * ssw + xc);
        const float T0 = ((1.0f + b.x) * vs0) + (b.x * Z.x);
        const float T1 = ((1.0f + b.y) * vs1) + (b.y * Z.y);
        st2(TXs + o, T0, T1);
        st2(U1Xs + o, (db.x * T0) + (b.x * P.x), (db.y * T1) + (b.y * P.y));
      }
      if (ztile && in && (z < ssw || z >= nz - ssw)) {
        const int zc = z < ssw ? z : z - (nz - 2 * ssw);
        const float bz = __ldg(&sBZ[z]), dbz = __ldg(&sDBZ[z]);
        const float opbz = 1.0f + bz;
        const float2 Z = ld2(LZZc + static_cast<size_t>(zc) * nx + x);
        const float2 P = ld2(LPZc + static_cast<size_t>(zc) * nx + x);
        const float T0 = (opbz * vs0) + (bz * Z.x);
        const float T1 = (opbz * vs1) + (bz * Z.y);
        st2(TZs + o, T0, T1);
        st2(U1Zs + o, (dbz * T0) + (bz * P.x), (dbz * T1) + (bz * P.y));
      }
    }
    __syncthreads();

    const int sx = 2 * pc + HX, sz = RPT * grp + HZ;
    const bool xpml = x < region || x + 1 >= nx - region;
    const int* sc = a.st.src_cell + 4 * shot;
    const float* res_t = a.residual + (static_cast<size_t>(unit) * a.nt + a.t) * a.st.nrec;
    const bool rec_rows = zr + RPT > a.rec_z0 && zr <= a.rec_z1;
    unsigned srcm = 0;
    {
      const int base = zr * nx + x;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int d = __ldg(&sc[k]) - base;
#pragma unroll
        for (int r = 0; r < RPT; ++r) {
          const unsigned o = static_cast<unsigned>(d - r * nx);
          if (o < 2u) srcm |= 1u << (2 * r + o);
        }
      }
    }
    const int xc = xstrip(x, nx, ssw);
    float* LPXn = a.PX + (static_cast<size_t>(1 - q) * a.units + unit) * xs_unit;
    float* LZXn = a.ZX + (static_cast<size_t>(1 - q) * a.units + unit) * xs_unit;
    float* LPZn = a.PZ + (static_cast<size_t>(1 - q) * a.units + unit) * zs_unit;
    float* LZZn = a.ZZ + (static_cast<size_t>(1 - q) * a.units + unit) * zs_unit;
#pragma unroll
    for (int r = 0; r < RPT; ++r) {
      const int z = zr + r;
      if (!xok || z < FD_PAD || z >= nz - FD_PAD) continue;
      const int cell = z * nx + x;
      const int so = (sz + r) * BX + sx;
      const float2 Vb = lds2(VS + so);
      float w0, w1;
      if (xpml) {
        const float2 Ta = lds2(TXs + so - 2), Tb = lds2(TXs + so), Tc = lds2(TXs + so + 2);
        const float2 Ua = lds2(U1Xs + so - 2), Ub = lds2(U1Xs + so), Uc = lds2(U1Xs + so + 2);
        const float2 Ba = ldg2(sBX + x - 2), Bb = ldg2(sBX + x), Bc = ldg2(sBX + x + 2);
        const float q0 = (1.0f + Ba.x) * Ta.x, q1 = (1.0f + Ba.y) * Ta.y, q2 = (1.0f + Bb.x) * Tb.x,
                    q3 = (1.0f + Bb.y) * Tb.y, q4 = (1.0f + Bc.x) * Tc.x, q5 = (1.0f + Bc.y) * Tc.y;
        const float du0 = ((F_D1A * (Ub.y - Ua.y)) + (A_D1B * (Uc.x - Ua.x))) * a.rh;
        const float dd0 = ((((F_D2A * q2) + (F_D2B * (q3 + q1))) + (A_D2C * (q4 + q0))) * a.rh) * a.rh;
        const float dt0 = ((F_D1A * (Tb.y - Ta.y)) + (A_D1B * (Tc.x - Ta.x))) * a.rh;
        const float du1 = ((F_D1A * (Uc.x - Ub.x)) + (A_D1B * (Uc.y - Ua.y))) * a.rh;
        const float dd1 = ((((F_D2A * q3) + (F_D2B * (q4 + q2))) + (A_D2C * (q5 + q1))) * a.rh) * a.rh;
        const float dt1 = ((F_D1A * (Tc.x - Tb.x)) + (A_D1B * (Tc.y - Ta.y))) * a.rh;
        w0 = (-du0) + dd0;
        w1 = (-du1) + dd1;
        const int xo = z * 2 * ssw + xc;
        const float2 P = ld2(LPXc + xo), Z = ld2(LZXc + xo);
        const float2 ax = ldg2(sAX + x);
        st2(LPXn + xo, ((-ax.x) * dt0) + (ax.x * P.x), ((-ax.y) * dt1) + (ax.y * P.y));
        st2(LZXn + xo, (ax.x * Vb.x) + (ax.x * Z.x), (ax.y * Vb.y) + (ax.y * Z.y));
      } else {
        const float2 Va = lds2(VS + so - 2), Vc = lds2(VS + so + 2);
        w0 = ((((F_D2A * Vb.x) + (F_D2B * (Vb.y + Va.y))) + (A_D2C * (Vc.x + Va.x))) * a.rh) * a.rh;
        w1 = ((((F_D2A * Vb.y) + (F_D2B * (Vc.x + Vb.x))) + (A_D2C * (Vc.y + Va.y))) * a.rh) * a.rh;
      }
      if (z < region || z >= nz - region) {
        const float2 Tm2 = lds2(TZs + so - 2 * BX), Tm1 = lds2(TZs + so - BX), T0 = lds2(TZs + so),
                     Tp1 = lds2(TZs + so + BX), Tp2 = lds2(TZs + so + 2 * BX);
        const float2 Um2 = lds2(U1Zs + so - 2 * BX), Um1 = lds2(U1Zs + so - BX), Up1 = lds2(U1Zs + so + BX),
                     Up2 = lds2(U1Zs + so + 2 * BX);
        const float om2 = 1.0f + __ldg(&sBZ[z - 2]), om1 = 1.0f + __ldg(&sBZ[z - 1]), o0 = 1.0f + __ldg(&sBZ[z]),
                    op1 = 1.0f + __ldg(&sBZ[z + 1]), op2 = 1.0f + __ldg(&sBZ[z + 2]);
        const float du0 = ((F_D1A * (Up1.x - Um1.x)) + (A_D1B * (Up2.x - Um2.x))) * a.rh;
        const float du1 = ((F_D1A * (Up1.y - Um1.y)) + (A_D1B * (Up2.y - Um2.y))) * a.rh;
        const float dd0 = ((((F_D2A * (o0 * T0.x)) + (F_D2B * ((op1 * Tp1.x) + (om1 * Tm1.x)))) +
                            (A_D2C * ((op2 * Tp2.x) + (om2 * Tm2.x)))) * a.rh) * a.rh;
        const float dd1 = ((((F_D2A * (o0 * T0.y)) + (F_D2B * ((op1 * Tp1.y) + (om1 * Tm1.y)))) +
                            (A_D2C * ((op2 * Tp2.y) + (om2 * Tm2.y)))) * a.rh) * a.rh;
        const float dt0 = ((F_D1A * (Tp1.x - Tm1.x)) + (A_D1B * (Tp2.x - Tm2.x))) * a.rh;
        const float dt1 = ((F_D1A * (Tp1.y - Tm1.y)) + (A_D1B * (Tp2.y - Tm2.y))) * a.rh;
        w0 = w0 + ((-du0) + dd0);
        w1 = w1 + ((-du1) + dd1);
        const int zc = z < ssw ? z : z - (nz - 2 * ssw);
        const int zo = zc * nx + x;
        const float az = __ldg(&sAZ[z]);
        const float2 P = ld2(LPZc + zo), Z = ld2(LZZc + zo);
        st2(LPZn + zo, ((-az) * dt0) + (az * P.x), ((-az) * dt1) + (az * P.y));
        st2(LZZn + zo, (az * Vb.x) + (az * Z.x), (az * Vb.y) + (az * Z.y));
      } else {
        const float2 Vm2 = lds2(VS + so - 2 * BX), Vm1 = lds2(VS + so - BX), Vp1 = lds2(VS + so + BX),
                     Vp2 = lds2(VS + so + 2 * BX);
        w0 = w0 + ((((F_D2A * Vb.x) + (F_D2B * (Vp1.x + Vm1.x))) + (A_D2C * (Vp2.x + Vm2.x))) * a.rh) * a.rh;
        w1 = w1 + ((((F_D2A * Vb.y) + (F_D2B * (Vp1.y + Vm1.y))) + (A_D2C * (Vp2.y + Vm2.y))) * a.rh) * a.rh;
      }
      const float2 lc = lds2(L + so);
      const float2 lp = lpv[r];
      float n0 = (w0 + (2.0f * lc.x)) - lp.x;
      float n1 = (w1 + (2.0f * lc.y)) - lp.y;
      const float2 sv = stv[r];
      float g0 = 0.0f + ((lc.x * sv.x) * 1.0f);
      float g1 = 0.0f + ((lc.y * sv.y) * 1.0f);
      if (rec_rows) {
        const int e0 = a.st.csr[cell], e1 = a.st.csr[cell + 1], e2 = a.st.csr[cell + 2];
        for (int e = e0; e < e1; ++e) n0 = n0 + (a.st.ent_w[e] * res_t[a.st.ent_rec[e]]);
        for (int e = e1; e < e2; ++e) n1 = n1 + (a.st.ent_w[e] * res_t[a.st.ent_rec[e]]);
      }
      const int ci = cell;
      if (srcm & (3u << (2 * r))) {
        const float2 v = ldg2(vel + cell);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const float wk = a.st.src_w[4 * shot + k];
          if (ci == sc[k]) g0 = g0 + lc.x * (((((-2.0f) * v.x) * a.dt2) * wk) * f);
          if (ci + 1 == sc[k]) g1 = g1 + lc.y * (((((-2.0f) * v.y) * a.dt2) * wk) * f);
        }
      }
      st2(gacc + cell, gav[r].x + g0, gav[r].y + g1);
      st2(Ln + cell, n0, n1);
    }
    __syncthreads();  // stage and derived arrays are reused by the next tile
  }
}

// ------------------------------------------------------------------------------------------------
// host side
// ------------------------------------------------------------------------------------------------

struct Buf {
  void* p = nullptr;
  size_t bytes = 0;
  ~Buf() {
    if (p) cudaFree(p);
  }
  cudaError_t ensure(size_t need) {
    if (need <= bytes) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
    cudaError_t e = cudaMalloc(&p, std::max<size_t>(need, 256));
    if (e != cudaSuccess) {
      cudaGetLastError();
      p = nullptr;
      return e;
    }
    bytes = need;
    return cudaSuccess;
  }
  float* f() const { return static_cast<float*>(p); }
};

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

// Tensor map over [2 * units][nz][nx] floats with a 72 x 36 x 1 box; out-of-range elements read 0.
int make_map(CUtensorMap* m, const float* base, int nx, int nz, int depth, int box_x = BX, int box_z = BZ) {
  auto fn = encode_fn();
  if (!fn) return report_error(WG_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
  const cuuint64_t dims[3] = {static_cast<cuuint64_t>(nx), static_cast<cuuint64_t>(nz),
                              static_cast<cuuint64_t>(depth)};
  const cuuint64_t strides[2] = {static_cast<cuuint64_t>(nx) * 4, static_cast<cuuint64_t>(nx) * nz * 4};
  const cuuint32_t box[3] = {static_cast<cuuint32_t>(box_x), static_cast<cuuint32_t>(box_z), 1};
  const cuuint32_t es[3] = {1, 1, 1};
  CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(base), dims, strides, box, es,
                  CU_TENSOR_MAP_INTERLEAVE_NONE,
                  CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return report_error(WG_ERR_CUDA, ("cuTensorMapEncodeTiled failed: " + std::to_string(r)).c_str());
  return WG_OK;
}

// Forward maps: the wavefield pair with and without halo, and the models' velocity.
int make_fwd_maps(FwdMaps* m, const float* W, const float* vel, int nx, int nz, int units, int models) {
  int rc = make_map(&m->u, W, nx, nz, 2 * units);
  if (rc == WG_OK) rc = make_map(&m->p, W, nx, nz, 2 * units, TX_, TZ_);
  if (rc == WG_OK) rc = make_map(&m->v, vel, nx, nz, models, TX_, TZ_);
  return rc;
}

constexpr size_t kAdjSmem = (7 * BZ * BX) * 4 + 16 + 128;

// Self-test of the time-out path: the kernels' bounded wait on an mbarrier that expects 16 bytes
// of a copy that is never issued. The wait gives up after `polls` polls, the CTA records ST_CUDA
// in `status` and the kernel returns (no copy is in flight, so there is nothing to drain).
__global__ void wait_timeout_probe_kernel(int* status, long polls) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0) mbar_expect_tx(&bar, 16);  // the arrival; the 16 bytes never land
  __syncthreads();
  if (__syncthreads_or(mbar_wait(&bar, 0, polls) ? 0 : 1) && threadIdx.x == 0) report(status);
}

}  // namespace

int wait_timeout_selftest(int* d_status, long long polls, cudaStream_t st) {
  wait_timeout_probe_kernel<<<1, 64, 0, st>>>(d_status, static_cast<long>(polls));
  return cudaGetLastError() == cudaSuccess ? WG_OK : report_error(WG_ERR_CUDA, "wait self-test launch failed");
}

struct StreamWork {
  Buf vpad, mask, traces, energy, scale, stored, ckpt, gacc;
  Buf W, PX, ZX, PZ, ZZ;        // forward state
  Buf Wtb, PXtb, ZXtb, PZtb, ZZtb;  // temporally blocked forward: two state sets
  Buf L, LPX, LZX, LPZ, LZZ;    // adjoint state
  Buf tile_rec_start, tile_rec;
  int rec_tiles_nx = -1, rec_tiles_nz = -1, rec_z0 = 0, rec_z1 = -1;
  int fwd_blocks = 0, adj_blocks = 0, tb_blocks = 0, sms = 0;
};

StreamWork* stream_work_new() { return new StreamWork(); }
void stream_work_free(StreamWork* w) { delete w; }

namespace {

#define SW_CK(expr)                                                                                     \
  do {                                                                                                  \
    cudaError_t e_ = (expr);                                                                            \
    if (e_ != cudaSuccess) {                                                                            \
      cudaGetLastError();                                                                               \
      return report_error(e_ == cudaErrorMemoryAllocation ? WG_ERR_OOM : WG_ERR_CUDA,                   \
                          (std::string(#expr) + ": " + cudaGetErrorString(e_)).c_str());               \
    }                                                                                                   \
  } while (0)

int strip_width(const EngineView& v) { return ((v.grid.region_adj + 3) + 1) & ~1; }

// Receivers recorded by each tile: the tile that holds a receiver's first corner.
int setup_receivers(StreamWork* w, const EngineView& v, const int* h_rec_cell) {
  const int tx = (v.nx + TX_ - 1) / TX_, tz = (v.nz + TZ_ - 1) / TZ_;
  if (w->rec_tiles_nx == tx && w->rec_tiles_nz == tz) return WG_OK;
  std::vector<int> start(tx * tz + 1, 0), list(v.nrec);
  std::vector<int> tile_of(v.nrec);
  int z0 = v.nz, z1 = -1;
  for (int r = 0; r < v.nrec; ++r) {
    const int c = h_rec_cell[4 * r];
    const int cz = c / v.nx, cx = c % v.nx;
    tile_of[r] = (cz / TZ_) * tx + cx / TX_;
    ++start[tile_of[r] + 1];
    for (int k = 0; k < 4; ++k) {
      const int zz = h_rec_cell[4 * r + k] / v.nx;
      z0 = std::min(z0, zz);
      z1 = std::max(z1, zz);
    }
  }
  for (int t = 0; t < tx * tz; ++t) start[t + 1] += start[t];
  std::vector<int> fill(start.begin(), start.end() - 1);
  for (int r = 0; r < v.nrec; ++r) list[fill[tile_of[r]]++] = r;
  SW_CK(w->tile_rec_start.ensure(start.size() * 4));
  SW_CK(w->tile_rec.ensure(std::max<size_t>(list.size(), 1) * 4));
  SW_CK(cudaMemcpy(w->tile_rec_start.p, start.data(), start.size() * 4, cudaMemcpyHostToDevice));
  if (!list.empty()) SW_CK(cudaMemcpy(w->tile_rec.p, list.data(), list.size() * 4, cudaMemcpyHostToDevice));
  w->rec_tiles_nx = tx;
  w->rec_tiles_nz = tz;
  w->rec_z0 = z0;
  w->rec_z1 = z1;
  return WG_OK;
}

int occupancy(StreamWork* w) {
  if (w->sms) return WG_OK;
  int dev = 0, sms = 0, fb = 0, ab = 0;
  SW_CK(cudaGetDevice(&dev));
  SW_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  SW_CK(cudaFuncSetAttribute(adj_stream_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(kAdjSmem)));
  SW_CK(cudaFuncSetAttribute(fwd_stream_kernel<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             static_cast<int>(kFwdSmem)));
  SW_CK(cudaFuncSetAttribute(fwd_stream_kernel<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             static_cast<int>(kFwdSmem)));
  SW_CK(cudaFuncSetAttribute(fwd_stream_kernel<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             static_cast<int>(kFwdSmem)));
  SW_CK(cudaFuncSetAttribute(fwd_tb_kernel<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             static_cast<int>(kTbSmem)));
  SW_CK(cudaFuncSetAttribute(fwd_tb_kernel<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             static_cast<int>(kTbSmem)));
  SW_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fb, fwd_stream_kernel<true, true>, FWD_THREADS, kFwdSmem));
  SW_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ab, adj_stream_kernel, NTH, kAdjSmem));
  int tb = 0;
  SW_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&tb, fwd_tb_kernel<true, true>, TB_THREADS, kTbSmem));
  w->sms = sms;
  w->fwd_blocks = sms * std::max(fb, 1);
  w->adj_blocks = sms * std::max(ab, 1);
  w->tb_blocks = sms * std::max(tb, 1);
  return WG_OK;
}

SArgs base_args(StreamWork* w, const EngineView& v, int units) {
  SArgs a{};
  a.nx = v.nx;
  a.nz = v.nz;
  a.units = units;
  a.shots = v.shots;
  a.tiles_x = (v.nx + TX_ - 1) / TX_;
  a.tiles_z = (v.nz + TZ_ - 1) / TZ_;
  a.ssw = strip_width(v);
  a.region = v.grid.region_adj;
  a.nt = v.nt;
  a.rh = v.grid.rh;
  a.dt2 = v.grid.dt2;
  a.d2a = v.grid.d2a;
  a.d2b = v.grid.d2b;
  a.prof = v.grid.prof;
  a.wavelet = v.grid.wavelet;
  a.st = v.stations;
  a.rec_z0 = w->rec_z0;
  a.rec_z1 = w->rec_z1;
  a.tile_rec_start = static_cast<const int*>(w->tile_rec_start.p);
  a.tile_rec = static_cast<const int*>(w->tile_rec.p);
  a.status = v.d_status;
  return a;
}

size_t xs_floats(const EngineView& v) { return static_cast<size_t>(v.nz) * 2 * strip_width(v); }
size_t zs_floats(const EngineView& v) { return static_cast<size_t>(2) * strip_width(v) * v.nx; }

// Forward state buffers (zeroed) for `units` units.
int alloc_forward(StreamWork* w, const EngineView& v, int units, cudaStream_t st) {
  const size_t cells = static_cast<size_t>(v.nx) * v.nz;
  SW_CK(w->W.ensure(2 * units * cells * 4));
  SW_CK(w->PX.ensure(2 * units * xs_floats(v) * 4));
  SW_CK(w->ZX.ensure(units * xs_floats(v) * 4));
  SW_CK(w->PZ.ensure(2 * units * zs_floats(v) * 4));
  SW_CK(w->ZZ.ensure(units * zs_floats(v) * 4));
  SW_CK(cudaMemsetAsync(w->W.p, 0, 2 * units * cells * 4, st));
  SW_CK(cudaMemsetAsync(w->PX.p, 0, 2 * units * xs_floats(v) * 4, st));
  SW_CK(cudaMemsetAsync(w->ZX.p, 0, units * xs_floats(v) * 4, st));
  SW_CK(cudaMemsetAsync(w->PZ.p, 0, 2 * units * zs_floats(v) * 4, st));
  SW_CK(cudaMemsetAsync(w->ZZ.p, 0, units * zs_floats(v) * 4, st));
  return WG_OK;
}

// One forward step over all units.
int fwd_step(StreamWork* w, const FwdMaps& map, SArgs a, int t, bool traces, bool store, cudaStream_t st) {
  a.t = t;
  const int jobs = a.units * a.tiles_x * a.tiles_z;
  const int blocks = std::min(jobs, w->fwd_blocks);
  note_launch();
  if (traces && store)
    fwd_stream_kernel<true, true><<<blocks, FWD_THREADS, kFwdSmem, st>>>(map, a);
  else if (traces)
    fwd_stream_kernel<true, false><<<blocks, FWD_THREADS, kFwdSmem, st>>>(map, a);
  else
    fwd_stream_kernel<false, true><<<blocks, FWD_THREADS, kFwdSmem, st>>>(map, a);
  SW_CK(cudaGetLastError());
  return WG_OK;
}

int adj_step(StreamWork* w, const CUtensorMap& map, SArgs a, int t, cudaStream_t st) {
  a.t = t;
  const int jobs = a.units * a.tiles_x * a.tiles_z;
  const int blocks = std::min(jobs, w->adj_blocks);
  note_launch();
  adj_stream_kernel<<<blocks, NTH, kAdjSmem, st>>>(map, a);
  SW_CK(cudaGetLastError());
  return WG_OK;
}

// Temporally blocked forward over all units from the zero state, TB_T steps per launch: receivers
// into `traces` and, when `stored` is given, every step's gradient term (the store-all scheme).
int tb_forward(StreamWork* w, const EngineView& v, int units, int models, float* traces, float* stored,
               cudaStream_t st) {
  const size_t cells = static_cast<size_t>(v.nx) * v.nz;
  const size_t nW = static_cast<size_t>(units) * cells, nX = units * xs_floats(v), nZ = units * zs_floats(v);
  SW_CK(w->Wtb.ensure(4 * nW * 4));
  SW_CK(w->PXtb.ensure(2 * nX * 4));
  SW_CK(w->ZXtb.ensure(2 * nX * 4));
  SW_CK(w->PZtb.ensure(2 * nZ * 4));
  SW_CK(w->ZZtb.ensure(2 * nZ * 4));
  SW_CK(cudaMemsetAsync(w->Wtb.p, 0, 4 * nW * 4, st));
  SW_CK(cudaMemsetAsync(w->PXtb.p, 0, 2 * nX * 4, st));
  SW_CK(cudaMemsetAsync(w->ZXtb.p, 0, 2 * nX * 4, st));
  SW_CK(cudaMemsetAsync(w->PZtb.p, 0, 2 * nZ * 4, st));
  SW_CK(cudaMemsetAsync(w->ZZtb.p, 0, 2 * nZ * 4, st));
  CUtensorMap um, vm;
  int rc = make_map(&um, w->Wtb.f(), v.nx, v.nz, 4 * units, TB_RX, TB_RZ);
  if (rc == WG_OK) rc = make_map(&vm, w->vpad.f(), v.nx, v.nz, models, TB_RX, TB_RZ);
  if (rc != WG_OK) return rc;
  TbArgs p{};
  p.a = base_args(w, v, units);
  p.a.vel = w->vpad.f();
  p.a.traces = traces;
  p.a.stored = stored;
  p.a.seg = v.nt;
  p.a.seg_t0 = 0;
  p.W = w->Wtb.f();
  p.PX = w->PXtb.f();
  p.ZX = w->ZXtb.f();
  p.PZ = w->PZtb.f();
  p.ZZ = w->ZZtb.f();
  const int jobs = units * p.a.tiles_x * p.a.tiles_z;
  const int blocks = std::min(jobs, w->tb_blocks);
  for (int t = 0, k = 0; t < v.nt; t += TB_T, ++k) {
    p.a.t = t;
    p.nsub = std::min(TB_T, v.nt - t);
    p.set_in = k & 1;
    note_launch();
    if (stored)
      fwd_tb_kernel<true, true><<<blocks, TB_THREADS, kTbSmem, st>>>(um, vm, p);
    else
      fwd_tb_kernel<true, false><<<blocks, TB_THREADS, kTbSmem, st>>>(um, vm, p);
    SW_CK(cudaGetLastError());
  }
  return WG_OK;
}

// Checkpoint slot layout: [W(t) | W(t-1) | PX(t) | ZX | PZ(t) | ZZ] for all units.
size_t ckpt_slot_floats(const EngineView& v, int units) {
  const size_t cells = static_cast<size_t>(v.nx) * v.nz;
  return static_cast<size_t>(units) * (2 * cells + 2 * xs_floats(v) + 2 * zs_floats(v));
}

// Copy the forward state at the start of step t into (save) or out of (!save) a checkpoint slot.
int ckpt_copy(StreamWork* w, const EngineView& v, int units, int t, float* slot, bool save, cudaStream_t st) {
  const size_t cells = static_cast<size_t>(v.nx) * v.nz;
  const int par = t & 1;
  const size_t nW = units * cells, nX = units * xs_floats(v), nZ = units * zs_floats(v);
  float* parts[6] = {w->W.f() + par * nW, w->W.f() + (1 - par) * nW, w->PX.f() + par * nX, w->ZX.f(),
                     w->PZ.f() + par * nZ, w->ZZ.f()};
  const size_t sizes[6] = {nW, nW, nX, nX, nZ, nZ};
  size_t off = 0;
  for (int k = 0; k < 6; ++k) {
    float* dst = save ? slot + off : parts[k];
    const float* src = save ? parts[k] : slot + off;
    SW_CK(cudaMemcpyAsync(dst, src, sizes[k] * 4, cudaMemcpyDeviceToDevice, st));
    off += sizes[k];
  }
  return WG_OK;
}

}  // namespace

bool stream_supported(const EngineView& v, std::string* why) {
  if (v.nx % 4 != 0) {
    if (why) *why = "the streamed path needs a padded width divisible by 4 (nx_vis + 2 (pml + 2))";
    return false;
  }
  if (v.nx < 2 * strip_width(v) || v.nz < 2 * strip_width(v)) {
    if (why) *why = "grid too small for the streamed path's PML strips";
    return false;
  }
  return true;
}

int stream_simulate(StreamWork* w, const EngineView& v, const int* h_rec_cell, const float* d_vis, int models,
                    float* d_traces, cudaStream_t st, const StreamTimer& timer) {
  std::string why;
  if (!stream_supported(v, &why)) return report_error(WG_ERR_UNSUPPORTED, why.c_str());
  int rc = setup_receivers(w, v, h_rec_cell);
  if (rc != WG_OK) return rc;
  if ((rc = occupancy(w)) != WG_OK) return rc;
  const size_t cells = static_cast<size_t>(v.nx) * v.nz;
  const int units = models * v.shots;
  SW_CK(w->vpad.ensure(models * cells * 4));
  note_launch();
  SW_CK(launch_pad_velocity(d_vis, models, v.nx_vis, v.nz_vis, v.pad, v.vmin, v.vmax, w->vpad.f(), nullptr, st));
  if (v.tblock) {
    timer.mark(0, true, st);
    if ((rc = tb_forward(w, v, units, models, d_traces, nullptr, st)) != WG_OK) return rc;
    timer.mark(0, false, st);
    return WG_OK;
  }
  if ((rc = alloc_forward(w, v, units, st)) != WG_OK) return rc;
  FwdMaps map;
  if ((rc = make_fwd_maps(&map, w->W.f(), w->vpad.f(), v.nx, v.nz, units, models)) != WG_OK) return rc;
  SArgs a = base_args(w, v, units);
  a.vel = w->vpad.f();
  a.W = w->W.f();
  a.PX = w->PX.f();
  a.ZX = w->ZX.f();
  a.PZ = w->PZ.f();
  a.ZZ = w->ZZ.f();
  a.traces = d_traces;
  timer.mark(0, true, st);
  for (int t = 0; t < v.nt; ++t)
    if ((rc = fwd_step(w, map, a, t, true, false, st)) != WG_OK) return rc;
  timer.mark(0, false, st);
  return WG_OK;
}

int stream_gradient(StreamWork* w, const EngineView& v, const int* h_rec_cell, const float* d_vis, const float* d_obs,
                    int models, double* d_loss, float* d_grad, cudaStream_t st, const StreamTimer& timer) {
  std::string why;
  if (!stream_supported(v, &why)) return report_error(WG_ERR_UNSUPPORTED, why.c_str());
  int rc = setup_receivers(w, v, h_rec_cell);
  if (rc != WG_OK) return rc;
  if ((rc = occupancy(w)) != WG_OK) return rc;
  const size_t cells = static_cast<size_t>(v.nx) * v.nz;
  const int units = models * v.shots;
  const size_t tr = static_cast<size_t>(v.nt) * v.nrec;
  SW_CK(w->vpad.ensure(models * cells * 4));
  SW_CK(w->mask.ensure(models * cells * 4));
  SW_CK(w->traces.ensure(units * tr * 4));
  SW_CK(w->energy.ensure(models * 8));
  SW_CK(w->scale.ensure(models * 4));
  SW_CK(w->gacc.ensure(units * cells * 4));
  note_launch();
  SW_CK(launch_pad_velocity(d_vis, models, v.nx_vis, v.nz_vis, v.pad, v.vmin, v.vmax, w->vpad.f(), w->mask.f(), st));
  note_launch();
  SW_CK(launch_energy(d_obs, models, v.shots * tr, static_cast<double*>(w->energy.p), w->scale.f(), v.d_status, st));
  if ((rc = alloc_forward(w, v, units, st)) != WG_OK) return rc;

  // Segment length: store every step's gradient terms when they fit in 70% of the free memory,
  // else checkpoints every k steps with k chosen (or given) so that one segment plus the
  // checkpoints fit.
  const size_t step_bytes = units * cells * 4;
  const size_t slot_bytes = ckpt_slot_floats(v, units) * 4;
  size_t free_b = 0, total_b = 0;
  SW_CK(cudaMemGetInfo(&free_b, &total_b));
  const size_t budget = free_b / 10 * 7 + w->stored.bytes + w->ckpt.bytes;
  int k = v.ck_every;
  if (k <= 0) {
    if (static_cast<size_t>(v.nt) * step_bytes <= budget) {
      k = v.nt;
    } else {
      k = 1;
      while (k < v.nt && (static_cast<size_t>(k) * step_bytes +
                          static_cast<size_t>((v.nt + k - 1) / k - 1) * slot_bytes) > budget) ++k;
      // prefer the smallest total memory among k that fit: sqrt balance
      int best = k;
      size_t best_mem = SIZE_MAX;
      for (int kk = k; kk <= std::min(v.nt, 4 * k + 64); ++kk) {
        const size_t mem = kk * step_bytes + static_cast<size_t>((v.nt + kk - 1) / kk - 1) * slot_bytes;
        if (mem <= budget && mem < best_mem) {
          best_mem = mem;
          best = kk;
        }
      }
      k = best;
    }
  }
  k = std::min(k, v.nt);
  const bool store_all = k >= v.nt;
  const int J = (v.nt + k - 1) / k;
  const int seg = store_all ? v.nt : k;
  SW_CK(w->stored.ensure(static_cast<size_t>(seg) * step_bytes));
  if (J > 1) SW_CK(w->ckpt.ensure(static_cast<size_t>(J - 1) * slot_bytes));

  FwdMaps fmap;
  if ((rc = make_fwd_maps(&fmap, w->W.f(), w->vpad.f(), v.nx, v.nz, units, models)) != WG_OK) return rc;
  SArgs f = base_args(w, v, units);
  f.vel = w->vpad.f();
  f.W = w->W.f();
  f.PX = w->PX.f();
  f.ZX = w->ZX.f();
  f.PZ = w->PZ.f();
  f.ZZ = w->ZZ.f();
  f.traces = w->traces.f();
  f.stored = w->stored.f();
  f.seg = seg;
  f.seg_t0 = 0;
  timer.mark(0, true, st);
  if (store_all && v.tblock) {
    if ((rc = tb_forward(w, v, units, models, w->traces.f(), w->stored.f(), st)) != WG_OK) return rc;
  } else {
    for (int t = 0; t < v.nt; ++t) {
      if (!store_all && t > 0 && t % k == 0)
        if ((rc = ckpt_copy(w, v, units, t, w->ckpt.f() + (t / k - 1) * (slot_bytes / 4), true, st)) != WG_OK)
          return rc;
      if ((rc = fwd_step(w, fmap, f, t, true, store_all, st)) != WG_OK) return rc;
    }
  }
  timer.mark(0, false, st);
  note_launch();
  SW_CK(launch_residual(w->traces.f(), d_obs, w->scale.f(), models, v.shots * tr, w->traces.f(), d_loss, st));

  // adjoint state
  const size_t xsf = xs_floats(v), zsf = zs_floats(v);
  SW_CK(w->L.ensure(2 * units * cells * 4));
  SW_CK(w->LPX.ensure(2 * units * xsf * 4));
  SW_CK(w->LZX.ensure(2 * units * xsf * 4));
  SW_CK(w->LPZ.ensure(2 * units * zsf * 4));
  SW_CK(w->LZZ.ensure(2 * units * zsf * 4));
  SW_CK(cudaMemsetAsync(w->L.p, 0, 2 * units * cells * 4, st));
  SW_CK(cudaMemsetAsync(w->LPX.p, 0, 2 * units * xsf * 4, st));
  SW_CK(cudaMemsetAsync(w->LZX.p, 0, 2 * units * xsf * 4, st));
  SW_CK(cudaMemsetAsync(w->LPZ.p, 0, 2 * units * zsf * 4, st));
  SW_CK(cudaMemsetAsync(w->LZZ.p, 0, 2 * units * zsf * 4, st));
  SW_CK(cudaMemsetAsync(w->gacc.p, 0, units * cells * 4, st));
  CUtensorMap amap;
  if ((rc = make_map(&amap, w->L.f(), v.nx, v.nz, 2 * units)) != WG_OK) return rc;
  SArgs b = base_args(w, v, units);
  b.vel = w->vpad.f();
  b.W = w->L.f();
  b.PX = w->LPX.f();
  b.ZX = w->LZX.f();
  b.PZ = w->LPZ.f();
  b.ZZ = w->LZZ.f();
  b.residual = w->traces.f();
  b.stored = w->stored.f();
  b.seg = seg;
  b.gacc = w->gacc.f();
  for (int j = J - 1; j >= 0; --j) {
    const int t0 = store_all ? 0 : j * k, t1 = store_all ? v.nt : std::min(v.nt, t0 + k);
    if (!store_all) {
      timer.mark(1, true, st);
      if (j > 0) {
        if ((rc = ckpt_copy(w, v, units, t0, w->ckpt.f() + (j - 1) * (slot_bytes / 4), false, st)) != WG_OK) return rc;
      } else if ((rc = alloc_forward(w, v, units, st)) != WG_OK) {
        return rc;
      }
      f.seg_t0 = t0;
      for (int t = t0; t < t1; ++t)
        if ((rc = fwd_step(w, fmap, f, t, false, true, st)) != WG_OK) return rc;
      timer.mark(1, false, st);
    }
    b.seg_t0 = t0;
    timer.mark(2, true, st);
    for (int t = t1 - 1; t >= t0; --t)
      if ((rc = adj_step(w, amap, b, t, st)) != WG_OK) return rc;
    timer.mark(2, false, st);
  }
  note_launch();
  SW_CK(launch_fold(w->gacc.f(), w->mask.f(), models, v.shots, v.nx, v.nz, v.pad, v.nx_vis, v.nz_vis, d_grad, st));
  return WG_OK;
}

}  // namespace wg
