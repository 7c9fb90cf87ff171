// Device helpers for the resident kernels: cluster rank/barrier, DSMEM stores, shared-memory
// layouts shared by host (sizing) and device (addressing).
#pragma once

#include <cuda_runtime.h>

#include "wave_common.cuh"

namespace wg {

__device__ __forceinline__ unsigned cluster_rank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}

// Full cluster barrier: arrive with release semantics, wait with acquire semantics, so that
// shared-memory stores into peer CTAs before the barrier are visible after it.
__device__ __forceinline__ void cluster_barrier() {
  asm volatile(
      "barrier.cluster.arrive.release.aligned;\n\t"
      "barrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// Store one float into the same shared-memory offset of CTA `peer` of this cluster.
__device__ __forceinline__ void st_peer(const float* local_ptr, unsigned peer, float v) {
  unsigned la = static_cast<unsigned>(__cvta_generic_to_shared(local_ptr));
  unsigned ra;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(ra) : "r"(la), "r"(peer));
  asm volatile("st.shared::cluster.f32 [%0], %1;" ::"r"(ra), "f"(v) : "memory");
}

// Split cluster barrier. Threads that stored into a peer CTA's shared memory since the last barrier
// fence first (cluster scope), so the relaxed arrive that follows publishes their stores to the
// peers' acquiring wait; independent work can run between arrive and wait.
__device__ __forceinline__ void fence_cluster() { asm volatile("fence.acq_rel.cluster;" ::: "memory"); }
__device__ __forceinline__ void cluster_arrive_relaxed() {
  asm volatile("barrier.cluster.arrive.relaxed.aligned;" ::: "memory");
}
__device__ __forceinline__ void cluster_wait_acquire() {
  asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
}

template <int C>
__device__ __forceinline__ void step_barrier() {
  if constexpr (C == 1) {
    __syncthreads();
  } else {
    cluster_barrier();
  }
}

// Rows [2, nz-2) are split over the C CTAs of a cluster; CTA `rank` updates rows [r0, r1).
__host__ __device__ inline int split_row(int nz, int C, int rank) {
  const int upd = nz - 2 * FD_PAD;
  return FD_PAD + (upd * rank) / C;
}

__host__ __device__ inline int max_rows(int nz, int C) {
  const int upd = nz - 2 * FD_PAD;
  return (upd + C - 1) / C;
}

// Forward shared-memory layout, in floats. Arrays are identical in every CTA of the cluster so
// that a peer's copy of an array sits at the same offset.
struct FwdLayout {
  int maxrows, lr, zs;
  int off_u, off_apx, off_apz, off_prof, off_rec, total;
};

__host__ __device__ inline FwdLayout fwd_layout(int nx, int nz, int sw, int C, int nrec) {
  FwdLayout L;
  L.maxrows = max_rows(nz, C);
  L.lr = L.maxrows + 2 * FD_PAD;
  L.zs = (C == 1 ? 2 : 1) * sw;
  L.off_u = 0;                                        // U[2][lr][nx]
  L.off_apx = L.off_u + 2 * L.lr * nx;                // APX[2][maxrows][2 sw]
  L.off_apz = L.off_apx + 2 * L.maxrows * 2 * sw;     // APZ[2][zs][nx]
  L.off_prof = L.off_apz + 2 * L.zs * nx;             // ax bx dbx az bz dbz
  L.off_rec = L.off_prof + 3 * (nx + nz);             // per receiver: 4 local cells (int) + 4 weights + flag
  L.total = L.off_rec + 9 * nrec;
  L.total = (L.total + 3) & ~3;
  return L;
}

// Adjoint shared-memory layout, in floats.
struct AdjLayout {
  int maxrows, lr, zs;
  int off_vs, off_tx, off_u1x, off_tz, off_u1z, off_lpx, off_lzx, off_lpz, off_lzz, off_prof, total;
};

__host__ __device__ inline AdjLayout adj_layout(int nx, int nz, int swa, int C) {
  AdjLayout L;
  L.maxrows = max_rows(nz, C);
  L.lr = L.maxrows + 2 * FD_PAD;
  L.zs = (C == 1 ? 2 : 1) * swa;
  const int sx = L.maxrows * 2 * swa;
  const int sz = L.zs * nx;
  L.off_vs = 0;                          // VS[2][lr][nx]   v^2 dt^2 lambda
  L.off_tx = L.off_vs + 2 * L.lr * nx;   // TX[2][maxrows][2 swa]
  L.off_u1x = L.off_tx + 2 * sx;         // U1X[2][maxrows][2 swa]
  L.off_tz = L.off_u1x + 2 * sx;         // TZ[2][zs][nx]
  L.off_u1z = L.off_tz + 2 * sz;         // U1Z[2][zs][nx]
  L.off_lpx = L.off_u1z + 2 * sz;        // LPX[maxrows][2 swa]  adjoint psi_x (owner only)
  L.off_lzx = L.off_lpx + sx;            // LZX[maxrows][2 swa]  adjoint zeta_x
  L.off_lpz = L.off_lzx + sx;            // LPZ[zs][nx]
  L.off_lzz = L.off_lpz + sz;            // LZZ[zs][nx]
  L.off_prof = L.off_lzz + sz;
  L.total = L.off_prof + 3 * (nx + nz);
  L.total = (L.total + 3) & ~3;
  return L;
}

// Packed strip column of x for a strip of width s on each side of a row of nx cells.
__host__ __device__ __forceinline__ int strip_col(int x, int nx, int s) { return x < s ? x : x - (nx - 2 * s); }

}  // namespace wg
