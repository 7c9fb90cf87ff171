// Constants and shared-memory layout of the generation-2 forward kernel (wave_kernels2.cuh),
// shared by the kernel and the host-side launch table.
#pragma once

#include "wave_device.cuh"

namespace wg {

constexpr int kPmlPairs = 16;            // column pairs per side owned by the PML warp
constexpr int kPmlCols = 2 * kPmlPairs;  // 32 columns per side: x in [2, 34) and [nx-34, nx-2)
constexpr int kSwx = kPmlCols + 4;       // packed a*psi_x strip width per side (reads reach x+3)


// Shared-memory layout of fwd2, in floats (identical in every CTA of a cluster).
struct Fwd2Layout {
  int maxrows, lr, zs;
  int off_u, off_apx, off_apz, off_zz, off_prof, off_rec, total;
};

__host__ __device__ inline Fwd2Layout fwd2_layout(int nx, int nz, int sw, int C, int nrec) {
  Fwd2Layout L;
  L.maxrows = max_rows(nz, C);
  L.lr = L.maxrows + 2 * FD_PAD;
  L.zs = (C == 1 ? 2 : 1) * sw;
  L.off_u = 0;                                        // U[2][lr][nx]
  L.off_apx = L.off_u + 2 * L.lr * nx;                // APX[2][maxrows][2 kSwx]
  L.off_apz = L.off_apx + 2 * L.maxrows * 2 * kSwx;   // APZ[2][zs][nx]
  L.off_zz = L.off_apz + 2 * L.zs * nx;               // ZZ[zs][nx] zeta_z (owner only)
  L.off_prof = L.off_zz + L.zs * nx;
  L.off_rec = L.off_prof + 3 * (nx + nz);
  L.total = L.off_rec + 9 * nrec;
  L.total = (L.total + 3) & ~3;
  return L;
}

}  // namespace wg
