// Shared-memory layouts of the generation-3 kernels (floats), identical in every CTA of a cluster,
// shared by the kernels and the host-side launch table.
#pragma once

#include "wave_device.cuh"

namespace wg {

__host__ __device__ inline int g3_sw(int pmlp) { return 2 * pmlp + 4; }  // packed strip width per side

struct F3Layout {
  int maxrows, lr, zs;
  int off_u, off_apx, off_zx, off_apz, off_zz, off_v2, off_c2, off_prof, off_rec, total;
};

__host__ __device__ inline F3Layout f3_layout_rt(int NX, int pmlp, int nz, int sw, int C, int nrec) {
  const int SW = g3_sw(pmlp);
  F3Layout L;
  L.maxrows = max_rows(nz, C);
  L.lr = L.maxrows + 2 * FD_PAD;
  L.zs = (C == 1 ? 2 : 1) * sw;
  L.off_u = 0;                                    // U[2][lr][NX]
  L.off_apx = L.off_u + 2 * L.lr * NX;            // APX[2][maxrows][2 SW]   a * psi_x
  L.off_zx = L.off_apx + 2 * L.maxrows * 2 * SW;  // ZX[maxrows][2 SW]      zeta_x (owner only)
  L.off_apz = L.off_zx + L.maxrows * 2 * SW;      // APZ[2][zs][NX]          a * psi_z
  L.off_zz = L.off_apz + 2 * L.zs * NX;           // ZZ[zs][NX]              zeta_z (owner only)
  L.off_v2 = L.off_zz + L.zs * NX;                // V2[maxrows][NX]         v^2 dt^2 (owner only)
  L.off_c2 = L.off_v2 + L.maxrows * NX;           // C2[maxrows][NX]         2 v dt^2 (owner only)
  L.off_prof = L.off_c2 + L.maxrows * NX;
  L.off_rec = L.off_prof + 3 * (NX + nz);
  L.total = (L.off_rec + 9 * nrec + 3) & ~3;
  return L;
}

struct A3Layout {
  int maxrows, lr, zs;
  int off_vs, off_tx, off_u1x, off_tz, off_u1z, off_lpx, off_lzx, off_lpz, off_lzz, off_v2, off_ga, off_prof, off_opb,
      total;
};

// VS is exchanged with the peer CTA and double-buffered; the x- and z-strip derived terms are read
// only inside the CTA and are single-buffered (a CTA barrier separates their reads and writes).
__host__ __device__ inline A3Layout a3_layout_rt(int NX, int pmlp, int nz, int swa, int C) {
  const int SW = g3_sw(pmlp);
  A3Layout L;
  L.maxrows = max_rows(nz, C);
  L.lr = L.maxrows + 2 * FD_PAD;
  L.zs = (C == 1 ? 2 : 1) * swa;
  const int sx = L.maxrows * 2 * SW, sz = L.zs * NX;
  L.off_vs = 0;                           // VS[2][lr][NX]   v^2 dt^2 lambda
  L.off_tx = L.off_vs + 2 * L.lr * NX;    // TX[maxrows][2 SW]
  L.off_u1x = L.off_tx + sx;              // U1X[maxrows][2 SW]
  L.off_tz = L.off_u1x + sx;              // TZ[zs][NX]
  L.off_u1z = L.off_tz + sz;              // U1Z[zs][NX]
  L.off_lpx = L.off_u1z + sz;             // LPX[maxrows][2 SW]  adjoint psi_x (owner only)
  L.off_lzx = L.off_lpx + sx;             // LZX[maxrows][2 SW]  adjoint zeta_x
  L.off_lpz = L.off_lzx + sx;             // LPZ[zs][NX]
  L.off_lzz = L.off_lpz + sz;             // LZZ[zs][NX]
  L.off_v2 = L.off_lzz + sz;              // V2[maxrows][NX]     v^2 dt^2 (owner only)
  L.off_ga = L.off_v2 + L.maxrows * NX;   // GA[maxrows][NX]     gradient accumulator (owner only)
  L.off_prof = L.off_ga + L.maxrows * NX; // ax bx dbx az bz dbz
  L.off_opb = L.off_prof + 3 * (NX + nz); // 1 + bx, per column
  L.total = (L.off_opb + NX + 3) & ~3;
  return L;
}

}  // namespace wg
