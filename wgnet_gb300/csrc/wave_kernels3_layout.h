// Shared-memory layouts of the generation-3 kernels (floats), identical in every CTA of a cluster,
// shared by the kernels and the host-side launch table. The z-strip arrays are sized for the widest
// strip the shape supports (g3_sw), so that for grids whose rows split evenly into the shape's
// segments every offset is a compile-time constant in the kernel.
#pragma once

#include "wave_device.cuh"

namespace wg {

__host__ __device__ inline int g3_sw(int pmlp) { return 2 * pmlp + 4; }  // packed strip width per side

// Wavelet samples kept in shared memory: a ring over the launch's steps, refilled half at a time.
constexpr int G3_WAV_STEPS = 128;

struct F3Layout {
  int maxrows, lr, zs;
  int off_u, off_apx, off_zx, off_apz, off_zz, off_v2, off_c2, off_prof, off_rec, off_src, total;
};

__host__ __device__ inline F3Layout f3_layout_rt(int NX, int pmlp, int nz, int sw, int C, int nrec) {
  const int SW = g3_sw(pmlp);
  F3Layout L;
  L.maxrows = max_rows(nz, C);
  L.lr = L.maxrows + 2 * FD_PAD;
  L.zs = (C == 1 ? 2 : 1) * SW;
  L.off_u = 0;                                    // U[2][lr][NX]
  L.off_apx = L.off_u + 2 * L.lr * NX;            // APX[2][maxrows][2 SW]   a * psi_x
  L.off_zx = L.off_apx + 2 * L.maxrows * 2 * SW;  // ZX[maxrows][2 SW]      zeta_x (owner only)
  L.off_apz = L.off_zx + L.maxrows * 2 * SW;      // APZ[2][zs][NX]          a * psi_z
  L.off_zz = L.off_apz + 2 * L.zs * NX;           // ZZ[zs][NX]              zeta_z (owner only)
  L.off_v2 = L.off_zz + L.zs * NX;                // V2[maxrows][NX]         v^2 dt^2 (owner only)
  L.off_c2 = L.off_v2 + L.maxrows * NX;           // C2[maxrows][NX]         2 v dt^2 (owner only)
  L.off_prof = L.off_c2 + L.maxrows * NX;
  L.off_rec = L.off_prof + 3 * (NX + nz);
  L.off_src = (L.off_rec + 9 * nrec + 3) & ~3;  // source corners: 4 cells (int), 4 factors, wavelet ring
  L.total = L.off_src + 8 + G3_WAV_STEPS;
  return L;
}

// Receiver rows of one CTA whose entry offsets the adjoint keeps in shared memory.
constexpr int G3_REC_ROWS = 4;

struct A3Layout {
  int maxrows, lr, zs;
  int off_vs, off_tx, off_u1x, off_tz, off_u1z, off_lpx, off_lzx, off_lpz, off_lzz, off_v2, off_ga, off_prof, off_opb,
      off_res, rcap, pcap, off_src, off_rrow, off_roff, off_ew, off_er, total;
};

// VS is exchanged with the peer CTA and double-buffered; the x- and z-strip derived terms are read
// only inside the CTA and are single-buffered (a CTA barrier separates their reads and writes).
__host__ __device__ inline A3Layout a3_layout_rt(int NX, int pmlp, int nz, int swa, int C, int nrec) {
  const int SW = g3_sw(pmlp);
  A3Layout L;
  L.maxrows = max_rows(nz, C);
  L.lr = L.maxrows + 2 * FD_PAD;
  L.zs = (C == 1 ? 2 : 1) * SW;
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
  L.off_src = (L.off_opb + NX + 3) & ~3;  // source corners: 4 cells (int), 4 factors, then the
                                          // wavelet samples of the launch's steps
  L.rcap = (nrec + 3) & ~3;
  L.pcap = 4 * L.rcap;                    // receiver entries of one CTA (4 corners per receiver)
  L.off_res = L.off_src + 8 + G3_WAV_STEPS;              // P[2][pcap]  weight x residual per entry, next two steps
  // receiver entries of the CTA's rows, a copy of the per-cell CSR: slot per local row (int, -1:
  // none), entry offsets of each slot's cells (int), entry weights and receivers (int)
  L.off_rrow = L.off_res + 2 * L.pcap;
  L.off_roff = L.off_rrow + ((L.maxrows + 3) & ~3);
  L.off_ew = L.off_roff + G3_REC_ROWS * (NX + 4);
  L.off_er = L.off_ew + L.pcap;
  L.total = L.off_er + L.pcap;
  return L;
}

}  // namespace wg
