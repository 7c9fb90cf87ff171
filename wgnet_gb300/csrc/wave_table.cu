#include <cuda_runtime.h>

#include "wave_device.cuh"
#include "wave_kernels3_layout.h"
#include "wave_launch.h"

// Launch table of the resident kernels. The kernel templates live in wave_kernels.cuh; each
// compiled shape is instantiated in one of the wave_inst_*.cu files so that they build in parallel.

namespace wg {

#define WG_SHAPES(X) \
  X(1, 1024, 12)     \
  X(2, 1024, 6)      \
  X(2, 512, 12)      \
  X(2, 1024, 10)     \
  X(2, 1024, 16)     \
  X(4, 1024, 8)      \
  X(4, 512, 16)

// generation-3 shapes (forward and adjoint): (NX, PML pairs per side, C, S rows per segment,
// segments, interior warps per segment)
#define WG_G3_SHAPES(X)         \
  X(114, 12, 2, 5, 11, 1)       \
  X(114, 12, 2, 4, 14, 1)       \
  X(114, 12, 4, 4, 7, 1)        \
  X(114, 12, 4, 2, 14, 1)       \
  X(114, 12, 1, 8, 14, 1)       \
  X(144, 12, 4, 5, 7, 2)        \
  X(144, 12, 4, 7, 5, 2)        \
  X(184, 12, 6, 6, 5, 3)        \
  X(184, 12, 6, 10, 3, 3)

// generation-3 shapes that also have a fast-arithmetic forward (one instantiation file each): the
// default shape of each of the 70x70, 100x100 and 140x140 grids at pml 20
#define WG_G3_FAST_SHAPES(X)    \
  X(114, 12, 2, 5, 11, 1)       \
  X(144, 12, 4, 5, 7, 2)        \
  X(184, 12, 6, 6, 5, 3)

#define WG_ADJ_SHAPES(X) \
  X(2, 1024, 6)          \
  X(2, 512, 12)          \
  X(4, 1024, 4)          \
  X(4, 1024, 8)          \
  X(4, 512, 16)


// Compiled launch shapes. A shape is usable for a grid when its cells-per-thread bound covers the
// CTA's rows and its shared-memory layout fits the 227 KB per-CTA limit.
#define WG_LIST(Cc, NTt, CPTt) Shape{Cc, NTt, CPTt, 1, 0, 0, 0},
#define WG_LIST3(NXs, PMLPs, Cc, Ss, NSEGs, NIs) Shape{Cc, NSEGs * 32 * (1 + NIs), 2 * Ss, 3, Ss, NSEGs, NIs, NXs, PMLPs},
static const Shape kFwdShapes[] = {WG_G3_SHAPES(WG_LIST3) WG_SHAPES(WG_LIST)};
static const Shape kAdjShapes[] = {WG_G3_SHAPES(WG_LIST3) WG_ADJ_SHAPES(WG_LIST)};
#undef WG_LIST
#undef WG_LIST3

// Whether the fast-arithmetic kernels exist for a generation-3 shape.
static bool g3_has_fast(const Shape& s) {
#define WG_HASF(NXs, PMLPs, Cc, Ss, NSEGs, NIs)                                                                  \
  if (s.kind == 3 && s.nxc == NXs && s.pmlp == PMLPs && s.cluster == Cc && s.seg_rows == Ss && s.nseg == NSEGs && \
      s.ni == NIs)                                                                                                 \
    return true;
  WG_G3_FAST_SHAPES(WG_HASF)
#undef WG_HASF
  return false;
}

static Shape with_fast(Shape s) {
  s.fast = g3_has_fast(s) ? 1 : 0;
  return s;
}

int fwd_shape_count() { return static_cast<int>(sizeof(kFwdShapes) / sizeof(kFwdShapes[0])); }
int adj_shape_count() { return static_cast<int>(sizeof(kAdjShapes) / sizeof(kAdjShapes[0])); }
Shape fwd_shape(int i) { return with_fast(kFwdShapes[i]); }
Shape adj_shape(int i) { return with_fast(kAdjShapes[i]); }

size_t fwd_smem_bytes(const Shape& s, int nx, int nz, int sw, int nrec) {
  if (s.kind == 3) return static_cast<size_t>(f3_layout_rt(s.nxc, s.pmlp, nz, sw, s.cluster, nrec).total) * sizeof(float);
  return static_cast<size_t>(fwd_layout(nx, nz, sw, s.cluster, nrec).total) * sizeof(float);
}
size_t adj_smem_bytes(const Shape& s, int nx, int nz, int swa, int nrec) {
  if (s.kind == 3)
    return static_cast<size_t>(a3_layout_rt(s.nxc, s.pmlp, nz, swa, s.cluster, nrec).total) * sizeof(float);
  return static_cast<size_t>(adj_layout(nx, nz, swa, s.cluster).total) * sizeof(float);
}

// A generation-3 shape fits when the grid width equals its compile-time width, its PML warp covers
// the adjoint's C-PML columns [2, region_adj) (which contain the forward's), its interior warps
// cover the columns in between and its segments cover the CTA's rows.
static bool g3_fits(const Shape& s, int nx, int nz, int rows, int region_adj) {
  if (nx != s.nxc || (nx & 1)) return false;
  if (FD_PAD + 2 * s.pmlp < region_adj) return false;
  const int ipairs = (nx - 2 * FD_PAD - 4 * s.pmlp) / 2;
  if (ipairs < 1 || ipairs > 32 * s.ni) return false;
  return rows <= s.seg_rows * s.nseg && nz >= 2 * g3_sw(s.pmlp);
}

bool fwd_shape_fits(const Shape& s, int nx, int nz, int sw, int nrec) {
  if (nx < 2 * sw || nz < 2 * sw) return false;  // left/right (top/bottom) strips must not overlap
  const int rows = max_rows(nz, s.cluster);
  if (s.kind == 3) {
    if (!g3_fits(s, nx, nz, rows, sw)) return false;  // forward strip width sw = region + 2 = region_adj
  } else if (static_cast<long>(rows) * (nx - 2 * FD_PAD) > static_cast<long>(s.threads) * s.cpt) {
    return false;
  }
  if (fwd_smem_bytes(s, nx, nz, sw, nrec) > kMaxSmemPerCta) return false;
  if (s.cluster > 1) {
    // Each z strip (sw rows) must be updated and read inside the first / last CTA.
    if (split_row(nz, s.cluster, 1) < sw || split_row(nz, s.cluster, s.cluster - 1) > nz - sw) return false;
  }
  return nx < 65536 && nz < 32768;
}

bool adj_shape_fits(const Shape& s, int nx, int nz, int swa, int nrec) {
  if (nx < 2 * swa || nz < 2 * swa) return false;
  const int rows = max_rows(nz, s.cluster);
  if (s.kind == 3) {
    if (!g3_fits(s, nx, nz, rows, swa - 2)) return false;
  } else if (static_cast<long>(rows) * (nx - 2 * FD_PAD) > static_cast<long>(s.threads) * s.cpt) {
    return false;
  }
  if (adj_smem_bytes(s, nx, nz, swa, nrec) > kMaxSmemPerCta) return false;
  if (s.cluster > 1) {
    if (split_row(nz, s.cluster, 1) < swa || split_row(nz, s.cluster, s.cluster - 1) > nz - swa) return false;
  }
  return nx < 65536 && nz < 32768;
}

cudaError_t launch_fwd(const Shape& s, bool traces, bool store, const FwdArgs& a, cudaStream_t stream) {
  const size_t smem = fwd_smem_bytes(s, a.g.nx, a.g.nz, a.g.sw, a.st.nrec);
  if (s.kind == 3) {
    if (a.fast) {  // shapes without fast-arithmetic kernels run the unfused ones
#define WG_FWD3F(NXs, PMLPs, Cc, Ss, NSEGs, NIs)                                                                 \
  if (s.nxc == NXs && s.pmlp == PMLPs && s.cluster == Cc && s.seg_rows == Ss && s.nseg == NSEGs && s.ni == NIs) \
    return fwd3f_dispatch<NXs, PMLPs, Cc, Ss, NSEGs, NIs>(traces, store, a, smem, stream);
      WG_G3_FAST_SHAPES(WG_FWD3F)
#undef WG_FWD3F
    }
#define WG_FWD3(NXs, PMLPs, Cc, Ss, NSEGs, NIs)                                                                  \
  if (s.nxc == NXs && s.pmlp == PMLPs && s.cluster == Cc && s.seg_rows == Ss && s.nseg == NSEGs && s.ni == NIs) \
    return fwd3_dispatch<NXs, PMLPs, Cc, Ss, NSEGs, NIs>(traces, store, a, smem, stream);
    WG_G3_SHAPES(WG_FWD3)
#undef WG_FWD3
    return cudaErrorInvalidValue;
  }
#define WG_FWD(Cc, NTt, CPTt) \
  if (s.cluster == Cc && s.threads == NTt && s.cpt == CPTt) return fwd_dispatch<Cc, NTt, CPTt>(traces, store, a, smem, stream);
  WG_SHAPES(WG_FWD)
#undef WG_FWD
  return cudaErrorInvalidValue;
}

cudaError_t launch_adj(const Shape& s, const AdjArgs& a, cudaStream_t stream) {
  const size_t smem = adj_smem_bytes(s, a.g.nx, a.g.nz, a.g.swa, a.st.nrec);
  if (s.kind == 3) {
#define WG_ADJ3(NXs, PMLPs, Cc, Ss, NSEGs, NIs)                                                                  \
  if (s.nxc == NXs && s.pmlp == PMLPs && s.cluster == Cc && s.seg_rows == Ss && s.nseg == NSEGs && s.ni == NIs) \
    return adj3_dispatch<NXs, PMLPs, Cc, Ss, NSEGs, NIs>(a, smem, stream);
    WG_G3_SHAPES(WG_ADJ3)
#undef WG_ADJ3
    return cudaErrorInvalidValue;
  }
#define WG_ADJ(Cc, NTt, CPTt) \
  if (s.cluster == Cc && s.threads == NTt && s.cpt == CPTt) return adj_dispatch<Cc, NTt, CPTt>(a, smem, stream);
  WG_ADJ_SHAPES(WG_ADJ)
#undef WG_ADJ
  return cudaErrorInvalidValue;
}

}  // namespace wg
