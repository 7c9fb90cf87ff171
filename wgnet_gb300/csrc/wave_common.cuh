// Shared definitions for the resident time-stepping kernels (forward, adjoint) of the acoustic
// C-PML solver. Device code targets sm_103a only.
//
// Arithmetic contract: the whole library is compiled with -fmad=false and every expression keeps
// the operation order of the reference shaders (crates/wave-gauss-rs/src/shaders/splatForward.wgsl,
// splatAdjoint.wgsl), so each f32 result is rounded exactly as in the reference: the GPU output
// equals the f32 CPU restatement bit for bit.
#pragma once

#include <cstddef>
#include <cstdint>

namespace wg {

constexpr int FD_PAD = 2;

// f32 literals of the reference stencils (splatForward.wgsl:86-96, splatAdjoint.wgsl:163-167).
constexpr float F_D2A = -2.5f;
constexpr float F_D2B = 1.3333333333333333f;
constexpr float F_D2C = 0.08333333333333333f;  // forward subtracts it
constexpr float F_D1A = 0.6666666666666666f;
constexpr float F_D1B = 0.08333333333333333f;  // forward subtracts it
constexpr float A_D1B = -0.08333333333333333f; // adjoint adds it
constexpr float A_D2C = -0.08333333333333333f;

// Geometry of one padded grid and its C-PML, shared by every launch of an engine.
struct Grid {
  int nx, nz;          // padded grid (visible + 2 (pml + FD_PAD))
  int pml;
  int region;          // forward PML region width: pml + 2 FD_PAD
  int region_adj;      // adjoint PML region width: pml + 3 FD_PAD
  int sw;              // forward strip width (region + 2): columns/rows that hold a*psi
  int swa;             // adjoint strip width (region_adj + 2)
  float rh, dt2;       // 1/h and dt*dt, computed in f32 on the host
  // The forward second derivative is scaled as (sum * d2a) * d2b: (rh, rh) reproduces the engine
  // shader (splatForward.wgsl:86), (rh*rh, 1) reproduces the CPU solver's rh2 (lib.rs:159-160).
  float d2a, d2b;
  int nt;
  const float* prof;   // ax bx dbx (nx each) | az bz dbz (nz each)
  const float* wavelet;  // [nt]
};

// Sources and receivers: 4 bilinear corners each (wave_wgpu.rs:217-230).
struct Stations {
  int shots, nrec;
  const int* src_cell;   // [shots][4]
  const float* src_w;    // [shots][4]
  const int* rec_cell;   // [nrec][4]
  const float* rec_w;    // [nrec][4]
  const int* csr;        // [cells + 1] receiver entries per cell, ordered by (cell, receiver)
  const int* ent_rec;    // [entries]
  const float* ent_w;    // [entries]
};

// Layout of one wavefield checkpoint (state at the start of a step), in floats:
//   U_cur [nz][nx] | U_prev [nz][nx] | APX [nz][2 sw] | APZ [2 sw][nx] | ZX [nz][2 sw] | ZZ [2 sw][nx]
// APX/APZ hold a * psi (what neighbours read), ZX/ZZ hold zeta. Strip columns/rows are packed:
// left strip x in [0, sw), right strip x in [nx - sw, nx) -> packed column x or x - (nx - 2 sw).
// Frame cells (within FD_PAD of the edge) are never written and read as zero.
__host__ __device__ inline size_t ckpt_floats(int nx, int nz, int sw) {
  size_t n = 2 * (size_t)nx * nz + 2 * ((size_t)nz * 2 * sw + (size_t)2 * sw * nx);
  return (n + 3) & ~(size_t)3;
}

// Adjoint state saved between segments, in floats:
//   L_cur [nz][nx] | L_prev [nz][nx] | LPX [nz][2 swa] | LZX [nz][2 swa] | LPZ [2 swa][nx] | LZZ [2 swa][nx]
__host__ __device__ inline size_t adjstate_floats(int nx, int nz, int swa) {
  size_t n = 2 * (size_t)nx * nz + 2 * ((size_t)nz * 2 * swa + (size_t)2 * swa * nx);
  return (n + 3) & ~(size_t)3;
}

struct FwdArgs {
  Grid g;
  Stations st;
  const float* vel;      // [models][nz][nx] clamped, edge-replicated velocity (m/s)
  int units;             // models * shots
  int t0, t1;            // steps [t0, t1)
  float* traces;         // [units][nt][nrec] or null (recompute)
  const float* ck_in;    // [units][ck_slots] checkpoint to start from (null: zero state)
  int ck_in_slot;        // slot index within ck_in
  float* ck_out;         // [units][ck_slots][ckpt_floats] or null
  int ck_every;          // write a checkpoint at steps t % ck_every == 0, t > t0
  int ck_slots;          // checkpoint slots per unit
  float* stored;         // [units][t1 - t0][nz][nx] stored gradient terms 2 v dt^2 w, or null
  int* status;
  int fast;              // 1: fast-arithmetic kernels where the shape has them (fused, reassociated)
};

struct AdjArgs {
  Grid g;
  Stations st;
  const float* vel;
  int units;
  int t_hi, t_lo;        // process t = t_hi - 1 down to t_lo
  const float* residual; // [units][nt][nrec] scaled residuals dJ/dtraces
  const float* stored;   // [units][t_hi - t_lo][nz][nx], step t at index t - t_lo
  float* state;          // [units][adjstate_floats] in/out (read unless first, always written)
  int first;             // 1: start from zero state and zero gradient
  float* gacc;           // [units][nz][nx] gradient accumulator (per shot, padded grid)
  int* status;
  int prefetch;          // generation-3 adjoint: fetch the next step's stored terms a step ahead
};

// Status codes shared with the C ABI (include/wgnet_gb300.h defines the same numbers).
enum Status : int {
  ST_OK = 0,
  ST_ARG = 1,
  ST_CUDA = 2,
  ST_NONFINITE = 3,
  ST_ENERGY = 4,
  ST_UNSUPPORTED = 5,
  ST_CFL = 6,
  ST_OOM = 7,
};

// Kernel launch shape chosen per grid: kernel generation (1: flat cell mapping, 3: column-pair x
// segment mapping for a compile-time grid width), cluster size (CTAs per unit), threads per CTA and the static cells-per-thread
// bound the kernel was compiled with. Generation 3 also fixes the segment length S (rows), the
// number of segments and the number of interior warps per segment.
struct Shape {
  int cluster, threads, cpt;
  int kind = 1, seg_rows = 0, nseg = 0, ni = 0;
  int nxc = 0, pmlp = 0;  // generation 3: compile-time grid width and PML column pairs per side
  int fast = 0;           // generation 3: fast-arithmetic forward compiled for this shape
};

}  // namespace wg
