// Additive anisotropic-Gaussian renderer (python/wgnet/render.py:34-109) and its vector-Jacobian
// product, for the 70 x 70 grid with 35 x 35 slots, each drawn in its 25 x 25 pixel window.
//
// Forward gathers: each pixel sums the slots whose window covers it, in increasing slot order (the
// order in which index_add_ accumulates on the CPU), from per-slot constants staged in shared
// memory; one thread computes a 2 x 2 pixel quad, so each slot's constants serve up to four pixels.
// Backward: one warp per slot reduces the six parameter gradients over its window.
#include <cuda_runtime.h>

#include "wave_launch.h"
#include "wgnet_gb300.h"

namespace {

constexpr int GRID = 70;
constexpr int SIDE = 35;
constexpr int SLOTS = SIDE * SIDE;
constexpr int WIN = 12;
constexpr int NPAR = 6;

struct SlotC {
  float cx, cz, isx, isz, c, s, w;
};

__device__ __forceinline__ SlotC slot_consts(const float* p, int i) {
  const int iz = i / SIDE, ix = i % SIDE;
  SlotC k;
  k.cx = (2.0f * ix + 1.0f) + p[0];
  k.cz = (2.0f * iz + 1.0f) + p[1];
  k.isx = expf(-p[2]);
  k.isz = expf(-p[3]);
  sincosf(p[4], &k.s, &k.c);
  k.w = p[5];
  return k;
}

// One thread per 2 x 2 pixel quad (2n..2n+1, 2m..2m+1): row 2n is covered by the slots
// iz in [n-6, n+6], row 2n+1 by [n-5, n+6] (and the same for the columns), so each slot's
// constants, loaded once, serve up to four pixels. Every pixel still sums its slots in increasing
// slot order. Blocks (QBLK threads, blockIdx.y) split a model's 1225 quads; each block stages all
// slot constants of its model (blockIdx.x).
constexpr int QBLK = 256;
constexpr int QBLOCKS = (SLOTS + QBLK - 1) / QBLK;

__global__ void __launch_bounds__(QBLK) render_fwd_kernel(const float* __restrict__ params, float* __restrict__ field) {
  __shared__ float sh[7 * SLOTS];
  const int b = blockIdx.x;
  const float* pb = params + static_cast<size_t>(b) * SLOTS * NPAR;
  for (int i = threadIdx.x; i < SLOTS; i += blockDim.x) {
    const SlotC k = slot_consts(pb + i * NPAR, i);
    sh[i] = k.cx;
    sh[SLOTS + i] = k.cz;
    sh[2 * SLOTS + i] = k.isx;
    sh[3 * SLOTS + i] = k.isz;
    sh[4 * SLOTS + i] = k.c;
    sh[5 * SLOTS + i] = k.s;
    sh[6 * SLOTS + i] = k.w;
  }
  __syncthreads();
  const int q = blockIdx.y * QBLK + threadIdx.x;
  if (q >= SLOTS) return;
  const int n = q / SIDE, m = q % SIDE;
  const int iz0 = max(0, n - WIN / 2), iz1 = min(SIDE - 1, n + WIN / 2);
  const int ix0 = max(0, m - WIN / 2), ix1 = min(SIDE - 1, m + WIN / 2);
  const float fx0 = static_cast<float>(2 * m) + 0.5f, fx1 = static_cast<float>(2 * m + 1) + 0.5f;
  const float fz0 = static_cast<float>(2 * n) + 0.5f, fz1 = static_cast<float>(2 * n + 1) + 0.5f;
  float a00 = 0.0f, a01 = 0.0f, a10 = 0.0f, a11 = 0.0f;  // a[row][col]
  auto term = [](float fx, float fz, float cx, float cz, float c, float s, float isx, float isz, float w) {
    const float dx = fx - cx, dz = fz - cz;
    const float u = (dx * c + dz * s) * isx;
    const float v = (dz * c - dx * s) * isz;
    return w * expf(-0.5f * (u * u + v * v));
  };
  for (int iz = iz0; iz <= iz1; ++iz) {
    const bool row1 = iz >= n - WIN / 2 + 1;  // slot row iz also covers pixel row 2n + 1
    for (int ix = ix0; ix <= ix1; ++ix) {
      const bool col1 = ix >= m - WIN / 2 + 1;
      const int i = iz * SIDE + ix;
      const float cx = sh[i], cz = sh[SLOTS + i], isx = sh[2 * SLOTS + i], isz = sh[3 * SLOTS + i];
      const float c = sh[4 * SLOTS + i], s = sh[5 * SLOTS + i], w = sh[6 * SLOTS + i];
      a00 += term(fx0, fz0, cx, cz, c, s, isx, isz, w);
      if (col1) a01 += term(fx1, fz0, cx, cz, c, s, isx, isz, w);
      if (row1) {
        a10 += term(fx0, fz1, cx, cz, c, s, isx, isz, w);
        if (col1) a11 += term(fx1, fz1, cx, cz, c, s, isx, isz, w);
      }
    }
  }
  float* f = field + static_cast<size_t>(b) * GRID * GRID + (2 * n) * GRID + 2 * m;
  *reinterpret_cast<float2*>(f) = make_float2(a00, a01);
  *reinterpret_cast<float2*>(f + GRID) = make_float2(a10, a11);
}

__global__ void __launch_bounds__(256) render_bwd_kernel(const float* __restrict__ params, const float* __restrict__ cot,
                                                          int batch, float* __restrict__ grad) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= batch * SLOTS) return;
  const int b = warp / SLOTS, i = warp % SLOTS;
  const float* p = params + static_cast<size_t>(warp) * NPAR;
  const SlotC k = slot_consts(p, i);
  const int iz = i / SIDE, ix = i % SIDE;
  const float* cb = cot + static_cast<size_t>(b) * GRID * GRID;
  float g0 = 0.f, g1 = 0.f, g2 = 0.f, g3 = 0.f, g4 = 0.f, g5 = 0.f;
  for (int q = lane; q < (2 * WIN + 1) * (2 * WIN + 1); q += 32) {
    const int pz = 2 * iz + q / (2 * WIN + 1) - WIN;
    const int px = 2 * ix + q % (2 * WIN + 1) - WIN;
    if (pz < 0 || pz >= GRID || px < 0 || px >= GRID) continue;
    const float dx = (static_cast<float>(px) + 0.5f) - k.cx;
    const float dz = (static_cast<float>(pz) + 0.5f) - k.cz;
    const float ru = dx * k.c + dz * k.s;
    const float rv = dz * k.c - dx * k.s;
    const float u = ru * k.isx, v = rv * k.isz;
    const float e = expf(-0.5f * (u * u + v * v));
    const float ct = cb[pz * GRID + px];
    const float ge = ct * k.w * e;  // d/d(-0.5 (u^2 + v^2)) of the contribution, times cotangent
    // du/dcx = -c isx, dv/dcx = s isz; du/dcz = -s isx, dv/dcz = -c isz
    g0 += -ge * (u * (-k.c * k.isx) + v * (k.s * k.isz));
    g1 += -ge * (u * (-k.s * k.isx) + v * (-k.c * k.isz));
    g2 += ge * u * u;  // isx = exp(-log_sx): du/dlog_sx = -u
    g3 += ge * v * v;
    g4 += -ge * (u * rv * k.isx - v * ru * k.isz);  // dru/dangle = rv, drv/dangle = -ru
    g5 += ct * e;
  }
  for (int o = 16; o > 0; o >>= 1) {
    g0 += __shfl_down_sync(0xffffffffu, g0, o);
    g1 += __shfl_down_sync(0xffffffffu, g1, o);
    g2 += __shfl_down_sync(0xffffffffu, g2, o);
    g3 += __shfl_down_sync(0xffffffffu, g3, o);
    g4 += __shfl_down_sync(0xffffffffu, g4, o);
    g5 += __shfl_down_sync(0xffffffffu, g5, o);
  }
  if (lane == 0) {
    float* g = grad + static_cast<size_t>(warp) * NPAR;
    g[0] = g0;
    g[1] = g1;
    g[2] = g2;
    g[3] = g3;
    g[4] = g4;
    g[5] = g5;
  }
}

}  // namespace

extern "C" int wg_render_fwd_dev(const float* d_params, int batch, float* d_field, void* stream) {
  if (batch < 0 || (batch > 0 && (!d_params || !d_field))) return wg::report_error(WG_ERR_ARG, "bad render arguments");
  if (batch == 0) return WG_OK;
  render_fwd_kernel<<<dim3(batch, QBLOCKS), QBLK, 0, static_cast<cudaStream_t>(stream)>>>(d_params, d_field);
  wg::note_launch();
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? WG_OK : wg::report_error(WG_ERR_CUDA, cudaGetErrorString(e));
}

extern "C" int wg_render_bwd_dev(const float* d_params, const float* d_cot, int batch, float* d_grad, void* stream) {
  if (batch < 0 || (batch > 0 && (!d_params || !d_cot || !d_grad)))
    return wg::report_error(WG_ERR_ARG, "bad render arguments");
  if (batch == 0) return WG_OK;
  const int warps = batch * SLOTS;
  render_bwd_kernel<<<(warps + 7) / 8, 256, 0, static_cast<cudaStream_t>(stream)>>>(d_params, d_cot, batch, d_grad);
  wg::note_launch();
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? WG_OK : wg::report_error(WG_ERR_CUDA, cudaGetErrorString(e));
}
