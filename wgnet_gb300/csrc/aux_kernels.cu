// Small kernels around the time-stepping kernels: velocity padding, observed energy, residual and
// misfit, gradient shot-sum/mask/fold, causal band-limit FIR. All are HBM-bound elementwise or
// reduction passes; reductions use a fixed launch shape and a fixed tree so they are deterministic.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>

#include "wave_launch.h"

namespace wg {

namespace {

constexpr int kRedThreads = 512;

// Block-wide f64 sum with a fixed tree (deterministic for a fixed blockDim).
__device__ double block_sum(double v, double* sh) {
  const int tid = threadIdx.x;
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((tid & 31) == 0) sh[tid >> 5] = v;
  __syncthreads();
  double r = 0.0;
  if (tid < 32) {
    r = (tid < static_cast<int>(blockDim.x >> 5)) ? sh[tid] : 0.0;
    for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
  }
  return r;  // valid in thread 0
}

__global__ void pad_kernel(const float* __restrict__ vis, int nx_vis, int nz_vis, int pad, float vmin, float vmax,
                           float* __restrict__ padded, float* __restrict__ mask) {
  const int nx = nx_vis + 2 * pad, nz = nz_vis + 2 * pad;
  const int model = blockIdx.y;
  const size_t cells = static_cast<size_t>(nx) * nz;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < static_cast<int>(cells); i += gridDim.x * blockDim.x) {
    const int z = i / nx, x = i % nx;
    const int vz = min(max(z - pad, 0), nz_vis - 1);
    const int vx = min(max(x - pad, 0), nx_vis - 1);
    const float v = vis[static_cast<size_t>(model) * nx_vis * nz_vis + vz * nx_vis + vx];
    if (mask) mask[model * cells + i] = (v > vmin && v < vmax) ? 1.0f : 0.0f;
    // Rust f32::clamp: NaN stays NaN.
    padded[model * cells + i] = v < vmin ? vmin : (v > vmax ? vmax : v);
  }
}

__global__ void energy_kernel(const float* __restrict__ obs, size_t per_model, double* __restrict__ energy,
                              float* __restrict__ scale, int* __restrict__ status) {
  __shared__ double sh[32];
  const int model = blockIdx.x;
  const float* o = obs + static_cast<size_t>(model) * per_model;
  double acc = 0.0;
  for (size_t i = threadIdx.x; i < per_model; i += blockDim.x) {
    const double d = static_cast<double>(o[i]);
    acc += d * d;
  }
  const double e = block_sum(acc, sh);
  if (threadIdx.x == 0) {
    energy[model] = e;
    scale[model] = static_cast<float>(1.0 / e);
    if (!(e > 0.0) && status) atomicExch(status, static_cast<int>(ST_ENERGY));
  }
}

// wave_wgpu.rs:13-54: d = p - obs; r = d * scale; e = 0.5 * d * d * scale (f32), summed in f64.
__global__ void residual_kernel(const float* pred, const float* __restrict__ obs, const float* __restrict__ scale,
                                size_t per_model, float* res, double* __restrict__ loss) {
  __shared__ double sh[32];
  const int model = blockIdx.x;
  const size_t base = static_cast<size_t>(model) * per_model;
  const float sc = scale[model];
  double acc = 0.0;
  for (size_t i = threadIdx.x; i < per_model; i += blockDim.x) {
    const float d = pred[base + i] - obs[base + i];
    res[base + i] = d * sc;
    acc += static_cast<double>(((0.5f * d) * d) * sc);
  }
  const double e = block_sum(acc, sh);
  if (threadIdx.x == 0) loss[model] = e;
}

// wave_wgpu.rs:974-1005. One thread per visible node; the padded cells that fold onto it are
// visited row-major (the reference's accumulation order), summed in f64.
__global__ void fold_kernel(const float* __restrict__ gacc, const float* __restrict__ mask, int shots, int nx,
                            int nz, int pad, int nx_vis, int nz_vis, float* __restrict__ grad) {
  const int model = blockIdx.y;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nx_vis * nz_vis) return;
  const int vz = i / nx_vis, vx = i % nx_vis;
  const size_t cells = static_cast<size_t>(nx) * nz;
  const int z_lo = (vz == 0) ? 0 : vz + pad;
  const int z_hi = (vz == nz_vis - 1) ? nz : vz + pad + 1;
  const int x_lo = (vx == 0) ? 0 : vx + pad;
  const int x_hi = (vx == nx_vis - 1) ? nx : vx + pad + 1;
  const float* gm = gacc + static_cast<size_t>(model) * shots * cells;
  const float* mk = mask + static_cast<size_t>(model) * cells;
  double acc = 0.0;
  for (int z = z_lo; z < z_hi; ++z)
    for (int x = x_lo; x < x_hi; ++x) {
      const size_t c = static_cast<size_t>(z) * nx + x;
      float s = 0.0f;
      for (int k = 0; k < shots; ++k) s = s + gm[k * cells + c];
      acc += static_cast<double>(s * mk[c]);
    }
  grad[static_cast<size_t>(model) * nx_vis * nz_vis + i] = static_cast<float>(acc);
}

// Causal FIR along time for [series][nt][nrec] traces; one thread per output sample, the series'
// time window staged through shared memory in tiles.
__global__ void bandlimit_kernel(const float* __restrict__ in, const float* __restrict__ ker, int klen, int nt,
                                 int nrec, float* __restrict__ out) {
  const int s = blockIdx.z;
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  const int t = blockIdx.y;
  if (r >= nrec) return;
  const float* x = in + static_cast<size_t>(s) * nt * nrec;
  float acc = 0.0f;
  for (int k = 0; k < klen; ++k) {
    const int ts = t - (klen - 1) + k;
    if (ts >= 0) acc = acc + ker[k] * x[static_cast<size_t>(ts) * nrec + r];
  }
  out[(static_cast<size_t>(s) * nt + t) * nrec + r] = acc;
}

// Zero-phase FIR low-pass and decimation to FP16: out[s][j][r] = sum_k ker[k] in[s][j*factor + k -
// center][r] (zero outside [0, nt)), for j < nt_out. One thread per output sample; the series' time
// window is read through L1.
__global__ void decimate_kernel(const float* __restrict__ in, const float* __restrict__ ker, int klen, int center,
                                int factor, int nt, int nrec, int nt_out, __half* __restrict__ out) {
  const int s = blockIdx.z;
  const int j = blockIdx.y;
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrec) return;
  const float* x = in + static_cast<size_t>(s) * nt * nrec + r;
  const int t0 = j * factor - center;
  float acc = 0.0f;
  for (int k = 0; k < klen; ++k) {
    const int t = t0 + k;
    if (t >= 0 && t < nt) acc = acc + __ldg(&ker[k]) * __ldg(&x[static_cast<size_t>(t) * nrec]);
  }
  out[(static_cast<size_t>(s) * nt_out + j) * nrec + r] = __float2half_rn(acc);
}

__global__ void scale_kernel(const float* __restrict__ in, float alpha, size_t n, float* __restrict__ out) {
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<size_t>(gridDim.x) * blockDim.x)
    out[i] = in[i] * alpha;
}

}  // namespace

cudaError_t launch_pad_velocity(const float* vis, int models, int nx_vis, int nz_vis, int pad, float vmin, float vmax,
                                float* padded, float* mask, cudaStream_t s) {
  const int cells = (nx_vis + 2 * pad) * (nz_vis + 2 * pad);
  dim3 grid((cells + 255) / 256, models);
  pad_kernel<<<grid, 256, 0, s>>>(vis, nx_vis, nz_vis, pad, vmin, vmax, padded, mask);
  return cudaGetLastError();
}

cudaError_t launch_energy(const float* observed, int models, size_t per_model, double* energy, float* scale,
                          int* status, cudaStream_t s) {
  energy_kernel<<<models, kRedThreads, 0, s>>>(observed, per_model, energy, scale, status);
  return cudaGetLastError();
}

cudaError_t launch_residual(const float* pred, const float* observed, const float* scale, int models,
                            size_t per_model, float* residual, double* loss, cudaStream_t s) {
  residual_kernel<<<models, kRedThreads, 0, s>>>(pred, observed, scale, per_model, residual, loss);
  return cudaGetLastError();
}

cudaError_t launch_fold(const float* gacc, const float* mask, int models, int shots, int nx, int nz, int pad,
                        int nx_vis, int nz_vis, float* grad, cudaStream_t s) {
  dim3 grid((nx_vis * nz_vis + 255) / 256, models);
  fold_kernel<<<grid, 256, 0, s>>>(gacc, mask, shots, nx, nz, pad, nx_vis, nz_vis, grad);
  return cudaGetLastError();
}

cudaError_t launch_bandlimit(const float* in, const float* ker, int klen, int series, int nt, int nrec, float* out,
                             cudaStream_t s) {
  dim3 grid((nrec + 127) / 128, nt, series);
  bandlimit_kernel<<<grid, 128, 0, s>>>(in, ker, klen, nt, nrec, out);
  return cudaGetLastError();
}

cudaError_t launch_decimate(const float* in, const float* ker, int klen, int center, int factor, int series, int nt,
                            int nrec, int nt_out, void* out_half, cudaStream_t s) {
  dim3 grid((nrec + 63) / 64, nt_out, series);
  decimate_kernel<<<grid, 64, 0, s>>>(in, ker, klen, center, factor, nt, nrec, nt_out, static_cast<__half*>(out_half));
  return cudaGetLastError();
}

cudaError_t launch_scale(const float* in, float alpha, size_t n, float* out, cudaStream_t s) {
  const int blocks = static_cast<int>(std::min<size_t>((n + 255) / 256, 152 * 16));
  scale_kernel<<<blocks > 0 ? blocks : 1, 256, 0, s>>>(in, alpha, n, out);
  return cudaGetLastError();
}

}  // namespace wg
