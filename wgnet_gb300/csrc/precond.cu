// Kernels of the learned update network (a dilated residual conv net on the 70x70 model grid):
// lowering of 3x3 convolutions to the tensor-core GEMM (im2col / col2im), layout transposes, the
// elementwise glue of the residual blocks, input features, the training loss and the Adam update.
// No reference counterpart: WGNet's refine() (python/wgnet/refine.py:41-169) has no learned part.
//
// Layouts: activations [B][H][W][C] (channels contiguous); im2col columns [M][Kp] with
// M = B H W, k = tap * C + c (tap = 3 ky + kx), zero for k >= 9 C; weights [N][Kp] (GEMM B operand)
// and their transpose [Kp][N] (the data-gradient GEMM's B operand). BF16 where a GEMM reads it,
// FP32 elsewhere.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "wave_launch.h"
#include "wgnet_gb300.h"

namespace {

__global__ void im2col_kernel(const __nv_bfloat16* __restrict__ act, int B, int H, int W, int C, int dil, int Kp,
                              __nv_bfloat16* __restrict__ col) {
  const long M = static_cast<long>(B) * H * W;
  const int kv = Kp / 8;
  const long i = blockIdx.x * static_cast<long>(blockDim.x) + threadIdx.x;
  if (i >= M * kv) return;
  const long m = i / kv;
  const int k8 = static_cast<int>(i % kv) * 8;
  uint4 v = make_uint4(0, 0, 0, 0);
  if (k8 < 9 * C) {
    const int tap = k8 / C, c = k8 % C;
    const int x = static_cast<int>(m % W), y = static_cast<int>((m / W) % H);
    const long b = m / (static_cast<long>(W) * H);
    const int ys = y + (tap / 3 - 1) * dil, xs = x + (tap % 3 - 1) * dil;
    if (ys >= 0 && ys < H && xs >= 0 && xs < W)
      v = *reinterpret_cast<const uint4*>(act + ((b * H + ys) * W + xs) * C + c);
  }
  *reinterpret_cast<uint4*>(col + m * Kp + k8) = v;
}

// dact[m][c] (+)= sum over taps of dcol[m'][tap C + c], m' the pixel whose tap reads m.
__global__ void col2im_kernel(const float* __restrict__ dcol, int B, int H, int W, int C, int dil, int Kp,
                              float* __restrict__ dact, int accumulate) {
  const long M = static_cast<long>(B) * H * W;
  const long i = blockIdx.x * static_cast<long>(blockDim.x) + threadIdx.x;
  if (i >= M * C) return;
  const long m = i / C;
  const int c = static_cast<int>(i % C);
  const int x = static_cast<int>(m % W), y = static_cast<int>((m / W) % H);
  const long b = m / (static_cast<long>(W) * H);
  float acc = 0.0f;
#pragma unroll
  for (int tap = 0; tap < 9; ++tap) {
    const int ys = y - (tap / 3 - 1) * dil, xs = x - (tap % 3 - 1) * dil;
    if (ys >= 0 && ys < H && xs >= 0 && xs < W) acc += dcol[((b * H + ys) * W + xs) * Kp + tap * C + c];
  }
  dact[i] = accumulate ? dact[i] + acc : acc;
}

// out[c][r] = in[r][c] for a [R][Cc] bf16 matrix (32 x 32 tiles through shared memory).
__global__ void transpose_bf16_kernel(const __nv_bfloat16* __restrict__ in, long R, int Cc,
                                      __nv_bfloat16* __restrict__ out) {
  __shared__ __nv_bfloat16 t[32][33];
  const long r0 = static_cast<long>(blockIdx.x) * 32;
  const int c0 = blockIdx.y * 32;
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const long r = r0 + k;
    const int c = c0 + threadIdx.x;
    t[k][threadIdx.x] = (r < R && c < Cc) ? in[r * Cc + c] : __float2bfloat16(0.0f);
  }
  __syncthreads();
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const int c = c0 + k;
    const long r = r0 + threadIdx.x;
    if (c < Cc && r < R) out[static_cast<long>(c) * R + r] = t[threadIdx.x][k];
  }
}

// out = bf16(relu ? max(x, 0) : x); column slice: rows of ld floats, first `cols` used, out [rows][cols]
__global__ void cast_bf16_kernel(const float* __restrict__ x, long rows, int ld, int cols, int relu,
                                 __nv_bfloat16* __restrict__ out) {
  const long i = blockIdx.x * static_cast<long>(blockDim.x) + threadIdx.x;
  if (i >= rows * cols) return;
  float v = x[(i / cols) * ld + i % cols];
  if (relu) v = fmaxf(v, 0.0f);
  out[i] = __float2bfloat16(v);
}

// out = a + b (fp32), and its bf16 copy when out_bf16 != null
__global__ void add_kernel(const float* __restrict__ a, const float* __restrict__ b, long n, float* __restrict__ out,
                           __nv_bfloat16* __restrict__ out_bf16) {
  const long i = blockIdx.x * static_cast<long>(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  const float v = a[i] + b[i];
  out[i] = v;
  if (out_bf16) out_bf16[i] = __float2bfloat16(v);
}

// out = d where mask > 0 else 0 (the ReLU derivative from the stored bf16 activation)
__global__ void relu_grad_kernel(const float* __restrict__ d, const __nv_bfloat16* __restrict__ mask, long n,
                                 float* __restrict__ out) {
  const long i = blockIdx.x * static_cast<long>(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  out[i] = __bfloat162float(mask[i]) > 0.0f ? d[i] : 0.0f;
}

// Per-sample RMS of the gradient (f64 reduction, one block per sample).
__global__ void rms_kernel(const float* __restrict__ g, int P, float* __restrict__ rms) {
  __shared__ double red[256];
  const float* x = g + static_cast<long>(blockIdx.x) * P;
  double s = 0.0;
  for (int i = threadIdx.x; i < P; i += blockDim.x) s += static_cast<double>(x[i]) * x[i];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) rms[blockIdx.x] = static_cast<float>(sqrt(red[0] / P));
}

// Input features [B][H][W][8]: (v - 3) km/s, g / rms(g), one-hot band (4), depth z / H, 0.
__global__ void features_kernel(const float* __restrict__ vel_km, const float* __restrict__ grad,
                                const float* __restrict__ rms, const int* __restrict__ band, int B, int H, int W,
                                __nv_bfloat16* __restrict__ out) {
  const long i = blockIdx.x * static_cast<long>(blockDim.x) + threadIdx.x;
  const long n = static_cast<long>(B) * H * W;
  if (i >= n) return;
  const int b = static_cast<int>(i / (static_cast<long>(H) * W));
  const int y = static_cast<int>((i / W) % H);
  const float r = rms[b];
  const int bd = band[b];
  float f[8];
  f[0] = vel_km[i] - 3.0f;
  f[1] = r > 0.0f ? grad[i] / r : 0.0f;
  for (int k = 0; k < 4; ++k) f[2 + k] = (bd == k) ? 1.0f : 0.0f;
  f[6] = static_cast<float>(y) / static_cast<float>(H);
  f[7] = 0.0f;
  __align__(16) __nv_bfloat16 o[8];
  for (int k = 0; k < 8; ++k) o[k] = __float2bfloat16(f[k]);
  *reinterpret_cast<uint4*>(out + i * 8) = *reinterpret_cast<const uint4*>(o);
}

// Mean squared error of scale * out[m][0] against target[m]; writes dL/d out[m][0] (other columns
// of the row untouched: they stay zero) and accumulates the loss (f64) per block into loss.
__global__ void mse_kernel(const float* __restrict__ out, int ld, const float* __restrict__ target, float scale,
                           long M, double* __restrict__ loss, float* __restrict__ dout) {
  __shared__ double red[256];
  const long i = blockIdx.x * static_cast<long>(blockDim.x) + threadIdx.x;
  double l = 0.0;
  if (i < M) {
    const float e = scale * out[i * ld] - target[i];
    l = static_cast<double>(e) * e;
    dout[i * ld] = 2.0f * e * scale / static_cast<float>(M);
  }
  red[threadIdx.x] = l;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) atomicAdd(loss, red[0] / static_cast<double>(M));
}

// Adam on FP32 master weights w32 [N][Kp]; the gradient is the sum of the split-K partials of the
// transposed weight gradient [S][Kp][N]. Writes the BF16 weights [N][Kp] and their transpose.
__global__ void adam_kernel(const float* __restrict__ partial, int S, int N, int Kp, float* __restrict__ w32,
                            float* __restrict__ m1, float* __restrict__ m2, float lr, float b1, float b2, float eps,
                            float c1, float c2, __nv_bfloat16* __restrict__ w, __nv_bfloat16* __restrict__ wt) {
  const long i = blockIdx.x * static_cast<long>(blockDim.x) + threadIdx.x;
  if (i >= static_cast<long>(N) * Kp) return;
  const int n = static_cast<int>(i / Kp), k = static_cast<int>(i % Kp);
  float g = 0.0f;
  if (partial) {
    for (int s = 0; s < S; ++s) g += partial[(static_cast<long>(s) * Kp + k) * N + n];
    const float a = b1 * m1[i] + (1.0f - b1) * g;
    const float v = b2 * m2[i] + (1.0f - b2) * g * g;
    m1[i] = a;
    m2[i] = v;
    w32[i] -= lr * (a / c1) / (sqrtf(v / c2) + eps);
  }
  const __nv_bfloat16 q = __float2bfloat16(w32[i]);
  w[i] = q;
  wt[static_cast<long>(k) * N + n] = q;
}

inline unsigned blocks(long n, int t) { return static_cast<unsigned>((n + t - 1) / t); }

#define PC_LAUNCH(...)                                                         \
  do {                                                                         \
    wg::note_launch();                                                         \
    __VA_ARGS__;                                                               \
    cudaError_t e_ = cudaGetLastError();                                       \
    if (e_ != cudaSuccess) return wg::report_error(WG_ERR_CUDA, cudaGetErrorString(e_)); \
    return WG_OK;                                                              \
  } while (0)

}  // namespace

extern "C" {

int wg_pc_im2col(const void* act, int B, int H, int W, int C, int dil, int Kp, void* col, void* stream) {
  if (!act || !col || B < 1 || H < 1 || W < 1 || C < 8 || C % 8 || Kp % 64 || Kp < 9 * C || dil < 1)
    return wg::report_error(WG_ERR_ARG, "im2col: bad shape");
  const long n = static_cast<long>(B) * H * W * (Kp / 8);
  PC_LAUNCH(im2col_kernel<<<blocks(n, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      static_cast<const __nv_bfloat16*>(act), B, H, W, C, dil, Kp, static_cast<__nv_bfloat16*>(col)));
}

int wg_pc_col2im(const float* dcol, int B, int H, int W, int C, int dil, int Kp, float* dact, int accumulate,
                 void* stream) {
  if (!dcol || !dact || B < 1 || C < 1 || Kp < 9 * C || dil < 1) return wg::report_error(WG_ERR_ARG, "col2im: bad shape");
  const long n = static_cast<long>(B) * H * W * C;
  PC_LAUNCH(col2im_kernel<<<blocks(n, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(dcol, B, H, W, C, dil, Kp,
                                                                                        dact, accumulate));
}

int wg_pc_transpose_bf16(const void* in, long R, int Cc, void* out, void* stream) {
  if (!in || !out || R < 1 || Cc < 1) return wg::report_error(WG_ERR_ARG, "transpose: bad shape");
  dim3 grid(static_cast<unsigned>((R + 31) / 32), static_cast<unsigned>((Cc + 31) / 32));
  PC_LAUNCH(transpose_bf16_kernel<<<grid, dim3(32, 8), 0, static_cast<cudaStream_t>(stream)>>>(
      static_cast<const __nv_bfloat16*>(in), R, Cc, static_cast<__nv_bfloat16*>(out)));
}

int wg_pc_cast_bf16(const float* x, long rows, int ld, int cols, int relu, void* out, void* stream) {
  if (!x || !out || rows < 1 || cols < 1 || ld < cols) return wg::report_error(WG_ERR_ARG, "cast: bad shape");
  PC_LAUNCH(cast_bf16_kernel<<<blocks(rows * cols, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      x, rows, ld, cols, relu, static_cast<__nv_bfloat16*>(out)));
}

int wg_pc_add(const float* a, const float* b, long n, float* out, void* out_bf16, void* stream) {
  if (!a || !b || !out || n < 1) return wg::report_error(WG_ERR_ARG, "add: bad argument");
  PC_LAUNCH(add_kernel<<<blocks(n, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      a, b, n, out, static_cast<__nv_bfloat16*>(out_bf16)));
}

int wg_pc_relu_grad(const float* d, const void* mask, long n, float* out, void* stream) {
  if (!d || !mask || !out || n < 1) return wg::report_error(WG_ERR_ARG, "relu_grad: bad argument");
  PC_LAUNCH(relu_grad_kernel<<<blocks(n, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      d, static_cast<const __nv_bfloat16*>(mask), n, out));
}

int wg_pc_features(const float* vel_km, const float* grad, const int* band, int B, int H, int W, float* rms,
                   void* out, void* stream) {
  if (!vel_km || !grad || !band || !rms || !out || B < 1) return wg::report_error(WG_ERR_ARG, "features: bad argument");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  wg::note_launch();
  rms_kernel<<<B, 256, 0, st>>>(grad, H * W, rms);
  const long n = static_cast<long>(B) * H * W;
  PC_LAUNCH(features_kernel<<<blocks(n, 256), 256, 0, st>>>(vel_km, grad, rms, band, B, H, W,
                                                            static_cast<__nv_bfloat16*>(out)));
}

int wg_pc_mse(const float* out, int ld, const float* target, float scale, long M, double* loss, float* dout,
              void* stream) {
  if (!out || !target || !loss || !dout || M < 1) return wg::report_error(WG_ERR_ARG, "mse: bad argument");
  PC_LAUNCH(mse_kernel<<<blocks(M, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(out, ld, target, scale, M, loss,
                                                                                     dout));
}

int wg_pc_adam(const float* partial, int S, int N, int Kp, float* w32, float* m1, float* m2, float lr, float b1,
               float b2, float eps, int step, void* w, void* wt, void* stream) {
  if (!w32 || !m1 || !m2 || !w || !wt || N < 1 || Kp < 1 || (partial && (S < 1 || step < 1)))
    return wg::report_error(WG_ERR_ARG, "adam: bad argument");
  const float c1 = partial ? 1.0f - powf(b1, static_cast<float>(step)) : 1.0f;
  const float c2 = partial ? 1.0f - powf(b2, static_cast<float>(step)) : 1.0f;
  const long n = static_cast<long>(N) * Kp;
  PC_LAUNCH(adam_kernel<<<blocks(n, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      partial, S, N, Kp, w32, m1, m2, lr, b1, b2, eps, c1, c2, static_cast<__nv_bfloat16*>(w),
      static_cast<__nv_bfloat16*>(wt)));
}

}  // extern "C"
