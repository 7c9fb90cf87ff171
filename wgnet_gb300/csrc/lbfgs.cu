// FP64 reductions of the batched refinement: the L-BFGS two-loop recursion
// (python/wgnet/refine.py:41-53) and per-model dot products, one CTA per model with a fixed-order
// block reduction (deterministic).
#include <cuda_runtime.h>

#include "wave_launch.h"
#include "wgnet_gb300.h"

namespace {

constexpr int NT = 256;

__device__ double block_sum(double v, double* red) {
  red[threadIdx.x] = v;
  __syncthreads();
  for (int w = NT / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  const double s = red[0];
  __syncthreads();
  return s;
}

// History slots 0..count-1 hold the pairs oldest first. dir = -H g.
__global__ void __launch_bounds__(NT) lbfgs_kernel(const double* __restrict__ grad, const double* __restrict__ S,
                                                   const double* __restrict__ Y, const double* __restrict__ rho,
                                                   const int* __restrict__ count, int cap, long P,
                                                   double* __restrict__ dir) {
  __shared__ double red[NT];
  __shared__ double alpha[32];
  const int b = blockIdx.x;
  const int n = min(count[b], cap);
  const double* g = grad + b * P;
  double* q = dir + b * P;
  for (long i = threadIdx.x; i < P; i += NT) q[i] = g[i];
  __syncthreads();
  for (int j = n - 1; j >= 0; --j) {
    const double* s = S + (static_cast<long>(b) * cap + j) * P;
    const double* y = Y + (static_cast<long>(b) * cap + j) * P;
    double part = 0.0;
    for (long i = threadIdx.x; i < P; i += NT) part += s[i] * q[i];
    const double a = rho[b * cap + j] * block_sum(part, red);
    if (threadIdx.x == 0) alpha[j] = a;
    for (long i = threadIdx.x; i < P; i += NT) q[i] -= a * y[i];
    __syncthreads();
  }
  if (n > 0) {
    const double* s = S + (static_cast<long>(b) * cap + n - 1) * P;
    const double* y = Y + (static_cast<long>(b) * cap + n - 1) * P;
    double sy = 0.0, yy = 0.0;
    for (long i = threadIdx.x; i < P; i += NT) {
      sy += s[i] * y[i];
      yy += y[i] * y[i];
    }
    sy = block_sum(sy, red);
    yy = block_sum(yy, red);
    const double gamma = sy / fmax(yy, 1e-30);
    for (long i = threadIdx.x; i < P; i += NT) q[i] *= gamma;
    __syncthreads();
  }
  for (int j = 0; j < n; ++j) {
    const double* s = S + (static_cast<long>(b) * cap + j) * P;
    const double* y = Y + (static_cast<long>(b) * cap + j) * P;
    double part = 0.0;
    for (long i = threadIdx.x; i < P; i += NT) part += y[i] * q[i];
    const double c = alpha[j] - rho[b * cap + j] * block_sum(part, red);
    for (long i = threadIdx.x; i < P; i += NT) q[i] += s[i] * c;
    __syncthreads();
  }
  for (long i = threadIdx.x; i < P; i += NT) q[i] = -q[i];
}

__global__ void __launch_bounds__(NT) dot_kernel(const double* __restrict__ a, const double* __restrict__ b, long P,
                                                 double* __restrict__ out) {
  __shared__ double red[NT];
  const double* x = a + blockIdx.x * P;
  const double* y = b + blockIdx.x * P;
  double part = 0.0;
  for (long i = threadIdx.x; i < P; i += NT) part += x[i] * y[i];
  const double s = block_sum(part, red);
  if (threadIdx.x == 0) out[blockIdx.x] = s;
}

// Per-model misfit 0.5 sum (p - d)^2 / sum d^2 in f64 (the loss-only evaluation of
// python/wgnet/refine.py:100-104).
__global__ void __launch_bounds__(NT) misfit_kernel(const float* __restrict__ pred, const float* __restrict__ obs,
                                                    long per_model, double* __restrict__ loss) {
  __shared__ double red[NT];
  const float* p = pred + blockIdx.x * per_model;
  const float* d = obs + blockIdx.x * per_model;
  double num = 0.0, den = 0.0;
  for (long i = threadIdx.x; i < per_model; i += NT) {
    const double e = static_cast<double>(p[i]) - static_cast<double>(d[i]);
    num += e * e;
    den += static_cast<double>(d[i]) * d[i];
  }
  num = block_sum(num, red);
  den = block_sum(den, red);
  if (threadIdx.x == 0) loss[blockIdx.x] = 0.5 * num / den;
}

}  // namespace

extern "C" {

int wg_misfit_dev(const float* d_pred, const float* d_obs, int models, long per_model, double* d_loss, void* stream) {
  if (!d_pred || !d_obs || !d_loss || models < 1 || per_model < 1) return wg::report_error(WG_ERR_ARG, "misfit: bad argument");
  wg::note_launch();
  misfit_kernel<<<models, NT, 0, static_cast<cudaStream_t>(stream)>>>(d_pred, d_obs, per_model, d_loss);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? WG_OK : wg::report_error(WG_ERR_CUDA, cudaGetErrorString(e));
}


int wg_lbfgs_direction_dev(const double* d_grad, const double* d_s, const double* d_y, const double* d_rho,
                           const int* d_count, int models, int cap, long params, double* d_dir, void* stream) {
  if (!d_grad || !d_s || !d_y || !d_rho || !d_count || !d_dir || models < 1 || cap < 1 || cap > 32 || params < 1)
    return wg::report_error(WG_ERR_ARG, "lbfgs: bad argument");
  wg::note_launch();
  lbfgs_kernel<<<models, NT, 0, static_cast<cudaStream_t>(stream)>>>(d_grad, d_s, d_y, d_rho, d_count, cap, params,
                                                                     d_dir);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? WG_OK : wg::report_error(WG_ERR_CUDA, cudaGetErrorString(e));
}

int wg_dot_f64_dev(const double* d_a, const double* d_b, int models, long params, double* d_out, void* stream) {
  if (!d_a || !d_b || !d_out || models < 1 || params < 1) return wg::report_error(WG_ERR_ARG, "dot: bad argument");
  wg::note_launch();
  dot_kernel<<<models, NT, 0, static_cast<cudaStream_t>(stream)>>>(d_a, d_b, params, d_out);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? WG_OK : wg::report_error(WG_ERR_CUDA, cudaGetErrorString(e));
}

}  // extern "C"
