// Explicit instantiations of the generation-2 forward kernel (see wave_table.cu).
#include "wave_kernels2.cuh"

namespace wg {

template <>
cudaError_t fwd2_dispatch<2, 4, 14, 1>(bool traces, bool store, const FwdArgs& a, size_t smem, cudaStream_t s) {
  return fwd2_dispatch_impl<2, 4, 14, 1>(traces, store, a, smem, s);
}

template <>
cudaError_t fwd2_dispatch<2, 8, 7, 1>(bool traces, bool store, const FwdArgs& a, size_t smem, cudaStream_t s) {
  return fwd2_dispatch_impl<2, 8, 7, 1>(traces, store, a, smem, s);
}

template <>
cudaError_t fwd2_dispatch<1, 8, 14, 1>(bool traces, bool store, const FwdArgs& a, size_t smem, cudaStream_t s) {
  return fwd2_dispatch_impl<1, 8, 14, 1>(traces, store, a, smem, s);
}

template <>
cudaError_t fwd2_dispatch<4, 4, 7, 1>(bool traces, bool store, const FwdArgs& a, size_t smem, cudaStream_t s) {
  return fwd2_dispatch_impl<4, 4, 7, 1>(traces, store, a, smem, s);
}

template <>
cudaError_t fwd2_dispatch<4, 2, 14, 1>(bool traces, bool store, const FwdArgs& a, size_t smem, cudaStream_t s) {
  return fwd2_dispatch_impl<4, 2, 14, 1>(traces, store, a, smem, s);
}

template <>
cudaError_t fwd2_dispatch<4, 5, 7, 2>(bool traces, bool store, const FwdArgs& a, size_t smem, cudaStream_t s) {
  return fwd2_dispatch_impl<4, 5, 7, 2>(traces, store, a, smem, s);
}

template <>
cudaError_t fwd2_dispatch<4, 5, 9, 2>(bool traces, bool store, const FwdArgs& a, size_t smem, cudaStream_t s) {
  return fwd2_dispatch_impl<4, 5, 9, 2>(traces, store, a, smem, s);
}

}  // namespace wg
