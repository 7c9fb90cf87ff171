// Explicit instantiations of the resident kernels for some launch shapes (see wave_table.cu).
#include "wave_kernels.cuh"

namespace wg {

template <>
cudaError_t fwd_dispatch<4, 1024, 8>(bool traces, bool store, const FwdArgs& a, size_t smem, cudaStream_t s) {
  return fwd_dispatch_impl<4, 1024, 8>(traces, store, a, smem, s);
}

template <>
cudaError_t fwd_dispatch<4, 512, 16>(bool traces, bool store, const FwdArgs& a, size_t smem, cudaStream_t s) {
  return fwd_dispatch_impl<4, 512, 16>(traces, store, a, smem, s);
}

template <>
cudaError_t adj_dispatch<4, 1024, 4>(const AdjArgs& a, size_t smem, cudaStream_t s) {
  return adj_dispatch_impl<4, 1024, 4>(a, smem, s);
}

template <>
cudaError_t adj_dispatch<4, 1024, 8>(const AdjArgs& a, size_t smem, cudaStream_t s) {
  return adj_dispatch_impl<4, 1024, 8>(a, smem, s);
}

template <>
cudaError_t adj_dispatch<4, 512, 16>(const AdjArgs& a, size_t smem, cudaStream_t s) {
  return adj_dispatch_impl<4, 512, 16>(a, smem, s);
}

}  // namespace wg
