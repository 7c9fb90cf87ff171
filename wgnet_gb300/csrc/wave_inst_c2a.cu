// Explicit instantiations of the resident kernels for some launch shapes (see wave_table.cu).
#include "wave_kernels.cuh"

namespace wg {

template <>
cudaError_t fwd_dispatch<2, 1024, 6>(bool traces, bool store, const FwdArgs& a, size_t smem, cudaStream_t s) {
  return fwd_dispatch_impl<2, 1024, 6>(traces, store, a, smem, s);
}

template <>
cudaError_t adj_dispatch<2, 1024, 6>(const AdjArgs& a, size_t smem, cudaStream_t s) {
  return adj_dispatch_impl<2, 1024, 6>(a, smem, s);
}

template <>
cudaError_t fwd_dispatch<2, 512, 12>(bool traces, bool store, const FwdArgs& a, size_t smem, cudaStream_t s) {
  return fwd_dispatch_impl<2, 512, 12>(traces, store, a, smem, s);
}

template <>
cudaError_t adj_dispatch<2, 512, 12>(const AdjArgs& a, size_t smem, cudaStream_t s) {
  return adj_dispatch_impl<2, 512, 12>(a, smem, s);
}

}  // namespace wg
