// Explicit instantiations of the resident kernels for some launch shapes (see wave_table.cu).
#include "wave_kernels.cuh"

namespace wg {

template <>
cudaError_t fwd_dispatch<2, 1024, 10>(bool traces, bool store, const FwdArgs& a, size_t smem, cudaStream_t s) {
  return fwd_dispatch_impl<2, 1024, 10>(traces, store, a, smem, s);
}

template <>
cudaError_t fwd_dispatch<2, 1024, 16>(bool traces, bool store, const FwdArgs& a, size_t smem, cudaStream_t s) {
  return fwd_dispatch_impl<2, 1024, 16>(traces, store, a, smem, s);
}

}  // namespace wg
