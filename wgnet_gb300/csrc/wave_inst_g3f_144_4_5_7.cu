// Explicit instantiation of the generation-3 fast-arithmetic forward kernels for one launch shape (see
// wave_table.cu).
#include "wave_kernels3.cuh"

namespace wg {

template <>
cudaError_t fwd3f_dispatch<144, 12, 4, 5, 7, 2>(bool traces, bool store, const FwdArgs& a, size_t smem, cudaStream_t s) {
  return fwd3_dispatch_impl<144, 12, 4, 5, 7, 2, true>(traces, store, a, smem, s);
}

}  // namespace wg
