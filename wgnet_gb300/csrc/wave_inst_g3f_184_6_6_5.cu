// Explicit instantiation of the generation-3 fast-arithmetic forward kernels for one launch shape (see
// wave_table.cu).
#include "wave_kernels3.cuh"

namespace wg {

template <>
cudaError_t fwd3f_dispatch<184, 12, 6, 6, 5, 3>(bool traces, bool store, const FwdArgs& a, size_t smem, cudaStream_t s) {
  return fwd3_dispatch_impl<184, 12, 6, 6, 5, 3, true>(traces, store, a, smem, s);
}

}  // namespace wg
