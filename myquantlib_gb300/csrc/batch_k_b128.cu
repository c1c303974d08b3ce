// batch_k_b128.cu -- the persistent batch kernels with 128 threads per block.
#include "batch_inst.cuh"

namespace myql {

cudaError_t batch_dispatch_b128(const BatchParams *B, int klass, bool pd, int unroll, unsigned int blocks,
                               cudaStream_t st, int *occ) {
  return batch_dispatch<128>(B, klass, pd, unroll, blocks, st, occ);
}

}  // namespace myql
