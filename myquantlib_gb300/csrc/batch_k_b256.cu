// batch_k_b256.cu -- the persistent batch kernels with 256 threads per block.
#include "batch_inst.cuh"

namespace myql {

cudaError_t batch_dispatch_b256(const BatchParams *B, int klass, bool pd, int unroll, unsigned int blocks,
                               cudaStream_t st, int *occ) {
  return batch_dispatch<256>(B, klass, pd, unroll, blocks, st, occ);
}

}  // namespace myql
