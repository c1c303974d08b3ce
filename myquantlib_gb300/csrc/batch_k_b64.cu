// batch_k_b64.cu -- the persistent batch kernels with 64 threads per block.
#include "batch_inst.cuh"

namespace myql {

cudaError_t batch_dispatch_b64(const BatchParams *B, int klass, bool pd, int unroll, unsigned int blocks,
                               cudaStream_t st, int *occ) {
  return batch_dispatch<64>(B, klass, pd, unroll, blocks, st, occ);
}

}  // namespace myql
