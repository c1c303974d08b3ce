// batch_k_f01.cu -- instantiations of the per-class persistent batch kernel (f01).
#include "batch.cuh"

namespace myql {

template <int NF, int S1, int S2>
static cudaError_t go(const BatchParams &B, bool pd, unsigned int blocks, cudaStream_t st) {
  if (pd)
    dev::batch_kernel<NF, S1, S2, true><<<blocks, kSimBlock, 0, st>>>(B);
  else
    dev::batch_kernel<NF, S1, S2, false><<<blocks, kSimBlock, 0, st>>>(B);
  return cudaGetLastError();
}

template <int NF, int S1, int S2>
static int occ(bool pd) {
  int n = 0;
  cudaError_t e = pd ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, dev::batch_kernel<NF, S1, S2, true>, kSimBlock, 0)
                     : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, dev::batch_kernel<NF, S1, S2, false>, kSimBlock, 0);
  return e == cudaSuccess ? n : 1;
}

cudaError_t launch_batch_f01(const BatchParams &B, int klass, bool pd, unsigned int blocks, cudaStream_t st) {
  using namespace dev;
  switch (klass) {
    case BK_F0: return go<0, dev::SCH_NONE, dev::SCH_NONE>(B, pd, blocks, st);
    case BK_F1_NV: return go<1, dev::SCH_NV, dev::SCH_NONE>(B, pd, blocks, st);
    case BK_F1_EXACT: return go<1, dev::SCH_EXACT, dev::SCH_NONE>(B, pd, blocks, st);
    case BK_F1_NCI: return go<1, dev::SCH_NCI, dev::SCH_NONE>(B, pd, blocks, st);
    default: return cudaErrorInvalidValue;
  }
}

int occupancy_batch_f01(int klass, bool pd) {
  using namespace dev;
  switch (klass) {
    case BK_F0: return occ<0, dev::SCH_NONE, dev::SCH_NONE>(pd);
    case BK_F1_NV: return occ<1, dev::SCH_NV, dev::SCH_NONE>(pd);
    case BK_F1_EXACT: return occ<1, dev::SCH_EXACT, dev::SCH_NONE>(pd);
    case BK_F1_NCI: return occ<1, dev::SCH_NCI, dev::SCH_NONE>(pd);
    default: return 1;
  }
}

}  // namespace myql
