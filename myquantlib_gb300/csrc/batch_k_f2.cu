// batch_k_f2.cu -- instantiations of the per-class persistent batch kernel (f2).
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

cudaError_t launch_batch_f2(const BatchParams &B, int klass, bool pd, unsigned int blocks, cudaStream_t st) {
  using namespace dev;
  switch (klass) {
    case BK_F2_NV_NV: return go<2, dev::SCH_NV, dev::SCH_NV>(B, pd, blocks, st);
    case BK_F2_NV_EXACT: return go<2, dev::SCH_NV, dev::SCH_EXACT>(B, pd, blocks, st);
    case BK_F2_NV_NCI: return go<2, dev::SCH_NV, dev::SCH_NCI>(B, pd, blocks, st);
    case BK_F2_EXACT_NV: return go<2, dev::SCH_EXACT, dev::SCH_NV>(B, pd, blocks, st);
    case BK_F2_EXACT_EXACT: return go<2, dev::SCH_EXACT, dev::SCH_EXACT>(B, pd, blocks, st);
    case BK_F2_EXACT_NCI: return go<2, dev::SCH_EXACT, dev::SCH_NCI>(B, pd, blocks, st);
    case BK_F2_NCI_NV: return go<2, dev::SCH_NCI, dev::SCH_NV>(B, pd, blocks, st);
    case BK_F2_NCI_EXACT: return go<2, dev::SCH_NCI, dev::SCH_EXACT>(B, pd, blocks, st);
    case BK_F2_NCI_NCI: return go<2, dev::SCH_NCI, dev::SCH_NCI>(B, pd, blocks, st);
    default: return cudaErrorInvalidValue;
  }
}

int occupancy_batch_f2(int klass, bool pd) {
  using namespace dev;
  switch (klass) {
    case BK_F2_NV_NV: return occ<2, dev::SCH_NV, dev::SCH_NV>(pd);
    case BK_F2_NV_EXACT: return occ<2, dev::SCH_NV, dev::SCH_EXACT>(pd);
    case BK_F2_NV_NCI: return occ<2, dev::SCH_NV, dev::SCH_NCI>(pd);
    case BK_F2_EXACT_NV: return occ<2, dev::SCH_EXACT, dev::SCH_NV>(pd);
    case BK_F2_EXACT_EXACT: return occ<2, dev::SCH_EXACT, dev::SCH_EXACT>(pd);
    case BK_F2_EXACT_NCI: return occ<2, dev::SCH_EXACT, dev::SCH_NCI>(pd);
    case BK_F2_NCI_NV: return occ<2, dev::SCH_NCI, dev::SCH_NV>(pd);
    case BK_F2_NCI_EXACT: return occ<2, dev::SCH_NCI, dev::SCH_EXACT>(pd);
    case BK_F2_NCI_NCI: return occ<2, dev::SCH_NCI, dev::SCH_NCI>(pd);
    default: return 1;
  }
}

}  // namespace myql
