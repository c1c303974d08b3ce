// batch_inst.cuh -- instantiations of the persistent batch kernel for one block
// size: every kernel class x path dependence x unroll depth (0, 2).  Included by
// batch_k_b64.cu, batch_k_b128.cu and batch_k_b256.cu, one block size per
// translation unit so that they compile in parallel.
#pragma once
#include "batch.cuh"

namespace myql {

template <int NF, int S1, int S2, int BLOCK>
static cudaError_t batch_go(const BatchParams &B, bool pd, int unroll, unsigned int blocks, cudaStream_t st) {
  if (pd) {
    if (unroll == 2) dev::batch_kernel<NF, S1, S2, true, BLOCK, 2><<<blocks, BLOCK, 0, st>>>(B);
    else dev::batch_kernel<NF, S1, S2, true, BLOCK, 0><<<blocks, BLOCK, 0, st>>>(B);
  } else {
    if (unroll == 2) dev::batch_kernel<NF, S1, S2, false, BLOCK, 2><<<blocks, BLOCK, 0, st>>>(B);
    else dev::batch_kernel<NF, S1, S2, false, BLOCK, 0><<<blocks, BLOCK, 0, st>>>(B);
  }
  return cudaGetLastError();
}

template <int NF, int S1, int S2, int BLOCK>
static int batch_occ(bool pd, int unroll) {
  int n = 0;
  cudaError_t e;
  if (pd)
    e = unroll == 2 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, dev::batch_kernel<NF, S1, S2, true, BLOCK, 2>, BLOCK, 0)
                    : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, dev::batch_kernel<NF, S1, S2, true, BLOCK, 0>, BLOCK, 0);
  else
    e = unroll == 2 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, dev::batch_kernel<NF, S1, S2, false, BLOCK, 2>, BLOCK, 0)
                    : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, dev::batch_kernel<NF, S1, S2, false, BLOCK, 0>, BLOCK, 0);
  return e == cudaSuccess ? n : 1;
}

// launch (blocks > 0) or occupancy query (blocks == 0, result in *occ) of one class
template <int BLOCK>
cudaError_t batch_dispatch(const BatchParams *B, int klass, bool pd, int unroll, unsigned int blocks,
                           cudaStream_t st, int *occ) {
  using namespace dev;
#define MYQL_BATCH_CASE(K, NF, A, Bs)                                          \
  case K:                                                                      \
    if (occ) {                                                                 \
      *occ = batch_occ<NF, A, Bs, BLOCK>(pd, unroll);                          \
      return cudaSuccess;                                                      \
    }                                                                          \
    return batch_go<NF, A, Bs, BLOCK>(*B, pd, unroll, blocks, st);
  switch (klass) {
    MYQL_BATCH_CASE(BK_F0, 0, SCH_NONE, SCH_NONE)
    MYQL_BATCH_CASE(BK_F1_NV, 1, SCH_NV, SCH_NONE)
    MYQL_BATCH_CASE(BK_F1_EXACT, 1, SCH_EXACT, SCH_NONE)
    MYQL_BATCH_CASE(BK_F1_NCI, 1, SCH_NCI, SCH_NONE)
    MYQL_BATCH_CASE(BK_F2_NV_NV, 2, SCH_NV, SCH_NV)
    MYQL_BATCH_CASE(BK_F2_NV_EXACT, 2, SCH_NV, SCH_EXACT)
    MYQL_BATCH_CASE(BK_F2_NV_NCI, 2, SCH_NV, SCH_NCI)
    MYQL_BATCH_CASE(BK_F2_EXACT_NV, 2, SCH_EXACT, SCH_NV)
    MYQL_BATCH_CASE(BK_F2_EXACT_EXACT, 2, SCH_EXACT, SCH_EXACT)
    MYQL_BATCH_CASE(BK_F2_EXACT_NCI, 2, SCH_EXACT, SCH_NCI)
    MYQL_BATCH_CASE(BK_F2_NCI_NV, 2, SCH_NCI, SCH_NV)
    MYQL_BATCH_CASE(BK_F2_NCI_EXACT, 2, SCH_NCI, SCH_EXACT)
    MYQL_BATCH_CASE(BK_F2_NCI_NCI, 2, SCH_NCI, SCH_NCI)
    default: return cudaErrorInvalidValue;
  }
#undef MYQL_BATCH_CASE
}

}  // namespace myql
