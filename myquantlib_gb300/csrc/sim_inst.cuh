// sim_inst.cuh -- launch helper shared by the simulate instantiation units.
#pragma once
#include "simulate.cuh"

namespace myql {
template <int NF, int S1, int S2>
cudaError_t launch_sim_t(const SimParams &P, bool path_dep, cudaStream_t stream) {
  const unsigned int grid = (P.n_streams + kSimBlock - 1) / kSimBlock;
  if constexpr (NF >= 1 && S1 != dev::SCH_EXACT && S2 != dev::SCH_EXACT) {
    // Full Greeks of a European: every simulated scenario in lockstep
    constexpr int n_sc_full = NF == 2 ? 9 : 7;
    if (!path_dep && P.n_sc == n_sc_full) {
      if constexpr (NF == 1 && S1 == dev::SCH_NCI) {
        if (P.lock_merge && P.lock_precise) {  // myql_ctx_set_precise_theta
          dev::simulate_lockstep_kernel<NF, S1, S2, n_sc_full - 2, true, true><<<grid, kSimBlock, 0, stream>>>(P);
          return cudaGetLastError();
        }
      }
      if constexpr (S1 == dev::SCH_NCI && (NF == 1 || S2 == dev::SCH_NCI)) {
        if (P.lock_merge) {
          dev::simulate_lockstep_kernel<NF, S1, S2, n_sc_full - 2, true><<<grid, kSimBlock, 0, stream>>>(P);
          return cudaGetLastError();
        }
      }
      dev::simulate_lockstep_kernel<NF, S1, S2, n_sc_full - 2><<<grid, kSimBlock, 0, stream>>>(P);
      return cudaGetLastError();
    }
  }
  if (path_dep)
    dev::simulate_kernel<NF, S1, S2, true><<<grid, kSimBlock, 0, stream>>>(P);
  else
    dev::simulate_kernel<NF, S1, S2, false><<<grid, kSimBlock, 0, stream>>>(P);
  return cudaGetLastError();
}
}  // namespace myql
