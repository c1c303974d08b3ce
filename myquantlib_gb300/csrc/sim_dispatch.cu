// sim_dispatch.cu -- maps (factors, schemes, path dependence) to the compiled
// simulate_kernel instantiation.
#include "simulate.cuh"

namespace myql {
cudaError_t launch_sim_f0(const SimParams &P, bool pd, cudaStream_t st);
cudaError_t launch_sim_f1(const SimParams &P, int s1, bool pd, cudaStream_t st);
cudaError_t launch_sim_f2_nv(const SimParams &P, int s2, bool pd, cudaStream_t st);
cudaError_t launch_sim_f2_exact(const SimParams &P, int s2, bool pd, cudaStream_t st);
cudaError_t launch_sim_f2_nci(const SimParams &P, int s2, bool pd, cudaStream_t st);

cudaError_t launch_simulate(const SimParams &P, int s1, int s2, bool path_dep,
                            cudaStream_t stream) {
  switch (P.n_factors) {
    case 0: return launch_sim_f0(P, path_dep, stream);
    case 1: return launch_sim_f1(P, s1, path_dep, stream);
    case 2:
      switch (s1) {
        case dev::SCH_NV: return launch_sim_f2_nv(P, s2, path_dep, stream);
        case dev::SCH_EXACT: return launch_sim_f2_exact(P, s2, path_dep, stream);
        case dev::SCH_NCI: return launch_sim_f2_nci(P, s2, path_dep, stream);
        default: return cudaErrorInvalidValue;
      }
    default: return cudaErrorInvalidValue;
  }
}
}  // namespace myql
