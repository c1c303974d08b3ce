// MLMC level kernels, 0 and 1 CIR factors.
#include "mlmc.cuh"
namespace myql {
cudaError_t launch_mlmc_f01(const MlmcParams &M, int s1, bool pd, cudaStream_t st) {
  if (M.sim.n_factors == 0) return launch_mlmc_t<0, dev::SCH_NONE, dev::SCH_NONE>(M, pd, st);
  switch (s1) {
    case dev::SCH_NV: return launch_mlmc_t<1, dev::SCH_NV, dev::SCH_NONE>(M, pd, st);
    case dev::SCH_EXACT: return launch_mlmc_t<1, dev::SCH_EXACT, dev::SCH_NONE>(M, pd, st);
    case dev::SCH_NCI: return launch_mlmc_t<1, dev::SCH_NCI, dev::SCH_NONE>(M, pd, st);
    default: return cudaErrorInvalidValue;
  }
}
}  // namespace myql
