// MLMC level kernels, 2 CIR factors.
#include "mlmc.cuh"
namespace myql {
template <int S1>
static cudaError_t f2(const MlmcParams &M, int s2, bool pd, cudaStream_t st) {
  switch (s2) {
    case dev::SCH_NV: return launch_mlmc_t<2, S1, dev::SCH_NV>(M, pd, st);
    case dev::SCH_EXACT: return launch_mlmc_t<2, S1, dev::SCH_EXACT>(M, pd, st);
    case dev::SCH_NCI: return launch_mlmc_t<2, S1, dev::SCH_NCI>(M, pd, st);
    default: return cudaErrorInvalidValue;
  }
}
cudaError_t launch_mlmc_f2(const MlmcParams &M, int s1, int s2, bool pd, cudaStream_t st) {
  switch (s1) {
    case dev::SCH_NV: return f2<dev::SCH_NV>(M, s2, pd, st);
    case dev::SCH_EXACT: return f2<dev::SCH_EXACT>(M, s2, pd, st);
    case dev::SCH_NCI: return f2<dev::SCH_NCI>(M, s2, pd, st);
    default: return cudaErrorInvalidValue;
  }
}
}  // namespace myql
