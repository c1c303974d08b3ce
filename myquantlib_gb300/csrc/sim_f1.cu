// One CIR factor: Heston / Bates / Bates-Kou steppers (ASVJstepper.hpp:310-319).
#include "sim_inst.cuh"
namespace myql {
cudaError_t launch_sim_f1(const SimParams &P, int s1, bool pd, cudaStream_t st) {
  switch (s1) {
    case dev::SCH_NV: return launch_sim_t<1, dev::SCH_NV, dev::SCH_NONE>(P, pd, st);
    case dev::SCH_EXACT: return launch_sim_t<1, dev::SCH_EXACT, dev::SCH_NONE>(P, pd, st);
    case dev::SCH_NCI: return launch_sim_t<1, dev::SCH_NCI, dev::SCH_NONE>(P, pd, st);
    default: return cudaErrorInvalidValue;
  }
}
}  // namespace myql
