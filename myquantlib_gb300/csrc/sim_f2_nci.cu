// Two CIR factors with VolScheme1 = SchemeNCI: double Heston / Bates steppers
// (ASVJstepper.hpp:324-339).
#include "sim_inst.cuh"
namespace myql {
cudaError_t launch_sim_f2_nci(const SimParams &P, int s2, bool pd, cudaStream_t st) {
  switch (s2) {
    case dev::SCH_NV: return launch_sim_t<2, dev::SCH_NCI, dev::SCH_NV>(P, pd, st);
    case dev::SCH_EXACT: return launch_sim_t<2, dev::SCH_NCI, dev::SCH_EXACT>(P, pd, st);
    case dev::SCH_NCI: return launch_sim_t<2, dev::SCH_NCI, dev::SCH_NCI>(P, pd, st);
    default: return cudaErrorInvalidValue;
  }
}
}  // namespace myql
