// GBM (0 CIR factors): BlackScholes / Merton / Kou steppers (ASVJstepper.hpp:293-305).
#include "sim_inst.cuh"
namespace myql {
cudaError_t launch_sim_f0(const SimParams &P, bool pd, cudaStream_t st) {
  return launch_sim_t<0, dev::SCH_NONE, dev::SCH_NONE>(P, pd, st);
}
}  // namespace myql
