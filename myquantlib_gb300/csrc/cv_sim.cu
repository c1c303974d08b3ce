// cv_sim.cu -- path simulation for the control variate: the same stepping as
// simulate_kernel (one thread per xoshiro stream, paths s, s + S, ...), with
// every path stepped (per-step jumps and GBM increments) and a CvHook that
// records the features at the hedge times and the centred martingale
// increments of every hedge interval; the discounted payoff of the path is
// evaluated in place.
#include "cv.cuh"

namespace myql {
namespace dev {

template <int NF, int S1, int S2>
__global__ void __launch_bounds__(kSimBlock) cv_sim_kernel(const __grid_constant__ CvSimParams P) {
  const unsigned int s = blockIdx.x * kSimBlock + threadIdx.x;
  const unsigned int S = P.sim.n_streams;
  if (s >= S) return;
  Xo rng;
  rng.a = P.sim.states[s];
  rng.b = P.sim.states[(size_t)S + s];
  rng.c = P.sim.states[2 * (size_t)S + s];
  rng.d = P.sim.states[3 * (size_t)S + s];
  unsigned int caphits = 0, fallbacks = 0;
  const float K = (float)P.pay.strikes[0];
  const float df = (float)P.df;
  for (unsigned long long i = P.path_begin + s; i < P.path_end; i += S) {
    const unsigned long long li = i - P.path_begin;
    const unsigned long long pb = li >> 7;
    CvHook h;
    h.P = &P.fc;
    h.lane = (uint32_t)(li & 127u);
    h.tile0 = P.feat + pb * (unsigned long long)P.n_hedge * kCvTileBytes;
    h.dm0 = P.dM + pb * (unsigned long long)P.n_hedge * 128ull + h.lane;
    h.he = P.hedge_every;
    h.n = P.sim.n_steps;
    h.dt = P.sim.sc[0].dt;
    float r[kMaxFields];
    sim_path_h<NF, S1, S2, true>(P.sim, P.sim.sc[0], rng, r, caphits, fallbacks, h);
    const PathView v = record_view(P.pay, r);
    P.Y[li] = df * scenario_tri(P.pay, v, K, false).v;
  }
  P.sim.states[s] = rng.a;
  P.sim.states[(size_t)S + s] = rng.b;
  P.sim.states[2 * (size_t)S + s] = rng.c;
  P.sim.states[3 * (size_t)S + s] = rng.d;
  if (caphits) atomicAdd(P.sim.status, caphits);
  if (fallbacks) atomicAdd(P.sim.status + 1, fallbacks);
}

}  // namespace dev

cudaError_t launch_cv_sim(const CvSimParams &P, int klass, cudaStream_t st) {
  using namespace dev;
  const unsigned int blocks = (unsigned int)((P.sim.n_streams + kSimBlock - 1) / kSimBlock);
  switch (klass) {
    case BK_F0: cv_sim_kernel<0, SCH_NONE, SCH_NONE><<<blocks, kSimBlock, 0, st>>>(P); break;
    case BK_F1_NV: cv_sim_kernel<1, SCH_NV, SCH_NONE><<<blocks, kSimBlock, 0, st>>>(P); break;
    case BK_F1_EXACT: cv_sim_kernel<1, SCH_EXACT, SCH_NONE><<<blocks, kSimBlock, 0, st>>>(P); break;
    case BK_F1_NCI: cv_sim_kernel<1, SCH_NCI, SCH_NONE><<<blocks, kSimBlock, 0, st>>>(P); break;
    case BK_F2_NV_NV: cv_sim_kernel<2, SCH_NV, SCH_NV><<<blocks, kSimBlock, 0, st>>>(P); break;
    case BK_F2_NV_EXACT: cv_sim_kernel<2, SCH_NV, SCH_EXACT><<<blocks, kSimBlock, 0, st>>>(P); break;
    case BK_F2_NV_NCI: cv_sim_kernel<2, SCH_NV, SCH_NCI><<<blocks, kSimBlock, 0, st>>>(P); break;
    case BK_F2_EXACT_NV: cv_sim_kernel<2, SCH_EXACT, SCH_NV><<<blocks, kSimBlock, 0, st>>>(P); break;
    case BK_F2_EXACT_EXACT: cv_sim_kernel<2, SCH_EXACT, SCH_EXACT><<<blocks, kSimBlock, 0, st>>>(P); break;
    case BK_F2_EXACT_NCI: cv_sim_kernel<2, SCH_EXACT, SCH_NCI><<<blocks, kSimBlock, 0, st>>>(P); break;
    case BK_F2_NCI_NV: cv_sim_kernel<2, SCH_NCI, SCH_NV><<<blocks, kSimBlock, 0, st>>>(P); break;
    case BK_F2_NCI_EXACT: cv_sim_kernel<2, SCH_NCI, SCH_EXACT><<<blocks, kSimBlock, 0, st>>>(P); break;
    case BK_F2_NCI_NCI: cv_sim_kernel<2, SCH_NCI, SCH_NCI><<<blocks, kSimBlock, 0, st>>>(P); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace myql
