// mlmc_cv.cu -- MLMC level kernels with the neural control variate: the level
// kernel of mlmc.cuh (one persistent stream pool, paths s, s + U, ...) with the
// path observers of cv.cuh.  Each path writes its feature rows, its martingale
// increments (level 0: of the plain path; level l > 0: fine minus coarse) and
// its discounted level difference; the MLP and the reductions follow on the host
// side.  Every path is stepped (per-step jumps).
#include "cv.cuh"

namespace myql {
namespace dev {

template <int NF, int S1, int S2>
__global__ void __launch_bounds__(kSimBlock) mlmc_cv_level_kernel(const __grid_constant__ MlmcCvParams Q) {
  const MlmcParams &M = Q.M;
  const SimParams &P = M.sim;
  const unsigned int s = blockIdx.x * kSimBlock + threadIdx.x;
  const unsigned int S = P.n_streams, U = M.n_used;
  if (s >= U) return;
  unsigned int caphits = 0, fallbacks = 0;
  Xo rng;
  rng.a = P.states[s];
  rng.b = P.states[(size_t)S + s];
  rng.c = P.states[2 * (size_t)S + s];
  rng.d = P.states[3 * (size_t)S + s];
  const float K = (float)M.pay.strikes[0];
  const float df = (float)Q.df;
  for (unsigned long long i = s; i < M.dN; i += U) {
    const unsigned long long pb = i >> 7;
    const uint32_t lane = (uint32_t)(i & 127u);
    uint8_t *tile0 = Q.feat + pb * (unsigned long long)Q.n_hedge * kCvTileBytes;
    float *dm0 = Q.dM + pb * (unsigned long long)Q.n_hedge * 128ull + lane;
    float y;
    if (M.level == 0) {
      CvHook h;
      h.P = &Q.fine;
      h.tile0 = tile0;
      h.dm0 = dm0;
      h.lane = lane;
      h.he = Q.hedge_every;
      h.n = P.n_steps;
      h.dt = P.sc[0].dt;
      float r[kMaxFields];
      sim_path_h<NF, S1, S2, true>(P, P.sc[0], rng, r, caphits, fallbacks, h);
      y = record_price(M.pay, r, 0, K);
    } else {
      MlmcCvHook h;
      h.F = &Q.fine;
      h.Cc = &Q.coarse;
      h.tile0 = tile0;
      h.dm0 = dm0;
      h.lane = lane;
      h.hc = Q.hedge_every;
      h.nc = M.n_coarse;
      h.dtf = P.sc[0].dt;
      float rf[kMaxFields], rc[kMaxFields];
      coupled_path<NF, S1, S2, true, MlmcCvHook>(P, M.n_coarse, rng, rf, rc, caphits, fallbacks, h);
      y = record_price(M.pay, rf, 0, K) - record_price(M.pay, rc, 1, K);
    }
    Q.Y[i] = df * y;
  }
  P.states[s] = rng.a;
  P.states[(size_t)S + s] = rng.b;
  P.states[2 * (size_t)S + s] = rng.c;
  P.states[3 * (size_t)S + s] = rng.d;
  if (caphits) atomicAdd(P.status, caphits);
  if (fallbacks) atomicAdd(P.status + 1, fallbacks);
}

}  // namespace dev

cudaError_t launch_mlmc_cv_level(const MlmcCvParams &Q, int klass, cudaStream_t st) {
  using namespace dev;
  const unsigned int blocks = (Q.M.n_used + kSimBlock - 1) / kSimBlock;
  switch (klass) {
    case BK_F0: mlmc_cv_level_kernel<0, SCH_NONE, SCH_NONE><<<blocks, kSimBlock, 0, st>>>(Q); break;
    case BK_F1_NV: mlmc_cv_level_kernel<1, SCH_NV, SCH_NONE><<<blocks, kSimBlock, 0, st>>>(Q); break;
    case BK_F1_EXACT: mlmc_cv_level_kernel<1, SCH_EXACT, SCH_NONE><<<blocks, kSimBlock, 0, st>>>(Q); break;
    case BK_F1_NCI: mlmc_cv_level_kernel<1, SCH_NCI, SCH_NONE><<<blocks, kSimBlock, 0, st>>>(Q); break;
    case BK_F2_NV_NV: mlmc_cv_level_kernel<2, SCH_NV, SCH_NV><<<blocks, kSimBlock, 0, st>>>(Q); break;
    case BK_F2_NV_EXACT: mlmc_cv_level_kernel<2, SCH_NV, SCH_EXACT><<<blocks, kSimBlock, 0, st>>>(Q); break;
    case BK_F2_NV_NCI: mlmc_cv_level_kernel<2, SCH_NV, SCH_NCI><<<blocks, kSimBlock, 0, st>>>(Q); break;
    case BK_F2_EXACT_NV: mlmc_cv_level_kernel<2, SCH_EXACT, SCH_NV><<<blocks, kSimBlock, 0, st>>>(Q); break;
    case BK_F2_EXACT_EXACT: mlmc_cv_level_kernel<2, SCH_EXACT, SCH_EXACT><<<blocks, kSimBlock, 0, st>>>(Q); break;
    case BK_F2_EXACT_NCI: mlmc_cv_level_kernel<2, SCH_EXACT, SCH_NCI><<<blocks, kSimBlock, 0, st>>>(Q); break;
    case BK_F2_NCI_NV: mlmc_cv_level_kernel<2, SCH_NCI, SCH_NV><<<blocks, kSimBlock, 0, st>>>(Q); break;
    case BK_F2_NCI_EXACT: mlmc_cv_level_kernel<2, SCH_NCI, SCH_EXACT><<<blocks, kSimBlock, 0, st>>>(Q); break;
    case BK_F2_NCI_NCI: mlmc_cv_level_kernel<2, SCH_NCI, SCH_NCI><<<blocks, kSimBlock, 0, st>>>(Q); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace myql
