// qmc.cuh -- randomized quasi-Monte Carlo paths (myql_qmc_price, myql_cv_qmc_price): the
// parameters, the warp-wide Sobol generator and the path simulation shared by the pricing
// kernel and the control variate's Sobol paths (qmc.cu).
#pragma once
#include "cv.cuh"
#include "engine.h"

namespace myql {

constexpr int kQmcMaxSteps = 512;
constexpr int kQmcBits = 32;
constexpr int kQmcSeg = 32;  // steps per bridge segment
constexpr uint64_t kQmcDirectionSeed = MYQL_QMC_DEFAULT_DIRECTION_SEED;  // the default point set

struct QmcParams {
  SimParams P;                 // plan constants (records, trackers, scenario 0)
  const uint32_t *dirs;        // [32][D] direction numbers V_1..V_32, bit-major
  const uint32_t *shift;       // [R][D] digital shifts
  const int *br_mid, *br_left, *br_right;  // segmented Brownian bridge schedule (n entries)
  const float *br_wl, *br_wr, *br_sd;
  unsigned long long n_pts;    // points per replicate
  unsigned int D;              // dimensions per path = steps * (NG + NU)
  int sch[2];                  // scheme of each factor: SCH_NV or SCH_NCI
  int jump;                    // 0 none, 1 Merton (per step)
  int NG, NU;                  // Gaussian motions (spot + NV factors), uniforms per step
};

// The control variate on Sobol paths: the features, martingale increments and discounted
// payoffs of paths [path_begin, path_begin + n) of the replicated point set (path index
// i = replicate x n_pts + point), in the layout of CvSimParams.
struct QmcCvParams {
  QmcParams Q;
  PayoffParams pay;
  double df;
  uint8_t *feat;                  // feature tiles of this launch's paths
  float *dM;                      // [tile][128]
  float *Y;                       // discounted payoff per path (launch-local index)
  unsigned long long path_begin;  // a multiple of 2048
  int hedge_every, n_hedge;
  CvFeatConsts fc;
};

namespace dev {

// One warp's Sobol coordinates, 32 dimensions at a time, in dimension order.  The 32 lanes
// hold 32 consecutive points of one replicate, so the Gray code's bits >= 5 are the same
// for the whole warp and only bits 0..4 differ.  A fill gives lane l dimension d0 + l: it
// XORs the shift and the direction numbers of the shared high bits (coalesced loads from
// the bit-major table), then walks the 32 low Gray values in Gray-code order (one XOR
// each) and stores them in row l of the warp's 32 x 32 table; a draw is then one shared
// load at (row d - d0, column of the lane's low Gray bits).  Columns are XOR-swizzled by
// the row, so both the fill's stores and the draws' loads touch 32 distinct banks.
static __device__ __noinline__ void sobol_fill(uint32_t *tab, const uint32_t *V, const uint32_t *shift, uint32_t ghi,
                                        unsigned int D, unsigned int d0, int lane) {
  __syncwarp();  // every lane has read the previous block of dimensions
  const unsigned int d = d0 + (unsigned int)lane;
  if (d < D) {
    uint32_t h = __ldg(shift + d);
    for (uint32_t m = ghi; m; m &= m - 1u) h ^= __ldg(V + (size_t)(__ffs((int)m) - 1) * D + d);
    uint32_t v[5];
#pragma unroll
    for (int b = 0; b < 5; ++b) v[b] = __ldg(V + (size_t)b * D + d);
    uint32_t *row = tab + lane * 32;
    row[lane] = h;  // Gray value 0
#pragma unroll
    for (int j = 1; j < 32; ++j) {
      h ^= v[__ffs(j) - 1];
      row[(j ^ (j >> 1)) ^ lane] = h;
    }
  }
  __syncwarp();
}

struct SobolWarp {
  uint32_t *tab;          // [32][32] in shared memory
  const uint32_t *V;      // bit-major direction numbers [32][D]
  const uint32_t *shift;  // this replicate's shifts [D]
  uint32_t ghi, glo;      // Gray code: the warp's bits >= 5, the lane's bits 0..4
  unsigned int D, d0, pos;
  int lane;

  __device__ __forceinline__ void fill() { sobol_fill(tab, V, shift, ghi, D, d0, lane); }
  // the next dimension's shifted coordinate as a 64-bit draw: the centre of its 2^-32 cell,
  // so that u01_bits, u01c_bits and inv_normal_bits of it are the coordinate's uniform
  __device__ __forceinline__ unsigned long long next() {
    if (pos == 32u) {
      d0 += 32u;
      pos = 0u;
      fill();
    }
    const uint32_t x = tab[pos * 32u + (glo ^ pos)];
    ++pos;
    return ((unsigned long long)x << 32) | 0x80000000ull;
  }
};

// A warp's generator for global path index i (warp-aligned: i = 32 w + lane); the first
// 32 dimensions are filled on return.
__device__ __forceinline__ SobolWarp sobol_warp(const QmcParams &Q, uint32_t *tab, unsigned long long i) {
  const unsigned long long rep = i / Q.n_pts, pt = i % Q.n_pts;
  const uint32_t g = (uint32_t)(pt ^ (pt >> 1));  // Gray code
  SobolWarp sob;
  sob.tab = tab;
  sob.V = Q.dirs;
  sob.shift = Q.shift + rep * Q.D;
  sob.ghi = g & ~31u;
  sob.glo = g & 31u;
  sob.D = Q.D;
  sob.d0 = 0u;
  sob.pos = 0u;
  sob.lane = (int)(threadIdx.x & 31u);
  sob.fill();
  return sob;
}

// One path of the replicated point set, scenario 0, in dimension order.  The Brownian bridge
// of each Gaussian motion comes in segments of kQmcSeg steps: first its values at the segment
// boundaries (the coarse shape of the path, the lowest dimensions), then segment by segment
// the interior of the segment's bridge followed by the segment's steps with their per-step
// uniforms.  Only one segment's values are held at a time.  The hook sees every step as in
// sim_path_h (begin, diffusion, jump, step_end, finish).  Writes the tracker's terminal record.
template <int NF, bool PD, class Hook>
__device__ __forceinline__ void qmc_path(const QmcParams &Q, SobolWarp &sob, float (&out)[kMaxFields],
                                         unsigned int &caphits, unsigned int &fallbacks, Hook &hook) {
  const SimParams &P = Q.P;
  const int n = P.n_steps;
  constexpr int NC = 1 + NF;  // at most: the spot's motion and one per NV factor
  constexpr int kSegs = kQmcMaxSteps / kQmcSeg;
  const int NG = Q.NG;
  const int ns = (n + kQmcSeg - 1) / kQmcSeg;
  float Wc[NC][kSegs + 1];  // values at the segment boundaries
#pragma unroll
  for (int c = 0; c < NC; ++c) Wc[c][0] = 0.0f;
  for (int b = 0; b < ns; ++b) {
    const int m = Q.br_mid[b], l = Q.br_left[b], r = Q.br_right[b];
    const float wl = Q.br_wl[b], wr = Q.br_wr[b], sd = Q.br_sd[b];
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      if (c >= NG) break;
      const float z = inv_normal_bits(sob.next());
      Wc[c][m] = fmaf(wl, Wc[c][l], fmaf(wr, Wc[c][r], sd * z));
    }
  }
  const ScenarioConst &C = P.sc[0];
  float X = 0.0f, v[2] = {C.f[0].v0, C.f[1].v0};
  TrackerState ts;
  ts.init(P, PD);
  if (Hook::active) hook.begin(v[0], v[1]);
  const float dt = C.dt;
  int e = ns;  // next bridge schedule entry
  for (int sg = 0; sg < ns; ++sg) {
    const int k0 = sg * kQmcSeg, len = min(kQmcSeg, n - k0);
    float W[NC][kQmcSeg + 1];  // this segment's values, from its start
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      W[c][0] = Wc[c][sg];
      W[c][len] = Wc[c][sg + 1];
    }
    for (int b = 0; b < len - 1; ++b, ++e) {
      const int m = Q.br_mid[e], l = Q.br_left[e], r = Q.br_right[e];
      const float wl = Q.br_wl[e], wr = Q.br_wr[e], sd = Q.br_sd[e];
#pragma unroll
      for (int c = 0; c < NC; ++c) {
        if (c >= NG) break;
        const float z = inv_normal_bits(sob.next());
        W[c][m] = fmaf(wl, W[c][l], fmaf(wr, W[c][r], sd * z));
      }
    }
    for (int kk = 0; kk < len; ++kk) {  // the segment's steps, each with its NU uniforms
      const int k = k0 + kk;
      const float G = W[0][kk + 1] - W[0][kk];
      if (NF == 0) {
        X += fmaf(C.gbm_vol, G, C.gbm_drift);
        if (Hook::active) hook.diffusion(C.gbm_vol, G, C.gbm_drift);
      } else {
        float vn[2] = {0.0f, 0.0f};
        int gi = 1;  // next Gaussian motion (NV factors, in factor order)
  #pragma unroll
        for (int f = 0; f < NF; ++f) {
          const FactorConst &fc = C.f[f];
          if (Q.sch[f] == SCH_NV) {
            const float Z = gi == 1 ? W[1][kk + 1] - W[1][kk] : W[NC - 1][kk + 1] - W[NC - 1][kk];
            ++gi;
            const float rt = sqrt_approx(fmaf(fc.w0, v[f], fc.w1)) + fc.w2 * Z;
            vn[f] = fmaf(fc.w0 * rt, rt, fc.w1);
          } else {  // SchemeNCI: N ~ Poisson(C0 v) by inversion, then the table at the second uniform
            const unsigned long long xp = sob.next();
            const unsigned long long x2 = sob.next();
            const float lam = fc.w0 * v[f];
            const float Wp = lam > kPoissonAsymMin ? inv_normal_bits(xp) : 0.0f;
            const int N = poisson_core(lam, u01_bits(xp), Wp, xp, P.loop_cap, caphits);
            vn[f] = nci_quantile(P.nci[f], N, x2, P.nci_u999, fallbacks) * fc.w2;
          }
        }
        float root, drift;
        if (NF == 1) {
          const FactorConst &f0 = C.f[0];
          root = sqrt_approx(f0.C3 * (v[0] + vn[0]));
          drift = fmaf(f0.C2, vn[0], fmaf(f0.C1, v[0], f0.C0));
        } else {
          const FactorConst &f0 = C.f[0];
          const FactorConst &f1 = C.f[1];
          root = sqrt_approx(fmaf(f0.C3, v[0] + vn[0], f1.C3 * (v[1] + vn[1])));
          drift = fmaf(f1.C2, vn[1], fmaf(f1.C1, v[1], fmaf(f0.C2, vn[0], fmaf(f0.C1, v[0], f0.C0 + f1.C0))));
        }
        X += fmaf(root, G, drift);
        if (Hook::active) hook.diffusion(root, G, drift);
        v[0] = vn[0];
        v[1] = vn[1];
      }
      if (Q.jump) {  // Merton, per step: count by sequential inversion, then one normal for the sum
        const unsigned long long xc = sob.next();
        const unsigned long long xz = sob.next();
        const int nj = poisson_small_u(C.jump_mean, C.jump_exp_neg_mean, u01_bits(xc), P.loop_cap, caphits);
        float J = C.jump_comp;
        if (nj > 0) {
          const float fn = (float)nj;
          J += fn * P.merton_mu + sqrtf(fn) * P.merton_delta * inv_normal_bits(xz);
        }
        X += J;
        if (Hook::active) hook.jump(J);
      }
      if (PD) ts.step(P, k, dt, X);
      if (Hook::active) hook.step_end(k + 1, X, v[0], v[1], ts.acc, ts.tb >= 0.0f);
    }
  }
  if (Hook::active) hook.finish();
  ts.finish(P, C, X, PD, out);
}

}  // namespace dev

// Host: validates a job for quasi-Monte Carlo (factor schemes, jumps, steps, num_paths = M
// a multiple of 2048 x R), then fills Q's tables (Sobol directions and shifts for the job's
// seed, the bridge, the NCI tables) and constants from the plan; the records, status and
// path range are the caller's.
myql_status qmc_prepare(CtxBase *ctx, const myql_mc_job &job, const Plan &pl, uint64_t R, QmcParams &Q);
cudaError_t launch_qmc_cv(const QmcCvParams &P, unsigned long long n_paths, int nf, cudaStream_t st);

}  // namespace myql
