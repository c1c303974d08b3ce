// payoff.cu -- phase 2 and 3 of a pricing request.
//
// payoff_reduce_kernel turns the per-path terminal records into the per-path
// estimators of MonteCarloPricer.hpp:261-276 (price, pathwise FD delta and
// gamma) and :302-410 (CRN vega, vanna, theta, charm, rho), for every strike
// of the strip, and reduces sum and sum of squares over a tile of paths:
// FP32 over a batch of <= 32 paths, FP64 across batches and tiles.
//   * scalar instruments: each thread evaluates its own paths;
//   * strips: a warp stages 32 paths' records in shared memory and each lane
//     owns one strike of a 32-strike chunk (gridDim.y chunks), so the payoff
//     work is one evaluation per (path, strike) with no per-strike reduction.
// finalize_kernel sums the tile partials, a warp per (strike, quantity), in a fixed order
// (deterministic) and
// applies compute_stats (MonteCarloPricer.hpp:448-457).
#include "engine_types.h"
#include "device_numerics.cuh"
#include "payoff.cuh"

namespace myql {
namespace dev {

// PRE: field 0 is staged as e^X already (the strip path of SPEC = 1, which computes it once
// per path instead of once per strike lane); the product with S0 stays here, where the
// compiler may fuse it with the strike's subtraction exactly as for the unstaged record
template <int SPEC, bool PRE = false, class FLD>
__device__ __forceinline__ PathView make_view(const PayoffParams &P, FLD fld, int sc) {
  PathView v;
  const float X = fld(sc, 0);
  v.S = P.S0 * (PRE ? X : __expf(X));
  v.Y = 0.0f;
  v.hit[0] = v.hit[1] = v.hit[2] = -1.0f;
  if (SPEC == 1) return v;
  switch (P.tracker) {
    case TRK_GEO_ASIAN: v.Y = P.S0 * __expf(fmaf(P.avg_c1[sc], fld(sc, 1), P.avg_c0[sc])); break;
    case TRK_ARITH_ASIAN: v.Y = P.S0 * fmaf(P.avg_c1[sc], fld(sc, 1), P.avg_c0[sc]); break;
    case TRK_LOOKBACK: {
      // fixed strike: call uses the max, put the min; floating: call min, put max
      const bool use_max = (P.option_type == 0) == (P.fixed_strike != 0);
      v.Y = P.S0 * __expf(use_max ? fld(sc, 2) : fld(sc, 1));
      break;
    }
    case TRK_BARRIER_UP:
    case TRK_BARRIER_DOWN:
      v.hit[0] = fld(sc, 1);
      v.hit[1] = fld(sc, 2);
      v.hit[2] = fld(sc, 3);
      break;
    default: break;
  }
  return v;
}

// Per-path estimators of every quantity for strike K (MonteCarloPricer.hpp:261-276
// and :316-409), from the increments of each scenario.
template <int SPEC, bool PRE = false, class FLD>
__device__ __forceinline__ void path_quantities(const PayoffParams &P, FLD fld, float K,
                                                float (&q)[kQ]) {
  const bool bumps = P.mode != 0;
  const Tri b = scenario_tri<SPEC>(P, make_view<SPEC, PRE>(P, fld, 0), K, bumps);
  q[0] = b.v;
  if (!bumps) return;
  {  // delta and gamma as one packed pair: (dp - dm) / 2h, (dp + dm) / h^2
    const float2 dg = pk::fmul2(pk::fadd2(make_float2(b.dp, b.dp), make_float2(-b.dm, b.dm)),
                                make_float2(P.inv_2h, P.inv_h2));
    q[1] = dg.x;
    q[2] = dg.y;
  }
  if (P.mode == 1) return;
  const int nv = P.n_factors >= 2 ? 2 : 1;
  for (int fct = 0; fct < nv; ++fct) {
    const Tri u = scenario_tri<SPEC>(P, make_view<SPEC, PRE>(P, fld, fct == 0 ? SC_VUP0 : SC_VUP1), K, true);
    const Tri d = scenario_tri<SPEC>(P, make_view<SPEC, PRE>(P, fld, fct == 0 ? SC_VDN0 : SC_VDN1), K, true);
    q[fct == 0 ? 3 : 4] = (u.v - d.v) * P.vega_c[fct];
    q[fct == 0 ? 7 : 8] = ((u.dp - u.dm) - (d.dp - d.dm)) * P.vanna_c[fct];
  }
  {
    const Tri u = scenario_tri<SPEC>(P, make_view<SPEC, PRE>(P, fld, SC_TUP), K, true);
    const Tri d = scenario_tri<SPEC>(P, make_view<SPEC, PRE>(P, fld, SC_TDN), K, true);
    q[5] = ((u.v - d.v) + (u.v * P.dfm1_tup - d.v * P.dfm1_tdn)) * P.theta_c;
    const float du = u.dp - u.dm, dd = d.dp - d.dm;
    q[9] = ((du - dd) + (du * P.dfm1_tup - dd * P.dfm1_tdn)) * P.charm_c;
  }
  {
    const Tri u = scenario_tri<SPEC>(P, make_view<SPEC, PRE>(P, fld, SC_RUP), K, false);
    const Tri d = scenario_tri<SPEC>(P, make_view<SPEC, PRE>(P, fld, SC_RDN), K, false);
    q[6] = ((u.v - d.v) + (u.v * P.dfm1_rup - d.v * P.dfm1_rdn)) * P.rho_c;
  }
}

__device__ __forceinline__ int active_q(int mode) { return mode == 0 ? 1 : (mode == 1 ? 3 : kQ); }

// SPEC = 1 stages one record field per scenario (European terminal log-spots), so its
// blocks take a quarter of the staging memory and more of them fit on an SM.
template <int SPEC>
__global__ void __launch_bounds__(kPayoffBlock, SPEC == 1 ? 8 : 0) payoff_reduce_kernel(const __grid_constant__ PayoffParams P) {
  __shared__ float stage[kPayoffBlock / 32][kMaxScenarios * (SPEC == 1 ? 1 : kMaxFields)][33];
  __shared__ double red[kPayoffBlock / 32][2 * kQ][32];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const unsigned long long tile = blockIdx.x;
  const unsigned long long t0 = tile * (unsigned long long)P.tile_paths;
  const unsigned long long t1 = min(t0 + (unsigned long long)P.tile_paths, P.n_paths);
  const int nq = active_q(P.mode);
  const int F = P.n_fields;
  const size_t stride = P.rec_stride;

  if (P.n_strikes == 1) {
    const float K = (float)P.strikes[0];
    float s1[kQ], s2[kQ];
#pragma unroll
    for (int q = 0; q < kQ; ++q) s1[q] = s2[q] = 0.0f;
    for (unsigned long long i = t0 + threadIdx.x; i < t1; i += kPayoffBlock) {
      auto fld = [&](int sc, int f) { return P.records[(size_t)(sc * F + f) * stride + i]; };
      float q[kQ];
#pragma unroll
      for (int k = 0; k < kQ; ++k) q[k] = 0.0f;
      path_quantities<SPEC>(P, fld, K, q);
#pragma unroll
      for (int k = 0; k < kQ; ++k) {
        s1[k] += q[k];
        s2[k] = fmaf(q[k], q[k], s2[k]);
      }
    }
    // block reduction in FP64
#pragma unroll
    for (int k = 0; k < kQ; ++k) {
      double a = s1[k], b = s2[k];
      for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
      }
      if (lane == 0) {
        red[warp][2 * k][0] = a;
        red[warp][2 * k + 1][0] = b;
      }
    }
    __syncthreads();
    if (threadIdx.x < 2 * kQ) {
      double t = 0.0;
      for (int w = 0; w < kPayoffBlock / 32; ++w) t += red[w][threadIdx.x][0];
      const int k = threadIdx.x >> 1;
      if (k >= nq) t = 0.0;
      P.partials[((P.tile0 + tile) * 1 + 0) * (2 * kQ) + threadIdx.x] = t;
    }
    return;
  }

  // Strip: lane = strike within a 32-strike chunk; a warp walks 32-path batches.
  const int kidx = blockIdx.y * 32 + lane;
  const bool kvalid = kidx < P.n_strikes;
  const float K = kvalid ? (float)P.strikes[kidx] : 0.0f;
  // FP64 running sums per (warp, quantity, lane) in shared memory
#pragma unroll
  for (int q = 0; q < 2 * kQ; ++q) red[warp][q][lane] = 0.0;
  const int nsf = P.n_sc * F;
  const unsigned long long per_warp = (unsigned long long)P.tile_paths / (kPayoffBlock / 32);
  const unsigned long long w0 = t0 + (unsigned long long)warp * per_warp;
  const unsigned long long w1 = min(w0 + per_warp, t1);
  for (unsigned long long b0 = w0; b0 < w1; b0 += 32) {
    const unsigned long long i = b0 + lane;
    for (int j = 0; j < nsf; ++j) {
      const float x = i < w1 ? P.records[(size_t)j * stride + i] : 0.0f;
      stage[warp][j][lane] = SPEC == 1 ? __expf(x) : x;
    }
    __syncwarp();
    const int nb = (int)min((unsigned long long)32, w1 - b0);
    float s1[kQ], s2[kQ];
#pragma unroll
    for (int q = 0; q < kQ; ++q) s1[q] = s2[q] = 0.0f;
    if (kvalid) {
      for (int pth = 0; pth < nb; ++pth) {
        auto fld = [&](int sc, int f) { return stage[warp][sc * F + f][pth]; };
        float q[kQ];
#pragma unroll
        for (int k = 0; k < kQ; ++k) q[k] = 0.0f;
        path_quantities<SPEC, SPEC == 1>(P, fld, K, q);
        static_assert(kQ % 2 == 0, "quantities in pairs");
#pragma unroll
        for (int k = 0; k < kQ; k += 2) {  // packed FP32 pairs: each lane rounds as the scalar form
          const float2 qq = make_float2(q[k], q[k + 1]);
          const float2 a1 = pk::fadd2(make_float2(s1[k], s1[k + 1]), qq);
          const float2 a2 = pk::ffma2(qq, qq, make_float2(s2[k], s2[k + 1]));
          s1[k] = a1.x;
          s1[k + 1] = a1.y;
          s2[k] = a2.x;
          s2[k + 1] = a2.y;
        }
      }
    }
#pragma unroll
    for (int q = 0; q < kQ; ++q) {
      if (q < nq) {
        red[warp][2 * q][lane] += (double)s1[q];
        red[warp][2 * q + 1][lane] += (double)s2[q];
      }
    }
    __syncwarp();
  }
  __syncthreads();
  if (warp == 0 && kvalid) {
    double *dst = P.partials + ((P.tile0 + tile) * (unsigned long long)P.n_strikes + kidx) * (2 * kQ);
    for (int j = 0; j < 2 * kQ; ++j) {
      double t = 0.0;
      for (int w = 0; w < kPayoffBlock / 32; ++w) t += red[w][j][lane];
      if ((j >> 1) >= nq) t = 0.0;
      dst[j] = t;
    }
  }
}

// One warp per (strike, quantity): lane l sums tiles l, l + 32, ... in order, a fixed
// shuffle tree adds the lanes (deterministic for a given tile count), then mean * df and
// sqrt((E[x^2] - E[x]^2) / M) * df (MonteCarloPricer.hpp:448-457).
constexpr int kFinalizeBlock = 256;
__global__ void __launch_bounds__(kFinalizeBlock) finalize_kernel(const FinalizeParams P) {
  const int w = (int)((blockIdx.x * kFinalizeBlock + threadIdx.x) >> 5), lane = (int)(threadIdx.x & 31u);
  if (w >= P.n_strikes * kQ) return;  // whole warps
  const int k = w / kQ, q = w % kQ;
  double s = 0.0, ss = 0.0;
  if ((P.active_mask >> q) & 1) {
    for (unsigned long long t = (unsigned long long)lane; t < P.n_tiles; t += 32) {
      const double *src = P.partials + (t * (unsigned long long)P.n_strikes + k) * (2 * kQ);
      s += src[2 * q];
      ss += src[2 * q + 1];
    }
    for (int o = 16; o > 0; o >>= 1) {
      s += __shfl_xor_sync(0xffffffffu, s, o);
      ss += __shfl_xor_sync(0xffffffffu, ss, o);
    }
  }
  if (lane != 0) return;
  const double mean = s * P.inv_m;
  double var = ss * P.inv_m - mean * mean;
  if (var < 0.0) var = 0.0;
  P.out[(size_t)(2 * q) * P.n_strikes + k] = mean * P.df;
  P.out[(size_t)(2 * q + 1) * P.n_strikes + k] = sqrt(var * P.inv_m) * P.df;
}

}  // namespace dev

cudaError_t launch_payoff(const PayoffParams &P, unsigned long long n_tiles, cudaStream_t stream) {
  if (n_tiles == 0) return cudaSuccess;
  const dim3 grid((unsigned int)n_tiles, P.n_strikes == 1 ? 1u : (unsigned int)((P.n_strikes + 31) / 32));
  if (P.kind == 0 && P.payoff == 0 && P.tracker == TRK_EUROPEAN && P.n_sc * P.n_fields <= kMaxScenarios)
    dev::payoff_reduce_kernel<1><<<grid, kPayoffBlock, 0, stream>>>(P);
  else
    dev::payoff_reduce_kernel<0><<<grid, kPayoffBlock, 0, stream>>>(P);
  return cudaGetLastError();
}

cudaError_t launch_finalize(const FinalizeParams &P, cudaStream_t stream) {
  const long long threads = (long long)P.n_strikes * kQ * 32;
  dev::finalize_kernel<<<(unsigned int)((threads + dev::kFinalizeBlock - 1) / dev::kFinalizeBlock),
                         dev::kFinalizeBlock, 0, stream>>>(P);
  return cudaGetLastError();
}

}  // namespace myql
