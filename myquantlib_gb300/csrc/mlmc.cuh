// mlmc.cuh -- multilevel Monte Carlo level kernels (sm_103a).
//
// Level 0 simulates base_steps steps with the plain stepper (the reference's
// ASVJStepper, MultiLevelMonteCarloPricer.hpp:257-292); level l > 0 simulates a
// fine path of 2n steps and its coarse partner of n steps on the same random
// numbers, as CoupledASVJStepper::multi_step_coupled does
// (CoupledASVJStepper.hpp:170-517): the coarse Gaussian of each coarse step is
// built from the two fine ones (weighted by the fine diffusion amplitudes), the
// NV coarse variance from the summed fine Gaussians, NCI/Exact coarse variances
// copy the fine path, and both paths share every jump.  Each thread owns one
// stream of a persistent pool (the reference's per-thread rng_pool) and
// accumulates P_fine - P_coarse and its square in FP64.
#pragma once
#include "payoff.cuh"
#include "simulate.cuh"

namespace myql {

struct MlmcParams {
  SimParams sim;       // sc[0] = fine (level > 0) or base (level 0), sc[1] = coarse
  PayoffParams pay;    // scalar instrument; avg constants [0] fine, [1] coarse
  int level;
  int n_coarse;        // coarse steps (level 0: base steps)
  unsigned long long dN;
  unsigned int n_used; // streams used by this evaluation (<= n_streams)
  double *partials;    // [blocks][2]
};

namespace dev {

// NV step with a given Gaussian (SchemeNV::evolve_coupled, VolSchemes.hpp:61-65)
__device__ __forceinline__ float nv_step(float v, float Z, const FactorConst &f) {
  const float root = sqrt_approx(fmaf(f.w0, v, f.w1)) + f.w2 * Z;
  return fmaf(f.w0 * root, root, f.w1);
}

// Fine variance step of one factor; Z receives the Gaussian an NV factor used.
template <int SCH>
__device__ __forceinline__ float fine_vol(float v, Xo &rng, const FactorConst &f, const SimParams &P,
                                          int fi, float &Z, unsigned int &caphits,
                                          unsigned int &fallbacks) {
  if (SCH == SCH_NV) {
    Z = inv_normal_bits(draw(rng));
    return nv_step(v, Z, f);
  }
  return evolve<SCH>(v, rng, f, P, fi, caphits, fallbacks);
}

struct TrkState {
  float acc, mn, mx, tb, tu, td;
};

__device__ __forceinline__ void trk_init(const SimParams &P, TrkState &t) {
  t.acc = 0.0f;
  t.mn = P.lb_min0;
  t.mx = P.lb_max0;
  t.tb = t.tu = t.td = -1.0f;
  if (P.tracker == TRK_BARRIER_UP) {
    if (0.0f >= P.b_log[0]) t.tb = 0.0f;
    if (0.0f >= P.b_log[1]) t.tu = 0.0f;
    if (0.0f >= P.b_log[2]) t.td = 0.0f;
  } else if (P.tracker == TRK_BARRIER_DOWN) {
    if (0.0f <= P.b_log[0]) t.tb = 0.0f;
    if (0.0f <= P.b_log[1]) t.tu = 0.0f;
    if (0.0f <= P.b_log[2]) t.td = 0.0f;
  }
}

__device__ __forceinline__ void trk_update(const SimParams &P, TrkState &t, float X, float time) {
  switch (P.tracker) {
    case TRK_GEO_ASIAN: t.acc += X; break;
    case TRK_ARITH_ASIAN: t.acc += __expf(X); break;
    case TRK_LOOKBACK:
      t.mn = fminf(t.mn, X);
      t.mx = fmaxf(t.mx, X);
      break;
    case TRK_BARRIER_UP:
      if (t.tu < 0.0f && X >= P.b_log[1]) t.tu = time;
      if (t.tb < 0.0f && X >= P.b_log[0]) t.tb = time;
      if (t.td < 0.0f && X >= P.b_log[2]) t.td = time;
      break;
    case TRK_BARRIER_DOWN:
      if (t.td < 0.0f && X <= P.b_log[2]) t.td = time;
      if (t.tb < 0.0f && X <= P.b_log[0]) t.tb = time;
      if (t.tu < 0.0f && X <= P.b_log[1]) t.tu = time;
      break;
    default: break;
  }
}

__device__ __forceinline__ void trk_final(const SimParams &P, const TrkState &t, float X, float dt,
                                          float (&out)[kMaxFields]) {
  out[0] = X;
  switch (P.tracker) {
    case TRK_GEO_ASIAN: out[1] = dt * (t.acc - 0.5f * X); break;
    case TRK_ARITH_ASIAN: out[1] = dt * (0.5f + t.acc - 0.5f * __expf(X)); break;
    case TRK_LOOKBACK:
      out[1] = t.mn;
      out[2] = t.mx;
      break;
    case TRK_BARRIER_UP:
    case TRK_BARRIER_DOWN:
      out[1] = t.tb;
      out[2] = t.tu;
      out[3] = t.td;
      break;
    default: break;
  }
}

// Observer of a coupled (fine, coarse) path pair (the control variate of the
// level corrections); NoCoupledHook compiles away.  Each call gets the log-spot
// increment root * G + drift of one step and the variances it started from.
struct NoCoupledHook {
  static constexpr bool active = false;
  __device__ __forceinline__ void begin(float, float) {}
  __device__ __forceinline__ void fine(float, float, float, float, float) {}
  __device__ __forceinline__ void fine_jump(float) {}
  __device__ __forceinline__ void coarse(float, float, float, float, float) {}
  __device__ __forceinline__ void coarse_jump(float) {}
  // after coarse step kc (1-based): fine and coarse log-spots, fine variances, fine
  // tracker accumulator, fine base-barrier hit so far
  __device__ __forceinline__ void coarse_end(int, float, float, float, float, float, bool) {}
  __device__ __forceinline__ void finish() {}
};

// One coupled (fine, coarse) path pair.
template <int NF, int S1, int S2, bool PD, class Hook = NoCoupledHook>
__device__ __forceinline__ void coupled_path(const SimParams &P, int n_coarse, Xo &rng,
                                             float (&of)[kMaxFields], float (&oc)[kMaxFields],
                                             unsigned int &caphits, unsigned int &fallbacks,
                                             Hook hook = Hook()) {
  const ScenarioConst &Fc = P.sc[0];  // fine constants
  const ScenarioConst &Cc = P.sc[1];  // coarse constants
  float Xf = 0.0f, Xc = 0.0f;
  TrkState tf, tc;
  if (PD) {
    trk_init(P, tf);
    trk_init(P, tc);
  }
  if (NF == 0 && !PD) {
    // GBM European: one Gaussian for both levels, one shared jump (:187-218)
    const float G = inv_normal_bits(draw(rng));
    Xf = fmaf(Fc.gbm_vol, G, Fc.gbm_drift);
    Xc = fmaf(Cc.gbm_vol, G, Cc.gbm_drift);
    if (P.jump_kind) {
      const float J = jump_draw(P, Fc, rng, caphits);
      Xf += J;
      Xc += J;
    }
    of[0] = Xf;
    oc[0] = Xc;
    return;
  }
  if (!PD && NF > 0 && P.jump_kind) {  // European: shared jump before the loop (:225-230)
    const float J = jump_draw(P, Fc, rng, caphits);
    Xf += J;
    Xc += J;
  }
  float vf0 = Fc.f[0].v0, vf1 = Fc.f[1].v0, vc0 = Cc.f[0].v0, vc1 = Cc.f[1].v0;
  const float dtf = Fc.dt, dtc = Cc.dt;
  if (Hook::active) hook.begin(vf0, vf1);
  for (int k = 0; k < n_coarse; ++k) {
    const float G1 = inv_normal_bits(draw(rng));
    const float G2 = inv_normal_bits(draw(rng));
    float Gc = (G1 + G2) * 0.70710678118654752f;
    float j1 = 0.0f, j2 = 0.0f;
    if (NF == 0) {
      Xc += fmaf(Cc.gbm_vol, Gc, Cc.gbm_drift);
      Xf += fmaf(Fc.gbm_vol, G1, Fc.gbm_drift);
      if (Hook::active) {
        hook.coarse(Cc.gbm_vol, Gc, Cc.gbm_drift, 0.0f, 0.0f);
        hook.fine(Fc.gbm_vol, G1, Fc.gbm_drift, 0.0f, 0.0f);
      }
      if (PD) {
        if (P.jump_kind) j1 = jump_draw(P, Fc, rng, caphits);
        Xf += j1;
        if (Hook::active && P.jump_kind) hook.fine_jump(j1);
        trk_update(P, tf, Xf, (float)(2 * k + 1) * dtf);
      }
      Xf += fmaf(Fc.gbm_vol, G2, Fc.gbm_drift);
      if (Hook::active) hook.fine(Fc.gbm_vol, G2, Fc.gbm_drift, 0.0f, 0.0f);
      if (PD) {
        if (P.jump_kind) j2 = jump_draw(P, Fc, rng, caphits);
        Xf += j2;
        if (Hook::active && P.jump_kind) hook.fine_jump(j2);
        trk_update(P, tf, Xf, (float)(2 * k + 2) * dtf);
        Xc += j1 + j2;
        if (Hook::active && P.jump_kind) hook.coarse_jump(j1 + j2);
        trk_update(P, tc, Xc, (float)(k + 1) * dtc);
      }
      if (Hook::active) hook.coarse_end(k + 1, Xf, Xc, 0.0f, 0.0f, tf.acc, tf.tb >= 0.0f);
      continue;
    }
    // fine step 1
    float Z0a = 0.0f, Z1a = 0.0f, Z0b = 0.0f, Z1b = 0.0f;
    const FactorConst &ff0 = Fc.f[0], &ff1 = Fc.f[1], &fc0 = Cc.f[0], &fc1 = Cc.f[1];
    const float m0 = fine_vol<S1>(vf0, rng, ff0, P, 0, Z0a, caphits, fallbacks);
    float m1 = 0.0f;
    if (NF == 2) m1 = fine_vol<S2>(vf1, rng, ff1, P, 1, Z1a, caphits, fallbacks);
    float r1, d1;
    if (NF == 1) {
      r1 = sqrt_approx(ff0.C3 * (vf0 + m0));
      d1 = fmaf(ff0.C2, m0, fmaf(ff0.C1, vf0, ff0.C0));
    } else {
      r1 = sqrt_approx(fmaf(ff0.C3, vf0 + m0, ff1.C3 * (vf1 + m1)));
      d1 = fmaf(ff1.C2, m1, fmaf(ff1.C1, vf1, fmaf(ff0.C2, m0, fmaf(ff0.C1, vf0, ff0.C0 + ff1.C0))));
    }
    Xf += fmaf(r1, G1, d1);
    if (Hook::active) hook.fine(r1, G1, d1, vf0, vf1);
    if (PD) {
      if (P.jump_kind) j1 = jump_draw(P, Fc, rng, caphits);
      Xf += j1;
      if (Hook::active && P.jump_kind) hook.fine_jump(j1);
      trk_update(P, tf, Xf, (float)(2 * k + 1) * dtf);
    }
    // fine step 2
    const float n0 = fine_vol<S1>(m0, rng, ff0, P, 0, Z0b, caphits, fallbacks);
    float n1 = 0.0f;
    if (NF == 2) n1 = fine_vol<S2>(m1, rng, ff1, P, 1, Z1b, caphits, fallbacks);
    float r2, d2;
    if (NF == 1) {
      r2 = sqrt_approx(ff0.C3 * (m0 + n0));
      d2 = fmaf(ff0.C2, n0, fmaf(ff0.C1, m0, ff0.C0));
    } else {
      r2 = sqrt_approx(fmaf(ff0.C3, m0 + n0, ff1.C3 * (m1 + n1)));
      d2 = fmaf(ff1.C2, n1, fmaf(ff1.C1, m1, fmaf(ff0.C2, n0, fmaf(ff0.C1, m0, ff0.C0 + ff1.C0))));
    }
    Xf += fmaf(r2, G2, d2);
    if (Hook::active) hook.fine(r2, G2, d2, m0, m1);
    if (PD) {
      if (P.jump_kind) j2 = jump_draw(P, Fc, rng, caphits);
      Xf += j2;
      if (Hook::active && P.jump_kind) hook.fine_jump(j2);
      trk_update(P, tf, Xf, (float)(2 * k + 2) * dtf);
    }
    // coarse step
    const float c0n = S1 == SCH_NV ? nv_step(vc0, (Z0a + Z0b) * 0.70710678118654752f, fc0) : n0;
    float c1n = 0.0f;
    if (NF == 2) c1n = S2 == SCH_NV ? nv_step(vc1, (Z1a + Z1b) * 0.70710678118654752f, fc1) : n1;
    if (r1 + r2 > 1e-15f) Gc = (r1 * G1 + r2 * G2) * rsqrtf(fmaf(r1, r1, r2 * r2));
    float rc, dc;
    if (NF == 1) {
      rc = sqrt_approx(fc0.C3 * (vc0 + c0n));
      dc = fmaf(fc0.C2, c0n, fmaf(fc0.C1, vc0, fc0.C0));
    } else {
      rc = sqrt_approx(fmaf(fc0.C3, vc0 + c0n, fc1.C3 * (vc1 + c1n)));
      dc = fmaf(fc1.C2, c1n, fmaf(fc1.C1, vc1, fmaf(fc0.C2, c0n, fmaf(fc0.C1, vc0, fc0.C0 + fc1.C0))));
    }
    Xc += fmaf(rc, Gc, dc);
    if (Hook::active) hook.coarse(rc, Gc, dc, vc0, vc1);
    vf0 = n0;
    vf1 = n1;
    vc0 = c0n;
    vc1 = c1n;
    if (PD) {
      Xc += j1 + j2;
      if (Hook::active && P.jump_kind) hook.coarse_jump(j1 + j2);
      trk_update(P, tc, Xc, (float)(k + 1) * dtc);
    }
    if (Hook::active) hook.coarse_end(k + 1, Xf, Xc, vf0, vf1, PD ? tf.acc : 0.0f, PD && tf.tb >= 0.0f);
  }
  if (Hook::active) hook.finish();
  if (PD) {
    trk_final(P, tf, Xf, dtf, of);
    trk_final(P, tc, Xc, dtc, oc);
  } else {
    of[0] = Xf;
    oc[0] = Xc;
  }
}

// Price of a scalar instrument from one terminal record; `sc` selects the
// Asian averaging constants (0 fine / base, 1 coarse).
__device__ __forceinline__ float record_price(const PayoffParams &P, const float (&r)[kMaxFields],
                                              int sc, float K) {
  PathView v;
  v.S = P.S0 * __expf(r[0]);
  v.Y = 0.0f;
  v.hit[0] = v.hit[1] = v.hit[2] = -1.0f;
  switch (P.tracker) {
    case TRK_GEO_ASIAN: v.Y = P.S0 * __expf(fmaf(P.avg_c1[sc], r[1], P.avg_c0[sc])); break;
    case TRK_ARITH_ASIAN: v.Y = P.S0 * fmaf(P.avg_c1[sc], r[1], P.avg_c0[sc]); break;
    case TRK_LOOKBACK: {
      const bool use_max = (P.option_type == 0) == (P.fixed_strike != 0);
      v.Y = P.S0 * __expf(use_max ? r[2] : r[1]);
      break;
    }
    case TRK_BARRIER_UP:
    case TRK_BARRIER_DOWN:
      v.hit[0] = r[1];
      v.hit[1] = r[2];
      v.hit[2] = r[3];
      break;
    default: break;
  }
  return scenario_tri(P, v, K, false).v;
}

template <int NF, int S1, int S2, bool PD>
__global__ void __launch_bounds__(kSimBlock) mlmc_level_kernel(const __grid_constant__ MlmcParams M) {
  __shared__ double red[kSimBlock / 32][2];
  const SimParams &P = M.sim;
  const unsigned int s = blockIdx.x * kSimBlock + threadIdx.x;
  const unsigned int S = P.n_streams, U = M.n_used;
  double a = 0.0, b = 0.0;
  unsigned int caphits = 0, fallbacks = 0;
  if (s < U) {
    Xo rng;
    rng.a = P.states[s];
    rng.b = P.states[(size_t)S + s];
    rng.c = P.states[2 * (size_t)S + s];
    rng.d = P.states[3 * (size_t)S + s];
    const float K = (float)M.pay.strikes[0];
    for (unsigned long long i = s; i < M.dN; i += U) {
      float d;
      if (M.level == 0) {
        float r[kMaxFields];
        sim_path<NF, S1, S2, PD>(P, P.sc[0], rng, r, caphits, fallbacks);
        d = record_price(M.pay, r, 0, K);
      } else {
        float rf[kMaxFields], rc[kMaxFields];
        coupled_path<NF, S1, S2, PD>(P, M.n_coarse, rng, rf, rc, caphits, fallbacks);
        d = record_price(M.pay, rf, 0, K) - record_price(M.pay, rc, 1, K);
      }
      a += (double)d;
      b += (double)d * (double)d;
    }
    P.states[s] = rng.a;
    P.states[(size_t)S + s] = rng.b;
    P.states[2 * (size_t)S + s] = rng.c;
    P.states[3 * (size_t)S + s] = rng.d;
  }
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) {
    red[warp][0] = a;
    red[warp][1] = b;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double ta = 0.0, tb = 0.0;
    for (int w = 0; w < kSimBlock / 32; ++w) {
      ta += red[w][0];
      tb += red[w][1];
    }
    M.partials[2 * blockIdx.x] = ta;
    M.partials[2 * blockIdx.x + 1] = tb;
  }
  if (caphits) atomicAdd(P.status, caphits);
  if (fallbacks) atomicAdd(P.status + 1, fallbacks);
}

}  // namespace dev

cudaError_t launch_mlmc_level(const MlmcParams &M, int s1, int s2, bool path_dep, cudaStream_t st);

template <int NF, int S1, int S2>
cudaError_t launch_mlmc_t(const MlmcParams &M, bool pd, cudaStream_t stream) {
  const unsigned int grid = (M.n_used + kSimBlock - 1) / kSimBlock;
  if (pd)
    dev::mlmc_level_kernel<NF, S1, S2, true><<<grid, kSimBlock, 0, stream>>>(M);
  else
    dev::mlmc_level_kernel<NF, S1, S2, false><<<grid, kSimBlock, 0, stream>>>(M);
  return cudaGetLastError();
}

}  // namespace myql
