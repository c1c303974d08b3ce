// simulate.cuh -- phase 1 of a pricing request: path simulation.
//
// One thread owns one xoshiro256++ stream and simulates the paths
// i = s, s + S, s + 2S, ... of that stream (S = number of streams), keeping
// log-spot X = log(S_t / S0), the CIR variances and the tracker state in FP32
// registers.  For GreekMode::Full every path is replayed from the stream state
// saved at its start for each bumped scenario (common random numbers), exactly
// as MonteCarloPricer.hpp:302-410 replays `rng_start`; the base scenario is the
// one that advances the stream.  Each (scenario, path) leaves a compact
// terminal record that the payoff pass turns into prices and Greeks.
//
// Template parameters: number of CIR factors and the scheme of each factor
// (the Stepper's VolScheme1 / VolScheme2), and whether the instrument's tracker
// is path dependent.  Jump policy and tracker kind are uniform runtime values.
#pragma once
#include "device_numerics.cuh"
#include "engine_types.h"

namespace myql {
namespace dev {

enum { SCH_NONE = 0, SCH_NV = 1, SCH_EXACT = 2, SCH_NCI = 3 };

// Cell of a draw x2 on the SchemeNCI table's U grid (VolSchemes.hpp:334-370):
// the cubic Hermite cell and its fraction on the main grid, or on the tail grid
// for U >= 0.999.  It depends on the draw alone, not on the table row.
struct NciPos {
  int i;
  float t;
  bool tail;
};

__device__ __forceinline__ NciPos nci_pos(const NciTable &tab, unsigned long long x2,
                                          unsigned long long u999) {
  NciPos p;
  p.tail = x2 >= u999;
  if (!p.tail) {
    const unsigned long long hi = __umul64hi(x2, tab.pos_scale);  // U*inv_dx * 2^50
    p.i = min((int)(hi >> 50), kNciGrid - 2);
    p.t = (float)((unsigned int)(hi >> 26) & 0xFFFFFFu) * 5.9604644775390625e-8f;
  } else {
    const float w = -__logf(u01c_bits(x2));
    float pos = (w - tab.tail_w0) * tab.tail_inv_dw;
    pos = fminf(fmaxf(pos, 0.0f), (float)(kNciTail - 1) - 1e-3f);
    p.i = (int)pos;
    p.t = pos - (float)p.i;
  }
  return p;
}

// Hermite cell of row N (clamped to the table) at the position p.
__device__ __forceinline__ float4 nci_cell(const NciTable &tab, int N, const NciPos &p) {
  const size_t row = (size_t)min(N, tab.rows - 1);
  return p.tail ? __ldg(tab.tail + row * (kNciTail - 1) + p.i)
                : __ldg(tab.main + row * (kNciGrid - 1) + p.i);
}

__device__ __forceinline__ float nci_cubic(const float4 &c, float t) {
  return fmaf(fmaf(fmaf(c.w, t, c.z), t, c.y), t, c.x);
}

// Wilson-Hilferty cube for rows beyond the table (dof >= d + 2*rows).
__device__ __forceinline__ float nci_beyond_wh(float d, int N, unsigned long long x2) {
  const float nu = d + 2.0f * (float)N;
  const float z = inv_normal_bits(x2);
  const float h = 2.0f / (9.0f * nu);
  const float b = 1.0f - h + z * sqrtf(h);
  return fmaxf(nu * b * b * b, 0.0f);
}
// The same, out of line, for the lockstep kernels: with the headline tables a count past
// the rows is rare, and inline its inverse normal would sit in every step.  (The batched
// kernels' capped tables send many counts past the rows; they keep it inline.)
static __device__ __noinline__ float nci_beyond_cold(float d, int N, unsigned long long x2) {
  return nci_beyond_wh(d, N, x2);
}
__device__ __forceinline__ float nci_beyond(const NciTable &tab, int N, unsigned long long x2) {
  return nci_beyond_cold(tab.d, N, x2);
}

// Chi-squared quantile of row N (d + 2N degrees of freedom) at the cell p of x2.
__device__ __forceinline__ float nci_row(const NciTable &tab, int N, const NciPos &p,
                                         unsigned long long x2, unsigned int &fallbacks) {
  if (N < tab.rows) return nci_cubic(nci_cell(tab, N, p), p.t);
  ++fallbacks;
  return nci_beyond_wh(tab.d, N, x2);
}

__device__ __forceinline__ float nci_quantile(const NciTable &tab, int N,
                                              unsigned long long x2,
                                              unsigned long long u999,
                                              unsigned int &fallbacks) {
  return nci_row(tab, N, nci_pos(tab, x2, u999), x2, fallbacks);
}

// One step of the CIR variance under scheme SCH (VolSchemes.hpp evolve()).
template <int SCH>
__device__ __forceinline__ float evolve(float v, Xo &rng, const FactorConst &f,
                                        const SimParams &P, int fi, unsigned int &caphits,
                                        unsigned int &fallbacks) {
  if (SCH == SCH_NV) {
    // VolSchemes.hpp:52-57: v' = ex (sqrt(ex v + D psi) + s* Z)^2 + D psi
    const float Z = inv_normal_bits(draw(rng));
    const float root = sqrt_approx(fmaf(f.w0, v, f.w1)) + f.w2 * Z;
    return fmaf(f.w0 * root, root, f.w1);
  } else if (SCH == SCH_EXACT) {
    // VolSchemes.hpp:207-218: N ~ Poisson(C0 v), v' = Gamma(alpha + N) * scale
    const int N = poisson_inv(f.w0 * v, draw(rng), P.loop_cap, caphits);
    const float g = gamma_draw(f.w1, N, rng, P.sm_p[fi], P.sm_inv_p[fi], P.sm_1mp[fi],
                               P.sm_1ma[fi], P.sm_inv_a[fi], P.loop_cap, caphits);
    return g * f.w2;
  } else {
    // VolSchemes.hpp:334-370: N ~ Poisson(C0 v), v' = chi2_{d+2N}^{-1}(U) * scale
    const int N = poisson_inv(f.w0 * v, draw(rng), P.loop_cap, caphits);
    const unsigned long long x2 = draw(rng);
    return nci_quantile(P.nci[fi], N, x2, P.nci_u999, fallbacks) * f.w2;
  }
}

// Compound-Poisson log jump of one window (JumpPolicies.hpp:55-75, :111-135),
// for the jump count n of the window.
__device__ __forceinline__ float jump_of_count(const SimParams &P, const ScenarioConst &C, int n, Xo &rng) {
  if (n == 0) return C.jump_comp;
  if (P.jump_kind == 1) {
    const float Z = inv_normal_bits(draw(rng));
    const float fn = (float)n;
    return C.jump_comp + fn * P.merton_mu + sqrtf(fn) * P.merton_delta * Z;
  }
  float total = 0.0f;
  const int m = min(n, (int)P.loop_cap);
  for (int k = 0; k < m; ++k) {
    const float u = u01_bits(draw(rng));
    if (u < P.kou_p_up)
      total += exp_draw(rng, P.kou_inv_eta1);
    else
      total -= exp_draw(rng, P.kou_inv_eta2);
  }
  return C.jump_comp + total;
}

__device__ __forceinline__ float jump_draw(const SimParams &P, const ScenarioConst &C, Xo &rng,
                                           unsigned int &caphits) {
  return jump_of_count(P, C, poisson_small(C.jump_mean, C.jump_exp_neg_mean, rng, P.loop_cap, caphits), rng);
}

// Tracker state of one path (PathTrackers.hpp:8-301): the running sum of an
// average, the running extremes of log S, and the hit times of the three
// barriers (base, spot-up, spot-down; < 0 = not hit).
struct TrackerState {
  float acc, mn, mx, tb, tu, td;
  __device__ __forceinline__ void init(const SimParams &P, bool pd) {
    acc = 0.0f;
    mn = P.lb_min0;
    mx = P.lb_max0;
    tb = tu = td = -1.0f;
    if (pd && P.tracker >= TRK_BARRIER_UP) {  // Day-0 breach (PathTrackers.hpp:194-215)
      if (P.tracker == TRK_BARRIER_UP) {
        if (0.0f >= P.b_log[0]) tb = 0.0f;
        if (0.0f >= P.b_log[1]) tu = 0.0f;
        if (0.0f >= P.b_log[2]) td = 0.0f;
      } else {
        if (0.0f <= P.b_log[0]) tb = 0.0f;
        if (0.0f <= P.b_log[1]) tu = 0.0f;
        if (0.0f <= P.b_log[2]) td = 0.0f;
      }
    }
  }
  // after step k (0-based) with log-spot X
  __device__ __forceinline__ void step(const SimParams &P, int k, float dt, float X) {
    const float t = (float)(k + 1) * dt;
    switch (P.tracker) {
      case TRK_GEO_ASIAN: acc += X; break;
      case TRK_ARITH_ASIAN: acc += __expf(X); break;
      case TRK_LOOKBACK:
        mn = fminf(mn, X);
        mx = fmaxf(mx, X);
        break;
      case TRK_BARRIER_UP:
        if (tu < 0.0f && X >= P.b_log[1]) tu = t;
        if (tb < 0.0f && X >= P.b_log[0]) tb = t;
        if (td < 0.0f && X >= P.b_log[2]) td = t;
        break;
      case TRK_BARRIER_DOWN:
        if (td < 0.0f && X <= P.b_log[2]) td = t;
        if (tb < 0.0f && X <= P.b_log[0]) tb = t;
        if (tu < 0.0f && X <= P.b_log[1]) tu = t;
        break;
      default: break;
    }
  }
  // the terminal record: X, then the tracker's fields
  __device__ __forceinline__ void finish(const SimParams &P, const ScenarioConst &C, float X, bool pd,
                                         float (&out)[kMaxFields]) const {
    out[0] = X;
    if (!pd) return;
    switch (P.tracker) {
      case TRK_GEO_ASIAN: out[1] = C.dt * (acc - 0.5f * X); break;
      case TRK_ARITH_ASIAN: out[1] = C.dt * (0.5f + acc - 0.5f * __expf(X)); break;
      case TRK_LOOKBACK:
        out[1] = mn;
        out[2] = mx;
        break;
      case TRK_BARRIER_UP:
      case TRK_BARRIER_DOWN:
        out[1] = tb;
        out[2] = tu;
        out[3] = td;
        break;
      default: break;
    }
  }
};

// Observer of a path's steps (the control-variate kernels record hedge-time
// states and martingale increments through it).  NoHook compiles away.
struct NoHook {
  static constexpr bool active = false;
  __device__ __forceinline__ void begin(float, float) {}
  // log-spot increment of the step: root * G + drift, G ~ N(0,1) independent of the variances
  __device__ __forceinline__ void diffusion(float, float, float) {}
  __device__ __forceinline__ void jump(float) {}
  // after step k (1-based): log-spot, variances, tracker accumulator, base barrier hit so far
  __device__ __forceinline__ void step_end(int, float, float, float, float, bool) {}
  __device__ __forceinline__ void finish() {}
};

// Simulates one path of one scenario; writes the tracker's terminal record.
// With an active hook every path is stepped (no single-draw GBM European) and
// the hook sees each step.  UNROLL > 0 unrolls the time-step loop by that depth
// (the batch autotuner's knob); 0 leaves the loop to the compiler.  The
// arithmetic of every step is the same either way.
template <int NF, int S1, int S2, bool PD, class Hook, int UNROLL = 0>
__device__ __forceinline__ void sim_path_h(const SimParams &P, const ScenarioConst &C, Xo &rng,
                                           float (&out)[kMaxFields], unsigned int &caphits,
                                           unsigned int &fallbacks, Hook &hook) {
  float X = 0.0f;
  float va = C.f[0].v0, vb = C.f[1].v0;
  TrackerState ts;
  ts.init(P, PD);
  const int n = P.n_steps;
  if (Hook::active) hook.begin(va, vb);
  if (NF == 0 && !PD && !Hook::active) {
    // GBM European: one Gaussian over T plus one jump (ASVJstepper.hpp:145-161)
    const float G = inv_normal_bits(draw(rng));
    X = fmaf(C.gbm_vol, G, C.gbm_drift);
    if (P.jump_kind) X += jump_draw(P, C, rng, caphits);
  } else {
    const float dt = C.dt;
    auto one_step = [&](int k) {
      const float G = inv_normal_bits(draw(rng));
      if (NF == 0) {
        X += fmaf(C.gbm_vol, G, C.gbm_drift);
        if (Hook::active) hook.diffusion(C.gbm_vol, G, C.gbm_drift);
      } else if (NF == 1) {
        const FactorConst &f = C.f[0];
        const float vn = evolve<S1>(va, rng, f, P, 0, caphits, fallbacks);
        const float root = sqrt_approx(f.C3 * (va + vn));
        const float drift = fmaf(f.C2, vn, fmaf(f.C1, va, f.C0));
        X += fmaf(root, G, drift);
        if (Hook::active) hook.diffusion(root, G, drift);
        va = vn;
      } else {
        const FactorConst &f0 = C.f[0];
        const FactorConst &f1 = C.f[1];
        const float van = evolve<S1>(va, rng, f0, P, 0, caphits, fallbacks);
        const float vbn = evolve<S2>(vb, rng, f1, P, 1, caphits, fallbacks);
        const float root = sqrt_approx(fmaf(f0.C3, va + van, f1.C3 * (vb + vbn)));
        const float drift = fmaf(f1.C2, vbn, fmaf(f1.C1, vb, fmaf(f0.C2, van,
                                 fmaf(f0.C1, va, f0.C0 + f1.C0))));
        X += fmaf(root, G, drift);
        if (Hook::active) hook.diffusion(root, G, drift);
        va = van;
        vb = vbn;
      }
      if (PD) {
        if (P.jump_kind) {
          const float J = jump_draw(P, C, rng, caphits);
          X += J;
          if (Hook::active) hook.jump(J);
        }
        ts.step(P, k, dt, X);
      }
      if (Hook::active) hook.step_end(k + 1, X, va, vb, ts.acc, ts.tb >= 0.0f);
    };
    if constexpr (UNROLL > 0) {
#pragma unroll UNROLL
      for (int k = 0; k < n; ++k) one_step(k);
    } else {
      for (int k = 0; k < n; ++k) one_step(k);
    }
    if (!PD && (NF > 0 || Hook::active) && P.jump_kind) {
      const float J = jump_draw(P, C, rng, caphits);
      X += J;
      if (Hook::active) hook.jump(J);
    }
  }
  if (Hook::active) hook.finish();
  ts.finish(P, C, X, PD, out);
}

template <int NF, int S1, int S2, bool PD, int UNROLL = 0>
__device__ __forceinline__ void sim_path(const SimParams &P, const ScenarioConst &C, Xo &rng,
                                         float (&out)[kMaxFields], unsigned int &caphits,
                                         unsigned int &fallbacks) {
  NoHook h;
  sim_path_h<NF, S1, S2, PD, NoHook, UNROLL>(P, C, rng, out, caphits, fallbacks, h);
}

template <int NF, int S1, int S2, bool PD>
__global__ void __launch_bounds__(kSimBlock) simulate_kernel(const __grid_constant__ SimParams P) {
  const unsigned int s = blockIdx.x * kSimBlock + threadIdx.x;
  const unsigned int S = P.n_streams;
  if (s >= S) return;
  Xo rng;
  rng.a = P.states[s];
  rng.b = P.states[(size_t)S + s];
  rng.c = P.states[2 * (size_t)S + s];
  rng.d = P.states[3 * (size_t)S + s];
  unsigned int caphits = 0, fallbacks = 0;
  const int F = P.n_fields;
  for (unsigned long long i = P.path_begin + s; i < P.path_end; i += S) {
    const Xo start = rng;
    const size_t col = (size_t)(i - P.rec_offset);
    float x_base = 0.0f;
    for (int sc = 0; sc < P.n_sc; ++sc) {
      float f[kMaxFields];
      if (!PD && (sc == SC_RUP || sc == SC_RDN)) {
        // A rate bump moves only the drift: X_T(r') = X_T(r) + (r' - r) T on the same
        // variance path and jumps (the reference re-simulates it with the same numbers).
        P.records[(size_t)sc * F * P.rec_stride + col] = x_base + P.sc[sc].x_shift;
        continue;
      }
      Xo r = start;
      sim_path<NF, S1, S2, PD>(P, P.sc[sc], r, f, caphits, fallbacks);
      if (sc == 0) x_base = f[0];
      float *dst = P.records + (size_t)sc * F * P.rec_stride + col;
      dst[0] = f[0];
      if (PD) {
        if (F > 1) dst[P.rec_stride] = f[1];
        if (F > 2) dst[2 * P.rec_stride] = f[2];
        if (F > 3) dst[3 * P.rec_stride] = f[3];
      }
      if (sc == 0) rng = r;
    }
  }
  P.states[s] = rng.a;
  P.states[(size_t)S + s] = rng.b;
  P.states[2 * (size_t)S + s] = rng.c;
  P.states[3 * (size_t)S + s] = rng.d;
  if (caphits) atomicAdd(P.status, caphits);
  if (fallbacks) atomicAdd(P.status + 1, fallbacks);
}

// ---------------------------------------------------------------------------
// Scenario lockstep (GreekMode::Full, European instruments, NV / NCI factors).
//
// Under these schemes a step consumes the same draws in every scenario (one for
// the spot Gaussian, one per NV factor, two per NCI factor) and the jump of a
// European path is drawn once after the last step, so the replays of a path
// read the same random numbers step by step.  One thread then advances all
// simulated scenarios of its path together: the draws, the spot Gaussian, the
// Poisson draw's U and W and the chi-squared table cell are computed once per
// step, and only the parts that depend on a scenario's variance and constants
// run per scenario.  Every scenario's arithmetic is the per-scenario kernel's,
// so its record is bit-identical.


// Simulated scenarios of a European Full request in lockstep order: base,
// v0 (or factor-0 v0) up / down, T up / down, then factor-1 v0 up / down.
__host__ __device__ constexpr int lockstep_sc(int j) { return j < 5 ? j : j + 2; }

// Merged variance paths.  Under SchemeNCI the next variance depends on the
// current one only through the Poisson count N (the table row): a v0-bumped
// scenario shares the base's time step, so once its variance equals the
// base's bit for bit (from the first step at which both draw the same N), it
// stays equal for the rest of the path.  A step then evolves
// inline only the scenarios with their own time step -- base, T up, T down --
// and gives a merged scenario the base's new variance: the value its own
// evaluation would give.  A scenario that has not merged yet runs on its own
// (nci_step_one), on the lanes that need it.  Lockstep order of the shared
// subset: 0, 3, 4.
__host__ __device__ constexpr int lockstep_sub(int j) { return j == 0 ? 0 : j + 2; }
__host__ __device__ constexpr bool lockstep_merges(int j) { return j != 0 && j != 3 && j != 4; }

// The per-step draws of one factor, shared by every scenario.
template <int SCH>
struct FactorDraws {
  float Z = 0.0f;                     // NV: Gaussian of the variance step
  unsigned long long xp = 0, x2 = 0;  // NCI: Poisson and chi-squared draws
  float U = 0.0f;                     // NCI: uniform of xp
  float W = 0.0f;                     // NCI: normal quantile of xp (Giles' estimate)
  NciPos pos{};                       // NCI: table cell of x2
};

template <int SCH>
__device__ __forceinline__ void factor_draws(FactorDraws<SCH> &d, Xo &rng, const SimParams &P,
                                             int fi) {
  if (SCH == SCH_NV) {
    d.Z = inv_normal_bits(draw(rng));
  } else if (SCH == SCH_NCI) {
    d.xp = draw(rng);
    d.U = u01_bits(d.xp);
    d.W = inv_normal_bits(d.xp);  // once per step for every scenario's inversion
    d.x2 = draw(rng);
    d.pos = nci_pos(P.nci[fi], d.x2, P.nci_u999);
  }
}

// evolve<SCH> (above) of one factor for every scenario, with the step's draws
// given: the Poisson inversions of all scenarios first, then all their table
// gathers (independent loads in flight together), then the cubic cells.
// SUB: the NS = 3 scenarios of lockstep_sub; a table fallback of the base then
// stands for the base and its `merged` copies.
template <int SCH, int NS, bool SUB = false, bool PRECISE = false>
__device__ __forceinline__ void evolve_lockstep(const float (&v)[NS], float (&vn)[NS],
                                                const FactorDraws<SCH> &d, const SimParams &P,
                                                int fi, unsigned int &caphits,
                                                unsigned int &fallbacks, unsigned int merged = 0) {
  static_assert(!PRECISE || (SUB && NS == 3), "the T-bumped pair of the merged subset");
  auto sc = [](int j) { return SUB ? lockstep_sub(j) : lockstep_sc(j); };
  if (SCH == SCH_NV) {
#pragma unroll
    for (int j = 0; j < NS; ++j) {
      const FactorConst &f = P.sc[sc(j)].f[fi];
      const float root = sqrt_approx(fmaf(f.w0, v[j], f.w1)) + f.w2 * d.Z;
      vn[j] = fmaf(f.w0 * root, root, f.w1);
    }
  } else {
    float lam[NS];
    int N[NS];
    constexpr bool PAIR = NS == 3;  // scenarios 1 and 2 (T up, T down) on packed pairs
    if constexpr (PAIR) {
      lam[0] = P.sc[sc(0)].f[fi].w0 * v[0];
      float2 l = pk::fmul2(make_float2(P.sc[sc(1)].f[fi].w0, P.sc[sc(2)].f[fi].w0), make_float2(v[1], v[2]));
      if constexpr (PRECISE)  // + (w0 - fl(w0)) v
        l = pk::ffma2(make_float2(P.sc[sc(1)].lo[4], P.sc[sc(2)].lo[4]), make_float2(v[1], v[2]), l);
      lam[1] = l.x;
      lam[2] = l.y;
    } else {
#pragma unroll
      for (int j = 0; j < NS; ++j) lam[j] = P.sc[sc(j)].f[fi].w0 * v[j];
    }
    poisson_eval_n<NS>(lam, d.U, d.W, d.xp, P.loop_cap, caphits, N);
    const NciTable &tab = P.nci[fi];
    float4 c[NS];
#pragma unroll
    for (int j = 0; j < NS; ++j) c[j] = nci_cell(tab, N[j], d.pos);
    float q[NS];
    if constexpr (PAIR) {
      q[0] = nci_cubic(c[0], d.pos.t);
      const float2 t2 = make_float2(d.pos.t, d.pos.t);
      float2 h = pk::ffma2(make_float2(c[1].w, c[2].w), t2, make_float2(c[1].z, c[2].z));
      h = pk::ffma2(h, t2, make_float2(c[1].y, c[2].y));
      h = pk::ffma2(h, t2, make_float2(c[1].x, c[2].x));
      q[1] = h.x;
      q[2] = h.y;
    } else {
#pragma unroll
      for (int j = 0; j < NS; ++j) q[j] = nci_cubic(c[j], d.pos.t);
    }
#pragma unroll
    for (int j = 0; j < NS; ++j) {
      if (N[j] >= tab.rows) {
        fallbacks += (SUB && j == 0) ? 1 + merged : 1;
        q[j] = nci_beyond(tab, N[j], d.x2);
      }
    }
    if constexpr (PAIR) {
      vn[0] = q[0] * P.sc[sc(0)].f[fi].w2;
      float2 w = pk::fmul2(make_float2(q[1], q[2]), make_float2(P.sc[sc(1)].f[fi].w2, P.sc[sc(2)].f[fi].w2));
      if constexpr (PRECISE)  // + q (w2 - fl(w2))
        w = pk::ffma2(make_float2(q[1], q[2]), make_float2(P.sc[sc(1)].lo[5], P.sc[sc(2)].lo[5]), w);
      vn[1] = w.x;
      vn[2] = w.y;
    } else {
#pragma unroll
      for (int j = 0; j < NS; ++j) vn[j] = q[j] * P.sc[sc(j)].f[fi].w2;
    }
  }
}

// One NCI scenario on the step's shared draws, for the lanes whose scenario
// has not merged yet: the arithmetic of evolve_lockstep for one mean
// (poisson_eval_n gives each mean poisson_eval's N).  Inline: an out-of-line
// call cost 13 % at 200 steps in instruction-fetch stalls.
struct NciOne {
  float v;
  unsigned int caphits, fallbacks;
};
__device__ __forceinline__ NciOne nci_step_one(float lam, float scale, const NciTable &tab,
                                               unsigned long long xp, float U, float W,
                                               unsigned long long x2, NciPos pos,
                                               unsigned int cap) {
  NciOne o{0.0f, 0u, 0u};
  const int N = poisson_eval(lam, U, W, xp, cap, o.caphits);
  float q = nci_cubic(nci_cell(tab, N, pos), pos.t);
  if (N >= tab.rows) {
    o.fallbacks = 1;
    q = nci_beyond(tab, N, x2);
  }
  o.v = q * scale;
  return o;
}

// evolve_lockstep of one NCI factor with merged variance paths (see lockstep_sub).
template <int NS, bool PRECISE = false>
__device__ __forceinline__ void evolve_merged(const float (&v)[NS], float (&vn)[NS],
                                              const FactorDraws<SCH_NCI> &d, const SimParams &P,
                                              int fi, unsigned int &caphits,
                                              unsigned int &fallbacks) {
  bool same[NS];
  unsigned int nm = 0;
#pragma unroll
  for (int j = 0; j < NS; ++j) {
    same[j] = lockstep_merges(j) && v[j] == v[0];
    nm += same[j] ? 1u : 0u;
  }
  const float v3[3] = {v[0], v[3], v[4]};
  float o3[3];
  evolve_lockstep<SCH_NCI, 3, true, PRECISE>(v3, o3, d, P, fi, caphits, fallbacks, nm);
  unsigned int todo = 0;  // the v0-bumped scenarios that have not merged yet
#pragma unroll
  for (int j = 0; j < NS; ++j) {
    vn[j] = (j == 3 || j == 4) ? o3[j - 2] : o3[0];
    todo |= lockstep_merges(j) && !same[j] ? 1u << j : 0u;
  }
  // One copy of their inversion, run once per pending scenario: lanes waiting on different
  // scenarios run it together, and the step's code holds one copy instead of one per scenario.
#pragma unroll 1
  while (todo) {
    const int j = __ffs(todo) - 1;
    todo &= todo - 1;
    float vj = v[1];
#pragma unroll
    for (int k = 2; k < NS; ++k) vj = k == j ? v[k] : vj;
    const FactorConst &f = P.sc[lockstep_sc(j)].f[fi];
    const NciOne o = nci_step_one(f.w0 * vj, f.w2, P.nci[fi], d.xp, d.U, d.W, d.x2, d.pos, P.loop_cap);
#pragma unroll
    for (int k = 1; k < NS; ++k) vn[k] = k == j ? o.v : vn[k];
    caphits += o.caphits;
    fallbacks += o.fallbacks;
  }
}

// One time step of every simulated scenario of one path: the loop body of the lockstep
// kernels.  MERGE: the v0-bumped scenarios' variance paths merge into the base's (every
// factor on NCI, and P.lock_merge: the host found their NCI constants equal).
template <int NF, int S1, int S2, int NSIM, bool MERGE, bool PRECISE = false>
__device__ __forceinline__ void lockstep_step(const SimParams &P, Xo &rng, float (&X)[NSIM], float (&va)[NSIM],
                                              float (&vb)[NSIM], unsigned int &caphits,
                                              unsigned int &fallbacks) {
  const float G = inv_normal_bits(draw(rng));
  FactorDraws<S1> da;
  FactorDraws<S2> db;
  factor_draws<S1>(da, rng, P, 0);
  if (NF == 2) factor_draws<S2>(db, rng, P, 1);
  float van[NSIM], vbn[NSIM];
  static_assert(!PRECISE || (MERGE && NF == 1), "the merged one-factor kernel");
  if constexpr (MERGE) {
    evolve_merged<NSIM, PRECISE>(va, van, da, P, 0, caphits, fallbacks);
    if constexpr (NF == 2) evolve_merged<NSIM>(vb, vbn, db, P, 1, caphits, fallbacks);
  } else {
    evolve_lockstep<S1, NSIM>(va, van, da, P, 0, caphits, fallbacks);
    if (NF == 2) evolve_lockstep<S2, NSIM>(vb, vbn, db, P, 1, caphits, fallbacks);
  }
  if constexpr (NF == 1) {
    // scenarios 1..NSIM-1 in pairs on packed FP32 (each lane rounds as the scalar form)
    static_assert(NSIM % 2 == 1, "the base and pairs of bumped scenarios");
    {
      const FactorConst &f = P.sc[0].f[0];
      const float vn = van[0];
      const float root = sqrt_approx(f.C3 * (va[0] + vn));
      const float drift = fmaf(f.C2, vn, fmaf(f.C1, va[0], f.C0));
      X[0] += fmaf(root, G, drift);
      va[0] = vn;
    }
#pragma unroll
    for (int j = 1; j + 1 < NSIM; j += 2) {
      const FactorConst &f = P.sc[lockstep_sc(j)].f[0], &g = P.sc[lockstep_sc(j + 1)].f[0];
      const float2 v0 = make_float2(va[j], va[j + 1]), v1 = make_float2(van[j], van[j + 1]);
      const float2 sv = pk::fadd2(v0, v1);
      float2 c3 = pk::fmul2(make_float2(f.C3, g.C3), sv);
      float2 drift = pk::ffma2(make_float2(f.C2, g.C2), v1,
                                pk::ffma2(make_float2(f.C1, g.C1), v0, make_float2(f.C0, g.C0)));
      if constexpr (PRECISE) {
        if (lockstep_sc(j) == SC_TUP) {  // the T-bumped pair: + the constants' FP32 rounding errors
          const float *lf = P.sc[SC_TUP].lo, *lg = P.sc[SC_TDN].lo;
          c3 = pk::ffma2(make_float2(lf[3], lg[3]), sv, c3);
          drift = pk::fadd2(drift, pk::ffma2(make_float2(lf[2], lg[2]), v1,
                                             pk::ffma2(make_float2(lf[1], lg[1]), v0, make_float2(lf[0], lg[0]))));
        }
      }
      const float2 root = make_float2(sqrt_approx(c3.x), sqrt_approx(c3.y));
      const float2 x = pk::fadd2(make_float2(X[j], X[j + 1]), pk::ffma2(root, make_float2(G, G), drift));
      X[j] = x.x;
      X[j + 1] = x.y;
      va[j] = v1.x;
      va[j + 1] = v1.y;
    }
  } else {
#pragma unroll
    for (int j = 0; j < NSIM; ++j) {
      const ScenarioConst &C = P.sc[lockstep_sc(j)];
      const FactorConst &f0 = C.f[0];
      const FactorConst &f1 = C.f[1];
      const float root = sqrt_approx(fmaf(f0.C3, va[j] + van[j], f1.C3 * (vb[j] + vbn[j])));
      const float drift = fmaf(f1.C2, vbn[j], fmaf(f1.C1, vb[j], fmaf(f0.C2, van[j],
                               fmaf(f0.C1, va[j], f0.C0 + f1.C0))));
      X[j] += fmaf(root, G, drift);
      va[j] = van[j];
      vb[j] = vbn[j];
    }
  }
}

template <int NSIM>
__device__ __forceinline__ void lockstep_start(const SimParams &P, float (&X)[NSIM], float (&va)[NSIM],
                                               float (&vb)[NSIM]) {
#pragma unroll
  for (int j = 0; j < NSIM; ++j) {
    X[j] = 0.0f;
    va[j] = P.sc[lockstep_sc(j)].f[0].v0;
    vb[j] = P.sc[lockstep_sc(j)].f[1].v0;
  }
}

// Path end: one jump over each scenario's (bumped) maturity, drawn from the state after
// the last step (the base scenario's draws advance the stream), then the records,
// the two rho scenarios derived from the base.
template <int NSIM, bool PRECISE = false>
__device__ __forceinline__ void lockstep_finish(const SimParams &P, Xo &rng, float (&X)[NSIM], size_t col,
                                                unsigned int &caphits) {
  if (P.jump_kind) {
    Xo after = rng;
#pragma unroll
    for (int j = 0; j < NSIM; ++j) {
      Xo r = after;
      if (PRECISE && (lockstep_sc(j) == SC_TUP || lockstep_sc(j) == SC_TDN)) {
        // the T-bumped windows' means differ by 2 t_bump lambda: their count in FP64, and
        // the compensation's FP32 rounding error added back
        const ScenarioConst &C = P.sc[lockstep_sc(j)];
        const int2 nj = poisson_small_fp64(C.jump_mean_d, draw(r), P.loop_cap);
        caphits += (unsigned int)nj.y;
        X[j] += jump_of_count(P, C, nj.x, r) + C.lo[6];
      } else
        X[j] += jump_draw(P, P.sc[lockstep_sc(j)], r, caphits);
      if (j == 0) rng = r;
    }
  }
  const size_t F = (size_t)P.n_fields;
#pragma unroll
  for (int j = 0; j < NSIM; ++j)
    P.records[(size_t)lockstep_sc(j) * F * P.rec_stride + col] = X[j];
  P.records[(size_t)SC_RUP * F * P.rec_stride + col] = X[0] + P.sc[SC_RUP].x_shift;
  P.records[(size_t)SC_RDN * F * P.rec_stride + col] = X[0] + P.sc[SC_RDN].x_shift;
}

template <int NF, int S1, int S2, int NSIM, bool MERGE = false, bool PRECISE = false>
__global__ void __launch_bounds__(kSimBlock) simulate_lockstep_kernel(
    const __grid_constant__ SimParams P) {
  static_assert(NF >= 1 && S1 != SCH_EXACT && S2 != SCH_EXACT, "lockstep needs NV/NCI factors");
  static_assert(!MERGE || (S1 == SCH_NCI && (NF == 1 || S2 == SCH_NCI)), "merging needs NCI factors");
  const unsigned int s = blockIdx.x * kSimBlock + threadIdx.x;
  const unsigned int S = P.n_streams;
  if (s >= S) return;
  Xo rng;
  rng.a = P.states[s];
  rng.b = P.states[(size_t)S + s];
  rng.c = P.states[2 * (size_t)S + s];
  rng.d = P.states[3 * (size_t)S + s];
  unsigned int caphits = 0, fallbacks = 0;
  const int n = P.n_steps;
  for (unsigned long long i = P.path_begin + s; i < P.path_end; i += S) {
    float X[NSIM], va[NSIM], vb[NSIM];
    lockstep_start<NSIM>(P, X, va, vb);
    for (int k = 0; k < n; ++k) lockstep_step<NF, S1, S2, NSIM, MERGE, PRECISE>(P, rng, X, va, vb, caphits, fallbacks);
    lockstep_finish<NSIM, PRECISE>(P, rng, X, (size_t)(i - P.rec_offset), caphits);
  }
  P.states[s] = rng.a;
  P.states[(size_t)S + s] = rng.b;
  P.states[2 * (size_t)S + s] = rng.c;
  P.states[3 * (size_t)S + s] = rng.d;
  if (caphits) atomicAdd(P.status, caphits);
  if (fallbacks) atomicAdd(P.status + 1, fallbacks);
}

}  // namespace dev

// Host launcher: dispatches to the compiled instantiation (defined in sim_*.cu).
cudaError_t launch_simulate(const SimParams &P, int s1, int s2, bool path_dep,
                            cudaStream_t stream);

}  // namespace myql
