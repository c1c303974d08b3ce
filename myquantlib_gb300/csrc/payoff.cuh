// payoff.cuh -- payoff evaluation shared by the payoff/reduce kernel and the
// MLMC level kernel (Payoffs.hpp, options/*.hpp calculate_to_buffer).
#pragma once
#include "engine_types.h"

namespace myql {
namespace dev {

// Value of one (scenario, strike) at the spot bumps s = 0, +1, -1, returned as
// v = v(0) and the increments dp = v(+1) - v(0), dm = v(-1) - v(0).
// The increments are formed without subtracting two FP32 payoffs where the
// payoff is linear or smooth over the bump: on a linear piece of max(y, 0)
// they are exactly +-b or 0, and for the erfc-smoothed digitals they come from
// the Taylor series of Phi over the bump.  This keeps the pathwise
// finite-difference delta and gamma of MonteCarloPricer.hpp:269-271 free of
// FP32 cancellation noise (which would otherwise dominate deep in or out of
// the money and for homogeneous floating-strike payoffs).
struct Tri {
  float v, dp, dm;
};

// max(y0 + c, 0) - max(y0, 0)
__device__ __forceinline__ float ramp_incr(float y0, float c) {
  const float y1 = y0 + c;
  if (y0 >= 0.0f && y1 >= 0.0f) return c;
  if (y0 <= 0.0f && y1 <= 0.0f) return 0.0f;
  return fmaxf(y1, 0.0f) - fmaxf(y0, 0.0f);
}

// Phi(x + c) - Phi(x) for the smoothed digitals (Payoffs.hpp:345-368).
__device__ __forceinline__ float smooth_incr(float x, float c, float phi0) {
  if (fabsf(c) < 0.05f) {
    // sum_{n>=1} c^n / n! (-1)^(n-1) He_{n-1}(x) phi(x), He the Hermite polynomials
    const float x2 = x * x;
    const float h1 = x, h2 = x2 - 1.0f, h3 = x * (x2 - 3.0f), h4 = fmaf(x2, x2 - 6.0f, 3.0f);
    float t = fmaf(c * (1.0f / 120.0f), h4, -(1.0f / 24.0f) * h3);
    t = fmaf(c, t, (1.0f / 6.0f) * h2);
    t = fmaf(c, t, -0.5f * h1);
    t = fmaf(c, t, 1.0f);
    return c * t * phi0;
  }
  return 0.5f * erfcf(-(x + c) * 0.70710678f) - 0.5f * erfcf(-x * 0.70710678f);
}

// One payoff of Payoffs.hpp (call/put applied through the sign of y):
// y0 = +-(spot - strike) at s = 0, b = its change per unit bump,
// x = the spot-like argument (asset-or-nothing pays x * (1 + s * eps_rel)).
// SPEC = 1 compiles the vanilla European case alone (the strip workloads);
// SPEC = 0 dispatches on the request's runtime kind, tracker and payoff.
template <int SPEC = 0>
__device__ __forceinline__ Tri payoff_tri(const PayoffParams &P, float y0, float b, float x,
                                          bool smooth, bool bumps) {
  Tri r;
  if (SPEC == 1 || P.payoff == 0) {
    r.v = fmaxf(y0, 0.0f);
    if (bumps) {
      r.dp = ramp_incr(y0, b);
      r.dm = ramp_incr(y0, -b);
    }
    return r;
  }
  float H0, Hp = 0.0f, Hm = 0.0f;  // H(s) - H(0) for the bumps
  if (smooth) {
    const float k = P.smooth_eps;  // 1 / (eps sqrt 2)
    const float xs = y0 * k * 1.41421356f, cs = b * k * 1.41421356f;  // standardized
    H0 = 0.5f * erfcf(-y0 * k);
    if (bumps) {
      const float phi0 = 0.39894228f * __expf(-0.5f * xs * xs);
      Hp = smooth_incr(xs, cs, phi0);
      Hm = smooth_incr(xs, -cs, phi0);
    }
  } else {
    H0 = y0 > 0.0f ? 1.0f : 0.0f;
    if (bumps) {
      Hp = (y0 + b > 0.0f ? 1.0f : 0.0f) - H0;
      Hm = (y0 - b > 0.0f ? 1.0f : 0.0f) - H0;
    }
  }
  if (P.payoff == 1) {
    r.v = H0;
    r.dp = Hp;
    r.dm = Hm;
    return r;
  }
  const float ex = x * P.eps_rel;
  r.v = x * H0;
  r.dp = fmaf(x, Hp, ex * (H0 + Hp));
  r.dm = fmaf(x, Hm, -ex * (H0 + Hm));
  return r;
}

// Values of one (scenario, strike): S = terminal spot, Y = average / extreme,
// hit[3] = hit times (base, up, dn; < 0 = not hit).
struct PathView {
  float S, Y;
  float hit[3];
};

template <int SPEC = 0>
__device__ __forceinline__ Tri scenario_tri(const PayoffParams &P, const PathView &v, float K,
                                            bool bumps) {
  const float sgn = P.option_type == 0 ? 1.0f : -1.0f;
  if (SPEC == 1) return payoff_tri<1>(P, sgn * (v.S - K), sgn * v.S * P.eps_rel, v.S, false, bumps);
  float x, d0, slope;
  switch (P.kind) {
    case 1:  // Asian (Asian.hpp:114-121)
    case 2:
    case 3:  // Lookback (Lookback.hpp:191-202, 237-242); Y carries the extreme in use
      if (P.fixed_strike) {
        x = v.Y;
        d0 = v.Y - K;
        slope = v.Y;
      } else {
        x = v.S;
        d0 = v.S - v.Y;
        slope = d0;
      }
      break;
    default:  // European, Barrier
      x = v.S;
      d0 = v.S - K;
      slope = v.S;
      break;
  }
  const float y0 = sgn * d0, b = sgn * slope * P.eps_rel;
  if (P.kind != 4) return payoff_tri(P, y0, b, x, P.smooth != 0, bumps);
  // Barrier (Barrier.hpp:29-45): sharp payoff, knock state per bump.
  const Tri pay = payoff_tri(P, y0, b, x, false, bumps);
  auto rebate_at = [&](float th) {
    float rb = 0.0f;
    if (P.rebate_timing != 0) {
      rb = P.rebate;
      if (P.rebate_timing == 1 && th >= 0.0f) rb = P.rebate * __expf(P.barrier_rate * (P.T_instr - th));
    }
    return rb;
  };
  const bool h0 = v.hit[0] >= 0.0f;
  const bool knock_in = P.barrier_action == 0;
  auto value = [&](bool hit, float payv, float th) {
    return (hit == knock_in) ? payv : rebate_at(th);
  };
  Tri r;
  r.v = value(h0, pay.v, v.hit[0]);
  if (bumps) {
    const bool hp = v.hit[1] >= 0.0f, hm = v.hit[2] >= 0.0f;
    const bool pays0 = h0 == knock_in;
    if (hp == h0 && pays0) {
      r.dp = pay.dp;
    } else {
      r.dp = value(hp, pay.v + pay.dp, v.hit[1]) - r.v;
    }
    if (hm == h0 && pays0) {
      r.dm = pay.dm;
    } else {
      r.dm = value(hm, pay.v + pay.dm, v.hit[2]) - r.v;
    }
  }
  return r;
}

}  // namespace dev
}  // namespace myql
