// device_numerics.cuh -- FP32 samplers of the path kernels (sm_103a).
//
// Random numbers: xoshiro256++ (Blackman & Vigna), one 64-bit draw per uniform,
// exactly as boost::random::uniform_real_distribution<double>(0,1) consumes
// them (draws whose double rounds to 1.0 are rejected and redrawn).  Uniforms
// are formed in "q-space": the 64-bit integer is converted so that FP32 keeps
// full relative precision in BOTH tails (min(p, 1-p) is taken on the integer,
// before any rounding), which is what the inverse-normal and inverse-Poisson
// tails need.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace myql {
namespace dev {

struct Xo {
  unsigned long long a, b, c, d;
};

// Packed FP32 pairs (sm_100 and later): each lane rounds as the scalar instruction.
namespace pk {
__device__ __forceinline__ float2 ffma2(float2 a, float2 b, float2 c) {
  float2 r;
  asm("{\n\t.reg .b64 ra, rb, rc, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
      "mov.b64 rc, {%6, %7};\n\tfma.rn.f32x2 rd, ra, rb, rc;\n\tmov.b64 {%0, %1}, rd;\n\t}"
      : "=f"(r.x), "=f"(r.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
  return r;
}
__device__ __forceinline__ float2 fmul2(float2 a, float2 b) {
  float2 r;
  asm("{\n\t.reg .b64 ra, rb, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
      "mul.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"
      : "=f"(r.x), "=f"(r.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return r;
}
__device__ __forceinline__ float2 fadd2(float2 a, float2 b) {
  float2 r;
  asm("{\n\t.reg .b64 ra, rb, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
      "add.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"
      : "=f"(r.x), "=f"(r.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return r;
}
}  // namespace pk

__device__ __forceinline__ unsigned long long rotl64(unsigned long long x, int k) {
  return (x << k) | (x >> (64 - k));
}

// xoshiro256++ next(): output rotl(s0 + s3, 23) + s0, then the linear state update.
__device__ __forceinline__ unsigned long long xo_next(Xo &s) {
  const unsigned long long out = rotl64(s.a + s.d, 23) + s.a;
  const unsigned long long t = s.b << 17;
  s.c ^= s.a;
  s.d ^= s.b;
  s.b ^= s.c;
  s.a ^= s.d;
  s.c ^= t;
  s.d = rotl64(s.d, 45);
  return out;
}

// One uniform_real_distribution<double>(0,1) draw: the double of x / 2^64 is
// rejected when it rounds to 1.0, i.e. for x >= 2^64 - 2^10 (2^-54 of draws).
// The redraws run out of line, so the path kernels' loops hold no cold copy of
// the generator.
struct XoDraw {
  Xo s;
  unsigned long long x;
};
static __device__ __noinline__ XoDraw draw_again(Xo s) {
  unsigned long long x = xo_next(s);
  while (x >= 0xFFFFFFFFFFFFFC00ull) x = xo_next(s);
  return XoDraw{s, x};
}
__device__ __forceinline__ unsigned long long draw(Xo &s) {
  const unsigned long long x = xo_next(s);
  if (x < 0xFFFFFFFFFFFFFC00ull) return x;
  const XoDraw r = draw_again(s);
  s = r.s;
  return r.x;
}

// x * 2^-64 rounded down to 24 significant bits (relative precision at any scale).
__device__ __forceinline__ float u01_bits(unsigned long long x) {
  x = x ? x : 1ull;  // 0 -> 2^-64 (the only input clz cannot normalize)
  const int n = __clzll(x);
  const unsigned long long m = x << n;
  const unsigned int bits =
      ((unsigned int)(126 - n) << 23) | ((unsigned int)(m >> 40) & 0x7FFFFFu);
  return __uint_as_float(bits);
}

// 1 - x * 2^-64, with the same relative precision near 0.
__device__ __forceinline__ float u01c_bits(unsigned long long x) { return u01_bits(~x); }

__device__ __forceinline__ float sqrt_approx(float x) {
  float r;
  asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

__device__ __forceinline__ float rsqrt_approx(float x) {
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// Inverse normal CDF of p = x * 2^-64, FP32.
// Central region p in [6.2e-4, 1 - 6.2e-4] (w <= 6 below):
//   z = (p - 1/2) * R(w),  w = -log(4 p (1 - p)),
// R a degree-10 polynomial fitted to Phi^-1 (csrc/fit_inverse_normal.py;
// FP32 relative error ~1.3e-7).  The variable w stays bounded and smooth as
// |p - 1/2| -> 1/2, so the coefficients are small and FP32 Horner is well
// conditioned, and only ~4% of warps ever take the tail branch.
// Tails: the tail rational of Acklam's approximation (P. J. Acklam, 2003), the
// algorithm of Numerics::normcdfinv_as241 (math/Numerics.hpp:12-47), in
// sqrt(-2 log min(p, 1-p)); it is already at FP32 round-off there.
__device__ __forceinline__ float inv_normal_bits(unsigned long long x) {
  const long long d = (long long)(x ^ 0x8000000000000000ull);  // (p - 1/2) * 2^64
  const unsigned long long ad =
      d < 0 ? (unsigned long long)(-(d + 1)) + 1ull : (unsigned long long)d;
  const float tq = u01_bits(0x8000000000000000ull - ad);  // min(p, 1-p)
  const float u4 = 4.0f * tq * (1.0f - tq);               // 4 p (1 - p)
  if (u4 >= 2.4787522e-3f) {                              // w = -log(u4) <= 6
    const float w = -__logf(u4);
    const float q = (float)(int)(d >> 32) * 2.3283064365386963e-10f;  // p - 1/2
    float R = 1.909701598e-09f;
    R = fmaf(R, w, -7.265112394e-08f);
    R = fmaf(R, w, 1.133204774e-06f);
    R = fmaf(R, w, -8.579473369e-06f);
    R = fmaf(R, w, 2.189081831e-05f);
    R = fmaf(R, w, 1.026849726e-04f);
    R = fmaf(R, w, -3.292963357e-04f);
    R = fmaf(R, w, -6.626443656e-03f);
    R = fmaf(R, w, 3.267393829e-02f);
    R = fmaf(R, w, 6.562327410e-01f);
    R = fmaf(R, w, 2.506628297e+00f);
    return q * R;
  }
  const float r = sqrt_approx(-2.0f * __logf(tq));
  const float num =
      fmaf(fmaf(fmaf(fmaf(fmaf(-7.784894002430293e-03f, r, -3.223964580411365e-01f), r,
                          -2.400758277161838e+00f), r, -2.549732539343734e+00f), r,
                4.374664141464968e+00f), r, 2.938163982698783e+00f);
  const float den =
      fmaf(fmaf(fmaf(fmaf(7.784695709041462e-03f, r, 3.224671290700398e-01f), r,
                     2.445134137142996e+00f), r, 3.754408661907416e+00f), r, 1.0f);
  const float z = __fdividef(num, den);
  return d < 0 ? z : -z;
}

// (1 + e) log(1 + e) - e, accurate for small |e| (series) and large (direct).
__device__ __forceinline__ float xlogx_m1(float e) {
  if (fabsf(e) < 0.25f) {
    // sum_{n>=2} (-1)^n e^n / (n (n-1))
    float s = 1.0f / 110.0f;
    s = fmaf(s, -e, 1.0f / 90.0f);
    s = fmaf(s, -e, 1.0f / 72.0f);
    s = fmaf(s, -e, 1.0f / 56.0f);
    s = fmaf(s, -e, 1.0f / 42.0f);
    s = fmaf(s, -e, 1.0f / 30.0f);
    s = fmaf(s, -e, 1.0f / 20.0f);
    s = fmaf(s, -e, 1.0f / 12.0f);
    s = fmaf(s, -e, 1.0f / 6.0f);
    s = fmaf(s, -e, 0.5f);
    return s * e * e;
  }
  return (1.0f + e) * log1pf(e) - e;
}

// log(1 + w) - w, accurate for small |w|.
__device__ __forceinline__ float log1p_m(float w) {
  if (fabsf(w) < 0.25f) {
    // -w^2/2 + w^3/3 - w^4/4 + ...
    float s = -1.0f / 12.0f;
    s = fmaf(s, w, 1.0f / 11.0f);
    s = fmaf(s, w, -1.0f / 10.0f);
    s = fmaf(s, w, 1.0f / 9.0f);
    s = fmaf(s, w, -1.0f / 8.0f);
    s = fmaf(s, w, 1.0f / 7.0f);
    s = fmaf(s, w, -1.0f / 6.0f);
    s = fmaf(s, w, 1.0f / 5.0f);
    s = fmaf(s, w, -1.0f / 4.0f);
    s = fmaf(s, w, 1.0f / 3.0f);
    s = fmaf(s, w, -0.5f);
    return s * w * w;
  }
  return log1pf(w) - w;
}

// Inverse Poisson CDF: smallest N with F_lambda(N) >= U, U = x * 2^-64.
// Follows the structure of Giles' algorithm (ACM TOMS 955), as used by
// Numerics::poissinvcdf (math/Numerics.hpp:49-272): a normal-asymptotic
// estimate (with a Newton solve in the tails) whose floor is checked with
// Temme's uniform expansion when it lies within 2*Delta of an integer, and an
// explicit summation for small means and small tail estimates.  Giles sums
// for every estimate below 10; here a central estimate below 10 is final
// outside its window and decided by a short sum inside it (kPoissonAsymMin
// below).  FP32 throughout; the summation runs in plain (unscaled) form,
// which is exact up to FP32 rounding of the CDF.
// U = u01_bits(x) and, where lam > 4, W = inv_normal_bits(x) depend on the draw
// alone: callers that invert one draw for several means compute them once.
// The common regimes (central estimate, summation) are inline; the tail solve
// and the near-integer check, taken by a few lanes in a thousand, are out of
// line so that the inlined path stays small.

// Normal-asymptotic estimate S and its error window Del, lambda > 4, |W| < 3.
__device__ __forceinline__ void poisson_central(float lam, float W, float &S, float &Del) {
  const float ir = rsqrt_approx(lam);  // 1/sqrt(lam): sqrt(lam) = lam * ir, 1/lam = ir^2
  const float rl = lam * ir;
  const float li = ir * ir;
  const float S1 = rl * W + (1.0f / 3.0f + (1.0f / 6.0f) * W * W) *
                                (1.0f - W * (1.0f / 12.0f) * ir);
  Del = fmaf(fmaf(1.0f / 160.0f, W * W, 1.0f / 80.0f), W * W, 1.0f / 40.0f) * li;
  S = __fadd_rn(lam, S1 + Del);  // never contracted with the caller's product
}

// Tail estimate (|W| >= 3): Newton on sqrt(2((1-R) + R log R)) = W / sqrt(lambda);
// quadratic convergence reaches FP32 resolution in a few steps, so a fixed
// small budget replaces the FP64 tolerance loop.  Returns (S, Del).
static __device__ __noinline__ float2 poisson_newton(float lam, float W) {
  const float s = W / sqrt_approx(lam);
  // start from the inverse series R = 1 + s + s^2/6 - s^3/72 + O(s^4) of the equation
  float R = fmaxf(1.0f + s * (1.0f + s * (1.0f / 6.0f - s * (1.0f / 72.0f))), 0.1f), R2;
  for (int it = 0; it < 12; ++it) {
    R2 = R;
    const float T = log1pf(R - 1.0f);
    float S2 = sqrtf(2.0f * xlogx_m1(R - 1.0f));
    if (R < 1.0f) S2 = -S2;
    R = R2 - (S2 - s) * S2 * rcp_approx(T);  // the step only: the root is set by S2
    if (R < 0.1f * R2) R = 0.1f * R2;
    if (fabsf(R - R2) <= 2e-7f * R) break;
  }
  const float T = log1pf(R - 1.0f);
  // O(1) corrections to lam * R: approximate divisions are far inside Del
  float S = lam * R + __logf(sqrt_approx(2.0f * R * xlogx_m1(R - 1.0f)) * rcp_approx(fabsf(R - 1.0f))) *
                          rcp_approx(T);
  S = S - 0.0218f * rcp_approx(S + 0.065f * lam);
  const float Del = 0.01f * rcp_approx(S);
  return make_float2(S + Del, Del);
}

// floor(S) = X lies within 2 Del of an integer: decide between X - 1 and X
// from the CDF at X - 1.
// The decision compares a CDF value with U, so approximate reciprocals and
// square roots (relative error ~1e-7) change it only for U within ~1e-7 of it.
static __device__ __noinline__ float poisson_check(float lam, float X, float U,
                                                   unsigned long long x) {
  const float li = rcp_approx(lam);
  if (X > 0.5f * lam && X < 2.0f * lam) {
    // Temme's uniform asymptotic expansion of the CDF at X - 1 (TOMS 955).
    const float Xi = rcp_approx(X);
    float Eta = sqrt_approx(2.0f * xlogx_m1(X * li - 1.0f) * rcp_approx(X * li));
    if (X > lam) Eta = -Eta;
    float B1 = 8.0995211567045583e-16f, B0;
    float T = B1;
    B0 = -1.9752288294349411e-15f;  T = B0 + T * Eta;
    B1 = -5.1391118342426808e-16f + 25.0f * B1 * Xi;  T = B1 + T * Eta;
    B0 = 2.8534893807047458e-14f + 24.0f * B0 * Xi;   T = B0 + T * Eta;
    B1 = -1.3923887224181616e-13f + 23.0f * B1 * Xi;  T = B1 + T * Eta;
    B0 = 3.3717632624009806e-13f + 22.0f * B0 * Xi;   T = B0 + T * Eta;
    B1 = 1.1004392031956284e-13f + 21.0f * B1 * Xi;   T = B1 + T * Eta;
    B0 = -5.0276692801141763e-12f + 20.0f * B0 * Xi;  T = B0 + T * Eta;
    B1 = 2.4361948020667402e-11f + 19.0f * B1 * Xi;   T = B1 + T * Eta;
    B0 = -5.8307721325504166e-11f + 18.0f * B0 * Xi;  T = B0 + T * Eta;
    B1 = -2.5514193994946487e-11f + 17.0f * B1 * Xi;  T = B1 + T * Eta;
    B0 = 9.1476995822367933e-10f + 16.0f * B0 * Xi;   T = B0 + T * Eta;
    B1 = -4.3820360184533521e-09f + 15.0f * B1 * Xi;  T = B1 + T * Eta;
    B0 = 1.0261809784240299e-08f + 14.0f * B0 * Xi;   T = B0 + T * Eta;
    B1 = 6.7078535434015332e-09f + 13.0f * B1 * Xi;   T = B1 + T * Eta;
    B0 = -1.7665952736826086e-07f + 12.0f * B0 * Xi;  T = B0 + T * Eta;
    B1 = 8.2967113409530833e-07f + 11.0f * B1 * Xi;   T = B1 + T * Eta;
    B0 = -1.8540622107151585e-06f + 10.0f * B0 * Xi;  T = B0 + T * Eta;
    B1 = -2.1854485106799979e-06f + 9.0f * B1 * Xi;   T = B1 + T * Eta;
    B0 = 3.9192631785224383e-05f + 8.0f * B0 * Xi;    T = B0 + T * Eta;
    B1 = -0.00017875514403292177f + 7.0f * B1 * Xi;   T = B1 + T * Eta;
    B0 = 0.00035273368606701921f + 6.0f * B0 * Xi;    T = B0 + T * Eta;
    B1 = 0.0011574074074074078f + 5.0f * B1 * Xi;     T = B1 + T * Eta;
    B0 = -0.014814814814814815f + 4.0f * B0 * Xi;     T = B0 + T * Eta;
    B1 = 0.083333333333333329f + 3.0f * B1 * Xi;      T = B1 + T * Eta;
    B0 = -0.33333333333333331f + 2.0f * B0 * Xi;      T = B0 + T * Eta;
    T = T * rcp_approx(1.0f + B1 * Xi);
    T = T * __expf(-0.5f * X * Eta * Eta) * rsqrt_approx(2.0f * 3.14159265358979f * X);
    if (X < lam) {
      T += 0.5f * erfcf(Eta * sqrt_approx(0.5f * X));
      if (T > U) X -= 1.0f;
    } else {
      T -= 0.5f * erfcf(-Eta * sqrt_approx(0.5f * X));
      if (T > -u01c_bits(x)) X -= 1.0f;
    }
  } else {
    // Stirling-corrected ratio, then a 50-term summation (tails only).
    float Xi = rcp_approx(X);
    float T = -(691.0f / 360360.0f);
    T = (1.0f / 1188.0f) + T * Xi * Xi;
    T = -(1.0f / 1680.0f) + T * Xi * Xi;
    T = (1.0f / 1260.0f) + T * Xi * Xi;
    T = -(1.0f / 360.0f) + T * Xi * Xi;
    T = (1.0f / 12.0f) + T * Xi * Xi;
    T = T * Xi;
    T = (X - lam) - X * __logf(X * li) - T;
    if (X < lam) {
      const float E = __expf(-0.5f * T);
      float Ssum = 1.0f - E * (U * E) * sqrt_approx(2.0f * 3.14159265358979f * Xi) * lam;
      float Tt = 1.0f, Xr = X;
      for (int i = 1; i < 50; ++i) {
        Xr -= 1.0f;
        Tt *= Xr * li;
        Ssum += Tt;
      }
      if (Ssum > 0.0f) X -= 1.0f;
    } else {
      const float E = __expf(-0.5f * T);
      float Ssum = 1.0f - E * (u01c_bits(x) * E) * sqrt_approx(2.0f * 3.14159265358979f * X);
      float Xr = X;
      for (int i = 0; i < 50; ++i) {
        Xr += 1.0f;
        Ssum = Ssum * Xr * li + 1.0f;
      }
      if (Ssum < 0.0f) X -= 1.0f;
    }
  }
  return X;
}

// Explicit summation of the CDF from 0: p_n = p_{n-1} * (lam * (1/n)), F_n = F_{n-1} + p_n.
// It returns the first n with U <= F_n, or lim if that comes first (lim = X
// decides between X - 1 and X; kPoissonSumAll sums without limit).  A second
// exit, p_n < 5e-8 F_n (F has stopped moving), guards the deep upper tail; it
// cannot fire first when U < 1 - 1e-5, because it needs the remaining mass
// below ~3e-7 while FP32 rounding of F stays under ~3e-6, so F_n already
// exceeds U there, and such draws skip it.
constexpr float kPoissonUFast = 0.99999f;
constexpr float kPoissonSumAll = 1.0e30f;

// Means above this use the normal-asymptotic estimate S of Giles' algorithm.
// For them S is increasing in W on |W| < 3, and at every step of the CDF
// (U = F(n), checked for every n and means in (1, 40] on a grid of 1/10000)
// S(W(U)) lies in [n + 1, n + 1 + 2 Del): so floor(S) is the inverse outside
// the window [X, X + 2 Del), and X - 1 or X inside it.  Giles sums the CDF
// whenever X < 10; here only the window cases are decided by a short sum
// (to X - 1), which gives the same N.
constexpr float kPoissonAsymMin = 2.5f;

// Giles' estimate (mean above kPoissonAsymMin) and how to finish: done (X is
// the answer), or a summation with limit lim (see poisson_sum).
__device__ __forceinline__ bool poisson_finish(float lam, float S, float Del, bool central,
                                               float U, unsigned long long x, float &X,
                                               float &lim) {
  X = floorf(S);
  const bool win = S < X + 2.0f * Del;
  lim = kPoissonSumAll;
  if (win && S > 10.0f) {
    X = poisson_check(lam, X, U, x);
    return !central && X < 10.0f;
  }
  if (central) {
    lim = X;
    return win && X >= 1.0f;
  }
  return X < 10.0f;  // tail estimates below 10: Giles' summation
}

__device__ __forceinline__ float poisson_sum(float lam, float U, float lim, unsigned int cap,
                                             unsigned int &caphits) {
  const bool fast = U < kPoissonUFast;
  float p = __expf(-lam);
  float F = p;
  float nf = 0.0f;
  unsigned int n = 0;
  for (;;) {
    if (!(U > F) || nf >= lim || (!fast && p < F * 5.0e-8f)) return nf;
    if (++n > cap) {
      ++caphits;
      return (float)n;
    }
    nf = (float)n;
    p *= lam * rcp_approx(nf);
    F += p;
  }
}

// poisson_sum out of line, for the deep upper tail (U >= kPoissonUFast, one
// draw in 1e5) of the multi-mean inversion: (X, loop-cap hits).
static __device__ __noinline__ float2 poisson_sum_tail(float lam, float U, float lim, unsigned int cap) {
  unsigned int hits = 0;
  const float X = poisson_sum(lam, U, lim, cap, hits);
  return make_float2(X, (float)hits);
}

__device__ __forceinline__ int poisson_eval(float lam, float U, float W, unsigned long long x,
                                            unsigned int cap, unsigned int &caphits) {
  float X = 0.0f, lim = kPoissonSumAll;
  bool sum = true;
  if (lam > kPoissonAsymMin) {
    float S, Del;
    const bool central = fabsf(W) < 3.0f;
    if (central) {
      poisson_central(lam, W, S, Del);
    } else {
      const float2 sd = poisson_newton(lam, W);
      S = sd.x;
      Del = sd.y;
    }
    sum = poisson_finish(lam, S, Del, central, U, x, X, lim);
  }
  if (sum) X = poisson_sum(lam, U, lim, cap, caphits);
  return (int)X;
}

// poisson_eval for NS means on one draw (the bumped scenarios of one path):
// each N[j] equals poisson_eval(lam[j], U, W, x), W = inv_normal_bits(x) from
// the caller (read only where some mean is above kPoissonAsymMin).  The central estimates run as
// straight-line code and the summations share one loop, so the scenarios'
// arithmetic interleaves and the loop overhead is paid once.
template <int NS>
__device__ __forceinline__ void poisson_eval_n(const float (&lam)[NS], float U, float W,
                                               unsigned long long x, unsigned int cap,
                                               unsigned int &caphits, int (&N)[NS]) {
  float X[NS], lim[NS];
  bool act[NS];
  bool big = false;
#pragma unroll
  for (int j = 0; j < NS; ++j) {
    X[j] = 0.0f;
    lim[j] = kPoissonSumAll;
    act[j] = true;
    big |= lam[j] > kPoissonAsymMin;
  }
  if (big) {
    const bool central = fabsf(W) < 3.0f;
    float S[NS], Del[NS];
    if (central) {
#pragma unroll
      for (int j = 0; j < NS; ++j) poisson_central(lam[j], W, S[j], Del[j]);
    } else {
#pragma unroll
      for (int j = 0; j < NS; ++j) {
        S[j] = Del[j] = 0.0f;
        if (lam[j] > kPoissonAsymMin) {
          const float2 sd = poisson_newton(lam[j], W);
          S[j] = sd.x;
          Del[j] = sd.y;
        }
      }
    }
#pragma unroll
    for (int j = 0; j < NS; ++j)
      if (lam[j] > kPoissonAsymMin)
        act[j] = poisson_finish(lam[j], S[j], Del[j], central, U, x, X[j], lim[j]);
  }
  bool any = false;
#pragma unroll
  for (int j = 0; j < NS; ++j) any |= act[j];
  if (any && !(U < kPoissonUFast)) {
    // deep upper tail (one draw in 1e5): the scalar summation with its tail exit, out of line
#pragma unroll
    for (int j = 0; j < NS; ++j) {
      if (act[j]) {
        const float2 r = poisson_sum_tail(lam[j], U, lim[j], cap);
        X[j] = r.x;
        caphits += (unsigned int)r.y;
      }
    }
    any = false;
  }
  if (any) {
    // poisson_sum for every scenario that needs one, in one loop.  A
    // scenario's p and F are dead once it has finished, so the terms are
    // computed without branches.
    float p[NS], F[NS];
#pragma unroll
    for (int j = 0; j < NS; ++j) {
      p[j] = __expf(-lam[j]);
      F[j] = p[j];
    }
    float nf = 0.0f;
    unsigned int n = 0;
    for (;;) {
      any = false;
#pragma unroll
      for (int j = 0; j < NS; ++j) {
        const bool stop = !(U > F[j]) || nf >= lim[j];
        X[j] = act[j] && stop ? nf : X[j];
        act[j] = act[j] && !stop;
        any |= act[j];
      }
      if (!any) break;
      if (++n > cap) {
#pragma unroll
        for (int j = 0; j < NS; ++j) {
          if (act[j]) {
            ++caphits;
            X[j] = (float)n;
          }
        }
        break;
      }
      nf = (float)n;
      const float r = rcp_approx(nf);
      if constexpr (NS == 3) {  // means 1 and 2 on packed FP32 pairs
        p[0] *= lam[0] * r;
        F[0] += p[0];
        const float2 pp = pk::fmul2(make_float2(p[1], p[2]), pk::fmul2(make_float2(lam[1], lam[2]), make_float2(r, r)));
        const float2 ff = pk::fadd2(make_float2(F[1], F[2]), pp);
        p[1] = pp.x;
        p[2] = pp.y;
        F[1] = ff.x;
        F[2] = ff.y;
      } else {
#pragma unroll
        for (int j = 0; j < NS; ++j) {
          p[j] *= lam[j] * r;
          F[j] += p[j];
        }
      }
    }
  }
#pragma unroll
  for (int j = 0; j < NS; ++j) N[j] = (int)X[j];
}

// One out-of-line copy for the kernels that invert one mean per draw.
static __device__ __noinline__ int poisson_core(float lam, float U, float W,
                                                unsigned long long x, unsigned int cap,
                                                unsigned int &caphits) {
  return poisson_eval(lam, U, W, x, cap, caphits);
}

__device__ __forceinline__ int poisson_inv(float lam, unsigned long long x, unsigned int cap,
                                           unsigned int &caphits) {
  const float W = lam > kPoissonAsymMin ? inv_normal_bits(x) : 0.0f;
  return poisson_core(lam, u01_bits(x), W, x, cap, caphits);
}

// Poisson draw by sequential inversion, as boost::random::poisson_distribution
// does for means below 10: one uniform_01 draw, subtract pmf terms.  In FP32 the
// subtractions leave u a few 1e-8 above the true remainder, so for u within
// about 1e-7 of 1 the remainder can stay above every later term and the loop
// would only end at the cap.  Past the mode, once a term is below 1e-9 the
// remaining mass is too (below the FP32 resolution of u), so the draw is in
// the last 1e-8 of the distribution and k is returned; a draw that stops by
// the ordinary test never gets there (its last term is at least about 1e-8).
__device__ __forceinline__ int poisson_small_u(float mean, float exp_neg_mean, float u, unsigned int cap,
                                               unsigned int &caphits) {
  float p = exp_neg_mean;
  int k = 0;
  while (u > p) {
    if ((unsigned int)k >= cap) {
      ++caphits;
      break;
    }
    if (p < 1.0e-9f && (float)k > mean) break;
    u -= p;
    ++k;
    p = __fdividef(mean * p, (float)k);
  }
  return k;
}

__device__ __forceinline__ int poisson_small(float mean, float exp_neg_mean, Xo &rng,
                                             unsigned int cap, unsigned int &caphits) {
  return poisson_small_u(mean, exp_neg_mean, u01_bits(draw(rng)), cap, caphits);
}

// poisson_small_u in FP64 on the draw's FP64 uniform x 2^-64 (the reference's
// uniform_01<double> and sequential inversion, JumpPolicies.hpp:55-75): for a
// count whose probabilities must keep differences far below FP32 resolution.
// Out of line: it runs once per path, and inline its FP64 registers would raise the
// path kernel's register count.  Returns (count, 1 if the loop cap was hit).
static __device__ __noinline__ int2 poisson_small_fp64(double mean, unsigned long long x, unsigned int cap) {
  double u = (double)x * 5.421010862427522e-20;  // 2^-64
  double p = exp(-mean);
  int k = 0, hit = 0;
  while (u > p) {
    if ((unsigned int)k >= cap) {
      hit = 1;
      break;
    }
    if (p < 1.0e-18 && (double)k > mean) break;
    u -= p;
    ++k;
    p = mean * p / (double)k;
  }
  return make_int2(k, hit);
}

// Exponential(rate) draw: -log(1 - U) / rate from one uniform.
__device__ __forceinline__ float exp_draw(Xo &rng, float inv_rate) {
  return -__logf(u01c_bits(draw(rng))) * inv_rate;
}

// Gamma(alpha_base + N, 1) draw of SchemeExact::generate_gamma
// (VolSchemes.hpp:128-203): Marsaglia-Tsang for alpha > 1, the reference's
// exponential-rejection sampler for alpha <= 1.  Loops are capped.
static __device__ __noinline__ float gamma_draw(float alpha_base, int N, Xo &rng, float sm_p,
                                         float sm_inv_p, float sm_1mp, float sm_1ma,
                                         float sm_inv_a, unsigned int cap,
                                         unsigned int &caphits) {
  const float alpha = alpha_base + (float)N;
  if (alpha > 1.0f) {
    const float d = alpha - (1.0f / 3.0f);
    const float c = rsqrtf(9.0f * d);
    for (unsigned int it = 0; it < cap; ++it) {
      float Z, v;
      unsigned int jt = 0;
      do {
        Z = inv_normal_bits(draw(rng));
        v = 1.0f + c * Z;
      } while (v <= 0.0f && ++jt < cap);
      const float cz = c * Z;
      const float w = cz * (3.0f + cz * (3.0f + cz));  // (1 + cZ)^3 - 1
      v = 1.0f + w;
      const float U = u01_bits(draw(rng));
      const float Z2 = Z * Z;
      if (U < 1.0f - 0.0331f * Z2 * Z2) return d * v;
      if (__logf(U) < 0.5f * Z2 + d * log1p_m(w)) return d * v;
    }
    ++caphits;
    return d;
  }
  for (unsigned int it = 0; it < cap; ++it) {
    const float u = u01_bits(draw(rng));
    const float y = -__logf(u01c_bits(draw(rng)));
    if (u < sm_p) {
      const float xg = __expf(-y * sm_inv_a);
      if (u * sm_inv_p < 1.0f - xg) return xg;
      if (u < sm_p * __expf(-xg)) return xg;
    } else {
      const float xg = 1.0f + y;
      const float inv_h = 1.0f / (1.0f + sm_1ma * y);
      if (u < sm_p + sm_1mp * inv_h) return xg;
      if (u < sm_p + sm_1mp * __powf(xg, -sm_1ma)) return xg;
    }
  }
  ++caphits;
  return alpha;
}

}  // namespace dev
}  // namespace myql
