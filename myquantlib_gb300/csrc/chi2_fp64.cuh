// chi2_fp64.cuh -- FP64 chi-squared quantiles on the device.
//
// Used once per degrees-of-freedom offset d to build the SchemeNCI tables
// (the reference builds them with boost::math::quantile, VolSchemes.hpp:266-311).
// Method: regularized incomplete gamma by its power series (x < a + 1) or by
// the Legendre continued fraction evaluated with the modified Lentz algorithm
// (x >= a + 1); the quantile is a safeguarded Newton iteration on
// log P(a, x) (lower tail) or log Q(a, x) (upper tail) in u = log x, started
// from the Wilson-Hilferty cube or, for small P and shape below 1, from the
// leading power term x^a / Gamma(a + 1) -- or, along a table row, from the
// Taylor step of the quantile function from the previous node.
// chi2_nu^-1(p) = 2 * x with a = nu / 2.
#pragma once
#include <cuda_runtime.h>

namespace myql {
namespace dev {

// 1 / v in FP64 for the inner loops below: the hardware's approximate
// reciprocal as the seed, then two Newton-Raphson steps r <- r + r (1 - v r),
// each of which squares the relative error (a few ulp at the end, far inside
// the series' 1e-17 stopping rule).  An IEEE division costs several times
// more, and the series and continued fraction take one or two per term.
__device__ __forceinline__ double rcp_nr(double v) {
  double r;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(v));
  r = fma(r, fma(-v, r, 1.0), r);
  return fma(r, fma(-v, r, 1.0), r);
}

struct GammaEval {
  double logP, logQ;  // log of the regularized lower / upper incomplete gamma
  double xpdf_P;      // x * pdf(x) / P
  double xpdf_Q;      // x * pdf(x) / Q
};

__device__ inline GammaEval gamma_eval(double a, double x, double lga) {
  GammaEval g;
  const double lpre = -x + a * log(x) - lga;  // log(x^a e^-x / Gamma(a))
  if (x < a + 1.0) {
    // P = x^a e^-x / Gamma(a+1) * sum_{n>=0} x^n / ((a+1)...(a+n))
    double term = 1.0, sum = 1.0, ap = a;
    for (int n = 0; n < 2000; ++n) {
      ap += 1.0;
      term *= x * rcp_nr(ap);
      sum += term;
      if (term < sum * 1e-17) break;
    }
    g.logP = lpre - log(a) + log(sum);
    const double P = exp(g.logP);
    g.logQ = log1p(-P);
    g.xpdf_P = a / sum;
    g.xpdf_Q = exp(lpre - g.logQ);
  } else {
    // Q = x^a e^-x / Gamma(a) * h, h the continued fraction
    const double tiny = 1e-300;
    double b = x + 1.0 - a, c = 1.0 / tiny, d = 1.0 / b, h = d;
    for (int i = 1; i < 2000; ++i) {
      const double an = -i * (i - a);
      b += 2.0;
      d = an * d + b;
      if (fabs(d) < tiny) d = tiny;
      c = b + an * rcp_nr(c);
      if (fabs(c) < tiny) c = tiny;
      d = rcp_nr(d);
      const double del = d * c;
      h *= del;
      if (fabs(del - 1.0) < 1e-16) break;
    }
    g.logQ = lpre + log(h);
    const double Q = exp(g.logQ);
    g.logP = log1p(-Q);
    g.xpdf_Q = 1.0 / h;
    g.xpdf_P = exp(lpre - g.logP);
  }
  return g;
}

// Starting point u = log x (x = y / 2, the gamma variable of shape a) of the
// Newton iteration for the quantile at tail probability p (lp = log p).
__device__ inline double chi2_start(double a, double p, double lp, bool upper) {
  const double z = upper ? -normcdfinv(p) : normcdfinv(p);
  const double h = 1.0 / (9.0 * a);
  const double cwh = 1.0 - h + z * sqrt(h);
  const double u_small = (lp + lgamma(a + 1.0)) / a;  // log of (p Gamma(a+1))^(1/a)
  if (cwh > 0.0) {
    const double u = log(a) + 3.0 * log(cwh);
    return (!upper && a < 1.0 && u_small < u) ? u_small : u;
  }
  return upper ? log(a + 1.0) : u_small;
}

// Safeguarded Newton iteration on G(u) = log P(a, e^u) - lp (lower tail) or
// lp - log Q(a, e^u) (upper tail), both increasing in u, from u.  A step
// shorter than max(accept, 1e-14 max(1, |u|)) is taken and ends the iteration
// before the bracket test (a step that rounds to zero must not be mistaken for
// one that leaves the bracket).  The error left after a Newton step s is about
// |G''/(2 G')| s^2, and |G''/G'| stays below about sqrt(a) + 1 over the tables'
// range, so accept = 1e-8 leaves about 1e-15 relative in x.
__device__ inline double chi2_newton(double a, double lga, double lp, bool upper, double u,
                                     double accept) {
  double lo = -INFINITY, hi = INFINITY;
  for (int it = 0; it < 200; ++it) {
    const double x = exp(u);
    if (x <= 0.0) return -700.0;
    const GammaEval g = gamma_eval(a, x, lga);
    const double G = upper ? lp - g.logQ : g.logP - lp;
    const double step = G / (upper ? g.xpdf_Q : g.xpdf_P);
    if (fabs(step) < fmax(accept, 1e-14 * fmax(1.0, fabs(u)))) return u - step;
    if (G < 0.0) lo = u; else hi = u;
    double un = u - step;
    if (!(un > lo && un < hi)) {
      if (isinf(lo)) un = u - 2.0;
      else if (isinf(hi)) un = u + 2.0;
      else un = 0.5 * (lo + hi);
    }
    u = un;
  }
  return u;
}

// Quantile of chi-squared with nu degrees of freedom at lower-tail probability p
// (upper = false) or upper-tail probability p (upper = true).
__device__ inline double chi2_quantile(double nu, double p, bool upper) {
  if (p <= 0.0) return upper ? INFINITY : 0.0;
  if (p >= 1.0) return upper ? 0.0 : INFINITY;
  const double a = 0.5 * nu;
  const double lp = log(p);
  return 2.0 * exp(chi2_newton(a, lgamma(a), lp, upper, chi2_start(a, p, lp, upper), 0.0));
}

// chi-squared density (for the exact tail slopes)
__device__ inline double chi2_logpdf(double nu, double y) {
  const double a = 0.5 * nu, x = 0.5 * y;
  return (a - 1.0) * log(x) - x - lgamma(a) - log(2.0);
}

}  // namespace dev
}  // namespace myql
