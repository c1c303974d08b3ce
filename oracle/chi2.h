/*
 * oracle/chi2.h -- FP64 chi-squared quantile of the CPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY: used by the oracle's restatement of the MyQuantLib
 * Monte Carlo path (oracle/mc_oracle.c) and by the Boost-API shim that lets the
 * reference headers compile (oracle/compat/boost/math/distributions/chi_squared.hpp).
 * The reference calls boost::math::quantile(chi_squared_distribution(dof), p)
 * (include/myql/models/asvj/policies/VolSchemes.hpp:269,282,368-369); Boost is
 * not installed here, so this is an independent implementation of the same
 * function, checked against scipy.stats.chi2.ppf in the tests.
 *
 * Method: regularized incomplete gamma P(a,x) by its power series for x < a+1
 * and Q(a,x) by Legendre's continued fraction (modified Lentz) otherwise;
 * quantile by a bracketed Newton iteration on log P (or log Q for the upper
 * tail) in u = log x, started from the Wilson-Hilferty cube, or from the power
 * law x^a / Gamma(a+1) when a < 1 and p is small.  chi2 = 2x, a = dof/2.
 */
#ifndef MYQL_ORACLE_CHI2_H
#define MYQL_ORACLE_CHI2_H

#include <math.h>

/* Acklam's rational inverse normal followed by one Halley step on erfc: ~1e-15. */
static inline double oracle_norm_inv(double p) {
  static const double a[6] = {-3.969683028665376e+01, 2.209460984245205e+02,
                              -2.759285104469687e+02, 1.383577518672690e+02,
                              -3.066479806614716e+01, 2.506628277459239e+00};
  static const double b[5] = {-5.447609879822406e+01, 1.615858368580409e+02,
                              -1.556989798598866e+02, 6.680131188771972e+01,
                              -1.328068155288572e+01};
  static const double c[6] = {-7.784894002430293e-03, -3.223964580411365e-01,
                              -2.400758277161838e+00, -2.549732539343734e+00,
                              4.374664141464968e+00, 2.938163982698783e+00};
  static const double d[4] = {7.784695709041462e-03, 3.224671290700398e-01,
                              2.445134137142996e+00, 3.754408661907416e+00};
  double x;
  if (p <= 0.0) return -40.0;
  if (p >= 1.0) return 40.0;
  if (p > 0.02425 && p < 0.97575) {
    const double q = p - 0.5, r = q * q;
    x = (((((a[0] * r + a[1]) * r + a[2]) * r + a[3]) * r + a[4]) * r + a[5]) * q /
        (((((b[0] * r + b[1]) * r + b[2]) * r + b[3]) * r + b[4]) * r + 1.0);
  } else {
    const double q = p < 0.5 ? p : 1.0 - p;
    const double r = sqrt(-2.0 * log(q));
    x = (((((c[0] * r + c[1]) * r + c[2]) * r + c[3]) * r + c[4]) * r + c[5]) /
        ((((d[0] * r + d[1]) * r + d[2]) * r + d[3]) * r + 1.0);
    if (p >= 0.5) x = -x;
  }
  {
    const double e = 0.5 * erfc(-x / sqrt(2.0)) - p;
    const double u = e * sqrt(2.0 * 3.14159265358979323846) * exp(0.5 * x * x);
    x = x - u / (1.0 + 0.5 * x * u);
  }
  return x;
}

typedef struct {
  double logP, logQ, xpdf_P, xpdf_Q;
} oracle_gamma_eval;

static inline oracle_gamma_eval oracle_gamma(double a, double x, double lga) {
  oracle_gamma_eval g;
  const double lpre = -x + a * log(x) - lga;
  if (x < a + 1.0) {
    double term = 1.0, sum = 1.0, ap = a;
    for (int n = 0; n < 5000; ++n) {
      ap += 1.0;
      term *= x / ap;
      sum += term;
      if (term < sum * 1e-17) break;
    }
    g.logP = lpre - log(a) + log(sum);
    g.logQ = log1p(-exp(g.logP));
    g.xpdf_P = a / sum;
    g.xpdf_Q = exp(lpre - g.logQ);
  } else {
    const double tiny = 1e-300;
    double bb = x + 1.0 - a, cc = 1.0 / tiny, dd = 1.0 / bb, h = dd;
    for (int i = 1; i < 5000; ++i) {
      const double an = -i * (i - a);
      bb += 2.0;
      dd = an * dd + bb;
      if (fabs(dd) < tiny) dd = tiny;
      cc = bb + an / cc;
      if (fabs(cc) < tiny) cc = tiny;
      dd = 1.0 / dd;
      const double del = dd * cc;
      h *= del;
      if (fabs(del - 1.0) < 1e-16) break;
    }
    g.logQ = lpre + log(h);
    g.logP = log1p(-exp(g.logQ));
    g.xpdf_Q = 1.0 / h;
    g.xpdf_P = exp(lpre - g.logP);
  }
  return g;
}

/* Quantile of chi-squared(nu) at lower-tail probability p (upper == 0) or
 * upper-tail probability p (upper != 0). */
static inline double oracle_chi2_quantile_tail(double nu, double p, int upper) {
  if (p <= 0.0) return upper ? 1e300 : 0.0;
  if (p >= 1.0) return upper ? 0.0 : 1e300;
  const double a = 0.5 * nu, lga = lgamma(a), lp = log(p);
  const double z = upper ? -oracle_norm_inv(p) : oracle_norm_inv(p);
  const double h = 1.0 / (9.0 * a);
  const double cwh = 1.0 - h + z * sqrt(h);
  const double u_small = (lp + lgamma(a + 1.0)) / a;
  double u;
  if (cwh > 0.0) {
    u = log(a) + 3.0 * log(cwh);
    if (!upper && a < 1.0 && u_small < u) u = u_small;
  } else {
    u = upper ? log(a + 1.0) : u_small;
  }
  /* bracket kept with flags (not infinities), so the iteration is also exact
     when compiled with -ffast-math */
  double lo = 0.0, hi = 0.0;
  int have_lo = 0, have_hi = 0;
  for (int it = 0; it < 300; ++it) {
    const double x = exp(u);
    if (!(x > 0.0)) return 0.0;
    const oracle_gamma_eval g = oracle_gamma(a, x, lga);
    double G, dG;
    if (!upper) {
      G = g.logP - lp;
      dG = g.xpdf_P;
    } else {
      G = lp - g.logQ;
      dG = g.xpdf_Q;
    }
    if (G < 0.0) {
      lo = u;
      have_lo = 1;
    } else {
      hi = u;
      have_hi = 1;
    }
    double un = u - G / dG;
    const int inside = (!have_lo || un > lo) && (!have_hi || un < hi) && un == un;
    if (!inside) {
      if (!have_lo) un = u - 2.0;
      else if (!have_hi) un = u + 2.0;
      else un = 0.5 * (lo + hi);
    }
    if (fabs(un - u) < 1e-14 * fmax(1.0, fabs(u))) {
      u = un;
      break;
    }
    u = un;
  }
  return 2.0 * exp(u);
}

/* boost::math::quantile(chi_squared_distribution<double>(nu), p) */
static inline double oracle_chi2_quantile(double nu, double p) {
  return p <= 0.5 ? oracle_chi2_quantile_tail(nu, p, 0) : oracle_chi2_quantile_tail(nu, 1.0 - p, 1);
}

#endif
