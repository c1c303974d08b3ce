/*
 * oracle/mc_oracle.c -- CPU oracle of the MyQuantLib Monte Carlo path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py may load this library, and only to check or
 * time against it; the GPU engine never calls it.
 *
 * A plain-C FP64 restatement of the reference's path-simulation algorithm:
 *   MonteCarloPricer::calculate        pricers/montecarlo/MonteCarloPricer.hpp:95-481
 *   ASVJStepper ctor / multi_step      models/asvj/core/ASVJstepper.hpp:85-229,262-283
 *   SchemeNV / SchemeExact / SchemeNCI models/asvj/policies/VolSchemes.hpp:24-377
 *   MertonJump / KouJump               models/asvj/policies/JumpPolicies.hpp:32-136
 *   trackers                           instruments/trackers/PathTrackers.hpp:8-301
 *   payoffs, instruments               instruments/Payoffs.hpp, options/*.hpp
 *   normcdfinv_as241, poissinvcdf      math/Numerics.hpp:12-272
 * with the Boost samplers it uses restated as: xoshiro256++ seeded by
 * splitmix64 (boost::random::xoshiro256pp), uniform = x * 2^-64 with draws
 * that round to 1.0 rejected (uniform_real_distribution / uniform_01),
 * Poisson by sequential inversion (poisson_distribution for means < 10; also
 * used above 10 here), exponential by -log(1 - U) / rate, chi-squared quantile
 * by oracle/chi2.h.
 *
 * Two random-number layouts:
 *   MYQL_ORACLE_LAYOUT_REFERENCE: n_threads streams seeded with
 *     seed + t * 999983 (MonteCarloPricer.hpp:191), each running the
 *     contiguous block of paths OpenMP's static schedule gives thread t;
 *   MYQL_ORACLE_LAYOUT_STREAMS: the GPU engine's layout -- S streams, stream k
 *     = splitmix64(seed) advanced by k jump()s (2^128 steps each), stream k
 *     running paths k, k + S, k + 2S, ...  Per-path records can be returned
 *     for path-by-path comparison with the GPU.
 * Full Greeks on strips are evaluated per strike (the reference's strip Full
 * mode writes into empty vectors, MonteCarloPricer.hpp:233-240, 325-400).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "chi2.h"
#include "myql_gpu.h"

#define MYQL_ORACLE_LAYOUT_REFERENCE 0
#define MYQL_ORACLE_LAYOUT_STREAMS 1
#define NQ 10
#define MAXSC 9

/* ------------------------------------------------------------------ RNG */
typedef struct {
  uint64_t s[4];
} xo_t;

static inline uint64_t rotl64(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

static inline uint64_t xo_next(xo_t *r) {
  uint64_t *s = r->s;
  const uint64_t out = rotl64(s[0] + s[3], 23) + s[0];
  const uint64_t t = s[1] << 17;
  s[2] ^= s[0];
  s[3] ^= s[1];
  s[1] ^= s[2];
  s[0] ^= s[3];
  s[2] ^= t;
  s[3] = rotl64(s[3], 45);
  return out;
}

static void xo_seed(xo_t *r, uint64_t seed) {
  uint64_t x = seed;
  for (int i = 0; i < 4; ++i) {
    uint64_t z = (x += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    r->s[i] = z ^ (z >> 31);
  }
}

static void xo_jump(xo_t *r) {
  static const uint64_t J[4] = {0x180ec6d33cfd0abaull, 0xd5a61266f0c9392cull,
                                0xa9582618e03fc9aaull, 0x39abdc4529b1661cull};
  uint64_t a[4] = {0, 0, 0, 0};
  for (int w = 0; w < 4; ++w)
    for (int b = 0; b < 64; ++b) {
      if (J[w] & (1ull << b))
        for (int j = 0; j < 4; ++j) a[j] ^= r->s[j];
      (void)xo_next(r);
    }
  memcpy(r->s, a, sizeof a);
}

/* uniform_real_distribution<double>(0,1) and uniform_01<double> */
static inline double uni(xo_t *r) {
  for (;;) {
    const double u = (double)xo_next(r) * 5.421010862427522170037264e-20; /* 2^-64 */
    if (u < 1.0) return u;
  }
}

/* ------------------------------------------------------------------ numerics */
static double normcdfinv_as241(double p) { /* Numerics.hpp:12-47 */
  static const double a[] = {-3.969683028665376e+01, 2.209460984245205e+02,
                             -2.759285104469687e+02, 1.383577518672690e+02,
                             -3.066479806614716e+01, 2.506628277459239e+00};
  static const double b[] = {-5.447609879822406e+01, 1.615858368580409e+02,
                             -1.556989798598866e+02, 6.680131188771972e+01,
                             -1.328068155288572e+01};
  static const double c[] = {-7.784894002430293e-03, -3.223964580411365e-01,
                             -2.400758277161838e+00, -2.549732539343734e+00,
                             4.374664141464968e+00, 2.938163982698783e+00};
  static const double d[] = {7.784695709041462e-03, 3.224671290700398e-01,
                             2.445134137142996e+00, 3.754408661907416e+00};
  const double p_low = 0.02425, p_high = 1.0 - p_low;
  if (p > p_low && p < p_high) {
    const double q = p - 0.5, r = q * q;
    return (((((a[0] * r + a[1]) * r + a[2]) * r + a[3]) * r + a[4]) * r + a[5]) * q /
           (((((b[0] * r + b[1]) * r + b[2]) * r + b[3]) * r + b[4]) * r + 1.0);
  }
  const double q = (p <= p_low) ? p : 1.0 - p;
  const double r = sqrt(-2.0 * log(q));
  const double x = (((((c[0] * r + c[1]) * r + c[2]) * r + c[3]) * r + c[4]) * r + c[5]) /
                   ((((d[0] * r + d[1]) * r + d[2]) * r + d[3]) * r + 1.0);
  return (p <= p_low) ? x : -x;
}

/* Giles' inverse Poisson CDF (ACM TOMS 955), as in Numerics.hpp:49-272. */
static double poissinvcdf(double lambda, double U) {
  double V = 1.0 - U, X = 0.0, Xi, W, T, Del = 0.0, R, R2, S, S2, Eta, B0, B1;
  const double lambdai = 1.0 / lambda;
  if (U <= 0.0) return 0.0;
  if (U >= 1.0) return NAN;
  if (lambda > 4.0) {
    W = normcdfinv_as241(fmin(U, V));
    if (U > V) W = -W;
    if (fabs(W) < 3.0) {
      const double lr = sqrt(lambda);
      S = lr * W + ((1.0 / 3.0) + (1.0 / 6.0) * W * W) * (1.0 - W / (12.0 * lr));
      Del = (1.0 / 160.0);
      Del = (1.0 / 80.0) + Del * (W * W);
      Del = (1.0 / 40.0) + Del * (W * W);
      Del = Del * lambdai;
      S = lambda + (S + Del);
    } else {
      S = W / sqrt(lambda);
      R = 1.0 + S;
      if (R < 0.1) R = 0.1;
      do {
        T = log(R);
        R2 = R;
        S2 = sqrt(2.0 * ((1.0 - R) + R * T));
        if (R < 1.0) S2 = -S2;
        R = R2 - (S2 - S) * S2 / T;
        if (R < 0.1 * R2) R = 0.1 * R2;
      } while (fabs(R - R2) > 1e-8);
      T = log(R);
      S = lambda * R + log(sqrt(2.0 * R * ((1.0 - R) + R * T)) / fabs(R - 1.0)) / T;
      S = S - 0.0218 / (S + 0.065 * lambda);
      Del = 0.01 / S;
      S = S + Del;
    }
    X = floor(S);
    if (S > 10.0 && S < X + 2.0 * Del) {
      if (X > 0.5 * lambda && X < 2.0 * lambda) {
        Xi = 1.0 / X;
        Eta = X * lambdai;
        Eta = sqrt(2.0 * (1.0 - Eta + Eta * log(Eta)) / Eta);
        if (X > lambda) Eta = -Eta;
        /* Temme expansion (coefficients of the published algorithm) */
        B1 = 8.0995211567045583e-16;
        S = B1;
        B0 = -1.9752288294349411e-15;
        S = B0 + S * Eta;
        B1 = -5.1391118342426808e-16 + 25.0 * B1 * Xi;
        S = B1 + S * Eta;
        B0 = 2.8534893807047458e-14 + 24.0 * B0 * Xi;
        S = B0 + S * Eta;
        B1 = -1.3923887224181616e-13 + 23.0 * B1 * Xi;
        S = B1 + S * Eta;
        B0 = 3.3717632624009806e-13 + 22.0 * B0 * Xi;
        S = B0 + S * Eta;
        B1 = 1.1004392031956284e-13 + 21.0 * B1 * Xi;
        S = B1 + S * Eta;
        B0 = -5.0276692801141763e-12 + 20.0 * B0 * Xi;
        S = B0 + S * Eta;
        B1 = 2.4361948020667402e-11 + 19.0 * B1 * Xi;
        S = B1 + S * Eta;
        B0 = -5.8307721325504166e-11 + 18.0 * B0 * Xi;
        S = B0 + S * Eta;
        B1 = -2.5514193994946487e-11 + 17.0 * B1 * Xi;
        S = B1 + S * Eta;
        B0 = 9.1476995822367933e-10 + 16.0 * B0 * Xi;
        S = B0 + S * Eta;
        B1 = -4.3820360184533521e-09 + 15.0 * B1 * Xi;
        S = B1 + S * Eta;
        B0 = 1.0261809784240299e-08 + 14.0 * B0 * Xi;
        S = B0 + S * Eta;
        B1 = 6.7078535434015332e-09 + 13.0 * B1 * Xi;
        S = B1 + S * Eta;
        B0 = -1.7665952736826086e-07 + 12.0 * B0 * Xi;
        S = B0 + S * Eta;
        B1 = 8.2967113409530833e-07 + 11.0 * B1 * Xi;
        S = B1 + S * Eta;
        B0 = -1.8540622107151585e-06 + 10.0 * B0 * Xi;
        S = B0 + S * Eta;
        B1 = -2.1854485106799979e-06 + 9.0 * B1 * Xi;
        S = B1 + S * Eta;
        B0 = 3.9192631785224383e-05 + 8.0 * B0 * Xi;
        S = B0 + S * Eta;
        B1 = -0.00017875514403292177 + 7.0 * B1 * Xi;
        S = B1 + S * Eta;
        B0 = 0.00035273368606701921 + 6.0 * B0 * Xi;
        S = B0 + S * Eta;
        B1 = 0.0011574074074074078 + 5.0 * B1 * Xi;
        S = B1 + S * Eta;
        B0 = -0.014814814814814815 + 4.0 * B0 * Xi;
        S = B0 + S * Eta;
        B1 = 0.083333333333333329 + 3.0 * B1 * Xi;
        S = B1 + S * Eta;
        B0 = -0.33333333333333331 + 2.0 * B0 * Xi;
        S = B0 + S * Eta;
        S = S / (1.0 + B1 * Xi);
        S = S * exp(-0.5 * X * Eta * Eta) / sqrt(2.0 * 3.141592653589793 * X);
        if (X < lambda) {
          S += 0.5 * erfc(Eta * sqrt(0.5 * X));
          if (S > U) X -= 1.0;
        } else {
          S -= 0.5 * erfc(-Eta * sqrt(0.5 * X));
          if (S > -V) X -= 1.0;
        }
      } else {
        Xi = 1.0 / X;
        S = -(691.0 / 360360.0);
        S = (1.0 / 1188.0) + S * Xi * Xi;
        S = -(1.0 / 1680.0) + S * Xi * Xi;
        S = (1.0 / 1260.0) + S * Xi * Xi;
        S = -(1.0 / 360.0) + S * Xi * Xi;
        S = (1.0 / 12.0) + S * Xi * Xi;
        S = S * Xi;
        S = (X - lambda) - X * log(X * lambdai) - S;
        if (X < lambda) {
          T = exp(-0.5 * S);
          S = 1.0 - T * (U * T) * sqrt(2.0 * 3.141592653589793 * Xi) * lambda;
          T = 1.0;
          Xi = X;
          for (int i = 1; i < 50; i++) {
            Xi -= 1.0;
            T *= Xi * lambdai;
            S += T;
          }
          if (S > 0.0) X -= 1.0;
        } else {
          T = exp(-0.5 * S);
          S = 1.0 - T * (V * T) * sqrt(2.0 * 3.141592653589793 * X);
          Xi = X;
          for (int i = 0; i < 50; i++) {
            Xi += 1.0;
            S = S * Xi * lambdai + 1.0;
          }
          if (S < 0.0) X -= 1.0;
        }
      }
    }
  }
  if (X < 10.0) {
    X = 0.0;
    T = exp(0.5 * lambda);
    Del = 0.0;
    if (U > 0.5) Del = T * (1e-13 * T);
    S = 1.0 - T * (U * T) + Del;
    while (S < 0.0) {
      X += 1.0;
      T = X * lambdai;
      Del = T * Del;
      S = T * S + 1.0;
    }
    if (S < 2.0 * Del) {
      Del = 1e13 * Del;
      T = 1e17 * Del;
      Del = V * Del;
      while (Del < T) {
        X += 1.0;
        Del *= X * lambdai;
      }
      S = Del;
      T = 1.0;
      while (S > 0.0) {
        T *= X * lambdai;
        S -= T;
        X -= 1.0;
      }
    }
  }
  return X;
}

/* poisson_distribution<int,double>(mean): sequential inversion */
static int pois_draw(double mean, double exp_neg_mean, xo_t *r) {
  double p = exp_neg_mean;
  int x = 0;
  double u = uni(r);
  while (u > p) {
    u = u - p;
    ++x;
    p = mean * p / x;
  }
  return x;
}

/* exponential_distribution<double>(rate) */
static inline double exp_draw(double rate, xo_t *r) { return -log(1.0 - uni(r)) / rate; }

/* ------------------------------------------------------------------ schemes */
typedef struct {
  int scheme;     /* myql_scheme */
  double C[4];    /* log-S coefficients */
  double W[3];    /* scheme workspace */
  double v0;
  /* exact scheme global workspace */
  double ex_d[128], ex_c[128];
  int alpha_small;
  double sm_p, sm_inv_p, sm_1mp, sm_1ma, sm_inv_a;
  /* NCI global workspace */
  const double *y, *m;
  int n_max, grid;
  double dx, inv_dx;
} factor_t;

typedef struct {
  double *y, *m;
  int n_max, grid;
  double dx, inv_dx;
} nci_ws;

static void nci_build(nci_ws *g, const myql_heston_params *p, double dt) {
  const double d = (4.0 * p->kappa * p->theta) / (p->sigma * p->sigma);
  const double v_max = fmax(p->v0, 3.0 * p->theta);
  const double ex = exp(-p->kappa * dt);
  const double psi = (fabs(p->kappa) < 1e-10) ? dt : (1.0 - ex) / p->kappa;
  const double lambda_max = (2.0 * v_max * ex) / (p->sigma * p->sigma * psi);
  double nm = ceil(lambda_max + 4.0 * sqrt(lambda_max));
  if (nm < 23) nm = 23;
  if (nm > 1023) nm = 1023;
  g->n_max = (int)nm;
  g->grid = 10000;
  g->dx = 0.999 / (g->grid - 1);
  g->inv_dx = 1.0 / g->dx;
  const size_t total = (size_t)(g->n_max + 1) * g->grid;
  g->y = (double *)calloc(total, sizeof(double));
  g->m = (double *)calloc(total, sizeof(double));
#pragma omp parallel for schedule(dynamic)
  for (int k = 0; k <= g->n_max; ++k) {
    const double dof = d + 2.0 * (double)k;
    const size_t off = (size_t)k * g->grid;
    for (int i = 0; i < g->grid; ++i) g->y[off + i] = oracle_chi2_quantile(dof, i * g->dx);
    for (int i = 0; i < g->grid; ++i) {
      if (i == 0) {
        g->m[off + i] = (g->y[off + 1] - g->y[off]) * g->inv_dx;
      } else if (i == g->grid - 1) {
        g->m[off + i] = (g->y[off + i] - g->y[off + i - 1]) * g->inv_dx;
      } else {
        const double d1 = (g->y[off + i] - g->y[off + i - 1]) * g->inv_dx;
        const double d2 = (g->y[off + i + 1] - g->y[off + i]) * g->inv_dx;
        g->m[off + i] = (d1 * d2 > 0.0) ? 2.0 * d1 * d2 / (d1 + d2) : 0.0;
      }
    }
  }
}

static void factor_prepare(factor_t *f, const myql_heston_params *p, int scheme, double r_part,
                           double h, const nci_ws *nci) {
  memset(f, 0, sizeof *f);
  f->scheme = scheme;
  f->v0 = p->v0;
  const double kappa = p->kappa, theta = p->theta, sigma = p->sigma, rho = p->rho;
  f->C[0] = (r_part - rho * kappa * theta / sigma) * h;
  const double term = (kappa * rho / sigma - 0.5) * h * 0.5;
  f->C[1] = term - (rho / sigma);
  f->C[2] = term + (rho / sigma);
  f->C[3] = h * (1.0 - rho * rho) * 0.5;
  if (scheme == MYQL_SCHEME_NV) {
    const double ex = exp(-p->kappa * h * 0.5);
    const double psi = (fabs(p->kappa) < 1e-10) ? h * 0.5 : (1.0 - ex) / p->kappa;
    const double D = (p->kappa * p->theta) - (p->sigma * p->sigma * 0.25);
    f->W[0] = ex;
    f->W[1] = D * psi;
    f->W[2] = p->sigma * sqrt(h) * 0.5;
  } else {
    const double ex = exp(-p->kappa * h);
    const double psi = (fabs(p->kappa) < 1e-10) ? h : (1.0 - ex) / p->kappa;
    f->W[0] = (2.0 / (p->sigma * p->sigma * psi)) * ex;
    if (scheme == MYQL_SCHEME_EXACT) {
      f->W[1] = (2.0 * p->kappa * p->theta) / (p->sigma * p->sigma);
      f->W[2] = 0.5 * (p->sigma * p->sigma * psi);
      const double ab = f->W[1];
      for (int k = 0; k < 128; ++k) {
        const double alpha = ab + k;
        if (alpha > 1.0) {
          f->ex_d[k] = alpha - (1.0 / 3.0);
          f->ex_c[k] = 1.0 / sqrt(9.0 * f->ex_d[k]);
        }
      }
      f->alpha_small = ab <= 1.0;
      if (f->alpha_small) {
        const double e = 2.71828182845904523536;
        f->sm_p = e / (ab + e);
        f->sm_inv_p = 1.0 / f->sm_p;
        f->sm_1mp = 1.0 - f->sm_p;
        f->sm_1ma = 1.0 - ab;
        f->sm_inv_a = 1.0 / ab;
      }
    } else {
      f->W[1] = (4.0 * p->kappa * p->theta) / (p->sigma * p->sigma);
      f->W[2] = 0.25 * p->sigma * p->sigma * psi;
      f->y = nci->y;
      f->m = nci->m;
      f->n_max = nci->n_max;
      f->grid = nci->grid;
      f->dx = nci->dx;
      f->inv_dx = nci->inv_dx;
    }
  }
}

static double gamma_draw(const factor_t *f, double alpha_base, int N, xo_t *r) {
  const double alpha = alpha_base + N;
  if (alpha > 1.0) {
    double d, c, U, Z, v;
    if (N < 128) {
      d = f->ex_d[N];
      c = f->ex_c[N];
    } else {
      d = alpha - (1.0 / 3.0);
      c = 1.0 / sqrt(9.0 * d);
    }
    for (;;) {
      do {
        Z = normcdfinv_as241(uni(r));
        v = 1.0 + c * Z;
      } while (v <= 0.0);
      v = v * v * v;
      U = uni(r);
      if (U < 1.0 - 0.0331 * Z * Z * Z * Z) return d * v;
      if (log(U) < 0.5 * Z * Z + d * (1.0 - v + log(v))) return d * v;
    }
  }
  for (;;) {
    const double u = uni(r);
    const double y = exp_draw(1.0, r);
    if (u < f->sm_p) {
      const double x = exp(-y * f->sm_inv_a);
      if (u * f->sm_inv_p < 1.0 - x) return x;
      if (u < f->sm_p * exp(-x)) return x;
    } else {
      const double x = 1.0 + y;
      const double inv_h = 1.0 / (1.0 + f->sm_1ma * y);
      if (u < f->sm_p + f->sm_1mp * inv_h) return x;
      if (u < f->sm_p + f->sm_1mp * pow(x, -f->sm_1ma)) return x;
    }
  }
}

static double evolve(const factor_t *f, double v, xo_t *r) {
  if (f->scheme == MYQL_SCHEME_NV) {
    const double Z = normcdfinv_as241(uni(r));
    const double root = sqrt(f->W[0] * v + f->W[1]) + f->W[2] * Z;
    return f->W[0] * (root * root) + f->W[1];
  }
  if (f->scheme == MYQL_SCHEME_EXACT) {
    const double lambda = f->W[0] * v;
    const int N = (int)poissinvcdf(lambda, uni(r));
    return gamma_draw(f, f->W[1], N, r) * f->W[2];
  }
  {
    const double lambda = f->W[0] * v;
    const int N = (int)poissinvcdf(lambda, uni(r));
    const double U = uni(r);
    if (N <= f->n_max && U < 0.999) {
      const double pos = U * f->inv_dx;
      size_t i = (size_t)pos;
      if (i >= (size_t)f->grid - 1) i = f->grid - 2;
      const double t = pos - (double)i;
      const size_t off = (size_t)N * f->grid + i;
      const double y0 = f->y[off], y1 = f->y[off + 1], m0 = f->m[off], m1 = f->m[off + 1];
      const double t2 = t * t, t3 = t2 * t;
      return ((2 * t3 - 3 * t2 + 1) * y0 + (t3 - 2 * t2 + t) * f->dx * m0 + (-2 * t3 + 3 * t2) * y1 +
              (t3 - t2) * f->dx * m1) *
             f->W[2];
    }
    return oracle_chi2_quantile(f->W[1] + 2.0 * N, U) * f->W[2];
  }
}

/* ------------------------------------------------------------------ stepper */
typedef struct {
  int nf, jump, tracker, path_dep, n_steps;
  double dt, T_total_sim;  /* dt and n_steps*dt */
  factor_t f[2];
  double gbm_drift_dt, gbm_vol_dt;
  /* jump workspace */
  double j_mean, j_exp_neg_mean, j_comp;
  double mu, delta, p_up, eta1, eta2;
} stepper_t;

typedef struct { /* tracker configuration (options' get_tracker_config) */
  double past_avg_log, past_avg_S, t_elapsed;
  double hist_min_logS, hist_max_logS;
  double b_base, b_up, b_dn;
} tcfg_t;

typedef struct { /* Stepper::State after finalize */
  double logS;   /* terminal price after finalize */
  double sumLogS, sumS, minLogS, maxLogS;
  double current_time;
  int hit_base, hit_up, hit_dn;
  double t_base, t_up, t_dn;
} state_t;

enum { TRK_EUR = 0, TRK_GEO = 1, TRK_ARITH = 2, TRK_LB = 3, TRK_BUP = 4, TRK_BDN = 5 };

static void stepper_init(stepper_t *s, const myql_mc_job *job, double vol, const double v0[2],
                         double dt, double r, double total_time, nci_ws nci[2]) {
  const myql_model *m = &job->model;
  memset(s, 0, sizeof *s);
  s->nf = m->num_factors;
  s->jump = m->jump;
  s->dt = dt;
  s->n_steps = (int)job->config.time_steps;
  const double q = job->q;
  if (s->nf == 0) {
    const double var = vol * vol;
    s->gbm_drift_dt = (r - q - 0.5 * var) * dt;
    s->gbm_vol_dt = vol * sqrt(dt);
  } else {
    const double r_part = (r - q) / (double)s->nf;
    for (int i = 0; i < s->nf; ++i) {
      myql_heston_params hp = m->heston[i];
      hp.v0 = v0[i];
      factor_prepare(&s->f[i], &hp, job->config.scheme[i], r_part, dt, &nci[i]);
    }
  }
  const double window = s->path_dep ? dt : total_time;
  (void)window;
  s->mu = m->merton_mu;
  s->delta = m->merton_delta;
  s->p_up = m->kou_p_up;
  s->eta1 = m->kou_eta1;
  s->eta2 = m->kou_eta2;
}

static void stepper_jumps(stepper_t *s, const myql_model *m, double window) {
  if (m->jump == MYQL_JUMP_MERTON) {
    s->j_mean = m->jump_lambda * window;
    s->j_exp_neg_mean = exp(-s->j_mean);
    const double k = exp(m->merton_mu + 0.5 * m->merton_delta * m->merton_delta) - 1.0;
    s->j_comp = -m->jump_lambda * k * window;
  } else if (m->jump == MYQL_JUMP_KOU) {
    s->j_mean = m->jump_lambda * window;
    s->j_exp_neg_mean = exp(-s->j_mean);
    const double term_up = (m->kou_p_up * m->kou_eta1) / (m->kou_eta1 - 1.0);
    const double term_down = ((1.0 - m->kou_p_up) * m->kou_eta2) / (m->kou_eta2 + 1.0);
    const double k = term_up + term_down - 1.0;
    s->j_comp = -m->jump_lambda * k * window;
  }
}

static double log_jump(const stepper_t *s, xo_t *r) {
  if (s->jump == MYQL_JUMP_NONE) return 0.0;
  const int n = pois_draw(s->j_mean, s->j_exp_neg_mean, r);
  if (n == 0) return s->j_comp;
  if (s->jump == MYQL_JUMP_MERTON) {
    const double total_mu = n * s->mu;
    const double total_delta = sqrt((double)n) * s->delta;
    const double Z = normcdfinv_as241(uni(r));
    return s->j_comp + total_mu + total_delta * Z;
  }
  double total = 0.0;
  for (int i = 0; i < n; ++i) {
    const double u = uni(r);
    if (u < s->p_up)
      total += exp_draw(s->eta1, r);
    else
      total -= exp_draw(s->eta2, r);
  }
  return s->j_comp + total;
}

static void tracker_update(state_t *st, int trk, const tcfg_t *c, double dt) {
  switch (trk) {
    case TRK_GEO: st->sumLogS += st->logS * dt; break;
    case TRK_ARITH:
      st->sumLogS += st->logS * dt;
      st->sumS += exp(st->logS) * dt;
      break;
    case TRK_LB:
      st->maxLogS = (st->logS > st->maxLogS) ? st->logS : st->maxLogS;
      st->minLogS = (st->logS < st->minLogS) ? st->logS : st->minLogS;
      break;
    case TRK_BUP:
      st->current_time += dt;
      if (st->logS >= c->b_up) {
        if (!st->hit_up) { st->hit_up = 1; st->t_up = st->current_time; }
        if (st->logS >= c->b_base) {
          if (!st->hit_base) { st->hit_base = 1; st->t_base = st->current_time; }
          if (st->logS >= c->b_dn) {
            if (!st->hit_dn) { st->hit_dn = 1; st->t_dn = st->current_time; }
          }
        }
      }
      break;
    case TRK_BDN:
      st->current_time += dt;
      if (st->logS <= c->b_dn) {
        if (!st->hit_dn) { st->hit_dn = 1; st->t_dn = st->current_time; }
        if (st->logS <= c->b_base) {
          if (!st->hit_base) { st->hit_base = 1; st->t_base = st->current_time; }
          if (st->logS <= c->b_up) {
            if (!st->hit_up) { st->hit_up = 1; st->t_up = st->current_time; }
          }
        }
      }
      break;
    default: break;
  }
}

/* start_path + multi_step (ASVJstepper.hpp:120-229) */
static void run_path(const stepper_t *s, int trk, const tcfg_t *c, double S0, xo_t *r,
                     state_t *st) {
  memset(st, 0, sizeof *st);
  st->logS = log(S0);
  const double dt = s->dt;
  /* tracker init */
  switch (trk) {
    case TRK_GEO: st->sumLogS = c->past_avg_log * c->t_elapsed + 0.5 * st->logS * dt; break;
    case TRK_ARITH:
      st->sumLogS = c->past_avg_log * c->t_elapsed + 0.5 * st->logS * dt;
      st->sumS = c->past_avg_S * c->t_elapsed + 0.5 * exp(st->logS) * dt;
      break;
    case TRK_LB:
      st->minLogS = (c->hist_min_logS < 1e300) ? c->hist_min_logS : st->logS;
      st->maxLogS = (c->hist_max_logS > -1e300) ? c->hist_max_logS : st->logS;
      break;
    case TRK_BUP:
      if (st->logS >= c->b_base) st->hit_base = 1;
      if (st->logS >= c->b_up) st->hit_up = 1;
      if (st->logS >= c->b_dn) st->hit_dn = 1;
      break;
    case TRK_BDN:
      if (st->logS <= c->b_base) st->hit_base = 1;
      if (st->logS <= c->b_up) st->hit_up = 1;
      if (st->logS <= c->b_dn) st->hit_dn = 1;
      break;
    default: break;
  }
  const int n = s->n_steps;
  const double total_time = n * dt;
  double v0 = s->nf >= 1 ? s->f[0].v0 : 0.0, v1 = s->nf >= 2 ? s->f[1].v0 : 0.0;
  double lS = st->logS;
  const int pd = trk != TRK_EUR;
  if (s->nf == 0 && !pd) {
    const double G = normcdfinv_as241(uni(r));
    const double total_drift = s->gbm_drift_dt * n;
    const double total_vol = s->gbm_vol_dt * sqrt((double)n);
    lS += total_drift + total_vol * G;
    lS += log_jump(s, r);
  } else {
    for (int k = 0; k < n; ++k) {
      if (s->nf == 0) {
        const double G = normcdfinv_as241(uni(r));
        lS += s->gbm_drift_dt + s->gbm_vol_dt * G;
      } else if (s->nf == 1) {
        const double *C = s->f[0].C;
        const double G = normcdfinv_as241(uni(r));
        const double vn = evolve(&s->f[0], v0, r);
        const double root = sqrt(C[3] * (v0 + vn));
        lS += C[0] + C[1] * v0 + C[2] * vn + root * G;
        v0 = vn;
      } else {
        const double *C0 = s->f[0].C, *C1 = s->f[1].C;
        const double G = normcdfinv_as241(uni(r));
        const double v0n = evolve(&s->f[0], v0, r);
        const double v1n = evolve(&s->f[1], v1, r);
        const double root = sqrt(C0[3] * (v0 + v0n) + C1[3] * (v1 + v1n));
        lS += C0[0] + C0[1] * v0 + C0[2] * v0n + C1[0] + C1[1] * v1 + C1[2] * v1n + root * G;
        v0 = v0n;
        v1 = v1n;
      }
      if (pd) {
        lS += log_jump(s, r);
        st->logS = lS;
        tracker_update(st, trk, c, dt);
      }
    }
    if (!pd && s->nf > 0) lS += log_jump(s, r);
  }
  st->logS = lS;
  /* finalize */
  switch (trk) {
    case TRK_GEO:
      st->sumLogS -= 0.5 * st->logS * dt;
      st->sumLogS = exp(st->sumLogS / (total_time + c->t_elapsed));
      break;
    case TRK_ARITH:
      st->sumLogS -= 0.5 * st->logS * dt;
      st->sumS -= 0.5 * exp(st->logS) * dt;
      st->sumLogS = exp(st->sumLogS / (total_time + c->t_elapsed));
      st->sumS = st->sumS / (total_time + c->t_elapsed);
      break;
    case TRK_LB:
      st->minLogS = exp(st->minLogS);
      st->maxLogS = exp(st->maxLogS);
      break;
    default: break;
  }
  st->logS = exp(st->logS);
}

/* ------------------------------------------------------------------ payoffs */
typedef struct {
  int kind, payoff, call, fixed, action, timing, mode;
  double eps, rebate, rate, T;
} instr_t;

static double payoff_fn(const instr_t *in, double spot, double strike, int smooth) {
  const double diff = in->call ? (spot - strike) : (strike - spot);
  if (in->payoff == MYQL_PAYOFF_VANILLA) return diff > 0.0 ? diff : 0.0;
  double h;
  if (!smooth)
    h = diff > 0.0 ? 1.0 : 0.0;
  else
    h = 0.5 * erfc(-diff * 0.70710678118654752440 / in->eps);
  return in->payoff == MYQL_PAYOFF_CASH ? h : spot * h;
}

/* calculate_to_buffer for one strike: values at S0-bump s = 0 (base), +1, -1 */
static void payoff_triplet(const instr_t *in, const state_t *st, double S0, double h, double K,
                           double out[3]) {
  const double S_T = st->logS;
  double mult_up = 1.0, mult_dn = 1.0;
  const int greeks = in->mode != MYQL_GREEKS_NONE;
  if (greeks) {
    mult_up = (S0 + h) / S0;
    mult_dn = (S0 - h) / S0;
  }
  const int smooth = greeks;
  switch (in->kind) {
    case MYQL_INSTR_ASIAN_GEO:
    case MYQL_INSTR_ASIAN_ARITH: {
      const double avg = in->kind == MYQL_INSTR_ASIAN_GEO ? st->sumLogS : st->sumS;
      if (in->fixed) {
        out[0] = payoff_fn(in, avg, K, smooth);
        out[1] = payoff_fn(in, avg * mult_up, K, smooth);
        out[2] = payoff_fn(in, avg * mult_dn, K, smooth);
      } else {
        out[0] = payoff_fn(in, S_T, avg, smooth);
        out[1] = payoff_fn(in, S_T * mult_up, avg * mult_up, smooth);
        out[2] = payoff_fn(in, S_T * mult_dn, avg * mult_dn, smooth);
      }
      break;
    }
    case MYQL_INSTR_LOOKBACK: {
      double ext;
      if (in->fixed)
        ext = in->call ? st->maxLogS : st->minLogS;
      else
        ext = in->call ? st->minLogS : st->maxLogS;
      if (in->fixed) {
        out[0] = payoff_fn(in, ext, K, smooth);
        out[1] = payoff_fn(in, ext * mult_up, K, smooth);
        out[2] = payoff_fn(in, ext * mult_dn, K, smooth);
      } else {
        out[0] = payoff_fn(in, S_T, ext, smooth);
        out[1] = payoff_fn(in, S_T * mult_up, ext * mult_up, smooth);
        out[2] = payoff_fn(in, S_T * mult_dn, ext * mult_dn, smooth);
      }
      break;
    }
    case MYQL_INSTR_BARRIER: {
      const int hits[3] = {st->hit_base, st->hit_up, st->hit_dn};
      const double times[3] = {st->t_base, st->t_up, st->t_dn};
      const double mults[3] = {1.0, mult_up, mult_dn};
      for (int j = 0; j < 3; ++j) {
        double reb = 0.0;
        if (in->timing != MYQL_REBATE_NONE) {
          reb = in->rebate;
          if (in->timing == MYQL_REBATE_AT_HIT && hits[j]) reb = in->rebate * exp(in->rate * (in->T - times[j]));
        }
        const double pay = payoff_fn(in, S_T * mults[j], K, 0);
        if (in->action == MYQL_BARRIER_IN)
          out[j] = hits[j] ? pay : reb;
        else
          out[j] = hits[j] ? reb : pay;
      }
      break;
    }
    default:
      out[0] = payoff_fn(in, S_T, K, smooth);
      out[1] = payoff_fn(in, S_T * mult_up, K, smooth);
      out[2] = payoff_fn(in, S_T * mult_dn, K, smooth);
      break;
  }
}

/* ------------------------------------------------------------------ pricing */
typedef struct {
  stepper_t st[MAXSC];
  tcfg_t tcfg;
  instr_t in;
  int n_sc, trk, nf, mode;
  double S0, h, r, T;
  /* Greek constants */
  double inv_2dv, c_v[2], inv_2dT, inv_2dr, df_Tup, df_Tdn, df_rup, df_rdn;
} plan_t;

static double expected_avg_var(const myql_heston_params *h, double T) {
  if (fabs(h->kappa * T) > 1e-8) return h->theta + (h->v0 - h->theta) * (1.0 - exp(-h->kappa * T)) / (h->kappa * T);
  return h->v0;
}

static void plan_build(plan_t *P, const myql_mc_job *job, nci_ws nci[MAXSC][2]) {
  const myql_model *m = &job->model;
  const myql_instrument *ins = &job->instrument;
  const myql_mc_config *c = &job->config;
  memset(P, 0, sizeof *P);
  P->nf = m->num_factors;
  P->mode = c->greek_mode;
  P->S0 = job->S0;
  P->r = job->r;
  P->T = ins->maturity;
  P->h = job->S0 * c->fd_bump;
  switch (ins->kind) {
    case MYQL_INSTR_EUROPEAN: P->trk = TRK_EUR; break;
    case MYQL_INSTR_ASIAN_GEO: P->trk = TRK_GEO; break;
    case MYQL_INSTR_ASIAN_ARITH: P->trk = TRK_ARITH; break;
    case MYQL_INSTR_LOOKBACK: P->trk = TRK_LB; break;
    default: P->trk = ins->barrier_up ? TRK_BUP : TRK_BDN; break;
  }
  const int pd = P->trk != TRK_EUR;
  instr_t *in = &P->in;
  in->kind = ins->kind;
  in->payoff = ins->payoff;
  in->call = ins->option_type == MYQL_CALL;
  in->fixed = ins->fixed_strike;
  in->action = ins->barrier_action;
  in->timing = ins->rebate_timing;
  in->mode = c->greek_mode;
  in->rebate = ins->rebate;
  in->rate = ins->barrier_rate;
  in->T = ins->maturity;
  in->eps = ins->payoff_eps;
  if (c->greek_mode != MYQL_GREEKS_NONE && ins->payoff != MYQL_PAYOFF_VANILLA && in->eps < 0.0) {
    double var = 0.0;
    if (P->nf == 0) var += m->vol * m->vol;
    for (int f = 0; f < P->nf; ++f) var += expected_avg_var(&m->heston[f], P->T);
    if (m->jump == MYQL_JUMP_MERTON) var += m->jump_lambda * (m->merton_mu * m->merton_mu + m->merton_delta * m->merton_delta);
    if (m->jump == MYQL_JUMP_KOU)
      var += m->jump_lambda * (m->kou_p_up / (m->kou_eta1 * m->kou_eta1) + (1.0 - m->kou_p_up) / (m->kou_eta2 * m->kou_eta2));
    const double sigma_eff = sqrt(var);
    in->eps = ins->is_strip ? sigma_eff * job->S0 * sqrt(P->T) / 10.0 : sigma_eff * ins->strikes[0] * sqrt(P->T) / 10.0;
  }
  /* tracker config */
  tcfg_t *tc = &P->tcfg;
  tc->past_avg_log = ins->past_avg_log;
  tc->past_avg_S = ins->past_avg_S;
  tc->t_elapsed = ins->t_elapsed;
  tc->hist_min_logS = ins->hist_min_S > 0.0 ? log(ins->hist_min_S) : 1e300;
  tc->hist_max_logS = ins->hist_max_S > 0.0 ? log(ins->hist_max_S) : -1e300;
  if (ins->kind == MYQL_INSTR_BARRIER) {
    tc->b_base = log(ins->barrier);
    if (c->greek_mode != MYQL_GREEKS_NONE) {
      tc->b_up = log(ins->barrier * job->S0 / (job->S0 + P->h));
      tc->b_dn = log(ins->barrier * job->S0 / (job->S0 - P->h));
    } else {
      tc->b_up = tc->b_dn = tc->b_base;
    }
  }
  /* scenarios */
  const size_t steps = (size_t)c->time_steps;
  const double T = P->T, dt = T / (double)steps;
  double vol[MAXSC], v0[MAXSC][2], dts[MAXSC], Ts[MAXSC], rs[MAXSC];
  int n = 0;
  vol[0] = m->vol;
  v0[0][0] = m->heston[0].v0;
  v0[0][1] = m->heston[1].v0;
  dts[0] = dt;
  Ts[0] = T;
  rs[0] = job->r;
  n = 1;
  if (c->greek_mode == MYQL_GREEKS_FULL) {
    for (int s = 1; s < 9; ++s) {
      vol[s] = vol[0];
      v0[s][0] = v0[0][0];
      v0[s][1] = v0[0][1];
      dts[s] = dt;
      Ts[s] = T;
      rs[s] = job->r;
    }
    if (P->nf == 0) {
      vol[1] += c->vol_bump;
      vol[2] -= c->vol_bump;
    } else {
      v0[1][0] += c->vol_bump;
      v0[2][0] -= c->vol_bump;
    }
    Ts[3] = T + c->t_bump;
    dts[3] = Ts[3] / steps;
    Ts[4] = T - c->t_bump;
    dts[4] = Ts[4] / steps;
    rs[5] = job->r + c->r_bump;
    rs[6] = job->r - c->r_bump;
    v0[7][1] += c->vol_bump;
    v0[8][1] -= c->vol_bump;
    n = P->nf == 2 ? 9 : 7;
  }
  P->n_sc = n;
  for (int s = 0; s < n; ++s) {
    /* the rho steppers reuse the base workspace (MonteCarloPricer.hpp:294-295) */
    const int rho_sc = s == 5 || s == 6;
    for (int f = 0; f < P->nf; ++f)
      if (c->scheme[f] == MYQL_SCHEME_NCI && !rho_sc) {
        myql_heston_params hp = m->heston[f];
        hp.v0 = v0[s][f];
        nci_build(&nci[s][f], &hp, dts[s]);
      }
    P->st[s].path_dep = pd;
    stepper_init(&P->st[s], job, vol[s], v0[s], dts[s], rs[s], Ts[s], rho_sc ? nci[0] : nci[s]);
    P->st[s].path_dep = pd;
    stepper_jumps(&P->st[s], m, pd ? dts[s] : Ts[s]);
  }
  if (c->greek_mode == MYQL_GREEKS_FULL) {
    P->inv_2dv = 1.0 / (2.0 * c->vol_bump);
    P->c_v[0] = P->nf == 0 ? 1.0 : 2.0 * sqrt(m->heston[0].v0);
    P->c_v[1] = P->nf == 2 ? 2.0 * sqrt(m->heston[1].v0) : 0.0;
    P->inv_2dT = 1.0 / (2.0 * c->t_bump);
    P->inv_2dr = 1.0 / (2.0 * c->r_bump);
    P->df_Tup = exp(-job->r * c->t_bump);
    P->df_Tdn = exp(job->r * c->t_bump);
    P->df_rup = exp(-c->r_bump * T);
    P->df_rdn = exp(c->r_bump * T);
  }
}

/* per-path quantity estimators for one strike from the scenario states */
static void path_q(const plan_t *P, const state_t *sts, double K, double q[NQ]) {
  double b[3];
  memset(q, 0, sizeof(double) * NQ);
  payoff_triplet(&P->in, &sts[0], P->S0, P->h, K, b);
  q[0] = b[0];
  if (P->mode == MYQL_GREEKS_NONE) return;
  q[1] = (b[1] - b[2]) * (1.0 / (2.0 * P->h));
  q[2] = (b[1] - b[0] * 2.0 + b[2]) * (1.0 / (P->h * P->h));
  if (P->mode != MYQL_GREEKS_FULL) return;
  double u[3], d[3];
  for (int f = 0; f < (P->nf == 2 ? 2 : 1); ++f) {
    payoff_triplet(&P->in, &sts[f == 0 ? 1 : 7], P->S0, P->h, K, u);
    payoff_triplet(&P->in, &sts[f == 0 ? 2 : 8], P->S0, P->h, K, d);
    q[f == 0 ? 3 : 4] = (u[0] - d[0]) * P->inv_2dv * P->c_v[f];
    q[f == 0 ? 7 : 8] = ((u[1] - u[2]) - (d[1] - d[2])) * (P->inv_2dv / (2.0 * P->h)) * P->c_v[f];
  }
  payoff_triplet(&P->in, &sts[3], P->S0, P->h, K, u);
  payoff_triplet(&P->in, &sts[4], P->S0, P->h, K, d);
  q[5] = (u[0] * P->df_Tup - d[0] * P->df_Tdn) * P->inv_2dT;
  q[9] = ((u[1] - u[2]) * P->df_Tup - (d[1] - d[2]) * P->df_Tdn) * (P->inv_2dT / (2.0 * P->h));
  payoff_triplet(&P->in, &sts[5], P->S0, P->h, K, u);
  payoff_triplet(&P->in, &sts[6], P->S0, P->h, K, d);
  q[6] = (u[0] * P->df_rup - d[0] * P->df_rdn) * P->inv_2dr;
}

/* one path of a stream: base advances *rng, bumped scenarios replay from its start */
static void one_path(const plan_t *P, xo_t *rng, state_t sts[MAXSC]) {
  const xo_t start = *rng;
  for (int s = 0; s < P->n_sc; ++s) {
    xo_t r = start;
    run_path(&P->st[s], P->trk, &P->tcfg, P->S0, &r, &sts[s]);
    if (s == 0) *rng = r;
  }
}

static void accumulate(const plan_t *P, const state_t *sts, const double *K, int nk, double *sum,
                       double *sq) {
  for (int k = 0; k < nk; ++k) {
    double q[NQ];
    path_q(P, sts, K[k], q);
    for (int j = 0; j < NQ; ++j) {
      sum[k * NQ + j] += q[j];
      sq[k * NQ + j] += q[j] * q[j];
    }
  }
}

/* 6 doubles per (scenario, path): S_T, avg-or-min, max, t_hit base/up/dn (-1 = none) */
static void write_record(const state_t *st, int trk, double *dst) {
  dst[0] = st->logS;
  dst[1] = trk == TRK_GEO ? st->sumLogS : trk == TRK_ARITH ? st->sumS : trk == TRK_LB ? st->minLogS : 0.0;
  dst[2] = trk == TRK_LB ? st->maxLogS : 0.0;
  dst[3] = st->hit_base ? st->t_base : -1.0;
  dst[4] = st->hit_up ? st->t_up : -1.0;
  dst[5] = st->hit_dn ? st->t_dn : -1.0;
}

static void free_nci(nci_ws nci[MAXSC][2]) {
  for (int s = 0; s < MAXSC; ++s)
    for (int f = 0; f < 2; ++f) {
      free(nci[s][f].y);
      free(nci[s][f].m);
    }
}

/*
 * Prices one job.  layout: MYQL_ORACLE_LAYOUT_REFERENCE / _STREAMS.
 * n_threads: OpenMP threads (reference layout: also the number of RNG streams).
 * out: 2*NQ*n_strikes doubles, same layout as myql_mc_price.
 * records (streams layout only, may be NULL): n_sc * num_paths * 6 doubles,
 * [scenario][path][6].
 * Returns 0 on success, -1 on a bad argument.
 */
int myql_oracle_mc_price(const myql_mc_job *job, int layout, int n_threads, double *out,
                         double *records) {
  if (!job || !out || n_threads < 1) return -1;
  const int nk = (int)job->instrument.n_strikes;
  const uint64_t M = job->config.num_paths;
  nci_ws nci[MAXSC][2];
  memset(nci, 0, sizeof nci);
  plan_t *P = (plan_t *)calloc(1, sizeof(plan_t));
  plan_build(P, job, nci);
  const double *K = job->instrument.strikes;
  const size_t acc_n = (size_t)nk * NQ;
  double *tsum = (double *)calloc((size_t)n_threads * acc_n, sizeof(double));
  double *tsq = (double *)calloc((size_t)n_threads * acc_n, sizeof(double));

  if (layout == MYQL_ORACLE_LAYOUT_REFERENCE) {
#pragma omp parallel num_threads(n_threads)
    {
#ifdef _OPENMP
      const int tid = omp_get_thread_num(), nt = omp_get_num_threads();
#else
      const int tid = 0, nt = 1;
#endif
      xo_t rng;
      xo_seed(&rng, job->config.seed + ((uint64_t)tid * 999983ull));
      /* libgomp static schedule: q = M / nt, the first M % nt threads get one more */
      const uint64_t q = M / (uint64_t)nt, rem = M % (uint64_t)nt;
      const uint64_t b = (uint64_t)tid < rem ? (q + 1) * tid : q * tid + rem;
      const uint64_t e = b + ((uint64_t)tid < rem ? q + 1 : q);
      state_t sts[MAXSC];
      for (uint64_t i = b; i < e; ++i) {
        one_path(P, &rng, sts);
        accumulate(P, sts, K, nk, tsum + (size_t)tid * acc_n, tsq + (size_t)tid * acc_n);
      }
    }
  } else {
    /* default stream count of the engine: min(M, clamp(M / 8, 2^17, 2^19)) */
    uint64_t S = job->config.n_streams;
    if (!S) {
      S = M / 8;
      S = S < 131072ull ? 131072ull : (S > 524288ull ? 524288ull : S);
    }
    if (S > M) S = M;
    /* stream states: sequential jumps from the seeded generator */
    xo_t *streams = (xo_t *)malloc(S * sizeof(xo_t));
    xo_seed(&streams[0], job->config.seed);
    for (uint64_t k = 0; k < job->config.stream_offset; ++k) xo_jump(&streams[0]); /* first stream index */
    for (uint64_t k = 1; k < S; ++k) {
      streams[k] = streams[k - 1];
      xo_jump(&streams[k]);
    }
#pragma omp parallel for schedule(static) num_threads(n_threads)
    for (uint64_t s = 0; s < S; ++s) {
#ifdef _OPENMP
      const int tid = omp_get_thread_num();
#else
      const int tid = 0;
#endif
      xo_t rng = streams[s];
      state_t sts[MAXSC];
      for (uint64_t i = s; i < M; i += S) {
        one_path(P, &rng, sts);
        accumulate(P, sts, K, nk, tsum + (size_t)tid * acc_n, tsq + (size_t)tid * acc_n);
        if (records)
          for (int sc = 0; sc < P->n_sc; ++sc) write_record(&sts[sc], P->trk, records + ((size_t)sc * M + i) * 6);
      }
    }
    free(streams);
  }
  /* merge in thread order, then compute_stats (MonteCarloPricer.hpp:444-457) */
  const double df = exp(-P->r * P->T), inv_M = 1.0 / (double)M;
  int active = P->mode == MYQL_GREEKS_NONE ? 1 : P->mode == MYQL_GREEKS_ESSENTIAL ? 3 : NQ;
  for (int k = 0; k < nk; ++k)
    for (int j = 0; j < NQ; ++j) {
      double s = 0.0, s2 = 0.0;
      for (int t = 0; t < n_threads; ++t) {
        s += tsum[(size_t)t * acc_n + k * NQ + j];
        s2 += tsq[(size_t)t * acc_n + k * NQ + j];
      }
      double val = 0.0, err = 0.0;
      if (j < active) {
        const double mean = s * inv_M;
        const double var = (s2 * inv_M) - (mean * mean);
        val = mean * df;
        err = sqrt(var * inv_M) * df;
      }
      out[(size_t)(2 * j) * nk + k] = val;
      out[(size_t)(2 * j + 1) * nk + k] = err;
    }
  free(tsum);
  free(tsq);
  free_nci(nci);
  free(P);
  return 0;
}

/* Stream states of the streams layout, [stream][4] (sequential jumps). */
int myql_oracle_stream_states(uint64_t seed, uint64_t first, uint64_t n, uint64_t *out) {
  xo_t r;
  xo_seed(&r, seed);
  for (uint64_t k = 0; k < first; ++k) xo_jump(&r);
  for (uint64_t k = 0; k < n; ++k) {
    memcpy(out + 4 * k, r.s, 32);
    xo_jump(&r);
  }
  return 0;
}

/* Numerics probes for the tests. */
double myql_oracle_normcdfinv(double p) { return normcdfinv_as241(p); }
double myql_oracle_poissinvcdf(double lambda, double U) { return poissinvcdf(lambda, U); }
double myql_oracle_chi2_quantile(double nu, double p) { return oracle_chi2_quantile(nu, p); }
double myql_oracle_uniform_of(uint64_t x) {
  return (double)x * 5.421010862427522170037264e-20;
}

/* ================================================================== MLMC
 * Restatement of MultiLevelMonteCarloPricer::calculate / evaluate_level
 * (pricers/mlmc/MultiLevelMonteCarloPricer.hpp:46-341) and
 * CoupledASVJStepper::multi_step_coupled (models/asvj/core/CoupledASVJStepper.hpp:170-517).
 */

/* one fine/coarse pair of the coupled stepper; sf/sc prepared with dt_fine/dt_coarse */
static void coupled_path(const stepper_t *sf, const stepper_t *sc, int trk, const tcfg_t *c, double S0,
                         int n_coarse, xo_t *r, state_t *stf, state_t *stc) {
  memset(stf, 0, sizeof *stf);
  memset(stc, 0, sizeof *stc);
  const double lS0 = log(S0);
  const double dtf = sf->dt, dtc = sc->dt;
  /* start_path for both (tracker init with their own dt) */
  state_t *sts[2] = {stf, stc};
  const double dts[2] = {dtf, dtc};
  for (int w = 0; w < 2; ++w) {
    state_t *st = sts[w];
    st->logS = lS0;
    switch (trk) {
      case TRK_GEO: st->sumLogS = c->past_avg_log * c->t_elapsed + 0.5 * st->logS * dts[w]; break;
      case TRK_ARITH:
        st->sumLogS = c->past_avg_log * c->t_elapsed + 0.5 * st->logS * dts[w];
        st->sumS = c->past_avg_S * c->t_elapsed + 0.5 * exp(st->logS) * dts[w];
        break;
      case TRK_LB:
        st->minLogS = (c->hist_min_logS < 1e300) ? c->hist_min_logS : st->logS;
        st->maxLogS = (c->hist_max_logS > -1e300) ? c->hist_max_logS : st->logS;
        break;
      case TRK_BUP:
        if (st->logS >= c->b_base) st->hit_base = 1;
        if (st->logS >= c->b_up) st->hit_up = 1;
        if (st->logS >= c->b_dn) st->hit_dn = 1;
        break;
      case TRK_BDN:
        if (st->logS <= c->b_base) st->hit_base = 1;
        if (st->logS <= c->b_up) st->hit_up = 1;
        if (st->logS <= c->b_dn) st->hit_dn = 1;
        break;
      default: break;
    }
  }
  const int pd = trk != TRK_EUR;
  const int nf = sf->nf;
  double lf = lS0, lc = lS0;
  const double total_time = n_coarse * (2.0 * dtf);
  if (nf == 0 && !pd) {
    const double G = normcdfinv_as241(uni(r));
    lf += sf->gbm_drift_dt * (n_coarse * 2) + sf->gbm_vol_dt * sqrt((double)(n_coarse * 2)) * G;
    lc += sc->gbm_drift_dt * n_coarse + sc->gbm_vol_dt * sqrt((double)n_coarse) * G;
    const double J = log_jump(sf, r);
    lf += J;
    lc += J;
  } else {
    if (!pd && nf > 0) {
      const double J = log_jump(sf, r);
      lf += J;
      lc += J;
    }
    double vf[2] = {nf >= 1 ? sf->f[0].v0 : 0.0, nf >= 2 ? sf->f[1].v0 : 0.0};
    double vc[2] = {nf >= 1 ? sc->f[0].v0 : 0.0, nf >= 2 ? sc->f[1].v0 : 0.0};
    for (int k = 0; k < n_coarse; ++k) {
      const double G1 = normcdfinv_as241(uni(r));
      const double G2 = normcdfinv_as241(uni(r));
      double Gc = (G1 + G2) / 1.4142135623730951;
      double j1 = 0.0, j2 = 0.0;
      if (nf == 0) {
        Gc = (G1 + G2) / 1.4142135623730951;
        lc += sc->gbm_drift_dt + sc->gbm_vol_dt * Gc;
        lf += sf->gbm_drift_dt + sf->gbm_vol_dt * G1;
        if (pd) {
          j1 = log_jump(sf, r);
          lf += j1;
        }
        stf->logS = lf;
        if (pd) tracker_update(stf, trk, c, dtf);
        lf += sf->gbm_drift_dt + sf->gbm_vol_dt * G2;
        if (pd) {
          j2 = log_jump(sf, r);
          lf += j2;
        }
        stf->logS = lf;
        if (pd) {
          tracker_update(stf, trk, c, dtf);
          lc += j1 + j2;
          stc->logS = lc;
          tracker_update(stc, trk, c, dtc);
        }
      } else {
        double Z1[2] = {0.0, 0.0}, Z2[2] = {0.0, 0.0}, mid[2] = {0.0, 0.0}, nxt[2] = {0.0, 0.0};
        for (int i = 0; i < nf; ++i) {
          if (sf->f[i].scheme == MYQL_SCHEME_NV) {
            Z1[i] = normcdfinv_as241(uni(r));
            const double root = sqrt(sf->f[i].W[0] * vf[i] + sf->f[i].W[1]) + sf->f[i].W[2] * Z1[i];
            mid[i] = sf->f[i].W[0] * (root * root) + sf->f[i].W[1];
          } else {
            mid[i] = evolve(&sf->f[i], vf[i], r);
          }
        }
        double r1;
        if (nf == 1) {
          const double *C = sf->f[0].C;
          r1 = sqrt(C[3] * (vf[0] + mid[0]));
          lf += C[0] + C[1] * vf[0] + C[2] * mid[0] + r1 * G1;
        } else {
          const double *Ca = sf->f[0].C, *Cb = sf->f[1].C;
          r1 = sqrt(Ca[3] * (vf[0] + mid[0]) + Cb[3] * (vf[1] + mid[1]));
          lf += Ca[0] + Ca[1] * vf[0] + Ca[2] * mid[0] + Cb[0] + Cb[1] * vf[1] + Cb[2] * mid[1] + r1 * G1;
        }
        if (pd) {
          j1 = log_jump(sf, r);
          lf += j1;
        }
        stf->logS = lf;
        if (pd) tracker_update(stf, trk, c, dtf);
        for (int i = 0; i < nf; ++i) {
          if (sf->f[i].scheme == MYQL_SCHEME_NV) {
            Z2[i] = normcdfinv_as241(uni(r));
            const double root = sqrt(sf->f[i].W[0] * mid[i] + sf->f[i].W[1]) + sf->f[i].W[2] * Z2[i];
            nxt[i] = sf->f[i].W[0] * (root * root) + sf->f[i].W[1];
          } else {
            nxt[i] = evolve(&sf->f[i], mid[i], r);
          }
        }
        double r2;
        if (nf == 1) {
          const double *C = sf->f[0].C;
          r2 = sqrt(C[3] * (mid[0] + nxt[0]));
          lf += C[0] + C[1] * mid[0] + C[2] * nxt[0] + r2 * G2;
        } else {
          const double *Ca = sf->f[0].C, *Cb = sf->f[1].C;
          r2 = sqrt(Ca[3] * (mid[0] + nxt[0]) + Cb[3] * (mid[1] + nxt[1]));
          lf += Ca[0] + Ca[1] * mid[0] + Ca[2] * nxt[0] + Cb[0] + Cb[1] * mid[1] + Cb[2] * nxt[1] + r2 * G2;
        }
        if (pd) {
          j2 = log_jump(sf, r);
          lf += j2;
        }
        stf->logS = lf;
        if (pd) tracker_update(stf, trk, c, dtf);
        double cn[2] = {0.0, 0.0};
        for (int i = 0; i < nf; ++i) {
          if (sc->f[i].scheme == MYQL_SCHEME_NV) {
            const double Zc = (Z1[i] + Z2[i]) / 1.4142135623730951;
            const double root = sqrt(sc->f[i].W[0] * vc[i] + sc->f[i].W[1]) + sc->f[i].W[2] * Zc;
            cn[i] = sc->f[i].W[0] * (root * root) + sc->f[i].W[1];
          } else {
            cn[i] = nxt[i];
          }
        }
        if (r1 + r2 > 1e-15) Gc = (r1 * G1 + r2 * G2) / hypot(r1, r2);
        if (nf == 1) {
          const double *C = sc->f[0].C;
          const double rc = sqrt(C[3] * (vc[0] + cn[0]));
          lc += C[0] + C[1] * vc[0] + C[2] * cn[0] + rc * Gc;
        } else {
          const double *Ca = sc->f[0].C, *Cb = sc->f[1].C;
          const double rc = sqrt(Ca[3] * (vc[0] + cn[0]) + Cb[3] * (vc[1] + cn[1]));
          lc += Ca[0] + Ca[1] * vc[0] + Ca[2] * cn[0] + Cb[0] + Cb[1] * vc[1] + Cb[2] * cn[1] + rc * Gc;
        }
        for (int i = 0; i < nf; ++i) {
          vf[i] = nxt[i];
          vc[i] = cn[i];
        }
        if (pd) {
          lc += j1 + j2;
          stc->logS = lc;
          tracker_update(stc, trk, c, dtc);
        }
      }
      if (!pd) stc->logS = lc;
    }
  }
  /* finalize both */
  for (int w = 0; w < 2; ++w) {
    state_t *st = sts[w];
    st->logS = w == 0 ? lf : lc;
    switch (trk) {
      case TRK_GEO:
        st->sumLogS -= 0.5 * st->logS * dts[w];
        st->sumLogS = exp(st->sumLogS / (total_time + c->t_elapsed));
        break;
      case TRK_ARITH:
        st->sumLogS -= 0.5 * st->logS * dts[w];
        st->sumS -= 0.5 * exp(st->logS) * dts[w];
        st->sumLogS = exp(st->sumLogS / (total_time + c->t_elapsed));
        st->sumS = st->sumS / (total_time + c->t_elapsed);
        break;
      case TRK_LB:
        st->minLogS = exp(st->minLogS);
        st->maxLogS = exp(st->maxLogS);
        break;
      default: break;
    }
    st->logS = exp(st->logS);
  }
}

/* one stepper of the job at step dt (total_time = T) */
static void make_stepper(stepper_t *s, const myql_mc_job *job, int pd, double dt, double T, nci_ws nci[2]) {
  const double v0[2] = {job->model.heston[0].v0, job->model.heston[1].v0};
  stepper_init(s, job, job->model.vol, v0, dt, job->r, T, nci);
  s->path_dep = pd;
  stepper_jumps(s, &job->model, pd ? dt : T);
}

typedef struct {
  int layout, n_threads;
  uint64_t S;          /* streams layout: pool size */
  xo_t *pool;          /* n_threads (reference) or S (streams) persistent states */
} mlmc_rng;

/* evaluate_level: adds sum and sum of squares of P_fine - P_coarse over dN paths */
static void mlmc_eval(const plan_t *P, const myql_mc_job *job, uint64_t base_steps, int l, uint64_t dN,
                      mlmc_rng *R, double *sum, double *sum_sq) {
  const double T = P->T;
  const int pd = P->trk != TRK_EUR;
  nci_ws nci[2];
  memset(nci, 0, sizeof nci);
  stepper_t sf, sc;
  int n_coarse;
  if (l == 0) {
    const double dt = T / (double)base_steps;
    for (int f = 0; f < P->nf; ++f)
      if (job->config.scheme[f] == MYQL_SCHEME_NCI) nci_build(&nci[f], &job->model.heston[f], dt);
    make_stepper(&sf, job, pd, dt, T, nci);
    sf.n_steps = (int)base_steps;
    n_coarse = (int)base_steps;
  } else {
    const uint64_t fine = base_steps * (1ull << l);
    const double dtf = T / (double)fine;
    for (int f = 0; f < P->nf; ++f)
      if (job->config.scheme[f] == MYQL_SCHEME_NCI) nci_build(&nci[f], &job->model.heston[f], dtf);
    make_stepper(&sf, job, pd, dtf, T, nci);
    make_stepper(&sc, job, pd, dtf * 2.0, T, nci);
    n_coarse = (int)(fine / 2);
  }
  const double K = job->instrument.strikes[0];
  const int T_threads = R->layout == MYQL_ORACLE_LAYOUT_REFERENCE ? R->n_threads : R->n_threads;
  double *ts = (double *)calloc((size_t)T_threads, sizeof(double));
  double *tq = (double *)calloc((size_t)T_threads, sizeof(double));
  if (R->layout == MYQL_ORACLE_LAYOUT_REFERENCE) {
#pragma omp parallel num_threads(R->n_threads)
    {
#ifdef _OPENMP
      const int tid = omp_get_thread_num(), nt = omp_get_num_threads();
#else
      const int tid = 0, nt = 1;
#endif
      xo_t *rng = &R->pool[tid];
      const uint64_t q = dN / (uint64_t)nt, rem = dN % (uint64_t)nt;
      const uint64_t b = (uint64_t)tid < rem ? (q + 1) * tid : q * tid + rem;
      const uint64_t e = b + ((uint64_t)tid < rem ? q + 1 : q);
      state_t a, c;
      double pf[3], pc[3];
      for (uint64_t i = b; i < e; ++i) {
        double d;
        if (l == 0) {
          run_path(&sf, P->trk, &P->tcfg, P->S0, rng, &a);
          payoff_triplet(&P->in, &a, P->S0, P->h, K, pf);
          d = pf[0];
        } else {
          coupled_path(&sf, &sc, P->trk, &P->tcfg, P->S0, n_coarse, rng, &a, &c);
          payoff_triplet(&P->in, &a, P->S0, P->h, K, pf);
          payoff_triplet(&P->in, &c, P->S0, P->h, K, pc);
          d = pf[0] - pc[0];
        }
        ts[tid] += d;
        tq[tid] += d * d;
      }
    }
  } else {
    const uint64_t U = R->S < dN ? R->S : dN;
#pragma omp parallel for schedule(static) num_threads(R->n_threads)
    for (uint64_t s = 0; s < U; ++s) {
#ifdef _OPENMP
      const int tid = omp_get_thread_num();
#else
      const int tid = 0;
#endif
      xo_t *rng = &R->pool[s];
      state_t a, c;
      double pf[3], pc[3];
      for (uint64_t i = s; i < dN; i += U) {
        double d;
        if (l == 0) {
          run_path(&sf, P->trk, &P->tcfg, P->S0, rng, &a);
          payoff_triplet(&P->in, &a, P->S0, P->h, K, pf);
          d = pf[0];
        } else {
          coupled_path(&sf, &sc, P->trk, &P->tcfg, P->S0, n_coarse, rng, &a, &c);
          payoff_triplet(&P->in, &a, P->S0, P->h, K, pf);
          payoff_triplet(&P->in, &c, P->S0, P->h, K, pc);
          d = pf[0] - pc[0];
        }
        ts[tid] += d;
        tq[tid] += d * d;
      }
    }
  }
  for (int t = 0; t < T_threads; ++t) {
    *sum += ts[t];
    *sum_sq += tq[t];
  }
  free(ts);
  free(tq);
  for (int f = 0; f < 2; ++f) {
    free(nci[f].y);
    free(nci[f].m);
  }
}

/* MultiLevelMonteCarloPricer::calculate; returns 0 */
int myql_oracle_mlmc_price(const myql_mc_job *job_in, const myql_mlmc_config *cfg, int layout,
                           int n_threads, myql_mlmc_result *res) {
  if (!job_in || !cfg || !res || n_threads < 1) return -1;
  myql_mc_job job = *job_in;
  job.config.time_steps = cfg->base_steps;
  job.config.fd_bump = cfg->fd_bump;
  nci_ws nci_unused[MAXSC][2];
  memset(nci_unused, 0, sizeof nci_unused);
  /* the plan's tracker/payoff data (no NCI tables needed here: schemes set to NV temporarily) */
  myql_mc_job jp = job;
  jp.config.greek_mode = job.config.greek_mode;
  int saved[2] = {jp.config.scheme[0], jp.config.scheme[1]};
  jp.config.scheme[0] = jp.config.scheme[1] = MYQL_SCHEME_EXACT;
  plan_t *P = (plan_t *)calloc(1, sizeof(plan_t));
  plan_build(P, &jp, nci_unused);
  (void)saved;
  const double T = P->T, df = exp(-job.r * T);
  const size_t L_max = cfg->L_max;
  mlmc_rng R;
  R.layout = layout;
  R.n_threads = n_threads;
  R.S = cfg->n_streams ? cfg->n_streams : 131072ull;
  if (layout == MYQL_ORACLE_LAYOUT_REFERENCE) {
    R.pool = (xo_t *)malloc(sizeof(xo_t) * n_threads);
    for (int t = 0; t < n_threads; ++t) xo_seed(&R.pool[t], cfg->seed + (uint64_t)t * 999983ull);
  } else {
    R.pool = (xo_t *)malloc(sizeof(xo_t) * R.S);
    xo_seed(&R.pool[0], cfg->seed);
    for (uint64_t k = 0; k < job_in->config.stream_offset; ++k) xo_jump(&R.pool[0]); /* first stream */
    for (uint64_t k = 1; k < R.S; ++k) {
      R.pool[k] = R.pool[k - 1];
      xo_jump(&R.pool[k]);
    }
  }
  size_t L = cfg->L_min;
  uint64_t N_l[32] = {0};
  double sum_dP[32] = {0}, sum_sq_dP[32] = {0}, V_l[32] = {0}, cost_l[32] = {0};
  for (size_t l = 0; l <= L_max; ++l) cost_l[l] = (double)(cfg->base_steps * (1ull << l));
  double alpha = cfg->alpha, beta = cfg->beta;
  int converged = 0;
  while (!converged) {
    for (size_t l = 0; l <= L; ++l) {
      double sum_sqrt_VC_pilot = 0.0;
      for (size_t k = 0; k <= L; ++k) sum_sqrt_VC_pilot += sqrt(V_l[k] * cost_l[k]);
      uint64_t optimal_N = 0;
      if (V_l[l] > 1e-18)
        optimal_N = (uint64_t)ceil(2.0 * pow(cfg->epsilon, -2.0) * sqrt(V_l[l] / cost_l[l]) * sum_sqrt_VC_pilot);
      uint64_t pilot_N = cfg->N0 / (1ull << l);
      if (pilot_N < 20) pilot_N = 20;
      const uint64_t target_N = pilot_N > optimal_N ? pilot_N : optimal_N;
      if (N_l[l] < target_N) {
        const uint64_t dN = target_N - N_l[l];
        mlmc_eval(P, &job, cfg->base_steps, (int)l, dN, &R, &sum_dP[l], &sum_sq_dP[l]);
        N_l[l] += dN;
        if (N_l[l] > 1) {
          const double mean = sum_dP[l] / N_l[l];
          const double v = (sum_sq_dP[l] / N_l[l]) - (mean * mean);
          V_l[l] = v > 1e-18 ? v : 1e-18;
        }
      }
    }
    if (cfg->adaptive_rates && L >= 2) {
      double est[2];
      for (int which = 0; which < 2; ++which) {
        double sum_l = 0, sum_logV = 0, sum_l_logV = 0, sum_l2 = 0;
        int count = 0;
        const size_t start_l = L - 2;
        for (size_t l = start_l; l <= L; ++l) {
          const double val = which == 0 ? fabs(sum_dP[l] / N_l[l]) : V_l[l];
          if (val > 1e-16) {
            const double y = log(val), x = (double)(l - start_l);
            sum_l += x;
            sum_logV += y;
            sum_l_logV += x * y;
            sum_l2 += x * x;
            count++;
          }
        }
        est[which] = count < 2 ? -1.0
                               : -((count * sum_l_logV - sum_l * sum_logV) / (count * sum_l2 - sum_l * sum_l)) / log(2.0);
      }
      if (est[0] > 0.3) alpha = est[0] < 2.0 ? est[0] : 2.0;
      if (est[1] > 0.3) beta = est[1] < 2.0 ? est[1] : 2.0;
    }
    double sum_sqrt_VC = 0.0;
    for (size_t l = 0; l <= L; ++l) sum_sqrt_VC += sqrt(V_l[l] * cost_l[l]);
    int needs_more = 0;
    for (size_t l = 0; l <= L; ++l) {
      const uint64_t optimal_N = (uint64_t)ceil(2.0 * pow(cfg->epsilon, -2.0) * sqrt(V_l[l] / cost_l[l]) * sum_sqrt_VC);
      if (optimal_N > N_l[l]) needs_more = 1;
    }
    if (needs_more) continue;
    const double diff_mean_L = fabs(sum_dP[L] / N_l[L]);
    double effective = diff_mean_L;
    if (L > 0) {
      const double prev = 0.5 * fabs(sum_dP[L - 1] / N_l[L - 1]);
      effective = diff_mean_L > prev ? diff_mean_L : prev;
    }
    const double bias = effective / (pow(2.0, alpha) - 1.0);
    if (bias > cfg->epsilon / 1.4142135623730951) {
      if (L < L_max) L++;
      else converged = 1;
    } else {
      converged = 1;
    }
  }
  memset(res, 0, sizeof *res);
  res->alpha_estimated = alpha;
  res->beta_estimated = beta;
  res->n_levels = (uint32_t)(L + 1);
  double var_total = 0.0;
  for (size_t l = 0; l <= L; ++l) {
    res->paths_per_level[l] = N_l[l];
    const uint64_t spp = (l == 0) ? cfg->base_steps : (cfg->base_steps * (1ull << l) * 3 / 2);
    res->total_steps += N_l[l] * spp;
    const double mean = sum_dP[l] / N_l[l];
    res->mean_diffs[l] = mean * df;
    res->var_diffs[l] = V_l[l] * df * df;
    res->price += mean * df;
    var_total += V_l[l] / N_l[l];
  }
  res->price_std_err = sqrt(var_total) * df;
  free(R.pool);
  free(P);
  return 0;
}

/* One evaluate_level call from a freshly seeded pool (probe for the tests). */
int myql_oracle_mlmc_level(const myql_mc_job *job_in, const myql_mlmc_config *cfg, int layout,
                           int n_threads, uint32_t level, uint64_t dN, double *sums) {
  if (!job_in || !cfg || !sums || n_threads < 1) return -1;
  myql_mc_job job = *job_in;
  job.config.time_steps = cfg->base_steps;
  job.config.fd_bump = cfg->fd_bump;
  nci_ws nci_unused[MAXSC][2];
  memset(nci_unused, 0, sizeof nci_unused);
  myql_mc_job jp = job;
  jp.config.scheme[0] = jp.config.scheme[1] = MYQL_SCHEME_EXACT;
  plan_t *P = (plan_t *)calloc(1, sizeof(plan_t));
  plan_build(P, &jp, nci_unused);
  mlmc_rng R;
  R.layout = layout;
  R.n_threads = n_threads;
  R.S = cfg->n_streams ? cfg->n_streams : 131072ull;
  if (layout == MYQL_ORACLE_LAYOUT_REFERENCE) {
    R.pool = (xo_t *)malloc(sizeof(xo_t) * n_threads);
    for (int t = 0; t < n_threads; ++t) xo_seed(&R.pool[t], cfg->seed + (uint64_t)t * 999983ull);
  } else {
    const uint64_t U = R.S < dN ? R.S : dN;
    R.pool = (xo_t *)malloc(sizeof(xo_t) * R.S);
    xo_seed(&R.pool[0], cfg->seed);
    /* streams [offset, offset + S): the job's stream offset, as the GPU level evaluator */
    for (uint64_t k = 0; k < job_in->config.stream_offset; ++k) xo_jump(&R.pool[0]);
    for (uint64_t k = 1; k < U; ++k) {
      R.pool[k] = R.pool[k - 1];
      xo_jump(&R.pool[k]);
    }
  }
  sums[0] = sums[1] = 0.0;
  mlmc_eval(P, &job, cfg->base_steps, (int)level, dN, &R, &sums[0], &sums[1]);
  free(R.pool);
  free(P);
  return 0;
}
