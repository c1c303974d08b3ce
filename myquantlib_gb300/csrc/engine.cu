// engine.cu -- host side of the C ABI (include/myql_gpu.h): validation, FP64
// set-up of the per-scenario constants, device-memory management, and the
// launch sequence  seed streams -> simulate -> payoff/reduce -> finalize.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "engine.h"
#include "myql_gpu.h"
#include "rng_host.h"

namespace myql {

cudaError_t launch_simulate(const SimParams &P, int s1, int s2, bool path_dep, cudaStream_t stream);
cudaError_t launch_payoff(const PayoffParams &P, unsigned long long n_tiles, cudaStream_t stream);
cudaError_t launch_finalize(const FinalizeParams &P, cudaStream_t stream);
cudaError_t upload_jump_polys(const unsigned long long polys[64][4]);
cudaError_t launch_seed_streams(unsigned long long seed, unsigned long long first,
                                unsigned long long n, unsigned long long *out, cudaStream_t stream);
cudaError_t launch_rng_draws(const unsigned long long *states, unsigned long long n,
                             unsigned long long count, unsigned long long *out, cudaStream_t stream);
cudaError_t launch_nci_build(double d, int rows, double *tmp_main, double *tmp_ty, double *tmp_tm,
                             float4 *cells_main, float4 *cells_tail, double w0, double dw,
                             int exact_slopes, cudaStream_t stream);
cudaError_t launch_nci_nodes(double d, int rows, double *tmp_main, double *tmp_ty, double *tmp_tm,
                             double w0, double dw, cudaStream_t stream);
cudaError_t launch_chi2_probe(const double *dof, const double *p, double *out, size_t n,
                              cudaStream_t stream);
cudaError_t run_peak_probe(int kind, int sm_count, cudaStream_t stream, double *ops_per_s);
cudaError_t launch_sampler_probe(int kind, const unsigned long long *x, const double *lam,
                                 float *out, size_t n, unsigned int cap, unsigned int *status,
                                 cudaStream_t stream);

thread_local std::string g_err;

const char *g_err_message() { return g_err.c_str(); }

myql_status set_error(myql_status st, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_err = buf;
  return st;
}

myql_status cuda_status(cudaError_t e, const char *what) {
  if (e == cudaSuccess) return MYQL_OK;
  if (e == cudaErrorMemoryAllocation)
    return set_error(MYQL_ERR_OOM, "%s: %s", what, cudaGetErrorString(e));
  return set_error(MYQL_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

cudaError_t DevBuf::ensure(size_t bytes) {
  if (bytes <= cap) return cudaSuccess;
  if (p) cudaFree(p);
  p = nullptr;
  cap = 0;
  size_t want = std::max(bytes, (size_t)256);
  cudaError_t e = cudaMalloc(&p, want);
  if (e != cudaSuccess) {
    p = nullptr;
    return e;
  }
  cap = want;
  return cudaSuccess;
}

void DevBuf::release() {
  if (p) cudaFree(p);
  p = nullptr;
  cap = 0;
}

// ---------------------------------------------------------------------------
// jump polynomials (computed once per process, uploaded per context)
static std::once_flag g_poly_once;
static unsigned long long g_polys[64][4];
static bool g_polys_ok = false;

static void compute_polys() {
  uint64_t tmp[64][4];
  g_polys_ok = xo_jump_polys(tmp, 64);
  std::memcpy(g_polys, tmp, sizeof tmp);
}

// The jump polynomials for callers outside this file (nullptr if the derived
// polynomial failed its check against the published jump()).
const unsigned long long (*jump_polynomials())[4] {
  std::call_once(g_poly_once, compute_polys);
  return g_polys_ok ? g_polys : nullptr;
}

int tracker_of(const myql_instrument &in) {
  switch (in.kind) {
    case MYQL_INSTR_EUROPEAN: return TRK_EUROPEAN;
    case MYQL_INSTR_ASIAN_GEO: return TRK_GEO_ASIAN;
    case MYQL_INSTR_ASIAN_ARITH: return TRK_ARITH_ASIAN;
    case MYQL_INSTR_LOOKBACK: return TRK_LOOKBACK;
    case MYQL_INSTR_BARRIER: return in.barrier_up ? TRK_BARRIER_UP : TRK_BARRIER_DOWN;
    default: return -1;
  }
}

static bool finite(double x) { return std::isfinite(x); }

myql_status validate_job(const myql_mc_job &job) {
  const myql_model &m = job.model;
  const myql_instrument &in = job.instrument;
  const myql_mc_config &c = job.config;
  if (!(job.S0 > 0.0) || !finite(job.S0) || !finite(job.r) || !finite(job.q))
    return set_error(MYQL_ERR_INVALID_ARG, "S0 must be positive and S0, r, q finite");
  if (m.num_factors < 0 || m.num_factors > 2)
    return set_error(MYQL_ERR_INVALID_ARG, "num_factors must be 0, 1 or 2");
  if (m.jump < MYQL_JUMP_NONE || m.jump > MYQL_JUMP_KOU)
    return set_error(MYQL_ERR_INVALID_ARG, "unknown jump policy %d", m.jump);
  if (m.num_factors == 0 && !(m.vol >= 0.0 && finite(m.vol)))
    return set_error(MYQL_ERR_INVALID_ARG, "ZeroFactorModel vol must be >= 0");
  for (int f = 0; f < m.num_factors; ++f) {
    const myql_heston_params &h = m.heston[f];
    const int sch = c.scheme[f];
    if (sch != MYQL_SCHEME_NV && sch != MYQL_SCHEME_EXACT && sch != MYQL_SCHEME_NCI)
      return set_error(MYQL_ERR_INVALID_ARG, "factor %d: VolScheme must be NV, Exact or NCI", f);
    if (!(h.sigma > 0.0) || !(h.theta >= 0.0) || !(h.kappa >= 0.0) || !(h.v0 >= 0.0) ||
        !(std::fabs(h.rho) <= 1.0) || !finite(h.sigma + h.theta + h.kappa + h.v0 + h.rho))
      return set_error(MYQL_ERR_INVALID_ARG,
                       "factor %d: need sigma > 0, kappa, theta, v0 >= 0, |rho| <= 1", f);
    if (sch == MYQL_SCHEME_NV && h.sigma * h.sigma > 4.0 * h.kappa * h.theta)
      return set_error(MYQL_ERR_NV_CONDITION,
                       "SchemeNV violation: sigma^2 > 4*kappa*theta (factor %d)", f);
    if (sch != MYQL_SCHEME_NV && !(h.kappa * h.theta > 0.0))
      return set_error(MYQL_ERR_INVALID_ARG,
                       "factor %d: Exact/NCI schemes need kappa * theta > 0", f);
  }
  for (int f = m.num_factors; f < 2; ++f)
    if (c.scheme[f] != MYQL_SCHEME_NONE && f >= m.num_factors && m.num_factors == 2)
      return set_error(MYQL_ERR_INVALID_ARG, "scheme set for a missing factor");
  if (m.jump != MYQL_JUMP_NONE) {
    if (!(m.jump_lambda >= 0.0) || !finite(m.jump_lambda))
      return set_error(MYQL_ERR_INVALID_ARG, "jump intensity must be >= 0");
    if (m.jump == MYQL_JUMP_MERTON && !(m.merton_delta >= 0.0))
      return set_error(MYQL_ERR_INVALID_ARG, "Merton delta must be >= 0");
    if (m.jump == MYQL_JUMP_KOU &&
        (!(m.kou_eta1 > 1.0) || !(m.kou_eta2 > 0.0) || !(m.kou_p_up >= 0.0 && m.kou_p_up <= 1.0)))
      return set_error(MYQL_ERR_INVALID_ARG, "Kou needs eta1 > 1, eta2 > 0, 0 <= p_up <= 1");
  }
  if (tracker_of(in) < 0) return set_error(MYQL_ERR_INVALID_ARG, "unknown instrument kind %d", in.kind);
  if (in.payoff < MYQL_PAYOFF_VANILLA || in.payoff > MYQL_PAYOFF_ASSET)
    return set_error(MYQL_ERR_INVALID_ARG, "unknown payoff %d", in.payoff);
  if (in.option_type != MYQL_CALL && in.option_type != MYQL_PUT)
    return set_error(MYQL_ERR_INVALID_ARG, "unknown option type %d", in.option_type);
  if (!(in.maturity > 0.0) || !finite(in.maturity))
    return set_error(MYQL_ERR_INVALID_ARG, "maturity must be positive");
  if (in.n_strikes < 1 || !in.strikes)
    return set_error(MYQL_ERR_INVALID_ARG, "need at least one strike");
  if (in.n_strikes > (1 << 20))
    return set_error(MYQL_ERR_TOO_LARGE, "at most 2^20 strikes per request");
  if (!in.is_strip && in.n_strikes != 1)
    return set_error(MYQL_ERR_INVALID_ARG, "a scalar instrument has exactly one strike");
  for (int64_t k = 0; k < in.n_strikes; ++k)
    if (!finite(in.strikes[k])) return set_error(MYQL_ERR_INVALID_ARG, "strike %lld not finite", (long long)k);
  if (in.kind == MYQL_INSTR_BARRIER && !(in.barrier > 0.0))
    return set_error(MYQL_ERR_INVALID_ARG, "barrier must be positive");
  if (c.num_paths < 1) return set_error(MYQL_ERR_INVALID_ARG, "num_paths must be >= 1");
  if (c.time_steps < 1 || c.time_steps > (1ull << 30))
    return set_error(MYQL_ERR_INVALID_ARG, "time_steps must be in [1, 2^30]");
  if (c.greek_mode < MYQL_GREEKS_NONE || c.greek_mode > MYQL_GREEKS_FULL)
    return set_error(MYQL_ERR_INVALID_ARG, "unknown GreekMode %d", c.greek_mode);
  if (c.greek_mode != MYQL_GREEKS_NONE && !(c.fd_bump > 0.0 && c.fd_bump < 1.0))
    return set_error(MYQL_ERR_INVALID_ARG, "fd_bump must be in (0, 1)");
  if (c.greek_mode == MYQL_GREEKS_FULL) {
    if (!(c.vol_bump > 0.0) || !(c.t_bump > 0.0) || !(c.r_bump > 0.0))
      return set_error(MYQL_ERR_INVALID_ARG, "Full Greeks need positive vol/t/r bumps");
    if (!(in.maturity - c.t_bump > 0.0))
      return set_error(MYQL_ERR_INVALID_ARG, "t_bump must be below the maturity");
  }
  return MYQL_OK;
}

double expected_avg_variance(const myql_heston_params &h, double T) {
  if (std::fabs(h.kappa * T) > 1e-8)
    return h.theta + (h.v0 - h.theta) * (1.0 - std::exp(-h.kappa * T)) / (h.kappa * T);
  return h.v0;
}

double jump_variance(const myql_model &m) {
  if (m.jump == MYQL_JUMP_MERTON)
    return m.jump_lambda * (m.merton_mu * m.merton_mu + m.merton_delta * m.merton_delta);
  if (m.jump == MYQL_JUMP_KOU)
    return m.jump_lambda * (m.kou_p_up / (m.kou_eta1 * m.kou_eta1) +
                            (1.0 - m.kou_p_up) / (m.kou_eta2 * m.kou_eta2));
  return 0.0;
}

// Per-scenario model inputs (MonteCarloPricer.hpp:126-148, 284-295).
struct ScDef {
  double vol;
  double v0[2];
  double dt, T, r;
};

// x - (double)(float)x, rounded to FP32: what FP32 drops of x
static float fp32_lo(double x) { return (float)(x - (double)(float)x); }

void fill_factor(FactorConst &fc, const myql_heston_params &h, double v0, int scheme,
                        double r_part, double dt, float *lo) {
  const double k = h.kappa, th = h.theta, s = h.sigma, rho = h.rho;
  fc.v0 = (float)v0;
  // log-S coefficients (ASVJstepper.hpp:276-280)
  const double term = (k * rho / s - 0.5) * dt * 0.5;
  const double c0 = (r_part - rho * k * th / s) * dt, c1 = term - rho / s, c2 = term + rho / s,
               c3 = dt * (1.0 - rho * rho) * 0.5;
  fc.C0 = (float)c0;
  fc.C1 = (float)c1;
  fc.C2 = (float)c2;
  fc.C3 = (float)c3;
  if (lo) {
    lo[0] = fp32_lo(c0);
    lo[1] = fp32_lo(c1);
    lo[2] = fp32_lo(c2);
    lo[3] = fp32_lo(c3);
  }
  if (scheme == MYQL_SCHEME_NV) {  // VolSchemes.hpp:42-48
    const double ex = std::exp(-k * dt * 0.5);
    const double psi = std::fabs(k) < 1e-10 ? dt * 0.5 : (1.0 - ex) / k;
    const double D = k * th - s * s * 0.25;
    fc.w0 = (float)ex;
    fc.w1 = (float)(D * psi);
    fc.w2 = (float)(s * std::sqrt(dt) * 0.5);
  } else {  // VolSchemes.hpp:121-125 (Exact), :326-330 (NCI)
    const double ex = std::exp(-k * dt);
    const double psi = std::fabs(k) < 1e-10 ? dt : (1.0 - ex) / k;
    const double w0 = (2.0 / (s * s * psi)) * ex;
    fc.w0 = (float)w0;
    if (lo) lo[4] = fp32_lo(w0);
    if (scheme == MYQL_SCHEME_EXACT) {
      fc.w1 = (float)(2.0 * k * th / (s * s));
      fc.w2 = (float)(0.5 * s * s * psi);
    } else {
      fc.w1 = (float)(4.0 * k * th / (s * s));
      const double w2 = 0.25 * s * s * psi;
      fc.w2 = (float)w2;
      if (lo) lo[5] = fp32_lo(w2);
    }
  }
}

// SchemeNCI n_max of the reference for one time step (VolSchemes.hpp:245-255).
static int nci_nmax_ref(const myql_heston_params &p, double dt) {
  const double v_max = std::max(p.v0, 3.0 * p.theta);
  const double ex = std::exp(-p.kappa * dt);
  const double psi = std::fabs(p.kappa) < 1e-10 ? dt : (1.0 - ex) / p.kappa;
  const double lmax = (2.0 * v_max * ex) / (p.sigma * p.sigma * psi);
  double n = std::ceil(lmax + 4.0 * std::sqrt(lmax));
  n = std::max(23.0, std::min(1023.0, n));
  return (int)n;
}

// Rows to tabulate: the reference's n_max, extended so that Poisson indices
// reached from variances far in the CIR tail (stationary Gamma quantile near
// 1 - 1e-8, or v0 if larger) are looked up rather than approximated.
int nci_rows_wanted(const myql_heston_params &p, double dt_min) {
  const double shape = 2.0 * p.kappa * p.theta / (p.sigma * p.sigma);
  const double scale = p.sigma * p.sigma / (2.0 * p.kappa);
  const double v_hi = std::max(2.0 * p.v0, scale * (shape + 6.0 * std::sqrt(shape) + 25.0));
  const double ex = std::exp(-p.kappa * dt_min);
  const double psi = std::fabs(p.kappa) < 1e-10 ? dt_min : (1.0 - ex) / p.kappa;
  const double lam = (2.0 * v_hi * ex) / (p.sigma * p.sigma * psi);
  double rows = std::ceil(lam + 6.0 * std::sqrt(lam) + 16.0);
  rows = std::max(rows, (double)nci_nmax_ref(p, dt_min) + 1.0);
  return (int)std::min(rows, 1024.0);
}

unsigned long long u999_threshold() {
  // smallest x with double(x) * 2^-64 >= 0.999
  const double lim = kNciUmax * 18446744073709551616.0;
  unsigned long long x = (unsigned long long)lim;
  x -= 4096;
  while ((double)x * 5.421010862427522e-20 < kNciUmax) ++x;
  return x;
}

myql_status make_plan(const myql_mc_job &job, Plan &pl, bool stepped) {
  const myql_model &m = job.model;
  const myql_instrument &in = job.instrument;
  const myql_mc_config &c = job.config;
  pl.nf = m.num_factors;
  pl.s1 = pl.nf >= 1 ? c.scheme[0] : 0;
  pl.s2 = pl.nf >= 2 ? c.scheme[1] : 0;
  pl.tracker = tracker_of(in);
  pl.path_dep = pl.tracker != TRK_EUROPEAN || stepped;
  pl.n_fields = tracker_fields(pl.tracker);
  pl.mode = c.greek_mode;
  pl.M = c.num_paths;
  pl.steps = (int)c.time_steps;
  pl.T = in.maturity;
  const uint64_t S_req = c.n_streams ? c.n_streams : default_streams(pl.M);
  pl.S = std::min<uint64_t>(S_req, pl.M);
  if (pl.S > (1u << 26)) return set_error(MYQL_ERR_TOO_LARGE, "at most 2^26 streams");
  const double S0 = job.S0, r = job.r, q = job.q, T = in.maturity;
  const double h = S0 * c.fd_bump;
  const bool greeks = pl.mode != MYQL_GREEKS_NONE;

  // ---- scenarios
  std::vector<ScDef> sc;
  const double dt = T / (double)pl.steps;
  ScDef base{m.vol, {m.heston[0].v0, m.heston[1].v0}, dt, T, r};
  sc.push_back(base);
  if (pl.mode == MYQL_GREEKS_FULL) {
    auto vb = [&](int f, double s) {
      ScDef d = base;
      if (pl.nf == 0)
        d.vol += s * c.vol_bump;
      else
        d.v0[f] += s * c.vol_bump;
      return d;
    };
    sc.push_back(vb(0, +1));
    sc.push_back(vb(0, -1));
    ScDef tu = base, td = base;
    tu.T = T + c.t_bump;
    tu.dt = tu.T / (double)pl.steps;
    td.T = T - c.t_bump;
    td.dt = td.T / (double)pl.steps;
    sc.push_back(tu);
    sc.push_back(td);
    ScDef ru = base, rd = base;
    ru.r = r + c.r_bump;
    rd.r = r - c.r_bump;
    sc.push_back(ru);
    sc.push_back(rd);
    if (pl.nf == 2) {
      sc.push_back(vb(1, +1));
      sc.push_back(vb(1, -1));
    }
  }
  pl.n_sc = (int)sc.size();

  SimParams &P = pl.sim;
  std::memset(&P, 0, sizeof P);
  P.n_sc = pl.n_sc;
  P.n_factors = pl.nf;
  P.jump_kind = m.jump;
  P.tracker = pl.tracker;
  P.n_steps = pl.steps;
  P.n_fields = pl.n_fields;
  P.n_streams = (uint32_t)pl.S;
  P.num_paths = pl.M;
  P.merton_mu = (float)m.merton_mu;
  P.merton_delta = (float)m.merton_delta;
  P.kou_p_up = (float)m.kou_p_up;
  P.kou_inv_eta1 = m.jump == MYQL_JUMP_KOU ? (float)(1.0 / m.kou_eta1) : 0.0f;
  P.kou_inv_eta2 = m.jump == MYQL_JUMP_KOU ? (float)(1.0 / m.kou_eta2) : 0.0f;
  P.nci_u999 = u999_threshold();
  // barrier levels in X = log(S/S0) (Barrier.hpp:58-73)
  if (in.kind == MYQL_INSTR_BARRIER) {
    const double lb = std::log(in.barrier) - std::log(S0);
    P.b_log[0] = (float)lb;
    if (greeks) {
      P.b_log[1] = (float)(std::log(in.barrier * S0 / (S0 + h)) - std::log(S0));
      P.b_log[2] = (float)(std::log(in.barrier * S0 / (S0 - h)) - std::log(S0));
    } else {
      P.b_log[1] = P.b_log[2] = (float)lb;
    }
  }
  // lookback history (Lookback.hpp:216-227, PathTrackers.hpp:142-147)
  P.lb_min0 = in.hist_min_S > 0.0 ? (float)(std::log(in.hist_min_S) - std::log(S0)) : 0.0f;
  P.lb_max0 = in.hist_max_S > 0.0 ? (float)(std::log(in.hist_max_S) - std::log(S0)) : 0.0f;
  // exact scheme small-alpha constants (VolSchemes.hpp:95-103)
  for (int f = 0; f < pl.nf; ++f) {
    const myql_heston_params &hp = m.heston[f];
    const double ab = 2.0 * hp.kappa * hp.theta / (hp.sigma * hp.sigma);
    if (ab <= 1.0 && ab > 0.0) {
      const double e = 2.71828182845904523536;
      const double pp = e / (ab + e);
      P.sm_p[f] = (float)pp;
      P.sm_inv_p[f] = (float)(1.0 / pp);
      P.sm_1mp[f] = (float)(1.0 - pp);
      P.sm_1ma[f] = (float)(1.0 - ab);
      P.sm_inv_a[f] = (float)(1.0 / ab);
    }
  }
  // per-scenario constants
  double kjump = 0.0;
  if (m.jump == MYQL_JUMP_MERTON)
    kjump = std::exp(m.merton_mu + 0.5 * m.merton_delta * m.merton_delta) - 1.0;
  else if (m.jump == MYQL_JUMP_KOU)
    kjump = (m.kou_p_up * m.kou_eta1) / (m.kou_eta1 - 1.0) +
            ((1.0 - m.kou_p_up) * m.kou_eta2) / (m.kou_eta2 + 1.0) - 1.0;
  for (int i = 0; i < pl.n_sc; ++i) {
    const ScDef &d = sc[i];
    ScenarioConst &C = P.sc[i];
    C.dt = (float)d.dt;
    C.t_end = (float)(d.dt * pl.steps);
    if (pl.nf == 0) {  // ASVJstepper.hpp:97-101
      const double drift_dt = (d.r - q - 0.5 * d.vol * d.vol) * d.dt;
      const double vol_dt = d.vol * std::sqrt(d.dt);
      if (!pl.path_dep) {
        C.gbm_drift = (float)(drift_dt * pl.steps);
        C.gbm_vol = (float)(vol_dt * std::sqrt((double)pl.steps));
      } else {
        C.gbm_drift = (float)drift_dt;
        C.gbm_vol = (float)vol_dt;
      }
    } else {
      const double r_part = (d.r - q) / (double)pl.nf;
      for (int f = 0; f < pl.nf; ++f)
        fill_factor(C.f[f], m.heston[f], d.v0[f], c.scheme[f], r_part, d.dt, f == 0 ? C.lo : nullptr);
    }
    if (!pl.path_dep && (i == SC_RUP || i == SC_RDN)) C.x_shift = (float)((d.r - r) * d.T);
    // jump window: dt for path-dependent trackers, the whole (bumped) T otherwise
    const double window = pl.path_dep ? d.dt : d.T;
    if (m.jump != MYQL_JUMP_NONE) {
      const double mean = m.jump_lambda * window;
      C.jump_mean = (float)mean;
      C.jump_mean_d = mean;
      C.jump_exp_neg_mean = (float)std::exp(-mean);
      C.jump_comp = (float)(-m.jump_lambda * kjump * window);
      C.lo[6] = fp32_lo(-m.jump_lambda * kjump * window);
    }
  }
  // The lockstep kernel merges a v0-bumped scenario's variance path into the
  // base's when its NCI constants (Poisson mean factor, degrees of freedom,
  // table scale) are the base's for every factor.  (After a v0 bump of 1e-4 about
  // one lane in ten draws a different Poisson count at the first step, and such
  // paths merge over tens of steps; on the Bates strip merging still gains 2 %
  // at 50 steps and 18 % at 800.)
  P.lock_merge = 0;
  if (pl.mode == MYQL_GREEKS_FULL && pl.nf >= 1) {
    bool same = true;
    for (int i = 1; i < pl.n_sc; ++i) {
      if (i != SC_VUP0 && i != SC_VDN0 && i != SC_VUP1 && i != SC_VDN1) continue;
      for (int f = 0; f < pl.nf; ++f) {
        const FactorConst &a = P.sc[i].f[f], &b = P.sc[0].f[f];
        same = same && a.w0 == b.w0 && a.w1 == b.w1 && a.w2 == b.w2;
      }
    }
    P.lock_merge = same ? 1 : 0;
  }

  // ---- payoff pass
  PayoffParams &Q = pl.pay;
  std::memset(&Q, 0, sizeof Q);
  Q.n_sc = pl.n_sc;
  Q.n_fields = pl.n_fields;
  Q.tracker = pl.tracker;
  Q.kind = in.kind;
  Q.payoff = in.payoff;
  Q.option_type = in.option_type;
  Q.fixed_strike = in.fixed_strike;
  Q.barrier_action = in.barrier_action;
  Q.rebate_timing = in.rebate_timing;
  Q.mode = pl.mode;
  Q.n_factors = pl.nf;
  Q.n_strikes = (int)in.n_strikes;
  Q.S0 = (float)S0;
  Q.eps_rel = (float)c.fd_bump;
  Q.rebate = (float)in.rebate;
  Q.barrier_rate = (float)in.barrier_rate;
  Q.T_instr = (float)T;
  Q.tile_paths = 2048;
  // digital smoothing (MonteCarloPricer.hpp:51-74): active for GreekMode != None
  if (greeks && in.payoff != MYQL_PAYOFF_VANILLA && in.kind != MYQL_INSTR_BARRIER) {
    double eps = in.payoff_eps;
    if (eps < 0.0) {
      double var = jump_variance(m);
      if (pl.nf == 0) var += m.vol * m.vol;
      for (int f = 0; f < pl.nf; ++f) var += expected_avg_variance(m.heston[f], T);
      const double scale = in.is_strip ? S0 : in.strikes[0];
      eps = std::sqrt(var) * scale * std::sqrt(T) / 10.0;
    }
    Q.smooth = 1;
    Q.smooth_eps = (float)(1.0 / (eps * std::sqrt(2.0)));
  }
  for (int i = 0; i < pl.n_sc; ++i) {
    const double n_dt = sc[i].dt * pl.steps;
    const double Ttot = n_dt + in.t_elapsed;
    if (pl.tracker == TRK_GEO_ASIAN) {
      Q.avg_c0[i] = (float)((in.past_avg_log * in.t_elapsed + std::log(S0) * n_dt) / Ttot - std::log(S0));
      Q.avg_c1[i] = (float)(1.0 / Ttot);
    } else if (pl.tracker == TRK_ARITH_ASIAN) {
      Q.avg_c0[i] = (float)(in.past_avg_S * in.t_elapsed / (S0 * Ttot));
      Q.avg_c1[i] = (float)(1.0 / Ttot);
    }
  }
  if (greeks) {
    Q.inv_2h = (float)(1.0 / (2.0 * h));
    Q.inv_h2 = (float)(1.0 / (h * h));
  }
  if (pl.mode == MYQL_GREEKS_FULL) {
    for (int f = 0; f < (pl.nf == 2 ? 2 : 1); ++f) {
      double two_dv, cv;
      if (pl.nf == 0) {
        two_dv = 2.0 * c.vol_bump;
        cv = 1.0;
      } else {
        const int su = f == 0 ? SC_VUP0 : SC_VUP1, sd = f == 0 ? SC_VDN0 : SC_VDN1;
        two_dv = (double)P.sc[su].f[f].v0 - (double)P.sc[sd].f[f].v0;  // bump as simulated
        cv = 2.0 * std::sqrt(m.heston[f].v0);
      }
      Q.vega_c[f] = (float)(cv / two_dv);
      Q.vanna_c[f] = (float)(cv / two_dv / (2.0 * h));
    }
    const double inv_2dT = 1.0 / (2.0 * c.t_bump);
    Q.theta_c = (float)inv_2dT;
    Q.charm_c = (float)(inv_2dT / (2.0 * h));
    Q.dfm1_tup = (float)std::expm1(-r * c.t_bump);
    Q.dfm1_tdn = (float)std::expm1(r * c.t_bump);
    Q.rho_c = (float)(1.0 / (2.0 * c.r_bump));
    Q.dfm1_rup = (float)std::expm1(-c.r_bump * T);
    Q.dfm1_rdn = (float)std::expm1(c.r_bump * T);
  }
  pl.df = std::exp(-r * T);
  pl.active_mask = pl.mode == 0 ? 0x1 : (pl.mode == 1 ? 0x7 : 0x3FF);
  if (pl.mode == 2 && pl.nf < 2) pl.active_mask &= ~((1 << MYQL_Q_VEGA1) | (1 << MYQL_Q_VANNA1));
  return MYQL_OK;
}

}  // namespace myql

using namespace myql;

// ===========================================================================
// context
struct myql_ctx : public myql::CtxBase {};

static myql_status ctx_check(myql_ctx *ctx) {
  if (!ctx) return set_error(MYQL_ERR_INVALID_ARG, "null context");
  cudaError_t e = cudaSetDevice(ctx->device);
  return cuda_status(e, "cudaSetDevice");
}

namespace myql {

// Stream states of (seed, first, n) in ctx->st_cached (kept for the next call
// with the same seed and range); copied to st_work, which the kernels advance.
myql_status ensure_streams(CtxBase *ctx, uint64_t seed, uint64_t first, uint64_t n) {
  if (!(ctx->st_valid && ctx->st_seed == seed && ctx->st_first == first && ctx->st_n == n)) {
    cudaError_t e = ctx->st_cached.ensure(n * 32);
    if (e != cudaSuccess) return cuda_status(e, "stream table");
    e = launch_seed_streams(seed, first, n, (unsigned long long *)ctx->st_cached.p, ctx->stream);
    if (e != cudaSuccess) return cuda_status(e, "seed_streams launch");
    ctx->launches++;
    ctx->st_valid = true;
    ctx->st_seed = seed;
    ctx->st_first = first;
    ctx->st_n = n;
  }
  cudaError_t e = ctx->st_work.ensure(n * 32);
  if (e != cudaSuccess) return cuda_status(e, "stream work table");
  e = cudaMemcpyAsync(ctx->st_work.p, ctx->st_cached.p, n * 32, cudaMemcpyDeviceToDevice, ctx->stream);
  return cuda_status(e, "stream table copy");
}

myql_status ensure_nci(CtxBase *ctx, const myql_heston_params &p, double dt_min, NciTable &tab) {
  const double d = 4.0 * p.kappa * p.theta / (p.sigma * p.sigma);
  const int cap = ctx->nci_rows_cap;
  const int rows = cap ? std::min(cap, nci_rows_wanted(p, dt_min)) : nci_rows_wanted(p, dt_min);
  uint64_t key;
  std::memcpy(&key, &d, sizeof key);  // d > 0: the sign bit is free for the slope rule
  if (ctx->nci_slopes) key |= 1ull << 63;
  auto it = ctx->nci.find(key);
  if (it == ctx->nci.end() || it->second.rows < rows || (cap && it->second.rows > cap)) {
    if (it != ctx->nci.end()) {
      it->second.main.release();
      it->second.tail.release();
      ctx->nci.erase(it);
    }
    NciEntry ent;
    ent.rows = rows;
    ent.d = d;
    cudaError_t e = ent.main.ensure((size_t)rows * (kNciGrid - 1) * sizeof(float4));
    if (e == cudaSuccess) e = ent.tail.ensure((size_t)rows * (kNciTail - 1) * sizeof(float4));
    DevBuf tmp;
    const size_t nm = (size_t)rows * kNciGrid, nt = (size_t)rows * kNciTail;
    if (e == cudaSuccess) e = tmp.ensure((nm + 2 * nt) * sizeof(double));
    if (e != cudaSuccess) {
      ent.main.release();
      ent.tail.release();
      return cuda_status(e, "NCI table allocation");
    }
    double *tm = (double *)tmp.p;
    const double w0 = -std::log1p(-kNciUmax);
    const double dw = (kNciTailWmax - w0) / (kNciTail - 1);
    e = launch_nci_build(d, rows, tm, tm + nm, tm + nm + nt, (float4 *)ent.main.p,
                         (float4 *)ent.tail.p, w0, dw, ctx->nci_slopes, ctx->stream);
    ctx->launches += 4;
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    tmp.release();
    if (e != cudaSuccess) {
      ent.main.release();
      ent.tail.release();
      return cuda_status(e, "NCI table build");
    }
    it = ctx->nci.emplace(key, std::move(ent)).first;
  }
  const NciEntry &ent = it->second;
  tab.main = (const float4 *)ent.main.p;
  tab.tail = (const float4 *)ent.tail.p;
  tab.rows = ent.rows;
  tab.d = (float)d;
  const double w0 = -std::log1p(-kNciUmax);
  const double dw = (kNciTailWmax - w0) / (kNciTail - 1);
  tab.tail_w0 = (float)w0;
  tab.tail_inv_dw = (float)(1.0 / dw);
  const double inv_dx = (kNciGrid - 1) / kNciUmax;
  tab.pos_scale = (unsigned long long)std::floor(inv_dx * 1125899906842624.0);  // 2^50
  return MYQL_OK;
}

// Runs one planned job into ctx->out (device, [2kQ][n_strikes]).
myql_status run_plan(CtxBase *ctx, const myql_mc_job &job, Plan &pl, double *out_dev,
                     bool keep_records) {
  cudaStream_t st = ctx->stream;
  SimParams &P = pl.sim;
  PayoffParams &Q = pl.pay;
  myql_status s = ensure_streams(ctx, job.config.seed, job.config.stream_offset, pl.S);
  if (s != MYQL_OK) return s;
  P.states = (unsigned long long *)ctx->st_work.p;
  P.loop_cap = ctx->loop_cap;
  // opt-in: the one-factor NCI lockstep's T-bumped scenarios with their constants' FP32
  // rounding errors added back (myql_ctx_set_precise_theta)
  P.lock_precise = ctx->precise_theta && P.lock_merge && pl.nf == 1 && !pl.path_dep &&
                   pl.mode == MYQL_GREEKS_FULL && job.config.scheme[0] == MYQL_SCHEME_NCI;
  // NCI tables
  for (int f = 0; f < pl.nf; ++f) {
    if (job.config.scheme[f] != MYQL_SCHEME_NCI) continue;
    double dt_min = 1e300;
    for (int i = 0; i < pl.n_sc; ++i) dt_min = std::min(dt_min, (double)P.sc[i].dt);
    s = ensure_nci(ctx, job.model.heston[f], dt_min, P.nci[f]);
    if (s != MYQL_OK) return s;
  }
  // strikes
  const int nk = (int)job.instrument.n_strikes;
  cudaError_t e = ctx->strikes.ensure(nk * sizeof(double));
  if (e != cudaSuccess) return cuda_status(e, "strike buffer");
  e = cudaMemcpyAsync(ctx->strikes.p, job.instrument.strikes, nk * sizeof(double),
                      cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return cuda_status(e, "strike copy");
  Q.strikes = (const double *)ctx->strikes.p;
  // chunking of the per-path records
  const uint64_t bytes_per_path = (uint64_t)pl.n_sc * pl.n_fields * sizeof(float);
  uint64_t chunk = ctx->records_cap_bytes / bytes_per_path;
  chunk = std::max<uint64_t>(pl.S, chunk / pl.S * pl.S);
  if (keep_records) chunk = std::max<uint64_t>(chunk, pl.M);
  chunk = std::min<uint64_t>(chunk, pl.M);
  const uint64_t n_chunks = (pl.M + chunk - 1) / chunk;
  const uint64_t tile = (uint64_t)Q.tile_paths;
  uint64_t total_tiles = 0;
  for (uint64_t c0 = 0; c0 < pl.M; c0 += chunk) total_tiles += (std::min(chunk, pl.M - c0) + tile - 1) / tile;
  e = ctx->records.ensure(chunk * bytes_per_path);
  if (e == cudaSuccess) e = ctx->partials.ensure(total_tiles * (uint64_t)nk * 2 * kQ * sizeof(double));
  if (e == cudaSuccess) e = ctx->status.ensure(16);
  if (e != cudaSuccess) return cuda_status(e, "scratch allocation");
  e = cudaMemsetAsync(ctx->status.p, 0, 16, st);
  if (e != cudaSuccess) return cuda_status(e, "status reset");
  P.records = (float *)ctx->records.p;
  P.status = (unsigned int *)ctx->status.p;
  P.rec_stride = chunk;
  Q.records = (const float *)ctx->records.p;
  Q.rec_stride = chunk;
  Q.partials = (double *)ctx->partials.p;
  uint64_t tiles_done = 0;
  for (uint64_t ci = 0; ci < n_chunks; ++ci) {
    const uint64_t b = ci * chunk, en = std::min(pl.M, b + chunk);
    P.path_begin = b;
    P.path_end = en;
    P.rec_offset = b;
    cudaEvent_t sa = ctx->phase_event(), sb = ctx->phase_event();
    cudaEventRecord(sa, st);
    e = launch_simulate(P, pl.s1, pl.s2, pl.path_dep, st);
    cudaEventRecord(sb, st);
    ctx->ev_tags.push_back(0);
    if (e != cudaSuccess) return cuda_status(e, "simulate launch");
    ctx->launches++;
    if (keep_records) continue;
    Q.n_paths = en - b;
    Q.tile0 = tiles_done;
    const uint64_t nt = (en - b + tile - 1) / tile;
    cudaEvent_t pa = ctx->phase_event(), pb = ctx->phase_event();
    cudaEventRecord(pa, st);
    e = launch_payoff(Q, nt, st);
    cudaEventRecord(pb, st);
    ctx->ev_tags.push_back(1);
    if (e != cudaSuccess) return cuda_status(e, "payoff launch");
    ctx->launches++;
    tiles_done += nt;
  }
  if (keep_records) return MYQL_OK;
  FinalizeParams F;
  F.n_strikes = nk;
  F.n_tiles = tiles_done;
  F.partials = (const double *)ctx->partials.p;
  F.out = out_dev;
  F.inv_m = 1.0 / (double)pl.M;
  F.df = pl.df;
  F.active_mask = pl.active_mask;
  e = launch_finalize(F, st);
  if (e != cudaSuccess) return cuda_status(e, "finalize launch");
  ctx->launches++;
  return MYQL_OK;
}

// Sums the event-timed phases of the last call (after the stream has completed).
void phase_times(CtxBase *ctx, double *sim_ms, double *pay_ms) {
  *sim_ms = *pay_ms = 0.0;
  for (size_t i = 0; i < ctx->ev_tags.size(); ++i) {
    float ms = 0.0f;
    if (cudaEventElapsedTime(&ms, ctx->ev_pool[2 * i], ctx->ev_pool[2 * i + 1]) == cudaSuccess)
      (ctx->ev_tags[i] == 0 ? *sim_ms : *pay_ms) += ms;
  }
}

myql_status read_status(CtxBase *ctx, myql_mc_stats *stats) {
  unsigned int hs[4] = {0, 0, 0, 0};
  cudaError_t e = cudaMemcpyAsync(hs, ctx->status.p, 16, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_status(e, "status read");
  if (stats) {
    stats->loop_cap_hits = hs[0];
    stats->table_fallbacks = hs[1];
  }
  if (hs[0]) return set_error(MYQL_ERR_LOOP_CAP, "%u bounded device loops hit their cap", hs[0]);
  return MYQL_OK;
}

}  // namespace myql

// ===========================================================================
extern "C" {

int myql_abi_version(void) { return MYQL_ABI_VERSION; }

size_t myql_last_error(char *buf, size_t len) {
  const size_t n = g_err.size();
  if (buf && len) {
    const size_t c = std::min(n, len - 1);
    std::memcpy(buf, g_err.data(), c);
    buf[c] = 0;
  }
  return n;
}

myql_status myql_ctx_create(myql_ctx **out, int device) {
  if (!out) return set_error(MYQL_ERR_INVALID_ARG, "null output pointer");
  *out = nullptr;
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0)
    return set_error(MYQL_ERR_NO_DEVICE, "no CUDA device: %s", cudaGetErrorString(e));
  if (device < 0 || device >= count) return set_error(MYQL_ERR_INVALID_ARG, "bad device %d", device);
  cudaDeviceProp prop;
  e = cudaGetDeviceProperties(&prop, device);
  if (e != cudaSuccess) return cuda_status(e, "cudaGetDeviceProperties");
  if (prop.major * 10 + prop.minor < 100)
    return set_error(MYQL_ERR_NO_DEVICE, "device %d is sm_%d%d; the kernels are built for sm_103a",
                     device, prop.major, prop.minor);
  std::call_once(g_poly_once, compute_polys);
  if (!g_polys_ok)
    return set_error(MYQL_ERR_CUDA, "xoshiro256 jump polynomial does not match the published jump()");
  e = cudaSetDevice(device);
  if (e != cudaSuccess) return cuda_status(e, "cudaSetDevice");
  e = upload_jump_polys(g_polys);
  if (e != cudaSuccess) return cuda_status(e, "jump polynomial upload");
  myql_ctx *ctx = new myql_ctx();
  ctx->device = device;
  ctx->sm_count = prop.multiProcessorCount;
  e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev0);
  if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev1);
  if (e != cudaSuccess) {
    delete ctx;
    return cuda_status(e, "stream/event creation");
  }
  *out = ctx;
  return MYQL_OK;
}

myql_status myql_ctx_destroy(myql_ctx *ctx) {
  if (!ctx) return MYQL_OK;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  ctx->release_all();
  cudaEventDestroy(ctx->ev0);
  cudaEventDestroy(ctx->ev1);
  cudaStreamDestroy(ctx->stream);
  delete ctx;
  return MYQL_OK;
}

myql_status myql_ctx_set_loop_cap(myql_ctx *ctx, uint32_t cap) {
  if (!ctx) return set_error(MYQL_ERR_INVALID_ARG, "null context");
  ctx->loop_cap = cap ? cap : kDefaultLoopCap;
  return MYQL_OK;
}

myql_status myql_ctx_set_records_limit(myql_ctx *ctx, uint64_t bytes) {
  if (!ctx) return set_error(MYQL_ERR_INVALID_ARG, "null context");
  ctx->records_cap_bytes = bytes ? bytes : (2ull << 30);
  return MYQL_OK;
}

myql_status myql_ctx_set_nci_slopes(myql_ctx *ctx, int mode) {
  if (!ctx) return set_error(MYQL_ERR_INVALID_ARG, "null context");
  if (mode != 0 && mode != 1) return set_error(MYQL_ERR_INVALID_ARG, "NCI slope mode is 0 or 1");
  ctx->nci_slopes = mode;
  return MYQL_OK;
}

myql_status myql_ctx_set_precise_theta(myql_ctx *ctx, int on) {
  if (!ctx) return set_error(MYQL_ERR_INVALID_ARG, "null context");
  if (on != 0 && on != 1) return set_error(MYQL_ERR_INVALID_ARG, "precise theta is 0 or 1");
  ctx->precise_theta = on;
  return MYQL_OK;
}

myql_status myql_ctx_set_nci_rows(myql_ctx *ctx, int max_rows) {
  if (!ctx) return set_error(MYQL_ERR_INVALID_ARG, "null context");
  if (max_rows < 0 || max_rows > 1024) return set_error(MYQL_ERR_INVALID_ARG, "NCI row cap is 0 or 1..1024");
  ctx->nci_rows_cap = max_rows;
  return MYQL_OK;
}

myql_status myql_validate_job(const myql_mc_job *job) {
  if (!job) return set_error(MYQL_ERR_INVALID_ARG, "null job");
  myql_status s = validate_job(*job);
  if (s != MYQL_OK) return s;
  Plan pl;
  return make_plan(*job, pl);
}

myql_status myql_mc_price(myql_ctx *ctx, const myql_mc_job *job, double *out,
                          myql_mc_stats *stats) {
  myql_status s = ctx_check(ctx);
  if (s != MYQL_OK) return s;
  if (!job || !out) return set_error(MYQL_ERR_INVALID_ARG, "null job or output");
  s = validate_job(*job);
  if (s != MYQL_OK) return s;
  Plan pl;
  s = make_plan(*job, pl);
  if (s != MYQL_OK) return s;
  const size_t nout = MYQL_OUT_DOUBLES(job->instrument.n_strikes);
  cudaError_t e = ctx->out.ensure(nout * sizeof(double));
  if (e != cudaSuccess) return cuda_status(e, "output buffer");
  ctx->launches = 0;
  ctx->phase_reset();
  e = cudaEventRecord(ctx->ev0, ctx->stream);
  if (e != cudaSuccess) return cuda_status(e, "event");
  s = run_plan(ctx, *job, pl, (double *)ctx->out.p, false);
  if (s != MYQL_OK) return s;
  e = cudaEventRecord(ctx->ev1, ctx->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(out, ctx->out.p, nout * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_status(e, "pricing run");
  myql_mc_stats local{};
  myql_mc_stats *st = stats ? stats : &local;
  std::memset(st, 0, sizeof *st);
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
  st->device_ms = ms;
  st->paths = pl.M;
  st->scenarios = (uint32_t)pl.n_sc;
  st->path_steps = pl.M * (uint64_t)pl.n_sc * (uint64_t)pl.steps;
  st->kernel_launches = ctx->launches;
  phase_times(ctx, &st->simulate_ms, &st->payoff_ms);
  return read_status(ctx, st);
}

myql_status myql_mc_price_async(myql_ctx *ctx, const myql_mc_job *job, double *out_dev,
                                void *stream) {
  myql_status s = ctx_check(ctx);
  if (s != MYQL_OK) return s;
  if (!job || !out_dev) return set_error(MYQL_ERR_INVALID_ARG, "null job or output");
  s = validate_job(*job);
  if (s != MYQL_OK) return s;
  Plan pl;
  s = make_plan(*job, pl);
  if (s != MYQL_OK) return s;
  cudaStream_t user = (cudaStream_t)stream;
  cudaStream_t own = ctx->stream;
  if (user) ctx->stream = user;
  ctx->launches = 0;
  ctx->phase_reset();
  s = run_plan(ctx, *job, pl, out_dev, false);
  ctx->stream = own;
  return s;
}

myql_status myql_mc_paths(myql_ctx *ctx, const myql_mc_job *job, float *records,
                          size_t records_len, uint32_t *n_scenarios, uint32_t *n_fields) {
  myql_status s = ctx_check(ctx);
  if (s != MYQL_OK) return s;
  if (!job) return set_error(MYQL_ERR_INVALID_ARG, "null job");
  s = validate_job(*job);
  if (s != MYQL_OK) return s;
  Plan pl;
  s = make_plan(*job, pl);
  if (s != MYQL_OK) return s;
  const size_t need = (size_t)pl.n_sc * pl.n_fields * pl.M;
  if (n_scenarios) *n_scenarios = (uint32_t)pl.n_sc;
  if (n_fields) *n_fields = (uint32_t)pl.n_fields;
  if (!records) return MYQL_OK;
  if (records_len < need)
    return set_error(MYQL_ERR_INVALID_ARG, "records buffer holds %zu floats, need %zu", records_len, need);
  ctx->launches = 0;
  ctx->phase_reset();
  s = run_plan(ctx, *job, pl, nullptr, true);
  if (s != MYQL_OK) return s;
  cudaError_t e = cudaMemcpyAsync(records, ctx->records.p, need * sizeof(float),
                                  cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_status(e, "records copy");
  return read_status(ctx, nullptr);
}

myql_status myql_rng_stream_states(myql_ctx *ctx, uint64_t seed, uint64_t first, uint64_t n,
                                   uint64_t *out) {
  myql_status s = ctx_check(ctx);
  if (s != MYQL_OK) return s;
  if (!out || n == 0) return set_error(MYQL_ERR_INVALID_ARG, "need an output buffer and n > 0");
  cudaError_t e = ctx->probe_a.ensure(n * 32);
  if (e != cudaSuccess) return cuda_status(e, "probe buffer");
  e = launch_seed_streams(seed, first, n, (unsigned long long *)ctx->probe_a.p, ctx->stream);
  if (e != cudaSuccess) return cuda_status(e, "seed launch");
  std::vector<uint64_t> soa(4 * n);
  e = cudaMemcpyAsync(soa.data(), ctx->probe_a.p, n * 32, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_status(e, "seed copy");
  for (uint64_t k = 0; k < n; ++k)
    for (int w = 0; w < 4; ++w) out[4 * k + w] = soa[w * n + k];
  return MYQL_OK;
}

myql_status myql_rng_draws(myql_ctx *ctx, uint64_t seed, uint64_t first, uint64_t n,
                           uint64_t count, uint64_t *out) {
  myql_status s = ctx_check(ctx);
  if (s != MYQL_OK) return s;
  if (!out || n == 0 || count == 0) return set_error(MYQL_ERR_INVALID_ARG, "need output, n > 0, count > 0");
  cudaError_t e = ctx->probe_a.ensure(n * 32);
  if (e == cudaSuccess) e = ctx->probe_b.ensure(n * count * 8);
  if (e != cudaSuccess) return cuda_status(e, "probe buffer");
  e = launch_seed_streams(seed, first, n, (unsigned long long *)ctx->probe_a.p, ctx->stream);
  if (e == cudaSuccess)
    e = launch_rng_draws((const unsigned long long *)ctx->probe_a.p, n, count,
                         (unsigned long long *)ctx->probe_b.p, ctx->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(out, ctx->probe_b.p, n * count * 8, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  return cuda_status(e, "rng draws");
}

myql_status myql_chi2_quantile(myql_ctx *ctx, const double *dof, const double *p, double *out,
                               size_t n) {
  myql_status s = ctx_check(ctx);
  if (s != MYQL_OK) return s;
  if (!dof || !p || !out || n == 0) return set_error(MYQL_ERR_INVALID_ARG, "bad probe arguments");
  cudaError_t e = ctx->probe_a.ensure(n * 8);
  if (e == cudaSuccess) e = ctx->probe_b.ensure(n * 8);
  if (e == cudaSuccess) e = ctx->probe_c.ensure(n * 8);
  if (e == cudaSuccess) e = cudaMemcpyAsync(ctx->probe_a.p, dof, n * 8, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(ctx->probe_b.p, p, n * 8, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess)
    e = launch_chi2_probe((const double *)ctx->probe_a.p, (const double *)ctx->probe_b.p,
                          (double *)ctx->probe_c.p, n, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, ctx->probe_c.p, n * 8, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  return cuda_status(e, "chi2 probe");
}

myql_status myql_probe_nci_nodes(myql_ctx *ctx, double d, int rows, double *main_out,
                                 double *tail_out) {
  myql_status s = ctx_check(ctx);
  if (s != MYQL_OK) return s;
  if (!main_out || !tail_out || rows < 1 || rows > 1024 || !(d > 0.0) || !std::isfinite(d))
    return set_error(MYQL_ERR_INVALID_ARG, "bad probe arguments");
  const size_t nm = (size_t)rows * kNciGrid, nt = (size_t)rows * kNciTail;
  cudaError_t e = ctx->probe_a.ensure((nm + 2 * nt) * sizeof(double));
  double *tm = (double *)ctx->probe_a.p;
  const double w0 = -std::log1p(-kNciUmax);
  const double dw = (kNciTailWmax - w0) / (kNciTail - 1);
  if (e == cudaSuccess) e = launch_nci_nodes(d, rows, tm, tm + nm, tm + nm + nt, w0, dw, ctx->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(main_out, tm, nm * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(tail_out, tm + nm, nt * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  return cuda_status(e, "NCI node probe");
}

myql_status myql_probe_sampler(myql_ctx *ctx, int kind, const uint64_t *x, const double *lambda,
                               float *out, size_t n) {
  myql_status s = ctx_check(ctx);
  if (s != MYQL_OK) return s;
  if (!x || !out || n == 0 || (kind == 1 && !lambda) || kind < 0 || kind > 1)
    return set_error(MYQL_ERR_INVALID_ARG, "bad probe arguments");
  cudaError_t e = ctx->probe_a.ensure(n * 8);
  if (e == cudaSuccess) e = ctx->probe_b.ensure(n * 8);
  if (e == cudaSuccess) e = ctx->probe_c.ensure(n * 4 + 16);
  if (e == cudaSuccess) e = cudaMemcpyAsync(ctx->probe_a.p, x, n * 8, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess && kind == 1)
    e = cudaMemcpyAsync(ctx->probe_b.p, lambda, n * 8, cudaMemcpyHostToDevice, ctx->stream);
  unsigned int *status = (unsigned int *)((char *)ctx->probe_c.p + n * 4);
  if (e == cudaSuccess) e = cudaMemsetAsync(status, 0, 4, ctx->stream);
  if (e == cudaSuccess)
    e = launch_sampler_probe(kind, (const unsigned long long *)ctx->probe_a.p,
                             (const double *)ctx->probe_b.p, (float *)ctx->probe_c.p, n,
                             ctx->loop_cap, status, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, ctx->probe_c.p, n * 4, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  return cuda_status(e, "sampler probe");
}

myql_status myql_probe_peak(myql_ctx *ctx, int kind, double *ops_per_second) {
  myql_status s = ctx_check(ctx);
  if (s != MYQL_OK) return s;
  if (!ops_per_second || kind < 0 || kind > 1) return set_error(MYQL_ERR_INVALID_ARG, "bad peak probe arguments");
  return cuda_status(run_peak_probe(kind, ctx->sm_count, ctx->stream, ops_per_second), "peak probe");
}

}  // extern "C"
