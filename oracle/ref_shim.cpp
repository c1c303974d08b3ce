// oracle/ref_shim.cpp -- C entry point over the reference's own Monte Carlo
// pricer, compiled from the unmodified headers under <reference>/include with
// the Boost-API shim in oracle/compat.  TEST INFRASTRUCTURE ONLY (builds where
// the reference sources exist; output goes to oracle/_ref/).
//
// The reference is a set of templates; this file instantiates the
// configurations the tests and the CPU baseline use and picks one at run time
// from a myql_mc_job.  Heston SchemeNV and Black-Scholes get every instrument
// branch (Asian and lookback fixed/floating x call/put, barrier up/down x
// in/out x call/put x rebate timing); the other stepper families get the
// combinations the workloads use.  Unlisted combinations return -2.
#include <omp.h>

#include <cmath>
#include <cstring>
#include <type_traits>
#include <vector>

#include <myql/instruments/Payoffs.hpp>
#include <myql/instruments/options/Asian.hpp>
#include <myql/instruments/options/Barrier.hpp>
#include <myql/instruments/options/European.hpp>
#include <myql/instruments/options/Lookback.hpp>
#include <myql/models/asvj/core/ASVJmodel.hpp>
#include <myql/models/asvj/core/ASVJstepper.hpp>
#include <myql/pricers/fourier/FourierPricer.hpp>
#include <myql/models/asvj/core/CoupledASVJStepper.hpp>
#include <myql/pricers/mlmc/MultiLevelMonteCarloPricer.hpp>
#include <myql/pricers/montecarlo/MonteCarloPricer.hpp>

#include "myql_gpu.h"

namespace {

HestonParams hp(const myql_heston_params &h) { return HestonParams{h.kappa, h.theta, h.sigma, h.rho, h.v0}; }
MertonParams mp(const myql_model &m) { return MertonParams{m.jump_lambda, m.merton_mu, m.merton_delta}; }
KouParams kp(const myql_model &m) { return KouParams{m.jump_lambda, m.kou_p_up, m.kou_eta1, m.kou_eta2}; }

MonteCarloConfig cfg_of(const myql_mc_job &j) {
  MonteCarloConfig c;
  c.num_paths = j.config.num_paths;
  c.time_steps = j.config.time_steps;
  c.seed = j.config.seed;
  c.fd_bump = j.config.fd_bump;
  c.vol_bump = j.config.vol_bump;
  c.t_bump = j.config.t_bump;
  c.r_bump = j.config.r_bump;
  return c;
}

template <class T>
void put(double *out, int n, int q, const T &val, const T &err) {
  if constexpr (std::is_same_v<T, double>) {
    out[(size_t)(2 * q) * n] = val;
    out[(size_t)(2 * q + 1) * n] = err;
  } else {
    for (int k = 0; k < n; ++k) {
      out[(size_t)(2 * q) * n + k] = val[k];
      out[(size_t)(2 * q + 1) * n + k] = err[k];
    }
  }
}

template <GreekMode Mode, class R>
void store(const R &res, int n, double *out) {
  std::memset(out, 0, sizeof(double) * 2 * MYQL_Q_COUNT * n);
  put(out, n, MYQL_Q_PRICE, res.price, res.price_std_err);
  if constexpr (Mode != GreekMode::None) {
    put(out, n, MYQL_Q_DELTA, res.delta, res.delta_std_err);
    put(out, n, MYQL_Q_GAMMA, res.gamma, res.gamma_std_err);
  }
  if constexpr (Mode == GreekMode::Full) {
    put(out, n, MYQL_Q_VEGA0, res.vega[0], res.vega_std_err[0]);
    put(out, n, MYQL_Q_VEGA1, res.vega[1], res.vega_std_err[1]);
    put(out, n, MYQL_Q_THETA, res.theta, res.theta_std_err);
    put(out, n, MYQL_Q_RHO, res.rho, res.rho_std_err);
    put(out, n, MYQL_Q_VANNA0, res.vanna[0], res.vanna_std_err[0]);
    put(out, n, MYQL_Q_VANNA1, res.vanna[1], res.vanna_std_err[1]);
    put(out, n, MYQL_Q_CHARM, res.charm, res.charm_std_err);
  }
}

template <class Model, class Stepper, class Instr, GreekMode Mode>
int run(const Model &model, const Instr &ins, const myql_mc_job &j, double *out) {
  MonteCarloPricer<Model, Stepper, Instr, Mode> pricer(model, cfg_of(j));
  const auto res = pricer.calculate(j.S0, j.r, j.q, ins);
  store<Mode>(res, (int)ins.size(), out);
  return 0;
}

template <class Model, class Stepper, class Instr>
int run_mode(const Model &model, const Instr &ins, const myql_mc_job &j, double *out) {
  switch (j.config.greek_mode) {
    case MYQL_GREEKS_NONE: return run<Model, Stepper, Instr, GreekMode::None>(model, ins, j, out);
    case MYQL_GREEKS_ESSENTIAL: return run<Model, Stepper, Instr, GreekMode::Essential>(model, ins, j, out);
    default:
      if constexpr (std::is_same_v<typename Instr::ResultType, double>)
        return run<Model, Stepper, Instr, GreekMode::Full>(model, ins, j, out);
      return -2;  // strip Full mode is undefined behaviour in the reference
  }
}

bool is(const myql_mc_job &j, int nf, int s1, int s2, int jump) {
  return j.model.num_factors == nf && j.model.jump == jump && (nf < 1 || j.config.scheme[0] == s1) &&
         (nf < 2 || j.config.scheme[1] == s2);
}

using CallV = PayoffVanilla<OptionType::Call>;
using PutV = PayoffVanilla<OptionType::Put>;

// European instruments of one payoff type over a stepper.
template <class Model, class Stepper, class Pay>
int european(const Model &model, const myql_mc_job &j, double *out) {
  const auto &in = j.instrument;
  Pay pay;
  if constexpr (Pay::needs_smoothing) pay.eps = in.payoff_eps;
  if (in.is_strip) {
    std::vector<double> K(in.strikes, in.strikes + in.n_strikes);
    EuropeanOption<Pay, std::vector<double>> opt(K, in.maturity, pay);
    return run_mode<Model, Stepper, decltype(opt)>(model, opt, j, out);
  }
  EuropeanOption<Pay> opt(in.strikes[0], in.maturity, pay);
  return run_mode<Model, Stepper, decltype(opt)>(model, opt, j, out);
}

template <class Model, class V1, class V2, class Jump>
int european_any(const Model &model, const myql_mc_job &j, double *out) {
  using St = ASVJStepper<V1, V2, Jump, TrackerEuropean>;
  const auto &in = j.instrument;
  const bool call = in.option_type == MYQL_CALL;
  if (in.payoff == MYQL_PAYOFF_VANILLA)
    return call ? european<Model, St, CallV>(model, j, out) : european<Model, St, PutV>(model, j, out);
  if (in.payoff == MYQL_PAYOFF_CASH)
    return call ? european<Model, St, PayoffCashOrNothing<OptionType::Call>>(model, j, out)
                : european<Model, St, PayoffCashOrNothing<OptionType::Put>>(model, j, out);
  return call ? european<Model, St, PayoffAssetOrNothing<OptionType::Call>>(model, j, out)
              : european<Model, St, PayoffAssetOrNothing<OptionType::Put>>(model, j, out);
}

// Path-dependent scalar vanilla instruments over a stepper family: the
// combinations the batched and strip workloads use (fixed-strike Asian calls,
// floating lookback calls, up-and-out calls and down-and-out puts without
// rebate).  exotic_all below instantiates every branch for two families.
template <class Model, class V1, class V2, class Jump>
int exotic_any(const Model &model, const myql_mc_job &j, double *out) {
  const auto &in = j.instrument;
  if (in.is_strip || in.payoff != MYQL_PAYOFF_VANILLA) return -2;
  const bool call = in.option_type == MYQL_CALL;
  const double K = in.strikes[0], T = in.maturity;
  switch (in.kind) {
    case MYQL_INSTR_ASIAN_ARITH: {
      using St = ASVJStepper<V1, V2, Jump, TrackerArithAsian>;
      if (!in.fixed_strike || !call) return -2;
      AsianOption<TrackerArithAsian, CallV, true> opt(K, T, in.past_avg_S, in.past_avg_log, in.t_elapsed);
      return run_mode<Model, St, decltype(opt)>(model, opt, j, out);
    }
    case MYQL_INSTR_ASIAN_GEO: {
      using St = ASVJStepper<V1, V2, Jump, TrackerGeoAsian>;
      if (!in.fixed_strike || !call) return -2;
      AsianOption<TrackerGeoAsian, CallV, true> opt(K, T, in.past_avg_log, in.t_elapsed);
      return run_mode<Model, St, decltype(opt)>(model, opt, j, out);
    }
    case MYQL_INSTR_LOOKBACK: {
      using St = ASVJStepper<V1, V2, Jump, TrackerLookback>;
      if (in.fixed_strike || !call) return -2;
      LookbackOption<CallV, false> opt(K, T, in.hist_min_S, in.hist_max_S);
      return run_mode<Model, St, decltype(opt)>(model, opt, j, out);
    }
    case MYQL_INSTR_BARRIER: {
      if (in.rebate_timing != MYQL_REBATE_NONE) return -2;
      if (in.barrier_up && in.barrier_action == MYQL_BARRIER_OUT && call) {
        using St = ASVJStepper<V1, V2, Jump, TrackerBarrier<true>>;
        UpAndOutCall<> opt(K, in.barrier, T, in.barrier_rate, in.rebate);
        return run_mode<Model, St, decltype(opt)>(model, opt, j, out);
      }
      if (!in.barrier_up && in.barrier_action == MYQL_BARRIER_OUT && !call) {
        using St = ASVJStepper<V1, V2, Jump, TrackerBarrier<false>>;
        DownAndOutPut<> opt(K, in.barrier, T, in.barrier_rate, in.rebate);
        return run_mode<Model, St, decltype(opt)>(model, opt, j, out);
      }
      return -2;
    }
    default: return -2;
  }
}

// ---- every instrument branch of Asian.hpp, Lookback.hpp and Barrier.hpp

// AsianOption<Tracker, Payoff, FixedStrike> (Asian.hpp:7-131) with its in-flight
// constructor: arithmetic (:63-69) or geometric (:53-57).
template <class Model, class V1, class V2, class Jump, class Trk, class Pay, bool Fixed>
int asian_one(const Model &model, const myql_mc_job &j, double *out) {
  using St = ASVJStepper<V1, V2, Jump, Trk>;
  const auto &in = j.instrument;
  if constexpr (std::is_same_v<Trk, TrackerArithAsian>) {
    AsianOption<Trk, Pay, Fixed> opt(in.strikes[0], in.maturity, in.past_avg_S, in.past_avg_log, in.t_elapsed);
    return run_mode<Model, St, decltype(opt)>(model, opt, j, out);
  } else {
    AsianOption<Trk, Pay, Fixed> opt(in.strikes[0], in.maturity, in.past_avg_log, in.t_elapsed);
    return run_mode<Model, St, decltype(opt)>(model, opt, j, out);
  }
}

template <class Model, class V1, class V2, class Jump, class Trk>
int asian_all(const Model &model, const myql_mc_job &j, double *out) {
  const bool call = j.instrument.option_type == MYQL_CALL, fixed = j.instrument.fixed_strike != 0;
  if (fixed)
    return call ? asian_one<Model, V1, V2, Jump, Trk, CallV, true>(model, j, out)
                : asian_one<Model, V1, V2, Jump, Trk, PutV, true>(model, j, out);
  return call ? asian_one<Model, V1, V2, Jump, Trk, CallV, false>(model, j, out)
              : asian_one<Model, V1, V2, Jump, Trk, PutV, false>(model, j, out);
}

// LookbackOption<Payoff, FixedStrike> (Lookback.hpp:8-110) with historical extremes.
template <class Model, class V1, class V2, class Jump, class Pay, bool Fixed>
int lookback_one(const Model &model, const myql_mc_job &j, double *out) {
  using St = ASVJStepper<V1, V2, Jump, TrackerLookback>;
  const auto &in = j.instrument;
  LookbackOption<Pay, Fixed> opt(in.strikes[0], in.maturity, in.hist_min_S, in.hist_max_S);
  return run_mode<Model, St, decltype(opt)>(model, opt, j, out);
}

template <class Model, class V1, class V2, class Jump>
int lookback_all(const Model &model, const myql_mc_job &j, double *out) {
  const bool call = j.instrument.option_type == MYQL_CALL, fixed = j.instrument.fixed_strike != 0;
  if (fixed)
    return call ? lookback_one<Model, V1, V2, Jump, CallV, true>(model, j, out)
                : lookback_one<Model, V1, V2, Jump, PutV, true>(model, j, out);
  return call ? lookback_one<Model, V1, V2, Jump, CallV, false>(model, j, out)
              : lookback_one<Model, V1, V2, Jump, PutV, false>(model, j, out);
}

// BarrierOption<Payoff, Dir, Action, Timing> (Barrier.hpp:17-124): up/down x
// in/out x call/put x rebate {None, AtHit, AtMaturity}.
template <class Model, class V1, class V2, class Jump, class Pay, BarrierDirection D, BarrierAction A,
          RebateTiming R>
int barrier_one(const Model &model, const myql_mc_job &j, double *out) {
  using Opt = BarrierOption<Pay, D, A, R>;
  using St = ASVJStepper<V1, V2, Jump, typename Opt::Tracker>;
  const auto &in = j.instrument;
  Opt opt(in.strikes[0], in.barrier, in.maturity, in.barrier_rate, in.rebate);
  return run_mode<Model, St, Opt>(model, opt, j, out);
}

template <class Model, class V1, class V2, class Jump, class Pay, BarrierDirection D, BarrierAction A>
int barrier_rebate(const Model &model, const myql_mc_job &j, double *out) {
  switch (j.instrument.rebate_timing) {
    case MYQL_REBATE_NONE: return barrier_one<Model, V1, V2, Jump, Pay, D, A, RebateTiming::None>(model, j, out);
    case MYQL_REBATE_AT_HIT: return barrier_one<Model, V1, V2, Jump, Pay, D, A, RebateTiming::AtHit>(model, j, out);
    default: return barrier_one<Model, V1, V2, Jump, Pay, D, A, RebateTiming::AtMaturity>(model, j, out);
  }
}

template <class Model, class V1, class V2, class Jump, class Pay>
int barrier_all_pay(const Model &model, const myql_mc_job &j, double *out) {
  const auto &in = j.instrument;
  constexpr auto Up = BarrierDirection::Up, Dn = BarrierDirection::Down;
  constexpr auto In = BarrierAction::In, Out = BarrierAction::Out;
  if (in.barrier_up)
    return in.barrier_action == MYQL_BARRIER_OUT ? barrier_rebate<Model, V1, V2, Jump, Pay, Up, Out>(model, j, out)
                                                 : barrier_rebate<Model, V1, V2, Jump, Pay, Up, In>(model, j, out);
  return in.barrier_action == MYQL_BARRIER_OUT ? barrier_rebate<Model, V1, V2, Jump, Pay, Dn, Out>(model, j, out)
                                               : barrier_rebate<Model, V1, V2, Jump, Pay, Dn, In>(model, j, out);
}

template <class Model, class V1, class V2, class Jump>
int exotic_all(const Model &model, const myql_mc_job &j, double *out) {
  const auto &in = j.instrument;
  if (in.is_strip || in.payoff != MYQL_PAYOFF_VANILLA) return -2;
  switch (in.kind) {
    case MYQL_INSTR_ASIAN_ARITH: return asian_all<Model, V1, V2, Jump, TrackerArithAsian>(model, j, out);
    case MYQL_INSTR_ASIAN_GEO: return asian_all<Model, V1, V2, Jump, TrackerGeoAsian>(model, j, out);
    case MYQL_INSTR_LOOKBACK: return lookback_all<Model, V1, V2, Jump>(model, j, out);
    case MYQL_INSTR_BARRIER:
      return in.option_type == MYQL_CALL ? barrier_all_pay<Model, V1, V2, Jump, CallV>(model, j, out)
                                         : barrier_all_pay<Model, V1, V2, Jump, PutV>(model, j, out);
    default: return -2;
  }
}

MLMCConfig mlmc_cfg_of(const myql_mlmc_config &c) {
  MLMCConfig m;
  m.epsilon = c.epsilon;
  m.L_min = c.L_min;
  m.L_max = c.L_max;
  m.N0 = c.N0;
  m.base_steps = c.base_steps;
  m.alpha = c.alpha;
  m.beta = c.beta;
  m.adaptive_rates = c.adaptive_rates != 0;
  m.seed = c.seed;
  m.fd_bump = c.fd_bump;
  return m;
}

template <class Model, class Coupled, class Instr>
int run_mlmc(const Model &model, const Instr &ins, const myql_mc_job &j, const myql_mlmc_config &c,
             myql_mlmc_result *res) {
  MultiLevelMonteCarloPricer<Model, Coupled, Instr, GreekMode::None> pricer(model, mlmc_cfg_of(c));
  const auto r = pricer.calculate(j.S0, j.r, j.q, ins);
  std::memset(res, 0, sizeof *res);
  res->price = r.price;
  res->price_std_err = r.price_std_err;
  res->total_steps = r.total_steps;
  res->n_levels = (uint32_t)r.paths_per_level.size();
  for (size_t l = 0; l < r.paths_per_level.size() && l < MYQL_MLMC_MAX_LEVELS; ++l) {
    res->paths_per_level[l] = r.paths_per_level[l];
    res->mean_diffs[l] = r.mean_diffs[l];
    res->var_diffs[l] = r.var_diffs[l];
  }
  res->alpha_estimated = r.alpha_estimated;
  res->beta_estimated = r.beta_estimated;
  return 0;
}

}  // namespace

extern "C" {

// The reference's MultiLevelMonteCarloPricer (GreekMode::None) for the
// instantiated combinations; -2 otherwise.
int myql_ref_mlmc_price(const myql_mc_job *jp, const myql_mlmc_config *cp, int n_threads,
                        myql_mlmc_result *res) {
  if (!jp || !cp || !res) return -1;
  omp_set_num_threads(n_threads > 0 ? n_threads : 1);
  const myql_mc_job &j = *jp;
  const auto &m = j.model;
  const auto &in = j.instrument;
  const double K = in.strikes[0], T = in.maturity;
  const bool call = in.option_type == MYQL_CALL;
  if (in.payoff != MYQL_PAYOFF_VANILLA || in.is_strip) return -2;
  if (is(j, 1, MYQL_SCHEME_NV, 0, MYQL_JUMP_NONE)) {
    HestonModel model(hp(m.heston[0]));
    if (in.kind == MYQL_INSTR_BARRIER && !in.barrier_up && in.barrier_action == MYQL_BARRIER_OUT && !call &&
        in.rebate_timing == MYQL_REBATE_NONE) {
      DownAndOutPut<> opt(K, in.barrier, T, in.barrier_rate, in.rebate);
      return run_mlmc<HestonModel, CoupledHestonStepper<SchemeNV, TrackerBarrier<false>>, decltype(opt)>(model, opt, j, *cp, res);
    }
    if (in.kind == MYQL_INSTR_EUROPEAN && call) {
      EuropeanOption<CallV> opt(K, T);
      return run_mlmc<HestonModel, CoupledHestonStepper<SchemeNV, TrackerEuropean>, decltype(opt)>(model, opt, j, *cp, res);
    }
    return -2;
  }
  if (is(j, 1, MYQL_SCHEME_NCI, 0, MYQL_JUMP_MERTON) && in.kind == MYQL_INSTR_EUROPEAN && call) {
    BatesModel model(hp(m.heston[0]), mp(m));
    EuropeanOption<CallV> opt(K, T);
    return run_mlmc<BatesModel, CoupledBatesStepper<SchemeNCI, TrackerEuropean>, decltype(opt)>(model, opt, j, *cp, res);
  }
  if (is(j, 0, 0, 0, MYQL_JUMP_NONE) && in.kind == MYQL_INSTR_ASIAN_ARITH && call && in.fixed_strike) {
    BlackScholesModel model(m.vol);
    AsianOption<TrackerArithAsian, CallV, true> opt(K, T);
    return run_mlmc<BlackScholesModel, CoupledBlackScholesStepper<TrackerArithAsian>, decltype(opt)>(model, opt, j, *cp, res);
  }
  if (is(j, 2, MYQL_SCHEME_NV, MYQL_SCHEME_EXACT, MYQL_JUMP_KOU) && in.kind == MYQL_INSTR_LOOKBACK && call &&
      !in.fixed_strike) {
    DoubleBatesKouModel model(hp(m.heston[0]), hp(m.heston[1]), kp(m));
    LookbackOption<CallV, false> opt(K, T);
    return run_mlmc<DoubleBatesKouModel, CoupledDoubleBatesKouStepper<SchemeNV, SchemeExact, TrackerLookback>,
                    decltype(opt)>(model, opt, j, *cp, res);
  }
  return -2;
}


// Prices one job with the reference's MonteCarloPricer on n_threads OpenMP
// threads.  Returns 0, or -2 when the combination is not instantiated here.
int myql_ref_mc_price(const myql_mc_job *jp, int n_threads, double *out) {
  if (!jp || !out) return -1;
  omp_set_num_threads(n_threads > 0 ? n_threads : 1);
  const myql_mc_job &j = *jp;
  const auto &m = j.model;
  const bool eur = j.instrument.kind == MYQL_INSTR_EUROPEAN;
  if (is(j, 1, MYQL_SCHEME_NV, 0, MYQL_JUMP_NONE)) {
    HestonModel model(hp(m.heston[0]));
    return eur ? european_any<HestonModel, SchemeNV, NullVolScheme, NoJumps>(model, j, out)
               : exotic_all<HestonModel, SchemeNV, NullVolScheme, NoJumps>(model, j, out);
  }
  if (is(j, 1, MYQL_SCHEME_EXACT, 0, MYQL_JUMP_NONE) && eur) {
    HestonModel model(hp(m.heston[0]));
    return european_any<HestonModel, SchemeExact, NullVolScheme, NoJumps>(model, j, out);
  }
  if (is(j, 1, MYQL_SCHEME_NCI, 0, MYQL_JUMP_NONE) && eur) {
    HestonModel model(hp(m.heston[0]));
    return european_any<HestonModel, SchemeNCI, NullVolScheme, NoJumps>(model, j, out);
  }
  if (is(j, 1, MYQL_SCHEME_NCI, 0, MYQL_JUMP_MERTON) && eur) {
    BatesModel model(hp(m.heston[0]), mp(m));
    return european_any<BatesModel, SchemeNCI, NullVolScheme, MertonJump>(model, j, out);
  }
  if (is(j, 1, MYQL_SCHEME_NCI, 0, MYQL_JUMP_KOU)) {
    BatesKouModel model(hp(m.heston[0]), kp(m));
    return eur ? european_any<BatesKouModel, SchemeNCI, NullVolScheme, KouJump>(model, j, out)
               : exotic_any<BatesKouModel, SchemeNCI, NullVolScheme, KouJump>(model, j, out);
  }
  if (is(j, 2, MYQL_SCHEME_NCI, MYQL_SCHEME_NCI, MYQL_JUMP_NONE) && !eur) {
    DoubleHestonModel model(hp(m.heston[0]), hp(m.heston[1]));
    return exotic_any<DoubleHestonModel, SchemeNCI, SchemeNCI, NoJumps>(model, j, out);
  }
  if (is(j, 2, MYQL_SCHEME_NV, MYQL_SCHEME_NCI, MYQL_JUMP_MERTON) && !eur) {
    DoubleBatesModel model(hp(m.heston[0]), hp(m.heston[1]), mp(m));
    return exotic_any<DoubleBatesModel, SchemeNV, SchemeNCI, MertonJump>(model, j, out);
  }
  if (is(j, 2, MYQL_SCHEME_NV, MYQL_SCHEME_NV, MYQL_JUMP_KOU) && eur) {
    DoubleBatesKouModel model(hp(m.heston[0]), hp(m.heston[1]), kp(m));
    return european_any<DoubleBatesKouModel, SchemeNV, SchemeNV, KouJump>(model, j, out);
  }
  if (is(j, 0, 0, 0, MYQL_JUMP_NONE)) {
    BlackScholesModel model(m.vol);
    return eur ? european_any<BlackScholesModel, NullVolScheme, NullVolScheme, NoJumps>(model, j, out)
               : exotic_all<BlackScholesModel, NullVolScheme, NullVolScheme, NoJumps>(model, j, out);
  }
  return -2;
}

// The reference's FP64 Fourier (Gil-Pelaez) price and Greeks of a European
// vanilla call/put for the Heston family (tolerance as given).
int myql_ref_fourier(const myql_mc_job *jp, double tol, double *out) {
  if (!jp || !out) return -1;
  const myql_mc_job &j = *jp;
  const auto &m = j.model;
  FourierEngine::Config fc;
  fc.tolerance = tol;
  const double K = j.instrument.strikes[0], T = j.instrument.maturity;
  const bool call = j.instrument.option_type == MYQL_CALL;
  auto go = [&](const auto &model) {
    using Model = std::decay_t<decltype(model)>;
    auto one = [&](auto opt) {
      using Opt = decltype(opt);
      FourierPricer<Model, Opt, GreekMode::Full> pr(model, fc);
      const auto r = pr.calculate(j.S0, j.r, j.q, opt);
      const double v[MYQL_Q_COUNT] = {r.price, r.delta, r.gamma, r.vega[0], r.vega[1],
                                      r.theta, r.rho, r.vanna[0], r.vanna[1], r.charm};
      std::memcpy(out, v, sizeof v);
    };
    if (j.instrument.payoff == MYQL_PAYOFF_VANILLA) {
      if (call) one(EuropeanOption<CallV>(K, T)); else one(EuropeanOption<PutV>(K, T));
    } else if (j.instrument.payoff == MYQL_PAYOFF_CASH) {
      if (call) one(EuropeanOption<PayoffCashOrNothing<OptionType::Call>>(K, T));
      else one(EuropeanOption<PayoffCashOrNothing<OptionType::Put>>(K, T));
    } else {
      if (call) one(EuropeanOption<PayoffAssetOrNothing<OptionType::Call>>(K, T));
      else one(EuropeanOption<PayoffAssetOrNothing<OptionType::Put>>(K, T));
    }
  };
  const int nf = m.num_factors;
  if (nf == 0) {
    if (m.jump == MYQL_JUMP_NONE) go(BlackScholesModel(m.vol));
    else if (m.jump == MYQL_JUMP_MERTON) go(MertonModel(m.vol, mp(m)));
    else go(KouModel(m.vol, kp(m)));
  } else if (nf == 1) {
    if (m.jump == MYQL_JUMP_NONE) go(HestonModel(hp(m.heston[0])));
    else if (m.jump == MYQL_JUMP_MERTON) go(BatesModel(hp(m.heston[0]), mp(m)));
    else go(BatesKouModel(hp(m.heston[0]), kp(m)));
  } else {
    if (m.jump == MYQL_JUMP_NONE) go(DoubleHestonModel(hp(m.heston[0]), hp(m.heston[1])));
    else if (m.jump == MYQL_JUMP_MERTON) go(DoubleBatesModel(hp(m.heston[0]), hp(m.heston[1]), mp(m)));
    else go(DoubleBatesKouModel(hp(m.heston[0]), hp(m.heston[1]), kp(m)));
  }
  return 0;
}

}  // extern "C"
