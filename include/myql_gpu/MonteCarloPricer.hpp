// myql_gpu/MonteCarloPricer.hpp -- C++20 drop-in for MyQuantLib's Monte Carlo
// pricers on the GB300 engine.
//
// The types below carry the names, template parameters, constructors and
// result fields of the reference's public API:
//   HestonParams / NoJumpParams / MertonParams / KouParams   models/asvj/data/ModelParams.hpp:7-47
//   ZeroFactorModel / SingleFactorModel / DoubleFactorModel  models/asvj/core/ASVJmodel.hpp:14-87
//   NullVolScheme / SchemeNV / SchemeExact / SchemeNCI       models/asvj/policies/VolSchemes.hpp
//   NoJumps / MertonJump / KouJump                           models/asvj/policies/JumpPolicies.hpp
//   Tracker{European,GeoAsian,ArithAsian,Lookback,Barrier}   instruments/trackers/PathTrackers.hpp
//   ASVJStepper and its aliases                              models/asvj/core/ASVJstepper.hpp:18-340
//   CoupledASVJStepper aliases                               models/asvj/core/CoupledASVJStepper.hpp:577-617
//   Payoff{Vanilla,CashOrNothing,AssetOrNothing}             instruments/Payoffs.hpp:14-69
//   EuropeanOption / AsianOption / LookbackOption / BarrierOption   instruments/options/*.hpp
//   GreekMode, MonteCarloResult, MlmcResult                  core/PricingTypes.hpp
//   MonteCarloConfig, MonteCarloPricer (RNG parameter too)   pricers/montecarlo/MonteCarloPricer.hpp:16-96
//   MLMCConfig, MultiLevelMonteCarloPricer                   pricers/mlmc/MultiLevelMonteCarloPricer.hpp:16-47
// so that user code switches by namespace (myql_gpu::) and include.  Every
// calculate() lowers its template arguments to a myql_mc_job (include/myql_gpu.h)
// and runs on the GPU; errors surface as exceptions like the reference's
// (std::runtime_error, std::invalid_argument for bad parameters).  The policy
// types are tags: the computation lives in the CUDA library.
//
// Contexts: one engine context per host thread and device, created on first
// use (device 0 unless myql_gpu::set_device() was called on that thread).
#pragma once
#include <array>
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "../myql_gpu.h"

// The reference's pricers take the random engine as a template parameter
// (MonteCarloPricer.hpp:86, MultiLevelMonteCarloPricer.hpp:37), spelled
// boost::random::xoshiro256pp.  Where Boost's header is present the drop-in
// accepts that type too.
#if __has_include(<boost/random/xoshiro.hpp>)
#include <boost/random/xoshiro.hpp>
#define MYQL_GPU_HAVE_BOOST_XOSHIRO 1
#endif

namespace myql_gpu {

// ---------------------------------------------------------------- random engine
// The GPU engine always draws xoshiro256++ streams: stream k of seed s is the
// generator seeded with s (splitmix64 expansion) advanced by k jumps of 2^128.
// The RNG template parameter of the pricers is kept for source compatibility and
// must name a xoshiro256++ engine: this tag or Boost's.
struct xoshiro256pp {};
template <typename RNG> struct is_xoshiro256pp : std::false_type {};
template <> struct is_xoshiro256pp<xoshiro256pp> : std::true_type {};
#ifdef MYQL_GPU_HAVE_BOOST_XOSHIRO
template <> struct is_xoshiro256pp<boost::random::xoshiro256pp> : std::true_type {};
#endif

// ---------------------------------------------------------------- core types
enum class GreekMode { None, Essential, Full };
enum class OptionType { Call, Put };
enum class BarrierDirection { Up, Down };
enum class BarrierAction { In, Out };
enum class RebateTiming { None, AtHit, AtMaturity };

template <GreekMode Mode, typename T> struct MonteCarloResult;
template <typename T> struct MonteCarloResult<GreekMode::None, T> {
  T price;
  T price_std_err;
  size_t total_steps{};
};
template <typename T> struct MonteCarloResult<GreekMode::Essential, T> {
  T price;
  T price_std_err;
  T delta;
  T delta_std_err;
  T gamma;
  T gamma_std_err;
  size_t total_steps{};
};
template <typename T> struct MonteCarloResult<GreekMode::Full, T> {
  T price;
  T price_std_err;
  T delta;
  T delta_std_err;
  T gamma;
  T gamma_std_err;
  std::array<T, 2> vega{};
  std::array<T, 2> vega_std_err{};
  T theta;
  T theta_std_err;
  T rho;
  T rho_std_err;
  std::array<T, 2> vanna{};
  std::array<T, 2> vanna_std_err{};
  T charm;
  T charm_std_err;
  size_t total_steps{};
};

// MLMC results: the Greek fields exist for Essential / Full as in the reference, whose MLMC
// pricer computes prices only (the bumped payoffs of calculate_to_buffer are discarded,
// MultiLevelMonteCarloPricer.hpp:278-283, 320-326), so they stay zero there and here.
template <typename T> struct MlmcLevels {
  size_t total_steps{};
  std::vector<size_t> paths_per_level{};
  std::vector<T> mean_diffs{};
  std::vector<T> var_diffs{};
  double alpha_estimated{};
  double beta_estimated{};
};
template <GreekMode Mode, typename T> struct MlmcResult;
template <typename T> struct MlmcResult<GreekMode::None, T> : MlmcLevels<T> {
  T price{};
  T price_std_err{};
};
template <typename T> struct MlmcResult<GreekMode::Essential, T> : MlmcLevels<T> {
  T price{};
  T price_std_err{};
  T delta{};
  T delta_std_err{};
  T gamma{};
  T gamma_std_err{};
};
template <typename T> struct MlmcResult<GreekMode::Full, T> : MlmcLevels<T> {
  T price{};
  T price_std_err{};
  T delta{};
  T delta_std_err{};
  T gamma{};
  T gamma_std_err{};
  std::array<T, 2> vega{};
  std::array<T, 2> vega_std_err{};
  T theta{};
  T theta_std_err{};
  T rho{};
  T rho_std_err{};
  std::array<T, 2> vanna{};
  std::array<T, 2> vanna_std_err{};
  T charm{};
  T charm_std_err{};
};

// ---------------------------------------------------------------- model parameters
struct HestonParams {
  double kappa;
  double theta;
  double sigma;
  double rho;
  double v0;
  bool is_low_vol_regime() const { return sigma * sigma <= 4.0 * kappa * theta; }
  bool is_Feller_regime() const { return sigma * sigma <= 2.0 * kappa * theta; }
};
struct NoJumpParams {};
struct MertonParams {
  double lambda;
  double mu;
  double delta;
};
struct KouParams {
  double lambda;
  double p_up;
  double eta1;
  double eta2;
};

template <typename JumpParamType = NoJumpParams> struct ZeroFactorModel {
  static constexpr int num_variance_factors = 0;
  double vol;
  JumpParamType jump;
  ZeroFactorModel(double v, const JumpParamType &j = JumpParamType{}) : vol(v), jump(j) {}
};
template <typename JumpParamType> struct SingleFactorModel {
  static constexpr int num_variance_factors = 1;
  HestonParams heston;
  JumpParamType jump;
  SingleFactorModel(const HestonParams &h, const JumpParamType &j = JumpParamType()) : heston(h), jump(j) {}
};
template <typename JumpParamType> struct DoubleFactorModel {
  static constexpr int num_variance_factors = 2;
  HestonParams heston1;
  HestonParams heston2;
  JumpParamType jump;
  DoubleFactorModel(const HestonParams &h1, const HestonParams &h2, const JumpParamType &j = JumpParamType())
      : heston1(h1), heston2(h2), jump(j) {}
};
using BlackScholesModel = ZeroFactorModel<NoJumpParams>;
using MertonModel = ZeroFactorModel<MertonParams>;
using KouModel = ZeroFactorModel<KouParams>;
using HestonModel = SingleFactorModel<NoJumpParams>;
using BatesModel = SingleFactorModel<MertonParams>;
using BatesKouModel = SingleFactorModel<KouParams>;
using DoubleHestonModel = DoubleFactorModel<NoJumpParams>;
using DoubleBatesModel = DoubleFactorModel<MertonParams>;
using DoubleBatesKouModel = DoubleFactorModel<KouParams>;

// ---------------------------------------------------------------- policies (tags)
struct NullVolScheme { static constexpr int code = MYQL_SCHEME_NONE; };
struct SchemeNV { static constexpr int code = MYQL_SCHEME_NV; };
struct SchemeExact { static constexpr int code = MYQL_SCHEME_EXACT; };
struct SchemeNCI { static constexpr int code = MYQL_SCHEME_NCI; };

struct NoJumps { using Params = NoJumpParams; };
struct MertonJump { using Params = MertonParams; };
struct KouJump { using Params = KouParams; };

struct TrackerEuropean {};
struct TrackerGeoAsian {};
struct TrackerArithAsian {};
struct TrackerLookback {};
template <bool IsUpBarrier> struct TrackerBarrier {};

template <typename VolScheme1, typename VolScheme2 = NullVolScheme, typename JumpPolicy = NoJumps,
          typename TrackerPolicy = TrackerEuropean>
struct ASVJStepper {
  static constexpr int NumCirs =
      std::is_same_v<VolScheme1, NullVolScheme> ? 0 : (std::is_same_v<VolScheme2, NullVolScheme> ? 1 : 2);
  using Scheme1 = VolScheme1;
  using Scheme2 = VolScheme2;
  using Jump = JumpPolicy;
  using Tracker = TrackerPolicy;
};
template <typename Tracker = TrackerEuropean>
using BlackScholesStepper = ASVJStepper<NullVolScheme, NullVolScheme, NoJumps, Tracker>;
template <typename Tracker = TrackerEuropean>
using MertonJDStepper = ASVJStepper<NullVolScheme, NullVolScheme, MertonJump, Tracker>;
template <typename Tracker = TrackerEuropean>
using KouJDStepper = ASVJStepper<NullVolScheme, NullVolScheme, KouJump, Tracker>;
template <typename VolScheme, typename Tracker = TrackerEuropean>
using HestonStepper = ASVJStepper<VolScheme, NullVolScheme, NoJumps, Tracker>;
template <typename VolScheme, typename Tracker = TrackerEuropean>
using BatesStepper = ASVJStepper<VolScheme, NullVolScheme, MertonJump, Tracker>;
template <typename VolScheme, typename Tracker = TrackerEuropean>
using BatesKouStepper = ASVJStepper<VolScheme, NullVolScheme, KouJump, Tracker>;
template <typename VolScheme1, typename VolScheme2, typename Tracker = TrackerEuropean>
using DoubleHestonStepper = ASVJStepper<VolScheme1, VolScheme2, NoJumps, Tracker>;
template <typename VolScheme1, typename VolScheme2, typename Tracker = TrackerEuropean>
using DoubleBatesStepper = ASVJStepper<VolScheme1, VolScheme2, MertonJump, Tracker>;
template <typename VolScheme1, typename VolScheme2, typename Tracker = TrackerEuropean>
using DoubleBatesKouStepper = ASVJStepper<VolScheme1, VolScheme2, KouJump, Tracker>;

// coupled (MLMC) steppers: the same tags; the engine builds the coupled pair
template <typename VolScheme1, typename VolScheme2 = NullVolScheme, typename JumpPolicy = NoJumps,
          typename TrackerPolicy = TrackerEuropean>
using CoupledASVJStepper = ASVJStepper<VolScheme1, VolScheme2, JumpPolicy, TrackerPolicy>;
template <typename Tracker = TrackerEuropean> using CoupledBlackScholesStepper = BlackScholesStepper<Tracker>;
template <typename Tracker = TrackerEuropean> using CoupledMertonJDStepper = MertonJDStepper<Tracker>;
template <typename Tracker = TrackerEuropean> using CoupledKouJDStepper = KouJDStepper<Tracker>;
template <typename VolScheme, typename Tracker = TrackerEuropean>
using CoupledHestonStepper = HestonStepper<VolScheme, Tracker>;
template <typename VolScheme, typename Tracker = TrackerEuropean>
using CoupledBatesStepper = BatesStepper<VolScheme, Tracker>;
template <typename VolScheme, typename Tracker = TrackerEuropean>
using CoupledBatesKouStepper = BatesKouStepper<VolScheme, Tracker>;
template <typename V1, typename V2, typename Tracker = TrackerEuropean>
using CoupledDoubleHestonStepper = DoubleHestonStepper<V1, V2, Tracker>;
template <typename V1, typename V2, typename Tracker = TrackerEuropean>
using CoupledDoubleBatesStepper = DoubleBatesStepper<V1, V2, Tracker>;
template <typename V1, typename V2, typename Tracker = TrackerEuropean>
using CoupledDoubleBatesKouStepper = DoubleBatesKouStepper<V1, V2, Tracker>;

// ---------------------------------------------------------------- payoffs
template <OptionType OT> struct PayoffVanilla {
  static constexpr OptionType Type = OT;
  static constexpr int code = MYQL_PAYOFF_VANILLA;
  double eps = -1.0;  // unused by vanilla payoffs
};
template <OptionType OT> struct PayoffCashOrNothing {
  static constexpr OptionType Type = OT;
  static constexpr int code = MYQL_PAYOFF_CASH;
  double eps = -1.0;  // smoothing bandwidth (-1: automatic when GreekMode != None)
};
template <OptionType OT> struct PayoffAssetOrNothing {
  static constexpr OptionType Type = OT;
  static constexpr int code = MYQL_PAYOFF_ASSET;
  double eps = -1.0;
};

// ---------------------------------------------------------------- instruments
namespace detail {
template <typename C> struct is_strip : std::false_type {};
template <> struct is_strip<std::vector<double>> : std::true_type {};
template <typename C> std::vector<double> strikes_of(const C &k) {
  if constexpr (is_strip<C>::value) return k;
  else return std::vector<double>{k};
}
}  // namespace detail

template <typename PayoffPolicy, typename StrikeContainer = double> class EuropeanOption {
 public:
  using Tracker = TrackerEuropean;
  using ResultType = StrikeContainer;
  using PayoffType = PayoffPolicy;
  EuropeanOption(const StrikeContainer &K, double T, const PayoffPolicy &payoff = PayoffPolicy())
      : strikes_(K), T_(T), payoff_func_(payoff) {}
  double get_maturity() const { return T_; }
  void lower(myql_instrument &in) const {
    in.kind = MYQL_INSTR_EUROPEAN;
    in.fixed_strike = 1;  // a strike-vs-terminal payoff
    in.payoff = PayoffPolicy::code;
    in.option_type = PayoffPolicy::Type == OptionType::Call ? MYQL_CALL : MYQL_PUT;
    in.payoff_eps = payoff_func_.eps;
  }
  StrikeContainer strikes_;
  double T_;
  PayoffPolicy payoff_func_;
};

template <typename TrackerT, typename PayoffT, bool FixedStrike, typename StrikeContainer = double>
class AsianOption {
 public:
  using Tracker = TrackerT;
  using ResultType = StrikeContainer;
  using PayoffType = PayoffT;
  AsianOption(const StrikeContainer &K, double T, const PayoffT &payoff = PayoffT())
      : strikes_(K), T_(T), payoff_func_(payoff) {}
  AsianOption(const StrikeContainer &K, double T, double past_avg_log, double t_elapsed,
              const PayoffT &payoff = PayoffT())
      : strikes_(K), T_(T), payoff_func_(payoff), past_avg_log_(past_avg_log), t_elapsed_(t_elapsed) {}
  AsianOption(const StrikeContainer &K, double T, double past_avg_S, double past_avg_log, double t_elapsed,
              const PayoffT &payoff = PayoffT())
      : strikes_(K), T_(T), payoff_func_(payoff), past_avg_log_(past_avg_log), past_avg_S_(past_avg_S),
        t_elapsed_(t_elapsed) {}
  double get_maturity() const { return T_; }
  void lower(myql_instrument &in) const {
    in.kind = std::is_same_v<TrackerT, TrackerGeoAsian> ? MYQL_INSTR_ASIAN_GEO : MYQL_INSTR_ASIAN_ARITH;
    in.payoff = PayoffT::code;
    in.option_type = PayoffT::Type == OptionType::Call ? MYQL_CALL : MYQL_PUT;
    in.payoff_eps = payoff_func_.eps;
    in.fixed_strike = FixedStrike ? 1 : 0;
    in.past_avg_log = past_avg_log_;
    in.past_avg_S = past_avg_S_;
    in.t_elapsed = t_elapsed_;
  }
  StrikeContainer strikes_;
  double T_;
  PayoffT payoff_func_;
  double past_avg_log_ = 0.0, past_avg_S_ = 0.0, t_elapsed_ = 0.0;
};

template <typename PayoffT, bool FixedStrike, typename StrikeContainer = double> class LookbackOption {
 public:
  using Tracker = TrackerLookback;
  using ResultType = StrikeContainer;
  using PayoffType = PayoffT;
  LookbackOption(const StrikeContainer &K, double T, double hist_min_S = 0.0, double hist_max_S = 0.0,
                 const PayoffT &payoff = PayoffT())
      : strikes_(K), T_(T), payoff_func_(payoff), hist_min_S_(hist_min_S), hist_max_S_(hist_max_S) {}
  double get_maturity() const { return T_; }
  void lower(myql_instrument &in) const {
    in.kind = MYQL_INSTR_LOOKBACK;
    in.payoff = PayoffT::code;
    in.option_type = PayoffT::Type == OptionType::Call ? MYQL_CALL : MYQL_PUT;
    in.payoff_eps = payoff_func_.eps;
    in.fixed_strike = FixedStrike ? 1 : 0;
    in.hist_min_S = hist_min_S_;
    in.hist_max_S = hist_max_S_;
  }
  StrikeContainer strikes_;
  double T_;
  PayoffT payoff_func_;
  double hist_min_S_, hist_max_S_;
};

template <typename PayoffT, BarrierDirection Dir, BarrierAction Action, RebateTiming Timing,
          typename StrikeContainer = double>
class BarrierOption {
 public:
  using Tracker = TrackerBarrier<Dir == BarrierDirection::Up>;
  using ResultType = StrikeContainer;
  using PayoffType = PayoffT;
  BarrierOption(const StrikeContainer &K, double B, double T, double r = 0.0, double rebate = 0.0,
                const PayoffT &payoff = PayoffT())
      : strikes_(K), barrier_(B), T_(T), rate_(r), rebate_(rebate), payoff_func_(payoff) {}
  double get_maturity() const { return T_; }
  void lower(myql_instrument &in) const {
    in.kind = MYQL_INSTR_BARRIER;
    in.fixed_strike = 1;
    in.payoff = PayoffT::code;
    in.option_type = PayoffT::Type == OptionType::Call ? MYQL_CALL : MYQL_PUT;
    in.payoff_eps = payoff_func_.eps;
    in.barrier_up = Dir == BarrierDirection::Up ? 1 : 0;
    in.barrier_action = Action == BarrierAction::Out ? MYQL_BARRIER_OUT : MYQL_BARRIER_IN;
    in.rebate_timing = Timing == RebateTiming::None    ? MYQL_REBATE_NONE
                       : Timing == RebateTiming::AtHit ? MYQL_REBATE_AT_HIT
                                                       : MYQL_REBATE_AT_MATURITY;
    in.barrier = barrier_;
    in.rebate = rebate_;
    in.barrier_rate = rate_;
  }
  StrikeContainer strikes_;
  double barrier_, T_, rate_, rebate_;
  PayoffT payoff_func_;
};

#define MYQL_GPU_BARRIER_ALIAS(NAME, OT, DIR, ACT)                                        \
  template <RebateTiming Timing = RebateTiming::None>                                     \
  using NAME = BarrierOption<PayoffVanilla<OptionType::OT>, BarrierDirection::DIR, BarrierAction::ACT, Timing>;
MYQL_GPU_BARRIER_ALIAS(UpAndOutCall, Call, Up, Out)
MYQL_GPU_BARRIER_ALIAS(UpAndOutPut, Put, Up, Out)
MYQL_GPU_BARRIER_ALIAS(UpAndInCall, Call, Up, In)
MYQL_GPU_BARRIER_ALIAS(UpAndInPut, Put, Up, In)
MYQL_GPU_BARRIER_ALIAS(DownAndOutCall, Call, Down, Out)
MYQL_GPU_BARRIER_ALIAS(DownAndOutPut, Put, Down, Out)
MYQL_GPU_BARRIER_ALIAS(DownAndInCall, Call, Down, In)
MYQL_GPU_BARRIER_ALIAS(DownAndInPut, Put, Down, In)
#undef MYQL_GPU_BARRIER_ALIAS

// ---------------------------------------------------------------- configs
struct MonteCarloConfig {
  size_t num_paths = 100000;
  size_t time_steps = 100;
  unsigned long seed = 42;
  double fd_bump = 1e-4;
  double vol_bump = 1e-4;
  double t_bump = 1e-4;
  double r_bump = 1e-4;
};

struct MLMCConfig {
  double epsilon = 0.005;
  size_t L_min = 2;
  size_t L_max = 15;
  size_t N0 = 10000;
  size_t base_steps = 1;
  double alpha = 2.0;
  double beta = 1.0;
  bool adaptive_rates = true;
  unsigned long seed = 42;
  double fd_bump = 1e-4;
};

// ---------------------------------------------------------------- engine context
namespace detail {
inline int &thread_device() {
  thread_local int dev = 0;
  return dev;
}
// The SchemeNCI table mode of this thread's pricers: applied to every context the
// thread creates, so a later set_device() keeps it.
inline bool &thread_exact_nci() {
  thread_local bool on = false;
  return on;
}
// The precise-theta mode of this thread's pricers, kept the same way.
inline bool &thread_precise_theta() {
  thread_local bool on = false;
  return on;
}
struct ThreadCtx {
  myql_ctx *ctx = nullptr;
  int device = -1;
  ~ThreadCtx() {
    if (ctx) myql_ctx_destroy(ctx);
  }
};
[[noreturn]] inline void raise(myql_status s) {
  char buf[512];
  myql_last_error(buf, sizeof buf);
  const std::string msg = std::string("myql_gpu: ") + buf;
  if (s == MYQL_ERR_INVALID_ARG || s == MYQL_ERR_TOO_LARGE) throw std::invalid_argument(msg);
  throw std::runtime_error(msg);
}
inline myql_ctx *context() {
  thread_local ThreadCtx tc;
  const int dev = thread_device();
  if (!tc.ctx || tc.device != dev) {
    if (tc.ctx) myql_ctx_destroy(tc.ctx);
    tc.ctx = nullptr;
    myql_status s = myql_ctx_create(&tc.ctx, dev);
    if (s != MYQL_OK) raise(s);
    tc.device = dev;
    if (thread_exact_nci()) {
      s = myql_ctx_set_nci_slopes(tc.ctx, 1);
      if (s != MYQL_OK) raise(s);
    }
    if (thread_precise_theta()) {
      s = myql_ctx_set_precise_theta(tc.ctx, 1);
      if (s != MYQL_OK) raise(s);
    }
  }
  return tc.ctx;
}

inline void lower_heston(myql_heston_params &o, const HestonParams &h) {
  o.kappa = h.kappa;
  o.theta = h.theta;
  o.sigma = h.sigma;
  o.rho = h.rho;
  o.v0 = h.v0;
}
template <typename J> void lower_jump(myql_model &m, const J &j) {
  if constexpr (std::is_same_v<J, MertonParams>) {
    m.jump = MYQL_JUMP_MERTON;
    m.jump_lambda = j.lambda;
    m.merton_mu = j.mu;
    m.merton_delta = j.delta;
  } else if constexpr (std::is_same_v<J, KouParams>) {
    m.jump = MYQL_JUMP_KOU;
    m.jump_lambda = j.lambda;
    m.kou_p_up = j.p_up;
    m.kou_eta1 = j.eta1;
    m.kou_eta2 = j.eta2;
  } else {
    m.jump = MYQL_JUMP_NONE;
  }
}
template <typename J> void lower_model(myql_model &m, const ZeroFactorModel<J> &x) {
  m.num_factors = 0;
  m.vol = x.vol;
  lower_jump(m, x.jump);
}
template <typename J> void lower_model(myql_model &m, const SingleFactorModel<J> &x) {
  m.num_factors = 1;
  lower_heston(m.heston[0], x.heston);
  lower_jump(m, x.jump);
}
template <typename J> void lower_model(myql_model &m, const DoubleFactorModel<J> &x) {
  m.num_factors = 2;
  lower_heston(m.heston[0], x.heston1);
  lower_heston(m.heston[1], x.heston2);
  lower_jump(m, x.jump);
}
template <typename M> struct jump_params_of;
template <typename J> struct jump_params_of<ZeroFactorModel<J>> { using type = J; };
template <typename J> struct jump_params_of<SingleFactorModel<J>> { using type = J; };
template <typename J> struct jump_params_of<DoubleFactorModel<J>> { using type = J; };

// The whole request; `strikes` must outlive the job.
template <typename Model, typename Stepper, typename Instrument>
myql_mc_job lower_job(const Model &model, const Instrument &instr, GreekMode mode, size_t paths, size_t steps,
                      unsigned long seed, double fd_bump, double vol_bump, double t_bump, double r_bump, double S0,
                      double r, double q, const std::vector<double> &strikes) {
  static_assert(Stepper::NumCirs == Model::num_variance_factors,
                "the stepper's CIR factors must match the model's variance factors");
  static_assert(std::is_same_v<typename Stepper::Jump::Params, typename jump_params_of<Model>::type>,
                "the stepper's jump policy must match the model's jump parameters");
  static_assert(std::is_same_v<typename Stepper::Tracker, typename Instrument::Tracker>,
                "the stepper's tracker must match the instrument's");
  myql_mc_job job;
  std::memset(&job, 0, sizeof job);
  lower_model(job.model, model);
  instr.lower(job.instrument);
  job.instrument.is_strip = is_strip<typename Instrument::ResultType>::value ? 1 : 0;
  job.instrument.maturity = instr.get_maturity();
  job.instrument.strikes = strikes.data();
  job.instrument.n_strikes = (int64_t)strikes.size();
  job.config.num_paths = paths;
  job.config.time_steps = steps;
  job.config.seed = seed;
  job.config.fd_bump = fd_bump;
  job.config.vol_bump = vol_bump;
  job.config.t_bump = t_bump;
  job.config.r_bump = r_bump;
  job.config.scheme[0] = Stepper::Scheme1::code;
  job.config.scheme[1] = Stepper::Scheme2::code;
  job.config.greek_mode = mode == GreekMode::None ? MYQL_GREEKS_NONE
                          : mode == GreekMode::Essential ? MYQL_GREEKS_ESSENTIAL
                                                         : MYQL_GREEKS_FULL;
  job.S0 = S0;
  job.r = r;
  job.q = q;
  return job;
}

template <typename T> T pick(const std::vector<double> &out, int q, int se, size_t n) {
  const double *row = out.data() + (size_t)(2 * q + se) * n;
  if constexpr (std::is_same_v<T, double>) return row[0];
  else return T(row, row + n);
}
}  // namespace detail

// Selects the GPU the calling thread's pricers run on.
inline void set_device(int device) { detail::thread_device() = device; }

// SchemeNCI table cells of this thread's pricers: false (default) the reference's
// (VolSchemes.hpp:240-313), true cells that keep the exact chi-squared mean (the
// reference's first cell shortens it, which long, finely stepped paths turn into a
// price bias; see myql_ctx_set_nci_slopes).  The choice holds for the calling
// thread, across set_device(): every context the thread creates applies it.
inline void set_exact_nci_tables(bool on) {
  detail::thread_exact_nci() = on;
  const myql_status s = myql_ctx_set_nci_slopes(detail::context(), on ? 1 : 0);
  if (s != MYQL_OK) detail::raise(s);
}

// Theta and charm of this thread's one-factor SchemeNCI Full-Greek European pricers:
// false (default) every scenario in plain FP32 constants, true the T-bumped scenarios
// with their constants' FP32 rounding errors added back (see myql_ctx_set_precise_theta).
// The choice holds for the calling thread, across set_device().
inline void set_precise_theta(bool on) {
  detail::thread_precise_theta() = on;
  const myql_status s = myql_ctx_set_precise_theta(detail::context(), on ? 1 : 0);
  if (s != MYQL_OK) detail::raise(s);
}

// ---------------------------------------------------------------- pricers
template <typename Model, typename Stepper, typename Instrument, GreekMode Mode = GreekMode::None,
          typename RNG = xoshiro256pp>
class MonteCarloPricer {
  static_assert(is_xoshiro256pp<RNG>::value,
                "the GPU engine draws xoshiro256++ streams: RNG must be xoshiro256pp");

 public:
  using ResultType = typename Instrument::ResultType;
  using ReturnStruct = MonteCarloResult<Mode, ResultType>;

  MonteCarloPricer(const Model &model, const MonteCarloConfig &cfg) : model_(model), cfg_(cfg) {}

  // The request this pricer sends for (S0, r, q, instr); `strikes` keeps the strike storage alive.
  myql_mc_job job(double S0, double r, double q, const Instrument &instr, std::vector<double> &strikes) const {
    strikes = detail::strikes_of(instr.strikes_);
    return detail::lower_job<Model, Stepper, Instrument>(model_, instr, Mode, cfg_.num_paths, cfg_.time_steps,
                                                         cfg_.seed, cfg_.fd_bump, cfg_.vol_bump, cfg_.t_bump,
                                                         cfg_.r_bump, S0, r, q, strikes);
  }

  ReturnStruct calculate(double S0, double r, double q, const Instrument &instr) const {
    std::vector<double> strikes;
    const myql_mc_job jb = job(S0, r, q, instr, strikes);
    const size_t n = strikes.size();
    std::vector<double> out(MYQL_OUT_DOUBLES(n));
    myql_mc_stats st;
    const myql_status s = myql_mc_price(detail::context(), &jb, out.data(), &st);
    if (s != MYQL_OK) detail::raise(s);
    using T = ResultType;
    ReturnStruct res{};
    res.price = detail::pick<T>(out, MYQL_Q_PRICE, 0, n);
    res.price_std_err = detail::pick<T>(out, MYQL_Q_PRICE, 1, n);
    if constexpr (Mode != GreekMode::None) {
      res.delta = detail::pick<T>(out, MYQL_Q_DELTA, 0, n);
      res.delta_std_err = detail::pick<T>(out, MYQL_Q_DELTA, 1, n);
      res.gamma = detail::pick<T>(out, MYQL_Q_GAMMA, 0, n);
      res.gamma_std_err = detail::pick<T>(out, MYQL_Q_GAMMA, 1, n);
    }
    if constexpr (Mode == GreekMode::Full) {
      res.vega = {detail::pick<T>(out, MYQL_Q_VEGA0, 0, n), detail::pick<T>(out, MYQL_Q_VEGA1, 0, n)};
      res.vega_std_err = {detail::pick<T>(out, MYQL_Q_VEGA0, 1, n), detail::pick<T>(out, MYQL_Q_VEGA1, 1, n)};
      res.theta = detail::pick<T>(out, MYQL_Q_THETA, 0, n);
      res.theta_std_err = detail::pick<T>(out, MYQL_Q_THETA, 1, n);
      res.rho = detail::pick<T>(out, MYQL_Q_RHO, 0, n);
      res.rho_std_err = detail::pick<T>(out, MYQL_Q_RHO, 1, n);
      res.vanna = {detail::pick<T>(out, MYQL_Q_VANNA0, 0, n), detail::pick<T>(out, MYQL_Q_VANNA1, 0, n)};
      res.vanna_std_err = {detail::pick<T>(out, MYQL_Q_VANNA0, 1, n), detail::pick<T>(out, MYQL_Q_VANNA1, 1, n)};
      res.charm = detail::pick<T>(out, MYQL_Q_CHARM, 0, n);
      res.charm_std_err = detail::pick<T>(out, MYQL_Q_CHARM, 1, n);
    }
    res.total_steps = (size_t)st.path_steps;
    return res;
  }

 private:
  const Model &model_;  // held by reference, as the reference's pricer does
  MonteCarloConfig cfg_;
};

template <typename Model, typename CoupledStepperType, typename Instrument, GreekMode Mode = GreekMode::None,
          typename RNG = xoshiro256pp>
class MultiLevelMonteCarloPricer {
  static_assert(is_xoshiro256pp<RNG>::value,
                "the GPU engine draws xoshiro256++ streams: RNG must be xoshiro256pp");

 public:
  using ResultType = typename Instrument::ResultType;
  using ReturnStruct = MlmcResult<Mode, ResultType>;
  static_assert(std::is_same_v<ResultType, double>, "MLMC prices scalar instruments");

  MultiLevelMonteCarloPricer(const Model &model, const MLMCConfig &cfg) : model_(model), cfg_(cfg) {}

  ReturnStruct calculate(double S0, double r, double q, const Instrument &instr) const {
    std::vector<double> strikes = detail::strikes_of(instr.strikes_);
    const myql_mc_job jb = detail::lower_job<Model, CoupledStepperType, Instrument>(
        model_, instr, GreekMode::None, cfg_.N0, cfg_.base_steps, cfg_.seed, cfg_.fd_bump, 1e-4, 1e-4, 1e-4, S0, r,
        q, strikes);
    myql_mlmc_config mc;
    std::memset(&mc, 0, sizeof mc);
    mc.epsilon = cfg_.epsilon;
    mc.L_min = cfg_.L_min;
    mc.L_max = cfg_.L_max;
    mc.N0 = cfg_.N0;
    mc.base_steps = cfg_.base_steps;
    mc.alpha = cfg_.alpha;
    mc.beta = cfg_.beta;
    mc.adaptive_rates = cfg_.adaptive_rates ? 1 : 0;
    mc.seed = cfg_.seed;
    mc.fd_bump = cfg_.fd_bump;
    myql_mlmc_result out;
    const myql_status s = myql_mlmc_price(detail::context(), &jb, &mc, &out);
    if (s != MYQL_OK) detail::raise(s);
    ReturnStruct res{};
    res.price = out.price;
    res.price_std_err = out.price_std_err;
    res.total_steps = (size_t)out.total_steps;
    for (uint32_t l = 0; l < out.n_levels; ++l) {
      res.paths_per_level.push_back((size_t)out.paths_per_level[l]);
      res.mean_diffs.push_back(out.mean_diffs[l]);
      res.var_diffs.push_back(out.var_diffs[l]);
    }
    res.alpha_estimated = out.alpha_estimated;
    res.beta_estimated = out.beta_estimated;
    return res;
  }

 private:
  const Model &model_;
  MLMCConfig cfg_;
};

}  // namespace myql_gpu
