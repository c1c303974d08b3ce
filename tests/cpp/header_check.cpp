// Drop-in header check: builds pricers with the reference's template
// signatures, prints the C-ABI requests they lower to (mode "lower"), or
// prices through the GPU (mode "price").
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "myql_gpu/MonteCarloPricer.hpp"

using namespace myql_gpu;

static void dump(const char *name, const myql_mc_job &j) {
  const myql_model &m = j.model;
  const myql_instrument &in = j.instrument;
  const myql_mc_config &c = j.config;
  std::printf("{\"name\": \"%s\", \"num_factors\": %d, \"jump\": %d, \"vol\": %.17g, "
              "\"h0\": [%.17g, %.17g, %.17g, %.17g, %.17g], \"h1\": [%.17g, %.17g, %.17g, %.17g, %.17g], "
              "\"jump_params\": [%.17g, %.17g, %.17g, %.17g, %.17g, %.17g], "
              "\"kind\": %d, \"payoff\": %d, \"option_type\": %d, \"fixed_strike\": %d, \"barrier_up\": %d, "
              "\"barrier_action\": %d, \"rebate_timing\": %d, \"is_strip\": %d, \"maturity\": %.17g, "
              "\"barrier\": %.17g, \"rebate\": %.17g, \"barrier_rate\": %.17g, \"payoff_eps\": %.17g, "
              "\"strikes\": [",
              name, m.num_factors, m.jump, m.vol, m.heston[0].kappa, m.heston[0].theta, m.heston[0].sigma,
              m.heston[0].rho, m.heston[0].v0, m.heston[1].kappa, m.heston[1].theta, m.heston[1].sigma,
              m.heston[1].rho, m.heston[1].v0, m.jump_lambda, m.merton_mu, m.merton_delta, m.kou_p_up, m.kou_eta1,
              m.kou_eta2, in.kind, in.payoff, in.option_type, in.fixed_strike, in.barrier_up, in.barrier_action,
              in.rebate_timing, in.is_strip, in.maturity, in.barrier, in.rebate, in.barrier_rate, in.payoff_eps);
  for (int64_t k = 0; k < in.n_strikes; ++k) std::printf("%s%.17g", k ? ", " : "", in.strikes[k]);
  std::printf("], \"history\": [%.17g, %.17g, %.17g, %.17g, %.17g], \"num_paths\": %llu, \"time_steps\": %llu, "
              "\"seed\": %llu, \"bumps\": [%.17g, %.17g, %.17g, %.17g], \"scheme\": [%d, %d], \"greek_mode\": %d, "
              "\"S0\": %.17g, \"r\": %.17g, \"q\": %.17g, \"valid\": %d}\n",
              in.past_avg_log, in.past_avg_S, in.t_elapsed, in.hist_min_S, in.hist_max_S,
              (unsigned long long)c.num_paths, (unsigned long long)c.time_steps, (unsigned long long)c.seed,
              c.fd_bump, c.vol_bump, c.t_bump, c.r_bump, c.scheme[0], c.scheme[1], c.greek_mode, j.S0, j.r, j.q,
              (int)myql_validate_job(&j));
}

int main(int argc, char **argv) {
  const std::string mode = argc > 1 ? argv[1] : "lower";
  const HestonParams h1{1.5, 0.04, 0.3, -0.7, 0.04};
  const HestonParams h2{3.0, 0.02, 0.2, -0.3, 0.02};
  MonteCarloConfig cfg;
  cfg.num_paths = 1u << 18;
  cfg.time_steps = 100;

  HestonModel heston(h1);
  using Eur = EuropeanOption<PayoffVanilla<OptionType::Call>>;
  MonteCarloPricer<HestonModel, HestonStepper<SchemeNV>, Eur, GreekMode::Essential> p1(heston, cfg);

  DoubleBatesKouModel dbk(h1, h2, KouParams{0.7, 0.4, 10.0, 5.0});
  using ArithPutStrip = AsianOption<TrackerArithAsian, PayoffVanilla<OptionType::Put>, false, std::vector<double>>;
  MonteCarloPricer<DoubleBatesKouModel, DoubleBatesKouStepper<SchemeNCI, SchemeExact, TrackerArithAsian>,
                   ArithPutStrip, GreekMode::Full>
      p2(dbk, cfg);

  BatesModel bates(h1, MertonParams{0.5, -0.1, 0.15});
  MonteCarloPricer<BatesModel, BatesStepper<SchemeExact, TrackerBarrier<true>>, UpAndOutCall<RebateTiming::AtHit>>
      p3(bates, cfg);

  MertonModel merton(0.2, MertonParams{1.0, -0.05, 0.1});
  using LbDigital = LookbackOption<PayoffCashOrNothing<OptionType::Call>, true>;
  MonteCarloPricer<MertonModel, MertonJDStepper<TrackerLookback>, LbDigital, GreekMode::Essential> p4(merton, cfg);

  MLMCConfig mcfg;
  mcfg.epsilon = 0.05;
  MultiLevelMonteCarloPricer<HestonModel, CoupledHestonStepper<SchemeNV, TrackerBarrier<false>>,
                             DownAndOutPut<>, GreekMode::Essential>
      mlmc(heston, mcfg);
  if (mode == "lower") {
    std::vector<double> s;
    dump("heston_eur", p1.job(100.0, 0.02, 0.0, Eur(100.0, 1.0), s));
    dump("dbk_asian_strip", p2.job(100.0, 0.03, 0.01, ArithPutStrip({90.0, 100.0, 110.0}, 2.0, 101.0, 4.6, 0.25), s));
    dump("bates_uo", p3.job(100.0, 0.02, 0.0, UpAndOutCall<RebateTiming::AtHit>(95.0, 130.0, 1.0, 0.02, 1.5), s));
    LbDigital lb(100.0, 1.0, 95.0, 104.0);
    lb.payoff_func_.eps = 0.5;
    dump("merton_lookback", p4.job(100.0, 0.02, 0.0, lb, s));
    return 0;
  }
  // price: the Heston call (FP64 Fourier price 8.628108103110)
  const auto r = p1.calculate(100.0, 0.02, 0.0, Eur(100.0, 1.0));
  std::printf("{\"price\": %.17g, \"price_std_err\": %.17g, \"delta\": %.17g, \"gamma\": %.17g, \"total_steps\": %zu}\n",
              r.price, r.price_std_err, r.delta, r.gamma, r.total_steps);
  const auto ml = mlmc.calculate(100.0, 0.02, 0.0, DownAndOutPut<>(100.0, 80.0, 1.0));
  std::printf("{\"mlmc_price\": %.17g, \"mlmc_se\": %.17g, \"mlmc_levels\": %zu, \"mlmc_delta\": %.17g}\n",
              ml.price, ml.price_std_err, ml.paths_per_level.size(), ml.delta);
  // precise theta (one-factor SchemeNCI, Full Greeks): the same price, a theta of its own
  {
    const HestonParams hn{2.0, 0.05, 0.9, -0.6, 0.05};
    BatesModel bn(hn, MertonParams{0.5, -0.1, 0.15});
    MonteCarloConfig fc;
    fc.num_paths = 1u << 16;
    fc.time_steps = 200;
    MonteCarloPricer<BatesModel, BatesStepper<SchemeNCI>, Eur, GreekMode::Full> pf(bn, fc);
    const auto a = pf.calculate(100.0, 0.02, 0.0, Eur(100.0, 1.0));
    set_precise_theta(true);
    const auto b = pf.calculate(100.0, 0.02, 0.0, Eur(100.0, 1.0));
    set_precise_theta(false);
    std::printf("{\"full_price\": [%.17g, %.17g], \"full_theta\": [%.17g, %.17g], \"theta_se\": %.17g}\n",
                a.price, b.price, a.theta, b.theta, a.theta_std_err);
  }
  // an invalid request surfaces as the reference's exception type
  try {
    HestonModel bad(HestonParams{1.5, 0.04, 0.9, -0.7, 0.04});
    MonteCarloPricer<HestonModel, HestonStepper<SchemeNV>, Eur> p(bad, cfg);
    p.calculate(100.0, 0.02, 0.0, Eur(100.0, 1.0));
    std::printf("{\"nv_error\": \"none\"}\n");
  } catch (const std::runtime_error &e) {
    std::printf("{\"nv_error\": \"runtime_error\"}\n");
  }
  return 0;
}
