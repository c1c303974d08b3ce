// mlmc.cu -- host controller of the multilevel Monte Carlo pricer.
//
// Restates MultiLevelMonteCarloPricer::calculate
// (include/myql/pricers/mlmc/MultiLevelMonteCarloPricer.hpp:46-241): Giles'
// adaptive scheme with pilot samples N0 / 2^l (at least 20), the optimal
// allocation N_l = ceil(2 eps^-2 sqrt(V_l / C_l) sum_k sqrt(V_k C_k)),
// regression estimates of the weak/strong orders over the last three levels,
// and the bias test with the zero-crossing guard.  Every evaluate_level call is
// one launch of mlmc_level_kernel over a persistent pool of xoshiro streams
// that lives for the whole calculate() (the reference's rng_pool, :55-61).
#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <vector>

#include "cv.cuh"
#include "engine.h"
#include "mlmc.cuh"

namespace myql {

myql_status cv_level_eval(CtxBase *ctx, MlmcCvParams &Q, int klass, uint64_t dN, double *sums4);
myql_status cv_feat_consts(const myql_mc_job &job, const Plan &pl, const ScenarioConst &sc, double dt,
                           CvFeatConsts &F);

cudaError_t launch_mlmc_f01(const MlmcParams &M, int s1, bool pd, cudaStream_t st);
cudaError_t launch_mlmc_f2(const MlmcParams &M, int s1, int s2, bool pd, cudaStream_t st);

cudaError_t launch_mlmc_level(const MlmcParams &M, int s1, int s2, bool path_dep, cudaStream_t st) {
  if (M.sim.n_factors == 2) return launch_mlmc_f2(M, s1, s2, path_dep, st);
  return launch_mlmc_f01(M, s1, path_dep, st);
}

namespace {

// Scenario constants of one MLMC time step (fine or coarse) for the planned job.
void level_consts(const myql_mc_job &job, const Plan &pl, double dt, int n_steps, double T,
                  ScenarioConst &C) {
  const myql_model &m = job.model;
  std::memset(&C, 0, sizeof C);
  C.dt = (float)dt;
  C.t_end = (float)(dt * n_steps);
  if (pl.nf == 0) {
    const double drift_dt = (job.r - job.q - 0.5 * m.vol * m.vol) * dt;
    const double vol_dt = m.vol * std::sqrt(dt);
    if (!pl.path_dep) {
      C.gbm_drift = (float)(drift_dt * n_steps);
      C.gbm_vol = (float)(vol_dt * std::sqrt((double)n_steps));
    } else {
      C.gbm_drift = (float)drift_dt;
      C.gbm_vol = (float)vol_dt;
    }
  } else {
    const double r_part = (job.r - job.q) / (double)pl.nf;
    for (int f = 0; f < pl.nf; ++f)
      fill_factor(C.f[f], m.heston[f], m.heston[f].v0, job.config.scheme[f], r_part, dt);
  }
  if (m.jump != MYQL_JUMP_NONE) {
    double k = 0.0;
    if (m.jump == MYQL_JUMP_MERTON)
      k = std::exp(m.merton_mu + 0.5 * m.merton_delta * m.merton_delta) - 1.0;
    else
      k = (m.kou_p_up * m.kou_eta1) / (m.kou_eta1 - 1.0) +
          ((1.0 - m.kou_p_up) * m.kou_eta2) / (m.kou_eta2 + 1.0) - 1.0;
    const double window = pl.path_dep ? dt : T;
    const double mean = m.jump_lambda * window;
    C.jump_mean = (float)mean;
    C.jump_exp_neg_mean = (float)std::exp(-mean);
    C.jump_comp = (float)(-m.jump_lambda * k * window);
  }
}

void asian_consts(const myql_mc_job &job, const Plan &pl, double dt, int n_steps, int slot,
                  PayoffParams &Q) {
  const myql_instrument &in = job.instrument;
  const double n_dt = dt * n_steps, Ttot = n_dt + in.t_elapsed, S0 = job.S0;
  if (pl.tracker == TRK_GEO_ASIAN) {
    Q.avg_c0[slot] = (float)((in.past_avg_log * in.t_elapsed + std::log(S0) * n_dt) / Ttot - std::log(S0));
    Q.avg_c1[slot] = (float)(1.0 / Ttot);
  } else if (pl.tracker == TRK_ARITH_ASIAN) {
    Q.avg_c0[slot] = (float)(in.past_avg_S * in.t_elapsed / (S0 * Ttot));
    Q.avg_c1[slot] = (float)(1.0 / Ttot);
  }
}

}  // namespace
}  // namespace myql

using namespace myql;

// cv: when set, every level runs with the control variate of the context's
// network; plain_var (optional) receives the uncorrected level variances.
static myql_status mlmc_run(myql_ctx *ctx_, const myql_mc_job *job_in, const myql_mlmc_config *cfg,
                            myql_mlmc_result *res, int probe_level, uint64_t probe_dN,
                            double *probe_sums, bool cv = false, double *plain_var = nullptr,
                            bool ml2r = false);

// Weights of the multilevel Richardson-Romberg estimator (Lemaire & Pages,
// "Multilevel Richardson-Romberg extrapolation", Bernoulli 23(4A), 2017) over
// the levels 0..L with refinements n_l = 2^l and weak order alpha.  The
// Richardson weights w solve sum_l w_l x_l^k = [k == 0], k = 0..L, x_l = n_l^-alpha
// (w_l = prod_{s != l} x_s / (x_s - x_l)); the level-l difference carries
// W_l = sum_{r >= l} w_r, so W_0 = 1.
static std::vector<double> ml2r_weights(size_t L, double alpha) {
  std::vector<double> x(L + 1), w(L + 1), W(L + 1);
  for (size_t l = 0; l <= L; ++l) x[l] = std::pow(2.0, -alpha * (double)l);
  for (size_t l = 0; l <= L; ++l) {
    double t = 1.0;
    for (size_t s2 = 0; s2 <= L; ++s2)
      if (s2 != l) t *= x[s2] / (x[s2] - x[l]);
    w[l] = t;
  }
  double acc = 0.0;
  for (size_t l = L + 1; l-- > 0;) {
    acc += w[l];
    W[l] = acc;
  }
  return W;
}

extern "C" myql_status myql_ml2r_price(myql_ctx *ctx_, const myql_mc_job *job_in,
                                       const myql_mlmc_config *cfg, myql_mlmc_result *res) {
  if (!res || !cfg) return set_error(MYQL_ERR_INVALID_ARG, "null argument");
  if (!(cfg->alpha > 0.0)) return set_error(MYQL_ERR_INVALID_ARG, "ML2R needs the weak order alpha > 0");
  return mlmc_run(ctx_, job_in, cfg, res, -1, 0, nullptr, false, nullptr, true);
}

extern "C" myql_status myql_mlmc_price(myql_ctx *ctx_, const myql_mc_job *job_in,
                                       const myql_mlmc_config *cfg, myql_mlmc_result *res) {
  if (!res) return set_error(MYQL_ERR_INVALID_ARG, "null result");
  return mlmc_run(ctx_, job_in, cfg, res, -1, 0, nullptr);
}

extern "C" myql_status myql_mlmc_level(myql_ctx *ctx_, const myql_mc_job *job, const myql_mlmc_config *cfg,
                                       uint32_t level, uint64_t dN, double *sums) {
  if (!sums || dN == 0) return set_error(MYQL_ERR_INVALID_ARG, "need dN > 0 and an output");
  if (cfg && level > cfg->L_max) return set_error(MYQL_ERR_INVALID_ARG, "level above L_max");
  myql_mlmc_result unused;
  return mlmc_run(ctx_, job, cfg, &unused, (int)level, dN, sums);
}

extern "C" myql_status myql_mlmc_cv_price(myql_ctx *ctx_, const myql_mc_job *job_in, const myql_mlmc_config *cfg,
                                          const myql_cv_config *cv_cfg, myql_mlmc_result *res,
                                          double *plain_var) {
  if (!res || !job_in || !cfg) return set_error(MYQL_ERR_INVALID_ARG, "null argument");
  if (cv_cfg && cv_cfg->iterations > 0) {
    // the network learns the hedge on plain paths of a middle level's step
    myql_mc_job train = *job_in;
    train.config.time_steps = cfg->base_steps << std::min<uint64_t>(cfg->L_max, 5);
    train.config.greek_mode = MYQL_GREEKS_NONE;
    myql_cv_config c = *cv_cfg;
    c.hedge_every = 1;
    const myql_status s = myql_cv_train(ctx_, &train, &c, nullptr);
    if (s != MYQL_OK) return s;
  }
  return mlmc_run(ctx_, job_in, cfg, res, -1, 0, nullptr, true, plain_var);
}

extern "C" myql_status myql_mlmc_cv_level(myql_ctx *ctx_, const myql_mc_job *job, const myql_mlmc_config *cfg,
                                          uint32_t level, uint64_t dN, double *sums4) {
  if (!sums4 || dN == 0) return set_error(MYQL_ERR_INVALID_ARG, "need dN > 0 and an output");
  if (cfg && level > cfg->L_max) return set_error(MYQL_ERR_INVALID_ARG, "level above L_max");
  myql_mlmc_result unused;
  return mlmc_run(ctx_, job, cfg, &unused, (int)level, dN, sums4, true);
}

static myql_status mlmc_run(myql_ctx *ctx_, const myql_mc_job *job_in, const myql_mlmc_config *cfg,
                            myql_mlmc_result *res, int probe_level, uint64_t probe_dN,
                            double *probe_sums, bool cv, double *plain_var, bool ml2r) {
  CtxBase *ctx = reinterpret_cast<CtxBase *>(ctx_);
  if (!ctx || !job_in || !cfg || !res) return set_error(MYQL_ERR_INVALID_ARG, "null argument");
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) return cuda_status(e, "cudaSetDevice");
  if (!(cfg->epsilon > 0.0) || cfg->L_min > cfg->L_max || cfg->L_max + 1 > MYQL_MLMC_MAX_LEVELS ||
      cfg->base_steps < 1 || cfg->L_max > 20)
    return set_error(MYQL_ERR_INVALID_ARG, "MLMC needs epsilon > 0, L_min <= L_max <= 20, base_steps >= 1");
  if (job_in->instrument.is_strip || job_in->instrument.n_strikes != 1)
    return set_error(MYQL_ERR_UNSUPPORTED,
                     "MLMC prices scalar instruments (MultiLevelMonteCarloPricer.hpp:327)");
  // plan the base stepper: base_steps steps, GreekMode of the job, price only
  myql_mc_job job = *job_in;
  job.config.num_paths = 1;
  job.config.time_steps = cfg->base_steps;
  job.config.fd_bump = cfg->fd_bump;
  myql_status s = validate_job(job);
  if (s != MYQL_OK) return s;
  if (cv && tracker_of(job.instrument) == TRK_LOOKBACK)
    return set_error(MYQL_ERR_UNSUPPORTED, "control variates cover European, Asian and barrier instruments");
  Plan pl;
  s = make_plan(job, pl, cv);  // the control variate steps every path (per-step jumps)
  if (s != MYQL_OK) return s;
  const double T = job.instrument.maturity;
  const double df = std::exp(-job.r * T);
  const size_t L_max = cfg->L_max;

  // persistent stream pool: seed, streams [offset, offset + S) with the job's stream offset
  // (0 for a single controller; replicas and the multi-rank controller give disjoint blocks)
  const uint64_t S = cfg->n_streams ? cfg->n_streams : kDefaultStreams;
  s = ensure_streams(ctx, cfg->seed, job_in->config.stream_offset, S);
  if (s != MYQL_OK) return s;
  e = ctx->aux_a.ensure(S * 32);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(ctx->aux_a.p, ctx->st_cached.p, S * 32, cudaMemcpyDeviceToDevice, ctx->stream);
  const unsigned int max_blocks = (unsigned int)((S + kSimBlock - 1) / kSimBlock);
  if (e == cudaSuccess) e = ctx->aux_b.ensure((size_t)max_blocks * 2 * sizeof(double));
  if (e == cudaSuccess) e = ctx->strikes.ensure(sizeof(double));
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(ctx->strikes.p, job.instrument.strikes, sizeof(double), cudaMemcpyHostToDevice,
                        ctx->stream);
  if (e == cudaSuccess) e = ctx->status.ensure(16);
  if (e == cudaSuccess) e = cudaMemsetAsync(ctx->status.p, 0, 16, ctx->stream);
  if (e != cudaSuccess) return cuda_status(e, "MLMC buffers");

  MlmcParams M;
  std::memset(&M, 0, sizeof M);
  M.sim = pl.sim;
  M.pay = pl.pay;
  M.pay.strikes = (const double *)ctx->strikes.p;
  M.sim.states = (unsigned long long *)ctx->aux_a.p;
  M.sim.n_streams = (uint32_t)S;
  M.sim.status = (unsigned int *)ctx->status.p;
  M.sim.loop_cap = ctx->loop_cap;
  M.partials = (double *)ctx->aux_b.p;
  // NCI tables sized for the finest step the controller may reach
  for (int f = 0; f < pl.nf; ++f) {
    if (job.config.scheme[f] != MYQL_SCHEME_NCI) continue;
    const double dt_min = T / ((double)cfg->base_steps * (double)(1ull << L_max));
    s = ensure_nci(ctx, job.model.heston[f], dt_min, M.sim.nci[f]);
    if (s != MYQL_OK) return s;
  }

  std::vector<double> host_part((size_t)max_blocks * 2);
  std::vector<std::array<double, 2>> plain_sums(L_max + 1, {0.0, 0.0});
  std::vector<uint64_t> plain_n(L_max + 1, 0);
  cudaEventRecord(ctx->ev0, ctx->stream);
  uint32_t launches = 0;
  // With the control variate, a level keeps it only where it pays: after the level's first
  // (pilot) batch, both unbiased estimators' variances are known, and the CV stays if
  // Var(Y) > kappa_l Var(Y - C), kappa_l the cost of a CV path in plain coupled paths
  // (an MLP row costs about 25 coupled path-steps on this engine).  Otherwise the level's
  // statistics switch to the plain estimator of the same samples and its later batches run
  // the plain level kernel.
  std::vector<char> use_cv(L_max + 1, cv ? 1 : 0), decided(L_max + 1, 0);
  std::vector<double> cost_l(L_max + 1, 0.0);  // path cost of each level, in steps
  for (size_t l = 0; l <= L_max; ++l) cost_l[l] = (double)(cfg->base_steps * (1ull << l));
  auto cv_kappa = [&](size_t l) {
    const int n = l == 0 ? (int)cfg->base_steps : (int)((cfg->base_steps << l) / 2);
    const int he = std::max(1, n / 32), nh = (n + he - 1) / he;
    const double coupled_steps = l == 0 ? (double)cfg->base_steps : 1.5 * (double)(cfg->base_steps << l);
    return 1.0 + 25.0 * (double)nh / coupled_steps;
  };
  auto evaluate_level = [&](size_t l, uint64_t dN, double &sum, double &sum_sq) -> myql_status {
    const uint64_t fine = cfg->base_steps << l;
    if (l == 0) {
      const double dt = T / (double)cfg->base_steps;
      level_consts(job, pl, dt, (int)cfg->base_steps, T, M.sim.sc[0]);
      M.sim.n_steps = (int)cfg->base_steps;
      M.n_coarse = (int)cfg->base_steps;
      asian_consts(job, pl, dt, (int)cfg->base_steps, 0, M.pay);
    } else {
      const double dtf = T / (double)fine;
      const int nc = (int)(fine / 2);
      level_consts(job, pl, dtf, (int)fine, T, M.sim.sc[0]);
      level_consts(job, pl, 2.0 * dtf, nc, T, M.sim.sc[1]);
      // the coupled stepper prepares its jumps for the fine step (European: for T)
      M.sim.sc[1].jump_mean = M.sim.sc[0].jump_mean;
      M.sim.sc[1].jump_exp_neg_mean = M.sim.sc[0].jump_exp_neg_mean;
      M.sim.sc[1].jump_comp = M.sim.sc[0].jump_comp;
      M.sim.n_steps = (int)fine;
      M.n_coarse = nc;
      asian_consts(job, pl, dtf, (int)fine, 0, M.pay);
      asian_consts(job, pl, 2.0 * dtf, nc, 1, M.pay);
    }
    M.level = (int)l;
    M.dN = dN;
    M.n_used = (unsigned int)std::min<uint64_t>(S, dN);
    if (cv && (use_cv[l] || (probe_sums && probe_level >= 0))) {
      MlmcCvParams Q;
      std::memset(&Q, 0, sizeof Q);
      Q.M = M;
      Q.df = df;
      const int n = l == 0 ? (int)cfg->base_steps : M.n_coarse;  // steps (level 0) or coarse steps
      Q.hedge_every = std::max(1, n / 32);
      Q.n_hedge = (n + Q.hedge_every - 1) / Q.hedge_every;
      const double dt0 = l == 0 ? T / (double)cfg->base_steps : T / (double)fine;
      myql_status s2 = cv_feat_consts(job, pl, M.sim.sc[0], dt0, Q.fine);
      if (s2 == MYQL_OK && l > 0) s2 = cv_feat_consts(job, pl, M.sim.sc[1], 2.0 * dt0, Q.coarse);
      if (s2 != MYQL_OK) return s2;
      double s4[4] = {0, 0, 0, 0};
      s2 = cv_level_eval(ctx, Q, batch_class(pl.nf, pl.s1, pl.s2), dN, s4);
      if (s2 != MYQL_OK) return s2;
      launches += 3;
      if (probe_sums && probe_level >= 0) {  // level probe: discounted sums as they are
        for (int i = 0; i < 4; ++i) probe_sums[i] += s4[i];
        return MYQL_OK;
      }
      sum += s4[2] / df;
      sum_sq += s4[3] / (df * df);
      plain_sums[l][0] += s4[0] / df;
      plain_sums[l][1] += s4[1] / (df * df);
      plain_n[l] += dN;
      if (!decided[l] && plain_n[l] > 1) {
        decided[l] = 1;
        const double n = (double)plain_n[l];
        const double mp = plain_sums[l][0] / n, mc = sum / n;
        const double vp = plain_sums[l][1] / n - mp * mp, vc = sum_sq / n - mc * mc;
        if (!(vp > cv_kappa(l) * vc)) {
          use_cv[l] = 0;  // the plain estimator of the same samples
          sum = plain_sums[l][0];
          sum_sq = plain_sums[l][1];
        } else {
          cost_l[l] *= cv_kappa(l);
        }
      }
      return MYQL_OK;
    }
    cudaError_t er = launch_mlmc_level(M, pl.s1, pl.s2, pl.path_dep, ctx->stream);
    if (er != cudaSuccess) return cuda_status(er, "MLMC level launch");
    ++launches;
    const unsigned int blocks = (M.n_used + kSimBlock - 1) / kSimBlock;
    er = cudaMemcpyAsync(host_part.data(), M.partials, (size_t)blocks * 2 * sizeof(double),
                         cudaMemcpyDeviceToHost, ctx->stream);
    if (er == cudaSuccess) er = cudaStreamSynchronize(ctx->stream);
    if (er != cudaSuccess) return cuda_status(er, "MLMC level");
    double a = 0.0, b = 0.0;
    for (unsigned int i = 0; i < blocks; ++i) {
      a += host_part[2 * i];
      b += host_part[2 * i + 1];
    }
    sum += a;
    sum_sq += b;
    if (cv) {  // a level that dropped the control variate: its plain statistics
      plain_sums[l][0] += a;
      plain_sums[l][1] += b;
      plain_n[l] += dN;
    }
    return MYQL_OK;
  };

  if (probe_level >= 0) {
    probe_sums[0] = probe_sums[1] = 0.0;
    if (cv) probe_sums[2] = probe_sums[3] = 0.0;
    s = evaluate_level((size_t)probe_level, probe_dN, probe_sums[0], probe_sums[1]);
    if (s != MYQL_OK) return s;
    return read_status(ctx, nullptr);
  }
  // ---- Giles' adaptive controller (MultiLevelMonteCarloPricer.hpp:64-211)
  size_t L = ml2r ? std::max<uint64_t>(cfg->L_min, 1) : cfg->L_min;
  std::vector<uint64_t> N_l(L_max + 1, 0);
  std::vector<double> sum_dP(L_max + 1, 0.0), sum_sq_dP(L_max + 1, 0.0), V_l(L_max + 1, 0.0);
  double alpha = cfg->alpha, beta = cfg->beta;
  const double eps_m2 = std::pow(cfg->epsilon, -2.0);
  bool converged = false;
  int guard = 0;
  // level weights: 1 for MLMC; the ML2R weights of the current level count
  std::vector<double> Wt(L_max + 1, 1.0);
  auto set_weights = [&]() {
    if (!ml2r) return;
    const std::vector<double> W = ml2r_weights(L, alpha);
    for (size_t l = 0; l <= L; ++l) Wt[l] = W[l];
  };
  while (!converged) {
    if (++guard > 10000) return set_error(MYQL_ERR_LOOP_CAP, "MLMC controller did not converge");
    set_weights();
    for (size_t l = 0; l <= L; ++l) {
      double sum_sqrt_VC_pilot = 0.0;
      for (size_t k = 0; k <= L; ++k) sum_sqrt_VC_pilot += std::abs(Wt[k]) * std::sqrt(V_l[k] * cost_l[k]);
      uint64_t optimal_N = 0;
      if (V_l[l] > 1e-18)
        optimal_N = (uint64_t)std::ceil(2.0 * eps_m2 * std::abs(Wt[l]) * std::sqrt(V_l[l] / cost_l[l]) *
                                        sum_sqrt_VC_pilot);
      const uint64_t pilot_N = std::max<uint64_t>(20, cfg->N0 / (1ull << l));
      const uint64_t target_N = std::max(pilot_N, optimal_N);
      if (N_l[l] < target_N) {
        const uint64_t dN = target_N - N_l[l];
        s = evaluate_level(l, dN, sum_dP[l], sum_sq_dP[l]);
        if (s != MYQL_OK) return s;
        N_l[l] += dN;
        if (N_l[l] > 1) {
          const double mean = sum_dP[l] / N_l[l];
          V_l[l] = std::max(1e-18, (sum_sq_dP[l] / N_l[l]) - (mean * mean));
        }
      }
    }
    if (cfg->adaptive_rates && L >= 2) {
      auto estimate_order = [&](const std::vector<double> &values) {
        double sum_l = 0, sum_logV = 0, sum_l_logV = 0, sum_l2 = 0;
        int count = 0;
        const size_t start_l = L - 2;
        for (size_t l = start_l; l <= L; ++l) {
          if (values[l] > 1e-16) {
            const double y = std::log(values[l]);
            const double x = (double)(l - start_l);
            sum_l += x;
            sum_logV += y;
            sum_l_logV += x * y;
            sum_l2 += x * x;
            count++;
          }
        }
        if (count < 2) return -1.0;
        const double slope = (count * sum_l_logV - sum_l * sum_logV) / (count * sum_l2 - sum_l * sum_l);
        return -slope / std::log(2.0);
      };
      std::vector<double> abs_means(L + 1);
      for (size_t l = 0; l <= L; ++l) abs_means[l] = std::abs(sum_dP[l] / N_l[l]);
      const double est_alpha = estimate_order(abs_means);
      const double est_beta = estimate_order(V_l);
      if (est_alpha > 0.3) alpha = std::min(2.0, est_alpha);
      if (est_beta > 0.3) beta = std::min(2.0, est_beta);
    }
    set_weights();
    double sum_sqrt_VC = 0.0;
    for (size_t l = 0; l <= L; ++l) sum_sqrt_VC += std::abs(Wt[l]) * std::sqrt(V_l[l] * cost_l[l]);
    bool needs_more_paths = false;
    for (size_t l = 0; l <= L; ++l) {
      const uint64_t optimal_N =
          (uint64_t)std::ceil(2.0 * eps_m2 * std::abs(Wt[l]) * std::sqrt(V_l[l] / cost_l[l]) * sum_sqrt_VC);
      if (optimal_N > N_l[l]) needs_more_paths = true;
    }
    if (needs_more_paths) continue;
    if (ml2r) {
      // bias test: the extrapolations over L + 1 and over L levels, from the same level
      // means, differ by about the bias of the smaller one (conservative for the larger)
      const std::vector<double> Wm = ml2r_weights(L - 1, alpha);
      double est_L = 0.0, est_Lm1 = 0.0;
      for (size_t l = 0; l <= L; ++l) {
        const double m_l = sum_dP[l] / N_l[l];
        est_L += Wt[l] * m_l;
        if (l < L) est_Lm1 += Wm[l] * m_l;
      }
      if (std::abs(est_L - est_Lm1) > cfg->epsilon / 1.4142135623730951 && L < L_max)
        L++;
      else
        converged = true;
      continue;
    }
    const double diff_mean_L = std::abs(sum_dP[L] / N_l[L]);
    double effective_diff = diff_mean_L;
    if (L > 0) effective_diff = std::max(diff_mean_L, 0.5 * std::abs(sum_dP[L - 1] / N_l[L - 1]));
    const double bias_estimate = effective_diff / (std::pow(2.0, alpha) - 1.0);
    if (bias_estimate > cfg->epsilon / 1.4142135623730951) {  // std::numbers::sqrt2
      if (L < L_max)
        L++;
      else
        converged = true;
    } else {
      converged = true;
    }
  }
  // ---- aggregation (:213-238)
  std::memset(res, 0, sizeof *res);
  res->alpha_estimated = alpha;
  res->beta_estimated = beta;
  res->n_levels = (uint32_t)(L + 1);
  double var_total = 0.0;
  for (size_t l = 0; l <= L; ++l) {
    res->paths_per_level[l] = N_l[l];
    const uint64_t steps_per_path = (l == 0) ? cfg->base_steps : (cfg->base_steps * (1ull << l) * 3 / 2);
    res->total_steps += N_l[l] * steps_per_path;
    const double mean_dP = sum_dP[l] / N_l[l];
    res->mean_diffs[l] = mean_dP * df;
    res->var_diffs[l] = V_l[l] * df * df;
    res->price += Wt[l] * mean_dP * df;
    var_total += Wt[l] * Wt[l] * V_l[l] / N_l[l];
  }
  res->price_std_err = std::sqrt(var_total) * df;
  if (plain_var)
    for (size_t l = 0; l <= L; ++l) {
      const double n = (double)std::max<uint64_t>(plain_n[l], 1);
      const double mean = plain_sums[l][0] / n;
      plain_var[l] = std::max(plain_sums[l][1] / n - mean * mean, 0.0) * df * df;
    }
  cudaEventRecord(ctx->ev1, ctx->stream);
  cudaEventSynchronize(ctx->ev1);
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
  res->device_ms = ms;
  ctx->launches = launches;
  return read_status(ctx, nullptr);
}
