/*
 * myql_gpu.h -- C ABI of the GB300 (sm_103a) Monte Carlo path-simulation engine.
 *
 * This is the drop-in boundary for MyQuantLib's Monte Carlo hot path.  The
 * reference exposes the path as C++ templates; every entry point below lowers
 * one of those template calls to plain C types (PODs, pointers, sizes) so any
 * host language can bind it (ctypes, cgo, JNI, N-API).  No C++ or torch type
 * crosses this boundary.
 *
 *   reference call (MyQuantLib, header-only C++20)            entry point here
 *   ---------------------------------------------------------  ------------------------
 *   MonteCarloPricer<Model,Stepper,Instr,Mode>::calculate       myql_mc_price
 *       (include/myql/pricers/montecarlo/MonteCarloPricer.hpp:95)
 *   dispatcher::price_mc<Mode,Scheme>(AnyModel, AnyMCInstrument) myql_mc_price_batch
 *       (include/myql/dispatcher/PricingDispatch.hpp:93-126)     (many jobs, one launch)
 *   MultiLevelMonteCarloPricer<...>::calculate                  myql_mlmc_price
 *       (include/myql/pricers/mlmc/MultiLevelMonteCarloPricer.hpp:46)
 *   boost::random::xoshiro256pp(seed) + jump()                  myql_rng_stream_states
 *       (seeded at MonteCarloPricer.hpp:191)
 *
 * Ownership: the caller owns every buffer it passes.  A myql_ctx owns device
 * memory (stream-state tables, chi-squared tables, scratch) and is meant to be
 * used by one host thread at a time.  All calls are blocking unless they take
 * a cudaStream_t (passed as void*).
 *
 * Errors: every entry point returns a myql_status; myql_last_error() gives a
 * one-line message for the calling thread.  Invalid parameters (including the
 * SchemeNV condition sigma^2 <= 4 kappa theta, which the reference enforces by
 * throwing from VolSchemes.hpp:40-41) are rejected on the host before launch.
 */
#ifndef MYQL_GPU_H
#define MYQL_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MYQL_ABI_VERSION 1

typedef enum myql_status {
  MYQL_OK = 0,
  MYQL_ERR_INVALID_ARG = 1,  /* bad pointer, size or parameter            */
  MYQL_ERR_NV_CONDITION = 2, /* SchemeNV with sigma^2 > 4 kappa theta     */
  MYQL_ERR_OOM = 3,          /* device allocation failed                  */
  MYQL_ERR_CUDA = 4,         /* any other CUDA runtime error              */
  MYQL_ERR_LOOP_CAP = 5,     /* a bounded device loop hit its cap         */
  MYQL_ERR_TIMEOUT = 6,      /* a device wait gave up                     */
  MYQL_ERR_NO_DEVICE = 7,    /* no usable sm_103 device                   */
  MYQL_ERR_UNSUPPORTED = 8,  /* combination the engine does not provide   */
  MYQL_ERR_TOO_LARGE = 9     /* request exceeds a documented size limit   */
} myql_status;

/* --- policy choices (the reference's template parameters) ---------------- */
typedef enum myql_scheme { /* VolSchemes.hpp */
  MYQL_SCHEME_NONE = 0,    /* NullVolScheme (unused factor)          :19  */
  MYQL_SCHEME_NV = 1,      /* SchemeNV (Ninomiya-Victoir)            :24  */
  MYQL_SCHEME_EXACT = 2,   /* SchemeExact (Poisson-Gamma)            :71  */
  MYQL_SCHEME_NCI = 3      /* SchemeNCI (chi-squared inversion)      :230 */
} myql_scheme;

typedef enum myql_jump { /* JumpPolicies.hpp */
  MYQL_JUMP_NONE = 0,    /* NoJumps    :15 */
  MYQL_JUMP_MERTON = 1,  /* MertonJump :32 */
  MYQL_JUMP_KOU = 2      /* KouJump    :81 */
} myql_jump;

typedef enum myql_instrument_kind {
  MYQL_INSTR_EUROPEAN = 0,    /* EuropeanOption  (European.hpp:10)              */
  MYQL_INSTR_ASIAN_GEO = 1,   /* AsianOption<TrackerGeoAsian>   (Asian.hpp:7)   */
  MYQL_INSTR_ASIAN_ARITH = 2, /* AsianOption<TrackerArithAsian> (Asian.hpp:7)   */
  MYQL_INSTR_LOOKBACK = 3,    /* LookbackOption  (Lookback.hpp:8)               */
  MYQL_INSTR_BARRIER = 4      /* BarrierOption   (Barrier.hpp:17)               */
} myql_instrument_kind;

typedef enum myql_payoff { /* Payoffs.hpp */
  MYQL_PAYOFF_VANILLA = 0, /* PayoffVanilla        :14 */
  MYQL_PAYOFF_CASH = 1,    /* PayoffCashOrNothing  :39 */
  MYQL_PAYOFF_ASSET = 2    /* PayoffAssetOrNothing :57 */
} myql_payoff;

typedef enum myql_option_type { MYQL_CALL = 0, MYQL_PUT = 1 } myql_option_type;
typedef enum myql_greek_mode { /* PricingTypes.hpp:8-12 */
  MYQL_GREEKS_NONE = 0,
  MYQL_GREEKS_ESSENTIAL = 1,
  MYQL_GREEKS_FULL = 2
} myql_greek_mode;
typedef enum myql_barrier_action { MYQL_BARRIER_IN = 0, MYQL_BARRIER_OUT = 1 } myql_barrier_action;
typedef enum myql_rebate_timing { /* Barrier.hpp:12 */
  MYQL_REBATE_NONE = 0,
  MYQL_REBATE_AT_HIT = 1,
  MYQL_REBATE_AT_MATURITY = 2
} myql_rebate_timing;

/* --- model --------------------------------------------------------------- */
typedef struct myql_heston_params { /* HestonParams, ModelParams.hpp:7-25 */
  double kappa, theta, sigma, rho, v0;
} myql_heston_params;

typedef struct myql_model { /* ZeroFactorModel / SingleFactorModel / DoubleFactorModel, ASVJmodel.hpp:14-50 */
  int32_t num_factors;          /* 0 (GBM), 1 (Heston/Bates), 2 (double Heston/Bates) */
  int32_t jump;                 /* myql_jump */
  double vol;                   /* ZeroFactorModel::vol (num_factors == 0)            */
  myql_heston_params heston[2]; /* heston[0] = heston / heston1, heston[1] = heston2  */
  double jump_lambda;           /* MertonParams::lambda or KouParams::lambda         */
  double merton_mu, merton_delta;        /* MertonParams (ModelParams.hpp:35-39)      */
  double kou_p_up, kou_eta1, kou_eta2;   /* KouParams    (ModelParams.hpp:42-47)      */
} myql_model;

/* --- instrument ---------------------------------------------------------- */
typedef struct myql_instrument {
  int32_t kind;           /* myql_instrument_kind                                   */
  int32_t payoff;         /* myql_payoff                                            */
  int32_t option_type;    /* myql_option_type                                       */
  int32_t fixed_strike;   /* Asian/Lookback: 1 = fixed strike, 0 = floating strike  */
  int32_t barrier_up;     /* Barrier: 1 = BarrierDirection::Up, 0 = Down            */
  int32_t barrier_action; /* myql_barrier_action                                    */
  int32_t rebate_timing;  /* myql_rebate_timing                                     */
  int32_t is_strip;       /* 1 = ResultType std::vector<double>, 0 = double         */
  double maturity;        /* T                                                      */
  double barrier;         /* B                                                      */
  double rebate;          /* rebate amount                                          */
  double barrier_rate;    /* rate_ used for AtHit rebates (Barrier.hpp:36)          */
  double payoff_eps;      /* digital smoothing bandwidth; < 0 = automatic           */
  const double *strikes;  /* host array of n_strikes strikes                        */
  int64_t n_strikes;      /* 1 for scalar instruments                               */
  /* in-flight history (Asian.hpp:105-107, Lookback.hpp:184-185)                    */
  double past_avg_log, past_avg_S, t_elapsed;
  double hist_min_S, hist_max_S; /* 0 = not set                                     */
} myql_instrument;

/* --- Monte Carlo configuration (MonteCarloConfig, MonteCarloPricer.hpp:16-26) --- */
typedef struct myql_mc_config {
  uint64_t num_paths;
  uint64_t time_steps;
  uint64_t seed;
  double fd_bump, vol_bump, t_bump, r_bump;
  int32_t scheme[2];  /* myql_scheme per variance factor (the Stepper's VolScheme1/2) */
  int32_t greek_mode; /* myql_greek_mode (the pricer's GreekMode template argument)   */
  uint64_t n_streams; /* xoshiro streams; 0 = min(num_paths, clamp(num_paths / 8,
                         131072, 524288)); path i runs on stream i mod n_streams       */
  uint64_t stream_offset; /* index of the first stream: replicas or ranks that take
                             disjoint stream ranges draw independent paths          */
} myql_mc_config;

typedef struct myql_mc_job {
  myql_model model;
  myql_instrument instrument;
  myql_mc_config config;
  double S0, r, q;
} myql_mc_job;

/* --- results ------------------------------------------------------------- */
/* Quantities, in the order of MonteCarloResult<Full> (PricingTypes.hpp:68-97). */
typedef enum myql_quantity {
  MYQL_Q_PRICE = 0,
  MYQL_Q_DELTA = 1,
  MYQL_Q_GAMMA = 2,
  MYQL_Q_VEGA0 = 3,
  MYQL_Q_VEGA1 = 4,
  MYQL_Q_THETA = 5,
  MYQL_Q_RHO = 6,
  MYQL_Q_VANNA0 = 7,
  MYQL_Q_VANNA1 = 8,
  MYQL_Q_CHARM = 9,
  MYQL_Q_COUNT = 10
} myql_quantity;

/* Output layout for one job with n = instrument.n_strikes:
 *   out[(2*quantity + 0) * n + k] = value       of strike k
 *   out[(2*quantity + 1) * n + k] = std. error  of strike k
 * i.e. 2 * MYQL_Q_COUNT * n doubles.  Quantities the GreekMode does not
 * produce are written as 0. */
#define MYQL_OUT_DOUBLES(n_strikes) ((size_t)2 * MYQL_Q_COUNT * (size_t)(n_strikes))

typedef struct myql_mc_stats {
  uint64_t paths;              /* paths priced                                   */
  uint64_t path_steps;         /* simulated path-steps (base + bumped scenarios) */
  uint32_t scenarios;          /* simulated scenarios per path (1, 7 or 9)       */
  uint32_t loop_cap_hits;      /* bounded device loops that hit their cap        */
  uint32_t table_fallbacks;    /* NCI draws outside the chi-squared table        */
  uint32_t kernel_launches;    /* kernels launched by this call                  */
  double device_ms;            /* device time of the call (CUDA events)          */
  double simulate_ms;          /* of which: path-simulation kernels              */
  double payoff_ms;            /* of which: payoff / Greek reduction kernels     */
} myql_mc_stats;

/* --- context ------------------------------------------------------------- */
typedef struct myql_ctx myql_ctx;

myql_status myql_ctx_create(myql_ctx **ctx, int device);
myql_status myql_ctx_destroy(myql_ctx *ctx);
/* Copies the last error message of the calling thread (NUL-terminated). */
size_t myql_last_error(char *buf, size_t len);
int myql_abi_version(void);

/* Debug/limit knobs.  max_loop_iters caps every bounded device loop (Poisson,
 * Gamma rejection, Kou jump counts); 0 restores the defaults.  Used by tests
 * to provoke MYQL_ERR_LOOP_CAP without touching the GPU's health. */
myql_status myql_ctx_set_loop_cap(myql_ctx *ctx, uint32_t max_loop_iters);

/* Upper bound on the per-path record scratch of one launch (bytes; 0 = the
 * 2 GiB default).  Larger requests are simulated in chunks of whole stream
 * rounds; results do not depend on the chunking. */
myql_status myql_ctx_set_records_limit(myql_ctx *ctx, uint64_t bytes);

/* SchemeNCI table cells (VolSchemes.hpp:240-313).  mode 0 (default): the
 * reference's cells.  The cubic of the first cell runs from the node y(0) = 0,
 * while for many degrees of freedom the quantile is near y(dx) on almost all of
 * [0, dx].  So the cells' mean of the chi-squared draw falls short by 1.5e-5 to
 * 4e-5 relative (rows 25 to 1000).  Over hundreds of steps this becomes a price
 * bias of 0.2 to 1.6 % at 800 steps a year; through rho / sigma (v' - v) in the
 * log-spot step its sign is that of -rho.  mode 1: exact slopes 1 / f(y) and a
 * first cell that keeps the exact mean of its sliver, so the cells integrate to
 * the mean within about 1e-8.  Tables are cached per mode. */
myql_status myql_ctx_set_nci_slopes(myql_ctx *ctx, int mode);

/* Upper bound on the rows of this context's SchemeNCI tables (memory and L2
 * budget; 0, the default, leaves the sizing rule alone, which builds rows up to
 * lambda + 6 sqrt(lambda) + 16 at a high variance level, at least the
 * reference's n_max + 1 and at most 1024).  A Poisson count N at or beyond the
 * rows has no table row: its chi-squared quantile (d + 2N degrees of freedom)
 * is the Wilson-Hilferty cube, where the reference evaluates the exact quantile
 * past its own n_max (VolSchemes.hpp:368-369); such draws are counted in
 * myql_mc_stats.table_fallbacks.  Rows beyond 1024 have d + 2N > 2048, where
 * the cube is within 6e-6 relative of the exact quantile. */
myql_status myql_ctx_set_nci_rows(myql_ctx *ctx, int max_rows);

/* Theta and charm of one-factor SchemeNCI Europeans (on, 1; off, 0, the
 * default).  They difference the scenarios at maturity T +- t_bump, whose
 * per-step constants differ by about 2 t_bump / T relative; FP32 constants
 * carry that difference with a systematic relative error of 1e-4 to 1e-2,
 * which every path shares (the reference's FP64 constants carry it to about
 * 1e-11).  On, those two scenarios add each constant's FP32 rounding error back
 * as a second FP32 term (Poisson mean, table scale, drift, diffusion and jump
 * compensation), a few more FP32 operations per step for those two scenarios.
 * Their records then differ from requests that price T +- t_bump alone in the
 * last bits (and, rarely, by a Poisson count). */
myql_status myql_ctx_set_precise_theta(myql_ctx *ctx, int on);

/* Host-side validation of a job, without a device: the checks myql_mc_price
 * runs before any launch (MYQL_ERR_NV_CONDITION for SchemeNV with
 * sigma^2 > 4 kappa theta, as VolSchemes.hpp:40-41 throws). */
myql_status myql_validate_job(const myql_mc_job *job);

/* --- pricing entry points ------------------------------------------------ */

/* One pricing request: replaces MonteCarloPricer::calculate (MonteCarloPricer.hpp:95).
 * out: host buffer of MYQL_OUT_DOUBLES(n_strikes) doubles.  stats may be NULL. */
myql_status myql_mc_price(myql_ctx *ctx, const myql_mc_job *job, double *out,
                          myql_mc_stats *stats);

/* Same, with device-resident output (out_dev: device pointer, same layout) and
 * an explicit CUDA stream (cudaStream_t as void*; NULL = the legacy default
 * stream).  Returns once the work is enqueued; host-side validation and table
 * builds happen synchronously. */
myql_status myql_mc_price_async(myql_ctx *ctx, const myql_mc_job *job,
                                double *out_dev, void *stream);

/* Pricing without allocating device memory.  No counterpart in the reference
 * (its pricer allocates freely on the host).  For callers that must not
 * allocate GPU memory while they price -- their device memory belongs to their
 * own pool or to another framework's allocator, or allocation is forbidden
 * after start-up.  All scratch lives in one fixed device array of
 * MYQL_NOALLOC_SCRATCH_BYTES inside the library, which every GPU that loads the
 * library holds until the process exits; requests that need more (roughly
 * paths * fields * 4 + streams * 32 + strikes * 8 bytes plus tile partials)
 * return MYQL_ERR_TOO_LARGE.  Scope: GreekMode None and Essential, schemes NV
 * and Exact (NCI needs its chi-squared tables).  No context is needed: the
 * first call on each device does a one-time set-up on that device (it looks
 * up the array's device address and uploads the stream-jump polynomials), so
 * make that first call before any stream capture.  The call enqueues on
 * `stream` (cudaStream_t as void*, NULL = legacy default stream) and returns
 * once the stream has finished the request; out_dev is a device buffer of
 * MYQL_OUT_DOUBLES(n_strikes) doubles.  Every call shares the one array, so
 * calls that overlap on the GPU (other streams, other host threads) race:
 * serialize them. */
#define MYQL_NOALLOC_SCRATCH_BYTES (32 << 20)
myql_status myql_mc_price_noalloc(int device, const myql_mc_job *job, double *out_dev,
                                  void *stream);

/* Many uneven requests in one persistent launch: replaces a loop of
 * dispatcher::price_mc calls (PricingDispatch.hpp:93-126).
 * outs[j] is the host output buffer of job j (MYQL_OUT_DOUBLES of its strikes). */
myql_status myql_mc_price_batch(myql_ctx *ctx, const myql_mc_job *jobs,
                                size_t n_jobs, double *const *outs,
                                myql_mc_stats *stats);

/* The kernel classes of the last myql_mc_price_batch call on this context and
 * the launch shape the batch autotuner picked for each: threads per block,
 * streams (each with all of its paths) per thread, unroll depth of the
 * time-step loop (0 = the compiler's choice) and persistent grid size.  A class
 * is the factor count, the scheme of each factor (MYQL_SCHEME_*) and path
 * dependence.  tuned = 1 when the shape was timed among the candidates on the
 * class's leading items (tuned_ms; default_ms is the default shape 128 x 1 x 0
 * on the same items), 0 when the class had too few items to tune (default
 * shape), -1 when the shape was forced by myql_ctx_set_batch_shape. */
typedef struct {
  int32_t factors, scheme1, scheme2, path_dependent;
  int32_t block, streams_per_thread, unroll, tuned;
  uint32_t grid;
  uint64_t items;
  double tuned_ms, default_ms;
} myql_batch_class_plan;
myql_status myql_batch_last_plan(myql_ctx *ctx, myql_batch_class_plan *out, size_t cap, size_t *n_classes);

/* Forces one launch shape on every class of this context's batches: block 64,
 * 128 or 256 threads, 1, 2 or 4 streams per thread (block x streams a multiple
 * of 128), unroll 0 or 2.  block = 0 returns to the autotuner.  Results do not
 * depend on the shape beyond FP64 summation order. */
myql_status myql_ctx_set_batch_shape(myql_ctx *ctx, int block, int streams_per_thread, int unroll);

/* Per-path terminal records of one request (debug / parity): writes
 * n_scenarios * n_fields * num_paths floats in [scenario][field][path] order.
 * Fields per tracker: European {X}; Geo/Arith Asian {X, A}; Lookback
 * {X, minX, maxX}; Barrier {X, t_hit_base, t_hit_up, t_hit_dn} with
 * X = log(S_T / S0) and t_hit = -1 when the barrier was not hit. */
myql_status myql_mc_paths(myql_ctx *ctx, const myql_mc_job *job, float *records,
                          size_t records_len, uint32_t *n_scenarios,
                          uint32_t *n_fields);

/* --- MLMC (MultiLevelMonteCarloPricer.hpp:16-30, :46-241) --------------- */
typedef struct myql_mlmc_config {
  double epsilon;
  uint64_t L_min, L_max, N0, base_steps;
  double alpha, beta;
  int32_t adaptive_rates;
  uint64_t seed;
  double fd_bump;
  uint64_t n_streams; /* 0 = default */
} myql_mlmc_config;

#define MYQL_MLMC_MAX_LEVELS 24
typedef struct myql_mlmc_result { /* MlmcResult<None,double>, PricingTypes.hpp:104-115 */
  double price, price_std_err;
  uint64_t total_steps;
  uint32_t n_levels;
  uint64_t paths_per_level[MYQL_MLMC_MAX_LEVELS];
  double mean_diffs[MYQL_MLMC_MAX_LEVELS];
  double var_diffs[MYQL_MLMC_MAX_LEVELS];
  double alpha_estimated, beta_estimated;
  double device_ms;
} myql_mlmc_result;

/* job->config supplies scheme[] (the coupled stepper's VolScheme1/2); its
 * num_paths/time_steps/seed are ignored in favour of mlmc. */
myql_status myql_mlmc_price(myql_ctx *ctx, const myql_mc_job *job,
                            const myql_mlmc_config *mlmc,
                            myql_mlmc_result *result);

/* Multilevel Richardson-Romberg extrapolation (ML2R; listed as future work in
 * the reference's README.md:335) on the same coupled levels: the level-l
 * difference is weighted by W_l = sum_{r >= l} w_r, w the Richardson weights for
 * refinements 2^l and weak order mlmc->alpha (required > 0; re-estimated when
 * adaptive_rates is set), so the bias is O(h^(alpha (L + 1))) instead of O(h^alpha).
 * Levels are added while the extrapolations over L + 1 and L levels differ by
 * more than epsilon / sqrt(2).  result->price = sum_l W_l mean_diffs[l];
 * mean_diffs / var_diffs stay the unweighted level statistics.  The weights
 * assume a regular expansion of the weak error in powers of h^alpha: smooth
 * payoffs and Asians qualify; discretely monitored barriers do not (their error
 * oscillates with the barrier's position on the monitoring grid). */
myql_status myql_ml2r_price(myql_ctx *ctx, const myql_mc_job *job, const myql_mlmc_config *mlmc,
                            myql_mlmc_result *result);

/* Randomized quasi-Monte Carlo (the reference's future work, README.md:331):
 * Sobol points (Gray-code order; direction numbers from primitive polynomials by
 * the Bratley-Fox recurrence with seeded odd initial values), a Brownian bridge
 * per Brownian motion (the spot and each SchemeNV factor, bridge levels
 * interleaved), two Sobol uniforms per step for each SchemeNCI factor (its
 * Poisson count and chi-squared table, by inversion) and for Merton jumps (the
 * count and the normal of the jump sum, drawn per step for every instrument),
 * and n_replicates random digital shifts.  out: price rows as myql_mc_price
 * (standard error from the spread of the replicate estimates).  Factors on
 * SchemeNV or SchemeNCI, no jumps or Merton jumps (SchemeExact and Kou jumps
 * have no fixed number of draws per step), GreekMode None, at most 512 steps,
 * num_paths a multiple of 2048 * n_replicates (n_replicates >= 2). */
myql_status myql_qmc_price(myql_ctx *ctx, const myql_mc_job *job, uint32_t n_replicates, double *out,
                           myql_mc_stats *stats);
/* Sobol direction numbers: out[d * 32 + k - 1] = V_k of dimension d, the initial
 * values m_1..m_s of each dimension drawn from `seed` (host computation; needs no
 * GPU).  myql_qmc_price and myql_cv_qmc_price use one seed's for every job (see
 * myql_ctx_set_qmc_direction_seed); the job's seed draws their digital shifts. */
myql_status myql_qmc_directions(uint32_t D, uint64_t seed, uint32_t *out);
/* The point set of this context's randomized QMC (myql_qmc_price, myql_cv_qmc_price):
 * the seed of the initial direction numbers (myql_qmc_directions).  The default,
 * MYQL_QMC_DEFAULT_DIRECTION_SEED, had the best geometric-mean variance ratio over six
 * test integrands among 37 candidate seeds; another seed gives another randomly
 * initialised Sobol point set. */
#define MYQL_QMC_DEFAULT_DIRECTION_SEED 6
myql_status myql_ctx_set_qmc_direction_seed(myql_ctx *ctx, uint64_t seed);

/* One evaluate_level call of the MLMC pricer (MultiLevelMonteCarloPricer.hpp:244-341)
 * from a freshly seeded stream pool: dN paths of level l (0 = base stepper,
 * l > 0 = coupled fine/coarse pair).  sums[0] = sum of P_l - P_(l-1),
 * sums[1] = sum of squares (FP64).  Probe for per-level parity tests. */
myql_status myql_mlmc_level(myql_ctx *ctx, const myql_mc_job *job, const myql_mlmc_config *mlmc,
                            uint32_t level, uint64_t dN, double *sums);

/* --- RNG streams (bit-exact against boost::random::xoshiro256pp) -------- */
/* Writes the xoshiro256++ state of streams first..first+n-1 for `seed`:
 * stream k = state seeded by splitmix64(seed), advanced by k * 2^128 steps
 * (k applications of the standard xoshiro256 jump()).  out: host buffer of
 * 4*n uint64 in [stream][word] order.  Computed on the device. */
myql_status myql_rng_stream_states(myql_ctx *ctx, uint64_t seed, uint64_t first,
                                   uint64_t n, uint64_t *out);
/* Draws `count` consecutive 64-bit outputs of each listed stream on the
 * device: out[stream][i], host buffer of n*count uint64. */
myql_status myql_rng_draws(myql_ctx *ctx, uint64_t seed, uint64_t first,
                           uint64_t n, uint64_t count, uint64_t *out);

/* --- numerics probes (device functions evaluated on host-provided inputs) -- */
/* FP64 chi-squared quantiles computed on the device, as used to build the
 * SchemeNCI tables (VolSchemes.hpp:240-313). */
myql_status myql_chi2_quantile(myql_ctx *ctx, const double *dof, const double *p,
                               double *out, size_t n);
/* The FP64 nodes of the SchemeNCI table of degrees-of-freedom offset d, rows
 * 0..rows-1 (row k: chi-squared with d + 2k degrees of freedom), as the table
 * build computes them before fitting the Hermite cells
 * (VolSchemes.hpp:240-313).  main_out: rows * 10000 quantiles at p = i * 0.999
 * / 9999; tail_out: rows * 512 upper-tail quantiles at q = exp(-w_j), w_j =
 * w0 + j (44.5 - w0) / 511, w0 = -log(0.001).  1 <= rows <= 1024. */
myql_status myql_probe_nci_nodes(myql_ctx *ctx, double d, int rows, double *main_out,
                                 double *tail_out);
/* FP32 device samplers on given 64-bit draws: kind 0 = inverse normal of the
 * uniform of x, kind 1 = inverse Poisson CDF with mean lambda[i] of the uniform
 * of x.  out: n floats. */
myql_status myql_probe_sampler(myql_ctx *ctx, int kind, const uint64_t *x,
                               const double *lambda, float *out, size_t n);

/* Measured issue-rate ceilings of this GPU for the compute roofline of the
 * path kernels: kind 0 = FP32 FMA lane operations per second, kind 1 = MUFU
 * (special-function) operations per second.  Runs a short dependent-chain
 * microbenchmark on every SM. */
myql_status myql_probe_peak(myql_ctx *ctx, int kind, double *ops_per_second);

/* --- neural martingale control variate (no counterpart in the reference) --
 * An MLP g(t/T, log(S/S0), v1, v2, average to date, 1) -> 128 -> 128 -> 128
 * (SiLU) -> 1 with BF16 weights and FP32 accumulation on the tensor cores,
 * trained on pilot paths of the same model (an independent seed) to minimise
 * Var(Y - C), C = sum_j g(state at t_j) dM_j, where dM_j is the increment of
 * the discounted asset S e^{-(r-q)t} over the j-th hedge interval, centred
 * step by step under the discretisation scheme.  E[C] = 0 for any network, so
 * the price estimator mean(Y - C) is unbiased; the plain estimator mean(Y) of
 * the same paths is returned beside it.  Scalar European and Asian
 * instruments; GreekMode is ignored (prices only). */
#define MYQL_CV_PARAMS 35332 /* FP32 parameters: W1[128][16] b1 W2[128][128] b2 W3[128][128] b3 w4[128] b4 (+3 pad) */
typedef struct myql_cv_config {
  uint32_t hedge_every;  /* time steps per hedge interval (hedge times t_j = j * hedge_every * dt) */
  uint32_t iterations;   /* Adam steps (<= 4096)                                                */
  uint64_t pilot_paths;  /* training paths (rounded up to a multiple of 128)                    */
  uint64_t batch_paths;  /* paths per Adam step                                                 */
  double learning_rate;  /* peak Adam step size (cosine decay to 5 %)                           */
  uint64_t seed;         /* network initialisation                                              */
} myql_cv_config;

typedef struct myql_cv_result {
  double price, price_std_err;             /* control-variate estimator              */
  double plain_price, plain_std_err;       /* plain Monte Carlo on the same paths    */
  double variance_ratio;                   /* Var(Y) / Var(Y - C)                    */
  double initial_loss, final_loss;         /* training: first / last minibatch loss  */
  double train_ms, simulate_ms, mlp_ms, total_ms;
  uint64_t paths;
  uint32_t kernel_launches;
} myql_cv_result;

/* Pilot simulation + training; the network stays in the context.  res (may be
 * NULL) reports the in-sample estimators on the first min(pilot_paths, 2^17)
 * pilot paths (res->paths = pilot paths trained on). */
myql_status myql_cv_train(myql_ctx *ctx, const myql_mc_job *job, const myql_cv_config *cfg,
                          myql_cv_result *res);
/* Prices job (its own seed, paths and streams) with the context's network. */
myql_status myql_cv_price(myql_ctx *ctx, const myql_mc_job *job, const myql_cv_config *cfg,
                          myql_cv_result *res);
/* Prices job with the context's network on randomized quasi-Monte Carlo paths
 * (the Sobol points, bridges and digital shifts of myql_qmc_price, same
 * restrictions: SchemeNV / SchemeNCI factors, no jumps or Merton jumps, at most
 * 512 steps, num_paths a multiple of 2048 * n_replicates, n_replicates >= 2).
 * price / plain_price: the means of the n_replicates replicate estimates of the
 * control-variate and the plain estimator; the standard errors and
 * variance_ratio come from their spreads. */
myql_status myql_cv_qmc_price(myql_ctx *ctx, const myql_mc_job *job, const myql_cv_config *cfg,
                              uint32_t n_replicates, myql_cv_result *res);
/* Network parameters (MYQL_CV_PARAMS floats): fresh initialisation, read, write. */
myql_status myql_cv_init(myql_ctx *ctx, uint64_t seed);
myql_status myql_cv_get_params(myql_ctx *ctx, float *params, size_t n);
myql_status myql_cv_set_params(myql_ctx *ctx, const float *params, size_t n);
/* The MLP kernels on caller data (checks against a CPU MLP): rows are
 * (path p, hedge j) at p * n_hedge + j; feats[row][6], dM[row], Y[path].
 * forward: cv[p] = sum_j g_j dM_j and g[row] (g may be NULL).
 * gradient: the gradient of L = mean_p (Y_p - cv_p - mean(Y - cv))^2 with
 * respect to the parameter blob, and L. */
myql_status myql_cv_forward(myql_ctx *ctx, const float *feats, const float *dM, uint64_t n_paths,
                            uint32_t n_hedge, float *cv, float *g);
myql_status myql_cv_gradient(myql_ctx *ctx, const float *feats, const float *dM, const float *Y,
                             uint64_t n_paths, uint32_t n_hedge, float *grad, double *loss);

/* MLMC with the control variate on every level: level 0 prices plain paths
 * minus sum_j g dM_j; level l > 0 the difference P_fine - P_coarse minus
 * sum_j g(fine state at t_j) (dM_fine,j - dM_coarse,j), each increment centred
 * under its own discretisation, hedged every max(1, coarse steps / 32) coarse
 * steps.  When cv->iterations > 0 the network is first trained on plain paths
 * of base_steps * 2^min(L_max, 5) steps (hedged every step); with 0 the
 * context's network is used.  plain_var (optional, MYQL_MLMC_MAX_LEVELS
 * doubles) receives the uncorrected level variances of the same paths.
 * Scalar European, Asian and barrier instruments; every path is stepped. */
myql_status myql_mlmc_cv_price(myql_ctx *ctx, const myql_mc_job *job, const myql_mlmc_config *mlmc,
                               const myql_cv_config *cv, myql_mlmc_result *res, double *plain_var);
/* One level of the above with the context's network: sums4 = {sum Y, sum Y^2,
 * sum (Y - C), sum (Y - C)^2} of dN discounted level differences Y. */
myql_status myql_mlmc_cv_level(myql_ctx *ctx, const myql_mc_job *job, const myql_mlmc_config *mlmc,
                               uint32_t level, uint64_t dN, double *sums4);

/* FP64 Gil-Pelaez prices of a European instrument (every model; vanilla,
 * cash- and asset-or-nothing payoffs), the oracle of the Monte Carlo prices:
 * FourierPricer (pricers/fourier/FourierPricer.hpp) with the characteristic
 * exponents of CFPolicies.hpp and AffineTraits.hpp, integrated by 256-panel
 * Gauss-Legendre quadrature on the GPU.  greek_mode Essential adds delta and
 * gamma, Full every Greek, as FP64 central differences of these prices.
 * out: MYQL_OUT_DOUBLES(n_strikes) doubles in the myql_mc_price layout
 * (standard errors 0).  The job's schemes and Monte Carlo settings are ignored. */
myql_status myql_fourier_price(myql_ctx *ctx, const myql_mc_job *job, int32_t greek_mode, double *out);

/* One-tile tcgen05 GEMM D[128][N] = A[128][K] * B[N][K]^T with the operands
 * rounded to BF16 and FP32 accumulation, through the shared-memory operand
 * layouts and descriptors the control-variate MLP kernels use: mode 0 K = 16,
 * N = 128; mode 1 K = 128, N = 128; mode 2 K = 128, N = 16; mode 3 K = 128,
 * N = 128 with both operands stored MN-major.  A ([128][K]), B ([N][K]) and
 * D ([128][N]) are row-major host arrays. */
myql_status myql_probe_mma(myql_ctx *ctx, int32_t mode, const float *A, const float *B, float *D);

#ifdef __cplusplus
}
#endif
#endif /* MYQL_GPU_H */
