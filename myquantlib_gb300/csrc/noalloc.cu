// noalloc.cu -- a pricing entry point that allocates no device memory.
//
// Some callers cannot allocate GPU memory while they price: an application
// whose device memory is owned by its own pool or by another framework's
// caching allocator, a real-time process that forbids allocation (and the
// device-wide synchronisation cudaMalloc/cudaFree can imply) after start-up,
// or an embedding that has no context object to hold buffers between calls.
// myql_mc_price_noalloc serves them: it prices one request with the same
// kernels as myql_mc_price, but every piece of scratch it needs (stream
// states, the strike strip, the per-path terminal records, the tile
// partials and the status words) lives in one fixed file-scope device array,
// g_scratch, of MYQL_NOALLOC_SCRATCH_BYTES.  That array is part of the
// library image: every GPU that loads the library holds it until the process
// exits.  Requests that do not fit are rejected with MYQL_ERR_TOO_LARGE.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>

#include "engine.h"
#include "myql_gpu.h"

namespace myql {

cudaError_t launch_simulate(const SimParams &P, int s1, int s2, bool path_dep, cudaStream_t stream);
cudaError_t launch_payoff(const PayoffParams &P, unsigned long long n_tiles, cudaStream_t stream);
cudaError_t launch_finalize(const FinalizeParams &P, cudaStream_t stream);
cudaError_t upload_jump_polys(const unsigned long long polys[64][4]);
cudaError_t launch_seed_streams(unsigned long long seed, unsigned long long first,
                                unsigned long long n, unsigned long long *out, cudaStream_t stream);
const unsigned long long (*jump_polynomials())[4];

// The whole scratch of the no-alloc entry point.  In host code `g_scratch`
// names a host-side stand-in, not the device array: its device address comes
// from cudaGetSymbolAddress, fetched once per device below.
static __device__ __align__(256) unsigned char g_scratch[MYQL_NOALLOC_SCRATCH_BYTES];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
unsigned char *g_scratch_dev[kMaxDevices] = {nullptr};  // device address of g_scratch per device

// Per-device set-up, done by the first call on each device with that device
// current: the scratch array's device address and the jump polynomials the
// stream-seeding kernel reads from constant memory.
myql_status setup_device(int device, unsigned char **scratch) {
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (g_scratch_dev[device]) {
    *scratch = g_scratch_dev[device];
    return MYQL_OK;
  }
  const unsigned long long(*polys)[4] = jump_polynomials();
  if (!polys) return set_error(MYQL_ERR_CUDA, "xoshiro256 jump polynomial check failed");
  void *ptr = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&ptr, g_scratch);
  if (e != cudaSuccess) return cuda_status(e, "cudaGetSymbolAddress(g_scratch)");
  e = upload_jump_polys(polys);
  if (e != cudaSuccess) return cuda_status(e, "jump polynomial upload");
  g_scratch_dev[device] = static_cast<unsigned char *>(ptr);
  *scratch = g_scratch_dev[device];
  return MYQL_OK;
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace
}  // namespace myql

using namespace myql;

extern "C" myql_status myql_mc_price_noalloc(int device, const myql_mc_job *job, double *out_dev,
                                             void *stream_ptr) {
  if (!job || !out_dev) return set_error(MYQL_ERR_INVALID_ARG, "null job or output");
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0) return set_error(MYQL_ERR_NO_DEVICE, "no CUDA device");
  if (device < 0 || device >= count || device >= kMaxDevices)
    return set_error(MYQL_ERR_INVALID_ARG, "bad device %d", device);
  e = cudaSetDevice(device);
  if (e != cudaSuccess) return cuda_status(e, "cudaSetDevice");
  myql_status s = validate_job(*job);
  if (s != MYQL_OK) return s;
  const myql_mc_config &c = job->config;
  if (c.greek_mode == MYQL_GREEKS_FULL)
    return set_error(MYQL_ERR_UNSUPPORTED, "the no-alloc entry point prices GreekMode None and Essential");
  for (int f = 0; f < job->model.num_factors; ++f)
    if (c.scheme[f] == MYQL_SCHEME_NCI)
      return set_error(MYQL_ERR_UNSUPPORTED,
                       "the no-alloc entry point has no room for SchemeNCI tables (use NV or Exact)");
  unsigned char *scratch = nullptr;
  s = setup_device(device, &scratch);
  if (s != MYQL_OK) return s;

  // ---- plan of one scenario (the same constants myql_mc_price sets up)
  const myql_model &m = job->model;
  const myql_instrument &in = job->instrument;
  const uint64_t M = c.num_paths;
  // the stream rule of myql_mc_price: the same streams, so the same paths and result
  const uint64_t S = std::min<uint64_t>(c.n_streams ? c.n_streams : default_streams(M), M);
  if (S > (1u << 26)) return set_error(MYQL_ERR_TOO_LARGE, "at most 2^26 streams");
  const int steps = (int)c.time_steps;
  const int tracker = tracker_of(in);
  const bool path_dep = tracker != TRK_EUROPEAN;
  const int F = tracker_fields(tracker);
  const int nk = (int)in.n_strikes;
  const double S0 = job->S0, r = job->r, q = job->q, T = in.maturity, dt = T / (double)steps;
  const double h = S0 * c.fd_bump;
  const bool greeks = c.greek_mode != MYQL_GREEKS_NONE;
  const int tile_paths = 2048;
  const uint64_t tiles = (M + tile_paths - 1) / tile_paths;

  // ---- scratch layout and limits
  size_t off = 0;
  const size_t off_status = off;
  off = align256(off + 16);
  const size_t off_strikes = off;
  off = align256(off + (size_t)nk * sizeof(double));
  const size_t off_states = off;
  off = align256(off + (size_t)S * 32);
  const size_t off_partials = off;
  off = align256(off + (size_t)tiles * nk * 2 * kQ * sizeof(double));
  const size_t off_records = off;
  off = align256(off + (size_t)M * F * sizeof(float));
  if (off > (size_t)MYQL_NOALLOC_SCRATCH_BYTES)
    return set_error(MYQL_ERR_TOO_LARGE,
                     "request needs %zu bytes of scratch; the no-alloc entry point has %d (fewer paths, "
                     "streams or strikes fit)", off, (int)MYQL_NOALLOC_SCRATCH_BYTES);

  SimParams P;
  std::memset(&P, 0, sizeof P);
  P.n_sc = 1;
  P.n_factors = m.num_factors;
  P.jump_kind = m.jump;
  P.tracker = tracker;
  P.n_steps = steps;
  P.n_fields = F;
  P.n_streams = (uint32_t)S;
  P.loop_cap = kDefaultLoopCap;
  P.path_begin = 0;
  P.path_end = M;
  P.num_paths = M;
  P.rec_offset = 0;
  P.rec_stride = M;
  P.merton_mu = (float)m.merton_mu;
  P.merton_delta = (float)m.merton_delta;
  P.kou_p_up = (float)m.kou_p_up;
  P.kou_inv_eta1 = m.jump == MYQL_JUMP_KOU ? (float)(1.0 / m.kou_eta1) : 0.0f;
  P.kou_inv_eta2 = m.jump == MYQL_JUMP_KOU ? (float)(1.0 / m.kou_eta2) : 0.0f;
  P.nci_u999 = u999_threshold();
  if (in.kind == MYQL_INSTR_BARRIER) {
    const double lb = std::log(in.barrier) - std::log(S0);
    P.b_log[0] = (float)lb;
    P.b_log[1] = greeks ? (float)(std::log(in.barrier * S0 / (S0 + h)) - std::log(S0)) : (float)lb;
    P.b_log[2] = greeks ? (float)(std::log(in.barrier * S0 / (S0 - h)) - std::log(S0)) : (float)lb;
  }
  P.lb_min0 = in.hist_min_S > 0.0 ? (float)(std::log(in.hist_min_S) - std::log(S0)) : 0.0f;
  P.lb_max0 = in.hist_max_S > 0.0 ? (float)(std::log(in.hist_max_S) - std::log(S0)) : 0.0f;
  for (int f = 0; f < m.num_factors; ++f) {
    const myql_heston_params &hp = m.heston[f];
    const double ab = 2.0 * hp.kappa * hp.theta / (hp.sigma * hp.sigma);
    if (ab <= 1.0 && ab > 0.0) {
      const double ee = 2.71828182845904523536, pp = ee / (ab + ee);
      P.sm_p[f] = (float)pp;
      P.sm_inv_p[f] = (float)(1.0 / pp);
      P.sm_1mp[f] = (float)(1.0 - pp);
      P.sm_1ma[f] = (float)(1.0 - ab);
      P.sm_inv_a[f] = (float)(1.0 / ab);
    }
  }
  ScenarioConst &C = P.sc[0];
  C.dt = (float)dt;
  C.t_end = (float)(dt * steps);
  if (m.num_factors == 0) {
    const double drift_dt = (r - q - 0.5 * m.vol * m.vol) * dt, vol_dt = m.vol * std::sqrt(dt);
    C.gbm_drift = (float)(path_dep ? drift_dt : drift_dt * steps);
    C.gbm_vol = (float)(path_dep ? vol_dt : vol_dt * std::sqrt((double)steps));
  } else {
    const double r_part = (r - q) / (double)m.num_factors;
    for (int f = 0; f < m.num_factors; ++f)
      fill_factor(C.f[f], m.heston[f], m.heston[f].v0, c.scheme[f], r_part, dt);
  }
  if (m.jump != MYQL_JUMP_NONE) {
    const double k = m.jump == MYQL_JUMP_MERTON
                         ? std::exp(m.merton_mu + 0.5 * m.merton_delta * m.merton_delta) - 1.0
                         : (m.kou_p_up * m.kou_eta1) / (m.kou_eta1 - 1.0) +
                               ((1.0 - m.kou_p_up) * m.kou_eta2) / (m.kou_eta2 + 1.0) - 1.0;
    const double window = path_dep ? dt : T, mean = m.jump_lambda * window;
    C.jump_mean = (float)mean;
    C.jump_exp_neg_mean = (float)std::exp(-mean);
    C.jump_comp = (float)(-m.jump_lambda * k * window);
  }
  P.states = reinterpret_cast<unsigned long long *>(scratch + off_states);
  P.records = reinterpret_cast<float *>(scratch + off_records);
  P.status = reinterpret_cast<unsigned int *>(scratch + off_status);

  PayoffParams Q;
  std::memset(&Q, 0, sizeof Q);
  Q.n_sc = 1;
  Q.n_fields = F;
  Q.tracker = tracker;
  Q.kind = in.kind;
  Q.payoff = in.payoff;
  Q.option_type = in.option_type;
  Q.fixed_strike = in.fixed_strike;
  Q.barrier_action = in.barrier_action;
  Q.rebate_timing = in.rebate_timing;
  Q.mode = c.greek_mode;
  Q.n_factors = m.num_factors;
  Q.n_strikes = nk;
  Q.n_paths = M;
  Q.rec_stride = M;
  Q.tile0 = 0;
  Q.tile_paths = tile_paths;
  Q.strikes = reinterpret_cast<const double *>(scratch + off_strikes);
  Q.records = P.records;
  Q.partials = reinterpret_cast<double *>(scratch + off_partials);
  Q.S0 = (float)S0;
  Q.eps_rel = (float)c.fd_bump;
  Q.rebate = (float)in.rebate;
  Q.barrier_rate = (float)in.barrier_rate;
  Q.T_instr = (float)T;
  if (greeks && in.payoff != MYQL_PAYOFF_VANILLA && in.kind != MYQL_INSTR_BARRIER) {
    double eps = in.payoff_eps;
    if (eps < 0.0) {
      double var = jump_variance(m);
      if (m.num_factors == 0) var += m.vol * m.vol;
      for (int f = 0; f < m.num_factors; ++f) var += expected_avg_variance(m.heston[f], T);
      eps = std::sqrt(var) * (in.is_strip ? S0 : in.strikes[0]) * std::sqrt(T) / 10.0;
    }
    Q.smooth = 1;
    Q.smooth_eps = (float)(1.0 / (eps * std::sqrt(2.0)));
  }
  const double Ttot = dt * steps + in.t_elapsed;
  if (tracker == TRK_GEO_ASIAN) {
    Q.avg_c0[0] = (float)((in.past_avg_log * in.t_elapsed + std::log(S0) * dt * steps) / Ttot - std::log(S0));
    Q.avg_c1[0] = (float)(1.0 / Ttot);
  } else if (tracker == TRK_ARITH_ASIAN) {
    Q.avg_c0[0] = (float)(in.past_avg_S * in.t_elapsed / (S0 * Ttot));
    Q.avg_c1[0] = (float)(1.0 / Ttot);
  }
  if (greeks) {
    Q.inv_2h = (float)(1.0 / (2.0 * h));
    Q.inv_h2 = (float)(1.0 / (h * h));
  }

  // ---- launches: every kernel reads and writes only g_scratch and out_dev
  cudaStream_t st = static_cast<cudaStream_t>(stream_ptr);
  e = cudaMemsetAsync(scratch + off_status, 0, 16, st);  // status words start at zero
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(scratch + off_strikes, in.strikes, (size_t)nk * sizeof(double),
                        cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = launch_seed_streams(c.seed, c.stream_offset, S, P.states, st);
  if (e == cudaSuccess) e = launch_simulate(P, P.n_factors >= 1 ? c.scheme[0] : 0,
                                            P.n_factors >= 2 ? c.scheme[1] : 0, path_dep, st);
  if (e == cudaSuccess) e = launch_payoff(Q, tiles, st);
  FinalizeParams Fz;
  Fz.n_strikes = nk;
  Fz.n_tiles = tiles;
  Fz.partials = Q.partials;
  Fz.out = out_dev;
  Fz.inv_m = 1.0 / (double)M;
  Fz.df = std::exp(-r * T);
  Fz.active_mask = greeks ? 0x7 : 0x1;
  if (e == cudaSuccess) e = launch_finalize(Fz, st);
  unsigned int hs[4] = {0, 0, 0, 0};
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(hs, scratch + off_status, 16, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_status(e, "no-alloc pricing");
  if (hs[0]) return set_error(MYQL_ERR_LOOP_CAP, "%u bounded device loops hit their cap", hs[0]);
  return MYQL_OK;
}
