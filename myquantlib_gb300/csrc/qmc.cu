// qmc.cu -- randomized quasi-Monte Carlo pricing (myql_qmc_price).
//
// The reference lists quasi-Monte Carlo as future work (README.md:331).  Here a
// path's normals come from a Sobol point instead of xoshiro draws:
//   * Sobol points in Gray-code order (Antonov-Saleev), generated a warp at a time:
//     32 consecutive points share the Gray code's high bits, so one pass over 32
//     dimensions builds their 32 x 32 coordinates in shared memory (SobolWarp);
//     direction numbers from primitive polynomials over GF(2) by the Bratley-Fox
//     recurrence (ACM TOMS 659), dimension 0 the van der Corput sequence.  The
//     initial direction numbers m_1..m_s of each dimension are odd integers
//     m_k < 2^k drawn from splitmix64 with a fixed seed (a randomly initialised
//     Sobol sequence, not a published table), the same for every job;
//   * each Gaussian motion (the spot's and one per SchemeNV factor) is built by
//     a Brownian bridge on the step grid in segments of 32 steps: first its
//     values at the segment boundaries (breadth first, end point first), so
//     that the lowest Sobol dimensions carry the paths' coarse shape, then per
//     segment the interior of its bridge (breadth first); the motions
//     interleave at every bridge point.  A thread holds one segment's values
//     at a time (a whole-path bridge in local memory spilled to DRAM);
//   * R independent random digital shifts (one 32-bit XOR mask per replicate and
//     dimension) give R unbiased replicate estimates; the price is their mean and
//     the standard error comes from their spread.
// QMC needs a fixed number of draws per step, and these steppers have one:
//   * SchemeNV factors: one normal per step (VolSchemes.hpp:52-57), from a bridge
//     like the spot's;
//   * SchemeNCI factors: two uniforms per step (VolSchemes.hpp:334-370), the
//     Poisson count's by inversion and the chi-squared table's, taken directly
//     from two Sobol coordinates;
//   * Merton jumps: two uniforms per step, the count's by sequential inversion
//     and the normal of the jump sum (n mu + sqrt(n) delta Z, JumpPolicies.hpp:55-75);
//     the jumps of every instrument are drawn per step, whose sum has the law of
//     the one draw over T a European stepper makes.
// Dimension order: the boundary points (NG per point), then per segment its
// interior bridge points (NG each) followed by its steps' uniforms (NU each), so
// a path consumes its dimensions strictly in order.  SchemeExact (a
// rejection loop) and Kou jumps (one exponential per jump) have a variable number
// of draws and are not offered.  The log-spot steps as in ASVJstepper.hpp:134-229,
// with the trackers of the path kernels; the per-path records go through the
// engine's own payoff pass.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <utility>
#include <vector>

#include "qmc.cuh"

namespace myql {
namespace dev {

template <int NF, bool PD>
__global__ void __launch_bounds__(kSimBlock) qmc_kernel(const __grid_constant__ QmcParams Q) {
  // the grid covers path_end exactly (a multiple of 2048 paths) and n_pts is a multiple of
  // 2048, so every warp is full and its 32 points are consecutive within one replicate
  __shared__ uint32_t sobol_tab[kSimBlock / 32][32 * 32];
  const SimParams &P = Q.P;
  const unsigned long long i = blockIdx.x * (unsigned long long)kSimBlock + threadIdx.x;
  SobolWarp sob = sobol_warp(Q, sobol_tab[threadIdx.x >> 5], i);
  unsigned int caphits = 0, fallbacks = 0;
  float out[kMaxFields];
  NoHook h;
  qmc_path<NF, PD>(Q, sob, out, caphits, fallbacks, h);
  const int F = P.n_fields;
  for (int f = 0; f < F; ++f) P.records[(size_t)f * P.rec_stride + i] = out[f];
  if (caphits) atomicAdd(P.status, caphits);
  if (fallbacks) atomicAdd(P.status + 1, fallbacks);
}

// The control variate's Sobol paths: as cv_sim_kernel (features at the hedge times, centred
// martingale increments, the discounted payoff in place), one thread per point.
template <int NF>
__global__ void __launch_bounds__(kSimBlock) qmc_cv_kernel(const __grid_constant__ QmcCvParams C) {
  __shared__ uint32_t sobol_tab[kSimBlock / 32][32 * 32];
  const SimParams &P = C.Q.P;
  const unsigned long long li = blockIdx.x * (unsigned long long)kSimBlock + threadIdx.x;  // launch-local
  SobolWarp sob = sobol_warp(C.Q, sobol_tab[threadIdx.x >> 5], C.path_begin + li);
  const unsigned long long pb = li >> 7;
  CvHook h;
  h.P = &C.fc;
  h.lane = (uint32_t)(li & 127u);
  h.tile0 = C.feat + pb * (unsigned long long)C.n_hedge * kCvTileBytes;
  h.dm0 = C.dM + pb * (unsigned long long)C.n_hedge * 128ull + h.lane;
  h.he = C.hedge_every;
  h.n = P.n_steps;
  h.dt = P.sc[0].dt;
  unsigned int caphits = 0, fallbacks = 0;
  float r[kMaxFields];
  qmc_path<NF, true>(C.Q, sob, r, caphits, fallbacks, h);
  const PathView v = record_view(C.pay, r);
  C.Y[li] = (float)C.df * scenario_tri(C.pay, v, (float)C.pay.strikes[0], false).v;
  if (caphits) atomicAdd(P.status, caphits);
  if (fallbacks) atomicAdd(P.status + 1, fallbacks);
}

}  // namespace dev

namespace dev {
// out[i] = high word of splitmix64 value i + 1 of the sequence started at s0 (the host's
// splitmix(s) called i + 1 times): z = s0 + (i + 1) * golden, then the finaliser
__global__ void qmc_shift_kernel(unsigned long long s0, unsigned long long n, uint32_t *out) {
  const unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  unsigned long long z = s0 + (i + 1ull) * 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  out[i] = (uint32_t)((z ^ (z >> 31)) >> 32);
}
}  // namespace dev

static cudaError_t launch_qmc_shifts(unsigned long long s0, unsigned long long n, uint32_t *out, cudaStream_t st) {
  dev::qmc_shift_kernel<<<(unsigned int)((n + 255) / 256), 256, 0, st>>>(s0, n, out);
  return cudaGetLastError();
}

static cudaError_t launch_qmc(const QmcParams &Q, int nf, bool pd, cudaStream_t st) {
  const unsigned int grid = (unsigned int)((Q.P.path_end + kSimBlock - 1) / kSimBlock);
  switch (nf * 2 + (pd ? 1 : 0)) {
    case 0: dev::qmc_kernel<0, false><<<grid, kSimBlock, 0, st>>>(Q); break;
    case 1: dev::qmc_kernel<0, true><<<grid, kSimBlock, 0, st>>>(Q); break;
    case 2: dev::qmc_kernel<1, false><<<grid, kSimBlock, 0, st>>>(Q); break;
    case 3: dev::qmc_kernel<1, true><<<grid, kSimBlock, 0, st>>>(Q); break;
    case 4: dev::qmc_kernel<2, false><<<grid, kSimBlock, 0, st>>>(Q); break;
    case 5: dev::qmc_kernel<2, true><<<grid, kSimBlock, 0, st>>>(Q); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

// n_paths: a multiple of 2048 (whole warps of one replicate, whole 128-path tiles)
cudaError_t launch_qmc_cv(const QmcCvParams &P, unsigned long long n_paths, int nf, cudaStream_t st) {
  if (n_paths == 0 || n_paths % 2048 != 0 || P.path_begin % 2048 != 0) return cudaErrorInvalidValue;
  const unsigned int grid = (unsigned int)(n_paths / kSimBlock);
  switch (nf) {
    case 0: dev::qmc_cv_kernel<0><<<grid, kSimBlock, 0, st>>>(P); break;
    case 1: dev::qmc_cv_kernel<1><<<grid, kSimBlock, 0, st>>>(P); break;
    case 2: dev::qmc_cv_kernel<2><<<grid, kSimBlock, 0, st>>>(P); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

// ---------------------------------------------------------------------- host
namespace {

uint64_t splitmix(uint64_t &s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// x^e mod p over GF(2), p of degree s given with its x^s bit
uint32_t gf2_powmod(uint64_t e, uint32_t p, int s) {
  auto mulmod = [&](uint32_t a, uint32_t b) {
    uint32_t r = 0;
    while (b) {
      if (b & 1u) r ^= a;
      b >>= 1;
      a <<= 1;
      if (a >> s & 1u) a ^= p;
    }
    return r;
  };
  uint32_t r = 1, base = s == 1 ? 1u : 2u;  // x mod p (x mod (x + 1) = 1)
  while (e) {
    if (e & 1u) r = mulmod(r, base);
    base = mulmod(base, base);
    e >>= 1;
  }
  return r;
}

// primitive: x has multiplicative order 2^s - 1 modulo p
bool primitive(uint32_t p, int s) {
  const uint64_t order = (1ull << s) - 1;
  if (gf2_powmod(order, p, s) != 1u) return false;
  uint64_t m = order;
  for (uint64_t q = 2; q * q <= m; ++q) {
    if (m % q) continue;
    while (m % q == 0) m /= q;
    if (gf2_powmod(order / q, p, s) == 1u) return false;
  }
  if (m > 1 && m != order && gf2_powmod(order / m, p, s) == 1u) return false;
  return true;
}

// The first `count` primitive polynomials (with their degrees) in order of degree, then of
// coefficients, up to degree 20.  The search does not depend on the seed, so it runs once
// per process and grows as larger dimension counts are asked for; callers get a copy.
std::vector<std::pair<uint32_t, int>> primitive_polys(size_t count) {
  static std::mutex mu;
  static std::vector<std::pair<uint32_t, int>> polys;
  static int next_s = 1;
  static uint32_t next_low = 0;
  std::lock_guard<std::mutex> lock(mu);
  while (polys.size() < count && next_s <= 20) {
    const uint32_t p = (1u << next_s) | (next_low << 1) | 1u;  // x^s + a_1 x^(s-1) + ... + 1
    if (primitive(p, next_s)) polys.push_back({p, next_s});
    if (++next_low == 1u << (next_s - 1)) {
      next_low = 0;
      ++next_s;
    }
  }
  return std::vector<std::pair<uint32_t, int>>(polys.begin(), polys.begin() + std::min(count, polys.size()));
}

// direction numbers of D dimensions, [D][32]; dimension d >= 1 takes the d-th primitive
// polynomial, and the seed's splitmix stream draws its initial m_1..m_s in that order
std::vector<uint32_t> sobol_directions(unsigned int D, uint64_t seed) {
  std::vector<uint32_t> V((size_t)D * kQmcBits, 0u);
  for (int k = 1; k <= kQmcBits; ++k) V[k - 1] = 1u << (kQmcBits - k);  // van der Corput
  const std::vector<std::pair<uint32_t, int>> polys = primitive_polys(D - 1);
  uint64_t rs = seed ^ 0xD1B54A32D192ED03ull;
  uint64_t m[kQmcBits + 1];
  for (unsigned int d = 1; d < D && d - 1 < polys.size(); ++d) {
    const uint32_t p = polys[d - 1].first;
    const int s = polys[d - 1].second;
    for (int k = 1; k <= s && k <= kQmcBits; ++k) m[k] = ((splitmix(rs) % (1ull << (k - 1))) << 1) | 1ull;
    for (int k = s + 1; k <= kQmcBits; ++k) {
      uint64_t v = m[k - s] ^ (m[k - s] << s);
      for (int j = 1; j < s; ++j)
        if (p >> (s - j) & 1u) v ^= m[k - j] << j;  // coefficient a_j of x^(s-j)
      m[k] = v;
    }
    for (int k = 1; k <= kQmcBits; ++k) V[(size_t)d * kQmcBits + k - 1] = (uint32_t)(m[k] << (kQmcBits - k));
  }
  return V;
}

struct Bridge {
  std::vector<int> mid, left, right;
  std::vector<float> wl, wr, sd;
};

// Brownian bridge schedule on the unit step grid 0..n in segments of kQmcSeg steps.
// First the bridge over the segment boundaries 0, L, 2L, .., n (breadth first, indices in
// segments, the end point first), then per segment the bridge over its interior points
// (breadth first, in steps from the segment's start).  n entries in all.
Bridge segmented_bridge(int n) {
  const int L = kQmcSeg, ns = (n + L - 1) / L;
  auto pos = [&](int s) { return std::min(s * L, n); };
  Bridge B;
  auto push = [&](int m, int l, int r, double tm, double tl, double tr) {
    B.mid.push_back(m);
    B.left.push_back(l);
    B.right.push_back(r);
    B.wl.push_back((float)((tr - tm) / (tr - tl)));
    B.wr.push_back((float)((tm - tl) / (tr - tl)));
    B.sd.push_back((float)std::sqrt((tm - tl) * (tr - tm) / (tr - tl)));
  };
  auto breadth_first = [&](int a, int b, auto t) {  // interior points of (a, b), t(index) = step
    std::vector<std::pair<int, int>> q{{a, b}};
    for (size_t h = 0; h < q.size(); ++h) {
      const int l = q[h].first, r = q[h].second;
      if (r - l < 2) continue;
      const int m = (l + r) / 2;
      push(m, l, r, t(m), t(l), t(r));
      q.push_back({l, m});
      q.push_back({m, r});
    }
  };
  B.mid.push_back(ns);  // the end point: W(n) ~ N(0, n)
  B.left.push_back(0);
  B.right.push_back(0);
  B.wl.push_back(0.0f);
  B.wr.push_back(0.0f);
  B.sd.push_back((float)std::sqrt((double)n));
  breadth_first(0, ns, [&](int s) { return (double)pos(s); });
  for (int s = 0; s < ns; ++s) breadth_first(0, pos(s + 1) - pos(s), [](int k) { return (double)k; });
  return B;
}

struct QmcState : ExtState {
  DevBuf dirs, shift, bridge;
  unsigned int dirs_D = 0;
  uint64_t dirs_seed = kQmcDirectionSeed;  // the point set in use
  uint64_t want_seed = kQmcDirectionSeed;  // the point set asked for
  int bridge_n = -1;
};

QmcState &qmc_state(CtxBase *ctx) {
  if (!ctx->qmc) ctx->qmc.reset(new QmcState);
  return *static_cast<QmcState *>(ctx->qmc.get());
}

}  // namespace

extern "C" myql_status myql_ctx_set_qmc_direction_seed(myql_ctx *ctx_, uint64_t seed) {
  CtxBase *ctx = reinterpret_cast<CtxBase *>(ctx_);
  if (!ctx) return set_error(MYQL_ERR_INVALID_ARG, "null context");
  qmc_state(ctx).want_seed = seed;
  return MYQL_OK;
}

extern "C" myql_status myql_qmc_directions(uint32_t D, uint64_t seed, uint32_t *out) {
  if (!out || D == 0 || D > 1u << 16) return set_error(MYQL_ERR_INVALID_ARG, "need 1 <= D <= 65536 and an output");
  const std::vector<uint32_t> V = sobol_directions(D, seed);
  if (V[(size_t)(D - 1) * kQmcBits] == 0u) return set_error(MYQL_ERR_TOO_LARGE, "too many dimensions");
  std::memcpy(out, V.data(), V.size() * 4);
  return MYQL_OK;
}

myql_status qmc_prepare(CtxBase *ctx, const myql_mc_job &job, const Plan &pl, uint64_t R, QmcParams &Q) {
  const int nf = job.model.num_factors;
  int n_nv = 0, n_nci = 0;
  for (int f = 0; f < nf; ++f) {
    if (job.config.scheme[f] == MYQL_SCHEME_NV) ++n_nv;
    else if (job.config.scheme[f] == MYQL_SCHEME_NCI) ++n_nci;
    else
      return set_error(MYQL_ERR_UNSUPPORTED,
                       "quasi-Monte Carlo steps the CIR factors with SchemeNV or SchemeNCI (SchemeExact's "
                       "rejection loop has no fixed number of draws)");
  }
  if (job.model.jump == MYQL_JUMP_KOU)
    return set_error(MYQL_ERR_UNSUPPORTED,
                     "quasi-Monte Carlo supports Merton jumps or none (Kou draws one exponential per jump)");
  const uint64_t M = job.config.num_paths;
  if (R < 2 || M % (R * 2048ull) != 0)
    return set_error(MYQL_ERR_INVALID_ARG, "quasi-Monte Carlo needs >= 2 replicates and num_paths a multiple "
                                           "of 2048 x replicates");
  if (M / R > (1ull << 32)) return set_error(MYQL_ERR_TOO_LARGE, "at most 2^32 points per replicate");
  if (pl.steps > kQmcMaxSteps) return set_error(MYQL_ERR_UNSUPPORTED, "quasi-Monte Carlo takes at most 512 steps");
  QmcState &S = qmc_state(ctx);
  const int NG = 1 + n_nv, NU = 2 * n_nci + (job.model.jump == MYQL_JUMP_MERTON ? 2 : 0);
  const unsigned int D = (unsigned int)pl.steps * (unsigned int)(NG + NU);
  const uint64_t seed = job.config.seed;
  cudaStream_t st = ctx->stream;
  cudaError_t e = cudaSuccess;
  // tables: direction numbers, shifts, bridge
  // one point set per dimension count and direction seed (the context's, by default
  // kQmcDirectionSeed); the job's seed draws the digital shifts, which alone make the
  // replicates independent
  if (S.dirs_D != D || S.dirs_seed != S.want_seed) {
    const std::vector<uint32_t> V = sobol_directions(D, S.want_seed);
    if ((size_t)D * kQmcBits > V.size() || V[(size_t)(D - 1) * kQmcBits] == 0u)
      return set_error(MYQL_ERR_TOO_LARGE, "too many quasi-Monte Carlo dimensions");
    std::vector<uint32_t> Vt(V.size());  // bit-major on the device: a warp's dimensions are contiguous
    for (unsigned int d = 0; d < D; ++d)
      for (int k = 0; k < kQmcBits; ++k) Vt[(size_t)k * D + d] = V[(size_t)d * kQmcBits + k];
    e = S.dirs.ensure(Vt.size() * 4);
    if (e == cudaSuccess) e = cudaMemcpy(S.dirs.p, Vt.data(), Vt.size() * 4, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_status(e, "Sobol directions");
    S.dirs_D = D;
    S.dirs_seed = S.want_seed;
  }
  // the digital shifts: the high words of the splitmix64 sequence from seed ^ constant, drawn on
  // the device (value i of the counter-based sequence directly)
  const uint64_t n_shift = R * (uint64_t)D;
  e = S.shift.ensure(n_shift * 4);
  if (e == cudaSuccess) e = launch_qmc_shifts(seed ^ 0x8BB84B93962EACC9ull, n_shift, (uint32_t *)S.shift.p, st);
  if (e != cudaSuccess) return cuda_status(e, "digital shifts");
  ctx->launches++;
  const int n = pl.steps;
  if (S.bridge_n != n) {
    const Bridge B = segmented_bridge(n);
    std::vector<uint8_t> blob((size_t)n * 24);
    std::memcpy(blob.data(), B.mid.data(), n * 4);
    std::memcpy(blob.data() + 4 * n, B.left.data(), n * 4);
    std::memcpy(blob.data() + 8 * n, B.right.data(), n * 4);
    std::memcpy(blob.data() + 12 * n, B.wl.data(), n * 4);
    std::memcpy(blob.data() + 16 * n, B.wr.data(), n * 4);
    std::memcpy(blob.data() + 20 * n, B.sd.data(), n * 4);
    e = S.bridge.ensure(blob.size());
    if (e == cudaSuccess) e = cudaMemcpy(S.bridge.p, blob.data(), blob.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_status(e, "Brownian bridge");
    S.bridge_n = n;
  }
  std::memset(&Q, 0, sizeof Q);
  Q.P = pl.sim;
  Q.dirs = (const uint32_t *)S.dirs.p;
  Q.shift = (const uint32_t *)S.shift.p;
  const uint8_t *bb = (const uint8_t *)S.bridge.p;
  Q.br_mid = (const int *)bb;
  Q.br_left = (const int *)(bb + 4 * n);
  Q.br_right = (const int *)(bb + 8 * n);
  Q.br_wl = (const float *)(bb + 12 * n);
  Q.br_wr = (const float *)(bb + 16 * n);
  Q.br_sd = (const float *)(bb + 20 * n);
  Q.n_pts = M / R;
  Q.D = D;
  Q.NG = NG;
  Q.NU = NU;
  Q.jump = job.model.jump == MYQL_JUMP_MERTON ? 1 : 0;
  for (int f = 0; f < nf; ++f) {
    Q.sch[f] = job.config.scheme[f] == MYQL_SCHEME_NCI ? dev::SCH_NCI : dev::SCH_NV;
    if (Q.sch[f] == dev::SCH_NCI) {
      myql_status s = ensure_nci(ctx, job.model.heston[f], (double)pl.sim.sc[0].dt, Q.P.nci[f]);
      if (s != MYQL_OK) return s;
    }
  }
  Q.P.loop_cap = ctx->loop_cap;
  return MYQL_OK;
}

extern "C" myql_status myql_qmc_price(myql_ctx *ctx_, const myql_mc_job *job, uint32_t n_replicates,
                                      double *out, myql_mc_stats *stats) {
  CtxBase *ctx = reinterpret_cast<CtxBase *>(ctx_);
  if (!ctx || !job || !out) return set_error(MYQL_ERR_INVALID_ARG, "null argument");
  myql_status s = validate_job(*job);
  if (s != MYQL_OK) return s;
  if (job->config.greek_mode != MYQL_GREEKS_NONE)
    return set_error(MYQL_ERR_UNSUPPORTED, "quasi-Monte Carlo prices only (GreekMode None)");
  const uint64_t M = job->config.num_paths, R = n_replicates;
  Plan pl;
  s = make_plan(*job, pl, true);
  if (s != MYQL_OK) return s;
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) return cuda_status(e, "cudaSetDevice");
  cudaStream_t st = ctx->stream;
  ctx->launches = 0;
  ctx->phase_reset();
  e = cudaEventRecord(ctx->ev0, st);
  if (e != cudaSuccess) return cuda_status(e, "event");
  QmcParams Q;
  s = qmc_prepare(ctx, *job, pl, R, Q);
  if (s != MYQL_OK) return s;
  const int n = pl.steps, nf = job->model.num_factors;
  // buffers: records (one scenario), strikes, tile partials
  const int nk = (int)job->instrument.n_strikes;
  const uint64_t tiles = M / 2048;
  e = ctx->records.ensure(M * pl.n_fields * 4);
  if (e == cudaSuccess) e = ctx->strikes.ensure(nk * sizeof(double));
  if (e == cudaSuccess) e = ctx->partials.ensure(tiles * (uint64_t)nk * 2 * kQ * sizeof(double));
  if (e == cudaSuccess) e = ctx->status.ensure(16);
  if (e == cudaSuccess) e = cudaMemsetAsync(ctx->status.p, 0, 16, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(ctx->strikes.p, job->instrument.strikes, nk * sizeof(double), cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return cuda_status(e, "quasi-Monte Carlo buffers");
  Q.P.records = (float *)ctx->records.p;
  Q.P.status = (unsigned int *)ctx->status.p;
  Q.P.rec_stride = M;
  Q.P.path_begin = 0;
  Q.P.path_end = M;
  Q.P.rec_offset = 0;
  cudaEvent_t sa = ctx->phase_event(), sb = ctx->phase_event();
  cudaEventRecord(sa, st);
  e = launch_qmc(Q, nf, pl.path_dep, st);
  cudaEventRecord(sb, st);
  ctx->ev_tags.push_back(0);
  if (e != cudaSuccess) return cuda_status(e, "quasi-Monte Carlo launch");
  ctx->launches++;
  PayoffParams PQ = pl.pay;
  PQ.records = (const float *)ctx->records.p;
  PQ.rec_stride = M;
  PQ.partials = (double *)ctx->partials.p;
  PQ.strikes = (const double *)ctx->strikes.p;
  PQ.n_paths = M;
  PQ.tile0 = 0;
  cudaEvent_t pa = ctx->phase_event(), pb = ctx->phase_event();
  cudaEventRecord(pa, st);
  e = launch_payoff(PQ, tiles, st);
  cudaEventRecord(pb, st);
  ctx->ev_tags.push_back(1);
  if (e != cudaSuccess) return cuda_status(e, "payoff launch");
  ctx->launches++;
  e = cudaEventRecord(ctx->ev1, st);
  std::vector<double> part(tiles * (uint64_t)nk * 2 * kQ);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(part.data(), ctx->partials.p, part.size() * sizeof(double), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_status(e, "quasi-Monte Carlo run");
  // replicate estimates (tiles never straddle replicates) -> mean and its standard error
  const uint64_t tpr = tiles / R;
  std::memset(out, 0, MYQL_OUT_DOUBLES(nk) * sizeof(double));
  for (int k = 0; k < nk; ++k) {
    double sum = 0.0, sum_sq = 0.0;
    for (uint64_t r = 0; r < R; ++r) {
      double t = 0.0;
      for (uint64_t tl = r * tpr; tl < (r + 1) * tpr; ++tl) t += part[(tl * nk + k) * 2 * kQ];
      const double est = t / (double)Q.n_pts * pl.df;
      sum += est;
      sum_sq += est * est;
    }
    const double mean = sum / (double)R;
    const double var = std::max(sum_sq / (double)R - mean * mean, 0.0) * (double)R / (double)(R - 1);
    out[k] = mean;
    out[nk + k] = std::sqrt(var / (double)R);
  }
  myql_mc_stats local{};
  myql_mc_stats *stt = stats ? stats : &local;
  std::memset(stt, 0, sizeof *stt);
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
  stt->device_ms = ms;
  stt->paths = M;
  stt->scenarios = 1;
  stt->path_steps = M * (uint64_t)n;
  stt->kernel_launches = ctx->launches;
  phase_times(ctx, &stt->simulate_ms, &stt->payoff_ms);
  return read_status(ctx, stt);
}

}  // namespace myql
