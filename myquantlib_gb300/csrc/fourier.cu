// fourier.cu -- FP64 Gil-Pelaez prices of European instruments on the GPU: the
// FP64 oracle the Monte Carlo prices are checked against.
//
// Follows the reference's FourierPricer (pricers/fourier/FourierPricer.hpp,
// engines/fourier/kernels/GilPelaezKernel.hpp:21-100, CFPolicies.hpp:9-58):
//   P2 = 1/2 + 1/pi int_0^inf Re[e^{iu (r-q) T + psi(u) - iu ln(K/S0)} / (iu)] du
//   P1 = the same with psi(u - i)
// with psi the characteristic exponent of the log-martingale part: per Heston
// factor the "little trap" form, plus the compensated Merton / Kou jump
// exponent, or the Black-Scholes term.  Vanilla call = S0 e^{-qT} P1 - K e^{-rT} P2;
// cash-or-nothing call e^{-rT} P2; asset-or-nothing call S0 e^{-qT} P1; puts
// from the complements.  The integral runs over (0, U] with 256 Gauss-Legendre
// panels of 8 nodes; U is where the integrand envelope drops below 1e-15.
// Greeks are FP64 central differences of these prices (host side).
#include <cmath>
#include <cstring>
#include <vector>

#include "engine.h"

namespace myql {

struct FourierEval {
  int nf, jump, payoff, option_type;
  double S0, K, T, r, q, vol;
  double h[2][5];  // kappa, theta, sigma, rho, v0 per factor
  double lambda, mu, delta, p_up, eta1, eta2;
  double U;        // upper integration bound
};

struct cplx {
  double re, im;
};
__host__ __device__ inline cplx mk(double a, double b) { return {a, b}; }
__host__ __device__ inline cplx operator+(cplx a, cplx b) { return {a.re + b.re, a.im + b.im}; }
__host__ __device__ inline cplx operator-(cplx a, cplx b) { return {a.re - b.re, a.im - b.im}; }
__host__ __device__ inline cplx operator*(cplx a, cplx b) {
  return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
__host__ __device__ inline cplx operator*(double s, cplx a) { return {s * a.re, s * a.im}; }
__host__ __device__ inline cplx operator/(cplx a, cplx b) {
  const double d = b.re * b.re + b.im * b.im;
  return {(a.re * b.re + a.im * b.im) / d, (a.im * b.re - a.re * b.im) / d};
}
__host__ __device__ inline cplx cexp_(cplx a) {
  const double e = exp(a.re);
  return {e * cos(a.im), e * sin(a.im)};
}
__host__ __device__ inline cplx clog_(cplx a) { return {log(hypot(a.re, a.im)), atan2(a.im, a.re)}; }
__host__ __device__ inline cplx csqrt_(cplx a) {  // principal branch
  const double m = hypot(a.re, a.im);
  const double re = sqrt(0.5 * (m + a.re));
  double im = sqrt(0.5 * (m - a.re));
  if (a.im < 0.0) im = -im;
  return {re, im};
}

// Characteristic exponent of the log-martingale part at complex u.
__host__ __device__ inline cplx fourier_psi(const FourierEval &E, cplx u) {
  const cplx I = mk(0.0, 1.0);
  const cplx iu = I * u;
  cplx psi = mk(0.0, 0.0);
  if (E.nf == 0) {
    psi = (-0.5 * E.vol * E.vol * E.T) * (u * u + iu);
  }
  for (int f = 0; f < E.nf; ++f) {
    const double k = E.h[f][0], th = E.h[f][1], s = E.h[f][2], rho = E.h[f][3], v0 = E.h[f][4];
    const cplx beta = mk(k, 0.0) - (rho * s) * iu;
    const cplx d = csqrt_(beta * beta + (s * s) * (iu + u * u));
    const cplx g = (beta - d) / (beta + d);
    const cplx e = cexp_((-E.T) * d);
    const cplx one = mk(1.0, 0.0);
    const cplx D = (1.0 / (s * s)) * (beta - d) * ((one - e) / (one - g * e));
    const cplx C = (k * th / (s * s)) * ((E.T) * (beta - d) - 2.0 * clog_((one - g * e) / (one - g)));
    psi = psi + C + v0 * D;
  }
  if (E.jump == MYQL_JUMP_MERTON) {
    const double half = 0.5 * E.delta * E.delta;
    const cplx phi = cexp_(E.mu * iu - half * (u * u));
    const double kj = exp(E.mu + half) - 1.0;
    psi = psi + (E.lambda * E.T) * ((phi - mk(1.0, 0.0)) - kj * iu);
  } else if (E.jump == MYQL_JUMP_KOU) {
    const cplx up = (E.p_up * E.eta1) * (mk(1.0, 0.0) / (mk(E.eta1, 0.0) - iu));
    const cplx dn = ((1.0 - E.p_up) * E.eta2) * (mk(1.0, 0.0) / (mk(E.eta2, 0.0) + iu));
    const double kj = E.p_up * E.eta1 / (E.eta1 - 1.0) + (1.0 - E.p_up) * E.eta2 / (E.eta2 + 1.0) - 1.0;
    psi = psi + (E.lambda * E.T) * (up + dn - mk(1.0, 0.0) - kj * iu);
  }
  return psi;
}

constexpr int kPanels = 256, kGL = 8;

namespace dev {

// One block per evaluation; thread t integrates panel t.
__global__ void __launch_bounds__(kPanels) fourier_kernel(const FourierEval *evs, const double *gl_x,
                                                          const double *gl_w, double *out) {
  __shared__ double red[kPanels / 32][2];
  const FourierEval E = evs[blockIdx.x];
  const double a = E.U * threadIdx.x / kPanels, b = E.U * (threadIdx.x + 1) / kPanels;
  const double drift = (E.r - E.q) * E.T, logk = log(E.K / E.S0);
  double s1 = 0.0, s2 = 0.0;
  for (int i = 0; i < kGL; ++i) {
    const double u = 0.5 * (a + b) + 0.5 * (b - a) * gl_x[i];
    const double w = 0.5 * (b - a) * gl_w[i];
    const cplx iu = mk(0.0, u);
    const cplx lin = mk(0.0, u * (drift - logk));
    const cplx b2 = cexp_(lin + fourier_psi(E, mk(u, 0.0))) / iu;
    const cplx b1 = cexp_(lin + fourier_psi(E, mk(u, -1.0))) / iu;
    s1 += w * b1.re;
    s2 += w * b2.re;
  }
  for (int o = 16; o > 0; o >>= 1) {
    s1 += __shfl_xor_sync(0xffffffffu, s1, o);
    s2 += __shfl_xor_sync(0xffffffffu, s2, o);
  }
  if ((threadIdx.x & 31) == 0) {
    red[threadIdx.x >> 5][0] = s1;
    red[threadIdx.x >> 5][1] = s2;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t1 = 0.0, t2 = 0.0;
    for (int w = 0; w < kPanels / 32; ++w) {
      t1 += red[w][0];
      t2 += red[w][1];
    }
    const double pi = 3.14159265358979323846;
    const double P1 = 0.5 + t1 / pi, P2 = 0.5 + t2 / pi;
    const double dq = exp(-E.q * E.T), dr = exp(-E.r * E.T);
    const bool call = E.option_type == MYQL_CALL;
    double v;
    if (E.payoff == MYQL_PAYOFF_CASH)
      v = dr * (call ? P2 : 1.0 - P2);
    else if (E.payoff == MYQL_PAYOFF_ASSET)
      v = E.S0 * dq * (call ? P1 : 1.0 - P1);
    else
      v = call ? E.S0 * dq * P1 - E.K * dr * P2 : E.K * dr * (1.0 - P2) - E.S0 * dq * (1.0 - P1);
    out[blockIdx.x] = v;
  }
}

}  // namespace dev

namespace {

// Gauss-Legendre nodes and weights on [-1, 1] (Newton on the Legendre recurrence).
void gauss_legendre(int n, std::vector<double> &x, std::vector<double> &w) {
  x.assign(n, 0.0);
  w.assign(n, 0.0);
  const double pi = 3.14159265358979323846;
  for (int i = 0; i < n; ++i) {
    double z = std::cos(pi * (i + 0.75) / (n + 0.5)), dp = 0.0;
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = z;
      for (int k = 2; k <= n; ++k) {
        const double pk = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = pk;
      }
      dp = n * (z * p1 - p0) / (z * z - 1.0);
      const double dz = p1 / dp;
      z -= dz;
      if (std::fabs(dz) < 1e-16) break;
    }
    x[i] = z;
    w[i] = 2.0 / ((1.0 - z * z) * dp * dp);
  }
}

// Upper bound: where e^{Re psi(u)} / u (both integrands) falls below 1e-15.
double upper_bound(const FourierEval &E) {
  double U = 8.0;
  for (int it = 0; it < 40; ++it) {
    const double m2 = std::exp(fourier_psi(E, mk(U, 0.0)).re) / U;
    const double m1 = std::exp(fourier_psi(E, mk(U, -1.0)).re) / U;
    if (std::max(m1, m2) < 1e-15) break;
    U *= 1.25;
  }
  return std::min(U, 2.0e4);
}

FourierEval eval_of(const myql_mc_job &job, double K) {
  FourierEval E;
  std::memset(&E, 0, sizeof E);
  const myql_model &m = job.model;
  E.nf = m.num_factors;
  E.jump = m.jump;
  E.payoff = job.instrument.payoff;
  E.option_type = job.instrument.option_type;
  E.S0 = job.S0;
  E.K = K;
  E.T = job.instrument.maturity;
  E.r = job.r;
  E.q = job.q;
  E.vol = m.vol;
  for (int f = 0; f < m.num_factors; ++f) {
    const myql_heston_params &h = m.heston[f];
    E.h[f][0] = h.kappa;
    E.h[f][1] = h.theta;
    E.h[f][2] = h.sigma;
    E.h[f][3] = h.rho;
    E.h[f][4] = h.v0;
  }
  E.lambda = m.jump_lambda;
  E.mu = m.merton_mu;
  E.delta = m.merton_delta;
  E.p_up = m.kou_p_up;
  E.eta1 = m.kou_eta1;
  E.eta2 = m.kou_eta2;
  return E;
}

}  // namespace
}  // namespace myql

using namespace myql;

extern "C" myql_status myql_fourier_price(myql_ctx *ctx_, const myql_mc_job *job, int32_t greek_mode, double *out) {
  CtxBase *ctx = reinterpret_cast<CtxBase *>(ctx_);
  if (!ctx || !job || !out) return set_error(MYQL_ERR_INVALID_ARG, "null argument");
  myql_mc_job j = *job;
  j.config.scheme[0] = j.model.num_factors >= 1 ? MYQL_SCHEME_EXACT : MYQL_SCHEME_NONE;
  j.config.scheme[1] = j.model.num_factors >= 2 ? MYQL_SCHEME_EXACT : MYQL_SCHEME_NONE;
  myql_status s = validate_job(j);
  if (s != MYQL_OK) return s;
  if (job->instrument.kind != MYQL_INSTR_EUROPEAN)
    return set_error(MYQL_ERR_UNSUPPORTED, "the Fourier pricer takes European instruments");
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) return cuda_status(e, "cudaSetDevice");
  const int64_t n = job->instrument.n_strikes;
  const bool ess = greek_mode >= MYQL_GREEKS_ESSENTIAL, full = greek_mode >= MYQL_GREEKS_FULL;
  const double S0 = job->S0, T = job->instrument.maturity;
  // bumps (FP64 central differences of FP64 prices)
  const double hS = 1e-4 * S0, hT = 1e-5 * std::max(T, 1e-3), hr = 1e-6;
  std::vector<FourierEval> evs;
  struct Bump {
    double dS, dT, dr, dv0, dv1;
  };
  std::vector<Bump> bumps = {{0, 0, 0, 0, 0}};
  if (ess) {
    bumps.push_back({+hS, 0, 0, 0, 0});
    bumps.push_back({-hS, 0, 0, 0, 0});
  }
  const int nf = job->model.num_factors;
  double hv[2] = {0, 0};
  if (full) {
    for (int f = 0; f < std::max(nf, 1) && f < 2; ++f) {
      // vega per factor: v0 of the factor (volatility for 0 factors)
      hv[f] = nf == 0 ? 1e-4 * job->model.vol : 1e-4 * std::max(job->model.heston[f].v0, 1e-4);
      const double a = f == 0 ? hv[0] : 0.0, b = f == 1 ? hv[1] : 0.0;
      bumps.push_back({0, 0, 0, +a, +b});
      bumps.push_back({0, 0, 0, -a, -b});
      bumps.push_back({+hS, 0, 0, +a, +b});
      bumps.push_back({+hS, 0, 0, -a, -b});
      bumps.push_back({-hS, 0, 0, +a, +b});
      bumps.push_back({-hS, 0, 0, -a, -b});
    }
    bumps.push_back({0, +hT, 0, 0, 0});
    bumps.push_back({0, -hT, 0, 0, 0});
    bumps.push_back({+hS, +hT, 0, 0, 0});
    bumps.push_back({+hS, -hT, 0, 0, 0});
    bumps.push_back({-hS, +hT, 0, 0, 0});
    bumps.push_back({-hS, -hT, 0, 0, 0});
    bumps.push_back({0, 0, +hr, 0, 0});
    bumps.push_back({0, 0, -hr, 0, 0});
  }
  for (int64_t k = 0; k < n; ++k)
    for (const Bump &b : bumps) {
      FourierEval E = eval_of(j, job->instrument.strikes[k]);
      E.S0 += b.dS;
      E.T += b.dT;
      E.r += b.dr;
      if (nf == 0) {
        E.vol += b.dv0;
      } else {
        E.h[0][4] += b.dv0;
        if (nf == 2) E.h[1][4] += b.dv1;
      }
      E.U = upper_bound(E);
      evs.push_back(E);
    }
  std::vector<double> glx, glw;
  gauss_legendre(kGL, glx, glw);
  const size_t ne = evs.size();
  e = ctx->aux_c.ensure(ne * sizeof(FourierEval) + 2 * kGL * sizeof(double) + ne * sizeof(double));
  if (e != cudaSuccess) return cuda_status(e, "Fourier buffers");
  uint8_t *base = (uint8_t *)ctx->aux_c.p;
  FourierEval *d_ev = (FourierEval *)base;
  double *d_x = (double *)(base + ne * sizeof(FourierEval));
  double *d_w = d_x + kGL, *d_out = d_w + kGL;
  std::vector<double> res(ne);
  e = cudaMemcpyAsync(d_ev, evs.data(), ne * sizeof(FourierEval), cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_x, glx.data(), kGL * sizeof(double), cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_w, glw.data(), kGL * sizeof(double), cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) {
    dev::fourier_kernel<<<(unsigned int)ne, kPanels, 0, ctx->stream>>>(d_ev, d_x, d_w, d_out);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(res.data(), d_out, ne * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_status(e, "Fourier pricing");
  std::memset(out, 0, MYQL_OUT_DOUBLES(n) * sizeof(double));
  const size_t nb = bumps.size();
  for (int64_t k = 0; k < n; ++k) {
    const double *p = res.data() + k * nb;
    auto q = [&](int qi, double v) { out[(size_t)(2 * qi) * n + k] = v; };
    q(MYQL_Q_PRICE, p[0]);
    if (!ess) continue;
    q(MYQL_Q_DELTA, (p[1] - p[2]) / (2 * hS));
    q(MYQL_Q_GAMMA, (p[1] - 2 * p[0] + p[2]) / (hS * hS));
    if (!full) continue;
    size_t o = 3;
    for (int f = 0; f < std::max(nf, 1) && f < 2; ++f, o += 6) {
      // d/d sigma_f with sigma = sqrt(v0): chain factor 2 sqrt(v0) (AffineTraits.hpp:232-246)
      const double chain = nf == 0 ? 1.0 : 2.0 * std::sqrt(job->model.heston[f].v0);
      q(f == 0 ? MYQL_Q_VEGA0 : MYQL_Q_VEGA1, (p[o] - p[o + 1]) / (2 * hv[f]) * chain);
      const double vanna = ((p[o + 2] - p[o + 3]) - (p[o + 4] - p[o + 5])) / (4 * hS * hv[f]) * chain;
      q(f == 0 ? MYQL_Q_VANNA0 : MYQL_Q_VANNA1, vanna);
    }
    q(MYQL_Q_THETA, (p[o] - p[o + 1]) / (2 * hT));
    q(MYQL_Q_CHARM, ((p[o + 2] - p[o + 3]) - (p[o + 4] - p[o + 5])) / (4 * hS * hT));
    q(MYQL_Q_RHO, (p[o + 6] - p[o + 7]) / (2 * hr));
  }
  return MYQL_OK;
}
