// tables.cu -- device set-up kernels: xoshiro stream seeding (jump-ahead) and
// the FP64 build of the SchemeNCI chi-squared tables; plus numerics probes.
#include "chi2_fp64.cuh"
#include "device_numerics.cuh"
#include "engine_types.h"

#include <algorithm>

namespace myql {

__constant__ unsigned long long c_jump[64][4];

namespace dev {

__device__ __forceinline__ void xo_transition(Xo &s) {
  const unsigned long long t = s.b << 17;
  s.c ^= s.a;
  s.d ^= s.b;
  s.b ^= s.c;
  s.a ^= s.d;
  s.c ^= t;
  s.d = rotl64(s.d, 45);
}

// State advanced by 2^(128+i) steps (Vigna's jump loop with polynomial i).
__device__ void jump_apply(Xo &s, int i) {
  unsigned long long a0 = 0, a1 = 0, a2 = 0, a3 = 0;
  for (int w = 0; w < 4; ++w) {
    const unsigned long long poly = c_jump[i][w];
    for (int b = 0; b < 64; ++b) {
      if ((poly >> b) & 1ull) {
        a0 ^= s.a;
        a1 ^= s.b;
        a2 ^= s.c;
        a3 ^= s.d;
      }
      xo_transition(s);
    }
  }
  s.a = a0;
  s.b = a1;
  s.c = a2;
  s.d = a3;
}

__device__ Xo splitmix_seed(unsigned long long x) {
  Xo s;
  unsigned long long v[4];
  for (int i = 0; i < 4; ++i) {
    unsigned long long z = (x += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    v[i] = z ^ (z >> 31);
  }
  s.a = v[0];
  s.b = v[1];
  s.c = v[2];
  s.d = v[3];
  return s;
}

// Block b produces streams first + 128 b + t: thread 0 jumps the seeded state
// to the block's first stream (one polynomial per set bit of its index), then
// a doubling tree fills the other 127 states with one jump each.
constexpr int kSeedBlock = 128;
__global__ void __launch_bounds__(kSeedBlock) seed_streams_kernel(unsigned long long seed,
                                                                  unsigned long long first,
                                                                  unsigned long long n,
                                                                  unsigned long long *out) {
  __shared__ Xo sh[kSeedBlock];
  const unsigned long long base = first + (unsigned long long)blockIdx.x * kSeedBlock;
  if (threadIdx.x == 0) {
    Xo s = splitmix_seed(seed);
    for (int i = 0; i < 64; ++i)
      if ((base >> i) & 1ull) jump_apply(s, i);
    sh[0] = s;
  }
  __syncthreads();
  for (int r = 0; (1 << r) < kSeedBlock; ++r) {
    const int span = 1 << r;
    if ((int)threadIdx.x < span) {
      Xo s = sh[threadIdx.x];
      jump_apply(s, r);
      sh[threadIdx.x + span] = s;
    }
    __syncthreads();
  }
  const unsigned long long k = (unsigned long long)blockIdx.x * kSeedBlock + threadIdx.x;
  if (k < n) {
    const Xo s = sh[threadIdx.x];
    out[k] = s.a;
    out[n + k] = s.b;
    out[2 * n + k] = s.c;
    out[3 * n + k] = s.d;
  }
}

__global__ void rng_draws_kernel(const unsigned long long *states, unsigned long long n,
                                 unsigned long long count, unsigned long long *out) {
  const unsigned long long k = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  Xo s{states[k], states[n + k], states[2 * n + k], states[3 * n + k]};
  for (unsigned long long i = 0; i < count; ++i) out[k * count + i] = xo_next(s);
}

// ---- SchemeNCI table build (FP64) -----------------------------------------
// A thread fills a run of consecutive nodes of one row.  The first node of a
// run starts Newton from chi2_start; each later node starts from the Taylor
// step of the quantile function u(p) = log(y(p) / 2) from the previous node:
// with g = du/dp = 1 / (x f(x)) (f the gamma(a) density, x = e^u) and
// s = a - x, d2u/dp2 = -s g^2 and d3u/dp3 = (x + 2 s^2) g^3.  The step is used
// while g dx (1 + |s|) < 0.2, where its error is far below the Newton
// acceptance step, so most nodes take one evaluation of the incomplete gamma.
constexpr int kNciRunMain = 16;
constexpr int kNciRunTail = 4;
constexpr int kNciRunsMain = (kNciGrid + kNciRunMain - 1) / kNciRunMain;
constexpr int kNciRunsTail = (kNciTail + kNciRunTail - 1) / kNciRunTail;
constexpr double kNciAccept = 1e-8;
constexpr double kNciStepGate = 0.2;

__global__ void nci_nodes_main_kernel(double d, int rows, double dx, double *y) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)rows * kNciRunsMain) return;
  const int k = (int)(idx / kNciRunsMain), i0 = (int)(idx % kNciRunsMain) * kNciRunMain;
  const int i1 = min(i0 + kNciRunMain, kNciGrid);
  const double a = 0.5 * d + k, lga = lgamma(a);
  double *yr = y + (size_t)k * kNciGrid;
  double u = 0.0;
  bool have = false;
  for (int i = i0; i < i1; ++i) {
    if (i == 0) {
      yr[0] = 0.0;
      continue;
    }
    const double p = i * dx;
    const bool upper = p > 0.5;
    const double pt = upper ? 1.0 - p : p;
    const double lp = log(pt);
    double u0 = 0.0;
    bool warm = false;
    if (have) {
      const double x = exp(u), gh = exp(lga + x - a * u) * dx, s = a - x;
      if (gh * (1.0 + fabs(s)) < kNciStepGate) {
        u0 = u + gh * (1.0 + gh * (-0.5 * s + gh * (x + 2.0 * s * s) * (1.0 / 6.0)));
        warm = true;
      }
    }
    if (!warm) u0 = chi2_start(a, pt, lp, upper);
    u = chi2_newton(a, lga, lp, upper, u0, kNciAccept);
    have = true;
    yr[i] = 2.0 * exp(u);
  }
}

// Tail nodes at upper-tail probability q = e^-w, w = w0 + j dw.  Along w,
// g = du/dw = q / (x f(x)) and d2u/dw2 = -g (1 + s g); the warm start is the
// second-order step from the previous node.
__global__ void nci_nodes_tail_kernel(double d, int rows, double w0, double dw, double *y,
                                      double *m) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)rows * kNciRunsTail) return;
  const int k = (int)(idx / kNciRunsTail), j0 = (int)(idx % kNciRunsTail) * kNciRunTail;
  const int j1 = min(j0 + kNciRunTail, kNciTail);
  const double nu = d + 2.0 * k;
  const double a = 0.5 * nu, lga = lgamma(a);
  double u = 0.0, w_prev = 0.0;
  bool have = false;
  for (int j = j0; j < j1; ++j) {
    const double w = w0 + j * dw;
    double u0 = 0.0;
    bool warm = false;
    if (have) {
      const double x = exp(u), gd = exp(-w_prev - (a * u - x - lga)) * dw, s = a - x;
      if (gd * (1.0 + fabs(s)) < kNciStepGate) {
        u0 = u + gd - 0.5 * gd * (dw + s * gd);
        warm = true;
      }
    }
    if (!warm) u0 = chi2_start(a, exp(-w), -w, true);
    u = chi2_newton(a, lga, -w, true, u0, kNciAccept);
    have = true;
    w_prev = w;
    const double v = 2.0 * exp(u);
    const size_t o = (size_t)k * kNciTail + j;
    y[o] = v;
    m[o] = exp(-w - chi2_logpdf(nu, v));  // dy/dw = q / f(y)
  }
}

// Monotone cubic Hermite cells with the reference's harmonic-mean slopes
// (VolSchemes.hpp:292-310), stored as monomial coefficients in t.
__device__ __forceinline__ double nci_slope(const double *yr, int i, double inv_dx) {
  if (i == 0) return (yr[1] - yr[0]) * inv_dx;
  if (i == kNciGrid - 1) return (yr[i] - yr[i - 1]) * inv_dx;
  const double d1 = (yr[i] - yr[i - 1]) * inv_dx;
  const double d2 = (yr[i + 1] - yr[i]) * inv_dx;
  return d1 * d2 > 0.0 ? 2.0 * d1 * d2 / (d1 + d2) : 0.0;
}

__device__ __forceinline__ float4 hermite_cell(double y0, double y1, double hm0, double hm1) {
  return make_float4((float)y0, (float)hm0, (float)(3.0 * (y1 - y0) - (2.0 * hm0 + hm1)),
                     (float)(2.0 * (y0 - y1) + (hm0 + hm1)));
}

// Exact slope dy/dU = 1 / f(y) of the quantile function at an interior node
// (f the chi-squared density with nu degrees of freedom); the first node keeps
// the secant, since the derivative is 0 or unbounded at U = 0.
__device__ __forceinline__ double nci_exact_slope(const double *yr, int i, double nu, double inv_dx) {
  if (i == 0) return (yr[1] - yr[0]) * inv_dx;
  return exp(-chi2_logpdf(nu, yr[i]));
}

// exact 0: the reference's cells (harmonic-mean slopes, the first cell a
// Hermite cubic from the node y(0) = 0).  Their integral falls short of the
// conditional mean d + 2k by 1.5e-5 to 4e-5 relative for rows k >= 25, almost
// all of it in the first cell: for many degrees of freedom the quantile rises
// from 0 to near y(dx) within a sliver of U, which a cubic from y(0) = 0 misses.
// exact 1: exact slopes 1 / f(y) at the nodes, and, for rows k >= 4, a first
// cell c(t) = y1 + h m1 (t - 1) + q (t - 1)^2 whose integral is the exact mean
// of the quantile over [0, dx], nu P(nu/2 + 1, y1/2) / dx: the cells then
// integrate to the mean within about 1e-8 relative.
__global__ void nci_cells_main_kernel(int rows, const double *y, double dx, float4 *cells, double d,
                                      int exact) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)rows * (kNciGrid - 1)) return;
  const int k = (int)(idx / (kNciGrid - 1)), i = (int)(idx % (kNciGrid - 1));
  const double *yr = y + (size_t)k * kNciGrid;
  const double inv_dx = 1.0 / dx;
  double m0, m1;
  if (exact) {
    const double nu = d + 2.0 * k;
    m0 = nci_exact_slope(yr, i, nu, inv_dx);
    m1 = nci_exact_slope(yr, i + 1, nu, inv_dx);
    if (i == 0 && k >= 4) {
      const double a = 0.5 * nu + 1.0, y1 = yr[1], hm1 = dx * m1;
      const double mean = nu * exp(gamma_eval(a, 0.5 * y1, lgamma(a)).logP) * inv_dx;
      const double q = 3.0 * (mean - y1 + 0.5 * hm1);
      cells[idx] = make_float4((float)(y1 - hm1 + q), (float)(hm1 - 2.0 * q), (float)q, 0.0f);
      return;
    }
  } else {
    m0 = nci_slope(yr, i, inv_dx);
    m1 = nci_slope(yr, i + 1, inv_dx);
  }
  cells[idx] = hermite_cell(yr[i], yr[i + 1], dx * m0, dx * m1);
}

__global__ void nci_cells_tail_kernel(int rows, const double *y, const double *m, double dw,
                                      float4 *cells) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)rows * (kNciTail - 1)) return;
  const int k = (int)(idx / (kNciTail - 1)), j = (int)(idx % (kNciTail - 1));
  const size_t o = (size_t)k * kNciTail + j;
  cells[idx] = hermite_cell(y[o], y[o + 1], dw * m[o], dw * m[o + 1]);
}

// ---- probes --------------------------------------------------------------
__global__ void chi2_probe_kernel(const double *dof, const double *p, double *out, size_t n) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] = p[i] <= 0.5 ? chi2_quantile(dof[i], p[i], false) : chi2_quantile(dof[i], 1.0 - p[i], true);
}

__global__ void sampler_probe_kernel(int kind, const unsigned long long *x, const double *lam,
                                     float *out, size_t n, unsigned int cap, unsigned int *status) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  unsigned int hits = 0;
  if (kind == 0)
    out[i] = inv_normal_bits(x[i]);
  else
    out[i] = (float)poisson_inv((float)lam[i], x[i], cap, hits);
  if (hits) atomicAdd(status, hits);
}

}  // namespace dev

cudaError_t upload_jump_polys(const unsigned long long polys[64][4]) {
  return cudaMemcpyToSymbol(c_jump, polys, sizeof(unsigned long long) * 64 * 4);
}

cudaError_t launch_seed_streams(unsigned long long seed, unsigned long long first,
                                unsigned long long n, unsigned long long *out,
                                cudaStream_t stream) {
  const unsigned int blocks = (unsigned int)((n + dev::kSeedBlock - 1) / dev::kSeedBlock);
  dev::seed_streams_kernel<<<blocks, dev::kSeedBlock, 0, stream>>>(seed, first, n, out);
  return cudaGetLastError();
}

cudaError_t launch_rng_draws(const unsigned long long *states, unsigned long long n,
                             unsigned long long count, unsigned long long *out,
                             cudaStream_t stream) {
  dev::rng_draws_kernel<<<(unsigned int)((n + 127) / 128), 128, 0, stream>>>(states, n, count, out);
  return cudaGetLastError();
}

cudaError_t launch_nci_nodes(double d, int rows, double *tmp_main, double *tmp_ty, double *tmp_tm,
                             double w0, double dw, cudaStream_t stream) {
  const double dx = kNciUmax / (kNciGrid - 1);
  const long long nm = (long long)rows * dev::kNciRunsMain, nt = (long long)rows * dev::kNciRunsTail;
  dev::nci_nodes_main_kernel<<<(unsigned int)((nm + 127) / 128), 128, 0, stream>>>(d, rows, dx, tmp_main);
  dev::nci_nodes_tail_kernel<<<(unsigned int)((nt + 63) / 64), 64, 0, stream>>>(d, rows, w0, dw, tmp_ty, tmp_tm);
  return cudaGetLastError();
}

cudaError_t launch_nci_build(double d, int rows, double *tmp_main, double *tmp_ty, double *tmp_tm,
                             float4 *cells_main, float4 *cells_tail, double w0, double dw,
                             int exact, cudaStream_t stream) {
  const double dx = kNciUmax / (kNciGrid - 1);
  cudaError_t e = launch_nci_nodes(d, rows, tmp_main, tmp_ty, tmp_tm, w0, dw, stream);
  if (e != cudaSuccess) return e;
  const long long cm = (long long)rows * (kNciGrid - 1), ct = (long long)rows * (kNciTail - 1);
  dev::nci_cells_main_kernel<<<(unsigned int)((cm + 255) / 256), 256, 0, stream>>>(rows, tmp_main, dx, cells_main,
                                                                                   d, exact);
  dev::nci_cells_tail_kernel<<<(unsigned int)((ct + 255) / 256), 256, 0, stream>>>(rows, tmp_ty, tmp_tm, dw, cells_tail);
  return cudaGetLastError();
}

cudaError_t launch_chi2_probe(const double *dof, const double *p, double *out, size_t n,
                              cudaStream_t stream) {
  dev::chi2_probe_kernel<<<(unsigned int)((n + 127) / 128), 128, 0, stream>>>(dof, p, out, n);
  return cudaGetLastError();
}

cudaError_t launch_sampler_probe(int kind, const unsigned long long *x, const double *lam,
                                 float *out, size_t n, unsigned int cap, unsigned int *status,
                                 cudaStream_t stream) {
  dev::sampler_probe_kernel<<<(unsigned int)((n + 127) / 128), 128, 0, stream>>>(kind, x, lam, out, n, cap, status);
  return cudaGetLastError();
}

}  // namespace myql

// ---- issue-rate ceilings (compute roofline denominators) -------------------
namespace myql {
namespace dev {
constexpr int kPeakIters = 4096;

// 8 independent FMA chains per thread: the FP32 pipe's sustained lane rate.
__global__ void __launch_bounds__(256) fma_peak_kernel(float *sink, float seed) {
  float a0 = seed + threadIdx.x, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3;
  float a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6, a7 = a0 + 7;
  const float m = 0.999999f, c = 1e-7f;
#pragma unroll 16
  for (int i = 0; i < kPeakIters; ++i) {
    a0 = fmaf(a0, m, c); a1 = fmaf(a1, m, c); a2 = fmaf(a2, m, c); a3 = fmaf(a3, m, c);
    a4 = fmaf(a4, m, c); a5 = fmaf(a5, m, c); a6 = fmaf(a6, m, c); a7 = fmaf(a7, m, c);
  }
  const float s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
  sink[blockIdx.x * blockDim.x + threadIdx.x] = s;  // keeps every chain live
}

// 8 independent ex2.approx chains per thread: the MUFU rate.
__global__ void __launch_bounds__(256) mufu_peak_kernel(float *sink, float seed) {
  float a[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) a[j] = -1e-3f * (seed + threadIdx.x + j);
#pragma unroll 8
  for (int i = 0; i < kPeakIters; ++i) {
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      float r;
      asm volatile("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(a[j]));
      a[j] = -r;
    }
  }
  float s = 0.0f;
#pragma unroll
  for (int j = 0; j < 8; ++j) s += a[j];
  sink[blockIdx.x * blockDim.x + threadIdx.x] = s;  // keeps every chain live
}
}  // namespace dev

cudaError_t run_peak_probe(int kind, int sm_count, cudaStream_t stream, double *ops_per_s) {
  float *sink = nullptr;
  cudaEvent_t e0, e1;
  const int blocks = sm_count * 8;
  cudaError_t e = cudaMalloc(&sink, (size_t)blocks * 256 * sizeof(float));
  if (e != cudaSuccess) return e;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  double best = 0.0;
  for (int rep = 0; rep < 4 && e == cudaSuccess; ++rep) {
    cudaEventRecord(e0, stream);
    if (kind == 0)
      dev::fma_peak_kernel<<<blocks, 256, 0, stream>>>(sink, 1.0f + rep);
    else
      dev::mufu_peak_kernel<<<blocks, 256, 0, stream>>>(sink, 1.0f + rep);
    cudaEventRecord(e1, stream);
    e = cudaEventSynchronize(e1);
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    const double ops = (double)blocks * 256.0 * dev::kPeakIters * 8.0;
    if (rep > 0 && ms > 0.0f) best = std::max(best, ops / (ms * 1e-3));
  }
  if (e == cudaSuccess) e = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(sink);
  *ops_per_s = best;
  return e;
}
}  // namespace myql
