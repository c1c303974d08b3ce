// batch.cuh -- many uneven pricing requests in one persistent launch.
//
// The reference prices a heterogeneous set of requests by calling
// dispatcher::price_mc once per request (PricingDispatch.hpp:93-126), each a
// full OpenMP fork/join.  Here all requests run in one persistent kernel: the
// host splits every job into work items of 128 streams (one thread per
// stream, all of that stream's paths), sorts the items by cost (paths per
// stream x steps, longest first) and the resident blocks pull items from a
// global atomic counter.  Each job keeps its own stream layout (path i on
// stream i mod S_j) so a batched job returns exactly what the same job priced
// alone returns.  Per item the block reduces price (and pathwise delta and
// gamma) in FP64 into its own partial slot; a second kernel sums the slots of
// each job in item order (deterministic).
#pragma once
#include "mlmc.cuh"  // record_price, payoff evaluation, sim_path

namespace myql {

constexpr int kBatchItemStreams = kSimBlock;
constexpr int kBatchQ = 3;  // price, delta, gamma

struct BatchJob {
  SimParams sim;     // n_sc = 1; states -> the seed table of the job's seed
  PayoffParams pay;  // scalar instrument
  int klass;         // kernel class (factors, schemes, path dependence)
  int mode;          // GreekMode (None / Essential)
  unsigned long long first_item;
  unsigned long long n_items;
  unsigned long long state_stride;  // stride of the seed table's [4][stride] layout
  unsigned long long stream_base;   // index of the job's first stream in that table
  double df;                        // exp(-r T)
};

struct BatchItem {
  unsigned int job;
  unsigned int stream0;  // first stream of the item
};

// One segment of the item list: the items of one kernel class, cost-sorted;
// its persistent blocks pull items [item_begin, item_end) through `counter`.
struct BatchParams {
  const BatchJob *jobs;
  const BatchItem *items;
  const unsigned int *item_slot;  // partial slot of each item (= its index within the job order)
  unsigned long long item_begin, item_end;
  unsigned int *counter;
  double *partials;        // [slot][kBatchQ][2]
};

namespace dev {

template <int NF, int S1, int S2, bool PD>
__device__ __forceinline__ void batch_item(const BatchJob &J, unsigned int stream0, double (&acc)[kBatchQ][2],
                                           unsigned int &caphits, unsigned int &fallbacks) {
  const SimParams &P = J.sim;
  const unsigned int s = stream0 + threadIdx.x;
  if (s >= P.n_streams) return;
  const unsigned int S = P.n_streams;
  const size_t g = J.stream_base + s, st = J.state_stride;
  Xo rng;
  rng.a = P.states[g];
  rng.b = P.states[st + g];
  rng.c = P.states[2 * st + g];
  rng.d = P.states[3 * st + g];
  const float K = (float)J.pay.strikes[0];
  float s1[kBatchQ] = {0.0f, 0.0f, 0.0f}, s2[kBatchQ] = {0.0f, 0.0f, 0.0f};
  for (unsigned long long i = s; i < P.num_paths; i += S) {
    float r[kMaxFields];
    sim_path<NF, S1, S2, PD>(P, P.sc[0], rng, r, caphits, fallbacks);
    PathView v;
    v.S = J.pay.S0 * __expf(r[0]);
    v.Y = 0.0f;
    v.hit[0] = v.hit[1] = v.hit[2] = -1.0f;
    switch (J.pay.tracker) {
      case TRK_GEO_ASIAN: v.Y = J.pay.S0 * __expf(fmaf(J.pay.avg_c1[0], r[1], J.pay.avg_c0[0])); break;
      case TRK_ARITH_ASIAN: v.Y = J.pay.S0 * fmaf(J.pay.avg_c1[0], r[1], J.pay.avg_c0[0]); break;
      case TRK_LOOKBACK: {
        const bool use_max = (J.pay.option_type == 0) == (J.pay.fixed_strike != 0);
        v.Y = J.pay.S0 * __expf(use_max ? r[2] : r[1]);
        break;
      }
      case TRK_BARRIER_UP:
      case TRK_BARRIER_DOWN:
        v.hit[0] = r[1];
        v.hit[1] = r[2];
        v.hit[2] = r[3];
        break;
      default: break;
    }
    const Tri t = scenario_tri(J.pay, v, K, J.mode != 0);
    s1[0] += t.v;
    s2[0] = fmaf(t.v, t.v, s2[0]);
    if (J.mode != 0) {
      const float d = (t.dp - t.dm) * J.pay.inv_2h, g = (t.dp + t.dm) * J.pay.inv_h2;
      s1[1] += d;
      s2[1] = fmaf(d, d, s2[1]);
      s1[2] += g;
      s2[2] = fmaf(g, g, s2[2]);
    }
  }
#pragma unroll
  for (int q = 0; q < kBatchQ; ++q) {
    acc[q][0] = s1[q];
    acc[q][1] = s2[q];
  }
}

}  // namespace dev

// Kernel classes of the persistent batch kernel.
enum BatchClass : int {
  BK_F0 = 0,
  BK_F1_NV = 1, BK_F1_EXACT = 2, BK_F1_NCI = 3,
  BK_F2_NV_NV = 4, BK_F2_NV_EXACT = 5, BK_F2_NV_NCI = 6,
  BK_F2_EXACT_NV = 7, BK_F2_EXACT_EXACT = 8, BK_F2_EXACT_NCI = 9,
  BK_F2_NCI_NV = 10, BK_F2_NCI_EXACT = 11, BK_F2_NCI_NCI = 12,
  BK_COUNT = 13
};

inline int batch_class(int nf, int s1, int s2) {
  if (nf == 0) return BK_F0;
  if (nf == 1) return s1;  // 1, 2, 3
  return 4 + (s1 - 1) * 3 + (s2 - 1);
}

// Persistent kernel of one class (klass, path dependence) over one segment; each
// class is its own instantiation with its own register allocation.
cudaError_t launch_batch(const BatchParams &B, int klass, bool pd, unsigned int blocks, cudaStream_t st);
cudaError_t launch_batch_finalize(const BatchJob *jobs, unsigned int n_jobs, const double *partials,
                                  double *outs, cudaStream_t st);
int batch_blocks_per_sm(int klass, bool pd);

namespace dev {

// Persistent: every block loops pulling items of its segment until it is empty.
template <int NF, int S1, int S2, bool PD>
__global__ void __launch_bounds__(kSimBlock) batch_kernel(const BatchParams B) {
  __shared__ unsigned int item_sh;
  __shared__ double red[kSimBlock / 32][kBatchQ][2];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  unsigned int caphits = 0, fallbacks = 0;
  unsigned int *status = nullptr;
  const unsigned long long n = B.item_end - B.item_begin;
  for (;;) {
    if (threadIdx.x == 0) item_sh = atomicAdd(B.counter, 1u);
    __syncthreads();
    const unsigned long long k = item_sh;
    __syncthreads();
    if (k >= n) break;
    const unsigned long long it = B.item_begin + k;
    const BatchItem I = B.items[it];
    const BatchJob &J = B.jobs[I.job];
    status = J.sim.status;
    double acc[kBatchQ][2] = {{0.0, 0.0}, {0.0, 0.0}, {0.0, 0.0}};
    batch_item<NF, S1, S2, PD>(J, I.stream0, acc, caphits, fallbacks);
#pragma unroll
    for (int q = 0; q < kBatchQ; ++q)
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        double v = acc[q][c];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) red[warp][q][c] = v;
      }
    __syncthreads();
    if (threadIdx.x < kBatchQ * 2) {
      const int q = threadIdx.x >> 1, c = threadIdx.x & 1;
      double t = 0.0;
      for (int w = 0; w < kSimBlock / 32; ++w) t += red[w][q][c];
      B.partials[((size_t)B.item_slot[it] * kBatchQ + q) * 2 + c] = t;
    }
  }
  if (status && (caphits || fallbacks)) {
    if (caphits) atomicAdd(status, caphits);
    if (fallbacks) atomicAdd(status + 1, fallbacks);
  }
}

}  // namespace dev

}  // namespace myql
