// batch.cuh -- many uneven pricing requests in one persistent launch.
//
// The reference prices a heterogeneous set of requests by calling
// dispatcher::price_mc once per request (PricingDispatch.hpp:93-126), each a
// full OpenMP fork/join.  Here all requests run in one persistent kernel per
// kernel class: the host splits every job into work items of 128 streams
// (all of each stream's paths), sorts the items by cost (paths per stream x
// steps, longest first) and the resident blocks pull items from a global
// atomic counter.  Each job keeps its own stream layout (path i on stream
// i mod S_j) so a batched job returns what the same job priced alone returns.
// Per item the block reduces price (and pathwise delta and gamma) in FP64 into
// the item's partial slot; a second kernel sums the slots of each job in item
// order (deterministic).
//
// Launch shape (picked per kernel class by the host's autotuner): BLOCK threads
// per block (64, 128 or 256), `streams_per_thread` streams simulated one after
// another by each thread (1, 2 or 4), so a block pulls BLOCK x streams_per_thread
// / 128 items at a time, and the unroll depth of the time-step loop (0 = the
// compiler's choice, or 2).  The per-stream arithmetic is the same for every
// shape; only the FP64 grouping of the per-item sums differs.
#pragma once
#include "mlmc.cuh"  // record_price, payoff evaluation, sim_path

namespace myql {

constexpr int kBatchItemStreams = 128;  // streams per work item
constexpr int kBatchQ = 3;              // price, delta, gamma
constexpr int kBatchMaxSpt = 4;         // most streams per thread of a launch shape

// A launch shape of the persistent batch kernel (the autotuner's candidates).
struct BatchShape {
  int block;               // threads per block: 64, 128 or 256
  int streams_per_thread;  // 1, 2 or 4; block * streams_per_thread is a multiple of 128
  int unroll;              // time-step loop unroll depth: 0 (compiler) or 2
};

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
  unsigned int streams_per_thread;  // of the launch shape
  unsigned int items_per_pull;      // block * streams_per_thread / 128
};

namespace dev {

// All paths of stream s of job J; FP32 sums over the stream's paths, added to acc in FP64.
template <int NF, int S1, int S2, bool PD, int UNROLL>
__device__ __forceinline__ void batch_stream(const BatchJob &J, unsigned int s, double (&acc)[kBatchQ][2],
                                             unsigned int &caphits, unsigned int &fallbacks) {
  const SimParams &P = J.sim;
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
    sim_path<NF, S1, S2, PD, UNROLL>(P, P.sc[0], rng, r, caphits, fallbacks);
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
    acc[q][0] += s1[q];
    acc[q][1] += s2[q];
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

// Persistent kernel of one class (klass, path dependence) and launch shape over one
// segment; each (class, shape) is its own instantiation with its own register allocation.
cudaError_t launch_batch(const BatchParams &B, int klass, bool pd, const BatchShape &shape, unsigned int blocks,
                         cudaStream_t st);
cudaError_t launch_batch_finalize(const BatchJob *jobs, unsigned int n_jobs, const double *partials,
                                  double *outs, cudaStream_t st);
int batch_blocks_per_sm(int klass, bool pd, const BatchShape &shape);

namespace dev {

// Persistent: every block loops pulling items_per_pull items of its segment at a
// time until it is empty.  Thread t simulates the streams t + j BLOCK (j <
// streams_per_thread) of the pulled items' 128 x items_per_pull streams; a warp's
// 32 streams always lie in one item.  Each warp's sums go to shared memory per j,
// and the item's partial is their sum in (j, warp) order.
template <int NF, int S1, int S2, bool PD, int BLOCK, int UNROLL>
__global__ void __launch_bounds__(BLOCK) batch_kernel(const BatchParams B) {
  constexpr int W = BLOCK / 32;
  __shared__ unsigned int item_sh;
  __shared__ double red[kBatchMaxSpt][W][kBatchQ][2];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const unsigned int spt = B.streams_per_thread, ipp = B.items_per_pull;
  unsigned int caphits = 0, fallbacks = 0;
  unsigned int *status = nullptr;
  const unsigned long long n = B.item_end - B.item_begin;
  for (;;) {
    if (threadIdx.x == 0) item_sh = atomicAdd(B.counter, ipp);
    __syncthreads();
    const unsigned long long k0 = item_sh;
    __syncthreads();
    if (k0 >= n) break;
    for (unsigned int j = 0; j < spt; ++j) {
      const unsigned int u = j * BLOCK + threadIdx.x;  // stream slot within the pull
      const unsigned long long k = k0 + u / kBatchItemStreams;
      double acc[kBatchQ][2] = {{0.0, 0.0}, {0.0, 0.0}, {0.0, 0.0}};
      if (k < n) {
        const BatchItem I = B.items[B.item_begin + k];
        const BatchJob &J = B.jobs[I.job];
        status = J.sim.status;
        batch_stream<NF, S1, S2, PD, UNROLL>(J, I.stream0 + u % kBatchItemStreams, acc, caphits, fallbacks);
      }
#pragma unroll
      for (int q = 0; q < kBatchQ; ++q)
#pragma unroll
        for (int c = 0; c < 2; ++c) {
          double v = acc[q][c];
          for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
          if (lane == 0) red[j][warp][q][c] = v;
        }
    }
    __syncthreads();
    if (threadIdx.x < ipp * kBatchQ * 2) {
      const unsigned int i = threadIdx.x / (kBatchQ * 2), q = (threadIdx.x >> 1) % kBatchQ, c = threadIdx.x & 1;
      const unsigned long long k = k0 + i;
      if (k < n) {
        double t = 0.0;
        for (unsigned int j = 0; j < spt; ++j)
          for (int w = 0; w < W; ++w)
            if ((j * BLOCK + w * 32) / kBatchItemStreams == i) t += red[j][w][q][c];
        B.partials[((size_t)B.item_slot[B.item_begin + k] * kBatchQ + q) * 2 + c] = t;
      }
    }
    __syncthreads();  // red is rewritten by the next pull
  }
  if (status && (caphits || fallbacks)) {
    if (caphits) atomicAdd(status, caphits);
    if (fallbacks) atomicAdd(status + 1, fallbacks);
  }
}

}  // namespace dev

}  // namespace myql
