// batch.cu -- host side of myql_mc_price_batch: many uneven requests in one
// persistent launch (the work the reference's runtime dispatcher does one
// request at a time, PricingDispatch.hpp:93-126).
//
// Per call: plan every job (the same constants as myql_mc_price), seed one
// stream table per distinct seed, cut every job into items of 128 streams,
// order the items by cost (longest first), then
//   H2D(job descriptors, items)  ->  persistent batch_kernel  ->  per-job finalize  ->  D2H
// captured once as a CUDA graph per batch shape and replayed afterwards (only
// the pinned staging buffers change between calls).  Per kernel class, a small
// autotuner picks the launch shape -- threads per block, streams (all of their
// paths) per thread, unroll depth of the time-step loop -- and the persistent
// grid size on the first batch of a shape, timing each candidate on the class's
// leading (most expensive) items; the choice is cached and reported by
// myql_batch_last_plan.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <numeric>
#include <vector>

#include "batch.cuh"
#include "engine.h"

namespace myql {
namespace {

struct PinnedBuf {
  void *p = nullptr;
  size_t cap = 0;
  cudaError_t ensure(size_t bytes) {
    if (bytes <= cap) return cudaSuccess;
    if (p) cudaFreeHost(p);
    p = nullptr;
    cap = 0;
    cudaError_t e = cudaHostAlloc(&p, bytes, cudaHostAllocDefault);
    if (e == cudaSuccess) cap = bytes;
    return e;
  }
  ~PinnedBuf() {
    if (p) cudaFreeHost(p);
  }
};

struct BatchState : ExtState {
  PinnedBuf h_jobs, h_items, h_slots, h_out;
  DevBuf d_jobs, d_items, d_slots, d_partials, d_out, d_counter;
  std::map<uint64_t, DevBuf> seed_tables;  // seed -> [4][kDefaultStreams] states
  cudaGraphExec_t graph = nullptr;
  uint64_t graph_key = 0;
  struct Tuned {
    BatchShape shape;
    unsigned int blocks;
    int tuned;
    double tuned_ms, default_ms;
  };
  std::map<uint64_t, Tuned> tuned;  // (segment class, batch shape) -> launch shape and grid
  std::vector<myql_batch_class_plan> last_plan;  // the segments of the last call
  BatchShape forced{0, 0, 0};                    // block 0: the autotuner decides
  static constexpr int kSide = 4;                  // side streams of the concurrent class kernels
  cudaStream_t side[kSide] = {};
  cudaEvent_t fork = nullptr, join[kSide] = {};
  cudaError_t ensure_streams() {
    if (fork) return cudaSuccess;
    cudaError_t e = cudaEventCreateWithFlags(&fork, cudaEventDisableTiming);
    for (int i = 0; i < kSide && e == cudaSuccess; ++i) {
      e = cudaStreamCreateWithFlags(&side[i], cudaStreamNonBlocking);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&join[i], cudaEventDisableTiming);
    }
    return e;
  }
  ~BatchState() {
    if (graph) cudaGraphExecDestroy(graph);
    for (int i = 0; i < kSide; ++i) {
      if (side[i]) cudaStreamDestroy(side[i]);
      if (join[i]) cudaEventDestroy(join[i]);
    }
    if (fork) cudaEventDestroy(fork);
  }
};

// Items of one kernel class (klass, path dependence): [begin, end) of the sorted list.
struct Segment {
  int klass;
  bool pd;
  uint64_t begin, end;
  unsigned int blocks;
  BatchShape shape;
};

// The autotuner's launch shapes; the first is the default.
constexpr BatchShape kShapes[] = {{128, 1, 0}, {64, 2, 0}, {256, 1, 0}, {128, 2, 0}, {256, 2, 0}, {128, 1, 2}};

unsigned int items_per_pull(const BatchShape &sh) {
  return (unsigned int)(sh.block * sh.streams_per_thread / kBatchItemStreams);
}

bool shape_ok(const BatchShape &sh) {
  return (sh.block == 64 || sh.block == 128 || sh.block == 256) &&
         (sh.streams_per_thread == 1 || sh.streams_per_thread == 2 || sh.streams_per_thread == 4) &&
         (sh.unroll == 0 || sh.unroll == 2) && (sh.block * sh.streams_per_thread) % kBatchItemStreams == 0;
}

uint64_t mix(uint64_t h, uint64_t v) { return (h ^ v) * 0x100000001b3ull + (h >> 29); }

}  // namespace

cudaError_t launch_seed_streams(unsigned long long seed, unsigned long long first,
                                unsigned long long n, unsigned long long *out, cudaStream_t stream);

}  // namespace myql

using namespace myql;

extern "C" myql_status myql_mc_price_batch(myql_ctx *ctx_, const myql_mc_job *jobs, size_t n_jobs,
                                           double *const *outs, myql_mc_stats *stats) {
  CtxBase *ctx = reinterpret_cast<CtxBase *>(ctx_);
  if (!ctx || !jobs || !outs || n_jobs == 0) return set_error(MYQL_ERR_INVALID_ARG, "null batch argument");
  if (n_jobs > (1u << 24)) return set_error(MYQL_ERR_TOO_LARGE, "at most 2^24 jobs per batch");
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) return cuda_status(e, "cudaSetDevice");
  if (!ctx->batch) ctx->batch.reset(new BatchState);
  BatchState &B = *static_cast<BatchState *>(ctx->batch.get());
  cudaStream_t st = ctx->stream;

  // ---- plan every job
  std::vector<Plan> plans(n_jobs);
  uint64_t total_items = 0, path_steps = 0, paths = 0;
  std::map<uint64_t, uint64_t> seed_need;  // seed -> streams needed (offset + S)
  for (size_t j = 0; j < n_jobs; ++j) {
    const myql_mc_job &job = jobs[j];
    if (!outs[j]) return set_error(MYQL_ERR_INVALID_ARG, "job %zu: null output", j);
    myql_status s = validate_job(job);
    if (s != MYQL_OK) return set_error(s, "job %zu: %s", j, g_err_message());
    if (job.instrument.is_strip || job.instrument.n_strikes != 1 || job.config.greek_mode == MYQL_GREEKS_FULL)
      return set_error(MYQL_ERR_UNSUPPORTED,
                       "job %zu: batches take scalar instruments with GreekMode None or Essential", j);
    s = make_plan(job, plans[j]);
    if (s != MYQL_OK) return s;
    const uint64_t need = job.config.stream_offset + plans[j].S;
    if (need > kDefaultStreams * 64ull) return set_error(MYQL_ERR_TOO_LARGE, "job %zu: stream range too large", j);
    uint64_t &cur = seed_need[job.config.seed];
    cur = std::max(cur, need);
    total_items += (plans[j].S + kBatchItemStreams - 1) / kBatchItemStreams;
    path_steps += plans[j].M * (uint64_t)plans[j].steps;
    paths += plans[j].M;
  }
  // ---- stream tables, one per seed (kept across calls; 32 bytes per stream)
  uint64_t table_bytes = 0;
  for (auto &kv : seed_need) table_bytes += ((kv.second + 1023) & ~1023ull) * 32;
  if (table_bytes > (8ull << 30))
    return set_error(MYQL_ERR_TOO_LARGE, "stream tables of the batch's seeds exceed 8 GiB");
  {
    uint64_t cached = 0;
    for (auto &kv : B.seed_tables) cached += kv.second.cap;
    if (cached > (2ull << 30))  // drop the tables this batch does not use
      for (auto it = B.seed_tables.begin(); it != B.seed_tables.end();)
        it = seed_need.count(it->first) ? std::next(it) : B.seed_tables.erase(it);
  }
  std::map<uint64_t, std::pair<const unsigned long long *, uint64_t>> tables;
  ctx->launches = 0;
  for (auto &kv : seed_need) {
    DevBuf &tb = B.seed_tables[kv.first];
    const uint64_t n = (kv.second + 1023) & ~1023ull;
    if (tb.cap < n * 32) {
      e = tb.ensure(n * 32);
      if (e == cudaSuccess) e = launch_seed_streams(kv.first, 0, n, (unsigned long long *)tb.p, st);
      if (e != cudaSuccess) return cuda_status(e, "batch seed table");
      ctx->launches++;
    }
    tables[kv.first] = {(const unsigned long long *)tb.p, tb.cap / 32};
  }
  e = ctx->status.ensure(16);
  if (e == cudaSuccess) e = cudaMemsetAsync(ctx->status.p, 0, 16, st);
  if (e != cudaSuccess) return cuda_status(e, "status");

  // ---- host staging: jobs, items, slots
  e = B.h_jobs.ensure(n_jobs * sizeof(BatchJob));
  if (e == cudaSuccess) e = B.h_items.ensure(total_items * sizeof(BatchItem));
  if (e == cudaSuccess) e = B.h_slots.ensure(total_items * sizeof(unsigned int));
  if (e == cudaSuccess) e = B.h_out.ensure(n_jobs * 2 * kQ * sizeof(double));
  if (e == cudaSuccess) e = B.d_jobs.ensure(n_jobs * sizeof(BatchJob));
  if (e == cudaSuccess) e = B.d_items.ensure(total_items * sizeof(BatchItem));
  if (e == cudaSuccess) e = B.d_slots.ensure(total_items * sizeof(unsigned int));
  if (e == cudaSuccess) e = B.d_partials.ensure(total_items * kBatchQ * 2 * sizeof(double));
  if (e == cudaSuccess) e = B.d_out.ensure(n_jobs * 2 * kQ * sizeof(double));
  if (e == cudaSuccess) e = B.d_counter.ensure(256);
  if (e == cudaSuccess) e = ctx->strikes.ensure(n_jobs * sizeof(double));
  if (e != cudaSuccess) return cuda_status(e, "batch buffers");
  BatchJob *hj = (BatchJob *)B.h_jobs.p;
  BatchItem *hi = (BatchItem *)B.h_items.p;
  unsigned int *hs = (unsigned int *)B.h_slots.p;
  std::vector<double> strikes(n_jobs);
  std::vector<double> cost(total_items);
  std::vector<int> seg_key(total_items);  // 2 klass + path dependence
  uint64_t item = 0;
  uint64_t signature = 0;
  // NCI tables: a later job may grow (reallocate) a table an earlier job of the
  // same dimension d already points at, so build everything first and take the
  // pointers in a second pass.
  for (int pass = 0; pass < 2; ++pass)
    for (size_t j = 0; j < n_jobs; ++j)
      for (int f = 0; f < plans[j].nf; ++f)
        if (jobs[j].config.scheme[f] == MYQL_SCHEME_NCI) {
          myql_status s = ensure_nci(ctx, jobs[j].model.heston[f], plans[j].sim.sc[0].dt, plans[j].sim.nci[f]);
          if (s != MYQL_OK) return s;
        }
  for (size_t j = 0; j < n_jobs; ++j) {
    const myql_mc_job &job = jobs[j];
    Plan &pl = plans[j];
    BatchJob &J = hj[j];
    std::memset(&J, 0, sizeof J);
    J.sim = pl.sim;
    J.pay = pl.pay;
    const auto &tb = tables[job.config.seed];
    J.sim.states = const_cast<unsigned long long *>(tb.first);
    J.sim.status = (unsigned int *)ctx->status.p;
    J.sim.loop_cap = ctx->loop_cap;
    J.state_stride = tb.second;
    J.stream_base = job.config.stream_offset;
    strikes[j] = job.instrument.strikes[0];
    J.pay.strikes = (const double *)ctx->strikes.p + j;
    J.klass = batch_class(pl.nf, pl.s1, pl.s2);
    J.mode = pl.mode;
    J.df = pl.df;
    J.first_item = item;
    J.n_items = (pl.S + kBatchItemStreams - 1) / kBatchItemStreams;
    const double per_stream = (double)((pl.M + pl.S - 1) / pl.S) * pl.steps *
                              (1.0 + pl.nf + (pl.s1 >= 2 ? 1.5 : 0.0) + (pl.s2 >= 2 ? 1.5 : 0.0));
    for (uint64_t k = 0; k < J.n_items; ++k, ++item) {
      hi[item].job = (unsigned int)j;
      hi[item].stream0 = (unsigned int)(k * kBatchItemStreams);
      cost[item] = per_stream;
      seg_key[item] = 2 * J.klass + (pl.path_dep ? 1 : 0);
    }
    signature = mix(signature, (uint64_t)J.klass * 1315423911ull + pl.steps * 2 + (pl.path_dep ? 1 : 0));
  }
  // grouped by kernel class, longest items first within a class; slot = item index in
  // job order (finalize sums slots in order)
  std::vector<uint64_t> order(total_items);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](uint64_t a, uint64_t b) {
    return seg_key[a] != seg_key[b] ? seg_key[a] < seg_key[b] : cost[a] > cost[b];
  });
  std::vector<Segment> segs;
  for (uint64_t k = 0; k < total_items; ++k) {
    const int key = seg_key[order[k]];
    if (segs.empty() || 2 * segs.back().klass + (segs.back().pd ? 1 : 0) != key)
      segs.push_back({key / 2, (key & 1) != 0, k, k, 0u, kShapes[0]});
    segs.back().end = k + 1;
  }
  if (segs.size() > 64) return set_error(MYQL_ERR_TOO_LARGE, "too many kernel classes");
  {
    std::vector<BatchItem> tmp(hi, hi + total_items);
    for (uint64_t k = 0; k < total_items; ++k) {
      hi[k] = tmp[order[k]];
      hs[k] = (unsigned int)order[k];
    }
  }
  e = cudaMemcpyAsync(ctx->strikes.p, strikes.data(), n_jobs * sizeof(double), cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return cuda_status(e, "batch strikes");

  e = B.ensure_streams();
  if (e != cudaSuccess) return cuda_status(e, "batch streams");
  auto params_of = [&](const Segment &g, size_t gi) {
    BatchParams P;
    P.jobs = (const BatchJob *)B.d_jobs.p;
    P.items = (const BatchItem *)B.d_items.p;
    P.item_slot = (const unsigned int *)B.d_slots.p;
    P.item_begin = g.begin;
    P.item_end = g.end;
    P.counter = (unsigned int *)B.d_counter.p + gi;
    P.partials = (double *)B.d_partials.p;
    P.streams_per_thread = (unsigned int)g.shape.streams_per_thread;
    P.items_per_pull = items_per_pull(g.shape);
    return P;
  };

  // ---- autotune each class segment's launch shape and persistent grid once per batch
  // shape: every candidate runs the segment's leading (most expensive) items
  signature = mix(signature, n_jobs);
  bool uploaded = false;
  const bool forced = B.forced.block != 0;
  B.last_plan.clear();
  for (size_t gi = 0; gi < segs.size(); ++gi) {
    Segment &g = segs[gi];
    const uint64_t n = g.end - g.begin;
    auto grid_of = [&](const BatchShape &sh, int per_sm) {
      const uint64_t pulls = (n + items_per_pull(sh) - 1) / items_per_pull(sh);
      return (unsigned int)std::max<uint64_t>(1, std::min<uint64_t>(pulls, (uint64_t)per_sm * ctx->sm_count));
    };
    const uint64_t tkey = mix(signature, 2 * g.klass + (g.pd ? 1 : 0));
    BatchState::Tuned tu{forced ? B.forced : kShapes[0], 0u, 0, 0.0, 0.0};
    auto cached = B.tuned.find(tkey);
    if (forced) {
      tu.blocks = grid_of(tu.shape, batch_blocks_per_sm(g.klass, g.pd, tu.shape));
    } else if (cached != B.tuned.end()) {
      tu = cached->second;
    } else {
      const int occ0 = batch_blocks_per_sm(g.klass, g.pd, kShapes[0]);
      tu.blocks = grid_of(kShapes[0], occ0);
      if (n > (uint64_t)8 * occ0 * ctx->sm_count) {
        if (!uploaded) {
          e = cudaMemcpyAsync(B.d_jobs.p, hj, n_jobs * sizeof(BatchJob), cudaMemcpyHostToDevice, st);
          if (e == cudaSuccess) e = cudaMemcpyAsync(B.d_items.p, hi, total_items * sizeof(BatchItem), cudaMemcpyHostToDevice, st);
          if (e == cudaSuccess) e = cudaMemcpyAsync(B.d_slots.p, hs, total_items * sizeof(unsigned int), cudaMemcpyHostToDevice, st);
          if (e != cudaSuccess) return cuda_status(e, "batch autotune upload");
          uploaded = true;
        }
        // the same leading items for every candidate
        const uint64_t n_tune = std::min<uint64_t>(n, (uint64_t)4 * occ0 * ctx->sm_count);
        auto time_one = [&](const BatchShape &sh, unsigned int blocks, uint64_t items, float &ms) {
          Segment t = g;
          t.shape = sh;
          BatchParams T = params_of(t, gi);
          T.item_end = g.begin + items;
          cudaError_t er = cudaMemsetAsync(T.counter, 0, 4, st);
          if (er == cudaSuccess) er = cudaEventRecord(ctx->ev0, st);
          if (er == cudaSuccess) er = launch_batch(T, g.klass, g.pd, sh, blocks, st);
          if (er == cudaSuccess) er = cudaEventRecord(ctx->ev1, st);
          if (er == cudaSuccess) er = cudaEventSynchronize(ctx->ev1);
          ms = 0.0f;
          if (er == cudaSuccess) cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
          ctx->launches++;
          return er;
        };
        float best = 1e30f;
        int best_occ = occ0;
        for (const BatchShape &sh : kShapes) {
          const int occ = batch_blocks_per_sm(g.klass, g.pd, sh);
          const unsigned int pulls = (unsigned int)((n_tune + items_per_pull(sh) - 1) / items_per_pull(sh));
          const unsigned int blocks = std::min<unsigned int>(pulls, (unsigned int)occ * (unsigned int)ctx->sm_count);
          float ms = 0.0f;
          e = time_one(sh, 1, items_per_pull(sh), ms);  // first launch of the variant: loads the kernel
          if (e == cudaSuccess) e = time_one(sh, blocks, n_tune, ms);
          if (e != cudaSuccess) return cuda_status(e, "batch autotune");
          if (&sh == &kShapes[0]) tu.default_ms = ms;
          if (ms < best) {
            best = ms;
            tu.shape = sh;
            best_occ = occ;
          }
        }
        // the persistent grid of the chosen shape: full occupancy (timed above), half, one
        // block per SM
        const unsigned int pulls = (unsigned int)((n_tune + items_per_pull(tu.shape) - 1) / items_per_pull(tu.shape));
        const unsigned int full = std::min<unsigned int>(pulls, (unsigned int)best_occ * (unsigned int)ctx->sm_count);
        int per_sm = best_occ;
        for (int cand : {std::max(1, best_occ / 2), 1}) {
          const unsigned int c = (unsigned int)cand * (unsigned int)ctx->sm_count;
          if (cand >= per_sm || c >= full) continue;
          float ms = 0.0f;
          e = time_one(tu.shape, c, n_tune, ms);
          if (e != cudaSuccess) return cuda_status(e, "batch autotune");
          if (ms < best) {
            best = ms;
            per_sm = cand;
          }
        }
        tu.tuned = 1;
        tu.tuned_ms = best;
        tu.blocks = grid_of(tu.shape, per_sm);
      }
      B.tuned[tkey] = tu;
    }
    g.shape = tu.shape;
    g.blocks = tu.blocks;
    myql_batch_class_plan cp;
    std::memset(&cp, 0, sizeof cp);
    cp.factors = g.klass == BK_F0 ? 0 : (g.klass < BK_F2_NV_NV ? 1 : 2);
    cp.scheme1 = g.klass == BK_F0 ? 0 : (g.klass < BK_F2_NV_NV ? g.klass : 1 + (g.klass - BK_F2_NV_NV) / 3);
    cp.scheme2 = g.klass < BK_F2_NV_NV ? 0 : 1 + (g.klass - BK_F2_NV_NV) % 3;
    cp.path_dependent = g.pd ? 1 : 0;
    cp.block = g.shape.block;
    cp.streams_per_thread = g.shape.streams_per_thread;
    cp.unroll = g.shape.unroll;
    cp.tuned = forced ? -1 : tu.tuned;
    cp.grid = g.blocks;
    cp.items = n;
    cp.tuned_ms = tu.tuned_ms;
    cp.default_ms = tu.default_ms;
    B.last_plan.push_back(cp);
  }

  // ---- the batch itself, through a CUDA graph per shape: the class kernels run
  // concurrently on side streams between the uploads and the finalize
  uint64_t key = mix(signature, total_items);
  for (const Segment &g : segs)
    key = mix(mix(mix(key, g.end), g.blocks), (uint64_t)(g.shape.block * 64 + g.shape.streams_per_thread * 4 + g.shape.unroll));
  for (const void *ptr : {B.h_jobs.p, B.h_items.p, B.h_slots.p, B.h_out.p, B.d_jobs.p, B.d_items.p, B.d_slots.p,
                          B.d_partials.p, B.d_out.p, B.d_counter.p})
    key = mix(key, (uint64_t)(uintptr_t)ptr);
  if (!B.graph || B.graph_key != key) {
    if (B.graph) cudaGraphExecDestroy(B.graph);
    B.graph = nullptr;
    cudaGraph_t gr = nullptr;
    e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) e = cudaMemcpyAsync(B.d_jobs.p, B.h_jobs.p, n_jobs * sizeof(BatchJob), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(B.d_items.p, B.h_items.p, total_items * sizeof(BatchItem), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(B.d_slots.p, B.h_slots.p, total_items * sizeof(unsigned int), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(B.d_counter.p, 0, segs.size() * 4, st);
    if (e == cudaSuccess) e = cudaEventRecord(B.fork, st);
    const int ns = (int)std::min<size_t>(segs.size(), (size_t)BatchState::kSide);
    for (int i = 0; i < ns && e == cudaSuccess; ++i) e = cudaStreamWaitEvent(B.side[i], B.fork, 0);
    for (size_t gi = 0; gi < segs.size() && e == cudaSuccess; ++gi)
      e = launch_batch(params_of(segs[gi], gi), segs[gi].klass, segs[gi].pd, segs[gi].shape, segs[gi].blocks,
                       B.side[gi % BatchState::kSide]);
    for (int i = 0; i < ns && e == cudaSuccess; ++i) {
      e = cudaEventRecord(B.join[i], B.side[i]);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(st, B.join[i], 0);
    }
    if (e == cudaSuccess)
      e = launch_batch_finalize((const BatchJob *)B.d_jobs.p, (unsigned int)n_jobs, (const double *)B.d_partials.p,
                                (double *)B.d_out.p, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(B.h_out.p, B.d_out.p, n_jobs * 2 * kQ * sizeof(double), cudaMemcpyDeviceToHost, st);
    cudaError_t e2 = cudaStreamEndCapture(st, &gr);
    if (e == cudaSuccess) e = e2;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&B.graph, gr, 0);
    if (gr) cudaGraphDestroy(gr);
    if (e != cudaSuccess) {
      B.graph = nullptr;
      return cuda_status(e, "batch graph capture");
    }
    B.graph_key = key;
  }
  e = cudaEventRecord(ctx->ev0, st);
  if (e == cudaSuccess) e = cudaGraphLaunch(B.graph, st);
  if (e == cudaSuccess) e = cudaEventRecord(ctx->ev1, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_status(e, "batch run");
  ctx->launches += (uint32_t)segs.size() + 1;
  const double *ho = (const double *)B.h_out.p;
  for (size_t j = 0; j < n_jobs; ++j) {
    // [quantity][value, se] -> the myql_mc_price layout [2q + (0|1)][strike]
    std::memcpy(outs[j], ho + j * 2 * kQ, 2 * kQ * sizeof(double));
  }
  if (stats) {
    std::memset(stats, 0, sizeof *stats);
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    stats->device_ms = ms;
    stats->simulate_ms = ms;
    stats->paths = paths;
    stats->path_steps = path_steps;
    stats->scenarios = 1;
    stats->kernel_launches = ctx->launches;
  }
  return read_status(ctx, stats);
}

extern "C" myql_status myql_batch_last_plan(myql_ctx *ctx_, myql_batch_class_plan *out, size_t cap,
                                            size_t *n_classes) {
  CtxBase *ctx = reinterpret_cast<CtxBase *>(ctx_);
  if (!ctx || !n_classes || (cap && !out)) return set_error(MYQL_ERR_INVALID_ARG, "null argument");
  *n_classes = 0;
  if (!ctx->batch) return MYQL_OK;
  const BatchState &B = *static_cast<const BatchState *>(ctx->batch.get());
  *n_classes = B.last_plan.size();
  for (size_t i = 0; i < B.last_plan.size() && i < cap; ++i) out[i] = B.last_plan[i];
  return MYQL_OK;
}

extern "C" myql_status myql_ctx_set_batch_shape(myql_ctx *ctx_, int block, int streams_per_thread, int unroll) {
  CtxBase *ctx = reinterpret_cast<CtxBase *>(ctx_);
  if (!ctx) return set_error(MYQL_ERR_INVALID_ARG, "null context");
  const BatchShape sh{block, streams_per_thread, unroll};
  if (block != 0 && !shape_ok(sh))
    return set_error(MYQL_ERR_INVALID_ARG,
                     "batch shape: block 64/128/256, streams per thread 1/2/4 (block x streams a multiple "
                     "of 128), unroll 0 or 2; block 0 returns to the autotuner");
  if (!ctx->batch) ctx->batch.reset(new BatchState);
  static_cast<BatchState *>(ctx->batch.get())->forced = block ? sh : BatchShape{0, 0, 0};
  return MYQL_OK;
}
