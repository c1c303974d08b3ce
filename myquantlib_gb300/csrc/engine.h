// engine.h -- host-side context shared by the C ABI translation units.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "engine_types.h"
#include "myql_gpu.h"

namespace myql {

constexpr uint32_t kDefaultLoopCap = 100000u;

// Device buffer that only grows.
struct DevBuf {
  void *p = nullptr;
  size_t cap = 0;
  DevBuf() = default;
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  DevBuf(DevBuf &&o) noexcept : p(o.p), cap(o.cap) { o.p = nullptr, o.cap = 0; }
  ~DevBuf() { release(); }
  cudaError_t ensure(size_t bytes);
  void release();
};

struct NciEntry {
  int rows = 0;
  double d = 0.0;
  DevBuf main, tail;
};

// Per-context state owned by another subsystem (batch queue, control variates).
struct ExtState {
  virtual ~ExtState() = default;
};

struct CtxBase {
  int device = 0;
  int sm_count = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  uint32_t loop_cap = kDefaultLoopCap;
  int nci_slopes = 0;  // NCI table cells: 0 the reference's, 1 exact slopes and a mean-preserving first cell
  int nci_rows_cap = 0;  // at most this many NCI table rows (0: the sizing rule alone, at most 1024)
  int precise_theta = 0;  // myql_ctx_set_precise_theta
  uint32_t launches = 0;
  uint64_t records_cap_bytes = 2ull << 30;  // per-path record scratch per chunk
  // xoshiro stream-state table of the last (seed, n)
  bool st_valid = false;
  uint64_t st_seed = 0, st_first = 0, st_n = 0;
  DevBuf st_cached, st_work;
  std::map<uint64_t, NciEntry> nci;  // keyed by the bits of d = 4 kappa theta / sigma^2
  DevBuf records, partials, out, status, strikes;
  DevBuf probe_a, probe_b, probe_c;
  DevBuf aux_a, aux_b, aux_c, aux_d;  // batch / MLMC / control-variate work buffers
  std::unique_ptr<ExtState> batch, cv, qmc;  // released with the context
  // event pairs around the phase launches of the current call (tag 0 = simulate, 1 = payoff)
  std::vector<cudaEvent_t> ev_pool;
  std::vector<int> ev_tags;
  size_t ev_used = 0;
  void phase_reset() { ev_used = 0; ev_tags.clear(); }
  cudaEvent_t phase_event() {
    if (ev_used == ev_pool.size()) {
      cudaEvent_t e;
      cudaEventCreate(&e);
      ev_pool.push_back(e);
    }
    return ev_pool[ev_used++];
  }
  void release_all() {
    batch.reset();
    cv.reset();
    qmc.reset();
    for (cudaEvent_t e : ev_pool) cudaEventDestroy(e);
    ev_pool.clear();
    st_cached.release();
    st_work.release();
    nci.clear();
    records.release();
    partials.release();
    out.release();
    status.release();
    strikes.release();
    probe_a.release();
    probe_b.release();
    probe_c.release();
    aux_a.release();
    aux_b.release();
    aux_c.release();
    aux_d.release();
  }
};

myql_status set_error(myql_status st, const char *fmt, ...);
myql_status cuda_status(cudaError_t e, const char *what);
const char *g_err_message();  // the calling thread's last error text

// Job planning: everything the launches need, computed in FP64 on the host.
struct Plan {
  int nf = 0, s1 = 0, s2 = 0, tracker = 0, n_fields = 1, n_sc = 1, mode = 0;
  bool path_dep = false;
  uint64_t M = 0, S = 0;
  int steps = 0;
  double T = 0, df = 1;
  SimParams sim;
  PayoffParams pay;
  int active_mask = 1;
};


// planning helpers (engine.cu)
int tracker_of(const myql_instrument &in);
myql_status validate_job(const myql_mc_job &job);
// stepped: per-step GBM and jump constants even for Europeans (control variates)
myql_status make_plan(const myql_mc_job &job, Plan &pl, bool stepped = false);
void fill_factor(FactorConst &fc, const myql_heston_params &h, double v0, int scheme, double r_part,
                 double dt, float *lo = nullptr);
unsigned long long u999_threshold();
double expected_avg_variance(const myql_heston_params &h, double T);
double jump_variance(const myql_model &m);
int nci_rows_wanted(const myql_heston_params &p, double dt_min);
myql_status ensure_streams(CtxBase *ctx, uint64_t seed, uint64_t first, uint64_t n);
myql_status ensure_nci(CtxBase *ctx, const myql_heston_params &p, double dt_min, NciTable &tab);
myql_status read_status(CtxBase *ctx, myql_mc_stats *stats);
// event-timed simulate / payoff phases of the last call
void phase_times(CtxBase *ctx, double *sim_ms, double *pay_ms);
cudaError_t launch_payoff(const PayoffParams &P, unsigned long long n_tiles, cudaStream_t stream);

}  // namespace myql
