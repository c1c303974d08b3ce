// engine.h -- host-side context shared by the C ABI translation units.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <string>

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

struct CtxBase {
  int device = 0;
  int sm_count = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  uint32_t loop_cap = kDefaultLoopCap;
  uint32_t launches = 0;
  uint64_t records_cap_bytes = 2ull << 30;  // per-path record scratch per chunk
  // xoshiro stream-state table of the last (seed, n)
  bool st_valid = false;
  uint64_t st_seed = 0, st_n = 0;
  DevBuf st_cached, st_work;
  std::map<uint64_t, NciEntry> nci;  // keyed by the bits of d = 4 kappa theta / sigma^2
  DevBuf records, partials, out, status, strikes;
  DevBuf probe_a, probe_b, probe_c;
  DevBuf aux_a, aux_b, aux_c, aux_d;  // batch / MLMC / control-variate work buffers
  void release_all() {
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

}  // namespace myql
