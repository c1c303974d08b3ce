// batch_kernel.cu -- launchers of the per-class persistent batch kernels
// (instantiated per block size in batch_k_b64.cu, batch_k_b128.cu, batch_k_b256.cu) and the
// per-job finalize.
#include "batch.cuh"

namespace myql {

cudaError_t batch_dispatch_b64(const BatchParams *B, int klass, bool pd, int unroll, unsigned int blocks,
                               cudaStream_t st, int *occ);
cudaError_t batch_dispatch_b128(const BatchParams *B, int klass, bool pd, int unroll, unsigned int blocks,
                                cudaStream_t st, int *occ);
cudaError_t batch_dispatch_b256(const BatchParams *B, int klass, bool pd, int unroll, unsigned int blocks,
                                cudaStream_t st, int *occ);

static cudaError_t batch_dispatch_any(const BatchParams *B, int klass, bool pd, const BatchShape &sh,
                                      unsigned int blocks, cudaStream_t st, int *occ) {
  switch (sh.block) {
    case 64: return batch_dispatch_b64(B, klass, pd, sh.unroll, blocks, st, occ);
    case 128: return batch_dispatch_b128(B, klass, pd, sh.unroll, blocks, st, occ);
    case 256: return batch_dispatch_b256(B, klass, pd, sh.unroll, blocks, st, occ);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_batch(const BatchParams &B, int klass, bool pd, const BatchShape &shape, unsigned int blocks,
                         cudaStream_t st) {
  if (blocks == 0) return cudaErrorInvalidValue;
  return batch_dispatch_any(&B, klass, pd, shape, blocks, st, nullptr);
}

int batch_blocks_per_sm(int klass, bool pd, const BatchShape &shape) {
  int n = 0;
  if (batch_dispatch_any(nullptr, klass, pd, shape, 0, nullptr, &n) != cudaSuccess) return 1;
  return n > 0 ? n : 1;
}

namespace dev {

// One thread per (job, quantity): fixed-order sum of the job's item slots.
__global__ void batch_finalize_kernel(const BatchJob *jobs, unsigned int n_jobs, const double *partials,
                                      double *outs) {
  const unsigned int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n_jobs * kQ) return;
  const unsigned int j = idx / kQ, q = idx % kQ;
  const BatchJob &J = jobs[j];
  double s = 0.0, ss = 0.0;
  const bool active = q == 0 || (J.mode != 0 && q < kBatchQ);
  if (active)
    for (unsigned long long t = 0; t < J.n_items; ++t) {
      const double *p = partials + ((J.first_item + t) * kBatchQ + q) * 2;
      s += p[0];
      ss += p[1];
    }
  const double inv_m = 1.0 / (double)J.sim.num_paths;
  const double mean = s * inv_m;
  double var = ss * inv_m - mean * mean;
  if (var < 0.0) var = 0.0;
  outs[(size_t)j * 2 * kQ + 2 * q] = mean * J.df;
  outs[(size_t)j * 2 * kQ + 2 * q + 1] = sqrt(var * inv_m) * J.df;
}

}  // namespace dev

cudaError_t launch_batch_finalize(const BatchJob *jobs, unsigned int n_jobs, const double *partials,
                                  double *outs, cudaStream_t st) {
  const unsigned int n = n_jobs * kQ;
  dev::batch_finalize_kernel<<<(n + 127) / 128, 128, 0, st>>>(jobs, n_jobs, partials, outs);
  return cudaGetLastError();
}

}  // namespace myql
