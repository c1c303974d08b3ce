// batch_kernel.cu -- launchers of the per-class persistent batch kernels
// (instantiated in batch_k_f01.cu and batch_k_f2.cu) and the per-job finalize.
#include "batch.cuh"

namespace myql {

cudaError_t launch_batch_f01(const BatchParams &B, int klass, bool pd, unsigned int blocks, cudaStream_t st);
cudaError_t launch_batch_f2(const BatchParams &B, int klass, bool pd, unsigned int blocks, cudaStream_t st);
int occupancy_batch_f01(int klass, bool pd);
int occupancy_batch_f2(int klass, bool pd);

cudaError_t launch_batch(const BatchParams &B, int klass, bool pd, unsigned int blocks, cudaStream_t st) {
  return klass < BK_F2_NV_NV ? launch_batch_f01(B, klass, pd, blocks, st) : launch_batch_f2(B, klass, pd, blocks, st);
}

int batch_blocks_per_sm(int klass, bool pd) {
  const int n = klass < BK_F2_NV_NV ? occupancy_batch_f01(klass, pd) : occupancy_batch_f2(klass, pd);
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
