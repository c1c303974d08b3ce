// batch_kernel.cu -- the persistent batch kernel and its per-job finalize.
#include "batch.cuh"

namespace myql {
namespace dev {

template <bool PD>
__device__ __forceinline__ void dispatch_item(const BatchJob &J, unsigned int stream0,
                                              double (&acc)[kBatchQ][2], unsigned int &caphits,
                                              unsigned int &fallbacks) {
  switch (J.klass) {
    case BK_F0: batch_item<0, SCH_NONE, SCH_NONE, PD>(J, stream0, acc, caphits, fallbacks); break;
    case BK_F1_NV: batch_item<1, SCH_NV, SCH_NONE, PD>(J, stream0, acc, caphits, fallbacks); break;
    case BK_F1_EXACT: batch_item<1, SCH_EXACT, SCH_NONE, PD>(J, stream0, acc, caphits, fallbacks); break;
    case BK_F1_NCI: batch_item<1, SCH_NCI, SCH_NONE, PD>(J, stream0, acc, caphits, fallbacks); break;
    case BK_F2_NV_NV: batch_item<2, SCH_NV, SCH_NV, PD>(J, stream0, acc, caphits, fallbacks); break;
    case BK_F2_NV_EXACT: batch_item<2, SCH_NV, SCH_EXACT, PD>(J, stream0, acc, caphits, fallbacks); break;
    case BK_F2_NV_NCI: batch_item<2, SCH_NV, SCH_NCI, PD>(J, stream0, acc, caphits, fallbacks); break;
    case BK_F2_EXACT_NV: batch_item<2, SCH_EXACT, SCH_NV, PD>(J, stream0, acc, caphits, fallbacks); break;
    case BK_F2_EXACT_EXACT: batch_item<2, SCH_EXACT, SCH_EXACT, PD>(J, stream0, acc, caphits, fallbacks); break;
    case BK_F2_EXACT_NCI: batch_item<2, SCH_EXACT, SCH_NCI, PD>(J, stream0, acc, caphits, fallbacks); break;
    case BK_F2_NCI_NV: batch_item<2, SCH_NCI, SCH_NV, PD>(J, stream0, acc, caphits, fallbacks); break;
    case BK_F2_NCI_EXACT: batch_item<2, SCH_NCI, SCH_EXACT, PD>(J, stream0, acc, caphits, fallbacks); break;
    default: batch_item<2, SCH_NCI, SCH_NCI, PD>(J, stream0, acc, caphits, fallbacks); break;
  }
}

// Persistent: every block loops pulling items until the queue is empty.
__global__ void __launch_bounds__(kSimBlock) batch_kernel(const BatchParams B) {
  __shared__ unsigned int item_sh;
  __shared__ double red[kSimBlock / 32][kBatchQ][2];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  unsigned int caphits = 0, fallbacks = 0;
  unsigned int *status = nullptr;
  for (;;) {
    if (threadIdx.x == 0) item_sh = atomicAdd(B.counter, 1u);
    __syncthreads();
    const unsigned long long it = item_sh;
    __syncthreads();
    if (it >= B.n_items) break;
    const BatchItem I = B.items[it];
    const BatchJob &J = B.jobs[I.job];
    status = J.sim.status;
    double acc[kBatchQ][2] = {{0.0, 0.0}, {0.0, 0.0}, {0.0, 0.0}};
    if (J.sim.tracker != TRK_EUROPEAN)
      dispatch_item<true>(J, I.stream0, acc, caphits, fallbacks);
    else
      dispatch_item<false>(J, I.stream0, acc, caphits, fallbacks);
#pragma unroll
    for (int q = 0; q < kBatchQ; ++q)
#pragma unroll
      for (int k = 0; k < 2; ++k) {
        double v = acc[q][k];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) red[warp][q][k] = v;
      }
    __syncthreads();
    if (threadIdx.x < kBatchQ * 2) {
      const int q = threadIdx.x >> 1, k = threadIdx.x & 1;
      double t = 0.0;
      for (int w = 0; w < kSimBlock / 32; ++w) t += red[w][q][k];
      B.partials[((size_t)B.item_slot[it] * kBatchQ + q) * 2 + k] = t;
    }
  }
  if (status && (caphits || fallbacks)) {
    if (caphits) atomicAdd(status, caphits);
    if (fallbacks) atomicAdd(status + 1, fallbacks);
  }
}

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
  const double df = J.df;
  const double mean = s * inv_m;
  double var = ss * inv_m - mean * mean;
  if (var < 0.0) var = 0.0;
  outs[(size_t)j * 2 * kQ + 2 * q] = mean * df;
  outs[(size_t)j * 2 * kQ + 2 * q + 1] = sqrt(var * inv_m) * df;
}

}  // namespace dev

cudaError_t launch_batch(const BatchParams &B, unsigned int blocks, cudaStream_t st) {
  dev::batch_kernel<<<blocks, kSimBlock, 0, st>>>(B);
  return cudaGetLastError();
}

cudaError_t launch_batch_finalize(const BatchJob *jobs, unsigned int n_jobs, const double *partials,
                                  double *outs, cudaStream_t st) {
  const unsigned int n = n_jobs * kQ;
  dev::batch_finalize_kernel<<<(n + 127) / 128, 128, 0, st>>>(jobs, n_jobs, partials, outs);
  return cudaGetLastError();
}

int batch_blocks_per_sm() {
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, dev::batch_kernel, kSimBlock, 0) != cudaSuccess) return 1;
  return n > 0 ? n : 1;
}

}  // namespace myql
