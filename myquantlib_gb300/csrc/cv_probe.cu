// cv_probe.cu -- one-tile tcgen05 GEMM used to check the operand-image and
// descriptor conventions of tc.cuh against a host product: D[128][N] =
// A[128][K] * B[N][K]^T with BF16 operands and FP32 accumulation.
//   mode 0: K = 16,  IMG16 operands, N = 128
//   mode 1: K = 128, IMG128 operands, N = 128
//   mode 2: K = 128, IMG128 operands, N = 16
//   mode 3: K = 128, N = 128, both operands MN-major: the IMG128 image of the
//           transposed matrix ([K][M] and [K][N]); leading offset = stride
//           between 64-element MN blocks (16 KB), stride offset = stride
//           between 8-row K groups (1024 B)
#include <cuda_bf16.h>

#include <cstring>
#include <vector>

#include "engine.h"
#include "tc.cuh"

namespace myql {
namespace dev {

__global__ void __launch_bounds__(128) mma_probe_kernel(const uint4 *a_img, uint32_t a_bytes, const uint4 *b_img,
                                                        uint32_t b_bytes, int mode, int N, float *D,
                                                        unsigned int *status) {
  extern __shared__ uint8_t dyn[];
  __shared__ uint64_t mbar;
  __shared__ uint32_t tmem_base;
  const uint32_t base = tc::smem_u32(dyn);
  uint8_t *sa = dyn + (((base + 1023u) & ~1023u) - base);
  uint8_t *sb = sa + ((a_bytes + 1023u) & ~1023u);
  for (uint32_t i = threadIdx.x; i < a_bytes / 16; i += blockDim.x) reinterpret_cast<uint4 *>(sa)[i] = a_img[i];
  for (uint32_t i = threadIdx.x; i < b_bytes / 16; i += blockDim.x) reinterpret_cast<uint4 *>(sb)[i] = b_img[i];
  tc::fence_proxy_async();
  const int warp = threadIdx.x >> 5;
  if (warp == 0) {
    tc::tmem_alloc(&tmem_base, 128);
    tc::tmem_relinquish();
  }
  if (threadIdx.x == 0) {
    tc::mbar_init(&mbar, 1);
    tc::fence_mbar_init();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tm = tmem_base;
  if (threadIdx.x == 0) {
    if (mode == 0) {
      tc::mma_bf16(tm, tc::desc_img16(tc::smem_u32(sa)), tc::desc_img16(tc::smem_u32(sb)), tc::idesc_bf16(128, N), 0);
    } else if (mode == 3) {
      for (int kk = 0; kk < 8; ++kk) {
        const uint32_t o = (uint32_t)kk * 16u * 128u;
        tc::mma_bf16(tm, tc::desc_sw128_mn(tc::smem_u32(sa) + o, 16384u), tc::desc_sw128_mn(tc::smem_u32(sb) + o, 16384u),
                     tc::idesc_bf16_mn(128, N, true, true), kk > 0 ? 1u : 0u);
      }
    } else {
      for (int kk = 0; kk < 8; ++kk) {
        const uint32_t ao = (uint32_t)(kk >> 2) * 128u * 128u + (uint32_t)(kk & 3) * 32u;
        const uint32_t bo = (uint32_t)(kk >> 2) * (uint32_t)N * 128u + (uint32_t)(kk & 3) * 32u;
        tc::mma_bf16(tm, tc::desc_sw128(tc::smem_u32(sa) + ao), tc::desc_sw128(tc::smem_u32(sb) + bo),
                     tc::idesc_bf16(128, N), kk > 0 ? 1u : 0u);
      }
    }
    tc::mma_commit(&mbar);
  }
  const bool ok = tc::mbar_wait(&mbar, 0, 1000000000ull);
  tc::fence_after_sync();
  if (ok) {
    const int row = threadIdx.x;
    for (int c = 0; c < N; c += 32) {
      float v[32];
      tc::tmem_ld32(tm + ((uint32_t)(warp * 32) << 16) + (uint32_t)c, v);
      for (int i = 0; i < 32 && c + i < N; ++i) D[row * N + c + i] = v[i];
    }
  } else if (threadIdx.x == 0) {
    atomicAdd(status + 2, 1u);
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (warp == 0) tc::tmem_dealloc(tm, 128);
}

}  // namespace dev

// Host packing of a row-major FP32 matrix into a BF16 operand image.
// mn_major: the image of the transpose ([K][rows], 64-element lines along rows).
void pack_image(const float *m, int rows, int K, std::vector<uint8_t> &img, bool mn_major = false) {
  img.assign((size_t)rows * K * 2, 0);
  for (int r = 0; r < rows; ++r)
    for (int k = 0; k < K; ++k) {
      const uint32_t off = mn_major ? tc::img128_offset(k, r, K)
                                    : (K == 16 ? tc::img16_offset(r, k) : tc::img128_offset(r, k, rows));
      const __nv_bfloat16 b = __float2bfloat16_rn(m[(size_t)r * K + k]);
      std::memcpy(&img[off], &b, 2);
    }
}

}  // namespace myql

using namespace myql;

extern "C" myql_status myql_probe_mma(myql_ctx *ctx_, int32_t mode, const float *A, const float *B, float *D) {
  CtxBase *ctx = reinterpret_cast<CtxBase *>(ctx_);
  if (!ctx || !A || !B || !D || mode < 0 || mode > 3) return set_error(MYQL_ERR_INVALID_ARG, "bad probe arguments");
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) return cuda_status(e, "cudaSetDevice");
  const int K = mode == 0 ? 16 : 128, N = mode == 2 ? 16 : 128;
  std::vector<uint8_t> ai, bi;
  pack_image(A, 128, K, ai, mode >= 3);
  pack_image(B, N, K, bi, mode >= 3);
  e = ctx->probe_a.ensure(ai.size() + bi.size() + (size_t)128 * N * 4);
  if (e == cudaSuccess) e = ctx->status.ensure(16);
  if (e != cudaSuccess) return cuda_status(e, "probe buffers");
  uint8_t *d = (uint8_t *)ctx->probe_a.p;
  float *dD = (float *)(d + ai.size() + bi.size());
  e = cudaMemcpyAsync(d, ai.data(), ai.size(), cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d + ai.size(), bi.data(), bi.size(), cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(ctx->status.p, 0, 16, ctx->stream);
  const uint32_t smem = (uint32_t)(((ai.size() + 1023) & ~1023ull) + bi.size() + 1024);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(dev::mma_probe_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess) {
    dev::mma_probe_kernel<<<1, 128, smem, ctx->stream>>>((const uint4 *)d, (uint32_t)ai.size(),
                                                          (const uint4 *)(d + ai.size()), (uint32_t)bi.size(), mode,
                                                          N, dD, (unsigned int *)ctx->status.p);
    e = cudaGetLastError();
  }
  unsigned int st[4] = {0, 0, 0, 0};
  if (e == cudaSuccess) e = cudaMemcpyAsync(D, dD, (size_t)128 * N * 4, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(st, ctx->status.p, 16, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_status(e, "mma probe");
  if (st[2]) return set_error(MYQL_ERR_TIMEOUT, "mma probe: the MMA completion wait ran out");
  return MYQL_OK;
}
