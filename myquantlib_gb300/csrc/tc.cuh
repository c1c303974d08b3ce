// tc.cuh -- Blackwell (sm_103a) tensor-core primitives in inline PTX: TMEM
// allocation and loads, tcgen05.mma (kind::f16, BF16 in, FP32 accumulate),
// tcgen05.commit to an mbarrier, bounded mbarrier waits, and the bulk async
// copy engine (cp.async.bulk / cp.async.bulk.tensor with complete_tx).
//
// Operand images in shared memory (K-major, the canonical tcgen05 layouts):
//   IMG128: a [rows][K] BF16 matrix with K a multiple of 64, stored as
//           K/64 blocks of [rows][128 bytes] with the 128-byte swizzle (the
//           16-byte chunk c of row r sits at chunk c ^ (r % 8)); every block
//           starts on a 1024-byte boundary.  Descriptor: SWIZZLE_128B,
//           stride between 8-row groups 1024 B; the k-th 16-element slice of
//           a block starts 32 k bytes into it.
//   IMG16:  a [rows][16] BF16 matrix without swizzle: 8 x 16-byte core
//           matrices, [rows/8][2][8][16 B]; the two K halves of a row group
//           are 128 B apart (leading offset), row groups 256 B apart (stride).
// Every wait in this file is bounded; a wait that runs out returns false and
// the caller records an error status and leaves.
#pragma once
#include <cuda_bf16.h>
#include <cstdint>

#include "device_numerics.cuh"

namespace myql {
namespace tc {

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// ---- operand images -------------------------------------------------------
__host__ __device__ __forceinline__ uint32_t img128_offset(uint32_t r, uint32_t k, uint32_t rows) {
  const uint32_t blk = k >> 6, c = (k >> 3) & 7, e = k & 7;
  return blk * rows * 128u + r * 128u + ((c ^ (r & 7u)) << 4) + (e << 1);
}
__host__ __device__ __forceinline__ uint32_t img16_offset(uint32_t r, uint32_t k) {
  return (r >> 3) * 256u + (k >> 3) * 128u + (r & 7u) * 16u + (k & 7u) * 2u;
}

// ---- descriptors ----------------------------------------------------------
__device__ __forceinline__ uint64_t desc_sw128(uint32_t saddr) {
  uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)1u << 16;               // leading offset (unused by swizzled K-major)
  d |= (uint64_t)(1024u >> 4) << 32;     // stride offset: 8 rows x 128 B
  d |= (uint64_t)1u << 46;               // descriptor version for tcgen05
  d |= (uint64_t)2u << 61;               // SWIZZLE_128B
  return d;
}
__device__ __forceinline__ uint64_t desc_img16(uint32_t saddr) {
  uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)(128u >> 4) << 16;      // leading offset: next 8 K-elements
  d |= (uint64_t)(256u >> 4) << 32;      // stride offset: next 8 rows
  d |= (uint64_t)1u << 46;
  return d;                              // no swizzle
}
// SWIZZLE_128B operand stored MN-major (the IMG128 image of the transposed
// matrix): lines of 64 MN-elements, 8 K-rows per swizzle atom.  Leading offset
// = byte stride between 64-element MN blocks, stride offset = byte stride
// between 8-row K groups (1024 B); a 16-row K step advances the start by 2 KB.
__device__ __forceinline__ uint64_t desc_sw128_mn(uint32_t saddr, uint32_t mn_block_stride) {
  uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((mn_block_stride >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)(1024u >> 4) << 32;
  d |= (uint64_t)1u << 46;
  d |= (uint64_t)2u << 61;
  return d;
}
// kind::f16 instruction descriptor: D FP32, A and B BF16, both K-major.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}
// the same with A and/or B MN-major (transpose bits 15 and 16)
__host__ __device__ constexpr uint32_t idesc_bf16_mn(int M, int N, bool a_mn, bool b_mn) {
  return idesc_bf16(M, N) | (a_mn ? (1u << 15) : 0u) | (b_mn ? (1u << 16) : 0u);
}

// ---- tcgen05 ----------------------------------------------------------------
__device__ __forceinline__ void tmem_alloc(uint32_t *dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
               :: "r"(smem_u32(dst)), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// generic-proxy shared-memory writes -> visible to the async proxy (MMA, bulk copies)
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n"
      :: "r"(d_tmem), "l"(a), "l"(b), "r"(idesc), "r"(accumulate) : "memory");
}
// arrives on the mbarrier once every MMA this thread issued before has completed
__device__ __forceinline__ void mma_commit(uint64_t *mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
               :: "r"(smem_u32(mbar)) : "memory");
}
// 32 consecutive FP32 columns of this thread's TMEM lane (warp w reads lanes 32 (w % 4) ..)
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31]) : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// 64 consecutive columns of this warp's 32 lanes, with the wait in the same
// statement (the registers are defined when it completes)
__device__ __forceinline__ void tmem_ld64(uint32_t taddr, float (&v)[64]) {
  uint32_t r[64];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x64.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31, %32, %33, %34, %35, %36, %37, %38, %39, %40, %41, %42, %43, %44, %45, %46, %47, %48, %49, %50, %51, %52, %53, %54, %55, %56, %57, %58, %59, %60, %61, %62, %63}, [%64];\n\t"
               "tcgen05.wait::ld.sync.aligned;"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31]), "=r"(r[32]), "=r"(r[33]), "=r"(r[34]), "=r"(r[35]), "=r"(r[36]), "=r"(r[37]), "=r"(r[38]), "=r"(r[39]), "=r"(r[40]), "=r"(r[41]), "=r"(r[42]), "=r"(r[43]), "=r"(r[44]), "=r"(r[45]), "=r"(r[46]), "=r"(r[47]), "=r"(r[48]), "=r"(r[49]), "=r"(r[50]), "=r"(r[51]), "=r"(r[52]), "=r"(r[53]), "=r"(r[54]), "=r"(r[55]), "=r"(r[56]), "=r"(r[57]), "=r"(r[58]), "=r"(r[59]), "=r"(r[60]), "=r"(r[61]), "=r"(r[62]), "=r"(r[63])
               : "r"(taddr)
               : "memory");
#pragma unroll
  for (int i = 0; i < 64; ++i) v[i] = __uint_as_float(r[i]);
}

// ---- mbarriers and bulk copies ----------------------------------------------
__device__ __forceinline__ void mbar_init(uint64_t *b, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_u32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *b, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok) : "r"(smem_u32(b)), "r"(parity) : "memory");
  return ok != 0;
}
// Bounded wait for the phase with the given parity to complete: gives up after
// `max_ns` nanoseconds of %globaltimer and returns false.
__device__ __forceinline__ bool mbar_wait(uint64_t *b, uint32_t parity, uint64_t max_ns) {
  if (mbar_try_wait(b, parity)) return true;
  uint64_t t0;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
  for (uint32_t it = 0; it < (1u << 26); ++it) {
    if (mbar_try_wait(b, parity)) return true;
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    if (t - t0 > max_ns) return false;
  }
  return false;
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *b, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(smem_u32(b)), "r"(bytes)
               : "memory");
}
// bulk copy global -> shared (16-byte aligned addresses, size a multiple of 16)
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *b) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
               :: "r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(b)) : "memory");
}

// Packed FP32 pairs: the engine's helpers (device_numerics.cuh)
using dev::pk::ffma2;

// SiLU through tanh.approx: x * sigmoid(x) = 0.5 x (1 + tanh(x / 2)).
__device__ __forceinline__ float tanh_fast(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float silu(float z) {
  const float h = 0.5f * z;
  return fmaf(h, tanh_fast(h), h);
}
// silu(z + b) of two columns from hb = 0.5 b: h = fma(z, 0.5, hb) is exactly 0.5 (z + b)
// (scaling by 2^-1 commutes with rounding), so each lane equals silu(z + b) bit for bit
__device__ __forceinline__ float2 silu2_half_bias(float2 z, float2 hb) {
  const float2 h = ffma2(z, make_float2(0.5f, 0.5f), hb);
  return ffma2(h, make_float2(tanh_fast(h.x), tanh_fast(h.y)), h);
}
// d silu / dz = s (1 + z (1 - s)), s = sigmoid(z) = 0.5 (1 + tanh(z / 2))
__device__ __forceinline__ float silu_grad(float z) {
  const float s = fmaf(0.5f, tanh_fast(0.5f * z), 0.5f);
  return s * fmaf(z, 1.0f - s, 1.0f);
}

}  // namespace tc
}  // namespace myql
