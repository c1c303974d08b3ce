// cv_mlp.cu -- the control variate's MLP on the tcgen05 tensor cores.
//
// cv_mlp_kernel (forward, persistent, one block per SM): weights stay in shared
// memory; four groups of four warps each run their own 128-row tiles.  Per
// tile three MMA chains (K = 16, 128, 128) accumulate FP32 in the group's TMEM
// columns, and the group's warps turn each accumulator row into SiLU
// activations (BF16, written back as the next layer's A operand) while the
// other groups' MMAs run.  Feature tiles stream in by bulk copy behind the
// first layer.  The output layer is a per-row FP32 dot product, multiplied by
// the row's martingale increment and summed per path over the hedge times.
//
// cv_bwd_kernel (training): per tile, the forward pass again (keeping h1, h2
// in shared memory), then back-propagation of dL/dg = coef_path * dM_row:
//   dz3 = dg * w4 * silu'(z3)
//   dh2 = dz3 W3        (W3's image read MN-major)      dW3 += dz3^T h2 (MN-major operands)
//   dz2 = dh2 * silu'(z2)  (z2 recomputed into spare TMEM)
//   dh1 = dz2 W2                                        dW2 += dz2^T h1
//   dz1 = dh1 * silu'(z1)  (z1 recomputed)              dW1 += dz1^T x
// dW2, dW3 accumulate in TMEM over the block's tiles, dW1 in registers, the
// bias and output-layer gradients through warp reductions.  Each block writes
// its gradient to its own slice of a partial buffer, and cv_grad_reduce_kernel
// sums the slices in block order, so the gradient is deterministic.
//
// Every mbarrier wait is bounded; a wait that runs out sets status[2], makes
// the whole block leave its tile loop, waits (bounded) for its own bulk
// copies in flight and frees its TMEM.
#include <algorithm>
#include <atomic>

#include "cv.cuh"

namespace myql {
namespace dev {

__device__ __forceinline__ uint8_t *align1024(uint8_t *p) {
  const uint32_t a = tc::smem_u32(p);
  return p + (((a + 1023u) & ~1023u) - a);
}

// z (TMEM, columns [32 c0, 32 c1) of this thread's row) + bias -> SiLU -> BF16 IMG128 row of H.
// hb = 0.5 x the layer's bias (16-byte aligned, shared): the bias, the halving and SiLU's
// final fma run on column pairs (packed FP32), with the values of the scalar form.
__device__ __forceinline__ void epi_hidden(uint32_t tm_row, const float *hb, uint8_t *H, uint32_t row, int c0 = 0,
                                           int c1 = 4) {
#pragma unroll 1
  for (int c = c0; c < c1; c += 2) {
    float v[64];
    tc::tmem_ld64(tm_row + (uint32_t)(c * 32), v);  // columns [32 c, 32 c + 64): one round trip
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const float4 b0 = *reinterpret_cast<const float4 *>(hb + c * 32 + q * 8);
      const float4 b1 = *reinterpret_cast<const float4 *>(hb + c * 32 + q * 8 + 4);
      const float2 bp[4] = {make_float2(b0.x, b0.y), make_float2(b0.z, b0.w), make_float2(b1.x, b1.y),
                            make_float2(b1.z, b1.w)};
      uint32_t w[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const float2 s = tc::silu2_half_bias(make_float2(v[q * 8 + 2 * e], v[q * 8 + 2 * e + 1]), bp[e]);
        __nv_bfloat162 p = __floats2bfloat162_rn(s.x, s.y);
        w[e] = *reinterpret_cast<uint32_t *>(&p);
      }
      *reinterpret_cast<uint4 *>(H + tc::img128_offset(row, (uint32_t)(c * 32 + q * 8), 128)) =
          make_uint4(w[0], w[1], w[2], w[3]);
    }
  }
}

// output layer over columns [32 c0, 32 c1): sum_k silu(z3_k + b3_k) w4_k (+ b4 when c0 == 0),
// from hb3 = 0.5 b3, on column pairs with four partial sums (a fixed order: deterministic)
__device__ __forceinline__ float epi_out(uint32_t tm_row, const float *vec, const float *hb3, int c0 = 0,
                                         int c1 = 4) {
  float2 ga = make_float2(c0 == 0 ? vec[kVecB4] : 0.0f, 0.0f), gb = make_float2(0.0f, 0.0f);
#pragma unroll 1
  for (int c = c0; c < c1; c += 2) {
    float v[64];
    tc::tmem_ld64(tm_row + (uint32_t)(c * 32), v);
#pragma unroll
    for (int i = 0; i < 64; i += 4) {
      const int k = c * 32 + i;
      const float4 h4 = *reinterpret_cast<const float4 *>(hb3 + k);
      const float4 w4 = *reinterpret_cast<const float4 *>(vec + kVecW4 + k);
      const float2 s0 = tc::silu2_half_bias(make_float2(v[i], v[i + 1]), make_float2(h4.x, h4.y));
      const float2 s1 = tc::silu2_half_bias(make_float2(v[i + 2], v[i + 3]), make_float2(h4.z, h4.w));
      ga = tc::ffma2(s0, make_float2(w4.x, w4.y), ga);
      gb = tc::ffma2(s1, make_float2(w4.z, w4.w), gb);
    }
  }
  return (ga.x + ga.y) + (gb.x + gb.y);
}

// D[128 x N] (TMEM) = A (IMG128, [128][K]) * B (IMG128, [N][K])^T, K = 128, both K-major
__device__ __forceinline__ void mma_k128(uint32_t d, const uint8_t *A, const uint8_t *B, int N, uint32_t acc0) {
  const uint32_t a = tc::smem_u32(A), b = tc::smem_u32(B);
#pragma unroll
  for (int kk = 0; kk < 8; ++kk) {
    const uint32_t ao = (uint32_t)(kk >> 2) * 16384u + (uint32_t)(kk & 3) * 32u;
    const uint32_t bo = (uint32_t)(kk >> 2) * (uint32_t)N * 128u + (uint32_t)(kk & 3) * 32u;
    tc::mma_bf16(d, tc::desc_sw128(a + ao), tc::desc_sw128(b + bo), tc::idesc_bf16(128, N),
                 (kk > 0 || acc0) ? 1u : 0u);
  }
}

// D[128 x N] = A^T B over K = 128 rows where A ([128 rows][128]) and B ([128 rows][N])
// are natural IMG128 row images read MN-major (lines along M / N, 8-row K groups)
__device__ __forceinline__ void mma_tn_rows(uint32_t d, const uint8_t *A, const uint8_t *B, int N, uint32_t acc0) {
  const uint32_t a = tc::smem_u32(A), b = tc::smem_u32(B);
#pragma unroll
  for (int kk = 0; kk < 8; ++kk) {
    const uint32_t o = (uint32_t)kk * 2048u;
    tc::mma_bf16(d, tc::desc_sw128_mn(a + o, 16384u), tc::desc_sw128_mn(b + o, 16384u),
                 tc::idesc_bf16_mn(128, N, true, true), (kk > 0 || acc0) ? 1u : 0u);
  }
}

// D[128 rows x N] = A (IMG128 [128 rows][K], K-major) * W where W's IMG128 image
// [K rows][N] is read MN-major: the back-propagation product dz * W.
__device__ __forceinline__ void mma_nn(uint32_t d, const uint8_t *A, const uint8_t *W, int N) {
  const uint32_t a = tc::smem_u32(A), b = tc::smem_u32(W);
#pragma unroll
  for (int kk = 0; kk < 8; ++kk) {
    const uint32_t ao = (uint32_t)(kk >> 2) * 16384u + (uint32_t)(kk & 3) * 32u;
    tc::mma_bf16(d, tc::desc_sw128(a + ao), tc::desc_sw128_mn(b + (uint32_t)kk * 2048u, 16384u),
                 tc::idesc_bf16_mn(128, N, false, true), kk > 0 ? 1u : 0u);
  }
}

// all threads: bounded wait on a commit barrier, then agree on the outcome
__device__ __forceinline__ bool block_wait(uint64_t *bar, uint32_t &phase) {
  const bool ok = tc::mbar_wait(bar, phase & 1u, kCvWaitNs);
  ++phase;
  const int bad = __syncthreads_or(!ok);
  tc::fence_after_sync();
  return bad == 0;
}
__device__ __forceinline__ void block_sync_async() {
  tc::fence_proxy_async();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
}

// ------------------------------------------------------------------ forward
// One block per SM: 16 warps in 4 groups of 4.  Group g owns a tile slot:
// TMEM columns [128 g, 128 g + 128), an activation image H[g] and a feature
// buffer X[g].  Its warps cover the 128 TMEM lanes (warp w reads lanes
// 32 (w % 4) ..), so each thread owns one row of the tile and all 128 columns.
// A group runs its tiles on its own: its elected thread issues the MMAs, the
// group waits on its own commit barrier and synchronises with a named barrier
// of 128 threads, so four tiles are in flight per SM and one group's MMAs run
// under the others' epilogues.  The weights are loaded once per block.
constexpr int kFwdGroups = 4;
constexpr int kFwdThreads = 128 * kFwdGroups;
constexpr uint32_t kFwdH = kImgFwdBytes;                       // H[g] at kFwdH + g * 32 KB
constexpr uint32_t kFwdX = kFwdH + kFwdGroups * 32768u;         // X[g] at kFwdX + g * 4 KB
constexpr uint32_t kFwdSmemBytes = kFwdX + kFwdGroups * kCvTileBytes;

__device__ __forceinline__ void group_sync(int id) {
  asm volatile("bar.sync %0, 128;" ::"r"(id) : "memory");
}
// named barrier of one group that also ORs a predicate over its 128 threads
__device__ __forceinline__ bool group_sync_or(int id, bool pred) {
  uint32_t r;
  asm volatile("{\n\t.reg .pred p, q;\n\tsetp.ne.u32 p, %1, 0;\n\tbar.red.or.pred q, %2, 128, p;\n\t"
               "selp.u32 %0, 1, 0, q;\n\t}"
               : "=r"(r)
               : "r"((uint32_t)pred), "r"(id)
               : "memory");
  return r != 0;
}

__global__ void __launch_bounds__(kFwdThreads, 1) cv_mlp_kernel(const __grid_constant__ CvMlpParams P) {
  extern __shared__ uint8_t dyn[];
  __shared__ __align__(8) uint64_t bar_w, bar_x[kFwdGroups], bar_mma[kFwdGroups];
  __shared__ uint32_t tmem_base;
  __shared__ __align__(16) float vec[kVecCount];
  __shared__ __align__(16) float hbias[kHalfBias];
  uint8_t *sm = align1024(dyn);
  uint8_t *sW1 = sm + kImgW1, *sW2 = sm + kImgW2, *sW3 = sm + kImgW3;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int grp = warp >> 2, gtid = tid & 127;
  const bool elected = gtid == 0;
  const int bar_id = 1 + grp;  // named barrier of the group (0 is __syncthreads)
  const uint32_t row = (uint32_t)gtid;  // = 32 (warp % 4) + lane
  uint8_t *sH = sm + kFwdH + (uint32_t)grp * 32768u;
  uint8_t *sX = sm + kFwdX + (uint32_t)grp * kCvTileBytes;
  for (int i = tid; i < kVecCount; i += kFwdThreads) vec[i] = P.vec[i];
  for (int i = tid; i < kHalfBias; i += kFwdThreads) hbias[i] = 0.5f * P.vec[kVecB1 + i];
  if (tid == 0) {
    tc::mbar_init(&bar_w, 1);
    for (int g = 0; g < kFwdGroups; ++g) {
      tc::mbar_init(&bar_x[g], 1);
      tc::mbar_init(&bar_mma[g], 1);
    }
    tc::fence_mbar_init();
  }
  if (warp == 0) {
    tc::tmem_alloc(&tmem_base, 128 * kFwdGroups);
    tc::tmem_relinquish();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tm = tmem_base + (uint32_t)(grp * 128);
  const uint32_t tm_row = tm + ((uint32_t)((warp & 3) * 32) << 16);
  // path-major: whole path blocks per group (per-path sums in registers);
  // tile-major: tiles round robin over all groups (per-row products to P.gdm)
  const unsigned long long G = (unsigned long long)blockIdx.x * kFwdGroups + grp;
  const unsigned long long NG = (unsigned long long)gridDim.x * kFwdGroups;
  const unsigned long long n_tiles = (unsigned long long)P.n_pb * P.n_hedge;
  unsigned long long total;
  if (P.tile_major) {
    total = n_tiles > G ? (n_tiles - 1 - G) / NG + 1 : 0;
  } else {
    const unsigned long long n_mine = P.n_pb > G ? (P.n_pb - 1 - G) / NG + 1 : 0;
    total = n_mine * P.n_hedge;
  }
  auto tile_of = [&](unsigned long long t) {
    if (P.tile_major) return G + t * NG;
    return (G + (t / P.n_hedge) * NG) * P.n_hedge + t % P.n_hedge;
  };
  bool x_pending = false;  // elected thread: a feature copy in flight on bar_x[grp]
  uint32_t xphase = 0, mphase = 0;
  if (tid == 0) {
    tc::mbar_arrive_expect_tx(&bar_w, kImgFwdBytes);
    tc::bulk_g2s(sm, P.img, kImgFwdBytes, &bar_w);
  }
  if (elected && total > 0) {
    tc::mbar_arrive_expect_tx(&bar_x[grp], kCvTileBytes);
    tc::bulk_g2s(sX, P.feat + tile_of(0) * kCvTileBytes, kCvTileBytes, &bar_x[grp]);
    x_pending = true;
  }
  bool ok = tc::mbar_wait(&bar_w, 0, kCvWaitNs);
  bool err = __syncthreads_or(!ok) != 0;
  float acc = 0.0f;
  auto mma_wait = [&]() {
    const bool w = tc::mbar_wait(&bar_mma[grp], mphase & 1u, kCvWaitNs);
    ++mphase;
    const bool bad = group_sync_or(bar_id, !w);
    tc::fence_after_sync();
    return !bad;
  };
  auto before_mma = [&]() {  // the group's H writes and TMEM reads done before the next MMA
    tc::fence_proxy_async();
    tc::fence_before_sync();
    group_sync(bar_id);
    tc::fence_after_sync();
  };
  for (unsigned long long t = 0; t < total && !err; ++t) {
    const unsigned long long tile = tile_of(t);
    const unsigned int j = (unsigned int)(tile % P.n_hedge);
    // layer 1: features landed, and the group's last tile left TMEM (its loads done)
    ok = true;
    if (elected) {
      ok = tc::mbar_wait(&bar_x[grp], xphase & 1u, kCvWaitNs);
      ++xphase;
      x_pending = !ok;
    }
    tc::fence_before_sync();
    if (group_sync_or(bar_id, !ok)) { err = true; break; }
    tc::fence_after_sync();
    if (elected) {
      tc::mma_bf16(tm, tc::desc_img16(tc::smem_u32(sX)), tc::desc_img16(tc::smem_u32(sW1)),
                   tc::idesc_bf16(128, 128), 0u);
      tc::mma_commit(&bar_mma[grp]);
    }
    if (!mma_wait()) { err = true; break; }
    // X is free: the group's next features stream in under layers 2 and 3
    if (elected && t + 1 < total) {
      tc::mbar_arrive_expect_tx(&bar_x[grp], kCvTileBytes);
      tc::bulk_g2s(sX, P.feat + tile_of(t + 1) * kCvTileBytes, kCvTileBytes, &bar_x[grp]);
      x_pending = true;
    }
    epi_hidden(tm_row, hbias, sH, row);
    before_mma();
    if (elected) {
      mma_k128(tm, sH, sW2, 128, 0u);
      tc::mma_commit(&bar_mma[grp]);
    }
    if (!mma_wait()) { err = true; break; }
    epi_hidden(tm_row, hbias + 128, sH, row);
    before_mma();
    if (elected) {
      mma_k128(tm, sH, sW3, 128, 0u);
      tc::mma_commit(&bar_mma[grp]);
    }
    if (!mma_wait()) { err = true; break; }
    const float g = epi_out(tm_row, vec, hbias + 256);
    const unsigned long long r = tile * 128ull + row;
    if (P.g_out) P.g_out[r] = g;
    if (P.tile_major) {
      P.gdm[r] = g * P.dM[r];
    } else {
      acc = fmaf(g, P.dM[r], acc);
      if (j == P.n_hedge - 1) {
        const unsigned long long path = (tile / P.n_hedge) * 128ull + row;
        if (path < P.n_paths) P.cv[path] = acc;
        acc = 0.0f;
      }
    }
  }
  if (err && elected) {
    atomicAdd(P.status + 2, 1u);
    if (x_pending) tc::mbar_wait(&bar_x[grp], xphase & 1u, kCvWaitNs);
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (warp == 0) tc::tmem_dealloc(tmem_base, 128 * kFwdGroups);
}

// ------------------------------------------------------------------ backward
// Column sums over a warp's 32 rows of a per-row 32-vector by transposed
// halving: 31 shuffles; afterwards lane l holds the sum of column l.
__device__ __forceinline__ float warp_colsum32(float (&v)[32], int lane) {
#pragma unroll
  for (int off = 16; off >= 1; off >>= 1) {
    const bool upper = (lane & off) != 0;
#pragma unroll
    for (int i = 0; i < off; ++i) {
      const float send = upper ? v[i] : v[i + off];
      const float keep = upper ? v[i + off] : v[i];
      v[i] = keep + __shfl_xor_sync(0xffffffffu, send, off);
    }
  }
  return v[0];
}

__device__ __forceinline__ void store_bf16_chunk(uint8_t *img, uint32_t row, int k0, const float *x) {
  uint32_t w[4];
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    __nv_bfloat162 p = __floats2bfloat162_rn(x[2 * e], x[2 * e + 1]);
    w[e] = *reinterpret_cast<uint32_t *>(&p);
  }
  *reinterpret_cast<uint4 *>(img + tc::img128_offset(row, (uint32_t)k0, 128)) = make_uint4(w[0], w[1], w[2], w[3]);
}

// 8 warps: warp w serves rows 32 (w % 4) .. (its TMEM lane quarter) and the
// column half w / 4 of every 128-wide layer.
constexpr int kBwdThreads = 256;

__global__ void __launch_bounds__(kBwdThreads, 1) cv_bwd_kernel(const __grid_constant__ CvMlpParams P) {
  extern __shared__ uint8_t dyn[];
  __shared__ __align__(8) uint64_t bar_w, bar_mma;
  __shared__ uint32_t tmem_base;
  __shared__ __align__(16) float vec[kVecCount];
  __shared__ __align__(16) float hbias[kHalfBias];
  uint8_t *sm = align1024(dyn);
  // [W1x64 16K][W2 32K][W3 32K][X64 16K][H1 32K][H2 32K][D 32K]
  uint8_t *sW1 = sm, *sW2 = sm + 16384, *sW3 = sm + 49152, *sX = sm + 81920, *sH1 = sm + 98304;
  uint8_t *sH2 = sm + 131072, *sD = sm + 163840;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t row = (uint32_t)(tid & 127);
  const int half = warp >> 2, c0 = 2 * half, c1 = 2 * half + 2;
  for (int i = tid; i < kVecCount; i += kBwdThreads) vec[i] = P.vec[i];
  for (int i = tid; i < kHalfBias; i += kBwdThreads) hbias[i] = 0.5f * P.vec[kVecB1 + i];
  // padding chunks of the x image stay zero
  for (int i = tid; i < 128 * 6; i += kBwdThreads)
    *reinterpret_cast<uint4 *>(sX + tc::img128_offset((uint32_t)(i / 6), (uint32_t)((2 + i % 6) * 8), 128)) =
        make_uint4(0, 0, 0, 0);
  if (tid == 0) {
    tc::mbar_init(&bar_w, 1);
    tc::mbar_init(&bar_mma, 1);
    tc::fence_mbar_init();
  }
  if (warp == 0) {
    tc::tmem_alloc(&tmem_base, 512);
    tc::tmem_relinquish();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tm = tmem_base;
  const uint32_t lane_off = (uint32_t)((warp & 3) * 32) << 16;
  const uint32_t T0 = tm, T1 = tm + 128, TW3 = tm + 256, TW2 = tm + 384;
  if (tid == 0) {
    tc::mbar_arrive_expect_tx(&bar_w, 16384u + 65536u);
    tc::bulk_g2s(sW1, P.img + kImgW1x64, 16384u, &bar_w);
    tc::bulk_g2s(sW2, P.img + kImgW2, 65536u, &bar_w);  // W2 and W3 are adjacent
  }
  bool ok = true;
  if (tid == 0) ok = tc::mbar_wait(&bar_w, 0, kCvWaitNs);
  bool err = __syncthreads_or(!ok) != 0;
  // tiles round robin over the blocks
  const unsigned long long n_tiles = (unsigned long long)P.n_pb * P.n_hedge;
  const unsigned long long total = n_tiles > blockIdx.x ? (n_tiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
  uint32_t phase = 0;
  float dw1[kCvIn];
#pragma unroll
  for (int i = 0; i < kCvIn; ++i) dw1[i] = 0.0f;
  // column sums, column = 64 half + 32 (c - c0) + lane, over this warp's row quarter
  float gb1[2] = {0.0f, 0.0f}, gb2[2] = {0.0f, 0.0f}, gb3[2] = {0.0f, 0.0f}, gw4[2] = {0.0f, 0.0f};
  float gb4 = 0.0f;
  for (unsigned long long t = 0; t < total && !err; ++t) {
    const unsigned long long tile = (unsigned long long)blockIdx.x + t * gridDim.x;
    const unsigned long long pb = tile / P.n_hedge;
    const unsigned long long path = pb * 128ull + row;
    const float dg = path < P.n_paths ? P.coef[path] * P.dM[tile * 128ull + row] : 0.0f;
    if (half == 0) {  // x row -> X64 image (features 0..15; 16..63 stay zero)
      const uint8_t *ft = P.feat + tile * kCvTileBytes;
      *reinterpret_cast<uint4 *>(sX + tc::img128_offset(row, 0, 128)) =
          *reinterpret_cast<const uint4 *>(ft + tc::img16_offset(row, 0));
      *reinterpret_cast<uint4 *>(sX + tc::img128_offset(row, 8, 128)) =
          *reinterpret_cast<const uint4 *>(ft + tc::img16_offset(row, 8));
      gb4 += dg;
    }
    block_sync_async();
    // F1: z1 = x W1^T (K = 64)
    if (tid == 0) {
      const uint32_t a = tc::smem_u32(sX), b = tc::smem_u32(sW1);
      for (int kk = 0; kk < 4; ++kk)
        tc::mma_bf16(T0, tc::desc_sw128(a + (uint32_t)kk * 32u), tc::desc_sw128(b + (uint32_t)kk * 32u),
                     tc::idesc_bf16(128, 128), kk > 0 ? 1u : 0u);
      tc::mma_commit(&bar_mma);
    }
    if (!block_wait(&bar_mma, phase)) { err = true; break; }
    epi_hidden(T0 + lane_off, hbias, sH1, row, c0, c1);
    block_sync_async();
    // F2: z2 = h1 W2^T
    if (tid == 0) {
      mma_k128(T0, sH1, sW2, 128, 0u);
      tc::mma_commit(&bar_mma);
    }
    if (!block_wait(&bar_mma, phase)) { err = true; break; }
    epi_hidden(T0 + lane_off, hbias + 128, sH2, row, c0, c1);
    block_sync_async();
    // F3: z3 = h2 W3^T
    if (tid == 0) {
      mma_k128(T0, sH2, sW3, 128, 0u);
      tc::mma_commit(&bar_mma);
    }
    if (!block_wait(&bar_mma, phase)) { err = true; break; }
    // e3: dz3 = dg w4 silu'(z3 + b3) -> D; column sums for b3 and w4
#pragma unroll 1
    for (int c = c0; c < c1; ++c) {
      float v[32], dz[32], hw[32];
      tc::tmem_ld32(T0 + lane_off + (uint32_t)(c * 32), v);
#pragma unroll
      for (int i = 0; i < 32; ++i) {
        const int k = c * 32 + i;
        const float z = v[i] + vec[kVecB3 + k];
        dz[i] = dg * vec[kVecW4 + k] * tc::silu_grad(z);
        hw[i] = dg * tc::silu(z);
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) store_bf16_chunk(sD, row, c * 32 + q * 8, dz + q * 8);
      gb3[c - c0] += warp_colsum32(dz, lane);
      gw4[c - c0] += warp_colsum32(hw, lane);
    }
    block_sync_async();
    // B3: dh2 = dz3 W3 -> T0; dW3 += dz3^T h2 -> TW3; z2 again -> T1
    if (tid == 0) {
      mma_nn(T0, sD, sW3, 128);
      mma_tn_rows(TW3, sD, sH2, 128, t > 0 ? 1u : 0u);
      mma_k128(T1, sH1, sW2, 128, 0u);
      tc::mma_commit(&bar_mma);
    }
    if (!block_wait(&bar_mma, phase)) { err = true; break; }
#pragma unroll 1
    for (int c = c0; c < c1; ++c) {
      float dh[32], z[32], dz[32];
      tc::tmem_ld32(T0 + lane_off + (uint32_t)(c * 32), dh);
      tc::tmem_ld32(T1 + lane_off + (uint32_t)(c * 32), z);
#pragma unroll
      for (int i = 0; i < 32; ++i) dz[i] = dh[i] * tc::silu_grad(z[i] + vec[kVecB2 + c * 32 + i]);
#pragma unroll
      for (int q = 0; q < 4; ++q) store_bf16_chunk(sD, row, c * 32 + q * 8, dz + q * 8);
      gb2[c - c0] += warp_colsum32(dz, lane);
    }
    block_sync_async();
    // B2: dh1 = dz2 W2 -> T0; dW2 += dz2^T h1 -> TW2; z1 again -> T1
    if (tid == 0) {
      mma_nn(T0, sD, sW2, 128);
      mma_tn_rows(TW2, sD, sH1, 128, t > 0 ? 1u : 0u);
      const uint32_t a = tc::smem_u32(sX), b = tc::smem_u32(sW1);
      for (int kk = 0; kk < 4; ++kk)
        tc::mma_bf16(T1, tc::desc_sw128(a + (uint32_t)kk * 32u), tc::desc_sw128(b + (uint32_t)kk * 32u),
                     tc::idesc_bf16(128, 128), kk > 0 ? 1u : 0u);
      tc::mma_commit(&bar_mma);
    }
    if (!block_wait(&bar_mma, phase)) { err = true; break; }
#pragma unroll 1
    for (int c = c0; c < c1; ++c) {
      float dh[32], z[32], dz[32];
      tc::tmem_ld32(T0 + lane_off + (uint32_t)(c * 32), dh);
      tc::tmem_ld32(T1 + lane_off + (uint32_t)(c * 32), z);
#pragma unroll
      for (int i = 0; i < 32; ++i) dz[i] = dh[i] * tc::silu_grad(z[i] + vec[kVecB1 + c * 32 + i]);
#pragma unroll
      for (int q = 0; q < 4; ++q) store_bf16_chunk(sD, row, c * 32 + q * 8, dz + q * 8);
      gb1[c - c0] += warp_colsum32(dz, lane);
    }
    block_sync_async();
    // B1: dW1 (tile) = dz1^T x -> T0 columns 0..63 (only the 16 input slots are kept)
    if (tid == 0) {
      mma_tn_rows(T0, sD, sX, 64, 0u);
      tc::mma_commit(&bar_mma);
    }
    if (!block_wait(&bar_mma, phase)) { err = true; break; }
    if (half == 0) {
      float v[32];
      tc::tmem_ld32(T0 + lane_off, v);
#pragma unroll
      for (int i = 0; i < kCvIn; ++i) dw1[i] += v[i];
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
  }
  // flush: this block's gradient to its own slice of P.gpart (plain vector stores;
  // cv_grad_reduce_kernel sums the slices in a fixed order).  Thread (quarter, half)
  // owns output row o = row of dW2, dW3 (TMEM lane o), the columns of its half.
  const bool flush = !err && total > 0;
  float *gp = P.gpart + (size_t)blockIdx.x * kPCount;
  if (flush) {
    for (int c = c0; c < c1; ++c) {
      float v[32];
      tc::tmem_ld32(TW3 + lane_off + (uint32_t)(c * 32), v);
#pragma unroll
      for (int q = 0; q < 8; ++q)
        *reinterpret_cast<float4 *>(gp + kPW3 + row * 128 + c * 32 + 4 * q) =
            make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
      tc::tmem_ld32(TW2 + lane_off + (uint32_t)(c * 32), v);
#pragma unroll
      for (int q = 0; q < 8; ++q)
        *reinterpret_cast<float4 *>(gp + kPW2 + row * 128 + c * 32 + 4 * q) =
            make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
    }
    if (half == 0) {
#pragma unroll
      for (int q = 0; q < kCvIn / 4; ++q)
        *reinterpret_cast<float4 *>(gp + kPW1 + row * kCvIn + 4 * q) =
            make_float4(dw1[4 * q], dw1[4 * q + 1], dw1[4 * q + 2], dw1[4 * q + 3]);
    }
  }
  // bias and output-layer sums: the four row quarters meet in the (idle) D buffer
  float *red = reinterpret_cast<float *>(sD);  // [quarter][b1, b2, b3, w4][128], then b4[quarter]
  const int qt = warp & 3;
  if (flush) {
    for (int c = c0; c < c1; ++c) {
      const int col = c * 32 + lane;
      red[(qt * 4 + 0) * 128 + col] = gb1[c - c0];
      red[(qt * 4 + 1) * 128 + col] = gb2[c - c0];
      red[(qt * 4 + 2) * 128 + col] = gb3[c - c0];
      red[(qt * 4 + 3) * 128 + col] = gw4[c - c0];
    }
    float s = gb4;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0 && half == 0) red[2048 + qt] = s;
  }
  __syncthreads();
  if (flush) {
    const int dst[4] = {kPB1, kPB2, kPB3, kPW4};
    for (int i = tid; i < 4 * 128; i += kBwdThreads) {
      const int v = i >> 7, col = i & 127;
      gp[dst[v] + col] = ((red[(0 * 4 + v) * 128 + col] + red[(1 * 4 + v) * 128 + col]) +
                          red[(2 * 4 + v) * 128 + col]) + red[(3 * 4 + v) * 128 + col];
    }
    if (tid < 4) gp[kPB4 + tid] = tid == 0 ? ((red[2048] + red[2049]) + red[2050]) + red[2051] : 0.0f;
  } else {
    for (int i = tid; i < kPCount; i += kBwdThreads) gp[i] = 0.0f;
  }
  if (err && tid == 0) atomicAdd(P.status + 2, 1u);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (warp == 0) tc::tmem_dealloc(tm, 512);
}

// ------------------------------------------------------------------ small kernels
// FP32 parameters -> BF16 images and the FP32 vectors
__global__ void cv_pack_kernel(const float *p, uint8_t *img, float *vec) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < 128 * kCvIn) {  // W1 [o][k]
    const int o = i / kCvIn, k = i % kCvIn;
    const __nv_bfloat16 b = __float2bfloat16_rn(p[kPW1 + i]);
    *reinterpret_cast<__nv_bfloat16 *>(img + kImgW1 + tc::img16_offset(o, k)) = b;
    *reinterpret_cast<__nv_bfloat16 *>(img + kImgW1x64 + tc::img128_offset(o, k, 128)) = b;
  }
  if (i < 128 * 64 && (i % 64) >= kCvIn) {  // W1x64 padding
    const int o = i / 64, k = i % 64;
    *reinterpret_cast<__nv_bfloat16 *>(img + kImgW1x64 + tc::img128_offset(o, k, 128)) = __float2bfloat16_rn(0.0f);
  }
  if (i < 128 * 128) {
    const int o = i / 128, k = i % 128;
    *reinterpret_cast<__nv_bfloat16 *>(img + kImgW2 + tc::img128_offset(o, k, 128)) = __float2bfloat16_rn(p[kPW2 + i]);
    *reinterpret_cast<__nv_bfloat16 *>(img + kImgW3 + tc::img128_offset(o, k, 128)) = __float2bfloat16_rn(p[kPW3 + i]);
  }
  if (i < 128) {
    vec[kVecB1 + i] = p[kPB1 + i];
    vec[kVecB2 + i] = p[kPB2 + i];
    vec[kVecB3 + i] = p[kPB3 + i];
    vec[kVecW4 + i] = p[kPW4 + i];
  }
  if (i == 0) vec[kVecB4] = p[kPB4];
}

// Adam (bias-corrected): b1t = 1 - beta1^t, b2t = 1 - beta2^t
__global__ void cv_adam_kernel(float *p, float *m, float *v, const float *g, float lr, float b1t, float b2t) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kPCount) return;
  const float gi = g[i];
  const float mi = fmaf(0.9f, m[i], 0.1f * gi);
  const float vi = fmaf(0.999f, v[i], 0.001f * gi * gi);
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr * (mi / b1t) / (sqrtf(vi / b2t) + 1e-8f);
}

// r_p = Y_p - C_p - mean(Y - C); coef_p = dL/dC_p = -2 r_p / n; loss = mean r^2.
// Pass 1 sums Y - C into acc[0]; pass 2 writes coef and sums r^2 into acc[1].
// grad[p] = sum over the backward blocks' slices, block 0 first (deterministic)
__global__ void cv_grad_reduce_kernel(const float *gpart, unsigned int nb, float *grad) {
  const unsigned int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= (unsigned int)kPCount) return;
  float s = 0.0f;
  for (unsigned int b = 0; b < nb; ++b) s += gpart[(size_t)b * kPCount + p];
  grad[p] = s;
}

// Deterministic block sum of 256 threads' FP64 values (warp shuffles, then the
// 8 warp sums in order); the result is valid in thread 0.
__device__ __forceinline__ double block_sum256(double v) {
  __shared__ double ws[8];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < 8; ++w) t += ws[w];
  return t;
}

// residuals r = Y - cv - mean(Y - cv): kResidBlocks partial sums of Y - cv, then
// per path the loss gradient coef = -2 r / n and kResidBlocks partial sums of r^2 / n.
// Fixed grid and fixed summation order: the results do not depend on scheduling.
__global__ void __launch_bounds__(256) cv_resid_sum_kernel(const float *Y, const float *cv, unsigned long long n,
                                                           double *part) {
  double s = 0.0;
  for (unsigned long long i = blockIdx.x * 256ull + threadIdx.x; i < n; i += (unsigned long long)gridDim.x * 256ull)
    s += (double)Y[i] - (double)cv[i];
  const double t = block_sum256(s);
  if (threadIdx.x == 0) part[blockIdx.x] = t;
}
__global__ void __launch_bounds__(256) cv_resid_coef_kernel(const float *Y, const float *cv, unsigned long long n,
                                                            const double *part, float *coef, double *loss_part) {
  __shared__ double mu_s;
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (unsigned int b = 0; b < gridDim.x; ++b) t += part[b];
    mu_s = t / (double)n;
  }
  __syncthreads();
  const double mu = mu_s;
  double ss = 0.0;
  for (unsigned long long i = blockIdx.x * 256ull + threadIdx.x; i < n; i += (unsigned long long)gridDim.x * 256ull) {
    const double r = (double)Y[i] - (double)cv[i] - mu;
    ss += r * r;
    coef[i] = (float)(-2.0 * r / (double)n);
  }
  const double t = block_sum256(ss);
  if (threadIdx.x == 0) loss_part[blockIdx.x] = t / (double)n;
}

// cv[p] = sum_j gdm[row (p, j)] in hedge order (tile-major forward)
__global__ void cv_rowsum_kernel(const float *gdm, unsigned long long n, unsigned int n_hedge, float *cv) {
  const unsigned long long p = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
  if (p >= n) return;
  const unsigned long long base = (p >> 7) * n_hedge * 128ull + (p & 127u);
  float s = 0.0f;
  for (unsigned int j = 0; j < n_hedge; ++j) s += gdm[base + (unsigned long long)j * 128ull];
  cv[p] = s;
}

// sums4 += {sum Y, sum Y^2, sum (Y - C), sum (Y - C)^2} and the hedge-ratio sums: per-block
// FP64 partials (fixed grid, warps summed in order), folded into the running sums by
// cv_fold_kernel in a fixed order: deterministic.
__global__ void __launch_bounds__(256) cv_reduce_kernel(const float *Y, const float *cv, unsigned long long n,
                                                        double *part) {
  double a[4] = {0.0, 0.0, 0.0, 0.0};
  for (unsigned long long i = blockIdx.x * 256ull + threadIdx.x; i < n; i += (unsigned long long)gridDim.x * 256ull) {
    const double y = Y[i], z = (double)Y[i] - (double)cv[i];
    a[0] += y;
    a[1] += y * y;
    a[2] += z;
    a[3] += z * z;
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const double t = block_sum256(a[q]);
    if (threadIdx.x == 0) part[blockIdx.x * 4 + q] = t;
  }
}
__global__ void __launch_bounds__(256) cv_beta_kernel(const float *Y, const float *dM, unsigned long long n,
                                                      unsigned int n_hedge, double *part) {
  double a[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  for (unsigned long long p = blockIdx.x * 256ull + threadIdx.x; p < n; p += (unsigned long long)gridDim.x * 256ull) {
    const unsigned long long pb = p >> 7, lane = p & 127u;
    double sp = 0.0;
    for (unsigned int j = 0; j < n_hedge; ++j) sp += (double)dM[(pb * n_hedge + j) * 128ull + lane];
    const double y = Y[p];
    a[0] += sp;
    a[1] += sp * sp;
    a[2] += y * sp;
    a[3] += y;
    a[4] += y * y;
  }
#pragma unroll
  for (int q = 0; q < 5; ++q) {
    const double t = block_sum256(a[q]);
    if (threadIdx.x == 0) part[blockIdx.x * 5 + q] = t;
  }
}
// sums[q] += sum over blocks b of part[b][q]: warp q, lane l sums b = l, l + 32, ...
// in order, then a fixed shuffle tree (deterministic)
__global__ void cv_fold_kernel(const double *part, unsigned int nb, unsigned int nq, double *sums) {
  const unsigned int q = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (q >= nq) return;
  double t = 0.0;
  for (unsigned int b = lane; b < nb; b += 32) t += part[(size_t)b * nq + q];
  for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  if (lane == 0) sums[q] += t;
}

}  // namespace dev

cudaError_t launch_cv_beta(const float *Y, const float *dM, unsigned long long n, unsigned int n_hedge,
                           double *sums5, double *part, cudaStream_t st) {
  dev::cv_beta_kernel<<<kFoldBlocks, 256, 0, st>>>(Y, dM, n, n_hedge, part);
  dev::cv_fold_kernel<<<1, 32 * 5, 0, st>>>(part, kFoldBlocks, 5, sums5);
  return cudaGetLastError();
}

static constexpr uint32_t kFwdSmem = dev::kFwdSmemBytes + 1024u;
static constexpr uint32_t kBwdSmem = 196608u + 1024u;

// Function attributes are set once per device (a bit per device ordinal).
static bool attr_needed(std::atomic<unsigned long long> &done) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev >= 64) return true;
  return (done.load() >> dev & 1ull) == 0;
}
static void attr_set(std::atomic<unsigned long long> &done) {
  int dev = 0;
  if (cudaGetDevice(&dev) == cudaSuccess && dev < 64) done.fetch_or(1ull << dev);
}

static std::atomic<unsigned long long> g_fwd_attr{0}, g_bwd_attr{0};

static cudaError_t fwd_attributes() {
  if (!attr_needed(g_fwd_attr)) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(dev::cv_mlp_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kFwdSmem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(dev::cv_mlp_kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                             (int)cudaSharedmemCarveoutMaxShared);
  if (e == cudaSuccess) attr_set(g_fwd_attr);
  return e;
}

static cudaError_t bwd_attributes() {
  if (!attr_needed(g_bwd_attr)) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(dev::cv_bwd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kBwdSmem);
  if (e == cudaSuccess) attr_set(g_bwd_attr);
  return e;
}

// The function attributes of both MLP kernels on the current device, set ahead of a
// stream capture (no attribute call then happens while the training loop is captured).
cudaError_t cv_prepare_kernels() {
  cudaError_t e = fwd_attributes();
  return e == cudaSuccess ? bwd_attributes() : e;
}

cudaError_t launch_cv_mlp(const CvMlpParams &P, unsigned int blocks, cudaStream_t st) {
  cudaError_t e = fwd_attributes();
  if (e != cudaSuccess) return e;
  dev::cv_mlp_kernel<<<blocks, dev::kFwdThreads, kFwdSmem, st>>>(P);
  return cudaGetLastError();
}

cudaError_t launch_cv_bwd(const CvMlpParams &P, unsigned int blocks, cudaStream_t st) {
  cudaError_t e = bwd_attributes();
  if (e != cudaSuccess) return e;
  dev::cv_bwd_kernel<<<blocks, dev::kBwdThreads, kBwdSmem, st>>>(P);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  dev::cv_grad_reduce_kernel<<<(kPCount + 255) / 256, 256, 0, st>>>(P.gpart, blocks, P.grad);
  return cudaGetLastError();
}

cudaError_t launch_cv_pack(const float *params, uint8_t *img, float *vec, cudaStream_t st) {
  dev::cv_pack_kernel<<<(128 * 128 + 255) / 256, 256, 0, st>>>(params, img, vec);
  return cudaGetLastError();
}

cudaError_t launch_cv_adam(float *params, float *m, float *v, const float *grad, float lr, float b1t, float b2t,
                           cudaStream_t st) {
  dev::cv_adam_kernel<<<(kPCount + 255) / 256, 256, 0, st>>>(params, m, v, grad, lr, b1t, b2t);
  return cudaGetLastError();
}

// part: kResidBlocks doubles of scratch; loss_part: kResidBlocks partial sums of
// r^2 / n (the loss is their sum, in order)
cudaError_t launch_cv_resid(const float *Y, const float *cv, unsigned long long n, float *coef, double *loss_part,
                            double *part, cudaStream_t st) {
  dev::cv_resid_sum_kernel<<<kResidBlocks, 256, 0, st>>>(Y, cv, n, part);
  dev::cv_resid_coef_kernel<<<kResidBlocks, 256, 0, st>>>(Y, cv, n, part, coef, loss_part);
  return cudaGetLastError();
}

cudaError_t launch_cv_rowsum(const float *gdm, unsigned long long n_paths, unsigned int n_hedge, float *cv,
                             cudaStream_t st) {
  dev::cv_rowsum_kernel<<<(unsigned int)((n_paths + 255) / 256), 256, 0, st>>>(gdm, n_paths, n_hedge, cv);
  return cudaGetLastError();
}

cudaError_t launch_cv_reduce(const float *Y, const float *cv, unsigned long long n, double *sums4, double *part,
                             cudaStream_t st) {
  dev::cv_reduce_kernel<<<kFoldBlocks, 256, 0, st>>>(Y, cv, n, part);
  dev::cv_fold_kernel<<<1, 32 * 4, 0, st>>>(part, kFoldBlocks, 4, sums4);
  return cudaGetLastError();
}

}  // namespace myql
