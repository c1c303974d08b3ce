// cv.cuh -- neural martingale control variate (no counterpart in the reference).
//
// A small MLP g(t, log S, v1, v2, running average) -> R is trained on pilot
// paths of the engine itself and then used as the control
//     C = sum_j g(state at t_j) * dM_j,
// where dM_j is the martingale increment of the discounted asset
// M_t = S_t e^{-(r-q) t} over the hedge interval [t_j, t_{j+1}).  Per step k
// the increment is centred by its exact conditional mean under the discrete
// scheme: with dX_k = C0 + C1 v + C2 v' + sqrt(C3 (v + v')) G (summed over the
// factors) and the variance transition's moment generating function,
//     log E[e^{dX_k} | v] = mu_k = A + B_1 v_1 + B_2 v_2        (affine in v)
//     dM_k = M_k e^{mu_k - (r-q) dt} expm1(dX_k - mu_k) + M_k' expm1(J_k)
// (E[e^{J}] = 1 for the compensated jumps), so E[g_j dM_k] = 0 for any g_j
// that depends on the path up to t_j: the estimator Y - C is unbiased whatever
// the network.
//
// Network: 16 input slots (6 used: t/T, x-scaled log-spot, scaled v1, v2, the
// average to date (Asian) or the knocked flag (barrier), 1) -> 128 -> 128 -> 128 (SiLU) -> 1, BF16 weights and
// activations, FP32 accumulation on the tcgen05 tensor cores.
//
// Data layout (HBM): rows are (path, hedge time); a tile is 128 consecutive
// paths at one hedge time, tiles ordered [path block][hedge time].  Feature
// tiles are stored as the IMG16 shared-memory image (4 KB, moved by one bulk
// copy); dM is FP32 [tile][128].
#pragma once
#include <cuda_bf16.h>

#include "batch.cuh"
#include "tc.cuh"

namespace myql {

constexpr int kCvHidden = 128;
constexpr int kCvIn = 16;
constexpr int kCvFeatures = 6;
constexpr uint32_t kCvTileBytes = 128u * kCvIn * 2u;  // 4096
constexpr uint64_t kCvInSamplePaths = 1ull << 17;  // pilot paths of the in-sample diagnostic
constexpr unsigned int kResidBlocks = 64;           // fixed grid of the residual reductions
constexpr unsigned int kFoldBlocks = 608;           // fixed grid of the price / hedge-ratio sums

// FP32 parameter blob: W1 [128][16], b1, W2 [128][128], b2, W3 [128][128], b3, w4 [128], b4
constexpr int kPW1 = 0;
constexpr int kPB1 = kPW1 + 128 * 16;
constexpr int kPW2 = kPB1 + 128;
constexpr int kPB2 = kPW2 + 128 * 128;
constexpr int kPW3 = kPB2 + 128;
constexpr int kPB3 = kPW3 + 128 * 128;
constexpr int kPW4 = kPB3 + 128;
constexpr int kPB4 = kPW4 + 128;
constexpr int kPCount = kPB4 + 4;

// Packed BF16 weight images: W1 IMG16 [128][16], W2 and W3 IMG128 [128][128],
// W1 zero-padded to K = 64 as IMG128 [128][64] (backward kernel).
constexpr uint32_t kImgW1 = 0, kImgW2 = 4096, kImgW3 = 4096 + 32768, kImgW1x64 = 4096 + 65536;
constexpr uint32_t kImgBytes = kImgW1x64 + 16384;
constexpr uint32_t kImgFwdBytes = kImgW1x64;  // W1, W2, W3
// FP32 vectors beside the images: b1, b2, b3, w4 (128 each), b4
constexpr int kVecB1 = 0, kVecB2 = 128, kVecB3 = 256, kVecW4 = 384, kVecB4 = 512, kVecCount = 516;
constexpr int kHalfBias = 384;  // 0.5 x (b1, b2, b3), kept in shared memory by the MLP kernels

constexpr unsigned long long kCvWaitNs = 2000000000ull;  // bounded waits: 2 s

// Per-discretisation constants of the hedge features and increments.
struct CvFeatConsts {
  float rq_dt;                      // (r - q) dt
  float inv_T, x_scale, va_scale, vb_scale, S0;
  float mu_A, mu_Ba, mu_Bb;         // log E[e^{dX} | v] = mu_A + mu_Ba v1 + mu_Bb v2
  int tracker;
};

struct CvSimParams {
  SimParams sim;        // one scenario (base), path-dependent stepping
  PayoffParams pay;     // scalar instrument
  double df;
  uint8_t *feat;        // feature tiles of this launch's paths
  float *dM;            // [tile][128]
  float *Y;             // discounted payoff per path (launch-local index)
  unsigned long long path_begin, path_end;
  int hedge_every, n_hedge;
  CvFeatConsts fc;
};

struct CvMlpParams {
  const uint8_t *feat;
  const float *dM;
  const uint8_t *img;   // packed weights (kImgBytes)
  const float *vec;     // kVecCount floats
  float *cv;            // per path: sum_j g_j dM_j (path-major forward)
  float *g_out;         // optional per-row g
  float *gdm;           // tile-major forward: per-row g dM, summed per path by cv_rowsum_kernel
  int tile_major;       // forward: 1 = blocks take tiles round robin, 0 = whole path blocks
  const float *coef;    // backward: dL/dC per path
  float *grad;          // backward: FP32 parameter-blob gradient (written by the reduction)
  float *gpart;         // backward: per-block gradient slices [gridDim.x][kPCount]
  unsigned long long n_paths;
  unsigned int n_pb, n_hedge;
  unsigned int *status;  // [2] += 1 on a wait that ran out
};

// One MLMC level evaluation with the control variate: level 0 plain paths
// (CvHook), level l > 0 coupled pairs (MlmcCvHook); Y = df (P_fine - P_coarse).
struct MlmcCvParams {
  MlmcParams M;
  uint8_t *feat;
  float *dM;
  float *Y;
  int hedge_every;  // steps (level 0) or coarse steps (level > 0) per hedge interval
  int n_hedge;
  CvFeatConsts fine, coarse;
  double df;
};

namespace dev {

// One feature row (IMG16 slot `lane` of a tile): t/T, scaled log-spot, scaled
// variances, path state, 1.
__device__ __forceinline__ void cv_write_feat(const CvFeatConsts *P, uint8_t *tile, uint32_t lane, float t,
                                              float X, float va, float vb, float st) {
  __nv_bfloat162 p0 = __floats2bfloat162_rn(t * P->inv_T, X * P->x_scale);
  __nv_bfloat162 p1 = __floats2bfloat162_rn(va * P->va_scale, vb * P->vb_scale);
  __nv_bfloat162 p2 = __floats2bfloat162_rn(st, 1.0f);
  uint4 c0;
  c0.x = *reinterpret_cast<uint32_t *>(&p0);
  c0.y = *reinterpret_cast<uint32_t *>(&p1);
  c0.z = *reinterpret_cast<uint32_t *>(&p2);
  c0.w = 0u;
  *reinterpret_cast<uint4 *>(tile + tc::img16_offset(lane, 0)) = c0;
  *reinterpret_cast<uint4 *>(tile + tc::img16_offset(lane, 8)) = make_uint4(0u, 0u, 0u, 0u);
}

// Path state beside (t, X, v) after k steps of size dt: the average to date
// (Asian) or the knocked flag of the base barrier (barrier instruments).
__device__ __forceinline__ float cv_path_state(const CvFeatConsts *P, int k, float dt, float X, float trk,
                                               bool hit) {
  if (k == 0) return 0.0f;
  if (P->tracker == TRK_ARITH_ASIAN) return dt * (0.5f + trk - 0.5f * __expf(X)) * P->inv_T;
  if (P->tracker == TRK_GEO_ASIAN) return dt * (trk - 0.5f * X) * P->inv_T;
  if (P->tracker >= TRK_BARRIER_UP) return hit ? 1.0f : 0.0f;
  return 0.0f;
}

// Centred increment of the discounted asset over one step that started at m
// (relative to S0) with log-spot increment dx = root G + drift and start
// variances (va, vb): m e^{mu - (r-q) dt} expm1(dx - mu), mu = log E[e^{dx} | v].
__device__ __forceinline__ float cv_step_incr(const CvFeatConsts *P, float m, float dx, float va, float vb) {
  const float mu = fmaf(P->mu_Bb, vb, fmaf(P->mu_Ba, va, P->mu_A));
  return m * __expf(mu - P->rq_dt) * expm1f(dx - mu);
}

// Path observer writing the features at hedge times and the centred
// martingale increments of every hedge interval.
struct CvHook {
  static constexpr bool active = true;
  const CvFeatConsts *P;
  uint8_t *tile0;  // feature tile of hedge 0 for this path's block
  float *dm0;      // dM entry of hedge 0 for this path
  uint32_t lane;
  int j, he, n;
  float m, m_mid, acc, dt;
  float va_c, vb_c;  // variances at the start of the current step

  __device__ __forceinline__ void begin(float va, float vb) {
    m = 1.0f;
    acc = 0.0f;
    j = 0;
    va_c = va;
    vb_c = vb;
    cv_write_feat(P, tile0, lane, 0.0f, 0.0f, va, vb, 0.0f);
  }
  __device__ __forceinline__ void diffusion(float root, float G, float drift) {
    const float dx = fmaf(root, G, drift);
    acc += cv_step_incr(P, m, dx, va_c, vb_c);
    m_mid = m * __expf(dx - P->rq_dt);
  }
  __device__ __forceinline__ void jump(float J) { acc = fmaf(m_mid, expm1f(J), acc); }
  __device__ __forceinline__ void step_end(int k, float X, float va, float vb, float trk, bool hit) {
    va_c = va;
    vb_c = vb;
    m = __expf(X - P->rq_dt * (float)k);
    if (k < n && k % he == 0) {
      dm0[(size_t)j * 128] = acc * P->S0;
      acc = 0.0f;
      ++j;
      cv_write_feat(P, tile0 + (size_t)j * kCvTileBytes, lane, (float)k * dt, X, va, vb,
                    cv_path_state(P, k, dt, X, trk, hit));
    }
  }
  __device__ __forceinline__ void finish() { dm0[(size_t)j * 128] = acc * P->S0; }
};

// Observer of a coupled (fine, coarse) path pair: features of the fine path at
// the hedge times (every `hc` coarse steps) and, per hedge interval, the
// difference of the fine and coarse centred increments -- the martingale part
// of the level correction's asset exposure.
struct MlmcCvHook {
  static constexpr bool active = true;
  const CvFeatConsts *F, *Cc;  // fine / coarse discretisation
  uint8_t *tile0;
  float *dm0;
  uint32_t lane;
  int j, hc, nc;
  float mf, mf_mid, mc, mc_mid, acc, dtf;

  __device__ __forceinline__ void begin(float va, float vb) {
    mf = mc = 1.0f;
    acc = 0.0f;
    j = 0;
    cv_write_feat(F, tile0, lane, 0.0f, 0.0f, va, vb, 0.0f);
  }
  __device__ __forceinline__ void fine(float root, float G, float drift, float va, float vb) {
    const float dx = fmaf(root, G, drift);
    acc += cv_step_incr(F, mf, dx, va, vb);
    mf_mid = mf * __expf(dx - F->rq_dt);
    mf = mf_mid;
  }
  __device__ __forceinline__ void fine_jump(float J) {
    acc = fmaf(mf_mid, expm1f(J), acc);
    mf = mf_mid * __expf(J);
  }
  __device__ __forceinline__ void coarse(float root, float G, float drift, float va, float vb) {
    const float dx = fmaf(root, G, drift);
    acc -= cv_step_incr(Cc, mc, dx, va, vb);
    mc_mid = mc * __expf(dx - Cc->rq_dt);
    mc = mc_mid;
  }
  __device__ __forceinline__ void coarse_jump(float J) {
    acc = fmaf(-mc_mid, expm1f(J), acc);
    mc = mc_mid * __expf(J);
  }
  __device__ __forceinline__ void coarse_end(int kc, float Xf, float Xc, float va, float vb, float trk, bool hit) {
    mf = __expf(Xf - F->rq_dt * (float)(2 * kc));
    mc = __expf(Xc - Cc->rq_dt * (float)kc);
    if (kc < nc && kc % hc == 0) {
      dm0[(size_t)j * 128] = acc * F->S0;
      acc = 0.0f;
      ++j;
      cv_write_feat(F, tile0 + (size_t)j * kCvTileBytes, lane, (float)(2 * kc) * dtf, Xf, va, vb,
                    cv_path_state(F, 2 * kc, dtf, Xf, trk, hit));
    }
  }
  __device__ __forceinline__ void finish() { dm0[(size_t)j * 128] = acc * F->S0; }
};

// Terminal record -> the payoff pass's view of one path (base scenario).
__device__ __forceinline__ PathView record_view(const PayoffParams &Q, const float (&r)[kMaxFields]) {
  PathView v;
  v.S = Q.S0 * __expf(r[0]);
  v.Y = 0.0f;
  v.hit[0] = v.hit[1] = v.hit[2] = -1.0f;
  switch (Q.tracker) {
    case TRK_GEO_ASIAN: v.Y = Q.S0 * __expf(fmaf(Q.avg_c1[0], r[1], Q.avg_c0[0])); break;
    case TRK_ARITH_ASIAN: v.Y = Q.S0 * fmaf(Q.avg_c1[0], r[1], Q.avg_c0[0]); break;
    case TRK_BARRIER_UP:
    case TRK_BARRIER_DOWN:
      v.hit[0] = r[1];
      v.hit[1] = r[2];
      v.hit[2] = r[3];
      break;
    default: break;
  }
  return v;
}

}  // namespace dev

cudaError_t launch_cv_sim(const CvSimParams &P, int klass, cudaStream_t st);
cudaError_t launch_mlmc_cv_level(const MlmcCvParams &Q, int klass, cudaStream_t st);
cudaError_t launch_cv_mlp(const CvMlpParams &P, unsigned int blocks, cudaStream_t st);
cudaError_t launch_cv_bwd(const CvMlpParams &P, unsigned int blocks, cudaStream_t st);
cudaError_t cv_prepare_kernels();
cudaError_t launch_cv_pack(const float *params, uint8_t *img, float *vec, cudaStream_t st);
cudaError_t launch_cv_adam(float *params, float *m, float *v, const float *grad, float lr, float b1t, float b2t,
                           cudaStream_t st);
cudaError_t launch_cv_resid(const float *Y, const float *cv, unsigned long long n, float *coef, double *loss_part,
                            double *part, cudaStream_t st);
cudaError_t launch_cv_beta(const float *Y, const float *dM, unsigned long long n, unsigned int n_hedge,
                           double *sums5, double *part, cudaStream_t st);
cudaError_t launch_cv_rowsum(const float *gdm, unsigned long long n_paths, unsigned int n_hedge, float *cv,
                             cudaStream_t st);
cudaError_t launch_cv_reduce(const float *Y, const float *cv, unsigned long long n, double *sums4, double *part,
                             cudaStream_t st);

}  // namespace myql
