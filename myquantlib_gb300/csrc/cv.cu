// cv.cu -- host side of the neural control variate (myql_cv_*).
//
//   train:  pilot paths (an independent seed) -> features, increments, payoffs;
//           Adam on L = mean_p (Y_p - C_p - mean(Y - C))^2 over minibatches of
//           path blocks: forward (cv_mlp_kernel) -> residuals -> backward
//           (cv_bwd_kernel) -> Adam + repacking of the BF16 images.
//   price:  chunks of paths: simulate (cv_sim_kernel) -> forward -> FP64 sums of
//           Y and Y - C; returns the control-variate and the plain estimator of
//           the same paths and their variance ratio.
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "cv.cuh"
#include "engine.h"
#include "qmc.cuh"

namespace myql {
static_assert(kPCount == MYQL_CV_PARAMS, "parameter blob size");
namespace {

struct CvState : ExtState {
  DevBuf params, adam_m, adam_v, grad, img, vec, coef, loss, sums;
  DevBuf p_feat, p_dM, p_Y, p_cv;  // pilot set
  DevBuf feat, dM, Y, cv;          // pricing chunk / caller data
  DevBuf gdm;                      // per-row g dM of the tile-major forward
  DevBuf gpart;                    // per-block gradient slices of the backward
  DevBuf rpart;                    // per-block residual sums
  DevBuf fpart;                    // per-block price / hedge-ratio sums
  bool init = false;
  uint64_t adam_t = 0;
  // the Adam loop of the last training shape, as one CUDA graph
  cudaGraphExec_t train_graph = nullptr;
  uint64_t train_key = 0;
  uint32_t train_launches = 0;
  ~CvState() {
    if (train_graph) cudaGraphExecDestroy(train_graph);
  }
};

uint64_t splitmix(uint64_t &s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

void init_params(std::vector<float> &p, uint64_t seed) {
  p.assign(kPCount, 0.0f);
  uint64_t s = seed;
  auto uni = [&](float a) { return (float)(((double)(splitmix(s) >> 11) * 0x1.0p-53 * 2.0 - 1.0) * a); };
  const float a1 = 1.0f / std::sqrt((float)kCvFeatures), a2 = 1.0f / std::sqrt(128.0f);
  for (int o = 0; o < 128; ++o)
    for (int k = 0; k < kCvFeatures; ++k) p[kPW1 + o * kCvIn + k] = uni(a1);
  for (int o = 0; o < 128; ++o) p[kPB1 + o] = uni(a1);
  for (int i = 0; i < 128 * 128; ++i) p[kPW2 + i] = uni(a2);
  for (int o = 0; o < 128; ++o) p[kPB2 + o] = uni(a2);
  for (int i = 0; i < 128 * 128; ++i) p[kPW3 + i] = uni(a2);
  for (int o = 0; o < 128; ++o) p[kPB3 + o] = uni(a2);
  for (int o = 0; o < 128; ++o) p[kPW4 + o] = uni(0.1f * a2);
}

CvState &state(CtxBase *ctx) {
  if (!ctx->cv) ctx->cv.reset(new CvState);
  return *static_cast<CvState *>(ctx->cv.get());
}

myql_status upload_params(CtxBase *ctx, CvState &S, const float *p) {
  cudaError_t e = S.params.ensure(kPCount * 4);
  if (e == cudaSuccess) e = S.adam_m.ensure(kPCount * 4);
  if (e == cudaSuccess) e = S.adam_v.ensure(kPCount * 4);
  if (e == cudaSuccess) e = S.grad.ensure(kPCount * 4);
  if (e == cudaSuccess) e = S.img.ensure(kImgBytes);
  if (e == cudaSuccess) e = S.vec.ensure(kVecCount * 4);
  if (e == cudaSuccess) e = S.loss.ensure(8ull * 4096 * kResidBlocks);  // [iteration][block] loss partials
  if (e == cudaSuccess) e = S.sums.ensure(128);
  if (e == cudaSuccess) e = S.rpart.ensure(8 * kResidBlocks);
  if (e == cudaSuccess) e = S.fpart.ensure(8 * 5 * kFoldBlocks);
  if (e == cudaSuccess) e = cudaMemcpyAsync(S.params.p, p, kPCount * 4, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(S.adam_m.p, 0, kPCount * 4, ctx->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(S.adam_v.p, 0, kPCount * 4, ctx->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(S.img.p, 0, kImgBytes, ctx->stream);
  if (e == cudaSuccess) e = launch_cv_pack((const float *)S.params.p, (uint8_t *)S.img.p, (float *)S.vec.p, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_status(e, "control-variate parameters");
  S.init = true;
  S.adam_t = 0;
  return MYQL_OK;
}

myql_status check_job(const myql_mc_job &job) {
  myql_status s = validate_job(job);
  if (s != MYQL_OK) return s;
  const int trk = tracker_of(job.instrument);
  if (job.instrument.is_strip || job.instrument.n_strikes != 1)
    return set_error(MYQL_ERR_UNSUPPORTED, "control variates take scalar instruments");
  if (trk == TRK_LOOKBACK)
    return set_error(MYQL_ERR_UNSUPPORTED, "control variates cover European, Asian and barrier instruments");
  return MYQL_OK;
}

myql_status check_cfg(const myql_cv_config *c) {
  if (!c || c->hedge_every < 1 || c->iterations > 4096 || c->batch_paths < 128 || !(c->learning_rate > 0.0))
    return set_error(MYQL_ERR_INVALID_ARG, "control-variate config: hedge_every >= 1, iterations <= 4096, "
                                           "batch_paths >= 128, learning_rate > 0");
  return MYQL_OK;
}

}  // namespace
myql_status cv_feat_consts(const myql_mc_job &job, const Plan &pl, const ScenarioConst &sc, double dt,
                           CvFeatConsts &F);
namespace {

// Simulation constants of the control-variate kernels for one job.
myql_status cv_plan(CtxBase *ctx, const myql_mc_job &job, const myql_cv_config &cfg, Plan &pl, CvSimParams &C,
                    int &klass) {
  myql_status s = make_plan(job, pl, true);
  if (s != MYQL_OK) return s;
  for (int f = 0; f < pl.nf; ++f)
    if (job.config.scheme[f] == MYQL_SCHEME_NCI) {
      s = ensure_nci(ctx, job.model.heston[f], pl.sim.sc[0].dt, pl.sim.nci[f]);
      if (s != MYQL_OK) return s;
    }
  cudaError_t e = ctx->strikes.ensure(sizeof(double));
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(ctx->strikes.p, job.instrument.strikes, sizeof(double), cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) e = ctx->status.ensure(16);
  if (e == cudaSuccess) e = cudaMemsetAsync(ctx->status.p, 0, 16, ctx->stream);
  if (e != cudaSuccess) return cuda_status(e, "control-variate set-up");
  std::memset(&C, 0, sizeof C);
  C.sim = pl.sim;
  C.sim.status = (unsigned int *)ctx->status.p;
  C.sim.loop_cap = ctx->loop_cap;
  C.pay = pl.pay;
  C.pay.strikes = (const double *)ctx->strikes.p;
  C.df = pl.df;
  C.hedge_every = (int)cfg.hedge_every;
  C.n_hedge = (pl.steps + (int)cfg.hedge_every - 1) / (int)cfg.hedge_every;
  klass = batch_class(pl.nf, pl.s1, pl.s2);
  return cv_feat_consts(job, pl, pl.sim.sc[0], job.instrument.maturity / pl.steps, C.fc);
}
}  // namespace

// Feature scales and the conditional mean of e^{dX} per step for one
// discretisation (its scenario constants, step dt).
myql_status cv_feat_consts(const myql_mc_job &job, const Plan &pl, const ScenarioConst &sc, double dt,
                           CvFeatConsts &F) {
  const double T = job.instrument.maturity;
  F.rq_dt = (float)((job.r - job.q) * dt);
  F.inv_T = (float)(1.0 / T);
  double vref = 0.0;
  if (pl.nf == 0) vref = job.model.vol * job.model.vol;
  for (int f = 0; f < pl.nf; ++f) vref += std::max(job.model.heston[f].theta, 1e-4);
  F.x_scale = (float)(1.0 / std::sqrt(std::max(vref, 1e-6) * T));
  F.va_scale = pl.nf >= 1 ? (float)(1.0 / std::max(job.model.heston[0].theta, 1e-4)) : 0.0f;
  F.vb_scale = pl.nf >= 2 ? (float)(1.0 / std::max(job.model.heston[1].theta, 1e-4)) : 0.0f;
  F.S0 = (float)job.S0;
  F.tracker = pl.tracker;
  // conditional mean of e^{dX} per step, from the FP32 constants the kernel steps with
  double A = 0.0, B[2] = {0.0, 0.0};
  if (pl.nf == 0) {
    A = (double)sc.gbm_drift + 0.5 * (double)sc.gbm_vol * (double)sc.gbm_vol;
  } else {
    for (int f = 0; f < pl.nf; ++f) {
      const FactorConst &fc = sc.f[f];
      const double C0 = fc.C0, C1 = fc.C1, C2 = fc.C2, C3 = fc.C3, w0 = fc.w0, w1 = fc.w1, w2 = fc.w2;
      const double u = C2 + 0.5 * C3;  // exponent of v' in e^{dX} after averaging over G
      double alpha = 0.0, beta = 0.0;
      const int sch = job.config.scheme[f];
      if (sch == MYQL_SCHEME_NV) {  // v' = w0 (sqrt(w0 v + w1) + w2 Z)^2 + w1
        const double den = 1.0 - 2.0 * u * w0 * w2 * w2;
        if (!(den > 0.0)) return set_error(MYQL_ERR_UNSUPPORTED, "E[S_T] is infinite under this discretisation");
        alpha = u * w0 * w0 / den;
        beta = u * w1 + u * w0 * w1 / den - 0.5 * std::log(den);
      } else if (sch == MYQL_SCHEME_EXACT) {  // v' = Gamma(w1 + N) w2, N ~ Poisson(w0 v)
        const double den = 1.0 - u * w2;
        if (!(den > 0.0)) return set_error(MYQL_ERR_UNSUPPORTED, "E[S_T] is infinite under this discretisation");
        alpha = w0 * u * w2 / den;
        beta = -w1 * std::log(den);
      } else {  // NCI: v' = chi2_{w1 + 2N} w2, N ~ Poisson(w0 v)
        const double den = 1.0 - 2.0 * u * w2;
        if (!(den > 0.0)) return set_error(MYQL_ERR_UNSUPPORTED, "E[S_T] is infinite under this discretisation");
        alpha = w0 * 2.0 * u * w2 / den;
        beta = -0.5 * w1 * std::log(den);
      }
      A += C0 + beta;
      B[f] = C1 + 0.5 * C3 + alpha;
    }
  }
  F.mu_A = (float)A;
  F.mu_Ba = (float)B[0];
  F.mu_Bb = (float)B[1];
  return MYQL_OK;
}
namespace {

// Simulates paths [0, M) of (seed, stream_offset) into feat / dM / Y, in chunks
// that are multiples of the stream count; `chunk_cb` consumes each chunk.
template <class F>
myql_status simulate_chunks(CtxBase *ctx, CvSimParams C, int klass, uint64_t seed, uint64_t offset, uint64_t M,
                            uint64_t S, uint64_t chunk, DevBuf &feat, DevBuf &dM, DevBuf &Y, F chunk_cb) {
  myql_status s = ensure_streams(ctx, seed, offset, S);
  if (s != MYQL_OK) return s;
  C.sim.states = (unsigned long long *)ctx->st_work.p;
  C.sim.n_streams = (unsigned int)S;
  C.sim.num_paths = M;
  const uint64_t nh = (uint64_t)C.n_hedge;
  const uint64_t pbs = (chunk + 127) / 128;
  cudaError_t e = feat.ensure(pbs * nh * kCvTileBytes);
  if (e == cudaSuccess) e = dM.ensure(pbs * nh * 128 * 4);
  if (e == cudaSuccess) e = Y.ensure(pbs * 128 * 4);
  if (e != cudaSuccess) return cuda_status(e, "control-variate path buffers");
  C.feat = (uint8_t *)feat.p;
  C.dM = (float *)dM.p;
  C.Y = (float *)Y.p;
  for (uint64_t b = 0; b < M; b += chunk) {
    C.path_begin = b;
    C.path_end = std::min(M, b + chunk);
    e = launch_cv_sim(C, klass, ctx->stream);
    if (e != cudaSuccess) return cuda_status(e, "cv_sim launch");
    ctx->launches++;
    s = chunk_cb(C.path_end - C.path_begin);
    if (s != MYQL_OK) return s;
  }
  return MYQL_OK;
}

// persistent grids: one block per SM
unsigned int mlp_blocks(const CtxBase *ctx, uint64_t n_units) {
  return (unsigned int)std::max<uint64_t>(1, std::min<uint64_t>(n_units, (uint64_t)ctx->sm_count));
}

myql_status forward(CtxBase *ctx, CvState &S, const uint8_t *feat, const float *dM, uint64_t n_paths, uint32_t nh,
                    float *cv, float *g_out) {
  CvMlpParams F;
  std::memset(&F, 0, sizeof F);
  const uint64_t n_pb = (n_paths + 127) / 128;
  // few path blocks (training minibatches): spread the tiles over every SM
  if (n_pb < (uint64_t)ctx->sm_count * 8) {
    cudaError_t e = S.gdm.ensure(n_pb * nh * 128 * 4);
    if (e != cudaSuccess) return cuda_status(e, "control-variate row buffer");
    F.tile_major = 1;
    F.gdm = (float *)S.gdm.p;
  }
  F.feat = feat;
  F.dM = dM;
  F.img = (const uint8_t *)S.img.p;
  F.vec = (const float *)S.vec.p;
  F.cv = cv;
  F.g_out = g_out;
  F.n_paths = n_paths;
  F.n_pb = (unsigned int)((n_paths + 127) / 128);
  F.n_hedge = nh;
  F.status = (unsigned int *)ctx->status.p;
  // one block per SM, four tile groups per block
  const uint64_t units = F.tile_major ? n_pb * nh : n_pb;
  cudaError_t e = launch_cv_mlp(F, mlp_blocks(ctx, (units + 3) / 4), ctx->stream);
  ctx->launches++;
  if (e == cudaSuccess && F.tile_major) {
    e = launch_cv_rowsum(F.gdm, n_paths, nh, cv, ctx->stream);
    ctx->launches++;
  }
  return cuda_status(e, "cv_mlp launch");
}

myql_status backward(CtxBase *ctx, CvState &S, const uint8_t *feat, const float *dM, uint64_t n_paths, uint32_t nh) {
  CvMlpParams B;
  std::memset(&B, 0, sizeof B);
  B.feat = feat;
  B.dM = dM;
  B.img = (const uint8_t *)S.img.p;
  B.vec = (const float *)S.vec.p;
  B.coef = (const float *)S.coef.p;
  B.grad = (float *)S.grad.p;
  B.n_paths = n_paths;
  B.n_pb = (unsigned int)((n_paths + 127) / 128);
  B.n_hedge = nh;
  B.status = (unsigned int *)ctx->status.p;
  const unsigned int blocks = mlp_blocks(ctx, (uint64_t)B.n_pb * nh);
  cudaError_t e = S.gpart.ensure((size_t)blocks * kPCount * 4);
  if (e != cudaSuccess) return cuda_status(e, "control-variate gradient slices");
  B.gpart = (float *)S.gpart.p;
  e = launch_cv_bwd(B, blocks, ctx->stream);
  ctx->launches += 2;
  return cuda_status(e, "cv_bwd launch");
}

myql_status wait_status(CtxBase *ctx) {
  unsigned int hs[4] = {0, 0, 0, 0};
  cudaError_t e = cudaMemcpyAsync(hs, ctx->status.p, 16, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_status(e, "control-variate status");
  if (hs[2]) return set_error(MYQL_ERR_TIMEOUT, "a tensor-core pipeline wait ran out (%u blocks)", hs[2]);
  if (hs[0]) return set_error(MYQL_ERR_LOOP_CAP, "%u bounded device loops hit their cap", hs[0]);
  return MYQL_OK;
}

// host rows [p][j][6] -> tile images [pb][j] and dM [tile][128] (zero padding)
void pack_rows(const float *feats, const float *dM, uint64_t n, uint32_t nh, std::vector<uint8_t> &img,
               std::vector<float> &dm) {
  const uint64_t pbs = (n + 127) / 128;
  img.assign(pbs * nh * kCvTileBytes, 0);
  dm.assign(pbs * nh * 128, 0.0f);
  for (uint64_t p = 0; p < n; ++p)
    for (uint32_t j = 0; j < nh; ++j) {
      const uint64_t tile = (p / 128) * nh + j, lane = p % 128, row = p * nh + j;
      uint8_t *t = img.data() + tile * kCvTileBytes;
      for (int k = 0; k < kCvFeatures; ++k) {
        const __nv_bfloat16 b = __float2bfloat16_rn(feats[row * kCvFeatures + k]);
        std::memcpy(t + tc::img16_offset((uint32_t)lane, (uint32_t)k), &b, 2);
      }
      dm[tile * 128 + lane] = dM ? dM[row] : 0.0f;
    }
}

double ms_since(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace
}  // namespace myql

namespace myql {

// One MLMC level evaluation with the context's network: simulate (features,
// increments, discounted differences), MLP forward, FP64 sums
// {sum Y, sum Y^2, sum (Y - C), sum (Y - C)^2} added into sums4.
myql_status cv_level_eval(CtxBase *ctx, MlmcCvParams &Q, int klass, uint64_t dN, double *sums4) {
  CvState &S = state(ctx);
  if (!S.init) return set_error(MYQL_ERR_INVALID_ARG, "no control-variate network in this context");
  // chunks of a multiple of the streams in use (every stream continues its own paths)
  // with at most ~2 GiB of features
  const uint64_t U = Q.M.n_used, nh = (uint64_t)Q.n_hedge;
  uint64_t chunk = (2ull << 30) / (nh * (kCvTileBytes / 128 + 4));
  chunk = std::max<uint64_t>(U, chunk / U * U);
  chunk = std::min<uint64_t>(chunk, dN);
  const uint64_t pbs = (chunk + 127) / 128;
  cudaError_t e = S.feat.ensure(pbs * nh * kCvTileBytes);
  if (e == cudaSuccess) e = S.dM.ensure(pbs * nh * 128 * 4);
  if (e == cudaSuccess) e = S.Y.ensure(pbs * 128 * 4);
  if (e == cudaSuccess) e = S.cv.ensure(pbs * 128 * 4);
  if (e == cudaSuccess) e = cudaMemsetAsync(S.sums.p, 0, 32, ctx->stream);
  if (e != cudaSuccess) return cuda_status(e, "MLMC control-variate buffers");
  Q.feat = (uint8_t *)S.feat.p;
  Q.dM = (float *)S.dM.p;
  Q.Y = (float *)S.Y.p;
  for (uint64_t done = 0; done < dN; done += chunk) {
    const uint64_t n = std::min(chunk, dN - done);
    Q.M.dN = n;
    e = launch_mlmc_cv_level(Q, klass, ctx->stream);
    if (e != cudaSuccess) return cuda_status(e, "MLMC control-variate level launch");
    myql_status s = forward(ctx, S, (const uint8_t *)S.feat.p, (const float *)S.dM.p, n, (uint32_t)nh,
                            (float *)S.cv.p, nullptr);
    if (s != MYQL_OK) return s;
    e = launch_cv_reduce((const float *)S.Y.p, (const float *)S.cv.p, n, (double *)S.sums.p, (double *)S.fpart.p,
                         ctx->stream);
    if (e != cudaSuccess) return cuda_status(e, "MLMC control-variate reduction");
    ctx->launches += 2;
  }
  double h4[4] = {0, 0, 0, 0};
  e = cudaMemcpyAsync(h4, S.sums.p, 32, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_status(e, "MLMC control-variate sums");
  for (int i = 0; i < 4; ++i) sums4[i] += h4[i];
  return MYQL_OK;
}

myql_status cv_feat_consts(const myql_mc_job &job, const Plan &pl, const ScenarioConst &sc, double dt,
                           CvFeatConsts &F);

}  // namespace myql

using namespace myql;

extern "C" {

myql_status myql_cv_set_params(myql_ctx *ctx_, const float *params, size_t n) {
  CtxBase *ctx = reinterpret_cast<CtxBase *>(ctx_);
  if (!ctx || !params || n != (size_t)MYQL_CV_PARAMS) return set_error(MYQL_ERR_INVALID_ARG, "need MYQL_CV_PARAMS floats");
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) return cuda_status(e, "cudaSetDevice");
  return upload_params(ctx, state(ctx), params);
}

myql_status myql_cv_get_params(myql_ctx *ctx_, float *params, size_t n) {
  CtxBase *ctx = reinterpret_cast<CtxBase *>(ctx_);
  if (!ctx || !params || n != (size_t)MYQL_CV_PARAMS) return set_error(MYQL_ERR_INVALID_ARG, "need MYQL_CV_PARAMS floats");
  CvState &S = state(ctx);
  if (!S.init) return set_error(MYQL_ERR_INVALID_ARG, "no control-variate network in this context");
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e == cudaSuccess) e = cudaMemcpyAsync(params, S.params.p, kPCount * 4, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  return cuda_status(e, "control-variate parameters");
}

myql_status myql_cv_init(myql_ctx *ctx_, uint64_t seed) {
  CtxBase *ctx = reinterpret_cast<CtxBase *>(ctx_);
  if (!ctx) return set_error(MYQL_ERR_INVALID_ARG, "null context");
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) return cuda_status(e, "cudaSetDevice");
  std::vector<float> p;
  init_params(p, seed);
  return upload_params(ctx, state(ctx), p.data());
}

myql_status myql_cv_forward(myql_ctx *ctx_, const float *feats, const float *dM, uint64_t n_paths,
                            uint32_t n_hedge, float *cv, float *g) {
  CtxBase *ctx = reinterpret_cast<CtxBase *>(ctx_);
  if (!ctx || !feats || !dM || !cv || n_paths == 0 || n_hedge == 0 || n_paths * n_hedge > (1ull << 26))
    return set_error(MYQL_ERR_INVALID_ARG, "bad control-variate forward arguments");
  CvState &S = state(ctx);
  if (!S.init) return set_error(MYQL_ERR_INVALID_ARG, "no control-variate network in this context");
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) return cuda_status(e, "cudaSetDevice");
  std::vector<uint8_t> img;
  std::vector<float> dm;
  pack_rows(feats, dM, n_paths, n_hedge, img, dm);
  const uint64_t pbs = (n_paths + 127) / 128;
  e = S.feat.ensure(img.size());
  if (e == cudaSuccess) e = S.dM.ensure(dm.size() * 4);
  if (e == cudaSuccess) e = S.cv.ensure(pbs * 128 * 4);
  if (e == cudaSuccess) e = S.Y.ensure(dm.size() * 4);  // per-row g
  if (e == cudaSuccess) e = ctx->status.ensure(16);
  if (e == cudaSuccess) e = cudaMemsetAsync(ctx->status.p, 0, 16, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(S.feat.p, img.data(), img.size(), cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(S.dM.p, dm.data(), dm.size() * 4, cudaMemcpyHostToDevice, ctx->stream);
  if (e != cudaSuccess) return cuda_status(e, "control-variate forward buffers");
  myql_status s = forward(ctx, S, (const uint8_t *)S.feat.p, (const float *)S.dM.p, n_paths, n_hedge,
                          (float *)S.cv.p, (float *)S.Y.p);
  if (s != MYQL_OK) return s;
  std::vector<float> gr(dm.size());
  e = cudaMemcpyAsync(cv, S.cv.p, n_paths * 4, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(gr.data(), S.Y.p, gr.size() * 4, cudaMemcpyDeviceToHost, ctx->stream);
  if (e != cudaSuccess) return cuda_status(e, "control-variate forward results");
  s = wait_status(ctx);
  if (s != MYQL_OK) return s;
  if (g)
    for (uint64_t p = 0; p < n_paths; ++p)
      for (uint32_t j = 0; j < n_hedge; ++j) g[p * n_hedge + j] = gr[((p / 128) * n_hedge + j) * 128 + p % 128];
  return MYQL_OK;
}

myql_status myql_cv_gradient(myql_ctx *ctx_, const float *feats, const float *dM, const float *Y, uint64_t n_paths,
                             uint32_t n_hedge, float *grad, double *loss) {
  CtxBase *ctx = reinterpret_cast<CtxBase *>(ctx_);
  if (!ctx || !feats || !dM || !Y || !grad || n_paths == 0 || n_hedge == 0 || n_paths * n_hedge > (1ull << 26))
    return set_error(MYQL_ERR_INVALID_ARG, "bad control-variate gradient arguments");
  CvState &S = state(ctx);
  if (!S.init) return set_error(MYQL_ERR_INVALID_ARG, "no control-variate network in this context");
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) return cuda_status(e, "cudaSetDevice");
  std::vector<uint8_t> img;
  std::vector<float> dm;
  pack_rows(feats, dM, n_paths, n_hedge, img, dm);
  const uint64_t pbs = (n_paths + 127) / 128;
  e = S.feat.ensure(img.size());
  if (e == cudaSuccess) e = S.dM.ensure(dm.size() * 4);
  if (e == cudaSuccess) e = S.cv.ensure(pbs * 128 * 4);
  if (e == cudaSuccess) e = S.Y.ensure(pbs * 128 * 4);
  if (e == cudaSuccess) e = S.coef.ensure(pbs * 128 * 4);
  if (e == cudaSuccess) e = ctx->status.ensure(16);
  if (e == cudaSuccess) e = cudaMemsetAsync(ctx->status.p, 0, 16, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(S.feat.p, img.data(), img.size(), cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(S.dM.p, dm.data(), dm.size() * 4, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(S.Y.p, Y, n_paths * 4, cudaMemcpyHostToDevice, ctx->stream);
  if (e != cudaSuccess) return cuda_status(e, "control-variate gradient buffers");
  myql_status s = forward(ctx, S, (const uint8_t *)S.feat.p, (const float *)S.dM.p, n_paths, n_hedge,
                          (float *)S.cv.p, nullptr);
  if (s != MYQL_OK) return s;
  e = launch_cv_resid((const float *)S.Y.p, (const float *)S.cv.p, n_paths, (float *)S.coef.p, (double *)S.loss.p,
                      (double *)S.rpart.p, ctx->stream);
  if (e != cudaSuccess) return cuda_status(e, "cv_resid launch");
  s = backward(ctx, S, (const uint8_t *)S.feat.p, (const float *)S.dM.p, n_paths, n_hedge);
  if (s != MYQL_OK) return s;
  double lp[kResidBlocks];
  e = cudaMemcpyAsync(grad, S.grad.p, kPCount * 4, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(lp, S.loss.p, sizeof lp, cudaMemcpyDeviceToHost, ctx->stream);
  if (e != cudaSuccess) return cuda_status(e, "control-variate gradient results");
  s = wait_status(ctx);
  if (s == MYQL_OK && loss) {
    double t = 0.0;
    for (unsigned int b = 0; b < kResidBlocks; ++b) t += lp[b];
    *loss = t;
  }
  return s;
}

myql_status myql_cv_train(myql_ctx *ctx_, const myql_mc_job *job, const myql_cv_config *cfg, myql_cv_result *res) {
  CtxBase *ctx = reinterpret_cast<CtxBase *>(ctx_);
  if (!ctx || !job) return set_error(MYQL_ERR_INVALID_ARG, "null argument");
  myql_status s = check_job(*job);
  if (s == MYQL_OK) s = check_cfg(cfg);
  if (s != MYQL_OK) return s;
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) return cuda_status(e, "cudaSetDevice");
  const auto t0 = std::chrono::steady_clock::now();
  CvState &S = state(ctx);
  std::vector<float> p0;
  init_params(p0, cfg->seed);
  s = upload_params(ctx, S, p0.data());
  if (s != MYQL_OK) return s;
  Plan pl;
  CvSimParams C;
  int klass = 0;
  s = cv_plan(ctx, *job, *cfg, pl, C, klass);
  if (s != MYQL_OK) return s;
  const uint32_t nh = (uint32_t)C.n_hedge;
  const uint64_t P = std::max<uint64_t>(128, (cfg->pilot_paths + 127) / 128 * 128);
  const uint64_t Sp = std::min<uint64_t>(kDefaultStreams, P);
  if (P * nh > (1ull << 31)) return set_error(MYQL_ERR_TOO_LARGE, "pilot paths x hedge times above 2^31");
  // pilot paths on an independent seed, one chunk
  const uint64_t pilot_seed = job->config.seed ^ 0x6A09E667F3BCC909ull;
  s = simulate_chunks(ctx, C, klass, pilot_seed, 0, P, Sp, (P + Sp - 1) / Sp * Sp, S.p_feat, S.p_dM, S.p_Y,
                      [](uint64_t) { return MYQL_OK; });
  if (s != MYQL_OK) return s;
  // start from the best constant hedge: b4 = Cov(Y, S) / Var(S), S = sum_j dM_j
  {
    double m5[5] = {0, 0, 0, 0, 0};
    e = cudaMemsetAsync(S.sums.p, 0, 40, ctx->stream);
    if (e == cudaSuccess)
      e = launch_cv_beta((const float *)S.p_Y.p, (const float *)S.p_dM.p, P, nh, (double *)S.sums.p,
                         (double *)S.fpart.p, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(m5, S.sums.p, 40, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_status(e, "control-variate constant hedge");
    const double n = (double)P, ms = m5[0] / n, my = m5[3] / n;
    const double var_s = m5[1] / n - ms * ms, cov = m5[2] / n - my * ms;
    p0[kPB4] = var_s > 0.0 ? (float)(cov / var_s) : 0.0f;
    s = upload_params(ctx, S, p0.data());
    if (s != MYQL_OK) return s;
  }
  const uint64_t bp = std::min<uint64_t>(P, (cfg->batch_paths + 127) / 128 * 128);
  const uint64_t n_pb = P / 128, b_pb = bp / 128;
  e = S.p_cv.ensure(P * 4);
  if (e == cudaSuccess) e = S.coef.ensure(P * 4);
  if (e != cudaSuccess) return cuda_status(e, "control-variate training buffers");
  double *loss = (double *)S.loss.p;
  const uint32_t iters = cfg->iterations;
  const auto t_train = std::chrono::steady_clock::now();
  // One Adam step: forward, residuals, backward, Adam, re-pack (7 to 8 launches).  The
  // minibatch offsets, the cosine learning rate and the bias corrections depend on the
  // step index alone (adam_t restarts at 0 with every training).
  auto adam_loop = [&]() -> myql_status {
    for (uint32_t it = 0; it < iters; ++it) {
      const uint64_t b0 = (it * b_pb) % n_pb;
      const uint64_t nb = std::min(b_pb, n_pb - b0);
      const uint8_t *f = (const uint8_t *)S.p_feat.p + b0 * nh * kCvTileBytes;
      const float *dm = (const float *)S.p_dM.p + b0 * nh * 128;
      const float *Y = (const float *)S.p_Y.p + b0 * 128;
      float *cvb = (float *)S.p_cv.p + b0 * 128;
      myql_status s2 = forward(ctx, S, f, dm, nb * 128, nh, cvb, nullptr);
      if (s2 != MYQL_OK) return s2;
      cudaError_t e2 = launch_cv_resid(Y, cvb, nb * 128, (float *)S.coef.p, loss + (size_t)it * kResidBlocks,
                                       (double *)S.rpart.p, ctx->stream);
      if (e2 != cudaSuccess) return cuda_status(e2, "cv_resid launch");
      s2 = backward(ctx, S, f, dm, nb * 128, nh);
      if (s2 != MYQL_OK) return s2;
      const double pi = 3.14159265358979323846;
      const double lr = cfg->learning_rate * (0.05 + 0.95 * 0.5 * (1.0 + std::cos(pi * it / std::max(1u, iters))));
      const double t = (double)(it + 1);
      e2 = launch_cv_adam((float *)S.params.p, (float *)S.adam_m.p, (float *)S.adam_v.p, (const float *)S.grad.p,
                          (float)lr, (float)(1.0 - std::pow(0.9, t)), (float)(1.0 - std::pow(0.999, t)), ctx->stream);
      if (e2 == cudaSuccess)
        e2 = launch_cv_pack((const float *)S.params.p, (uint8_t *)S.img.p, (float *)S.vec.p, ctx->stream);
      if (e2 != cudaSuccess) return cuda_status(e2, "cv_adam launch");
      ctx->launches += 3;
    }
    return MYQL_OK;
  };
  // The loop runs as one CUDA graph, captured on the first training of a shape (pilot
  // paths, minibatch, hedge times, step count, learning rate, buffers) and replayed by the
  // next training of the same shape: 7-8 launches per step become one graph launch.  Every
  // buffer the loop touches is allocated, and the kernels' attributes set, before capture.
  uint64_t key = 0xcbf29ce484222325ull;
  auto mixk = [&](uint64_t v) { key = (key ^ v) * 0x100000001b3ull + (key >> 29); };
  uint64_t lr_bits;
  std::memcpy(&lr_bits, &cfg->learning_rate, 8);
  for (uint64_t v : {P, (uint64_t)nh, bp, (uint64_t)iters, lr_bits})
    mixk(v);
  if (iters) {
    // tile-major forward (fewer than 8 path blocks per SM): its row buffer at the largest such minibatch
    const uint64_t tm_pb = std::min<uint64_t>(b_pb, (uint64_t)ctx->sm_count * 8 - 1);
    e = S.gdm.ensure(tm_pb * nh * 128 * 4);
    if (e == cudaSuccess) e = S.gpart.ensure((size_t)mlp_blocks(ctx, b_pb * nh) * kPCount * 4);
    if (e == cudaSuccess) e = cv_prepare_kernels();
    if (e != cudaSuccess) return cuda_status(e, "control-variate training set-up");
  }
  for (const DevBuf *b : {&S.p_feat, &S.p_dM, &S.p_Y, &S.p_cv, &S.coef, &S.loss, &S.params, &S.adam_m, &S.adam_v,
                          &S.grad, &S.img, &S.vec, &S.gdm, &S.gpart, &S.rpart, &ctx->status})
    mixk((uint64_t)(uintptr_t)b->p);
  if (iters && (!S.train_graph || S.train_key != key)) {
    if (S.train_graph) cudaGraphExecDestroy(S.train_graph);
    S.train_graph = nullptr;
    const uint32_t l0 = ctx->launches;
    cudaGraph_t gr = nullptr;
    e = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return cuda_status(e, "control-variate training capture");
    s = adam_loop();
    cudaError_t e2 = cudaStreamEndCapture(ctx->stream, &gr);
    if (s != MYQL_OK) {
      if (gr) cudaGraphDestroy(gr);
      return s;
    }
    e = e2;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&S.train_graph, gr, 0);
    if (gr) cudaGraphDestroy(gr);
    if (e != cudaSuccess) {
      S.train_graph = nullptr;
      return cuda_status(e, "control-variate training graph");
    }
    S.train_key = key;
    S.train_launches = ctx->launches - l0;
    ctx->launches = l0;
  }
  if (iters) {
    e = cudaGraphLaunch(S.train_graph, ctx->stream);
    if (e != cudaSuccess) return cuda_status(e, "control-variate training graph launch");
    ctx->launches += S.train_launches;
    S.adam_t = iters;
  }
  // in-sample variance before / after, on the first min(P, 2^17) pilot paths (a diagnostic:
  // the out-of-sample ratio of myql_cv_price is the one that counts)
  const uint64_t Pe = std::min<uint64_t>(P, kCvInSamplePaths);
  s = forward(ctx, S, (const uint8_t *)S.p_feat.p, (const float *)S.p_dM.p, Pe, nh, (float *)S.p_cv.p, nullptr);
  if (s != MYQL_OK) return s;
  e = cudaMemsetAsync(S.sums.p, 0, 32, ctx->stream);
  if (e == cudaSuccess) e = launch_cv_reduce((const float *)S.p_Y.p, (const float *)S.p_cv.p, Pe, (double *)S.sums.p,
                                                  (double *)S.fpart.p, ctx->stream);
  double sums[4] = {0, 0, 0, 0};
  std::vector<double> lparts((size_t)std::max(1u, iters) * kResidBlocks, 0.0);
  if (e == cudaSuccess) e = cudaMemcpyAsync(sums, S.sums.p, 32, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess && iters)
    e = cudaMemcpyAsync(lparts.data(), loss, (size_t)iters * kResidBlocks * 8, cudaMemcpyDeviceToHost, ctx->stream);
  if (e != cudaSuccess) return cuda_status(e, "control-variate training results");
  s = wait_status(ctx);
  if (s != MYQL_OK) return s;
  if (res) {
    std::memset(res, 0, sizeof *res);
    const double n = (double)Pe;
    const double my = sums[0] / n, vy = std::max(sums[1] / n - my * my, 0.0);
    const double mz = sums[2] / n, vz = std::max(sums[3] / n - mz * mz, 0.0);
    res->plain_price = my;
    res->plain_std_err = std::sqrt(vy / n);
    res->price = mz;
    res->price_std_err = std::sqrt(vz / n);
    res->variance_ratio = vz > 0.0 ? vy / vz : 0.0;
    auto loss_of = [&](uint32_t it) {  // the step's block partials, in order
      double t = 0.0;
      for (unsigned int b = 0; b < kResidBlocks; ++b) t += lparts[(size_t)it * kResidBlocks + b];
      return t;
    };
    res->initial_loss = iters ? loss_of(0) : 0.0;
    res->final_loss = iters ? loss_of(iters - 1) : 0.0;
    res->paths = P;
    res->train_ms = ms_since(t_train);
    res->total_ms = ms_since(t0);
    res->kernel_launches = ctx->launches;
  }
  return MYQL_OK;
}

myql_status myql_cv_price(myql_ctx *ctx_, const myql_mc_job *job, const myql_cv_config *cfg, myql_cv_result *res) {
  CtxBase *ctx = reinterpret_cast<CtxBase *>(ctx_);
  if (!ctx || !job || !res) return set_error(MYQL_ERR_INVALID_ARG, "null argument");
  myql_status s = check_job(*job);
  if (s == MYQL_OK) s = check_cfg(cfg);
  if (s != MYQL_OK) return s;
  CvState &S = state(ctx);
  if (!S.init) return set_error(MYQL_ERR_INVALID_ARG, "train the control variate first (myql_cv_train)");
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) return cuda_status(e, "cudaSetDevice");
  const auto t0 = std::chrono::steady_clock::now();
  ctx->launches = 0;
  Plan pl;
  CvSimParams C;
  int klass = 0;
  s = cv_plan(ctx, *job, *cfg, pl, C, klass);
  if (s != MYQL_OK) return s;
  const uint32_t nh = (uint32_t)C.n_hedge;
  const uint64_t M = pl.M, Sn = pl.S;
  // chunk: a multiple of the stream count with at most ~4 GiB of features
  uint64_t chunk = (4ull << 30) / ((uint64_t)nh * (kCvTileBytes / 128 + 4));
  chunk = std::max<uint64_t>(Sn, chunk / Sn * Sn);
  chunk = std::min<uint64_t>(chunk, (M + Sn - 1) / Sn * Sn);
  e = S.cv.ensure((chunk + 127) / 128 * 128 * 4);
  if (e == cudaSuccess) e = cudaMemsetAsync(S.sums.p, 0, 32, ctx->stream);
  if (e != cudaSuccess) return cuda_status(e, "control-variate pricing buffers");
  ctx->phase_reset();
  cudaEvent_t ev[3];
  for (int i = 0; i < 3; ++i) ev[i] = ctx->phase_event();
  float sim_ms = 0.0f, mlp_ms = 0.0f;
  e = cudaEventRecord(ev[0], ctx->stream);
  if (e != cudaSuccess) return cuda_status(e, "event");
  // per chunk: [ev0] simulate [ev1] forward [ev2] reduce
  s = simulate_chunks(ctx, C, klass, job->config.seed, job->config.stream_offset, M, Sn, chunk, S.feat, S.dM, S.Y,
                      [&](uint64_t n) -> myql_status {
                        cudaError_t e2 = cudaEventRecord(ev[1], ctx->stream);
                        myql_status s2 = forward(ctx, S, (const uint8_t *)S.feat.p, (const float *)S.dM.p, n, nh,
                                                 (float *)S.cv.p, nullptr);
                        if (s2 != MYQL_OK) return s2;
                        if (e2 == cudaSuccess) e2 = cudaEventRecord(ev[2], ctx->stream);
                        if (e2 == cudaSuccess)
                          e2 = launch_cv_reduce((const float *)S.Y.p, (const float *)S.cv.p, n, (double *)S.sums.p,
                                                (double *)S.fpart.p, ctx->stream);
                        ctx->launches++;
                        if (e2 == cudaSuccess) e2 = cudaEventSynchronize(ev[2]);
                        float a = 0.0f, b = 0.0f;
                        if (e2 == cudaSuccess) e2 = cudaEventElapsedTime(&a, ev[0], ev[1]);
                        if (e2 == cudaSuccess) e2 = cudaEventElapsedTime(&b, ev[1], ev[2]);
                        sim_ms += a;
                        mlp_ms += b;
                        if (e2 == cudaSuccess) e2 = cudaEventRecord(ev[0], ctx->stream);
                        return cuda_status(e2, "control-variate chunk");
                      });
  if (s != MYQL_OK) return s;
  double sums[4] = {0, 0, 0, 0};
  e = cudaMemcpyAsync(sums, S.sums.p, 32, cudaMemcpyDeviceToHost, ctx->stream);
  if (e != cudaSuccess) return cuda_status(e, "control-variate sums");
  s = wait_status(ctx);
  if (s != MYQL_OK) return s;
  std::memset(res, 0, sizeof *res);
  const double n = (double)M;
  const double my = sums[0] / n, vy = std::max(sums[1] / n - my * my, 0.0);
  const double mz = sums[2] / n, vz = std::max(sums[3] / n - mz * mz, 0.0);
  res->plain_price = my;
  res->plain_std_err = std::sqrt(vy / n);
  res->price = mz;
  res->price_std_err = std::sqrt(vz / n);
  res->variance_ratio = vz > 0.0 ? vy / vz : 0.0;
  res->paths = M;
  res->simulate_ms = sim_ms;
  res->mlp_ms = mlp_ms;
  res->total_ms = ms_since(t0);
  res->kernel_launches = ctx->launches;
  return MYQL_OK;
}

// The trained control variate on randomized QMC paths (myql_qmc_price's Sobol points,
// bridges and digital shifts): R replicates of the control-variate estimator, each the mean
// of Y - C over its points, with the standard error from their spread.  Y - C stays unbiased
// under the digitally shifted points, whose every point is uniform on the unit cube.
myql_status myql_cv_qmc_price(myql_ctx *ctx_, const myql_mc_job *job, const myql_cv_config *cfg,
                              uint32_t n_replicates, myql_cv_result *res) {
  CtxBase *ctx = reinterpret_cast<CtxBase *>(ctx_);
  if (!ctx || !job || !res) return set_error(MYQL_ERR_INVALID_ARG, "null argument");
  myql_status s = check_job(*job);
  if (s == MYQL_OK) s = check_cfg(cfg);
  if (s != MYQL_OK) return s;
  CvState &S = state(ctx);
  if (!S.init) return set_error(MYQL_ERR_INVALID_ARG, "train the control variate first (myql_cv_train)");
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) return cuda_status(e, "cudaSetDevice");
  const auto t0 = std::chrono::steady_clock::now();
  ctx->launches = 0;
  Plan pl;
  CvSimParams C;
  int klass = 0;
  s = cv_plan(ctx, *job, *cfg, pl, C, klass);
  if (s != MYQL_OK) return s;
  const uint64_t M = job->config.num_paths, R = n_replicates;
  QmcCvParams Q;
  std::memset(&Q, 0, sizeof Q);
  s = qmc_prepare(ctx, *job, pl, R, Q.Q);
  if (s != MYQL_OK) return s;
  Q.Q.P.status = C.sim.status;
  Q.pay = C.pay;
  Q.df = C.df;
  Q.hedge_every = C.hedge_every;
  Q.n_hedge = C.n_hedge;
  Q.fc = C.fc;
  const uint32_t nh = (uint32_t)C.n_hedge;
  const uint64_t n_pts = M / R;
  // chunk: whole 2048-point blocks with at most ~4 GiB of features
  uint64_t chunk = (4ull << 30) / ((uint64_t)nh * (kCvTileBytes / 128 + 4));
  chunk = std::min<uint64_t>(std::max<uint64_t>(chunk / 2048 * 2048, 2048), M);
  const uint64_t pbs = chunk / 128;
  e = S.feat.ensure(pbs * nh * kCvTileBytes);
  if (e == cudaSuccess) e = S.dM.ensure(pbs * nh * 128 * 4);
  if (e == cudaSuccess) e = S.Y.ensure(chunk * 4);
  if (e == cudaSuccess) e = S.cv.ensure(chunk * 4);
  if (e == cudaSuccess) e = S.sums.ensure(R * 4 * sizeof(double));
  if (e == cudaSuccess) e = cudaMemsetAsync(S.sums.p, 0, R * 4 * sizeof(double), ctx->stream);
  if (e != cudaSuccess) return cuda_status(e, "control-variate QMC buffers");
  Q.feat = (uint8_t *)S.feat.p;
  Q.dM = (float *)S.dM.p;
  Q.Y = (float *)S.Y.p;
  ctx->phase_reset();
  cudaEvent_t ev[3];
  for (int i = 0; i < 3; ++i) ev[i] = ctx->phase_event();
  float sim_ms = 0.0f, mlp_ms = 0.0f;
  for (uint64_t b = 0; b < M; b += chunk) {
    const uint64_t n = std::min(chunk, M - b);  // a multiple of 2048, as are b and n_pts
    Q.path_begin = b;
    e = cudaEventRecord(ev[0], ctx->stream);
    if (e == cudaSuccess) e = launch_qmc_cv(Q, n, pl.nf, ctx->stream);
    if (e != cudaSuccess) return cuda_status(e, "qmc_cv launch");
    ctx->launches++;
    e = cudaEventRecord(ev[1], ctx->stream);
    if (e != cudaSuccess) return cuda_status(e, "event");
    s = forward(ctx, S, (const uint8_t *)S.feat.p, (const float *)S.dM.p, n, nh, (float *)S.cv.p, nullptr);
    if (s != MYQL_OK) return s;
    e = cudaEventRecord(ev[2], ctx->stream);
    // the chunk's share of each replicate, into that replicate's sums
    for (uint64_t r = b / n_pts; e == cudaSuccess && r * n_pts < b + n; ++r) {
      const uint64_t lo = std::max(b, r * n_pts), hi = std::min(b + n, (r + 1) * n_pts);
      e = launch_cv_reduce((const float *)S.Y.p + (lo - b), (const float *)S.cv.p + (lo - b), hi - lo,
                           (double *)S.sums.p + 4 * r, (double *)S.fpart.p, ctx->stream);
      ctx->launches += 2;
    }
    if (e == cudaSuccess) e = cudaEventSynchronize(ev[2]);
    float a = 0.0f, c = 0.0f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&a, ev[0], ev[1]);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&c, ev[1], ev[2]);
    if (e != cudaSuccess) return cuda_status(e, "control-variate QMC chunk");
    sim_ms += a;
    mlp_ms += c;
  }
  std::vector<double> sums(R * 4);
  e = cudaMemcpyAsync(sums.data(), S.sums.p, sums.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
  if (e != cudaSuccess) return cuda_status(e, "control-variate QMC sums");
  s = wait_status(ctx);
  if (s != MYQL_OK) return s;
  // replicate estimates of the plain and the control-variate estimator
  double sy = 0.0, syy = 0.0, sz = 0.0, szz = 0.0;
  for (uint64_t r = 0; r < R; ++r) {
    const double y = sums[4 * r] / (double)n_pts, z = sums[4 * r + 2] / (double)n_pts;
    sy += y;
    syy += y * y;
    sz += z;
    szz += z * z;
  }
  const double Rd = (double)R;
  const double my = sy / Rd, mz = sz / Rd;
  const double vy = std::max(syy / Rd - my * my, 0.0) * Rd / (Rd - 1.0);
  const double vz = std::max(szz / Rd - mz * mz, 0.0) * Rd / (Rd - 1.0);
  std::memset(res, 0, sizeof *res);
  res->plain_price = my;
  res->plain_std_err = std::sqrt(vy / Rd);
  res->price = mz;
  res->price_std_err = std::sqrt(vz / Rd);
  res->variance_ratio = vz > 0.0 ? vy / vz : 0.0;
  res->paths = M;
  res->simulate_ms = sim_ms;
  res->mlp_ms = mlp_ms;
  res->total_ms = ms_since(t0);
  res->kernel_launches = ctx->launches;
  return MYQL_OK;
}

}  // extern "C"
