// engine_types.h -- launch-parameter structs shared by the host engine and the
// sm_103a kernels.  Everything here is plain data: the host fills it in FP64,
// rounds the per-step constants to FP32 and passes it by value (__grid_constant__).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace myql {

constexpr int kMaxScenarios = 9;   // base + v0 bumps (2 per factor) + T bumps + r bumps
constexpr int kMaxFields = 4;      // per-path terminal record fields
constexpr int kQ = 10;             // quantities (myql_quantity)
constexpr int kSimBlock = 128;     // threads per block of the path kernels
constexpr int kPayoffBlock = 128;  // threads per block of the payoff kernel
constexpr uint32_t kDefaultStreams = 131072u;
// Default xoshiro stream count of a request of M paths: min(M, clamp(M / 8, 2^17, 2^19)).
// Large requests get more streams (at most 8 paths each up to 2^22 paths), so the path
// kernels keep every SM full; the layout depends only on M, never on the GPU.
inline unsigned long long default_streams(unsigned long long M) {
  unsigned long long s = M / 8;
  s = s < 131072ull ? 131072ull : (s > 524288ull ? 524288ull : s);
  return s < M ? s : M;
}

// Scenario slots, in the order the reference simulates them for GreekMode::Full
// (MonteCarloPricer.hpp:302-410).
enum Scenario : int {
  SC_BASE = 0, SC_VUP0 = 1, SC_VDN0 = 2, SC_TUP = 3, SC_TDN = 4,
  SC_RUP = 5, SC_RDN = 6, SC_VUP1 = 7, SC_VDN1 = 8
};

enum Tracker : int {  // PathTrackers.hpp
  TRK_EUROPEAN = 0, TRK_GEO_ASIAN = 1, TRK_ARITH_ASIAN = 2,
  TRK_LOOKBACK = 3, TRK_BARRIER_UP = 4, TRK_BARRIER_DOWN = 5
};

inline __host__ __device__ int tracker_fields(int trk) {
  return trk == TRK_EUROPEAN ? 1 : trk == TRK_LOOKBACK ? 3 : (trk >= TRK_BARRIER_UP ? 4 : 2);
}

// One CIR factor of one scenario: the log-S coefficients of ASVJstepper.hpp:276-280
// and the scheme workspace of VolSchemes.hpp (prepare()).
struct FactorConst {
  float v0;
  float C0, C1, C2, C3;
  float w0, w1, w2;  // NV {ex, D*psi, s_star}; Exact {lambda_fac, alpha_base, scale}; NCI {lambda_fac, d, scale}
};

// SchemeNCI chi-squared table of one factor.  Rows depend only on d = 4 kappa theta / sigma^2,
// so one table serves every time step and every bumped scenario.
struct NciTable {
  const float4 *main;  // [rows][kNciGrid - 1] monomial cubic coefficients per cell (U grid)
  const float4 *tail;  // [rows][kNciTail - 1] cells on the w = -log(1-U) grid, U >= 0.999
  int rows;            // rows built (N < rows is looked up)
  float d;             // degrees of freedom offset
  float tail_w0, tail_inv_dw;
  unsigned long long pos_scale;  // floor(inv_dx * 2^50), fixed-point U -> cell position
};

constexpr int kNciGrid = 10000;  // VolSchemes.hpp:257
constexpr int kNciTail = 512;
constexpr double kNciUmax = 0.999;  // VolSchemes.hpp:258,342
constexpr double kNciTailWmax = 44.5;  // tail grid w = -log(1 - U) in [-log(1 - kNciUmax), 44.5]

struct ScenarioConst {
  FactorConst f[2];
  float gbm_drift, gbm_vol;   // 0-factor: per-step drift and vol (ASVJstepper.hpp:100-101)
  float dt;                   // step of this scenario
  float t_end;                // n_steps * dt (barrier clock end, informative)
  float jump_mean;            // Poisson mean of one jump window (dt or T)
  float jump_exp_neg_mean;    // exp(-jump_mean)
  float jump_comp;            // drift compensation of the window
  float x_shift;              // rho bumps of European instruments: log-spot shift (r' - r) T
                              // of a scenario derived from the base path, not simulated
  // The FP32 rounding of each constant's own FP32 rounding error (exact - (double)(float)
  // exact): factor 0's C0, C1, C2, C3, w0, w2, then jump_comp.  The precise lockstep kernel
  // adds them for the T-bumped scenarios, whose constants differ from each other by about
  // 2 t_bump / T relative: the difference then survives FP32 (myql_ctx_set_precise_theta).
  float lo[7];
  double jump_mean_d;         // jump_mean in FP64 (the precise kernel's T-bumped jump counts)
};

struct SimParams {
  int n_sc;            // simulated scenarios per path
  int n_factors;
  int jump_kind;       // myql_jump
  int tracker;         // Tracker
  int n_steps;
  int n_fields;
  uint32_t n_streams;
  uint32_t loop_cap;
  unsigned long long path_begin, path_end;  // paths [begin, end) of this launch
  unsigned long long num_paths;             // total paths of the job (record stride)
  unsigned long long rec_offset;            // first path held in `records`
  unsigned long long rec_stride;            // paths per (scenario, field) row of `records`
  float b_log[3];      // barrier levels in X = log(S/S0): base, up, dn
  float lb_min0, lb_max0;
  float merton_mu, merton_delta;
  float kou_p_up, kou_inv_eta1, kou_inv_eta2;
  NciTable nci[2];
  unsigned long long nci_u999;  // smallest 64-bit draw whose uniform is >= 0.999
  int lock_merge;               // lockstep kernel: v0-bumped variance paths merge into the base's
  int lock_precise;             // one-factor NCI lockstep: T-bumped scenarios add ScenarioConst::lo
  // exact-scheme small-alpha constants (VolSchemes.hpp:95-103), per factor
  float sm_p[2], sm_inv_p[2], sm_1mp[2], sm_1ma[2], sm_inv_a[2];
  unsigned long long *states;  // [4][n_streams] xoshiro states, updated in place
  float *records;              // [sc][field][rec_stride]
  unsigned int *status;        // [0] loop-cap hits, [1] table fallbacks
  ScenarioConst sc[kMaxScenarios];
};

// Payoff / Greek-combination pass over the terminal records.
struct PayoffParams {
  int n_sc, n_fields, tracker, kind, payoff, option_type, fixed_strike;
  int barrier_action, rebate_timing, mode, n_factors;
  int n_strikes;
  int smooth;                  // digital smoothing active (GreekMode != None, non-barrier)
  unsigned long long n_paths;  // paths in this pass
  unsigned long long rec_stride;
  unsigned long long tile0;    // global index of the first tile of this pass
  int tile_paths;
  const double *strikes;       // device
  const float *records;
  double *partials;            // [tile][strike][kQ][2]
  float S0, eps_rel;           // h / S0 (fd_bump)
  float smooth_eps;            // payoff eps
  float rebate, barrier_rate, T_instr;
  float avg_c0[kMaxScenarios], avg_c1[kMaxScenarios];  // Asian average = c0 + c1 * field1
  float inv_2h, inv_h2;
  float vega_c[2], vanna_c[2];
  float theta_c, charm_c, dfm1_tup, dfm1_tdn;  // discount factors minus one (FP64-rounded)
  float rho_c, dfm1_rup, dfm1_rdn;
};

struct FinalizeParams {
  int n_strikes;
  unsigned long long n_tiles;
  const double *partials;
  double *out;             // [2*kQ][n_strikes]
  double inv_m, df;
  int active_mask;         // bit q set = quantity q produced by the mode
};

}  // namespace myql
