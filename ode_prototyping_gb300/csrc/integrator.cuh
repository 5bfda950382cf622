// integrator.cuh -- device-resident adaptive embedded RK integrator state.
#pragma once

#include "force.cuh"

namespace gb {

// Controller state of one system, resident in device memory.  Written only
// by the last CTA of the final-stage kernel of an attempt (and by the start
// kernels); every kernel reads it once at entry.
struct Ctrl {
  double t, dt, t0, tf;
  double err;         // last scaled error norm
  double err_prev;    // PI memory: last accepted error (>= 1e-4)
  double safety;      // 0.38^(1/(1+q)) (RKEmbeddedParallel.hpp:24)
  double dt_initial;
  double pi_alpha, pi_beta;
  double max_abs_acc; // max |a| over bodies at the last attempt's final stage
  double min_r2;      // min pair separation^2 seen in the last first stage (learned features)
  double dt_hist[3];  // last three attempted step sizes
  double err_hist[3]; // last three error norms
  double learned_dt;  // last learned proposal
  double log_tol;     // log max(atol, rtol) for scalar tolerances, 0 for vector ones
                      // (the learned proposer's tolerance feature)
  // Logs the learned controller reuses from attempt to attempt (lg_valid):
  // each is the same log call on the same argument as the value it stands
  // for, so features and proposals keep their bits while the one controller
  // thread evaluates far fewer FP64 logs per attempt.
  double lg_dt[3];    // log fmax(dt_hist[k], 1e-300)
  double lg_err[3];   // log fmax(err_hist[k], 1e-30)
  double lg_err_prev; // log fmax(err_prev, 1e-30)
  double lg_safety;   // log safety
  double lg_n;        // log N
  int lg_valid;
  long long n_accepted, n_rejected, n_attempts, n_rhs, n_rhs_saved;
  long long max_attempts;
  long long n_learned, n_learned_rejected;
  long long log_count;
  int cur;            // ring slot holding x0
  int done;
  int status;
  int k0_valid;       // the k slot k0slot holds f(x0)
  int k0slot;         // physical k slot of stage 0: 0 or S-1
  int px;             // packed slot of x0 (mixed)
  int reject_prev;
  int controller;
  int fsal;
  int q;
  int last_accepted;
  int learned_active; // the current attempt uses a learned proposal
  int exact_pow;      // step-size formulas with the correctly rounded pow
  // dense output (DOPRI5): output times [dense_lo, dense_hi) fall in the
  // step just accepted; its first / last stage derivatives are in these slots
  long long dense_next, dense_lo, dense_hi;
  int dense_k0, dense_klast;
  unsigned ticket;
  unsigned ticket2;
};

// Log record of one attempt (learned-controller training data).
struct StepLog {
  float feat[16];
  float log_dt;       // log of the attempted step
  float log_err;      // log of the resulting scaled error
  float accepted;
  float log_dt_ideal; // log of the step the I-controller formula proposes
};

// most partner chunks per i-tile in the split stage kernel
constexpr int kMaxChunks = 32;

struct FusedParams {
  Ctrl* ctrl;
  double* ring;        // R * n_var states; x0 = ring + cur * n_var
  double* times_ring;  // R times
  double* ks;          // S * n_var stage derivatives
  double* Y;           // 2 * n_var stage states
  PackedBody* PX;      // 2 * n packed (x0 / x_new), mixed only
  PackedBody* PY;      // 2 * n packed stage positions, mixed only
  const double* atol;  // n_var or null (scalar)
  const double* rtol;
  double atol_s, rtol_s;
  const double* masses;
  double mass;
  double eps2;
  float eps2f;
  int R;
  const double* cref;  // reference point for hi/lo packing
  double* partials;    // n_parts: per (i-tile, cluster rank) scaled-square sums
  double* sq;          // n_var (exact mode)
  double* aux;         // n_parts (max |a| partials)
  StepLog* log;        // log_capacity records or null
  long long log_capacity;
  const void* mlp;     // device MLP weights (learned controller) or null
  long long n, n_var, n_itiles, n_parts;
  int exact;
  int f64_fast;        // FP64 stages: refined-rsqrt pair term (not exact mode)
  int S;
  // partner-chunk split without clusters (packed mixed path)
  int n_chunks;          // partner chunks per i-tile
  double* chunk_sums;    // n_itiles * n_chunks * 3 * bodies per tile, 8 bytes each
  unsigned* tile_count;  // n_itiles arrival counts, zero between launches
  double* pre;           // n_var: velocity elements' sums over the earlier stages
  float4* BX;            // 2 * n_itiles boxes of the packed x0 / x_new tiles (split stage)
  float4* BY;            // 2 * n_itiles boxes of the packed stage-state tiles
  int cull;              // split stage: far half tiles skip the close-pair test
  long long chunk_start[kMaxChunks + 1];  // partner range of chunk c: [start[c], start[c+1])
  // spatially sorted mixed path
  const int* perm;       // sorted position -> body (spatially sorted and split paths)
  float4* PXF;           // 2 * n far records (x0 / x_new)
  float4* PYF;           // 2 * n far records (stage states)
  TileMeta* MX;          // 2 * n_itiles tile metadata (x0 / x_new)
  TileMeta* MY;          // 2 * n_itiles (stage states)
  // dense output
  const double* dense_t; // n_dense output times (ascending), or null
  long long n_dense;
  double* dense_out;     // n_dense * n_var
};

}  // namespace gb
