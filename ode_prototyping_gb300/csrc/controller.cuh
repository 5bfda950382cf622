// controller.cuh -- step-size controllers run by one device thread at the end
// of every attempt (no host round trip).
#pragma once

#include "ddpow.cuh"
#include "integrator.cuh"
#include "mlp.cuh"

namespace gb {

constexpr double kMaxStepScale = 6.0;   // RKEmbeddedParallel.hpp:21
constexpr double kMinStepScale = 0.33;  // RKEmbeddedParallel.hpp:22
// The learned proposal is a correction of at most this log factor (x3 either
// way) to the PI controller's log step ratio.  Without the bound, a proposer
// fed states outside its training distribution can keep shrinking steps that
// the error estimate keeps accepting (measured: a configuration-3 batch ran
// into its attempt budget), since acceptance only guards against steps that
// are too long.
constexpr double kLearnedMaxLogCorrection = 1.0986122886681098;  // log(3)

// The reference's elementary controller (RKEmbeddedParallel.hpp:65-74):
// dtnew = dt * safety / err^(1/(1+q)), clamped to x6 / x0.33, with a floor
// at (tf - t0) * 1e-12 reached only inside the clamp window.
__device__ __forceinline__ double reference_step(double dt, double err, double safety, int q,
                                                 double t0, double tf, bool exact_pow) {
  const double e = 1.0 / (1.0 + q);
  const double dtnew = dt * safety / (exact_pow ? dd_pow(err, e) : pow(err, e));
  if (fabs(dtnew) > kMaxStepScale * fabs(dt)) return dt * kMaxStepScale;
  if (fabs(dtnew) < kMinStepScale * fabs(dt)) return dt * kMinStepScale;
  if (dtnew / (tf - t0) < 1.0e-12) return (tf - t0) * 1.0e-12;
  return dtnew;
}

// PI controller in the form of Hairer, Norsett & Wanner (and Numerical
// Recipes' StepperDopr5::Controller, NumericalRecipes/StepperDopr5.hpp:
// 236-272): scale = safety * err^-alpha * err_prev^beta with
// alpha = 1/(1+q) - 0.75 beta, clamped to the reference's [0.33, 6]; no
// increase directly after a rejection.
__device__ __forceinline__ double pi_step(Ctrl& c, double dt, double err, bool accepted) {
  double scale;
  if (accepted) {
    if (err == 0.0) {
      scale = kMaxStepScale;
    } else {
      scale = c.safety * pow(err, -c.pi_alpha) * pow(c.err_prev, c.pi_beta);
      scale = fmin(fmax(scale, kMinStepScale), kMaxStepScale);
    }
    if (c.reject_prev) scale = fmin(scale, 1.0);
    c.err_prev = fmax(err, 1.0e-4);
    c.reject_prev = 0;
  } else {
    scale = fmax(c.safety * pow(err, -c.pi_alpha), kMinStepScale);
    c.reject_prev = 1;
  }
  double dtn = dt * scale;
  if (dtn / (c.tf - c.t0) < 1.0e-12) dtn = (c.tf - c.t0) * 1.0e-12;
  return dtn;
}

// Per-system environment of the end-of-attempt decision.
struct CtrlEnv {
  StepLog* log;          // controller log (training data) or null
  long long log_capacity;
  double* times_ring;    // time of each ring slot, or null
  int R;                 // ring slots
  long long n;           // bodies
};

// Fills the learned controller's log caches from the histories (at start;
// other controllers leave them unused).
__device__ __forceinline__ void init_log_cache(Ctrl& c, long long n) {
  c.lg_valid = c.controller == GB_CTRL_LEARNED;
  if (!c.lg_valid) return;
  for (int k = 0; k < 3; ++k) {
    c.lg_dt[k] = log(fmax(c.dt_hist[k], 1e-300));
    c.lg_err[k] = log(fmax(c.err_hist[k], 1e-30));
  }
  c.lg_err_prev = log(fmax(c.err_prev, 1e-30));
  c.lg_safety = log(c.safety);
  c.lg_n = log((double)n);
}

// Shifts the step/error history as finish_attempt will (used to build the
// learned controller's features before the decision is applied).
__device__ __forceinline__ void preview_history(Ctrl& c, double err, bool accepted) {
  for (int k = 2; k > 0; --k) {
    c.dt_hist[k] = c.dt_hist[k - 1];
    c.err_hist[k] = c.err_hist[k - 1];
  }
  c.dt_hist[0] = c.dt;
  c.err_hist[0] = isfinite(err) ? err : 1e300;
  c.last_accepted = accepted ? 1 : 0;
  if (c.lg_valid) {
    for (int k = 2; k > 0; --k) {
      c.lg_dt[k] = c.lg_dt[k - 1];
      c.lg_err[k] = c.lg_err[k - 1];
    }
    c.lg_dt[0] = log(fmax(c.dt_hist[0], 1e-300));
    c.lg_err[0] = log(fmax(c.err_hist[0], 1e-30));
  }
}

// End-of-attempt decision by one thread: acceptance (err <= 1,
// RKEmbeddedParallel.hpp:58-62), step-size update (:65-74 or PI or learned),
// last-step clamp (:77-79) and the loop condition t < tf (:35).
__device__ inline void finish_attempt(const DevTableau& tab, const CtrlEnv& P, Ctrl& c,
                                      double err, double learned_log_scale, bool have_learned) {
  const double dt = c.dt;
  c.err = err;
  c.n_attempts += 1;
  const bool finite = isfinite(err);
  const bool accepted = finite && err <= 1.0;
  if (c.learned_active) {
    c.n_learned += 1;
    if (!accepted) c.n_learned_rejected += 1;
  }
  preview_history(c, err, accepted);
  // controller log (training data of the learned controller): the features
  // the controller sees after this attempt, and the attempt's outcome
  if (P.log && c.log_count < P.log_capacity) {
    StepLog& L = P.log[c.log_count];
    make_features(c, tab, P.n, L.feat);
    L.log_dt = (float)log(dt);
    L.log_err = (float)log(fmax(err, 1e-300));
    L.accepted = accepted ? 1.f : 0.f;
    double ideal = finite ? dt * c.safety / pow(fmax(err, 1e-300), 1.0 / (1.0 + c.q)) : dt * 0.33;
    L.log_dt_ideal = (float)log(ideal);
    c.log_count += 1;
  }
  if (!finite) {
    c.status = GB_ERR_NOT_FINITE;
    c.done = 1;
    return;
  }
  if (accepted) {
    // slots of this attempt's first and last stage derivatives (dense output)
    c.dense_k0 = c.k0slot;
    c.dense_klast = (c.k0slot == 0) ? tab.n_stages - 1 : 0;
    c.t += dt;
    c.cur = (c.cur + 1) % P.R;
    if (P.times_ring) P.times_ring[c.cur] = c.t;
    c.n_accepted += 1;
    c.px ^= 1;
    if (c.fsal) {
      c.k0slot = (c.k0slot == 0) ? tab.n_stages - 1 : 0;
      c.k0_valid = 1;
    } else {
      c.k0_valid = 0;
    }
  } else {
    c.n_rejected += 1;
    c.k0_valid = 1;  // x0 unchanged: f(x0) is still in its slot
  }
  double dtn;
  c.learned_active = 0;
  if (c.controller == GB_CTRL_PI) {
    dtn = pi_step(c, dt, err, accepted);
  } else if (c.controller == GB_CTRL_LEARNED) {
    if (accepted && have_learned) {
      // The network proposes a correction to the PI controller's log step
      // ratio log(safety) - alpha log(err) + beta log(err_prev) (a network
      // that has learned nothing reproduces PI); the embedded error
      // estimate of the next attempt still decides acceptance.
      // log(err) is the cached log fmax(err, 1e-30) when err >= 1e-30 (the
      // same value); log(err_prev) is the cached one (err_prev >= 1e-4)
      const double lerr = err >= 1e-30 ? c.lg_err[0] : log(err);
      const double base = err > 0.0 ? c.lg_safety - c.pi_alpha * lerr +
                                          c.pi_beta * c.lg_err_prev
                                    : log(kMaxStepScale);
      const double res = fmin(fmax(learned_log_scale, -kLearnedMaxLogCorrection),
                              kLearnedMaxLogCorrection);
      const double lg = fmin(fmax(base + res, log(kMinStepScale)),
                             log(kMaxStepScale));
      double scale = exp(lg);
      if (c.reject_prev) scale = fmin(scale, 1.0);
      dtn = dt * scale;
      c.learned_dt = dtn;
      c.learned_active = 1;
      // keep the PI memory current
      c.err_prev = fmax(err, 1.0e-4);
      c.lg_err_prev = err >= 1.0e-4 ? lerr : log(fmax(c.err_prev, 1e-30));
      c.reject_prev = 0;
    } else {
      dtn = pi_step(c, dt, err, accepted);  // fallback on every rejection
      if (accepted && c.lg_valid) c.lg_err_prev = log(fmax(c.err_prev, 1e-30));
    }
  } else {
    dtn = reference_step(dt, err, c.safety, c.q, c.t0, c.tf, c.exact_pow != 0);
  }
  c.dt = dtn;
  if (c.t + c.dt > c.tf) c.dt = c.tf - c.t;
  if (!(c.t < c.tf)) c.done = 1;
  if (!c.done && c.max_attempts > 0 && c.n_attempts >= c.max_attempts) {
    c.status = GB_ERR_BUDGET;
    c.done = 1;
  }
}

}  // namespace gb
