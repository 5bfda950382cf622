// controller.cuh -- step-size controllers run by one device thread at the end
// of every attempt (no host round trip).
#pragma once

#include "integrator.cuh"

namespace gb {

constexpr double kMaxStepScale = 6.0;   // RKEmbeddedParallel.hpp:21
constexpr double kMinStepScale = 0.33;  // RKEmbeddedParallel.hpp:22

// The reference's elementary controller (RKEmbeddedParallel.hpp:65-74):
// dtnew = dt * safety / err^(1/(1+q)), clamped to x6 / x0.33, with a floor
// at (tf - t0) * 1e-12 reached only inside the clamp window.
__device__ __forceinline__ double reference_step(double dt, double err, double safety, int q,
                                                 double t0, double tf) {
  const double dtnew = dt * safety / pow(err, 1.0 / (1.0 + q));
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

}  // namespace gb
