// gb_internal.cuh -- shared device/host helpers of libgbode (not installed).
#pragma once

#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "gbode.h"

namespace gb {

namespace cg = cooperative_groups;

// Records the CUDA error and returns GB_ERR_CUDA from the enclosing function.
void note_cuda_error(cudaError_t e);
#define GB_CUDA_TRY(expr)                 \
  do {                                    \
    cudaError_t gb_e_ = (expr);           \
    if (gb_e_ != cudaSuccess) {           \
      ::gb::note_cuda_error(gb_e_);       \
      return GB_ERR_CUDA;                 \
    }                                     \
  } while (0)
#define GB_TRY(expr)          \
  do {                        \
    int gb_s_ = (expr);       \
    if (gb_s_ != GB_OK) {     \
      return gb_s_;           \
    }                         \
  } while (0)

inline cudaStream_t as_cuda(gb_stream_t s) { return reinterpret_cast<cudaStream_t>(s); }

int num_sms();
int check_tableau(const gb_tableau* tab);

// Tableau handed to kernels by value (a __grid_constant__ parameter lives in
// the constant bank) with b - bt folded as in RKEmbeddedParallel.hpp:108-114.
struct DevTableau {
  int n_stages;
  int p;
  int pt;
  int fsal;  // a[S-2][:] == b[:S-1] and b[S-1] == 0: last stage == f(x_new)
  double a[GB_MAX_STAGES][GB_MAX_STAGES];
  double b[GB_MAX_STAGES];
  double db[GB_MAX_STAGES];
  // non-zero patterns (bit j set when the coefficient of k_j is not zero),
  // so device code tests integer bits instead of comparing doubles (an FP64
  // compare occupies the FP64 pipe like a multiply)
  unsigned anz[GB_MAX_STAGES];  // row s-1 of a: coefficients of stage s
  unsigned bnz, dbnz;
};
DevTableau make_dev_tableau(const gb_tableau& t);

// ----- exact FP64 arithmetic helpers (no contraction) -----------------------
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }

// One softened pair term with the reference's operation order
// (NBodyODE.hpp:89-98): r2 = dx*dx + dy*dy + dz*dz + eps2, den = sqrt(r2)*r2,
// a = d / den, all IEEE-rounded.
__device__ __forceinline__ void pair_term_f64(double xi, double yi, double zi, double xj,
                                              double yj, double zj, double eps2, double& ax,
                                              double& ay, double& az) {
  const double dx = dsub(xj, xi);
  const double dy = dsub(yj, yi);
  const double dz = dsub(zj, zi);
  const double r2 = dadd(dadd(dadd(dmul(dx, dx), dmul(dy, dy)), dmul(dz, dz)), eps2);
  const double den = dmul(__dsqrt_rn(r2), r2);
  ax = __ddiv_rn(dx, den);
  ay = __ddiv_rn(dy, den);
  az = __ddiv_rn(dz, den);
}

// r^-3 of one softened pair from r2 = |d|^2 + eps^2, for the FP64 pair loops
// that need not reproduce the reference's operation order: y = 1/sqrt(r2)
// from the SFU's FP64 approximation, refined by two Newton steps for the
// reciprocal square root, y <- y + y (1/2 - (r2/2) y^2) (each step squares the
// relative error), then y^3.  Within a few ulp of the correctly rounded value,
// in 9 FP64 operations where sqrt(r2) * r2 and three divisions take ~45.
__device__ __forceinline__ double rinv3_f64(double r2) {
  double y;
  asm("rsqrt.approx.f64 %0, %1;" : "=d"(y) : "d"(r2));
  const double h = 0.5 * r2;
  y = fma(y, fma(-h * y, y, 0.5), y);
  y = fma(y, fma(-h * y, y, 0.5), y);
  return y * y * y;
}

// Splits v (FP64) into hi + lo FP32 parts: hi = fl32(v), lo = fl32(v - hi).
__device__ __forceinline__ void split_hilo(double v, float& hi, float& lo) {
  hi = __double2float_rn(v);
  lo = __double2float_rn(dsub(v, (double)hi));
}

// Bounded spin helpers ------------------------------------------------------
constexpr long long kSpinLimit = 1LL << 26;

}  // namespace gb
