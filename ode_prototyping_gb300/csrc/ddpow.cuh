// ddpow.cuh -- x^y for x > 0 evaluated in double-double arithmetic (about
// 100 significant bits) and rounded once to double, i.e. correctly rounded
// except when the exact result lies within ~2^-90 of a rounding boundary.
// Used by the exact mode so that the step-size formulas give the same double
// as a correctly rounding host pow (the reference's controller,
// RKEmbeddedParallel.hpp:65 and :197, calls std::pow on the host).
//
// Method (textbook): error-free transformations TwoSum / TwoProd (Knuth,
// Dekker); log x = k ln 2 + 2 atanh((m-1)/(m+1)) with m in [1/sqrt2, sqrt2)
// and the atanh series summed by Horner; exp r with r = y log x - k ln 2,
// the argument scaled by 2^-10, a Taylor series, then ten squarings.
#pragma once

#include <cuda_runtime.h>

namespace gb {

struct dd {
  double hi, lo;
};

__device__ __forceinline__ dd dd_two_sum(double a, double b) {
  const double s = a + b;
  const double bb = s - a;
  return {s, (a - (s - bb)) + (b - bb)};
}

__device__ __forceinline__ dd dd_fast(double a, double b) {  // |a| >= |b|
  const double s = a + b;
  return {s, b - (s - a)};
}

__device__ __forceinline__ dd dd_add(dd a, dd b) {
  dd s = dd_two_sum(a.hi, b.hi);
  dd t = dd_two_sum(a.lo, b.lo);
  s.lo += t.hi;
  s = dd_fast(s.hi, s.lo);
  s.lo += t.lo;
  return dd_fast(s.hi, s.lo);
}

__device__ __forceinline__ dd dd_mul(dd a, dd b) {
  const double p = a.hi * b.hi;
  double e = fma(a.hi, b.hi, -p);
  e = fma(a.hi, b.lo, e);
  e = fma(a.lo, b.hi, e);
  return dd_fast(p, e);
}

__device__ __forceinline__ dd dd_mul_d(dd a, double b) {
  const double p = a.hi * b;
  double e = fma(a.hi, b, -p);
  e = fma(a.lo, b, e);
  return dd_fast(p, e);
}

__device__ __forceinline__ dd dd_div(dd a, dd b) {
  const double q1 = a.hi / b.hi;
  dd r = dd_add(a, dd_mul_d(b, -q1));
  const double q2 = r.hi / b.hi;
  r = dd_add(r, dd_mul_d(b, -q2));
  const double q3 = r.hi / b.hi;
  dd q = dd_fast(q1, q2);
  return dd_add(q, dd{q3, 0.0});
}

// ln 2 to double-double precision (hi = nearest double, lo = remainder).
__device__ __forceinline__ dd dd_ln2() {
  return {0.6931471805599452862268, 2.319046813846299558e-17};
}

__device__ inline dd dd_log(double x) {
  int k;
  double m = frexp(x, &k);  // x = m 2^k, m in [0.5, 1)
  if (m < 0.70710678118654752440) {
    m *= 2.0;
    k -= 1;
  }
  // z = (m - 1) / (m + 1); m - 1 is exact for m in [1/sqrt2, sqrt2)
  const dd num = {m - 1.0, 0.0};
  const dd den = dd_two_sum(m, 1.0);
  const dd z = dd_div(num, den);
  const dd z2 = dd_mul(z, z);
  // atanh(z) / z = sum_j z^(2j) / (2j + 1), |z| <= 0.1716: 24 terms
  dd s = {1.0 / 47.0, 0.0};
  for (int j = 22; j >= 0; --j) {
    const dd c = dd_div(dd{1.0, 0.0}, dd{2.0 * j + 1.0, 0.0});
    s = dd_add(dd_mul(s, z2), c);
  }
  dd l = dd_mul(dd_mul_d(z, 2.0), s);
  return dd_add(dd_mul_d(dd_ln2(), (double)k), l);
}

__device__ inline dd dd_exp(dd y) {
  const double kf = rint(y.hi / 0.6931471805599452862268);
  dd r = dd_add(y, dd_mul_d(dd_ln2(), -kf));
  r = dd_mul_d(r, 1.0 / 1024.0);  // exact scaling
  // exp(r) = 1 + r (1 + r/2 (1 + r/3 (1 + ... (1 + r/12)))), Horner from the top
  dd t = {1.0, 0.0};
  for (int j = 12; j >= 2; --j) t = dd_add(dd{1.0, 0.0}, dd_div(dd_mul(t, r), dd{(double)j, 0.0}));
  dd e = dd_add(dd{1.0, 0.0}, dd_mul(t, r));
  for (int j = 0; j < 10; ++j) e = dd_mul(e, e);
  return {ldexp(e.hi, (int)kf), ldexp(e.lo, (int)kf)};
}

// x^y, x > 0 finite; pow(0, y > 0) = 0.
__device__ inline double dd_pow(double x, double y) {
  if (x == 0.0) return y > 0.0 ? 0.0 : (y == 0.0 ? 1.0 : __longlong_as_double(0x7ff0000000000000LL));
  if (x == 1.0 || y == 0.0) return 1.0;
  const dd l = dd_log(x);
  const dd e = dd_exp(dd_mul_d(l, y));
  return e.hi + e.lo;
}

}  // namespace gb
