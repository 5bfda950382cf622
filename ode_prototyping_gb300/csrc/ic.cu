// ic.cu -- seeded initial conditions (host code).  All systems use G = 1,
// total mass 1 (equal masses 1/N) and have the centre-of-mass position and
// velocity removed.  Output layout is the reference state layout
// [positions 3N | velocities 3N].
//
// Random numbers: xoshiro256** seeded through splitmix64 (Blackman & Vigna),
// uniform doubles from the top 53 bits, normals by Box-Muller.
#include <cmath>
#include <cstring>
#include <vector>

#include "gbode.h"

namespace {

struct Rng {
  uint64_t s[4];
  explicit Rng(uint64_t seed) {
    uint64_t z = seed;
    for (int i = 0; i < 4; ++i) {
      z += 0x9e3779b97f4a7c15ULL;
      uint64_t x = z;
      x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ULL;
      x = (x ^ (x >> 27)) * 0x94d049bb133111ebULL;
      s[i] = x ^ (x >> 31);
    }
  }
  static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
  uint64_t next() {
    const uint64_t r = rotl(s[1] * 5, 7) * 9;
    const uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl(s[3], 45);
    return r;
  }
  double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }  // [0,1)
  double uniform_open() {  // (0,1)
    double u;
    do u = uniform();
    while (u <= 0.0);
    return u;
  }
  double normal() {
    const double u1 = uniform_open(), u2 = uniform();
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
  }
  void unit_vector(double& x, double& y, double& z) {
    const double c = 2.0 * uniform() - 1.0;
    const double ph = 6.283185307179586 * uniform();
    const double s = std::sqrt(1.0 - c * c);
    x = s * std::cos(ph);
    y = s * std::sin(ph);
    z = c;
  }
};

void remove_com(double* x, long long n) {
  double c[6] = {0, 0, 0, 0, 0, 0};
  for (long long i = 0; i < n; ++i)
    for (int k = 0; k < 3; ++k) {
      c[k] += x[3 * i + k];
      c[3 + k] += x[3 * n + 3 * i + k];
    }
  for (int k = 0; k < 6; ++k) c[k] /= (double)n;
  for (long long i = 0; i < n; ++i)
    for (int k = 0; k < 3; ++k) {
      x[3 * i + k] -= c[k];
      x[3 * n + 3 * i + k] -= c[3 + k];
    }
}

// Plummer sphere, scale radius a, total mass 1 (Aarseth, Henon & Wielen
// 1974): r = a / sqrt(X^{-2/3} - 1) with X < 0.999 (mass cut at 99.9%),
// speed v = q sqrt(2) (1 + r^2/a^2)^{-1/4} / sqrt(a) with q drawn from
// g(q) = q^2 (1 - q^2)^{7/2} by rejection.
void plummer_body(Rng& g, double a, double* p, double* v) {
  double X;
  do X = g.uniform();
  while (X <= 0.0 || X >= 0.999);
  const double r = a / std::sqrt(std::pow(X, -2.0 / 3.0) - 1.0);
  double ux, uy, uz;
  g.unit_vector(ux, uy, uz);
  p[0] = r * ux;
  p[1] = r * uy;
  p[2] = r * uz;
  double q, y;
  do {
    q = g.uniform();
    y = 0.1 * g.uniform();
  } while (y > q * q * std::pow(1.0 - q * q, 3.5));
  const double sp = q * std::sqrt(2.0) * std::pow(1.0 + r * r / (a * a), -0.25) / std::sqrt(a);
  g.unit_vector(ux, uy, uz);
  v[0] = sp * ux;
  v[1] = sp * uy;
  v[2] = sp * uz;
}

double potential_energy(const double* x, long long n, double eps) {
  const double m = 1.0 / (double)n, e2 = eps * eps;
  double w = 0.0;
  for (long long i = 0; i < n; ++i) {
    double wi = 0.0;
    for (long long j = i + 1; j < n; ++j) {
      const double dx = x[3 * j] - x[3 * i], dy = x[3 * j + 1] - x[3 * i + 1],
                   dz = x[3 * j + 2] - x[3 * i + 2];
      wi += 1.0 / std::sqrt(dx * dx + dy * dy + dz * dz + e2);
    }
    w -= m * m * wi;
  }
  return w;
}

double kinetic_energy(const double* x, long long n) {
  const double m = 1.0 / (double)n;
  double k = 0.0;
  for (long long i = 0; i < 3 * n; ++i) k += 0.5 * m * x[3 * n + i] * x[3 * n + i];
  return k;
}

}  // namespace

extern "C" {

// Uniform in the unit ball (rejection), velocities N(0, sigma^2) per component.
int gb_ic_uniform_ball(int64_t n, uint64_t seed, double sigma_v, double* x) {
  if (n < 2 || !x) return GB_ERR_INVALID_ARGUMENT;
  Rng g(seed);
  for (long long i = 0; i < n; ++i) {
    double p[3];
    do {
      for (int k = 0; k < 3; ++k) p[k] = 2.0 * g.uniform() - 1.0;
    } while (p[0] * p[0] + p[1] * p[1] + p[2] * p[2] > 1.0);
    for (int k = 0; k < 3; ++k) x[3 * i + k] = p[k];
  }
  for (long long i = 0; i < 3 * n; ++i) x[3 * n + i] = sigma_v * g.normal();
  remove_com(x, n);
  return GB_OK;
}

// Plummer sphere with scale radius a, velocities from its distribution function.
int gb_ic_plummer(int64_t n, uint64_t seed, double a, double* x) {
  if (n < 2 || !x || !(a > 0.0)) return GB_ERR_INVALID_ARGUMENT;
  Rng g(seed);
  for (long long i = 0; i < n; ++i) plummer_body(g, a, x + 3 * i, x + 3 * n + 3 * i);
  remove_com(x, n);
  return GB_OK;
}

// Rescales velocities so that the virial ratio 2K/|W| equals q (softened W).
int gb_ic_set_virial_ratio(int64_t n, double q, double eps, double* x) {
  if (n < 2 || !x || !(q >= 0.0)) return GB_ERR_INVALID_ARGUMENT;
  const double w = potential_energy(x, n, eps);
  const double k = kinetic_energy(x, n);
  if (!(k > 0.0)) return GB_ERR_INVALID_ARGUMENT;
  const double f = std::sqrt(q * std::fabs(w) / (2.0 * k));
  for (long long i = 0; i < 3 * n; ++i) x[3 * n + i] *= f;
  return GB_OK;
}

// Cold uniform sphere of radius 1: velocities N(0, s^2) per component with
// s = noise * sqrt(3/5) / sqrt(3) (noise relative to the virial speed
// sqrt(3GM/5R) of a uniform sphere).
int gb_ic_cold_sphere(int64_t n, uint64_t seed, double noise, double* x) {
  if (n < 2 || !x) return GB_ERR_INVALID_ARGUMENT;
  Rng g(seed);
  for (long long i = 0; i < n; ++i) {
    double p[3];
    do {
      for (int k = 0; k < 3; ++k) p[k] = 2.0 * g.uniform() - 1.0;
    } while (p[0] * p[0] + p[1] * p[1] + p[2] * p[2] > 1.0);
    for (int k = 0; k < 3; ++k) x[3 * i + k] = p[k];
  }
  const double s = noise * std::sqrt(3.0 / 5.0) / std::sqrt(3.0);
  for (long long i = 0; i < 3 * n; ++i) x[3 * n + i] = s * g.normal();
  remove_com(x, n);
  return GB_OK;
}

// Plummer sphere (a = 1) in which a fraction `binary_frac` of the bodies are
// in circular bound pairs with semimajor axes log-uniform in [amin, amax]:
// the pair's centre of mass is a Plummer body, the members sit at +-a/2 with
// relative speed sqrt(2m / a) in a random orbital plane.
int gb_ic_binary_plummer(int64_t n, uint64_t seed, double binary_frac, double amin, double amax,
                         double* x) {
  if (n < 2 || !x || !(binary_frac >= 0.0) || !(amin > 0.0) || !(amax >= amin))
    return GB_ERR_INVALID_ARGUMENT;
  Rng g(seed);
  long long n_pairs = (long long)(binary_frac * (double)n / 2.0);
  const double m = 1.0 / (double)n;
  long long i = 0;
  for (long long pr = 0; pr < n_pairs && i + 1 < n; ++pr) {
    double c[3], cv[3];
    plummer_body(g, 1.0, c, cv);
    const double a = amin * std::exp(g.uniform() * std::log(amax / amin));
    double ux, uy, uz, wx, wy, wz;
    g.unit_vector(ux, uy, uz);
    // a velocity direction perpendicular to the separation
    g.unit_vector(wx, wy, wz);
    double px = uy * wz - uz * wy, py = uz * wx - ux * wz, pz = ux * wy - uy * wx;
    const double pn = std::sqrt(px * px + py * py + pz * pz);
    px /= pn;
    py /= pn;
    pz /= pn;
    const double vrel = std::sqrt(2.0 * m / a);
    const double sep[3] = {ux * a / 2, uy * a / 2, uz * a / 2};
    const double dv[3] = {px * vrel / 2, py * vrel / 2, pz * vrel / 2};
    for (int k = 0; k < 3; ++k) {
      x[3 * i + k] = c[k] + sep[k];
      x[3 * (i + 1) + k] = c[k] - sep[k];
      x[3 * n + 3 * i + k] = cv[k] + dv[k];
      x[3 * n + 3 * (i + 1) + k] = cv[k] - dv[k];
    }
    i += 2;
  }
  for (; i < n; ++i) plummer_body(g, 1.0, x + 3 * i, x + 3 * n + 3 * i);
  remove_com(x, n);
  return GB_OK;
}

}  // extern "C"
