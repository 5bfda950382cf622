// energy.cu -- FP64 energy and momentum diagnostics on the device.
// Restates the softened potential energy and kinetic energy of
// scripts/nbody_physics/energy.py:146-192 (PE = -sum_{i<j} m_i m_j /
// sqrt(r^2 + eps^2), KE = sum m v^2 / 2; the reference has unit masses) with
// masses, plus linear and angular momentum.  Owner-computes: body i sums
// -m_j / sqrt(r_ij^2 + eps^2) over all j != i; PE = 1/2 sum_i m_i phi_i.
// Deterministic: per-CTA tree sums, then CTA partials added in order.
#include "force.cuh"

namespace gb {
namespace {

constexpr int kT = 128;

__global__ void __launch_bounds__(kT)
    energy_partial_kernel(const double* __restrict__ x, long long n, double eps2, double mass,
                          const double* __restrict__ masses, double* __restrict__ partial) {
  __shared__ double sh[4 * kT];
  __shared__ double red[8][kT];
  const long long i = blockIdx.x * (long long)kT + threadIdx.x;
  const double* pos = x;
  const double* vel = x + 3 * n;
  double xi = 0, yi = 0, zi = 0;
  if (i < n) {
    xi = pos[3 * i];
    yi = pos[3 * i + 1];
    zi = pos[3 * i + 2];
  }
  double phi = 0.0;
  for (long long j0 = 0; j0 < n; j0 += kT) {
    const int cnt = (int)min((long long)kT, n - j0);
    __syncthreads();
    for (int k = threadIdx.x; k < cnt; k += kT) {
      sh[4 * k] = pos[3 * (j0 + k)];
      sh[4 * k + 1] = pos[3 * (j0 + k) + 1];
      sh[4 * k + 2] = pos[3 * (j0 + k) + 2];
      sh[4 * k + 3] = masses ? masses[j0 + k] : mass;
    }
    __syncthreads();
    if (i < n) {
      for (int k = 0; k < cnt; ++k) {
        if (j0 + k == i) continue;
        const double dx = sh[4 * k] - xi, dy = sh[4 * k + 1] - yi, dz = sh[4 * k + 2] - zi;
        phi -= sh[4 * k + 3] / sqrt(dx * dx + dy * dy + dz * dz + eps2);
      }
    }
  }
  double v[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  if (i < n) {
    const double mi = masses ? masses[i] : mass;
    const double vx = vel[3 * i], vy = vel[3 * i + 1], vz = vel[3 * i + 2];
    v[0] = 0.5 * mi * (vx * vx + vy * vy + vz * vz);
    v[1] = 0.5 * mi * phi;
    v[2] = mi * vx;
    v[3] = mi * vy;
    v[4] = mi * vz;
    v[5] = mi * (yi * vz - zi * vy);
    v[6] = mi * (zi * vx - xi * vz);
    v[7] = mi * (xi * vy - yi * vx);
  }
  for (int c = 0; c < 8; ++c) red[c][threadIdx.x] = v[c];
  __syncthreads();
  for (int st = kT / 2; st > 0; st /= 2) {
    if ((int)threadIdx.x < st)
      for (int c = 0; c < 8; ++c) red[c][threadIdx.x] += red[c][threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x < 8) partial[blockIdx.x * 8 + threadIdx.x] = red[threadIdx.x][0];
}

__global__ void energy_final_kernel(const double* __restrict__ partial, int nb,
                                    double* __restrict__ out) {
  const int c = threadIdx.x;
  if (c >= 8) return;
  double s = 0.0;
  for (int b = 0; b < nb; ++b) s += partial[b * 8 + c];
  out[c] = s;
}

}  // namespace
}  // namespace gb

using namespace gb;

extern "C" size_t gb_nbody_energy_workspace_bytes(int64_t n) {
  if (n < 1) return 0;
  return (size_t)((n + kT - 1) / kT) * 8 * sizeof(double);
}

// out_dev[0] = kinetic, [1] = potential, [2..4] = linear momentum,
// [5..7] = angular momentum (about the origin).
extern "C" int gb_nbody_energy_f64(const double* x, int64_t n, double softening, double mass,
                                   const double* masses, void* work, size_t work_bytes,
                                   double* out_dev, gb_stream_t stream) {
  if (!x || n < 1 || !work || !out_dev || !(softening >= 0.0)) return GB_ERR_INVALID_ARGUMENT;
  if (!masses && !(mass > 0.0)) return GB_ERR_INVALID_ARGUMENT;
  if (work_bytes < gb_nbody_energy_workspace_bytes(n)) return GB_ERR_CAPACITY;
  cudaStream_t s = as_cuda(stream);
  const int nb = (int)((n + kT - 1) / kT);
  double* partial = reinterpret_cast<double*>(work);
  energy_partial_kernel<<<nb, kT, 0, s>>>(x, n, softening * softening, mass, masses, partial);
  GB_CUDA_TRY(cudaGetLastError());
  energy_final_kernel<<<1, 32, 0, s>>>(partial, nb, out_dev);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}
