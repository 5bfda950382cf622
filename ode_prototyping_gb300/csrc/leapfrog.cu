// leapfrog.cu -- fixed-step kick-drift-kick leapfrog on the N-body force
// kernels.  Replaces ParallelLeapfrogIntegrator::integrate
// (src/integrator/leapfrog/LeapfrogParallel.hpp:11-41) and its kernels
// (:57-73): pos += dt * (vel + 0.5 * dt * acc0); acc1 = a(pos);
// vel += 0.5 * dt * (acc0 + acc1); acc0 = acc1; t += dt -- the same
// operation order, IEEE-rounded, so with the serial force tiling the states
// equal the reference's bit for bit.
#include <vector>

#include "force.cuh"

namespace gb {
namespace {

__global__ void drift_kernel(double* __restrict__ pos, const double* __restrict__ vel,
                             const double* __restrict__ acc0, double dt, long long n_dof) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n_dof) return;
  pos[i] = dadd(pos[i], dmul(dt, dadd(vel[i], dmul(dmul(0.5, dt), acc0[i]))));
}

__global__ void kick_kernel(double* __restrict__ vel, double* __restrict__ acc0,
                            const double* __restrict__ acc1, double dt, long long n_dof) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n_dof) return;
  vel[i] = dadd(vel[i], dmul(dmul(0.5, dt), dadd(acc0[i], acc1[i])));
  acc0[i] = acc1[i];
}

}  // namespace
}  // namespace gb

using namespace gb;

extern "C" int gb_leapfrog_nbody(const gb_nbody_system* sys, double* x, double t0, double tf,
                                 double dt, int32_t precision, const gb_force_tiling* tiling,
                                 gb_save_fn save, void* user, int64_t* n_steps,
                                 gb_stream_t stream) {
  if (!sys || !x || sys->n_particles < 1 || !(dt > 0.0) || !std::isfinite(t0) ||
      !std::isfinite(tf))
    return GB_ERR_INVALID_ARGUMENT;
  if (precision != GB_PREC_F64 && precision != GB_PREC_MIXED) return GB_ERR_INVALID_ARGUMENT;
  const long long n = sys->n_particles, n_dof = 3 * n, n_var = 6 * n;
  cudaStream_t s = as_cuda(stream);
  double *acc = nullptr, *rhs = nullptr;
  void* work = nullptr;
  size_t work_bytes = 0;
  cudaError_t e = cudaMalloc((void**)&acc, 2 * n_dof * sizeof(double));
  if (e == cudaSuccess && precision == GB_PREC_MIXED) {
    e = cudaMalloc((void**)&rhs, n_var * sizeof(double));
    work_bytes = gb_nbody_mixed_workspace_bytes(n);
    if (e == cudaSuccess) e = cudaMalloc(&work, work_bytes);
  }
  if (e != cudaSuccess) {
    note_cuda_error(e);
    cudaFree(acc);
    cudaFree(rhs);
    cudaFree(work);
    return GB_ERR_CUDA;
  }
  double* acc0 = acc;
  double* acc1 = acc + n_dof;
  std::vector<double> host(save ? n_var : 0);
  auto accel = [&](double* out) -> int {  // NBodyODE::acc (NBodyODE.hpp:41-46)
    if (precision == GB_PREC_F64)
      return gb_nbody_acc_f64(x, out, n, sys->softening, sys->mass, sys->masses_dev, 0, tiling,
                              stream);
    int rc = gb_nbody_rhs_mixed(x, rhs, n, sys->softening, sys->mass, sys->masses_dev, work,
                                tiling, stream);
    if (rc == GB_OK) {
      cudaError_t ce = cudaMemcpyAsync(out, rhs + n_dof, n_dof * sizeof(double),
                                       cudaMemcpyDeviceToDevice, s);
      if (ce != cudaSuccess) {
        note_cuda_error(ce);
        return GB_ERR_CUDA;
      }
    }
    return rc;
  };
  auto emit = [&](double t) -> int {
    if (!save) return GB_OK;
    cudaError_t ce = cudaMemcpyAsync(host.data(), x, n_var * sizeof(double),
                                     cudaMemcpyDeviceToHost, s);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
    if (ce != cudaSuccess) {
      note_cuda_error(ce);
      return GB_ERR_CUDA;
    }
    save(user, t, host.data(), n_var);
    return GB_OK;
  };
  const unsigned blocks = (unsigned)((n_dof + 255) / 256);
  double t = t0;
  long long steps = 0;
  int rc = emit(t);
  if (rc == GB_OK) rc = accel(acc0);
  while (rc == GB_OK && t < tf) {
    drift_kernel<<<blocks, 256, 0, s>>>(x, x + n_dof, acc0, dt, n_dof);
    rc = accel(acc1);
    if (rc != GB_OK) break;
    kick_kernel<<<blocks, 256, 0, s>>>(x + n_dof, acc0, acc1, dt, n_dof);
    cudaError_t ce = cudaGetLastError();
    if (ce != cudaSuccess) {
      note_cuda_error(ce);
      rc = GB_ERR_CUDA;
      break;
    }
    t += dt;
    ++steps;
    rc = emit(t);
  }
  cudaStreamSynchronize(s);
  cudaFree(acc);
  cudaFree(rhs);
  cudaFree(work);
  if (n_steps) *n_steps = steps;
  return rc;
}
