// rk.cu -- element-wise embedded Runge-Kutta kernels with a host-scalar dt,
// the deterministic scaled-RMS norm, the built-in tableaus and the library's
// small C-ABI helpers.
//
// Replaces the reference's element-wise kernels in
// src/integrator/RKEmbeddedParallel/RKEmbeddedParallel.hpp:91-149 run through
// CudaExecutor (src/par_exec/CudaExecutor.cuh:80-126).  Each kernel keeps the
// reference's accumulation order (sum from 0.0 with the stage index
// ascending, then x0 + sum * dt) with IEEE-rounded operations, so the results
// equal the reference's element for element; coefficients that are exactly
// zero are skipped, which can only change the sign of a zero result.
#include <cstdint>
#include <cstdio>
#include <cstring>

#include "gb_internal.cuh"

namespace gb {

namespace {
int g_last_cuda_error = 0;
}

void note_cuda_error(cudaError_t e) { g_last_cuda_error = (int)e; }

int num_sms() {
  static int sms = 0;
  if (sms == 0) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        sms <= 0)
      sms = 152;
  }
  return sms;
}

int check_tableau(const gb_tableau* tab) {
  if (!tab || tab->n_stages < 1 || tab->n_stages > GB_MAX_STAGES || tab->p < 1 || tab->pt < 1)
    return GB_ERR_INVALID_ARGUMENT;
  return GB_OK;
}

DevTableau make_dev_tableau(const gb_tableau& t) {
  DevTableau d;
  std::memset(&d, 0, sizeof d);
  d.n_stages = t.n_stages;
  d.p = t.p;
  d.pt = t.pt;
  std::memcpy(d.a, t.a, sizeof d.a);
  std::memcpy(d.b, t.b, sizeof d.b);
  for (int j = 0; j < GB_MAX_STAGES; ++j) d.db[j] = t.b[j] - t.bt[j];
  for (int r = 0; r < GB_MAX_STAGES; ++r)
    for (int j = 0; j < GB_MAX_STAGES; ++j)
      if (t.a[r][j] != 0.0) d.anz[r] |= 1u << j;
  for (int j = 0; j < GB_MAX_STAGES; ++j) {
    if (d.b[j] != 0.0) d.bnz |= 1u << j;
    if (d.db[j] != 0.0) d.dbnz |= 1u << j;
  }
  const int S = t.n_stages;
  int fsal = S >= 2 && t.b[S - 1] == 0.0;
  for (int j = 0; fsal && j < S - 1; ++j)
    if (t.a[S - 2][j] != t.b[j]) fsal = 0;
  d.fsal = fsal;
  return d;
}

namespace {

constexpr int kBlock = 256;

unsigned blocks_for(long long n) {
  long long b = (n + kBlock - 1) / kBlock;
  if (b < 1) b = 1;
  if (b > (1LL << 30)) b = 1LL << 30;
  return (unsigned)b;
}

// One linear combination's coefficients, uniform across the grid: c[j] for
// the sum written to the first output, d[j] for an optional second one.
struct Coef {
  double c[GB_MAX_STAGES];
  double d[GB_MAX_STAGES];
  unsigned cnz, dnz;  // bit j: c[j] (d[j]) is not zero; tested as integers on the device
};

// V consecutive doubles per thread and iteration (V = 2: 16-byte loads).
template <int V>
struct Vec;
template <>
struct Vec<1> {
  double v[1];
  __device__ __forceinline__ void load(const double* __restrict__ p, long long e) { v[0] = p[e]; }
  __device__ __forceinline__ void store(double* __restrict__ p, long long e) const { p[e] = v[0]; }
};
template <>
struct Vec<2> {
  double v[2];
  __device__ __forceinline__ void load(const double* __restrict__ p, long long e) {
    const double2 t = reinterpret_cast<const double2*>(p)[e];
    v[0] = t.x;
    v[1] = t.y;
  }
  __device__ __forceinline__ void store(double* __restrict__ p, long long e) const {
    reinterpret_cast<double2*>(p)[e] = make_double2(v[0], v[1]);
  }
};

// temp = x0 + dt * sum_{j<S} c[j] k_j (rk_stage_kernel, RKEmbeddedParallel.hpp:91-101).
// Every k_j with a non-zero coefficient is loaded before the ordered sum, so
// S loads per element are in flight at once; the sum itself keeps the
// reference's order (from 0.0, j ascending, then * dt, then + x0).
template <int S, int V>
__global__ void __launch_bounds__(kBlock) stage_kernel(const __grid_constant__ Coef cf, double dt,
                                                       const double* __restrict__ x0,
                                                       const double* __restrict__ ks,
                                                       double* __restrict__ temp, long long n) {
  const long long m = n / V;
  for (long long e = blockIdx.x * (long long)kBlock + threadIdx.x; e < m;
       e += (long long)gridDim.x * kBlock) {
    Vec<V> k[S], x;
#pragma unroll
    for (int j = 0; j < S; ++j)
      if ((cf.cnz >> j) & 1u) k[j].load(ks + (long long)j * n, e);
    x.load(x0, e);
    Vec<V> out;
#pragma unroll
    for (int u = 0; u < V; ++u) {
      double v = 0.0;
#pragma unroll
      for (int j = 0; j < S; ++j)
        if ((cf.cnz >> j) & 1u) v = dadd(v, dmul(cf.c[j], k[j].v[u]));
      out.v[u] = dadd(x.v[u], dmul(v, dt));
    }
    out.store(temp, e);
  }
}

// x = x0 + dt * sum b_j k_j, err = dt * sum (b_j - bt_j) k_j
// (update_state_and_error_kernel, RKEmbeddedParallel.hpp:103-123).
template <int S, int V>
__global__ void __launch_bounds__(kBlock) update_kernel(const __grid_constant__ Coef cf, double dt,
                                                        const double* __restrict__ x0,
                                                        const double* __restrict__ ks,
                                                        double* __restrict__ x,
                                                        double* __restrict__ err, long long n) {
  const long long m = n / V;
  for (long long e = blockIdx.x * (long long)kBlock + threadIdx.x; e < m;
       e += (long long)gridDim.x * kBlock) {
    Vec<V> k[S], x0v;
#pragma unroll
    for (int j = 0; j < S; ++j)
      if (((cf.cnz | cf.dnz) >> j) & 1u) k[j].load(ks + (long long)j * n, e);
    x0v.load(x0, e);
    Vec<V> xo, eo;
#pragma unroll
    for (int u = 0; u < V; ++u) {
      double xv = 0.0, ev = 0.0;
#pragma unroll
      for (int j = 0; j < S; ++j) {
        if ((cf.cnz >> j) & 1u) xv = dadd(xv, dmul(cf.c[j], k[j].v[u]));
        if ((cf.dnz >> j) & 1u) ev = dadd(ev, dmul(cf.d[j], k[j].v[u]));
      }
      xo.v[u] = dadd(x0v.v[u], dmul(xv, dt));
      eo.v[u] = dmul(ev, dt);
    }
    xo.store(x, e);
    eo.store(err, e);
  }
}

template <int V>
__global__ void __launch_bounds__(kBlock) target_kernel(const double* __restrict__ atol,
                                                        const double* __restrict__ rtol,
                                                        const double* __restrict__ x,
                                                        const double* __restrict__ x0,
                                                        double* __restrict__ target, long long n) {
  const long long m = n / V;
  for (long long e = blockIdx.x * (long long)kBlock + threadIdx.x; e < m;
       e += (long long)gridDim.x * kBlock) {
    Vec<V> at, rt, xv, x0v, out;
    at.load(atol, e);
    rt.load(rtol, e);
    xv.load(x, e);
    x0v.load(x0, e);
#pragma unroll
    for (int u = 0; u < V; ++u) {
      const double a = fabs(xv.v[u]), b = fabs(x0v.v[u]);
      out.v[u] = dadd(at.v[u], dmul(rt.v[u], a < b ? b : a));
    }
    out.store(target, e);
  }
}

__global__ void fill_kernel(double* p, long long n, double v) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) p[i] = v;
}

constexpr int kNormMaxBlocks = 1024;

int norm_blocks(long long n) {
  long long b = (n + 4 * kBlock - 1) / (4 * kBlock);
  if (b < 1) b = 1;
  if (b > kNormMaxBlocks) b = kNormMaxBlocks;
  return (int)b;
}

// Per-block partial sums of (v/s)^2: each thread keeps four independent
// running sums over a grid-stride walk (four IEEE divisions in flight), adds
// them in a fixed order, then a fixed shared-memory tree.  Deterministic for
// a given n.
__global__ void __launch_bounds__(kBlock) sq_partial_kernel(const double* __restrict__ v,
                                                            const double* __restrict__ s,
                                                            long long n,
                                                            double* __restrict__ partial) {
  __shared__ double sh[kBlock];
  constexpr int U = 4;
  double acc[U] = {0.0, 0.0, 0.0, 0.0};
  const long long stride = (long long)gridDim.x * kBlock;
  for (long long i0 = blockIdx.x * (long long)kBlock + threadIdx.x; i0 < n; i0 += U * stride) {
    double vv[U], ss[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const long long i = i0 + u * stride;
      vv[u] = i < n ? v[i] : 0.0;
      ss[u] = i < n ? s[i] : 1.0;
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const double q = __ddiv_rn(vv[u], ss[u]);
      acc[u] = dadd(acc[u], dmul(q, q));
    }
  }
  sh[threadIdx.x] = dadd(dadd(acc[0], acc[1]), dadd(acc[2], acc[3]));
  __syncthreads();
  for (int st = kBlock / 2; st > 0; st /= 2) {
    if ((int)threadIdx.x < st) sh[threadIdx.x] = dadd(sh[threadIdx.x], sh[threadIdx.x + st]);
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

// Sums the partials in block order; out = sqrt(sum / n) or the sum itself.
__global__ void sq_final_kernel(const double* __restrict__ partial, int nb, long long n,
                                int take_sqrt, double* out) {
  __shared__ double sh[kBlock];
  double acc = 0.0;
  for (int i = threadIdx.x; i < nb; i += kBlock) acc = dadd(acc, partial[i]);
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int st = kBlock / 2; st > 0; st /= 2) {
    if ((int)threadIdx.x < st) sh[threadIdx.x] = dadd(sh[threadIdx.x], sh[threadIdx.x + st]);
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = take_sqrt ? sqrt(sh[0] / (double)n) : sh[0];
}

}  // namespace

namespace {

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

// Persistent-style grid for the streaming kernels: at most 8 blocks of 256
// threads per SM (all resident), grid-stride beyond that.
unsigned stream_blocks(long long m) {
  long long b = (m + kBlock - 1) / kBlock;
  const long long cap = (long long)num_sms() * 8;
  if (b > cap) b = cap;
  return (unsigned)(b < 1 ? 1 : b);
}

#define GB_STAGE_CASES(X) \
  X(1) X(2) X(3) X(4) X(5) X(6) X(7) X(8) X(9) X(10) X(11) X(12) X(13) X(14) X(15) X(16)

template <int V>
void launch_stage_v(int S, const Coef& cf, double dt, const double* x0, const double* ks,
                    double* temp, long long n, cudaStream_t st) {
  const unsigned g = stream_blocks(n / V);
  switch (S) {
#define GB_CASE(k) \
  case k: stage_kernel<k, V><<<g, kBlock, 0, st>>>(cf, dt, x0, ks, temp, n); break;
    GB_STAGE_CASES(GB_CASE)
#undef GB_CASE
    default: break;
  }
}

template <int V>
void launch_update_v(int S, const Coef& cf, double dt, const double* x0, const double* ks,
                     double* x, double* err, long long n, cudaStream_t st) {
  const unsigned g = stream_blocks(n / V);
  switch (S) {
#define GB_CASE(k) \
  case k: update_kernel<k, V><<<g, kBlock, 0, st>>>(cf, dt, x0, ks, x, err, n); break;
    GB_STAGE_CASES(GB_CASE)
#undef GB_CASE
    default: break;
  }
}

}  // namespace

int launch_norm(const double* v, const double* s, long long n, double* partial, double* out,
                int take_sqrt, cudaStream_t st) {
  const int nb = norm_blocks(n);
  sq_partial_kernel<<<nb, kBlock, 0, st>>>(v, s, n, partial);
  GB_CUDA_TRY(cudaGetLastError());
  sq_final_kernel<<<1, kBlock, 0, st>>>(partial, nb, n, take_sqrt, out);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

size_t norm_workspace_bytes(long long n) {
  // block partials + one result slot, rounded to 256 bytes
  size_t b = ((size_t)norm_blocks(n) + 1) * sizeof(double);
  return (b + 255) / 256 * 256;
}

}  // namespace gb

using namespace gb;

extern "C" const char* gb_status_string(int status) {
  switch (status) {
    case GB_OK: return "ok";
    case GB_ERR_INVALID_ARGUMENT: return "invalid argument";
    case GB_ERR_CUDA: return "CUDA error";
    case GB_ERR_UNSUPPORTED: return "unsupported configuration";
    case GB_ERR_NOT_FINITE: return "non-finite error estimate or state";
    case GB_ERR_BUDGET: return "attempt budget exhausted";
    case GB_ERR_TIMEOUT: return "bounded wait timed out";
    case GB_ERR_CAPACITY: return "workspace too small";
    case GB_ERR_STEP_UNDERFLOW: return "step size underflow";
    default: return "unknown status";
  }
}

extern "C" int gb_last_cuda_error(void) { return g_last_cuda_error; }
extern "C" int gb_version(void) { return 10000; }

extern "C" int gb_tableau_builtin(int32_t id, gb_tableau* t) {
  if (!t) return GB_ERR_INVALID_ARGUMENT;
  std::memset(t, 0, sizeof *t);
  auto A = [t](int r, int c, double v) { t->a[r][c] = v; };
  switch (id) {
    case GB_HE21:  // BTHE21.hpp:5-12 (Heun-Euler)
      t->n_stages = 2; t->p = 2; t->pt = 1;
      A(0, 0, 1.0);
      t->b[0] = 1.0 / 2.0; t->b[1] = 1.0 / 2.0;
      t->bt[0] = 1.0;
      return GB_OK;
    case GB_RKF45:  // BTRKF45.hpp:5-21 (Fehlberg 4(5))
      t->n_stages = 6; t->p = 4; t->pt = 5;
      A(0, 0, 1.0 / 4.0);
      A(1, 0, 3.0 / 32.0); A(1, 1, 9.0 / 32.0);
      A(2, 0, 1932.0 / 2197.0); A(2, 1, -7200.0 / 2197.0); A(2, 2, 7296.0 / 2197.0);
      A(3, 0, 439.0 / 216.0); A(3, 1, -8.0); A(3, 2, 3680.0 / 513.0); A(3, 3, -845.0 / 4104.0);
      A(4, 0, -8.0 / 27.0); A(4, 1, 2.0); A(4, 2, -3544.0 / 2565.0);
      A(4, 3, 1859.0 / 4104.0); A(4, 4, -11.0 / 40.0);
      t->b[0] = 25.0 / 216.0; t->b[2] = 1408.0 / 2565.0; t->b[3] = 2197.0 / 4104.0;
      t->b[4] = -0.2;
      t->bt[0] = 16.0 / 135.0; t->bt[2] = 6656.0 / 12825.0; t->bt[3] = 28561.0 / 56430.0;
      t->bt[4] = -9.0 / 50.0; t->bt[5] = 2.0 / 55.0;
      return GB_OK;
    case GB_DOPRI5:  // BTDOPRI5.hpp:5-26 (Dormand-Prince 5(4))
      t->n_stages = 7; t->p = 5; t->pt = 4;
      A(0, 0, 1.0 / 5.0);
      A(1, 0, 3.0 / 40.0); A(1, 1, 9.0 / 40.0);
      A(2, 0, 44.0 / 45.0); A(2, 1, -56.0 / 15.0); A(2, 2, 32.0 / 9.0);
      A(3, 0, 19372.0 / 6561.0); A(3, 1, -25360.0 / 2187.0); A(3, 2, 64448.0 / 6561.0);
      A(3, 3, -212.0 / 729.0);
      A(4, 0, 9017.0 / 3168.0); A(4, 1, -355.0 / 33.0); A(4, 2, 46732.0 / 5247.0);
      A(4, 3, 49.0 / 176.0); A(4, 4, -5103.0 / 18656.0);
      A(5, 0, 35.0 / 384.0); A(5, 2, 500.0 / 1113.0); A(5, 3, 125.0 / 192.0);
      A(5, 4, -2187.0 / 6784.0); A(5, 5, 11.0 / 84.0);
      t->b[0] = 35.0 / 384.0; t->b[2] = 500.0 / 1113.0; t->b[3] = 125.0 / 192.0;
      t->b[4] = -2187.0 / 6784.0; t->b[5] = 11.0 / 84.0;
      t->bt[0] = 5179.0 / 57600.0; t->bt[2] = 7571.0 / 16695.0; t->bt[3] = 393.0 / 640.0;
      t->bt[4] = -92097.0 / 339200.0; t->bt[5] = 187.0 / 2100.0; t->bt[6] = 1.0 / 40.0;
      return GB_OK;
    case GB_DVERK:  // BTDVERK.hpp:5-27 (Verner 6(5))
      t->n_stages = 8; t->p = 6; t->pt = 5;
      A(0, 0, 1.0 / 6.0);
      A(1, 0, 4.0 / 75.0); A(1, 1, 16.0 / 75.0);
      A(2, 0, 5.0 / 6.0); A(2, 1, -8.0 / 3.0); A(2, 2, 5.0 / 2.0);
      A(3, 0, -165.0 / 64.0); A(3, 1, 55.0 / 6.0); A(3, 2, -425.0 / 64.0);
      A(3, 3, 85.0 / 96.0);
      A(4, 0, 12.0 / 5.0); A(4, 1, -8.0); A(4, 2, 4015.0 / 612.0); A(4, 3, -11.0 / 36.0);
      A(4, 4, 88.0 / 255.0);
      A(5, 0, -8263.0 / 15000.0); A(5, 1, 124.0 / 75.0); A(5, 2, -643.0 / 680.0);
      A(5, 3, -81.0 / 250.0); A(5, 4, 2484.0 / 10625.0);
      A(6, 0, 3501.0 / 1720.0); A(6, 1, -300.0 / 43.0); A(6, 2, 297275.0 / 52632.0);
      A(6, 3, -319.0 / 2322.0); A(6, 4, 24068.0 / 84065.0); A(6, 6, 3850.0 / 26703.0);
      t->b[0] = 3.0 / 40.0; t->b[2] = 875.0 / 2244.0; t->b[3] = 23.0 / 72.0;
      t->b[4] = 264.0 / 1955.0; t->b[6] = 125.0 / 11592.0; t->b[7] = 43.0 / 616.0;
      t->bt[0] = 13.0 / 160.0; t->bt[2] = 2375.0 / 5984.0; t->bt[3] = 5.0 / 16.0;
      t->bt[4] = 12.0 / 85.0; t->bt[5] = 3.0 / 44.0;
      return GB_OK;
    case GB_RKF78:  // BTRKF78.hpp:5-45 (Fehlberg 7(8))
      t->n_stages = 13; t->p = 7; t->pt = 8;
      A(0, 0, 2.0 / 27.0);
      A(1, 0, 1.0 / 36.0); A(1, 1, 1.0 / 12.0);
      A(2, 0, 1.0 / 24.0); A(2, 2, 1.0 / 8.0);
      A(3, 0, 5.0 / 12.0); A(3, 2, -25.0 / 16.0); A(3, 3, 25.0 / 16.0);
      A(4, 0, 1.0 / 20.0); A(4, 3, 1.0 / 4.0); A(4, 4, 1.0 / 5.0);
      A(5, 0, -25.0 / 108.0); A(5, 3, 125.0 / 108.0); A(5, 4, -65.0 / 27.0);
      A(5, 5, 125.0 / 54.0);
      A(6, 0, 31.0 / 300.0); A(6, 4, 61.0 / 225.0); A(6, 5, -2.0 / 9.0);
      A(6, 6, 13.0 / 900.0);
      A(7, 0, 2.0); A(7, 3, -53.0 / 6.0); A(7, 4, 704.0 / 45.0); A(7, 5, -107.0 / 9.0);
      A(7, 6, 67.0 / 90.0); A(7, 7, 3.0);
      A(8, 0, -91.0 / 108.0); A(8, 3, 23.0 / 108.0); A(8, 4, -976.0 / 135.0);
      A(8, 5, 311.0 / 54.0); A(8, 6, -19.0 / 60.0); A(8, 7, 17.0 / 6.0);
      A(8, 8, -1.0 / 12.0);
      A(9, 0, 2383.0 / 4100.0); A(9, 3, -341.0 / 164.0); A(9, 4, 4496.0 / 1025.0);
      A(9, 5, -301.0 / 82.0); A(9, 6, 2133.0 / 4100.0); A(9, 7, 45.0 / 82.0);
      A(9, 8, 45.0 / 164.0); A(9, 9, 18.0 / 41.0);
      A(10, 0, 3.0 / 205.0); A(10, 5, -6.0 / 41.0); A(10, 6, -3.0 / 205.0);
      A(10, 7, -3.0 / 41.0); A(10, 8, 3.0 / 41.0); A(10, 9, 6.0 / 41.0);
      A(11, 0, -1777.0 / 4100.0); A(11, 3, -341.0 / 164.0); A(11, 4, 4496.0 / 1025.0);
      A(11, 5, -289.0 / 82.0); A(11, 6, 2193.0 / 4100.0); A(11, 7, 51.0 / 82.0);
      A(11, 8, 33.0 / 164.0); A(11, 9, 12.0 / 41.0); A(11, 11, 1.0);
      t->b[0] = 41.0 / 840.0; t->b[5] = 34.0 / 105.0; t->b[6] = 9.0 / 35.0;
      t->b[7] = 9.0 / 35.0; t->b[8] = 9.0 / 280.0; t->b[9] = 9.0 / 280.0;
      t->b[10] = 41.0 / 840.0;
      t->bt[5] = 34.0 / 105.0; t->bt[6] = 9.0 / 35.0; t->bt[7] = 9.0 / 35.0;
      t->bt[8] = 9.0 / 280.0; t->bt[9] = 9.0 / 280.0; t->bt[11] = 41.0 / 840.0;
      t->bt[12] = 41.0 / 840.0;
      return GB_OK;
    default:
      return GB_ERR_INVALID_ARGUMENT;
  }
}

extern "C" int gb_device_alloc(void** p, size_t bytes) {
  if (!p) return GB_ERR_INVALID_ARGUMENT;
  *p = nullptr;
  if (bytes == 0) return GB_OK;
  GB_CUDA_TRY(cudaMalloc(p, bytes));
  return GB_OK;
}

extern "C" int gb_device_free(void* p) {
  if (p) GB_CUDA_TRY(cudaFree(p));
  return GB_OK;
}

extern "C" int gb_memcpy(void* dst, const void* src, size_t bytes, int32_t kind) {
  if ((!dst || !src) && bytes) return GB_ERR_INVALID_ARGUMENT;
  cudaMemcpyKind k;
  switch (kind) {
    case 0: k = cudaMemcpyHostToDevice; break;
    case 1: k = cudaMemcpyDeviceToHost; break;
    case 2: k = cudaMemcpyDeviceToDevice; break;
    default: return GB_ERR_INVALID_ARGUMENT;
  }
  if (bytes) GB_CUDA_TRY(cudaMemcpy(dst, src, bytes, k));
  return GB_OK;
}

extern "C" int gb_memset_zero(void* p, size_t bytes) {
  if (!p && bytes) return GB_ERR_INVALID_ARGUMENT;
  if (bytes) GB_CUDA_TRY(cudaMemset(p, 0, bytes));
  return GB_OK;
}

// Replaces fill (src/state/StateUtils.hpp:5-16).
extern "C" int gb_fill_f64(double* p, int64_t n, double v, gb_stream_t stream) {
  if (!p || n < 0) return GB_ERR_INVALID_ARGUMENT;
  if (n == 0) return GB_OK;
  fill_kernel<<<blocks_for(n), kBlock, 0, as_cuda(stream)>>>(p, n, v);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

extern "C" int gb_pointer_kind(const void* p) {
  if (!p) return 0;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();  // clear: plain host memory
    return 0;
  }
  switch (a.type) {
    case cudaMemoryTypeDevice: return 1;
    case cudaMemoryTypeManaged: return 2;
    default: return 0;
  }
}

extern "C" int gb_stream_synchronize(gb_stream_t stream) {
  GB_CUDA_TRY(cudaStreamSynchronize(as_cuda(stream)));
  return GB_OK;
}

extern "C" int gb_rk_stage_f64(const gb_tableau* tab, int32_t stage, double dt, const double* x0,
                               const double* ks, double* temp, int64_t n, gb_stream_t stream) {
  GB_TRY(check_tableau(tab));
  if (!x0 || !ks || !temp || n < 1 || stage < 1 || stage >= tab->n_stages)
    return GB_ERR_INVALID_ARGUMENT;
  Coef cf;
  std::memset(&cf, 0, sizeof cf);
  for (int j = 0; j < stage; ++j) {
    cf.c[j] = tab->a[stage - 1][j];
    if (cf.c[j] != 0.0) cf.cnz |= 1u << j;
  }
  cudaStream_t st = as_cuda(stream);
  if (n % 2 == 0 && aligned16(x0) && aligned16(ks) && aligned16(temp))
    launch_stage_v<2>(stage, cf, dt, x0, ks, temp, n, st);
  else
    launch_stage_v<1>(stage, cf, dt, x0, ks, temp, n, st);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

extern "C" int gb_rk_update_state_and_error_f64(const gb_tableau* tab, double dt,
                                                const double* x0, const double* ks, double* x,
                                                double* err, int64_t n, gb_stream_t stream) {
  GB_TRY(check_tableau(tab));
  if (!x0 || !ks || !x || !err || n < 1) return GB_ERR_INVALID_ARGUMENT;
  Coef cf;
  std::memset(&cf, 0, sizeof cf);
  for (int j = 0; j < tab->n_stages; ++j) {
    cf.c[j] = tab->b[j];
    cf.d[j] = tab->b[j] - tab->bt[j];
    if (cf.c[j] != 0.0) cf.cnz |= 1u << j;
    if (cf.d[j] != 0.0) cf.dnz |= 1u << j;
  }
  cudaStream_t st = as_cuda(stream);
  if (n % 2 == 0 && aligned16(x0) && aligned16(ks) && aligned16(x) && aligned16(err))
    launch_update_v<2>(tab->n_stages, cf, dt, x0, ks, x, err, n, st);
  else
    launch_update_v<1>(tab->n_stages, cf, dt, x0, ks, x, err, n, st);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

extern "C" int gb_rk_error_target_f64(const double* atol, const double* rtol, const double* x,
                                      const double* x0, double* target, int64_t n,
                                      gb_stream_t stream) {
  if (!atol || !rtol || !x || !x0 || !target || n < 1) return GB_ERR_INVALID_ARGUMENT;
  cudaStream_t st = as_cuda(stream);
  if (n % 2 == 0 && aligned16(atol) && aligned16(rtol) && aligned16(x) && aligned16(x0) &&
      aligned16(target))
    target_kernel<2><<<stream_blocks(n / 2), kBlock, 0, st>>>(atol, rtol, x, x0, target, n);
  else
    target_kernel<1><<<stream_blocks(n), kBlock, 0, st>>>(atol, rtol, x, x0, target, n);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

extern "C" size_t gb_rk_norm_workspace_bytes(int64_t n) {
  return n < 1 ? 0 : norm_workspace_bytes(n);
}

extern "C" int gb_rk_norm_f64(const double* v, const double* s, int64_t n, void* work,
                              size_t work_bytes, double* norm_dev, gb_stream_t stream) {
  if (!v || !s || !work || !norm_dev || n < 1) return GB_ERR_INVALID_ARGUMENT;
  if (work_bytes < norm_workspace_bytes(n)) return GB_ERR_CAPACITY;
  return launch_norm(v, s, n, reinterpret_cast<double*>(work), norm_dev, 1, as_cuda(stream));
}

extern "C" int gb_rk_scaled_sq_sum_f64(const double* v, const double* s, int64_t n, void* work,
                                       size_t work_bytes, double* sum_host, gb_stream_t stream) {
  if (!v || !s || !work || !sum_host || n < 1) return GB_ERR_INVALID_ARGUMENT;
  if (work_bytes < norm_workspace_bytes(n)) return GB_ERR_CAPACITY;
  double* partial = reinterpret_cast<double*>(work);
  double* out = partial + norm_blocks(n);
  cudaStream_t st = as_cuda(stream);
  GB_TRY(launch_norm(v, s, n, partial, out, 0, st));
  GB_CUDA_TRY(cudaMemcpyAsync(sum_host, out, sizeof(double), cudaMemcpyDeviceToHost, st));
  GB_CUDA_TRY(cudaStreamSynchronize(st));
  return GB_OK;
}
