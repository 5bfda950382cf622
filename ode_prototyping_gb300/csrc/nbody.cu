// nbody.cu -- standalone right-hand-side entry points (FP64 and mixed).
// Replaces NBodyODE<double, 6N>::operator() / acc() (src/ode/NBodyODE.hpp:31-46)
// and its two kernels nbody_init_dxdt_kernel (:51-56) and nbody_acc_kernel
// (:68-133), which the reference runs as one thread per unordered pair with
// six FP64 atomicAdds; here each body's sum is owned by one lane group.
#include "force.cuh"
#include "sortpack.cuh"

namespace gb {

// Argument checks shared by the right-hand-side entry points (also the
// allocation-free one in noalloc.cu).
int validate_nbody(const void* a, const void* b, long long n, double softening, double mass,
                   const double* masses) {
  if (!a || !b || n < 1) return GB_ERR_INVALID_ARGUMENT;
  if (!(softening >= 0.0) || !std::isfinite(softening)) return GB_ERR_INVALID_ARGUMENT;
  if (!masses && !(mass > 0.0)) return GB_ERR_INVALID_ARGUMENT;
  return GB_OK;
}

namespace {

enum { kModeRhs = 0, kModeAccWrite = 1, kModeAccAdd = 2 };

template <int T, int L>
__global__ void __launch_bounds__(T) rhs_f64_kernel(const double* __restrict__ pos,
                                                    const double* __restrict__ vel,
                                                    double* __restrict__ out_vel,
                                                    double* __restrict__ out_acc, long long n,
                                                    double eps2, double mass,
                                                    const double* __restrict__ masses, int mode,
                                                    int fast) {
  constexpr int BI = T / L;
  __shared__ double sh_pos[3 * T];
  __shared__ double sh_m[T];
  __shared__ double part[BI][3];
  const ClusterInfo ci = cluster_info();
  const long long i0 = ci.itile * BI;
  long long jb, je;
  j_chunk(n, ci.rank, ci.size, T, jb, je);
  force_f64_cta<T, L>(pos, n, i0, jb, je, eps2, masses, sh_pos, sh_m, part, fast != 0);
  cluster_combine<BI>(part, ci.rank, ci.size);
  if (ci.rank != 0) return;
  const long long nb = min((long long)BI, n - i0);
  for (int e = threadIdx.x; e < 3 * nb; e += T) {
    const long long g = 3 * i0 + e;
    double a = part[e / 3][e % 3];
    if (!masses) a = dmul(a, mass);
    if (mode == kModeRhs) {
      out_vel[g] = vel[g];
      out_acc[g] = a;
    } else if (mode == kModeAccWrite) {
      out_acc[g] = a;
    } else {
      out_acc[g] = dadd(out_acc[g], a);
    }
  }
}

__global__ void centroid_kernel(const double* __restrict__ pos, long long n, double* c_out) {
  __shared__ double sh[3][1024];
  double s0 = 0.0, s1 = 0.0, s2 = 0.0;
  for (long long i = threadIdx.x; i < n; i += blockDim.x) {
    s0 += pos[3 * i];
    s1 += pos[3 * i + 1];
    s2 += pos[3 * i + 2];
  }
  sh[0][threadIdx.x] = s0;
  sh[1][threadIdx.x] = s1;
  sh[2][threadIdx.x] = s2;
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st /= 2) {
    if ((int)threadIdx.x < st) {
      sh[0][threadIdx.x] += sh[0][threadIdx.x + st];
      sh[1][threadIdx.x] += sh[1][threadIdx.x + st];
      sh[2][threadIdx.x] += sh[2][threadIdx.x + st];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    c_out[0] = sh[0][0] / (double)n;
    c_out[1] = sh[1][0] / (double)n;
    c_out[2] = sh[2][0] / (double)n;
  }
}

__global__ void pack_kernel(const double* __restrict__ pos, const double* __restrict__ masses,
                            const double* __restrict__ c, long long n, PackedBody* out) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float w = masses ? (float)masses[i] : 1.0f;
  out[i] = pack_body(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2], c[0], c[1], c[2], w);
}

template <int T, int L, int BPT, bool PACKED>
__global__ void __launch_bounds__(T) rhs_mixed_kernel(const PackedBody* __restrict__ packed,
                                                      const double* __restrict__ vel,
                                                      double* __restrict__ out_vel,
                                                      double* __restrict__ out_acc,
                                                      long long n, float eps2, double mass,
                                                      int uniform_mass) {
  constexpr int BI = (T / L) * BPT;
  constexpr int SH = PACKED ? jp_smem_bytes<T>() : (int)sizeof(PackedBody) * T;
  __shared__ __align__(16) unsigned char sh_raw[SH];
  __shared__ double part[BI][3];
  const ClusterInfo ci = cluster_info();
  const long long i0 = ci.itile * BI;
  long long jb, je;
  j_chunk(n, ci.rank, ci.size, T, jb, je);
  if constexpr (PACKED) {
    static_assert(BPT == 1 || BPT == 2, "packed loop: one or two bodies per thread");
    force_mixed_cta_jp<T, L, BPT>(packed, n, i0, jb, je, eps2, sh_raw, part);
  } else {
    PackedBody* sh = reinterpret_cast<PackedBody*>(sh_raw);
    if (uniform_mass)
      force_mixed_cta<T, L, BPT, true>(packed, n, i0, jb, je, eps2, sh, part);
    else
      force_mixed_cta<T, L, BPT, false>(packed, n, i0, jb, je, eps2, sh, part);
  }
  cluster_combine<BI>(part, ci.rank, ci.size);
  if (ci.rank != 0) return;
  const long long nb = min((long long)BI, n - i0);
  for (int e = threadIdx.x; e < 3 * nb; e += T) {
    const long long g = 3 * i0 + e;
    double a = part[e / 3][e % 3];
    if (uniform_mass) a = dmul(a, mass);
    out_vel[g] = vel[g];
    out_acc[g] = a;
  }
}

template <int T>
const void* pick_f64(int L) {
  switch (L) {
    case 1: return (const void*)rhs_f64_kernel<T, 1>;
    case 2: return (const void*)rhs_f64_kernel<T, 2>;
    case 4: return (const void*)rhs_f64_kernel<T, 4>;
    case 8: return (const void*)rhs_f64_kernel<T, 8>;
    default: return nullptr;
  }
}

template <int T, int BPT, bool PACKED>
const void* pick_mixed_L(int L) {
  switch (L) {
    case 1: return (const void*)rhs_mixed_kernel<T, 1, BPT, PACKED>;
    case 2: return (const void*)rhs_mixed_kernel<T, 2, BPT, PACKED>;
    case 4: return (const void*)rhs_mixed_kernel<T, 4, BPT, PACKED>;
    case 8: return (const void*)rhs_mixed_kernel<T, 8, BPT, PACKED>;
    default: return nullptr;
  }
}

// packed: the f32x2 path (pairs of bodies per thread, uniform masses)
template <int T>
const void* pick_mixed(int L, int BPT, bool packed = false) {
  if (packed && T <= 128 && BPT == 1) return pick_mixed_L<T, 1, true>(L);
  if (packed && T <= 128 && BPT == 2) return pick_mixed_L<T, 2, true>(L);
  switch (BPT) {
    case 1: return pick_mixed_L<T, 1, false>(L);
    case 2: return pick_mixed_L<T, 2, false>(L);
    default: return nullptr;
  }
}

// The packed loops run for uniform masses unless the tiling asks for the
// scalar loop (mixed_variant == 1).
bool use_packed(const gb_force_tiling* tiling, int BPT, const double* masses) {
  return (BPT == 1 || BPT == 2) && !masses && !(tiling && tiling->mixed_variant == 1);
}

int run_f64(const double* pos, const double* vel, double* out_vel, double* out_acc, long long n,
            double softening, double mass, const double* masses, int mode,
            const gb_force_tiling* tiling, cudaStream_t s) {
  ForceGeom g = choose_geom(n, GB_PREC_F64, tiling, 0);
  const void* k = nullptr;
  switch (g.T) {
    case 64: k = pick_f64<64>(g.L); break;
    case 128: k = pick_f64<128>(g.L); break;
    case 256: k = pick_f64<256>(g.L); break;
  }
  if (!k) return GB_ERR_UNSUPPORTED;
  double eps2 = softening * softening;
  // the standalone right-hand sides keep the reference's operation order
  // unless the tiling asks for the refined-rsqrt pair term
  int fast = (tiling && tiling->f64_pair == 1) ? 1 : 0;
  void* args[] = {(void*)&pos, (void*)&vel, (void*)&out_vel, (void*)&out_acc, (void*)&n,
                  (void*)&eps2, (void*)&mass, (void*)&masses, (void*)&mode, (void*)&fast};
  return launch_cluster(k, g, 0, s, args);
}

}  // namespace

// Right-hand side for the integrator's start-up (initial step estimate): FP64
// with the integrator's tiling, or mixed from an already packed state.
int rhs_for_start(int prec, const double* x, double* dxdt, long long n, double softening,
                  double mass, const double* masses, const PackedBody* packed, int exact,
                  const gb_force_tiling* tiling, cudaStream_t s) {
  if (prec == GB_PREC_F64) {
    gb_force_tiling t = {};
    if (tiling) t = *tiling;
    if (exact) {
      t.j_split = 1;
      t.lanes = 1;
    }
    return run_f64(x, x + 3 * n, dxdt, dxdt + 3 * n, n, softening, mass, masses, kModeRhs, &t,
                   s);
  }
  ForceGeom g = choose_geom(n, GB_PREC_MIXED, tiling, 0, masses == nullptr);
  const void* k = nullptr;
  switch (g.T) {
    case 64: k = pick_mixed<64>(g.L, g.BPT, use_packed(tiling, g.BPT, masses)); break;
    case 128: k = pick_mixed<128>(g.L, g.BPT, use_packed(tiling, g.BPT, masses)); break;
    case 256: k = pick_mixed<256>(g.L, g.BPT, use_packed(tiling, g.BPT, masses)); break;
  }
  if (!k) return GB_ERR_UNSUPPORTED;
  const double* vel = x + 3 * n;
  double* out_vel = dxdt;
  double* out_acc = dxdt + 3 * n;
  float eps2 = (float)(softening * softening);
  int uniform = masses ? 0 : 1;
  void* args[] = {(void*)&packed, (void*)&vel,  (void*)&out_vel, (void*)&out_acc,
                  (void*)&n,      (void*)&eps2, (void*)&mass,    (void*)&uniform};
  return launch_cluster(k, g, 0, s, args);
}

int launch_cluster(const void* kernel, const ForceGeom& g, size_t smem, cudaStream_t s,
                   void** args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(g.n_itiles * g.P), 1, 1);
  cfg.blockDim = dim3((unsigned)g.T, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)g.P;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (g.P > 8) {
    // clusters above 8 CTAs are opt-in per kernel; the attribute is set on
    // the first (uncaptured) launch and persists
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    GB_CUDA_TRY(cudaStreamIsCapturing(s, &cs));
    if (cs == cudaStreamCaptureStatusNone)
      GB_CUDA_TRY(
          cudaFuncSetAttribute(kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
  }
  GB_CUDA_TRY(cudaLaunchKernelExC(&cfg, kernel, args));
  return GB_OK;
}

ForceGeom choose_geom(long long n, int precision, const gb_force_tiling* tiling, int exact,
                      bool uniform_masses) {
  ForceGeom g;
  g.T = 128;
  g.L = 1;
  g.P = 1;
  g.BPT = 1;
  g.variant = 0;
  const int sms = num_sms();
  if (exact) {
    g.L = 1;
    g.P = 1;
  } else if (precision == GB_PREC_F64) {
    if (n >= 4096) {
      // 8 cluster ranks and lanes for about 2048 CTAs of 128 threads: the
      // FP64-pipe-bound pair loop then balances across the SMs (measured per
      // stage: N = 16384 23.9 ms at 8 x 2 against 25.5 ms at 4 x 1; N = 4096
      // 1.51 ms at 8 x 8 against 1.60 ms at 8 x 2)
      int L = 1;
      while (L < 8 && (long long)L * 2 * n <= 32768) L *= 2;
      g.P = 8;
      g.L = L;
    } else {
      // Aim for ~8 resident warps per SM over the whole grid.
      long long want = (long long)sms * 8 * 32;
      long long lp = (want + n - 1) / n;
      int P = 1;
      while (P < 8 && P < lp) P *= 2;
      int L = 1;
      while (L < 4 && (long long)P * L < lp) L *= 2;
      g.P = P;
      g.L = L;
    }
  } else {
    int v = tiling ? tiling->mixed_variant : 0;
    if (v < 1 || v > 3) v = kDefaultMixedVariant;
    if (!uniform_masses) v = 1;
    g.variant = v;
    g.BPT = v == 3 ? 1 : 2;
    // ~32 warps' worth of two-body threads per SM, each lane pair-loop at
    // least ~256 partners long; lanes only when the cluster split leaves the
    // grid well short of that (measured with the partner-pair loop: N = 4096
    // runs fastest at 8 ranks x 2 lanes, N = 16384 at 8 x 1, N = 65536 at 4 x 1).
    long long want = (long long)sms * 16 * 32 * 2;
    long long lp = (want + n - 1) / n;
    int P = 1;
    while (P < 8 && P < lp && n / (2 * P) >= 256) P *= 2;
    int L = 1;
    const int lmax = g.BPT == 1 ? 2 : 4;
    while (L < lmax && 2LL * P * L < lp && n / (2 * P * L) >= 128) L *= 2;
    g.P = P;
    g.L = L;
  }
  if (tiling) {
    if (tiling->j_split > 0) g.P = tiling->j_split;
    if (tiling->lanes > 0) g.L = tiling->lanes;
    if (tiling->bodies_per_cta > 0) {
      // bodies per CTA = (T / L) * BPT
      int t = tiling->bodies_per_cta * g.L / g.BPT;
      g.T = t <= 64 ? 64 : (t <= 128 ? 128 : 256);
    }
  }
  // the packed loops stage 2T partners per tile: 128 threads per CTA
  if (precision == GB_PREC_MIXED && g.variant != 1 && !exact) g.T = 128;
  const long long per_cta = g.bodies_per_cta();
  g.n_itiles = (n + per_cta - 1) / per_cta;
  return g;
}

}  // namespace gb

using namespace gb;

extern "C" int gb_nbody_rhs_f64(const double* x, double* dxdt, int64_t n, double softening,
                                double mass, const double* masses, const gb_force_tiling* tiling,
                                gb_stream_t stream) {
  GB_TRY(validate_nbody(x, dxdt, n, softening, mass, masses));
  return run_f64(x, x + 3 * n, dxdt, dxdt + 3 * n, n, softening, mass, masses, kModeRhs, tiling,
                 as_cuda(stream));
}

extern "C" int gb_nbody_acc_f64(const double* pos, double* acc, int64_t n, double softening,
                                double mass, const double* masses, int32_t accumulate,
                                const gb_force_tiling* tiling, gb_stream_t stream) {
  GB_TRY(validate_nbody(pos, acc, n, softening, mass, masses));
  return run_f64(pos, nullptr, nullptr, acc, n, softening, mass, masses,
                 accumulate ? kModeAccAdd : kModeAccWrite, tiling, as_cuda(stream));
}

namespace gb {
// Mixed-precision right-hand side into caller-located scratch: `packed`
// (n PackedBody records, 16-byte aligned) and `c` (3 doubles).  Both
// gb_nbody_rhs_mixed (workspace from the caller) and
// gb_nbody_rhs_mixed_noalloc (workspace inside the library) run through it,
// so the two give identical bits; allocates nothing.
int mixed_rhs_into(const double* x, double* dxdt, long long n, double softening, double mass,
                   const double* masses, PackedBody* packed, double* c,
                   const gb_force_tiling* tiling, cudaStream_t s) {
  centroid_kernel<<<1, 1024, 0, s>>>(x, n, c);
  GB_CUDA_TRY(cudaGetLastError());
  pack_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(x, masses, c, n, packed);
  GB_CUDA_TRY(cudaGetLastError());
  ForceGeom g = choose_geom(n, GB_PREC_MIXED, tiling, 0, masses == nullptr);
  const void* k = nullptr;
  switch (g.T) {
    case 64: k = pick_mixed<64>(g.L, g.BPT, use_packed(tiling, g.BPT, masses)); break;
    case 128: k = pick_mixed<128>(g.L, g.BPT, use_packed(tiling, g.BPT, masses)); break;
    case 256: k = pick_mixed<256>(g.L, g.BPT, use_packed(tiling, g.BPT, masses)); break;
  }
  if (!k) return GB_ERR_UNSUPPORTED;
  const double* vel = x + 3 * n;
  double* out_vel = dxdt;
  double* out_acc = dxdt + 3 * n;
  float eps2 = (float)(softening * softening);
  int uniform = masses ? 0 : 1;
  void* args[] = {(void*)&packed, (void*)&vel,  (void*)&out_vel, (void*)&out_acc,
                  (void*)&n,      (void*)&eps2, (void*)&mass,    (void*)&uniform};
  return launch_cluster(k, g, 0, s, args);
}
}  // namespace gb

namespace gb {
namespace {

// Mixed-precision right-hand side on Morton-sorted tiles (near hi/lo path
// plus the tile-centroid far path); rows are written back in body order.
template <int T, int L, bool UNIFORM>
__global__ void __launch_bounds__(T, 1024 / T)
    rhs_sorted_kernel(const PackedBody* __restrict__ near, const float4* __restrict__ far,
                      const TileMeta* __restrict__ meta, const int* __restrict__ perm,
                      const double* __restrict__ vel, double* __restrict__ out_vel,
                      double* __restrict__ out_acc, long long n, float eps2, double mass) {
  __shared__ __align__(16) PackedBody sh[T];
  __shared__ double part[T][3];
  const ClusterInfo ci = cluster_info();
  long long jb, je;
  j_chunk(n, ci.rank, ci.size, T, jb, je);
  force_mixed_sorted_cta<T, L, L, UNIFORM>(near, far, meta, n, ci.itile, jb, je, eps2, sh, part);
  cluster_combine<T>(part, ci.rank, ci.size);
  if (ci.rank != 0) return;
  const long long i = ci.itile * T + threadIdx.x;
  if (i >= n) return;
  const long long id = perm[i];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    out_vel[3 * id + c] = vel[3 * id + c];
    out_acc[3 * id + c] = UNIFORM ? dmul(part[threadIdx.x][c], mass) : part[threadIdx.x][c];
  }
}

struct SortedWork {
  PackedBody* near;
  float4* far;
  TileMeta* meta;
  SortBuffers sb;
  double* cref;
  size_t total;
};

size_t align256(size_t b) { return (b + 255) / 256 * 256; }

SortedWork sorted_layout(long long n, void* base) {
  const long long nt = (n + 127) / 128;
  char* p = static_cast<char*>(base);
  SortedWork w;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    char* q = p ? p + off : nullptr;
    off += align256(bytes);
    return q;
  };
  w.near = reinterpret_cast<PackedBody*>(take((size_t)n * sizeof(PackedBody)));
  w.far = reinterpret_cast<float4*>(take((size_t)n * sizeof(float4)));
  w.meta = reinterpret_cast<TileMeta*>(take((size_t)nt * sizeof(TileMeta)));
  w.sb.perm = reinterpret_cast<int*>(take((size_t)n * sizeof(int)));
  w.sb.vals = reinterpret_cast<int*>(take((size_t)n * sizeof(int)));
  w.sb.keys = reinterpret_cast<unsigned long long*>(take((size_t)n * 8));
  w.sb.keys_alt = reinterpret_cast<unsigned long long*>(take((size_t)n * 8));
  w.sb.bbox = reinterpret_cast<double*>(take(8 * sizeof(double)));
  w.cref = reinterpret_cast<double*>(take(4 * sizeof(double)));
  w.sb.cub_bytes = sort_temp_bytes(n);
  w.sb.cub_temp = take(w.sb.cub_bytes);
  w.total = off;
  return w;
}

template <int T, int L>
const void* pick_rhs_sorted(bool uniform) {
  return uniform ? (const void*)rhs_sorted_kernel<T, L, true>
                 : (const void*)rhs_sorted_kernel<T, L, false>;
}

}  // namespace
}  // namespace gb

extern "C" size_t gb_nbody_mixed_sorted_workspace_bytes(int64_t n) {
  return n < 1 ? 0 : gb::sorted_layout(n, nullptr).total;
}

extern "C" int gb_nbody_rhs_mixed_sorted(const double* x, double* dxdt, int64_t n,
                                         double softening, double mass, const double* masses,
                                         void* work, size_t work_bytes,
                                         const gb_force_tiling* tiling, gb_stream_t stream) {
  using namespace gb;
  GB_TRY(validate_nbody(x, dxdt, n, softening, mass, masses));
  if (!(softening > 0.0) || !work || (reinterpret_cast<uintptr_t>(work) & 255u))
    return GB_ERR_INVALID_ARGUMENT;
  SortedWork w = sorted_layout(n, work);
  if (work_bytes < w.total) return GB_ERR_CAPACITY;
  cudaStream_t s = as_cuda(stream);
  centroid_kernel<<<1, 1024, 0, s>>>(x, n, w.cref);
  GB_CUDA_TRY(cudaGetLastError());
  const long long nt = (n + 127) / 128;
  GB_TRY(sort_and_pack(x, nullptr, 0, n, w.sb, masses, w.cref, w.near, w.far, w.meta, nullptr,
                       nt, 128, s));
  ForceGeom g = choose_geom(n, GB_PREC_MIXED, tiling, 0, masses == nullptr);
  g.T = 128;
  if (g.L > 2) g.L = 2;
  g.BPT = g.L;
  g.n_itiles = nt;
  const void* k = g.L == 1 ? pick_rhs_sorted<128, 1>(masses == nullptr)
                           : pick_rhs_sorted<128, 2>(masses == nullptr);
  const PackedBody* near = w.near;
  const float4* far = w.far;
  const TileMeta* meta = w.meta;
  const int* perm = w.sb.perm;
  const double* vel = x + 3 * n;
  double* out_vel = dxdt;
  double* out_acc = dxdt + 3 * n;
  float eps2 = (float)(softening * softening);
  long long nn = n;
  void* args[] = {(void*)&near, (void*)&far, (void*)&meta, (void*)&perm, (void*)&vel,
                  (void*)&out_vel, (void*)&out_acc, (void*)&nn, (void*)&eps2, (void*)&mass};
  return launch_cluster(k, g, 0, s, args);
}

extern "C" size_t gb_nbody_mixed_workspace_bytes(int64_t n) {
  if (n < 1) return 0;
  // packed bodies + reference point (3 doubles), 256-byte aligned pieces
  size_t packed = ((size_t)n * sizeof(PackedBody) + 255) / 256 * 256;
  return packed + 256;
}

extern "C" int gb_nbody_rhs_mixed(const double* x, double* dxdt, int64_t n, double softening,
                                  double mass, const double* masses, void* work,
                                  const gb_force_tiling* tiling, gb_stream_t stream) {
  GB_TRY(validate_nbody(x, dxdt, n, softening, mass, masses));
  if (!work || (reinterpret_cast<uintptr_t>(work) & 15u)) return GB_ERR_INVALID_ARGUMENT;
  if (!(softening > 0.0)) return GB_ERR_INVALID_ARGUMENT;
  PackedBody* packed = reinterpret_cast<PackedBody*>(work);
  const size_t packed_bytes = ((size_t)n * sizeof(PackedBody) + 255) / 256 * 256;
  double* c = reinterpret_cast<double*>(reinterpret_cast<char*>(work) + packed_bytes);
  return mixed_rhs_into(x, dxdt, n, softening, mass, masses, packed, c, tiling, as_cuda(stream));
}
