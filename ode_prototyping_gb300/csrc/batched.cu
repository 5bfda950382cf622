// batched.cu -- many independent N-body systems of uneven size advanced
// together, each with its own step size, accept/reject decision and status.
//
// No counterpart in the reference (its state size is a compile-time
// constant, src/state/ODEState.hpp:7-23, so one integrate() call handles one
// system).  Each system follows the reference's loop
// (RKEmbeddedParallel.hpp:13-81) exactly as the single-system integrator
// does; only the scheduling differs:
//   * work units are (system, i-tile) pairs ordered by decreasing cost; a
//     persistent stage kernel (grid = a multiple of the SM count) takes them
//     round-robin, computes the tile's accelerations against all bodies of
//     its system and runs the shared stage epilogue;
//   * with G systems per CTA, systems small enough for one warp group's tile
//     share a CTA: each of G warp groups (own named barrier, own slice of
//     the shared buffers) integrates one whole small system;
//   * one warp per system reduces its tile partials in tile order and applies
//     that system's controller;
//   * an attempt (S stage launches + 1 control launch) is captured once in a
//     CUDA graph and replayed; systems that have reached tf skip their units;
//   * the tile geometry (threads, lanes, bodies per thread, systems per CTA)
//     and the grid size are chosen by an autotuner that times the candidates
//     on the actual batch.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <numeric>
#include <thread>
#include <vector>

#include "controller.cuh"
#include "epilogue.cuh"

namespace gb {

int launch_norm(const double* v, const double* s, long long n, double* partial, double* out,
                int take_sqrt, cudaStream_t st);

namespace {

struct BSys {
  long long n;          // bodies
  long long body_off;   // first body in the packed arrays
  long long var_off;    // first state element (6 * body_off)
  long long unit_off;   // first entry in sys_units
  int n_units;
  int pad;
  double eps2;
  float eps2f;
  float pad2;
  double mass;
  double atol, rtol;
};

struct BUnit {
  int sys;
  int tile;
};

struct BatchParams {
  const BSys* sys;
  const BUnit* units;
  const int2* work;      // work items: (first unit, 0) for a whole-CTA unit,
                         // (first unit, count) for count systems sharing a CTA
  long long n_work;
  const int* sys_units;  // unit ids of each system in tile order
  const int* body_sys;   // system of each body (packing)
  long long n_units;
  int n_sys;
  int exact;
  Ctrl* ctrl;
  double* ring;          // 2 * total_var
  double* ks;            // S * total_var
  double* Y;             // 2 * total_var
  PackedBody* PX;        // 2 * total_bodies
  PackedBody* PY;        // 2 * total_bodies
  double* cref;          // 3 per system
  double* partials;      // per unit
  double* aux;           // per unit
  unsigned* n_done;
  long long total_var, total_bodies;
  const void* mlp;       // learned proposer (device copy) or null
};

// Reductions over the TG threads of one group (the whole CTA or a warp
// group sharing it): the tree of block_sum / block_max.
template <int TG, class G>
__device__ __forceinline__ double group_sum(double v, double* red, const G& grp) {
  const unsigned t = grp.tid();
  red[t] = v;
  grp.sync();
  for (int st = TG / 2; st > 0; st /= 2) {
    if ((int)t < st) red[t] = dadd(red[t], red[t + st]);
    grp.sync();
  }
  const double r = red[0];
  grp.sync();
  return r;
}

template <int TG, class G>
__device__ __forceinline__ double group_max(double v, double* red, const G& grp) {
  const unsigned t = grp.tid();
  red[t] = v;
  grp.sync();
  for (int st = TG / 2; st > 0; st /= 2) {
    if ((int)t < st) red[t] = fmax(red[t], red[t + st]);
    grp.sync();
  }
  const double r = red[0];
  grp.sync();
  return r;
}

// Shared-memory bytes of the partner staging of TG threads.
template <int PREC, int TG>
constexpr int batch_smem_bytes() {
  return PREC == GB_PREC_F64 ? 32 * TG
                             : (TG <= 128 ? jp_smem_bytes<TG>() : (int)sizeof(PackedBody) * TG);
}

// One unit (system, i-tile) of one stage, run by TG threads (the whole CTA,
// or one warp group of it): the tile's accelerations against every body of
// its system, then the shared stage epilogue for the tile's bodies.
template <int PREC, int TG, int L, int BPT, class G>
__device__ __forceinline__ void stage_unit(const DevTableau& tab, const BatchParams& P, int s,
                                           long long u, unsigned char* sh_raw,
                                           double (*part)[3], double* red, const G& grp) {
  constexpr int BI = (TG / L) * BPT;
  // TG <= 128: the packed loop over pairs of partners (one or two bodies per thread)
  constexpr bool PK = PREC == GB_PREC_MIXED && TG <= 128;
  const int S = tab.n_stages;
  const BUnit un = P.units[u];
  const BSys sy = P.sys[un.sys];
  const Ctrl* C = P.ctrl + un.sys;
  if (C->done) return;
  const int cur = C->cur;
  const double dt = C->dt;
  const int k0_valid = C->k0_valid;
  const int k0slot = C->k0slot;
  const int px = C->px;
  const long long n = sy.n;
  const double* x0 = P.ring + (long long)cur * P.total_var + sy.var_off;
  const double* ysrc = (s == 0) ? x0 : P.Y + (long long)(s & 1) * P.total_var + sy.var_off;
  const long long i0 = (long long)un.tile * BI;
  const bool skip_force = (s == 0 && k0_valid);
  if (!skip_force) {
    if constexpr (PREC == GB_PREC_F64) {
      double* sh_pos = reinterpret_cast<double*>(sh_raw);
      force_f64_cta<TG, L>(ysrc, n, i0, 0, n, sy.eps2, nullptr, sh_pos, sh_pos + 3 * TG, part,
                           true, grp);
    } else {
      const PackedBody* src = (s == 0) ? P.PX + (long long)px * P.total_bodies + sy.body_off
                                       : P.PY + (long long)(s & 1) * P.total_bodies + sy.body_off;
      if constexpr (PK) {
        force_mixed_cta_jp<TG, L, BPT>(src, n, i0, 0, n, sy.eps2f, sh_raw, part, nullptr, 0,
                                       grp);
      } else {
        static_assert(std::is_same_v<G, WholeCta>, "scalar loop: whole CTAs only");
        force_mixed_cta<TG, L, BPT, true>(src, n, i0, 0, n, sy.eps2f,
                                          reinterpret_cast<PackedBody*>(sh_raw), part);
      }
    }
  }
  grp.sync();
  const bool last = (s == S - 1);
  EpiCtx E;
  E.tab = &tab;
  E.s = s;
  E.S = S;
  E.k0slot = k0slot;
  E.skip_force = skip_force;
  E.last = last;
  E.exact = false;
  E.dt = dt;
  E.n = n;
  E.x0 = x0;
  E.ysrc = ysrc;
  E.ks = P.ks + sy.var_off;
  E.kstride = P.total_var;
  E.ynext = P.Y + (long long)((s + 1) & 1) * P.total_var + sy.var_off;
  E.xnew = P.ring + (long long)((cur + 1) & 1) * P.total_var + sy.var_off;
  E.pnext = (last ? P.PX + (long long)(px ^ 1) * P.total_bodies
                  : P.PY + (long long)((s + 1) & 1) * P.total_bodies) +
            sy.body_off;
  E.atol = nullptr;
  E.rtol = nullptr;
  E.atol_s = sy.atol;
  E.rtol_s = sy.rtol;
  E.masses = nullptr;
  E.mass = sy.mass;
  E.cref = P.cref + 3 * un.sys;
  E.sq = nullptr;
  const long long nb = min((long long)BI, n - i0);
  double sq_acc = 0.0, amax = 0.0;
  for (int b = grp.tid(); b < nb; b += TG) body_epilogue<PREC>(E, i0 + b, part[b], sq_acc, amax);
  if (last) {
    const double m = group_max<TG>(amax, red, grp);
    if (grp.tid() == 0) P.aux[u] = m;
  }
  if (last) {
    const double ts = group_sum<TG>(sq_acc, red, grp);
    if (grp.tid() == 0) P.partials[u] = ts;
  }
  grp.sync();
}

// Persistent stage kernel over work items taken round-robin.  An item is one
// unit run by the whole CTA, or (G > 1) up to G small systems that share the
// CTA: warp group g of T / G threads, with its own named barrier and its own
// slice of the shared buffers, integrates one whole system (its single tile).
template <int PREC, int T, int L, int BPT, int G>
__global__ void __launch_bounds__(T)
    batch_stage_kernel(const __grid_constant__ DevTableau tab,
                       const __grid_constant__ BatchParams P, int s) {
  static_assert(G == 1 || (T / G >= 32 && T <= 128 && (T / G / L) * BPT >= 1),
                "systems per CTA: warp groups of the packed loop");
  constexpr int BI = (T / L) * BPT;
  constexpr int SMEM_BODY_BYTES = batch_smem_bytes<PREC, T>();
  __shared__ __align__(16) unsigned char sh_raw[SMEM_BODY_BYTES];
  __shared__ double part[BI][3];
  __shared__ double red[T];
  for (long long w = blockIdx.x; w < P.n_work; w += gridDim.x) {
    const int2 item = P.work[w];
    if constexpr (G == 1) {
      stage_unit<PREC, T, L, BPT>(tab, P, s, item.x, sh_raw, part, red, WholeCta{});
    } else if (item.y == 0) {
      stage_unit<PREC, T, L, BPT>(tab, P, s, item.x, sh_raw, part, red, WholeCta{});
    } else {
      constexpr int TG = T / G;
      const int g = (int)threadIdx.x / TG;
      if (g < item.y) {
        const WarpGroup<TG> grp{threadIdx.x % TG, 1 + g};
        stage_unit<PREC, TG, L, BPT>(tab, P, s, item.x + g,
                                     sh_raw + g * batch_smem_bytes<PREC, TG>(), part + g * (BI / G),
                                     red + g * TG, grp);
      }
      __syncthreads();
    }
  }
}

// One warp per system: ordered reduction of its tile partials, then the
// controller (lane 0); a learned proposal is evaluated by the whole warp.
__global__ void __launch_bounds__(128)
    batch_control_kernel(const __grid_constant__ DevTableau tab,
                         const __grid_constant__ BatchParams P) {
  __shared__ float feat[4][kIn];
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int k = blockIdx.x * 4 + warp;
  if (k >= P.n_sys) return;
  Ctrl* C = P.ctrl + k;
  if (C->done) return;
  const BSys sy = P.sys[k];
  const int S = tab.n_stages;
  double v = 0.0, m = 0.0;
  for (int t = lane; t < sy.n_units; t += 32) {
    const int u = P.sys_units[sy.unit_off + t];
    v = dadd(v, P.partials[u]);
    m = fmax(m, P.aux[u]);
  }
#pragma unroll
  for (int off = 16; off >= 1; off /= 2) {
    v = dadd(v, __shfl_xor_sync(0xffffffffu, v, off));
    m = fmax(m, __shfl_xor_sync(0xffffffffu, m, off));
  }
  const double err = sqrt(v / (double)(6 * sy.n));
  int want = 0;
  if (lane == 0) {
    Ctrl pre = *C;
    pre.max_abs_acc = m;
    want = P.mlp && pre.controller == GB_CTRL_LEARNED && isfinite(err) && err <= 1.0;
    if (want) {
      preview_history(pre, err, true);
      make_features(pre, tab, sy.n, feat[warp]);
    }
  }
  want = __shfl_sync(0xffffffffu, want, 0);
  __syncwarp();
  const float learned = want ? mlp_infer_warp(P.mlp, feat[warp]) : 0.f;
  if (lane == 0) {
    Ctrl c = *C;
    const int k0_valid = c.k0_valid;
    c.max_abs_acc = m;
    c.n_rhs += k0_valid ? S - 1 : S;
    if (k0_valid) c.n_rhs_saved += 1;
    const CtrlEnv env{nullptr, 0, nullptr, 2, sy.n};
    finish_attempt(tab, env, c, err, (double)learned, want != 0);
    *C = c;
    if (c.done) atomicAdd(P.n_done, 1u);
  }
}

// ---- start-up (per-system initial step, estimate_initial_step :170-200) ----
// One unit's right-hand side (positions' derivative = velocities, then the
// accelerations), run by TG threads.
template <int PREC, int TG, int L, int BPT, class G>
__device__ __forceinline__ void rhs_unit(const BatchParams& P, long long u,
                                         const double* __restrict__ x,
                                         const PackedBody* __restrict__ packed,
                                         double* __restrict__ out, unsigned char* sh_raw,
                                         double (*part)[3], const G& grp) {
  constexpr int BI = (TG / L) * BPT;
  constexpr bool PK = PREC == GB_PREC_MIXED && TG <= 128;
  const BUnit un = P.units[u];
  const BSys sy = P.sys[un.sys];
  const long long n = sy.n;
  const long long i0 = (long long)un.tile * BI;
  const double* xs = x + sy.var_off;
  if constexpr (PREC == GB_PREC_F64) {
    double* sh_pos = reinterpret_cast<double*>(sh_raw);
    force_f64_cta<TG, L>(xs, n, i0, 0, n, sy.eps2, nullptr, sh_pos, sh_pos + 3 * TG, part, false,
                         grp);
  } else {
    if constexpr (PK) {
      force_mixed_cta_jp<TG, L, BPT>(packed + sy.body_off, n, i0, 0, n, sy.eps2f, sh_raw, part,
                                     nullptr, 0, grp);
    } else {
      static_assert(std::is_same_v<G, WholeCta>, "scalar loop: whole CTAs only");
      force_mixed_cta<TG, L, BPT, true>(packed + sy.body_off, n, i0, 0, n, sy.eps2f,
                                        reinterpret_cast<PackedBody*>(sh_raw), part);
    }
  }
  grp.sync();
  const long long nb = min((long long)BI, n - i0);
  double* o = out + sy.var_off;
  for (int e = grp.tid(); e < 3 * nb; e += TG) {
    const long long g = 3 * i0 + e;
    o[g] = xs[3 * n + g];
    o[3 * n + g] = dmul(part[e / 3][e % 3], sy.mass);
  }
  grp.sync();
}

template <int PREC, int T, int L, int BPT, int G>
__global__ void __launch_bounds__(T)
    batch_rhs_kernel(const __grid_constant__ BatchParams P, const double* __restrict__ x,
                     const PackedBody* __restrict__ packed, double* __restrict__ out) {
  constexpr int BI = (T / L) * BPT;
  __shared__ __align__(16) unsigned char sh_raw[batch_smem_bytes<PREC, T>()];
  __shared__ double part[BI][3];
  for (long long w = blockIdx.x; w < P.n_work; w += gridDim.x) {
    const int2 item = P.work[w];
    if constexpr (G == 1) {
      rhs_unit<PREC, T, L, BPT>(P, item.x, x, packed, out, sh_raw, part, WholeCta{});
    } else if (item.y == 0) {
      rhs_unit<PREC, T, L, BPT>(P, item.x, x, packed, out, sh_raw, part, WholeCta{});
    } else {
      constexpr int TG = T / G;
      const int g = (int)threadIdx.x / TG;
      if (g < item.y) {
        const WarpGroup<TG> grp{threadIdx.x % TG, 1 + g};
        rhs_unit<PREC, TG, L, BPT>(P, item.x + g, x, packed, out,
                                   sh_raw + g * batch_smem_bytes<PREC, TG>(), part + g * (BI / G),
                                   grp);
      }
      __syncthreads();
    }
  }
}

__global__ void batch_centroid_kernel(const BatchParams P, const double* __restrict__ x) {
  __shared__ double sh[3][128];
  const BSys sy = P.sys[blockIdx.x];
  const double* p = x + sy.var_off;
  double a = 0, b = 0, c = 0;
  for (long long i = threadIdx.x; i < sy.n; i += blockDim.x) {
    a += p[3 * i];
    b += p[3 * i + 1];
    c += p[3 * i + 2];
  }
  sh[0][threadIdx.x] = a;
  sh[1][threadIdx.x] = b;
  sh[2][threadIdx.x] = c;
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st /= 2) {
    if ((int)threadIdx.x < st)
      for (int d = 0; d < 3; ++d) sh[d][threadIdx.x] += sh[d][threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x < 3) P.cref[3 * blockIdx.x + threadIdx.x] = sh[threadIdx.x][0] / (double)sy.n;
}

__global__ void batch_pack_kernel(const BatchParams P, const double* __restrict__ x,
                                  PackedBody* __restrict__ out) {
  const long long b = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (b >= P.total_bodies) return;
  const int k = P.body_sys[b];
  const BSys sy = P.sys[k];
  const long long i = b - sy.body_off;
  const double* p = x + sy.var_off;
  const double* c = P.cref + 3 * k;
  out[b] = pack_body(p[3 * i], p[3 * i + 1], p[3 * i + 2], c[0], c[1], c[2], 1.0f);
}

// mode 0: tg = |x0| rtol + atol; mode 1: x1 = x0 + f0 dt0(d); mode 2: df -= f0
__global__ void batch_elem_kernel(const BatchParams P, int mode, const double* __restrict__ a,
                                  const double* __restrict__ b, double* __restrict__ out,
                                  const double* __restrict__ d) {
  const int k = blockIdx.x;
  const BSys sy = P.sys[k];
  const long long nv = 6 * sy.n;
  double dt0 = 0.0;
  if (mode == 1) {
    const double d0 = d[3 * k], d1 = d[3 * k + 1];
    dt0 = (d0 < 1.0e-5 || d1 < 1.0e-5) ? 1.0e-6 : 0.01 * (d0 / d1);
  }
  for (long long e = threadIdx.x; e < nv; e += blockDim.x) {
    const long long g = sy.var_off + e;
    if (mode == 0) {
      out[g] = dadd(dmul(fabs(a[g]), sy.rtol), sy.atol);
    } else if (mode == 1) {
      out[g] = dadd(a[g], dmul(b[g], dt0));
    } else {
      out[g] = dsub(out[g], b[g]);
    }
  }
}

// Per-system RMS norm of v / s: one warp per system, fixed order.
__global__ void batch_norm_kernel(const BatchParams P, const double* __restrict__ v,
                                  const double* __restrict__ s, double* __restrict__ out,
                                  int slot) {
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int k = blockIdx.x * 4 + warp;
  if (k >= P.n_sys) return;
  const BSys sy = P.sys[k];
  const long long nv = 6 * sy.n;
  double acc = 0.0;
  for (long long e = lane; e < nv; e += 32) {
    const double q = __ddiv_rn(v[sy.var_off + e], s[sy.var_off + e]);
    acc = dadd(acc, dmul(q, q));
  }
#pragma unroll
  for (int off = 16; off >= 1; off /= 2) acc = dadd(acc, __shfl_xor_sync(0xffffffffu, acc, off));
  if (lane == 0) out[3 * k + slot] = sqrt(acc / (double)nv);
}

__global__ void batch_init_ctrl_kernel(const BatchParams P, const double* __restrict__ d,
                                       const double* __restrict__ t0v,
                                       const double* __restrict__ tfv, int p, int q, double safety,
                                       int controller, double pi_beta, int fsal,
                                       long long max_attempts) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= P.n_sys) return;
  const double d0 = d[3 * k], d1 = d[3 * k + 1];
  const double dt0 = (d0 < 1.0e-5 || d1 < 1.0e-5) ? 1.0e-6 : 0.01 * (d0 / d1);
  const double d2 = d[3 * k + 2] / dt0;
  const double dmax = d1 < d2 ? d2 : d1;
  double dt1;
  if (dmax <= 1.0e-15) {
    const double alt = dt0 * 1.0e-3;
    dt1 = alt < 1.0e-6 ? 1.0e-6 : alt;
  } else {
    dt1 = pow(0.01 / dmax, 1.0 / (1.0 + p));
  }
  const double big = 100.0 * dt0;
  Ctrl c;
  memset(&c, 0, sizeof c);
  c.t = t0v[k];
  c.t0 = t0v[k];
  c.tf = tfv[k];
  c.dt = dt1 < big ? dt1 : big;
  c.dt_initial = c.dt;
  c.safety = safety;
  c.q = q;
  c.controller = controller;
  c.pi_beta = pi_beta;
  c.pi_alpha = 1.0 / (1.0 + q) - 0.75 * pi_beta;
  c.err_prev = 1.0e-4;
  {
    // the learned proposer's tolerance feature (scalar tolerances per system)
    const double ts = fmax(P.sys[k].atol, P.sys[k].rtol);
    c.log_tol = ts > 0.0 ? log(ts) : 0.0;
  }
  c.fsal = fsal;
  c.k0_valid = 1;
  c.n_rhs = 2;
  c.max_attempts = max_attempts;
  for (int h = 0; h < 3; ++h) {
    c.dt_hist[h] = c.dt;
    c.err_hist[h] = 1.0;
  }
  init_log_cache(c, P.sys[k].n);
  c.done = (c.t < c.tf) ? 0 : 1;
  P.ctrl[k] = c;
  if (c.done) atomicAdd(P.n_done, 1u);
}

// ---- kernel tables ----------------------------------------------------------
struct BatchKernels {
  const void* stage;
  const void* rhs;
};

template <int PREC, int T, int L, int BPT, int G>
BatchKernels kernels_of() {
  return {(const void*)batch_stage_kernel<PREC, T, L, BPT, G>,
          (const void*)batch_rhs_kernel<PREC, T, L, BPT, G>};
}

// Geometries built into the library: (precision, threads, lanes, bodies per
// thread, systems per CTA).
bool pick_batch(int prec, int T, int L, int BPT, int G, BatchKernels* k) {
#define GB_BK(P_, T_, L_, B_, G_)                                            \
  if (prec == P_ && T == T_ && L == L_ && BPT == B_ && G == G_) {            \
    *k = kernels_of<P_, T_, L_, B_, G_>();                                   \
    return true;                                                             \
  }
  GB_BK(GB_PREC_MIXED, 128, 1, 1, 1) GB_BK(GB_PREC_MIXED, 128, 2, 1, 1)
  GB_BK(GB_PREC_MIXED, 128, 4, 1, 1) GB_BK(GB_PREC_MIXED, 128, 1, 2, 1)
  GB_BK(GB_PREC_MIXED, 128, 2, 2, 1) GB_BK(GB_PREC_MIXED, 128, 4, 2, 1)
  GB_BK(GB_PREC_MIXED, 256, 2, 1, 1) GB_BK(GB_PREC_MIXED, 256, 4, 1, 1)
  GB_BK(GB_PREC_MIXED, 256, 2, 2, 1) GB_BK(GB_PREC_MIXED, 256, 4, 2, 1)
  GB_BK(GB_PREC_MIXED, 64, 1, 1, 1) GB_BK(GB_PREC_MIXED, 64, 2, 1, 1)
  GB_BK(GB_PREC_MIXED, 128, 1, 1, 2) GB_BK(GB_PREC_MIXED, 128, 1, 1, 4)
  GB_BK(GB_PREC_MIXED, 128, 2, 1, 2) GB_BK(GB_PREC_MIXED, 128, 1, 2, 2)
  GB_BK(GB_PREC_MIXED, 128, 1, 2, 4) GB_BK(GB_PREC_MIXED, 128, 2, 2, 2)
  GB_BK(GB_PREC_MIXED, 64, 1, 1, 2)
  GB_BK(GB_PREC_F64, 128, 1, 1, 1) GB_BK(GB_PREC_F64, 128, 2, 1, 1)
  GB_BK(GB_PREC_F64, 128, 4, 1, 1) GB_BK(GB_PREC_F64, 64, 1, 1, 1)
  GB_BK(GB_PREC_F64, 64, 2, 1, 1)
  GB_BK(GB_PREC_F64, 128, 1, 1, 2) GB_BK(GB_PREC_F64, 128, 1, 1, 4)
  GB_BK(GB_PREC_F64, 128, 2, 1, 2) GB_BK(GB_PREC_F64, 64, 1, 1, 2)
#undef GB_BK
  return false;
}

}  // namespace
}  // namespace gb

// ---------------------------------------------------------------------------
// Host object
// ---------------------------------------------------------------------------
struct gb_batch_s {
  gb::DevTableau tab;
  gb_tableau htab;
  gb_batch_opts opts;
  int n_sys = 0, S = 0, A = 0;
  long long total_bodies = 0, total_var = 0;
  std::vector<long long> n;
  std::vector<double> soft, mass;
  // geometry
  int T = 128, L = 2, BPT = 1, G = 1, grid = 0;
  gb::BatchKernels k{};
  // device
  gb::BSys* sys = nullptr;
  gb::BUnit* units = nullptr;
  int2* work = nullptr;
  int* sys_units = nullptr;
  int* body_sys = nullptr;
  long long n_units = 0, n_work = 0, max_units = 0;
  gb::Ctrl* ctrl = nullptr;
  double *ring = nullptr, *ks = nullptr, *Y = nullptr, *cref = nullptr, *partials = nullptr,
         *aux = nullptr, *dscal = nullptr, *tv = nullptr;
  gb::PackedBody *PX = nullptr, *PY = nullptr;
  unsigned* n_done = nullptr;
  void* mlp_dev = nullptr;
  gb::Ctrl* hctrl = nullptr;
  unsigned* hdone = nullptr;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  cudaEvent_t ev = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  bool started = false;
  gb::BatchParams P{};
};

namespace gb {
namespace {

int wait_ev(cudaEvent_t ev, double timeout_s) {
  const auto t0 = std::chrono::steady_clock::now();
  for (;;) {
    cudaError_t e = cudaEventQuery(ev);
    if (e == cudaSuccess) return GB_OK;
    if (e != cudaErrorNotReady) {
      note_cuda_error(e);
      return GB_ERR_CUDA;
    }
    if (std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count() > timeout_s)
      return GB_ERR_TIMEOUT;
    std::this_thread::sleep_for(std::chrono::microseconds(20));
  }
}

// (Re)builds the unit list for the current geometry: units (system, i-tile)
// ordered by decreasing cost (tile bodies x system bodies).  With G systems
// per CTA, every system that fits one warp group's tile (n <= BI / G) is one
// unit, and such units are grouped G at a time, in cost order, into work
// items that share a CTA; every other unit is a work item of its own.  Work
// items are taken round-robin by the persistent grid.
int build_units(gb_batch_s* b) {
  const int BI = (b->T / b->L) * b->BPT;
  const int G = b->G;
  const long long small_n = G > 1 ? BI / G : 0;
  std::vector<BUnit> units;
  std::vector<long long> cost;
  for (int k = 0; k < b->n_sys; ++k) {
    const long long tiles = (b->n[k] + BI - 1) / BI;
    for (long long t = 0; t < tiles; ++t) {
      units.push_back({k, (int)t});
      cost.push_back(std::min<long long>(BI, b->n[k] - t * BI) * b->n[k]);
    }
  }
  std::vector<size_t> order(units.size());
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(),
                   [&](size_t x, size_t y) { return cost[x] > cost[y]; });
  std::vector<BUnit> sorted;
  std::vector<int2> work;
  std::vector<size_t> pending;
  sorted.reserve(units.size());
  auto flush_group = [&]() {
    if (pending.empty()) return;
    work.push_back(make_int2((int)sorted.size(), (int)pending.size()));
    for (size_t i : pending) sorted.push_back(units[i]);
    pending.clear();
  };
  for (size_t i : order) {
    if (G > 1 && b->n[units[i].sys] <= small_n) {
      pending.push_back(i);
      if ((int)pending.size() == G) flush_group();
    } else {
      work.push_back(make_int2((int)sorted.size(), 0));
      sorted.push_back(units[i]);
    }
  }
  flush_group();
  // unit ids of each system in tile order
  std::vector<BSys> hs(b->n_sys);
  std::vector<int> su(sorted.size());
  {
    std::vector<std::vector<int>> per(b->n_sys);
    for (size_t i = 0; i < sorted.size(); ++i) per[sorted[i].sys].push_back((int)i);
    long long off = 0, body = 0;
    for (int k = 0; k < b->n_sys; ++k) {
      std::sort(per[k].begin(), per[k].end(),
                [&](int x, int y) { return sorted[x].tile < sorted[y].tile; });
      BSys s;
      std::memset(&s, 0, sizeof s);
      s.n = b->n[k];
      s.body_off = body;
      s.var_off = 6 * body;
      s.unit_off = off;
      s.n_units = (int)per[k].size();
      s.eps2 = b->soft[k] * b->soft[k];
      s.eps2f = (float)s.eps2;
      s.mass = b->mass[k];
      hs[k] = s;
      for (int u : per[k]) su[off++] = u;
      body += b->n[k];
    }
  }
  b->n_units = (long long)sorted.size();
  if (b->n_units > b->max_units) return GB_ERR_UNSUPPORTED;
  // keep tolerances already set on the device copy
  std::vector<BSys> old(b->n_sys);
  GB_CUDA_TRY(cudaMemcpy(old.data(), b->sys, b->n_sys * sizeof(BSys), cudaMemcpyDeviceToHost));
  for (int k = 0; k < b->n_sys; ++k) {
    hs[k].atol = old[k].atol;
    hs[k].rtol = old[k].rtol;
  }
  GB_CUDA_TRY(cudaMemcpy(b->sys, hs.data(), hs.size() * sizeof(BSys), cudaMemcpyHostToDevice));
  GB_CUDA_TRY(cudaMemcpy(b->units, sorted.data(), sorted.size() * sizeof(BUnit),
                         cudaMemcpyHostToDevice));
  GB_CUDA_TRY(cudaMemcpy(b->work, work.data(), work.size() * sizeof(int2),
                         cudaMemcpyHostToDevice));
  b->n_work = (long long)work.size();
  b->P.n_work = b->n_work;
  GB_CUDA_TRY(cudaMemcpy(b->sys_units, su.data(), su.size() * sizeof(int),
                         cudaMemcpyHostToDevice));
  b->P.n_units = b->n_units;
  return GB_OK;
}

int set_geometry(gb_batch_s* b, int T, int L, int BPT, int G, int grid) {
  BatchKernels k;
  if (!pick_batch(b->opts.precision, T, L, BPT, G, &k)) return GB_ERR_UNSUPPORTED;
  b->T = T;
  b->L = L;
  b->BPT = BPT;
  b->G = G;
  b->k = k;
  b->grid = grid > 0 ? grid : num_sms() * 8;
  return build_units(b);
}

int launch_stage(gb_batch_s* b, int s) {
  void* args[] = {(void*)&b->tab, (void*)&b->P, (void*)&s};
  GB_CUDA_TRY(cudaLaunchKernel(b->k.stage, dim3(b->grid), dim3(b->T), args, 0, b->stream));
  return GB_OK;
}

int launch_attempt(gb_batch_s* b) {
  for (int s = 0; s < b->S; ++s) GB_TRY(launch_stage(b, s));
  batch_control_kernel<<<(b->n_sys + 3) / 4, 128, 0, b->stream>>>(b->tab, b->P);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

int rebuild_graph(gb_batch_s* b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->exec = nullptr;
  b->graph = nullptr;
  GB_CUDA_TRY(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  int rc = GB_OK;
  for (int a = 0; a < b->A && rc == GB_OK; ++a) rc = launch_attempt(b);
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(b->stream, &g);
  if (rc != GB_OK) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  GB_CUDA_TRY(e);
  b->graph = g;
  GB_CUDA_TRY(cudaGraphInstantiate(&b->exec, g, 0));
  return GB_OK;
}

int launch_rhs(gb_batch_s* b, const double* x, const PackedBody* packed, double* out) {
  void* args[] = {(void*)&b->P, (void*)&x, (void*)&packed, (void*)&out};
  GB_CUDA_TRY(cudaLaunchKernel(b->k.rhs, dim3(b->grid), dim3(b->T), args, 0, b->stream));
  return GB_OK;
}

int read_ctrl(gb_batch_s* b) {
  GB_CUDA_TRY(cudaMemcpyAsync(b->hctrl, b->ctrl, b->n_sys * sizeof(Ctrl), cudaMemcpyDeviceToHost,
                              b->stream));
  GB_CUDA_TRY(cudaMemcpyAsync(b->hdone, b->n_done, sizeof(unsigned), cudaMemcpyDeviceToHost,
                              b->stream));
  GB_CUDA_TRY(cudaEventRecord(b->ev, b->stream));
  return wait_ev(b->ev, b->opts.host_wait_timeout_s);
}

void free_batch(gb_batch_s* b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  void* bufs[] = {b->sys,  b->units, b->work,     b->sys_units, b->body_sys, b->ctrl,
                  b->ring, b->ks,    b->Y,        b->cref,      b->partials, b->aux,
                  b->dscal, b->tv,   b->PX,       b->PY,        b->n_done,   b->mlp_dev};
  for (void* p : bufs)
    if (p) cudaFree(p);
  if (b->hctrl) cudaFreeHost(b->hctrl);
  if (b->hdone) cudaFreeHost(b->hdone);
  if (b->ev) cudaEventDestroy(b->ev);
  if (b->stream && b->own_stream) cudaStreamDestroy(b->stream);
}

}  // namespace
}  // namespace gb

using namespace gb;

extern "C" int gb_batch_create(const gb_tableau* tab, int32_t n_sys, const int64_t* n_particles,
                               const double* softening, const double* mass,
                               const gb_batch_opts* opts_in, gb_stream_t stream, gb_batch* out) {
  if (!out) return GB_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  GB_TRY(check_tableau(tab));
  if (n_sys < 1 || !n_particles || !softening || !mass) return GB_ERR_INVALID_ARGUMENT;
  gb_batch_opts opts;
  std::memset(&opts, 0, sizeof opts);
  if (opts_in) opts = *opts_in;
  if (opts.precision != GB_PREC_F64 && opts.precision != GB_PREC_MIXED)
    return GB_ERR_INVALID_ARGUMENT;
  if (opts.controller < GB_CTRL_REFERENCE || opts.controller > GB_CTRL_LEARNED)
    return GB_ERR_INVALID_ARGUMENT;
  if (opts.controller == GB_CTRL_LEARNED && !opts.mlp) return GB_ERR_INVALID_ARGUMENT;
  if (opts.attempts_per_sync <= 0) opts.attempts_per_sync = 8;
  if (opts.host_wait_timeout_s <= 0.0) opts.host_wait_timeout_s = 600.0;
  if (opts.pi_beta <= 0.0) opts.pi_beta = 0.04;
  auto* b = new gb_batch_s();
  b->htab = *tab;
  b->tab = make_dev_tableau(*tab);
  if (!opts.fsal) b->tab.fsal = 0;
  b->opts = opts;
  b->n_sys = n_sys;
  b->S = tab->n_stages;
  b->A = opts.attempts_per_sync;
  b->n.assign(n_particles, n_particles + n_sys);
  b->soft.assign(softening, softening + n_sys);
  b->mass.assign(mass, mass + n_sys);
  auto fail = [&](int code) {
    free_batch(b);
    delete b;
    return code;
  };
  std::vector<int> body_sys;
  for (int k = 0; k < n_sys; ++k) {
    if (b->n[k] < 1 || !(b->soft[k] >= 0.0) || !(b->mass[k] > 0.0))
      return fail(GB_ERR_INVALID_ARGUMENT);
    if (opts.precision == GB_PREC_MIXED && !(b->soft[k] > 0.0)) return fail(GB_ERR_INVALID_ARGUMENT);
    b->total_bodies += b->n[k];
    for (long long i = 0; i < b->n[k]; ++i) body_sys.push_back(k);
  }
  b->total_var = 6 * b->total_bodies;
  // the smallest tile any candidate geometry uses is 32 bodies
  b->max_units = 0;
  for (int k = 0; k < n_sys; ++k) b->max_units += (b->n[k] + 31) / 32;
  const long long tv = b->total_var, tb = b->total_bodies;
  cudaError_t e = cudaSuccess;
  auto alloc = [&](void** p, size_t bytes) {
    if (e == cudaSuccess) e = cudaMalloc(p, bytes);
  };
  alloc((void**)&b->sys, n_sys * sizeof(BSys));
  alloc((void**)&b->units, b->max_units * sizeof(BUnit));
  alloc((void**)&b->work, b->max_units * sizeof(int2));
  alloc((void**)&b->sys_units, b->max_units * sizeof(int));
  alloc((void**)&b->body_sys, tb * sizeof(int));
  alloc((void**)&b->ctrl, n_sys * sizeof(Ctrl));
  alloc((void**)&b->ring, 2 * tv * sizeof(double));
  alloc((void**)&b->ks, (size_t)b->S * tv * sizeof(double));
  alloc((void**)&b->Y, 2 * tv * sizeof(double));
  alloc((void**)&b->cref, 3 * n_sys * sizeof(double));
  alloc((void**)&b->partials, b->max_units * sizeof(double));
  alloc((void**)&b->aux, b->max_units * sizeof(double));
  alloc((void**)&b->dscal, 3 * n_sys * sizeof(double));
  alloc((void**)&b->tv, 2 * n_sys * sizeof(double));
  alloc((void**)&b->n_done, sizeof(unsigned));
  if (opts.precision == GB_PREC_MIXED) {
    alloc((void**)&b->PX, 2 * tb * sizeof(PackedBody));
    alloc((void**)&b->PY, 2 * tb * sizeof(PackedBody));
  }
  if (e == cudaSuccess) e = cudaMallocHost((void**)&b->hctrl, n_sys * sizeof(Ctrl));
  if (e == cudaSuccess) e = cudaMallocHost((void**)&b->hdone, sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMemset(b->sys, 0, n_sys * sizeof(BSys));
  if (e == cudaSuccess) e = cudaMemset(b->ctrl, 0, n_sys * sizeof(Ctrl));
  if (e == cudaSuccess)
    e = cudaMemcpy(b->body_sys, body_sys.data(), tb * sizeof(int), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    if (stream) {
      b->stream = as_cuda(stream);
    } else {
      e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
      b->own_stream = true;
    }
  }
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev, cudaEventDisableTiming);
  if (e != cudaSuccess) {
    note_cuda_error(e);
    return fail(GB_ERR_CUDA);
  }
  BatchParams& P = b->P;
  P.sys = b->sys;
  P.units = b->units;
  P.work = b->work;
  P.sys_units = b->sys_units;
  P.body_sys = b->body_sys;
  P.n_sys = n_sys;
  P.ctrl = b->ctrl;
  P.ring = b->ring;
  P.ks = b->ks;
  P.Y = b->Y;
  P.PX = b->PX;
  P.PY = b->PY;
  P.cref = b->cref;
  P.partials = b->partials;
  P.aux = b->aux;
  P.n_done = b->n_done;
  P.total_var = tv;
  P.total_bodies = tb;
  if (opts.controller == GB_CTRL_LEARNED) {
    int mrc = GB_OK;
    b->mlp_dev = mlp_upload(opts.mlp, &mrc);
    if (!b->mlp_dev) return fail(mrc == GB_OK ? GB_ERR_INVALID_ARGUMENT : mrc);
    P.mlp = b->mlp_dev;
  }
  const int T = opts.tiling.threads_per_cta > 0 ? opts.tiling.threads_per_cta : 128;
  const int L = opts.tiling.lanes > 0 ? opts.tiling.lanes : 2;
  const int BPT = opts.precision == GB_PREC_F64
                      ? 1
                      : (opts.tiling.bodies_per_thread > 0 ? opts.tiling.bodies_per_thread : 1);
  const int G = opts.tiling.systems_per_cta > 0 ? opts.tiling.systems_per_cta : 1;
  int rc = set_geometry(b, T, L, BPT, G, opts.tiling.grid_ctas);
  if (rc != GB_OK) return fail(rc);
  *out = b;
  return GB_OK;
}

extern "C" int gb_batch_start(gb_batch b, const double* x0, const double* t0, const double* tf,
                              const double* atol, const double* rtol) {
  if (!b || !x0 || !t0 || !tf || !atol || !rtol) return GB_ERR_INVALID_ARGUMENT;
  const int ns = b->n_sys;
  const long long tv = b->total_var, tb = b->total_bodies;
  std::vector<BSys> hs(ns);
  GB_CUDA_TRY(cudaMemcpy(hs.data(), b->sys, ns * sizeof(BSys), cudaMemcpyDeviceToHost));
  for (int k = 0; k < ns; ++k) {
    if (!(atol[k] >= 0.0) || !(rtol[k] >= 0.0)) return GB_ERR_INVALID_ARGUMENT;
    hs[k].atol = atol[k];
    hs[k].rtol = rtol[k];
  }
  GB_CUDA_TRY(cudaMemcpy(b->sys, hs.data(), ns * sizeof(BSys), cudaMemcpyHostToDevice));
  std::vector<double> tt(2 * ns);
  std::copy(t0, t0 + ns, tt.begin());
  std::copy(tf, tf + ns, tt.begin() + ns);
  cudaStream_t s = b->stream;
  GB_CUDA_TRY(cudaMemcpyAsync(b->tv, tt.data(), 2 * ns * sizeof(double), cudaMemcpyHostToDevice, s));
  GB_CUDA_TRY(cudaMemsetAsync(b->n_done, 0, sizeof(unsigned), s));
  GB_CUDA_TRY(cudaMemcpyAsync(b->ring, x0, tv * sizeof(double), cudaMemcpyDeviceToDevice, s));
  const BatchParams& P = b->P;
  if (b->opts.precision == GB_PREC_MIXED) {
    batch_centroid_kernel<<<ns, 128, 0, s>>>(P, b->ring);
    batch_pack_kernel<<<(unsigned)((tb + 255) / 256), 256, 0, s>>>(P, b->ring, b->PX);
    GB_CUDA_TRY(cudaGetLastError());
  }
  double* tg = b->Y;
  double* x1 = b->Y + tv;
  double* f0 = b->ks;
  double* df = b->ks + tv;
  batch_elem_kernel<<<ns, 256, 0, s>>>(P, 0, b->ring, nullptr, tg, nullptr);
  GB_TRY(launch_rhs(b, b->ring, b->PX, f0));
  batch_norm_kernel<<<(ns + 3) / 4, 128, 0, s>>>(P, b->ring, tg, b->dscal, 0);
  batch_norm_kernel<<<(ns + 3) / 4, 128, 0, s>>>(P, f0, tg, b->dscal, 1);
  batch_elem_kernel<<<ns, 256, 0, s>>>(P, 1, b->ring, f0, x1, b->dscal);
  if (b->opts.precision == GB_PREC_MIXED)
    batch_pack_kernel<<<(unsigned)((tb + 255) / 256), 256, 0, s>>>(P, x1, b->PY);
  GB_TRY(launch_rhs(b, x1, b->PY, df));
  batch_elem_kernel<<<ns, 256, 0, s>>>(P, 2, nullptr, f0, df, nullptr);
  batch_norm_kernel<<<(ns + 3) / 4, 128, 0, s>>>(P, df, tg, b->dscal, 2);
  const int q = std::min(b->htab.p, b->htab.pt);
  const double safety = std::pow(0.38, 1.0 / (1.0 + q));
  batch_init_ctrl_kernel<<<(ns + 127) / 128, 128, 0, s>>>(P, b->dscal, b->tv, b->tv + ns,
                                                          b->htab.p, q, safety,
                                                          b->opts.controller, b->opts.pi_beta,
                                                          b->tab.fsal, b->opts.max_attempts);
  GB_CUDA_TRY(cudaGetLastError());
  if (!b->exec) GB_TRY(rebuild_graph(b));
  GB_TRY(read_ctrl(b));
  b->started = true;
  return GB_OK;
}

extern "C" int gb_batch_enqueue(gb_batch b, int64_t n_replays) {
  if (!b || !b->started) return GB_ERR_INVALID_ARGUMENT;
  for (int64_t r = 0; r < n_replays; ++r) GB_CUDA_TRY(cudaGraphLaunch(b->exec, b->stream));
  return GB_OK;
}

extern "C" int gb_batch_sync(gb_batch b) {
  if (!b) return GB_ERR_INVALID_ARGUMENT;
  return read_ctrl(b);
}

extern "C" int gb_batch_advance(gb_batch b, int64_t max_replays) {
  if (!b || !b->started) return GB_ERR_INVALID_ARGUMENT;
  int64_t r = 0;
  while (*b->hdone < (unsigned)b->n_sys) {
    if (max_replays > 0 && r >= max_replays) break;
    GB_CUDA_TRY(cudaGraphLaunch(b->exec, b->stream));
    ++r;
    GB_TRY(read_ctrl(b));
  }
  for (int k = 0; k < b->n_sys; ++k)
    if (b->hctrl[k].status != GB_OK) return b->hctrl[k].status;
  return GB_OK;
}

extern "C" int gb_batch_stats(gb_batch b, gb_integrate_stats* totals, gb_integrate_stats* per_sys) {
  if (!b) return GB_ERR_INVALID_ARGUMENT;
  gb_integrate_stats tot;
  std::memset(&tot, 0, sizeof tot);
  tot.t = 1e300;
  for (int k = 0; k < b->n_sys; ++k) {
    const Ctrl& c = b->hctrl[k];
    gb_integrate_stats s;
    std::memset(&s, 0, sizeof s);
    s.n_accepted = c.n_accepted;
    s.n_rejected = c.n_rejected;
    s.n_attempts = c.n_attempts;
    s.n_rhs = c.n_rhs;
    s.n_rhs_saved = c.n_rhs_saved;
    s.t = c.t;
    s.dt = c.dt;
    s.dt_initial = c.dt_initial;
    s.err_last = c.err;
    s.interactions = (double)c.n_rhs * (double)b->n[k] * (double)(b->n[k] - 1);
    s.status = c.status;
    s.done = c.done;
    s.n_learned_proposals = c.n_learned;
    s.n_learned_rejected = c.n_learned_rejected;
    if (per_sys) per_sys[k] = s;
    tot.n_accepted += s.n_accepted;
    tot.n_rejected += s.n_rejected;
    tot.n_attempts += s.n_attempts;
    tot.n_rhs += s.n_rhs;
    tot.n_rhs_saved += s.n_rhs_saved;
    tot.interactions += s.interactions;
    tot.n_learned_proposals += s.n_learned_proposals;
    tot.n_learned_rejected += s.n_learned_rejected;
    tot.t = std::min(tot.t, s.t);
    if (s.status != GB_OK) tot.status = s.status;
  }
  tot.done = *b->hdone >= (unsigned)b->n_sys;
  if (totals) *totals = tot;
  return GB_OK;
}

extern "C" int gb_batch_state(gb_batch b, double* x_dev, double* t_host) {
  if (!b || !b->started) return GB_ERR_INVALID_ARGUMENT;
  GB_TRY(read_ctrl(b));
  std::vector<BSys> hs(b->n_sys);
  GB_CUDA_TRY(cudaMemcpy(hs.data(), b->sys, b->n_sys * sizeof(BSys), cudaMemcpyDeviceToHost));
  for (int k = 0; k < b->n_sys; ++k) {
    const Ctrl& c = b->hctrl[k];
    if (x_dev)
      GB_CUDA_TRY(cudaMemcpyAsync(x_dev + hs[k].var_off,
                                  b->ring + (long long)c.cur * b->total_var + hs[k].var_off,
                                  6 * hs[k].n * sizeof(double), cudaMemcpyDeviceToDevice,
                                  b->stream));
    if (t_host) t_host[k] = c.t;
  }
  GB_CUDA_TRY(cudaStreamSynchronize(b->stream));
  return GB_OK;
}

extern "C" int gb_batch_launch_stage(gb_batch b, int32_t stage) {
  if (!b || !b->started || stage < 0 || stage >= b->S) return GB_ERR_INVALID_ARGUMENT;
  return launch_stage(b, stage);
}

// Times every candidate geometry on the batch (stage 1, `reps` launches each)
// and keeps the fastest; rebuilds the unit list and the graph.  Must follow
// gb_batch_start (the stage buffers must hold a valid attempt).  Candidates
// with several systems per CTA are timed only where some system fits a warp
// group's tile (otherwise they are the one-system geometry again).
extern "C" int gb_batch_autotune(gb_batch b, int32_t reps, gb_batch_tiling* chosen,
                                 double* best_ms) {
  if (!b || !b->started || b->S < 3) return GB_ERR_INVALID_ARGUMENT;
  if (reps < 1) reps = 3;
  struct Cand {
    int T, L, BPT, G, gridmul;
  };
  std::vector<Cand> cands;
  const int sms = num_sms();
  const long long n_min = *std::min_element(b->n.begin(), b->n.end());
  auto add = [&](int T, int L, int BPT, int G) {
    if (G > 1 && n_min > (long long)((T / L) * BPT / G)) return;
    for (int gm : {4, 8, 16}) cands.push_back({T, L, BPT, G, gm});
  };
  if (b->opts.precision == GB_PREC_MIXED) {
    const int tl[][4] = {{128, 1, 1, 1}, {128, 2, 1, 1}, {128, 4, 1, 1}, {128, 1, 2, 1},
                         {128, 2, 2, 1}, {128, 4, 2, 1}, {256, 2, 1, 1}, {256, 4, 1, 1},
                         {256, 2, 2, 1}, {256, 4, 2, 1}, {64, 1, 1, 1},  {64, 2, 1, 1},
                         {128, 1, 1, 2}, {128, 1, 1, 4}, {128, 2, 1, 2}, {128, 1, 2, 2},
                         {128, 1, 2, 4}, {128, 2, 2, 2}, {64, 1, 1, 2}};
    for (auto& t : tl) add(t[0], t[1], t[2], t[3]);
  } else {
    const int tl[][4] = {{128, 1, 1, 1}, {128, 2, 1, 1}, {128, 4, 1, 1}, {64, 1, 1, 1},
                         {64, 2, 1, 1},  {128, 1, 1, 2}, {128, 1, 1, 4}, {128, 2, 1, 2},
                         {64, 1, 1, 2}};
    for (auto& t : tl) add(t[0], t[1], t[2], t[3]);
  }
  cudaEvent_t e0, e1;
  GB_CUDA_TRY(cudaEventCreate(&e0));
  GB_CUDA_TRY(cudaEventCreate(&e1));
  double best = 1e300;
  Cand bc = {b->T, b->L, b->BPT, b->G, b->grid / sms};
  for (const Cand& c : cands) {
    if (set_geometry(b, c.T, c.L, c.BPT, c.G, c.gridmul * sms) != GB_OK) continue;
    GB_TRY(launch_stage(b, 1));  // warm
    GB_CUDA_TRY(cudaEventRecord(e0, b->stream));
    for (int r = 0; r < reps; ++r) GB_TRY(launch_stage(b, 1 + r % (b->S - 2)));
    GB_CUDA_TRY(cudaEventRecord(e1, b->stream));
    GB_CUDA_TRY(cudaEventSynchronize(e1));
    float ms = 0.f;
    GB_CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
    if (ms / reps < best) {
      best = ms / reps;
      bc = c;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  GB_TRY(set_geometry(b, bc.T, bc.L, bc.BPT, bc.G, bc.gridmul * sms));
  GB_TRY(rebuild_graph(b));
  if (chosen) {
    chosen->threads_per_cta = bc.T;
    chosen->lanes = bc.L;
    chosen->bodies_per_thread = bc.BPT;
    chosen->grid_ctas = bc.gridmul * sms;
    chosen->systems_per_cta = bc.G;
  }
  if (best_ms) *best_ms = best;
  return GB_OK;
}

extern "C" int gb_batch_geometry(gb_batch b, gb_batch_tiling* t, int64_t* n_units) {
  if (!b || !t) return GB_ERR_INVALID_ARGUMENT;
  t->threads_per_cta = b->T;
  t->lanes = b->L;
  t->bodies_per_thread = b->BPT;
  t->grid_ctas = b->grid;
  t->systems_per_cta = b->G;
  if (n_units) *n_units = b->n_units;
  return GB_OK;
}

extern "C" int gb_batch_destroy(gb_batch b) {
  if (!b) return GB_OK;
  cudaStreamSynchronize(b->stream);
  free_batch(b);
  delete b;
  return GB_OK;
}
