// epilogue.cuh -- row-local work that follows the accelerations of one stage:
// the stage derivative k_s = (v, a), then either the next stage state
//   y_{s+1} = x0 + dt * sum_{l<=s} a[s][l] k_l       (rk_stage_kernel,
//   RKEmbeddedParallel.hpp:91-101), or, after the last stage,
//   x = x0 + dt * sum b_l k_l,  err = dt * sum (b_l - bt_l) k_l   (:103-123),
//   target = atol + rtol * max(|x|, |x0|)                          (:125-130),
//   (err / target)^2                                              (:132-137),
// each in the reference's accumulation order with IEEE operations.  Used by
// the single-system fused kernel and by the batched kernel.
#pragma once

#include "integrator.cuh"

namespace gb {

__device__ __forceinline__ int kslot(int l, int S, int k0slot) {
  if (l == 0) return k0slot;
  if (l == S - 1) return k0slot == 0 ? S - 1 : 0;
  return l;
}

__device__ __forceinline__ double block_sum(double v, double* red) {
  red[threadIdx.x] = v;
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st /= 2) {
    if ((int)threadIdx.x < st) red[threadIdx.x] = dadd(red[threadIdx.x], red[threadIdx.x + st]);
    __syncthreads();
  }
  double r = red[0];
  __syncthreads();
  return r;
}

__device__ __forceinline__ double block_max(double v, double* red) {
  red[threadIdx.x] = v;
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st /= 2) {
    if ((int)threadIdx.x < st) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + st]);
    __syncthreads();
  }
  double r = red[0];
  __syncthreads();
  return r;
}

struct EpiCtx {
  const DevTableau* tab;
  int s, S, k0slot;
  bool skip_force, last, exact;
  double dt;
  long long n;           // bodies of the system
  const double* x0;      // all pointers below are already offset to the system
  const double* ysrc;    // stage state whose velocities give dx/dt
  double* ks;            // stage slot l is ks + l * kstride
  long long kstride;
  double* ynext;         // y_{s+1}
  double* xnew;          // candidate state (last stage)
  PackedBody* pnext;     // packed positions of y_{s+1} or x (mixed path)
  const double* atol;    // per-element tolerances or null (scalars below)
  const double* rtol;
  double atol_s, rtol_s;
  const double* masses;  // per-body masses or null (uniform `mass`)
  double mass;
  const double* cref;    // hi/lo reference point
  double* sq;            // per-element squares (exact mode) or null
};

// One body's six state elements.  `acc` is the unscaled pair sum (ignored
// when the stage derivative is reused).  Adds the body's scaled squares to
// sq_acc and its |a| to amax (both at the last stage).
template <int PREC>
__device__ __forceinline__ void body_epilogue(const EpiCtx& E, long long i, const double* acc,
                                              double& sq_acc, double& amax,
                                              double* newpos = nullptr) {
  const DevTableau& tab = *E.tab;
  const int s = E.s, S = E.S;
  const long long n = E.n;
  long long idx[6];
  double k[6];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    idx[c] = 3 * i + c;
    idx[3 + c] = 3 * n + 3 * i + c;
  }
  double* ks_s = E.ks + (long long)kslot(s, S, E.k0slot) * E.kstride;
  if (E.skip_force) {
#pragma unroll
    for (int e = 0; e < 6; ++e) k[e] = ks_s[idx[e]];
  } else {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      k[c] = E.ysrc[idx[3 + c]];  // dx/dt = v (nbody_init_dxdt_kernel)
      k[3 + c] = E.masses ? acc[c] : dmul(acc[c], E.mass);
    }
#pragma unroll
    for (int e = 0; e < 6; ++e) ks_s[idx[e]] = k[e];
    if (E.last) amax = fmax(amax, sqrt(k[3] * k[3] + k[4] * k[4] + k[5] * k[5]));
  }
  // Stage sums: the stage index runs outermost so that a stage's six loads
  // are in flight together; every element still sums its terms from 0.0 in
  // ascending stage order.
  double x0v[6];
#pragma unroll
  for (int e = 0; e < 6; ++e) x0v[e] = E.x0[idx[e]];
  if (!E.last) {
    double yn[6], v[6];
#pragma unroll
    for (int e = 0; e < 6; ++e) v[e] = 0.0;
#pragma unroll 1
    for (int l = 0; l <= s; ++l) {
      if (!((tab.anz[s] >> l) & 1u)) continue;
      const double a = tab.a[s][l];
      double kl[6];
      if (l == s) {
#pragma unroll
        for (int e = 0; e < 6; ++e) kl[e] = k[e];
      } else {
        const double* kp = E.ks + (long long)kslot(l, S, E.k0slot) * E.kstride;
#pragma unroll
        for (int e = 0; e < 6; ++e) kl[e] = kp[idx[e]];
      }
#pragma unroll
      for (int e = 0; e < 6; ++e) v[e] = dadd(v[e], dmul(a, kl[e]));
    }
#pragma unroll
    for (int e = 0; e < 6; ++e) {
      yn[e] = dadd(x0v[e], dmul(v[e], E.dt));
      E.ynext[idx[e]] = yn[e];
    }
    if (newpos) {
      newpos[0] = yn[0];
      newpos[1] = yn[1];
      newpos[2] = yn[2];
    } else if constexpr (PREC == GB_PREC_MIXED) {
      const float w = E.masses ? (float)E.masses[i] : 1.0f;
      E.pnext[i] = pack_body(yn[0], yn[1], yn[2], E.cref[0], E.cref[1], E.cref[2], w);
    }
  } else {
    double xn[6], xv[6], ev[6];
#pragma unroll
    for (int e = 0; e < 6; ++e) xv[e] = ev[e] = 0.0;
#pragma unroll 1
    for (int l = 0; l < S; ++l) {
      const unsigned bl = (tab.bnz >> l) & 1u, dl = (tab.dbnz >> l) & 1u;
      if (!(bl | dl)) continue;
      const double bb = tab.b[l], db = tab.db[l];
      double kl[6];
      if (l == s) {
#pragma unroll
        for (int e = 0; e < 6; ++e) kl[e] = k[e];
      } else {
        const double* kp = E.ks + (long long)kslot(l, S, E.k0slot) * E.kstride;
#pragma unroll
        for (int e = 0; e < 6; ++e) kl[e] = kp[idx[e]];
      }
#pragma unroll
      for (int e = 0; e < 6; ++e) {
        if (bl) xv[e] = dadd(xv[e], dmul(bb, kl[e]));
        if (dl) ev[e] = dadd(ev[e], dmul(db, kl[e]));
      }
    }
#pragma unroll
    for (int e = 0; e < 6; ++e) {
      const double x0e = x0v[e];
      xn[e] = dadd(x0e, dmul(xv[e], E.dt));
      const double er = dmul(ev[e], E.dt);
      E.xnew[idx[e]] = xn[e];
      const double at = E.atol ? E.atol[idx[e]] : E.atol_s;
      const double rt = E.rtol ? E.rtol[idx[e]] : E.rtol_s;
      const double ax = fabs(xn[e]), ax0 = fabs(x0e);
      const double tg = dadd(at, dmul(rt, ax < ax0 ? ax0 : ax));
      const double q = __ddiv_rn(er, tg);
      const double sq = dmul(q, q);
      if (E.exact) {
        E.sq[idx[e]] = sq;
      } else {
        sq_acc = dadd(sq_acc, sq);
      }
    }
    if (newpos) {
      newpos[0] = xn[0];
      newpos[1] = xn[1];
      newpos[2] = xn[2];
    } else if constexpr (PREC == GB_PREC_MIXED) {
      const float w = E.masses ? (float)E.masses[i] : 1.0f;
      E.pnext[i] = pack_body(xn[0], xn[1], xn[2], E.cref[0], E.cref[1], E.cref[2], w);
    }
  }
}

// The same work for rows [b_lo, b_hi) of an i-tile, one state element per
// thread instead of one body per thread: the rows' 3*cnt position elements
// and 3*cnt velocity elements are contiguous in the state, so a 16-row
// cluster slice runs its FP64 stage sums on three full warps with coalesced
// loads, where the body form keeps one half-warp busy for six elements
// (FP64 issues at 1/64 of the FP32 rate on this part, and the epilogue runs
// after every CTA's pair loop, where nothing hides it).  Each element's
// arithmetic is body_epilogue's, term for term and in the same order; only
// the per-thread grouping of the squares in sq_acc differs.  part[b] holds
// the cluster's pair sums on entry; on return it holds the new positions.
// Every thread of the CTA must call it (it synchronises the CTA).
template <int PREC, int T>
__device__ __forceinline__ void rows_epilogue(const EpiCtx& E, long long i0, int b_lo, int b_hi,
                                              double (*part)[3], double& sq_acc, double& amax) {
  const DevTableau& tab = *E.tab;
  const int s = E.s, S = E.S;
  const long long n = E.n;
  const int cnt = b_hi > b_lo ? b_hi - b_lo : 0;
  const int h3 = 3 * cnt, ne = 6 * cnt;
  const long long base = 3 * (i0 + b_lo);  // first position element of the rows
  double* ks_s = E.ks + (long long)kslot(s, S, E.k0slot) * E.kstride;
  if (!E.skip_force) {
    // k_s = (v, a): velocities of the stage state, scaled pair sums
#pragma unroll 1
    for (int v = threadIdx.x; v < ne; v += T) {
      double k;
      long long idx;
      if (v < h3) {
        idx = base + v;
        k = E.ysrc[3 * n + idx];
      } else {
        const int w = v - h3;
        idx = 3 * n + base + w;
        const double a = part[b_lo + w / 3][w % 3];
        k = E.masses ? a : dmul(a, E.mass);
      }
      ks_s[idx] = k;
    }
    if (E.last) {
#pragma unroll 1
      for (int r = threadIdx.x; r < cnt; r += T) {
        const double* a = part[b_lo + r];
        double k[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) k[c] = E.masses ? a[c] : dmul(a[c], E.mass);
        amax = fmax(amax, sqrt(k[0] * k[0] + k[1] * k[1] + k[2] * k[2]));
      }
    }
  }
  __syncthreads();  // part is read; the k_s writes are visible to the CTA
#pragma unroll 1
  for (int v = threadIdx.x; v < ne; v += T) {
    const bool pos = v < h3;
    const int w = pos ? v : v - h3;
    const long long idx = (pos ? 0 : 3 * n) + base + w;
    const double x0e = E.x0[idx];
    double out;
    if (!E.last) {
      // terms in groups of four: a group's loads are in flight together,
      // the sum still runs in stage order
      const unsigned m = tab.anz[s];
      double acc = 0.0;
#pragma unroll 1
      for (int l0 = 0; l0 <= s; l0 += 4) {
        double kl[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int l = l0 + u;
          if (l <= s && ((m >> l) & 1u)) kl[u] = E.ks[(long long)kslot(l, S, E.k0slot) * E.kstride + idx];
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int l = l0 + u;
          if (l <= s && ((m >> l) & 1u)) acc = dadd(acc, dmul(tab.a[s][l], kl[u]));
        }
      }
      out = dadd(x0e, dmul(acc, E.dt));
      E.ynext[idx] = out;
    } else {
      const unsigned m = tab.bnz | tab.dbnz;
      double xv = 0.0, ev = 0.0;
#pragma unroll 1
      for (int l0 = 0; l0 < S; l0 += 4) {
        double kl[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int l = l0 + u;
          if (l < S && ((m >> l) & 1u)) kl[u] = E.ks[(long long)kslot(l, S, E.k0slot) * E.kstride + idx];
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int l = l0 + u;
          if (l >= S) break;
          if ((tab.bnz >> l) & 1u) xv = dadd(xv, dmul(tab.b[l], kl[u]));
          if ((tab.dbnz >> l) & 1u) ev = dadd(ev, dmul(tab.db[l], kl[u]));
        }
      }
      out = dadd(x0e, dmul(xv, E.dt));
      const double er = dmul(ev, E.dt);
      E.xnew[idx] = out;
      const double at = E.atol ? E.atol[idx] : E.atol_s;
      const double rt = E.rtol ? E.rtol[idx] : E.rtol_s;
      const double ax = fabs(out), ax0 = fabs(x0e);
      const double tg = dadd(at, dmul(rt, ax < ax0 ? ax0 : ax));
      const double q = __ddiv_rn(er, tg);
      const double sq = dmul(q, q);
      if (E.exact) {
        E.sq[idx] = sq;
      } else {
        sq_acc = dadd(sq_acc, sq);
      }
    }
    if (pos) part[b_lo + w / 3][w % 3] = out;
  }
  if constexpr (PREC == GB_PREC_MIXED) {
    __syncthreads();
    PackedBody* dst = E.pnext;
#pragma unroll 1
    for (int r = threadIdx.x; r < cnt; r += T) {
      const double* p = part[b_lo + r];
      const long long i = i0 + b_lo + r;
      const float w = E.masses ? (float)E.masses[i] : 1.0f;
      dst[i] = pack_body(p[0], p[1], p[2], E.cref[0], E.cref[1], E.cref[2], w);
    }
  }
}

// Packs one sorted tile whose bodies' new positions are held one per thread
// (threadIdx.x < cnt): FP64 centroid and radius by block reductions, then the
// near record (hi/lo of x - c), the far record (FP32 x - c_J, weight) and the
// tile metadata.  All threads of the CTA must call it.
__device__ __forceinline__ void pack_sorted_tile(const double* p, bool valid, int cnt, float w,
                                                 const double* cref, PackedBody* near_out,
                                                 float4* far_out, TileMeta* meta_out,
                                                 double* red) {
  double c[3];
  for (int d = 0; d < 3; ++d) c[d] = block_sum(valid ? p[d] : 0.0, red) / (double)cnt;
  double r2 = 0.0;
  if (valid) {
    const double dx = p[0] - c[0], dy = p[1] - c[1], dz = p[2] - c[2];
    r2 = dx * dx + dy * dy + dz * dz;
  }
  const double rad = sqrt(block_max(r2, red));
  if (valid) {
    *near_out = pack_body(p[0], p[1], p[2], cref[0], cref[1], cref[2], w);
    *far_out = make_float4(__double2float_rn(p[0] - c[0]), __double2float_rn(p[1] - c[1]),
                           __double2float_rn(p[2] - c[2]), w);
  }
  if (threadIdx.x == 0) {
    TileMeta m;
    float h, l;
    split_hilo(c[0] - cref[0], h, l);
    m.chi.x = h;
    m.clo.x = l;
    split_hilo(c[1] - cref[1], h, l);
    m.chi.y = h;
    m.clo.y = l;
    split_hilo(c[2] - cref[2], h, l);
    m.chi.z = h;
    m.clo.z = l;
    m.chi.w = __double2float_ru(rad * (1.0 + 1e-6));
    m.clo.w = 0.f;
    *meta_out = m;
  }
}

}  // namespace gb
