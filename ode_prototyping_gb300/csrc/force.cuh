// force.cuh -- all-pairs softened gravity, the O(N^2) part of the right-hand
// side of NBodyODE (src/ode/NBodyODE.hpp:68-133), owner-computes form.
//
// Work decomposition (one launch covers every body of one system):
//   * a CTA owns an i-tile of BI = T / L bodies; L adjacent lanes share a body
//     and take interleaved partners (j = j0 + l, j0 + l + L, ...);
//   * the P CTAs of a thread-block cluster share the i-tile and split the
//     partner range into P contiguous chunks;
//   * partial sums are combined in a fixed order: warp shuffles over the L
//     lanes, then cluster rank 0 adds ranks 1..P-1 read through distributed
//     shared memory.  No atomics, bitwise reproducible run to run; with
//     L = P = 1 each body's terms are added in ascending partner order, which
//     is the order in which the reference's serial executor adds them (body k
//     receives pair (m, k) for m < k, then (k, m) for m > k, and
//     -(d/den) == (-d)/den), so the FP64 sums match it bit for bit.
#pragma once

#include <type_traits>

#include "gb_internal.cuh"

namespace gb {

// Per-body packed j-record of the mixed-precision path: hi parts + weight,
// then lo parts.  32 bytes, so a tile of JT bodies is one contiguous
// 32*JT-byte block (one bulk copy).
struct __align__(16) PackedBody {
  float4 hw;  // hx, hy, hz, w (w = m_j, or 1 when the mass is uniform)
  float4 lo;  // lx, ly, lz, 0
};

struct ClusterInfo {
  int rank;
  int size;
  long long itile;
};

__device__ __forceinline__ ClusterInfo cluster_info() {
  cg::cluster_group cl = cg::this_cluster();
  ClusterInfo ci;
  ci.rank = (int)cl.block_rank();
  ci.size = (int)cl.num_blocks();
  ci.itile = blockIdx.x / ci.size;
  return ci;
}

// Partner chunk of cluster rank r: [jb, je), multiples of the tile size.
__device__ __forceinline__ void j_chunk(long long n, int rank, int size, int jt, long long& jb,
                                        long long& je) {
  long long ntiles = (n + jt - 1) / jt;
  long long per = (ntiles + size - 1) / size;
  jb = (long long)rank * per * jt;
  je = jb + per * jt;
  if (jb > n) jb = n;
  if (je > n) je = n;
}

// Reduces v over the L lanes of a body group (tree over xor offsets).
template <int L>
__device__ __forceinline__ double lane_reduce(double v) {
#pragma unroll
  for (int off = L / 2; off >= 1; off /= 2) v = dadd(v, __shfl_down_sync(0xffffffffu, v, off, L));
  return v;
}

// Cluster-wide combine of per-body partials part[BI][3] held in each CTA's
// shared memory; on return rank 0's part holds the totals (ranks added in
// order 0, 1, ..., P-1).  All threads of all CTAs of the cluster must call it.
template <int BI>
__device__ __forceinline__ void cluster_combine(double (*part)[3], int rank, int size) {
  cg::cluster_group cl = cg::this_cluster();
  cl.sync();
  if (rank == 0 && size > 1) {
    for (int b = threadIdx.x; b < BI; b += blockDim.x) {
      double s0 = part[b][0], s1 = part[b][1], s2 = part[b][2];
      for (int r = 1; r < size; ++r) {
        double(*rp)[3] = cl.map_shared_rank(part, r);
        s0 = dadd(s0, rp[b][0]);
        s1 = dadd(s1, rp[b][1]);
        s2 = dadd(s2, rp[b][2]);
      }
      part[b][0] = s0;
      part[b][1] = s1;
      part[b][2] = s2;
    }
  }
  cl.sync();
}

// Cluster-wide combine that leaves every rank the totals of its own rows:
// rank r owns rows [r R, (r + 1) R), R = ceil(BI / size), and adds the ranks'
// partial sums in the order of cluster_combine (rank 0's value, then ranks
// 1, ..., size - 1), so the totals are bit-identical to it.  No rank reads
// another's rows inside that rank's own range, so each rank overwrites its
// rows in place.  All threads of all CTAs of the cluster must call it.
template <int BI>
__device__ __forceinline__ void cluster_combine_rows(double (*part)[3], int rank, int size) {
  cg::cluster_group cl = cg::this_cluster();
  cl.sync();
  if (size > 1) {
    const int R = (BI + size - 1) / size;
    const int lo = rank * R, hi = min(BI, lo + R);
    double(*p0)[3] = cl.map_shared_rank(part, 0);
    for (int b = lo + (int)threadIdx.x; b < hi; b += blockDim.x) {
      double s0 = p0[b][0], s1 = p0[b][1], s2 = p0[b][2];
      for (int r = 1; r < size; ++r) {
        double(*rp)[3] = cl.map_shared_rank(part, r);
        s0 = dadd(s0, rp[b][0]);
        s1 = dadd(s1, rp[b][1]);
        s2 = dadd(s2, rp[b][2]);
      }
      part[b][0] = s0;
      part[b][1] = s1;
      part[b][2] = s2;
    }
  }
  cl.sync();
}

// ---------------------------------------------------------------------------
// The threads that run one force tile together: the whole CTA (barrier 0,
// __syncthreads), or one of several groups of T consecutive threads (whole
// warps) that share a CTA, each synchronised by its own named barrier -- the
// batched integrator runs one small system per group.
// ---------------------------------------------------------------------------
struct WholeCta {
  __device__ __forceinline__ unsigned tid() const { return threadIdx.x; }
  __device__ __forceinline__ void sync() const { __syncthreads(); }
};

template <int T>
struct WarpGroup {
  static_assert(T % 32 == 0, "a named barrier counts whole warps");
  unsigned t;  // thread index within the group
  int bar;     // named barrier id, 1..4 (0 is __syncthreads)
  __device__ __forceinline__ unsigned tid() const { return t; }
  __device__ __forceinline__ void sync() const {
    // immediate ids, so the kernel reserves barriers 0..4 only
    switch (bar) {
      case 1: asm volatile("bar.sync 1, %0;" ::"n"(T) : "memory"); break;
      case 2: asm volatile("bar.sync 2, %0;" ::"n"(T) : "memory"); break;
      case 3: asm volatile("bar.sync 3, %0;" ::"n"(T) : "memory"); break;
      default: asm volatile("bar.sync 4, %0;" ::"n"(T) : "memory"); break;
    }
  }
};

// ---------------------------------------------------------------------------
// FP64: partial sums of one CTA (or thread group) over its partner chunk.
// sh_pos holds 3*T doubles, sh_m T doubles (per-body masses only).  Results
// land in part[b].  fast = false: every pair term in the reference's
// operation order (IEEE sqrt and divisions, NBodyODE.hpp:89-98), summed with
// IEEE adds; fast = true: r^-3 from the refined reciprocal square root
// (rinv3_f64) and fused multiply-add accumulation, a few ulp per term from
// the reference's.  With L lanes, lane l takes the partners j = l (mod L) in
// ascending order whatever T is, so the sums do not depend on the group size.
// ---------------------------------------------------------------------------
template <int T, int L, class G = WholeCta>
__device__ __forceinline__ void force_f64_cta(const double* __restrict__ pos, long long n,
                                              long long i0, long long jb, long long je,
                                              double eps2, const double* __restrict__ masses,
                                              double* sh_pos, double* sh_m, double (*part)[3],
                                              bool fast = false, const G& grp = G{}) {
  constexpr int BI = T / L;
  const unsigned tid = grp.tid();
  const int b = tid / L;
  const int l = tid % L;
  const long long i = i0 + b;
  double xi = 0.0, yi = 0.0, zi = 0.0;
  if (i < n) {
    xi = pos[3 * i];
    yi = pos[3 * i + 1];
    zi = pos[3 * i + 2];
  }
  double sx = 0.0, sy = 0.0, sz = 0.0;
  for (long long j0 = jb; j0 < je; j0 += T) {
    const int cnt = (int)min((long long)T, je - j0);
    grp.sync();
    for (int k = tid; k < 3 * cnt; k += T) sh_pos[k] = pos[3 * j0 + k];
    if (masses)
      for (int k = tid; k < cnt; k += T) sh_m[k] = masses[j0 + k];
    grp.sync();
    if (i >= n) continue;
    if (fast) {
      for (int jj = l; jj < cnt; jj += L) {
        if (j0 + jj == i) continue;
        const double dx = sh_pos[3 * jj] - xi;
        const double dy = sh_pos[3 * jj + 1] - yi;
        const double dz = sh_pos[3 * jj + 2] - zi;
        double r3 = rinv3_f64(fma(dz, dz, fma(dy, dy, fma(dx, dx, eps2))));
        if (masses) r3 *= sh_m[jj];
        sx = fma(dx, r3, sx);
        sy = fma(dy, r3, sy);
        sz = fma(dz, r3, sz);
      }
    } else {
      for (int jj = l; jj < cnt; jj += L) {
        const long long j = j0 + jj;
        if (j == i) continue;
        double ax, ay, az;
        pair_term_f64(xi, yi, zi, sh_pos[3 * jj], sh_pos[3 * jj + 1], sh_pos[3 * jj + 2], eps2,
                      ax, ay, az);
        if (masses) {
          const double mj = sh_m[jj];
          ax = dmul(ax, mj);
          ay = dmul(ay, mj);
          az = dmul(az, mj);
        }
        sx = dadd(sx, ax);
        sy = dadd(sy, ay);
        sz = dadd(sz, az);
      }
    }
  }
  sx = lane_reduce<L>(sx);
  sy = lane_reduce<L>(sy);
  sz = lane_reduce<L>(sz);
  if (l == 0) {
    part[b][0] = sx;
    part[b][1] = sy;
    part[b][2] = sz;
  }
  (void)BI;
}

// ---------------------------------------------------------------------------
// Mixed precision.  Positions are stored as hi + lo FP32 parts of (x - c),
// c a fixed reference point of the system; dx = (hj - hi) + (lj - li) keeps
// ~2^-23 relative accuracy even for close pairs (hj - hi is exact by
// Sterbenz's lemma when the bodies are close).  r^-3 from the SFU rsqrt.
// Each lane sums a j-tile's terms in FP32 and Kahan-adds the tile sum into
// its running (sum, compensation) pair; the pair is widened to FP64 for the
// lane and cluster combine.
// ---------------------------------------------------------------------------
// SFU reciprocal square root without the subnormal fix-up sequence: the
// argument is r^2 + eps^2 >= eps^2 > 0, far from the subnormal range.
__device__ __forceinline__ float rsqrt_sfu(float x) {
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__device__ __forceinline__ void kahan_add(float& s, float& c, float v) {
  const float y = __fsub_rn(v, c);
  const float t = __fadd_rn(s, y);
  c = __fsub_rn(__fsub_rn(t, s), y);
  s = t;
}

// Knuth's error-free sum: s + e == a + b exactly (explicit IEEE adds, so
// nothing is contracted or reassociated).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// (S, E) += (hi, lo) in double-single arithmetic (an unevaluated sum of two
// floats, about 48 significant bits), renormalised after each addition.
__device__ __forceinline__ void ds_add(float& S, float& E, float hi, float lo) {
  float s, e;
  two_sum(S, hi, s, e);
  e = __fadd_rn(e, __fadd_rn(E, lo));
  two_sum(s, e, S, E);
}

// Pair differences.  With hi = fl32(x - c) and lo = fl32(x - c - hi) (c the
// reference point), the hi-only difference hj - hi is off by at most
// 2^-24 (|x_i - c| + |x_j - c|) + 2^-24 |dx|, i.e. relatively by
// 2^-24 (1 + 2 |x_i - c| / r) for softened distance r; the pair force's
// relative error is about three times that.  Pairs with r >= |x_i - c| / 8
// therefore use hj - hi alone (relative force error <= 3 * 17 * 2^-24 =
// 3.0e-6, and such pairs carry little of a body's acceleration), and closer
// pairs add the lo parts, (hj - hi) + (lj - li), relative error ~2^-23.  The
// test compares the bit patterns of the two positive floats r^2 and
// (|h_i| / 8)^2, an integer comparison.  Measured on Plummer, binary-rich,
// uniform-ball and cold-collapse states: accelerations within 1.1e-7 of FP64
// normwise, the same as hi/lo on every pair, with 2-4 % of warp iterations
// taking the close-pair branch.
__device__ __forceinline__ int near_threshold_bits(float hx, float hy, float hz) {
  const float h2 = fmaf(hz, hz, fmaf(hy, hy, hx * hx));
  return __float_as_int(h2 * (1.0f / 64.0f));
}

template <int T, int L, int BPT, bool UNIFORM = false>
__device__ __forceinline__ void force_mixed_cta(const PackedBody* __restrict__ packed, long long n,
                                                long long i0, long long jb, long long je,
                                                float eps2, PackedBody* sh, double (*part)[3]) {
  constexpr int BG = T / L;        // body groups per CTA
  const int g = threadIdx.x / L;   // body group
  const int l = threadIdx.x % L;
  float hx[BPT], hy[BPT], hz[BPT], lx[BPT], ly[BPT], lz[BPT];
  float sx[BPT], sy[BPT], sz[BPT], cx[BPT], cy[BPT], cz[BPT];
  int near2[BPT];  // bit pattern of (|h_i| / 8)^2: below it a pair takes the hi/lo difference
#pragma unroll
  for (int q = 0; q < BPT; ++q) {
    const long long i = i0 + (long long)q * BG + g;
    PackedBody pb;
    if (i < n) {
      pb = packed[i];
    } else {
      pb.hw = make_float4(0.f, 0.f, 0.f, 0.f);
      pb.lo = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    hx[q] = pb.hw.x; hy[q] = pb.hw.y; hz[q] = pb.hw.z;
    lx[q] = pb.lo.x; ly[q] = pb.lo.y; lz[q] = pb.lo.z;
    sx[q] = sy[q] = sz[q] = 0.f;
    cx[q] = cy[q] = cz[q] = 0.f;
    near2[q] = near_threshold_bits(hx[q], hy[q], hz[q]);
  }
  constexpr int JT = T;  // bodies per j-tile: one record per thread
  // the next tile's record is loaded into registers while this tile computes
  PackedBody nxt;
  if (jb + threadIdx.x < je) nxt = packed[jb + threadIdx.x];
  for (long long j0 = jb; j0 < je; j0 += JT) {
    const int cnt = (int)min((long long)JT, je - j0);
    __syncthreads();
    if (threadIdx.x < cnt) sh[threadIdx.x] = nxt;
    __syncthreads();
    if (j0 + JT + threadIdx.x < je) nxt = packed[j0 + JT + threadIdx.x];
    float tx[BPT], ty[BPT], tz[BPT];
#pragma unroll
    for (int q = 0; q < BPT; ++q) tx[q] = ty[q] = tz[q] = 0.f;
    // Same scheme as the packed path: hi-only terms without branching, close
    // pairs marked per chunk of 32 partners and replaced afterwards.
    const int kn = (cnt - l + L - 1) / L;
    for (int k0 = 0; k0 < kn; k0 += 32) {
      const int kc = min(32, kn - k0);
      unsigned mask = 0;
#pragma unroll 4
      for (int u = 0; u < kc; ++u) {
        const int jj = l + (k0 + u) * L;
        const float4 hw = sh[jj].hw;
        bool close = false;
#pragma unroll
        for (int q = 0; q < BPT; ++q) {
          const float dx = hw.x - hx[q];
          const float dy = hw.y - hy[q];
          const float dz = hw.z - hz[q];
          const float r2 = fmaf(dz, dz, fmaf(dy, dy, fmaf(dx, dx, eps2)));
          close |= __float_as_int(r2) < near2[q];
          const float rinv = rsqrt_sfu(r2);
          const float sc = UNIFORM ? rinv * (rinv * rinv) : (hw.w * rinv) * (rinv * rinv);
          tx[q] = fmaf(sc, dx, tx[q]);
          ty[q] = fmaf(sc, dy, ty[q]);
          tz[q] = fmaf(sc, dz, tz[q]);
        }
        mask |= (unsigned)close << u;
      }
      while (mask) {
        const int u = __ffs(mask) - 1;
        mask &= mask - 1;
        const int jj = l + (k0 + u) * L;
        const float4 hw = sh[jj].hw;
        const float4 lo = sh[jj].lo;
#pragma unroll
        for (int q = 0; q < BPT; ++q) {
          float dx = hw.x - hx[q];
          float dy = hw.y - hy[q];
          float dz = hw.z - hz[q];
          float r2 = fmaf(dz, dz, fmaf(dy, dy, fmaf(dx, dx, eps2)));
          float rinv = rsqrt_sfu(r2);
          float sc = UNIFORM ? rinv * (rinv * rinv) : (hw.w * rinv) * (rinv * rinv);
          tx[q] = fmaf(-sc, dx, tx[q]);  // take the hi-only term out again
          ty[q] = fmaf(-sc, dy, ty[q]);
          tz[q] = fmaf(-sc, dz, tz[q]);
          dx = dx + (lo.x - lx[q]);
          dy = dy + (lo.y - ly[q]);
          dz = dz + (lo.z - lz[q]);
          r2 = fmaf(dz, dz, fmaf(dy, dy, fmaf(dx, dx, eps2)));
          rinv = rsqrt_sfu(r2);
          sc = UNIFORM ? rinv * (rinv * rinv) : (hw.w * rinv) * (rinv * rinv);
          tx[q] = fmaf(sc, dx, tx[q]);
          ty[q] = fmaf(sc, dy, ty[q]);
          tz[q] = fmaf(sc, dz, tz[q]);
        }
      }
    }
#pragma unroll
    for (int q = 0; q < BPT; ++q) {
      kahan_add(sx[q], cx[q], tx[q]);
      kahan_add(sy[q], cy[q], ty[q]);
      kahan_add(sz[q], cz[q], tz[q]);
    }
  }
#pragma unroll
  for (int q = 0; q < BPT; ++q) {
    double ax = dsub((double)sx[q], (double)cx[q]);
    double ay = dsub((double)sy[q], (double)cy[q]);
    double az = dsub((double)sz[q], (double)cz[q]);
    ax = lane_reduce<L>(ax);
    ay = lane_reduce<L>(ay);
    az = lane_reduce<L>(az);
    if (l == 0) {
      part[q * BG + g][0] = ax;
      part[q * BG + g][1] = ay;
      part[q * BG + g][2] = az;
    }
  }
}

// ---------------------------------------------------------------------------
// Blackwell's packed f32x2 instructions (add/sub/mul/fma on a pair of FP32
// values held in one 64-bit register; the two lanes are independent IEEE
// operations).  ncu shows each holding the FMA pipe for two cycles, so they
// save issue slots, not pipe cycles.
// ---------------------------------------------------------------------------
typedef unsigned long long f2_t;

__device__ __forceinline__ f2_t f2_pack(float a, float b) {
  f2_t r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ void f2_unpack(f2_t r, float& a, float& b) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(r));
}
__device__ __forceinline__ f2_t f2_sub(f2_t a, f2_t b) {
  f2_t r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ f2_t f2_add(f2_t a, f2_t b) {
  f2_t r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ f2_t f2_mul(f2_t a, f2_t b) {
  f2_t r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ f2_t f2_fma(f2_t a, f2_t b, f2_t c) {
  f2_t r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
  return r;
}

// ---------------------------------------------------------------------------
// Packed loop over pairs of partners: each f32x2 instruction carries
// partners j and j + 1 of the same body, so the staged partner records need
// no duplicated coordinates.  NB bodies per thread (1 or 2): body q of thread
// group g is i0 + q * (T / L) + g; with two, every 48-byte record feeds two
// independent instruction chains (four interactions per record read).  Tiles
// of 2T partners are copied with cp.async (no registers held across the
// compute loop); each thread copies two partners and builds one record from
// them.  A missing second partner (odd tail) is placed at 1e18: its r^-3
// underflows to zero, so its term is exactly zero.  A close pair for either
// body sends both bodies' terms of that record through the hi/lo revisit.
// ---------------------------------------------------------------------------
struct __align__(16) PartnerPair {
  ulonglong2 xy;  // (hx_j, hx_j+1), (hy_j, hy_j+1)
  ulonglong2 zl;  // (hz_j, hz_j+1), (lx_j, lx_j+1)
  ulonglong2 yz;  // (ly_j, ly_j+1), (lz_j, lz_j+1)
};

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;" ::: "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_group 0;" ::: "memory");
}

// Shared memory of force_mixed_cta_jp: 2 x T records + 2T raw bodies.
template <int T>
constexpr int jp_smem_bytes() {
  return 2 * (int)sizeof(PartnerPair) * T + 2 * T * (int)sizeof(PackedBody);
}

// Bounding box of a tile of packed positions (FP32 hi parts relative to the
// reference point): centre (x, y, z) and a radius (w) that bounds every hi
// point's distance from the rounded centre.
struct TileBox {
  float4 c;
};

// Box from FP32 extents [lo, hi] per axis: centre (x, y, z) and a radius (w)
// rounded outwards (the half-diagonal rounded up, widened by 1e-5 relative
// and by the rounding of the centre) so that it bounds the distance of every
// point of the extents from the rounded centre.
__device__ __forceinline__ float4 box_from_extents(float lx, float ly, float lz, float hx,
                                                   float hy, float hz) {
  float4 b;
  b.x = 0.5f * (lx + hx);
  b.y = 0.5f * (ly + hy);
  b.z = 0.5f * (lz + hz);
  const float ex = 0.5f * (hx - lx), ey = 0.5f * (hy - ly), ez = 0.5f * (hz - lz);
  const float r = __fsqrt_ru(__fmaf_ru(ez, ez, __fmaf_ru(ey, ey, __fmul_ru(ex, ex))));
  b.w = r * 1.00001f + 3.0e-7f * (fabsf(b.x) + fabsf(b.y) + fabsf(b.z));
  return b;
}

// True when no pair of the i-side (a box I, or a single body: I.w = 0, with
// near-pair threshold |h_i| / 8 <= ti) and the j-tile (box J) can be a close
// pair of the packed loop (r^2 < (|h_i| / 8)^2): the gap exceeds ti.  The
// margins (1e-5 relative) cover the FP32 rounding of this test and of the
// loop's r^2 and thresholds, so a far tile gives exactly the terms the
// close-pair test would (none revisited).
__device__ __forceinline__ bool tiles_far(float4 I, float ti, float4 J) {
  const float dx = I.x - J.x, dy = I.y - J.y, dz = I.z - J.z;
  const float d = __fsqrt_rn(__fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx))));
  return __fmul_rn(d, 1.0f - 1e-5f) - I.w - J.w > __fmul_rn(ti, 1.0f + 1e-5f);
}

// PAIRS (one lane per body): part is read as float2[BI][3] and receives each
// sum as its FP32 Kahan pair (s, -c), value s - c, with no FP64 arithmetic.
// CULL (one lane and one body per thread, 128 threads, partner ranges that
// start at multiples of 64): boxes[t] bounds the packed positions of bodies
// [64 t, 64 t + 64).  Every lane tests its own body against the box of each
// 64-partner quarter of a tile (tiles_far with the body's own threshold), and
// a quarter that is far for all 32 bodies of the warp (cull != 0) runs the
// pair loop without the close-pair test.  Its terms are the ones the test
// would have kept, so the sums are bit for bit those of the loop with the
// test.  (Measured at N = 16384: 0.1254 ms per RKF78 stage against 0.1276 ms
// for one box per warp of 32 bodies.)
template <int T, int L, int NB = 1, bool PAIRS = false, bool CULL = false, class G = WholeCta>
__device__ __forceinline__ void force_mixed_cta_jp(const PackedBody* __restrict__ packed,
                                                   long long n, long long i0, long long jb,
                                                   long long je, float eps2, unsigned char* smem,
                                                   double (*part)[3],
                                                   const float4* __restrict__ boxes = nullptr,
                                                   int cull = 0, const G& grp = G{}) {
  static_assert(!CULL || (L == 1 && NB == 1 && T == 128), "culling: 128 one-body threads");
  static_assert(!CULL || std::is_same_v<G, WholeCta>, "culling: the whole CTA");
  const unsigned tid = grp.tid();
  constexpr int BG = T / L;  // body groups per CTA (NB bodies each)
  constexpr int JT = 2 * T;  // partners per tile
  PartnerPair* recs = reinterpret_cast<PartnerPair*>(smem);  // two buffers of T records
  PackedBody* raw = reinterpret_cast<PackedBody*>(smem + 2 * sizeof(PartnerPair) * T);
  const int g = tid / L;
  const int l = tid % L;
  f2_t HX[NB], HY[NB], HZ[NB], LX[NB], LY[NB], LZ[NB];
  int near2[NB];
  // CULL: the body's point and its near-pair bound |h_i| / 8, rounded up
  float4 self = make_float4(0.f, 0.f, 0.f, 0.f);
  float self_ti = 0.f;
#pragma unroll
  for (int q = 0; q < NB; ++q) {
    const long long i = i0 + (long long)q * BG + g;
    PackedBody pb;
    if (i < n) {
      pb = packed[i];
    } else {
      pb.hw = make_float4(0.f, 0.f, 0.f, 0.f);
      pb.lo = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    HX[q] = f2_pack(pb.hw.x, pb.hw.x);
    HY[q] = f2_pack(pb.hw.y, pb.hw.y);
    HZ[q] = f2_pack(pb.hw.z, pb.hw.z);
    LX[q] = f2_pack(pb.lo.x, pb.lo.x);
    LY[q] = f2_pack(pb.lo.y, pb.lo.y);
    LZ[q] = f2_pack(pb.lo.z, pb.lo.z);
    near2[q] = near_threshold_bits(pb.hw.x, pb.hw.y, pb.hw.z);
    if constexpr (CULL) {
      self = make_float4(pb.hw.x, pb.hw.y, pb.hw.z, 0.f);
      self_ti = __fmul_ru(__fsqrt_ru(__fmaf_ru(pb.hw.z, pb.hw.z,
                                               __fmaf_ru(pb.hw.y, pb.hw.y,
                                                         __fmul_ru(pb.hw.x, pb.hw.x)))),
                          0.125f);
    }
  }
  const f2_t E2 = f2_pack(eps2, eps2);
  float sx[NB], sy[NB], sz[NB], cx[NB], cy[NB], cz[NB];
#pragma unroll
  for (int q = 0; q < NB; ++q) sx[q] = sy[q] = sz[q] = cx[q] = cy[q] = cz[q] = 0.f;
  // Thread t copies partners j0 + 2t and j0 + 2t + 1 of every tile into its
  // own two raw slots and later builds record t from them, so the single raw
  // area needs no barrier: a thread re-issues its slots only after reading
  // them (in issue order).  Records are double-buffered: tile k + 1's are
  // built at the end of tile k into the buffer tile k - 1 used, and one
  // barrier per tile both publishes them and retires tile k's.
  auto issue = [&](long long j0) {
    PackedBody* dst = raw + 2 * tid;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const long long j = j0 + 2 * tid + h;
      if (j < je) {
        cp_async16(&dst[h].hw, &packed[j].hw);
        cp_async16(&dst[h].lo, &packed[j].lo);
      }
    }
    cp_async_commit();
  };
  // Builds the records of the tile at j0 and returns (in every lane) the
  // warp's far mask of the tile's four 64-partner quarters.
  auto build = [&](long long j0, PartnerPair* out) -> unsigned {
    const int cnt = (int)min((long long)JT, je - j0);
    unsigned fm = 0;
    if constexpr (CULL) {
      if (cull) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const long long h0 = j0 + 64 * (long long)q;
          const bool far = h0 < je && tiles_far(self, self_ti, __ldg(boxes + h0 / 64));
          fm |= (unsigned)__all_sync(0xffffffffu, far) << q;
        }
      }
    }
    if ((int)tid < (cnt + 1) / 2) {
      const PackedBody a = raw[2 * tid];
      PackedBody b;
      if (2 * (int)tid + 1 < cnt) {
        b = raw[2 * tid + 1];
      } else {
        b.hw = make_float4(1e18f, 1e18f, 1e18f, 0.f);
        b.lo = make_float4(0.f, 0.f, 0.f, 0.f);
      }
      PartnerPair r;
      r.xy = make_ulonglong2(f2_pack(a.hw.x, b.hw.x), f2_pack(a.hw.y, b.hw.y));
      r.zl = make_ulonglong2(f2_pack(a.hw.z, b.hw.z), f2_pack(a.lo.x, b.lo.x));
      r.yz = make_ulonglong2(f2_pack(a.lo.y, b.lo.y), f2_pack(a.lo.z, b.lo.z));
      out[tid] = r;
    }
    return fm;
  };
  unsigned fm = 0, fm_next = 0;  // far quarters of the current / next tile
  if (jb < je) {
    issue(jb);
    cp_async_wait_all();
    fm = build(jb, recs);
    if (jb + JT < je) issue(jb + JT);
  }
  grp.sync();
  int buf = 0;
  for (long long j0 = jb; j0 < je; j0 += JT, buf ^= 1) {
    const int cnt = (int)min((long long)JT, je - j0);
    const int npair = (cnt + 1) / 2;
    const PartnerPair* rec = recs + buf * T;
    f2_t TX[NB], TY[NB], TZ[NB];
#pragma unroll
    for (int q = 0; q < NB; ++q) TX[q] = TY[q] = TZ[q] = 0ULL;
    // This lane's records are jj = l + L k, k < kn.  Every pair's hi-only term
    // is added without branching; a record with a close pair (the smaller r^2
    // bit pattern below the body's threshold) is marked by shifting a bit into
    // a 32-bit mask per chunk of 32 k (bit b is iteration kc - 1 - b), and the
    // marked records are revisited: hi-only terms out, hi/lo terms in.
    const int kn = (npair - l + L - 1) / L;
    for (int k0 = 0; k0 < kn; k0 += 32) {
      const int kc = min(32, kn - k0);
      if constexpr (CULL) {
        // records [32 q, 32 q + 32) hold the partners of quarter q
        if ((fm >> (k0 >> 5)) & 1u) {
#pragma unroll 4
          for (int u = 0; u < kc; ++u) {
            const int jj = k0 + u;
            const ulonglong2 xy = rec[jj].xy;
            const f2_t hz = rec[jj].zl.x;
            const f2_t dx = f2_sub(xy.x, HX[0]);
            const f2_t dy = f2_sub(xy.y, HY[0]);
            const f2_t dz = f2_sub(hz, HZ[0]);
            const f2_t r2 = f2_fma(dz, dz, f2_fma(dy, dy, f2_fma(dx, dx, E2)));
            float ra, rb;
            f2_unpack(r2, ra, rb);
            const f2_t ri = f2_pack(rsqrt_sfu(ra), rsqrt_sfu(rb));
            const f2_t sc = f2_mul(ri, f2_mul(ri, ri));
            TX[0] = f2_fma(sc, dx, TX[0]);
            TY[0] = f2_fma(sc, dy, TY[0]);
            TZ[0] = f2_fma(sc, dz, TZ[0]);
          }
          continue;
        }
      }
      unsigned mask = 0;
#pragma unroll(4 / NB)
      for (int u = 0; u < kc; ++u) {
        const int jj = l + (k0 + u) * L;
        const ulonglong2 xy = rec[jj].xy;
        const f2_t hz = rec[jj].zl.x;
        bool close = false;
#pragma unroll
        for (int q = 0; q < NB; ++q) {
          const f2_t dx = f2_sub(xy.x, HX[q]);
          const f2_t dy = f2_sub(xy.y, HY[q]);
          const f2_t dz = f2_sub(hz, HZ[q]);
          const f2_t r2 = f2_fma(dz, dz, f2_fma(dy, dy, f2_fma(dx, dx, E2)));
          float ra, rb;
          f2_unpack(r2, ra, rb);
          close |= min(__float_as_int(ra), __float_as_int(rb)) < near2[q];
          const f2_t ri = f2_pack(rsqrt_sfu(ra), rsqrt_sfu(rb));
          const f2_t sc = f2_mul(ri, f2_mul(ri, ri));
          TX[q] = f2_fma(sc, dx, TX[q]);
          TY[q] = f2_fma(sc, dy, TY[q]);
          TZ[q] = f2_fma(sc, dz, TZ[q]);
        }
        mask = (mask << 1) | (unsigned)close;
      }
      while (mask) {
        const int u = kc - __ffs(mask);
        mask &= mask - 1;
        const int jj = l + (k0 + u) * L;
        const ulonglong2 xy = rec[jj].xy;
        const ulonglong2 zl = rec[jj].zl;
        const ulonglong2 yz = rec[jj].yz;
#pragma unroll
        for (int q = 0; q < NB; ++q) {
          f2_t dx = f2_sub(xy.x, HX[q]);
          f2_t dy = f2_sub(xy.y, HY[q]);
          f2_t dz = f2_sub(zl.x, HZ[q]);
          f2_t r2 = f2_fma(dz, dz, f2_fma(dy, dy, f2_fma(dx, dx, E2)));
          float ra, rb;
          f2_unpack(r2, ra, rb);
          f2_t ri = f2_pack(rsqrt_sfu(ra), rsqrt_sfu(rb));
          const f2_t nsc = f2_mul(f2_mul(ri, f2_mul(ri, ri)), f2_pack(-1.f, -1.f));
          TX[q] = f2_fma(nsc, dx, TX[q]);
          TY[q] = f2_fma(nsc, dy, TY[q]);
          TZ[q] = f2_fma(nsc, dz, TZ[q]);
          dx = f2_add(dx, f2_sub(zl.y, LX[q]));
          dy = f2_add(dy, f2_sub(yz.x, LY[q]));
          dz = f2_add(dz, f2_sub(yz.y, LZ[q]));
          r2 = f2_fma(dz, dz, f2_fma(dy, dy, f2_fma(dx, dx, E2)));
          f2_unpack(r2, ra, rb);
          ri = f2_pack(rsqrt_sfu(ra), rsqrt_sfu(rb));
          const f2_t sc = f2_mul(ri, f2_mul(ri, ri));
          TX[q] = f2_fma(sc, dx, TX[q]);
          TY[q] = f2_fma(sc, dy, TY[q]);
          TZ[q] = f2_fma(sc, dz, TZ[q]);
        }
      }
    }
#pragma unroll
    for (int q = 0; q < NB; ++q) {
      float t0, t1;
      f2_unpack(TX[q], t0, t1);
      kahan_add(sx[q], cx[q], t0);
      kahan_add(sx[q], cx[q], t1);
      f2_unpack(TY[q], t0, t1);
      kahan_add(sy[q], cy[q], t0);
      kahan_add(sy[q], cy[q], t1);
      f2_unpack(TZ[q], t0, t1);
      kahan_add(sz[q], cz[q], t0);
      kahan_add(sz[q], cz[q], t1);
    }
    if (j0 + JT < je) {
      cp_async_wait_all();                 // this thread's copies of tile k + 1
      fm_next = build(j0 + JT, recs + (buf ^ 1) * T);
      if (j0 + 2 * JT < je) issue(j0 + 2 * JT);
    }
    grp.sync();
    fm = fm_next;
  }
  if constexpr (PAIRS) {
    static_assert(L == 1, "Kahan pairs out: one lane per body");
    float2(*pf)[3] = reinterpret_cast<float2(*)[3]>(part);
#pragma unroll
    for (int q = 0; q < NB; ++q) {
      pf[q * BG + g][0] = make_float2(sx[q], -cx[q]);
      pf[q * BG + g][1] = make_float2(sy[q], -cy[q]);
      pf[q * BG + g][2] = make_float2(sz[q], -cz[q]);
    }
  } else {
#pragma unroll
    for (int q = 0; q < NB; ++q) {
      double ax = dsub((double)sx[q], (double)cx[q]);
      double ay = dsub((double)sy[q], (double)cy[q]);
      double az = dsub((double)sz[q], (double)cz[q]);
      ax = lane_reduce<L>(ax);
      ay = lane_reduce<L>(ay);
      az = lane_reduce<L>(az);
      if (l == 0) {
        part[q * BG + g][0] = ax;
        part[q * BG + g][1] = ay;
        part[q * BG + g][2] = az;
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Mixed precision on spatially sorted bodies.  Bodies are processed in a
// Morton order, so consecutive 128-body tiles are compact.  Each j-tile J
// carries its centroid c_J (hi/lo FP32 parts of c_J - c) and radius R_J, and
// each body a second record: FP32 (x_j - c_J).  For a j-tile whose gap to the
// CTA's i-tile is at least R_J, the pair difference is one subtraction per
// component, dx = (x_j - c_J) - (x_i - c_J), with x_i - c_J formed once per
// tile from the i-body's hi/lo parts; its error is at most
// 2^-24 (R_J + |x_i - c_J| + |dx|) <= 2^-24 (2 R_J + 2|dx|) <= 4 * 2^-24 |dx|.
// Tiles closer than that use the hi/lo difference of force_mixed_cta.
// ---------------------------------------------------------------------------
struct TileMeta {
  float4 chi;  // hi parts of c_J - c, radius R_J in .w
  float4 clo;  // lo parts of c_J - c
};

// far when the gap between the two tiles' bounding spheres is >= 1.1 R_J
__device__ __forceinline__ bool tile_is_far(const TileMeta& I, const TileMeta& J) {
  const float dx = (J.chi.x - I.chi.x) + (J.clo.x - I.clo.x);
  const float dy = (J.chi.y - I.chi.y) + (J.clo.y - I.clo.y);
  const float dz = (J.chi.z - I.chi.z) + (J.clo.z - I.clo.z);
  const float d = sqrtf(dx * dx + dy * dy + dz * dz);
  return d - I.chi.w - J.chi.w >= 1.1f * J.chi.w;
}

template <int T, int L, int BPT, bool UNIFORM>
__device__ __forceinline__ void force_mixed_sorted_cta(
    const PackedBody* __restrict__ near, const float4* __restrict__ far,
    const TileMeta* __restrict__ meta, long long n, long long itile, long long jb, long long je,
    float eps2, PackedBody* sh, double (*part)[3]) {
  constexpr int BG = T / L;
  constexpr int BI = BG * BPT;
  static_assert(BI == T, "sorted tiles: i-tile and j-tile sizes must match");
  const int g = threadIdx.x / L;
  const int l = threadIdx.x % L;
  const long long i0 = itile * BI;
  float hx[BPT], hy[BPT], hz[BPT], lx[BPT], ly[BPT], lz[BPT];
  float sx[BPT], sy[BPT], sz[BPT], cx[BPT], cy[BPT], cz[BPT];
#pragma unroll
  for (int q = 0; q < BPT; ++q) {
    const long long i = i0 + (long long)q * BG + g;
    PackedBody pb;
    if (i < n) {
      pb = near[i];
    } else {
      pb.hw = make_float4(1e30f, 1e30f, 1e30f, 0.f);  // far from everything, weight 0
      pb.lo = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    hx[q] = pb.hw.x; hy[q] = pb.hw.y; hz[q] = pb.hw.z;
    lx[q] = pb.lo.x; ly[q] = pb.lo.y; lz[q] = pb.lo.z;
    sx[q] = sy[q] = sz[q] = 0.f;
    cx[q] = cy[q] = cz[q] = 0.f;
  }
  const TileMeta mi = meta[itile];
  constexpr int JT = T;
  for (long long j0 = jb; j0 < je; j0 += JT) {
    const int cnt = (int)min((long long)JT, je - j0);
    const TileMeta mj = meta[j0 / JT];
    const bool is_far = tile_is_far(mi, mj);
    __syncthreads();
    if (is_far) {
      float4* dst = reinterpret_cast<float4*>(sh);
      for (int k = threadIdx.x; k < cnt; k += T) dst[k] = far[j0 + k];
    } else {
      const float4* src = reinterpret_cast<const float4*>(near + j0);
      float4* dst = reinterpret_cast<float4*>(sh);
      for (int k = threadIdx.x; k < 2 * cnt; k += T) dst[k] = src[k];
    }
    __syncthreads();
    float tx[BPT], ty[BPT], tz[BPT];
#pragma unroll
    for (int q = 0; q < BPT; ++q) tx[q] = ty[q] = tz[q] = 0.f;
    if (is_far) {
      float rx[BPT], ry[BPT], rz[BPT];
#pragma unroll
      for (int q = 0; q < BPT; ++q) {  // x_i - c_J, once per tile
        rx[q] = (hx[q] - mj.chi.x) + (lx[q] - mj.clo.x);
        ry[q] = (hy[q] - mj.chi.y) + (ly[q] - mj.clo.y);
        rz[q] = (hz[q] - mj.chi.z) + (lz[q] - mj.clo.z);
      }
      const float4* shf = reinterpret_cast<const float4*>(sh);
#pragma unroll 4
      for (int jj = l; jj < cnt; jj += L) {
        const float4 pj = shf[jj];
#pragma unroll
        for (int q = 0; q < BPT; ++q) {
          const float dx = pj.x - rx[q];
          const float dy = pj.y - ry[q];
          const float dz = pj.z - rz[q];
          const float r2 = fmaf(dz, dz, fmaf(dy, dy, fmaf(dx, dx, eps2)));
          const float rinv = rsqrt_sfu(r2);
          const float s = UNIFORM ? rinv * (rinv * rinv) : (pj.w * rinv) * (rinv * rinv);
          tx[q] = fmaf(s, dx, tx[q]);
          ty[q] = fmaf(s, dy, ty[q]);
          tz[q] = fmaf(s, dz, tz[q]);
        }
      }
    } else {
#pragma unroll 4
      for (int jj = l; jj < cnt; jj += L) {
        const float4 hw = sh[jj].hw;
        const float4 lo = sh[jj].lo;
#pragma unroll
        for (int q = 0; q < BPT; ++q) {
          const float dx = (hw.x - hx[q]) + (lo.x - lx[q]);
          const float dy = (hw.y - hy[q]) + (lo.y - ly[q]);
          const float dz = (hw.z - hz[q]) + (lo.z - lz[q]);
          const float r2 = fmaf(dz, dz, fmaf(dy, dy, fmaf(dx, dx, eps2)));
          const float rinv = rsqrt_sfu(r2);
          const float s = UNIFORM ? rinv * (rinv * rinv) : (hw.w * rinv) * (rinv * rinv);
          tx[q] = fmaf(s, dx, tx[q]);
          ty[q] = fmaf(s, dy, ty[q]);
          tz[q] = fmaf(s, dz, tz[q]);
        }
      }
    }
#pragma unroll
    for (int q = 0; q < BPT; ++q) {
      kahan_add(sx[q], cx[q], tx[q]);
      kahan_add(sy[q], cy[q], ty[q]);
      kahan_add(sz[q], cz[q], tz[q]);
    }
  }
#pragma unroll
  for (int q = 0; q < BPT; ++q) {
    double ax = dsub((double)sx[q], (double)cx[q]);
    double ay = dsub((double)sy[q], (double)cy[q]);
    double az = dsub((double)sz[q], (double)cz[q]);
    ax = lane_reduce<L>(ax);
    ay = lane_reduce<L>(ay);
    az = lane_reduce<L>(az);
    if (l == 0) {
      part[q * BG + g][0] = ax;
      part[q * BG + g][1] = ay;
      part[q * BG + g][2] = az;
    }
  }
}

// Packs FP64 positions (and optional per-body masses) into PackedBody
// records relative to the reference point c.
__device__ __forceinline__ PackedBody pack_body(double x, double y, double z, double cx,
                                                double cy, double cz, float w) {
  PackedBody pb;
  float h, lo;
  split_hilo(dsub(x, cx), h, lo);
  pb.hw.x = h;
  pb.lo.x = lo;
  split_hilo(dsub(y, cy), h, lo);
  pb.hw.y = h;
  pb.lo.y = lo;
  split_hilo(dsub(z, cz), h, lo);
  pb.hw.z = h;
  pb.lo.z = lo;
  pb.hw.w = w;
  pb.lo.w = 0.f;
  return pb;
}

// Launch geometry shared by the standalone and fused kernels.
// Mixed pair loop used when the tiling leaves the choice open: 1 scalar FP32
// (two bodies per thread), 2 / 3 packed f32x2 over pairs of partners with two
// bodies / one body per thread.
constexpr int kDefaultMixedVariant = 3;

struct ForceGeom {
  int T;      // threads per CTA
  int L;      // lanes per body
  int P;      // cluster size
  int BPT;    // bodies per thread (mixed path)
  int variant;  // mixed pair loop: 1 scalar, 2 / 3 packed with two bodies / one body per thread
  long long n_itiles;
  int bodies_per_cta() const { return (T / L) * BPT; }
};

ForceGeom choose_geom(long long n, int precision, const gb_force_tiling* tiling, int exact,
                      bool uniform_masses = true);
int launch_cluster(const void* kernel, const ForceGeom& g, size_t smem, cudaStream_t s,
                   void** args);

}  // namespace gb
