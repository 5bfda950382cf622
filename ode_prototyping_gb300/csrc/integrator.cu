// integrator.cu -- device-resident adaptive embedded RK integrator for one
// N-body system.
//
// Replaces RKEmbeddedParallel<BT>::integrate (src/integrator/RKEmbeddedParallel/
// RKEmbeddedParallel.hpp:13-81) with estimate_initial_step (:170-200).  The
// reference runs every stage, combination, norm and decision as separate
// launches with a blocking device->host copy of the norm per attempt
// (src/par_exec/CudaExecutor.cuh:97-125).  Here one attempt is S launches of
// a fused kernel: stage s computes the accelerations of k_s for its i-tile
// and, in its epilogue, the next stage state y_{s+1} = x0 + dt sum_l a[s][l]
// k_l for the same rows (a row-local operation); the last stage forms
// x = x0 + dt sum b k, err = dt sum (b - bt) k, the error target and the
// scaled squares, reduces them deterministically and applies the step-size
// controller on the device.  Attempts are captured once in a CUDA graph and
// replayed; the host reads the controller state every `attempts_per_sync`
// attempts.  States live in a ring of R slots so that accepting a step is an
// index change, and accepted states can be streamed out without stalling the
// device.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <thread>
#include <vector>

#include "controller.cuh"
#include "epilogue.cuh"
#include "mlp.cuh"
#include "sortpack.cuh"

namespace gb {

int launch_norm(const double* v, const double* s, long long n, double* partial, double* out,
                int take_sqrt, cudaStream_t st);
size_t norm_workspace_bytes(long long n);

namespace {

template <int PREC, int T, int L, int BPT, bool PACKED = false>
__global__ void __launch_bounds__(T, PACKED ? 7 * 128 / T : 5 * 128 / T)
    fused_stage_kernel(const __grid_constant__ DevTableau tab,
                       const __grid_constant__ FusedParams P, int s) {
  constexpr int BI = (T / L) * BPT;
  constexpr int SMEM_BODY_BYTES =
      PREC == GB_PREC_F64
          ? 32 * T
          : (PACKED ? jp_smem_bytes<T>() : (int)sizeof(PackedBody) * T);
  __shared__ __align__(16) unsigned char sh_raw[SMEM_BODY_BYTES];
  __shared__ double part[BI][3];
  __shared__ double red[T];
  Ctrl* C = P.ctrl;
  if (C->done) return;
  const int cur = C->cur;
  const double dt = C->dt;
  const int k0_valid = C->k0_valid;
  const int k0slot = C->k0slot;
  const int px = C->px;
  const int S = tab.n_stages;
  const long long n = P.n, n_var = P.n_var;
  const double* x0 = P.ring + (long long)cur * n_var;
  const double* ysrc = (s == 0) ? x0 : P.Y + (long long)(s & 1) * n_var;
  const ClusterInfo ci = cluster_info();
  const long long i0 = ci.itile * BI;
  const bool skip_force = (s == 0 && k0_valid);
  if (!skip_force) {
    long long jb, je;
    j_chunk(n, ci.rank, ci.size, T, jb, je);
    if constexpr (PREC == GB_PREC_F64) {
      double* sh_pos = reinterpret_cast<double*>(sh_raw);
      double* sh_m = sh_pos + 3 * T;
      force_f64_cta<T, L>(ysrc, n, i0, jb, je, P.eps2, P.masses, sh_pos, sh_m, part,
                          P.f64_fast != 0);
    } else {
      const PackedBody* src = (s == 0) ? P.PX + (long long)px * n : P.PY + (long long)(s & 1) * n;
      if constexpr (PACKED) {
        static_assert(BPT == 1 || BPT == 2, "packed loop: one or two bodies per thread");
        force_mixed_cta_jp<T, L, BPT>(src, n, i0, jb, je, P.eps2f, sh_raw, part);
      } else if (P.masses) {
        force_mixed_cta<T, L, BPT, false>(src, n, i0, jb, je, P.eps2f,
                                          reinterpret_cast<PackedBody*>(sh_raw), part);
      } else {
        force_mixed_cta<T, L, BPT, true>(src, n, i0, jb, je, P.eps2f,
                                         reinterpret_cast<PackedBody*>(sh_raw), part);
      }
    }
    cluster_combine_rows<BI>(part, ci.rank, ci.size);
  }
  // every cluster rank finishes its own rows of the i-tile
  const int rows = (BI + ci.size - 1) / ci.size;
  const int b_lo = ci.rank * rows;
  const int b_hi = (int)min((long long)min(BI, b_lo + rows), n - i0);
  const bool last = (s == S - 1);
  EpiCtx E;
  E.tab = &tab;
  E.s = s;
  E.S = S;
  E.k0slot = k0slot;
  E.skip_force = skip_force;
  E.last = last;
  E.exact = P.exact != 0;
  E.dt = dt;
  E.n = n;
  E.x0 = x0;
  E.ysrc = ysrc;
  E.ks = P.ks;
  E.kstride = n_var;
  E.ynext = P.Y + (long long)((s + 1) & 1) * n_var;
  E.xnew = P.ring + (long long)((cur + 1) % P.R) * n_var;
  E.pnext = last ? P.PX + (long long)(px ^ 1) * n : P.PY + (long long)((s + 1) & 1) * n;
  E.atol = P.atol;
  E.rtol = P.rtol;
  E.atol_s = P.atol_s;
  E.rtol_s = P.rtol_s;
  E.masses = P.masses;
  E.mass = P.mass;
  E.cref = P.cref;
  E.sq = P.sq;
  double sq_acc = 0.0;
  double amax = 0.0;
  if constexpr (L >= 2) {
    // small systems (lanes split each body's partners): the epilogue is a
    // large share of the launch, one state element per thread
    rows_epilogue<PREC, T>(E, i0, b_lo, b_hi, part, sq_acc, amax);
  } else {
    // one lane per body: one body per thread (measured: the per-element form
    // slows the pair loop of these instantiations by 12-15 %)
#pragma unroll 1
    for (int b = b_lo + (int)threadIdx.x; b < b_hi; b += T)
      body_epilogue<PREC>(E, i0 + b, part[b], sq_acc, amax);
  }
  if (last) {
    const double m = block_max(amax, red);
    if (threadIdx.x == 0) P.aux[ci.itile * ci.size + ci.rank] = m;
  }
  if (!last) return;
  const double tile_sum = block_sum(sq_acc, red);
  if (threadIdx.x == 0) P.partials[ci.itile * ci.size + ci.rank] = tile_sum;
}

// Boxes of a sorted tile's new packed positions, one per 64 bodies, by the
// CTA that finishes the tile: min / max of the hi parts (warp shuffles, then
// warp pairs in shared memory), centre and a radius rounded outwards
// (box_from_extents).  The load (box_load, one body per thread) is issued
// early; box_write reduces and writes out[0] (bodies 0..63) and out[1]
// (64..127, when the tile has them).  All 128 threads must call box_write.
__device__ __forceinline__ float4 box_load(const PackedBody* __restrict__ p, int cnt) {
  return (int)threadIdx.x < cnt ? __ldcg(&p[threadIdx.x].hw)
                                : make_float4(nanf(""), 0.f, 0.f, 0.f);
}

__device__ __forceinline__ void box_write(float4 h, int cnt, float4* out, float* red) {
  const bool valid = !isnan(h.x);
  float v[6];
  if (valid) {
    v[0] = h.x; v[1] = h.y; v[2] = h.z;
    v[3] = -h.x; v[4] = -h.y; v[5] = -h.z;
  } else {
#pragma unroll
    for (int k = 0; k < 6; ++k) v[k] = 3.0e38f;
  }
#pragma unroll
  for (int k = 0; k < 6; ++k)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[k] = fminf(v[k], __shfl_xor_sync(0xffffffffu, v[k], o));
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0)
#pragma unroll
    for (int k = 0; k < 6; ++k) red[6 * w + k] = v[k];
  __syncthreads();
  if (threadIdx.x < 2 && 64 * (int)threadIdx.x < cnt) {
    const float* r0 = red + 12 * threadIdx.x;  // warps 2h and 2h + 1
    out[threadIdx.x] = box_from_extents(fminf(r0[0], r0[6]), fminf(r0[1], r0[7]),
                                        fminf(r0[2], r0[8]), -fminf(r0[3], r0[9]),
                                        -fminf(r0[4], r0[10]), -fminf(r0[5], r0[11]));
  }
  __syncthreads();
}

__device__ __forceinline__ void write_tile_box(const PackedBody* __restrict__ p, int cnt,
                                               float4* out, float* red) {
  box_write(box_load(p, cnt), cnt, out, red);
}

// One CTA of 128 threads per tile: packs the positions of x0 (ring slot
// *cur) in the order perm into out[*slot] and writes the tile's two boxes.
__global__ void __launch_bounds__(128)
    pack_boxes_kernel(const double* __restrict__ ring, const int* cur, long long n_var,
                      long long n, const int* __restrict__ perm, const double* __restrict__ cref,
                      PackedBody* out, const int* slot, float4* boxes, long long n_boxes) {
  __shared__ float red[32];
  const double* x = ring + (long long)*cur * n_var;
  PackedBody* o = out + (long long)*slot * n;
  const long long i0 = (long long)blockIdx.x * 128;
  const int cnt = (int)min(128LL, n - i0);
  if ((int)threadIdx.x < cnt) {
    const long long id = perm[i0 + threadIdx.x];
    o[i0 + threadIdx.x] =
        pack_body(x[3 * id], x[3 * id + 1], x[3 * id + 2], cref[0], cref[1], cref[2], 1.0f);
  }
  __threadfence_block();
  __syncthreads();
  write_tile_box(o + i0, cnt, boxes + (long long)*slot * n_boxes + 2 * blockIdx.x, red);
}

__global__ void iota_kernel(int* p, long long n) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) p[i] = (int)i;
}

// Rows [rb, rb + cnt) of a sorted i-tile (bodies perm[i0 + rb ..]): everything
// of the stage combination that does not need this stage's accelerations.  The position elements are finished here (their
// stage derivative is the stage state's velocity): k_s, the next stage state
// (or, at the last stage, the candidate state, its error, target and scaled
// square) and the packed hi/lo positions of the next stage at their sorted
// places.  The velocity elements get their sums over the earlier stages, in
// the ascending order the whole sum uses, so the tile's last CTA adds only
// the last term.  Every thread of the CTA must call it.
template <int T>
__device__ __forceinline__ void split_pre_rows(const DevTableau& tab, const FusedParams& P,
                                               const Ctrl* C, int s, long long i0, int rb,
                                               int cnt, double* sh_pos, double& sq_acc) {
  const int S = tab.n_stages;
  const bool last = (s == S - 1);
  const long long n = P.n, n_var = P.n_var;
  const int k0slot = C->k0slot;
  const double dt = C->dt;
  const int cur = C->cur;
  const double* x0 = P.ring + (long long)cur * n_var;
  const double* ysrc = (s == 0) ? x0 : P.Y + (long long)(s & 1) * n_var;
  const int h3 = 3 * cnt;
  double* ks_s = P.ks + (long long)kslot(s, S, k0slot) * n_var;
  for (int v = threadIdx.x; v < 2 * h3; v += T) {
    const bool pos = v < h3;
    const int w = pos ? v : v - h3;
    const long long body = P.perm[i0 + rb + w / 3];
    const long long e3 = 3 * body + w % 3;  // element of the 3N half
    const long long idx = (pos ? 0 : 3 * n) + e3;
    double ks_now = 0.0;
    if (pos) {
      ks_now = ysrc[3 * n + idx];  // dx/dt = v of the stage state
      ks_s[idx] = ks_now;
    }
    // every term's load in flight at once (this runs after the pair loop,
    // whose registers are no longer live), then the sum in stage order
    double kl[GB_MAX_STAGES];
    if (!last) {
      const unsigned m = tab.anz[s];
#pragma unroll
      for (int l = 0; l < GB_MAX_STAGES; ++l)
        if (l < s && ((m >> l) & 1u)) kl[l] = P.ks[(long long)kslot(l, S, k0slot) * n_var + idx];
      double acc = 0.0;
#pragma unroll
      for (int l = 0; l < GB_MAX_STAGES; ++l)
        if (l < s && ((m >> l) & 1u)) acc = dadd(acc, dmul(tab.a[s][l], kl[l]));
      if (pos) {
        if ((m >> s) & 1u) acc = dadd(acc, dmul(tab.a[s][s], ks_now));
        const double y = dadd(x0[idx], dmul(acc, dt));
        P.Y[(long long)((s + 1) & 1) * n_var + idx] = y;
        sh_pos[w] = y;
      } else {
        P.pre[e3] = acc;
      }
    } else {
      const unsigned mb = tab.bnz, md = tab.dbnz, m = mb | md;
      const int lend = pos ? S : S - 1;  // velocity elements: all but the last stage
#pragma unroll
      for (int l = 0; l < GB_MAX_STAGES; ++l)
        if (l < lend && ((m >> l) & 1u))
          kl[l] = (l == s) ? ks_now : P.ks[(long long)kslot(l, S, k0slot) * n_var + idx];
      double xv = 0.0, ev = 0.0;
#pragma unroll
      for (int l = 0; l < GB_MAX_STAGES; ++l) {
        if (l >= lend) break;
        if ((mb >> l) & 1u) xv = dadd(xv, dmul(tab.b[l], kl[l]));
        if ((md >> l) & 1u) ev = dadd(ev, dmul(tab.db[l], kl[l]));
      }
      if (pos) {
        const double x0e = x0[idx];
        const double xn = dadd(x0e, dmul(xv, dt));
        const double er = dmul(ev, dt);
        P.ring[(long long)((cur + 1) % P.R) * n_var + idx] = xn;
        const double at = P.atol ? P.atol[idx] : P.atol_s;
        const double rt = P.rtol ? P.rtol[idx] : P.rtol_s;
        const double ax = fabs(xn), ax0 = fabs(x0e);
        const double tg = dadd(at, dmul(rt, ax < ax0 ? ax0 : ax));
        const double q = __ddiv_rn(er, tg);
        sq_acc = dadd(sq_acc, dmul(q, q));
        sh_pos[w] = xn;
      } else {
        P.pre[e3] = xv;
        P.pre[3 * n + e3] = ev;
      }
    }
  }
  __syncthreads();
  PackedBody* dst = last ? P.PX + (long long)(C->px ^ 1) * n : P.PY + (long long)((s + 1) & 1) * n;
  for (int r = threadIdx.x; r < cnt; r += T) {
    const double* p = sh_pos + 3 * r;
    dst[i0 + rb + r] = pack_body(p[0], p[1], p[2], P.cref[0], P.cref[1], P.cref[2], 1.0f);
  }
}

// The packed mixed stage (uniform masses, from N = 8192) as independent
// (i-tile, partner chunk) CTAs on Morton-sorted bodies.  Clusters are not
// used: cluster-bound CTAs of one launch drained each SM from seven resident
// CTAs to one (the warp schedulers favour older CTAs: identical CTAs finished
// their pair loops between 45 and 128 us at N = 16384) while an 8-CTA cluster
// waited for its slowest rank; independent CTAs let the block scheduler
// refill every SM until the last chunks.  Each CTA runs the pair loop, in
// which every 64-partner quarter tile whose box is far from each of a
// warp's 32 bodies skips the close-pair test for that warp (sorted bodies are
// compact, so many are), and stores its chunk's sums as FP32 Kahan pairs;
// the CTAs of a middle band of chunks then finish a slice of the tile's rows
// as far as this stage's accelerations allow (split_pre_rows).  The CTA whose
// arrival completes the tile's count (an atomic increment; nothing waits)
// adds the chunks in chunk order, so the sums do not depend on which CTA
// arrives last, resets the count for the next launch, adds the last term of
// every velocity element and writes the boxes of the tile's new positions for
// the next stage.
template <int T, int L, int BPT>
__global__ void __launch_bounds__(T, 6 * 128 / T)
    fused_split_kernel(const __grid_constant__ DevTableau tab,
                       const __grid_constant__ FusedParams P, int s) {
  static_assert(L == 1 && BPT == 1 && T == 128, "partner chunks: 128 one-body threads");
  constexpr int BI = T;
  constexpr int BW = BI * 3;  // sums of one chunk (8 bytes each)
  __shared__ __align__(16) unsigned char sh_raw[jp_smem_bytes<T>()];
  __shared__ double part[BI][3];
  __shared__ double red[T];
  __shared__ double sh_pos[3 * BI];
  __shared__ int sh_last;
  Ctrl* C = P.ctrl;
  if (C->done) return;
  // chunk-major order: every tile's chunk 0, then every tile's chunk 1, ...
  // (chunk boundaries from the table in the parameters)
  const int nc = P.n_chunks;
  const long long itile = blockIdx.x % P.n_itiles;
  const int chunk = (int)(blockIdx.x / P.n_itiles);
  const long long n = P.n, n_var = P.n_var;
  const long long i0 = itile * BI;
  const int S = tab.n_stages;
  const bool last = (s == S - 1);
  const bool skip_force = (s == 0 && C->k0_valid);
  const int b_hi = (int)min((long long)BI, n - i0);
  PackedBody* pnext = last ? P.PX + (long long)(C->px ^ 1) * n : P.PY + (long long)((s + 1) & 1) * n;
  // boxes: two per tile (64 bodies each) per buffer
  float4* box_next = last ? P.BX + (long long)(C->px ^ 1) * 2 * P.n_itiles
                          : P.BY + (long long)((s + 1) & 1) * 2 * P.n_itiles;
  if (skip_force) {
    // the stage derivative is reused: one CTA per tile runs the whole epilogue
    if (chunk != 0) return;
    const int cur = C->cur;
    const double* x0 = P.ring + (long long)cur * n_var;
    EpiCtx E;
    E.tab = &tab;
    E.s = s;
    E.S = S;
    E.k0slot = C->k0slot;
    E.skip_force = true;
    E.last = last;
    E.exact = false;
    E.dt = C->dt;
    E.n = n;
    E.x0 = x0;
    E.ysrc = x0;
    E.ks = P.ks;
    E.kstride = n_var;
    E.ynext = P.Y + (long long)((s + 1) & 1) * n_var;
    E.xnew = P.ring + (long long)((cur + 1) % P.R) * n_var;
    E.pnext = nullptr;
    E.atol = P.atol;
    E.rtol = P.rtol;
    E.atol_s = P.atol_s;
    E.rtol_s = P.rtol_s;
    E.masses = nullptr;
    E.mass = P.mass;
    E.cref = P.cref;
    E.sq = nullptr;
    double sq_acc = 0.0, amax = 0.0;
    if ((int)threadIdx.x < b_hi) {
      double np[3];
      body_epilogue<GB_PREC_MIXED>(E, P.perm[i0 + threadIdx.x], part[threadIdx.x], sq_acc, amax,
                                   np);
      pnext[i0 + threadIdx.x] = pack_body(np[0], np[1], np[2], P.cref[0], P.cref[1], P.cref[2],
                                          1.0f);
    }
    __threadfence_block();
    __syncthreads();
    write_tile_box(pnext + i0, b_hi, box_next + 2 * itile, reinterpret_cast<float*>(red));
    return;
  }
  const long long jb = P.chunk_start[chunk], je = P.chunk_start[chunk + 1];
  const PackedBody* src = (s == 0) ? P.PX + (long long)C->px * n : P.PY + (long long)(s & 1) * n;
  const float4* boxes = (s == 0) ? P.BX + (long long)C->px * 2 * P.n_itiles
                                 : P.BY + (long long)(s & 1) * 2 * P.n_itiles;
  force_mixed_cta_jp<T, L, BPT, true, true>(src, n, i0, jb, je, P.eps2f, sh_raw, part, boxes,
                                            P.cull);
  __syncthreads();
  // the chunk's sums leave as FP32 Kahan pairs (s, -c)
  const float2* pf = reinterpret_cast<const float2*>(&part[0][0]);
  float2* mine = reinterpret_cast<float2*>(P.chunk_sums) + (itile * nc + chunk) * BW;
  for (int e = threadIdx.x; e < BW; e += T) mine[e] = pf[e];
  // The CTAs of chunks [nc/4, nc/2) finish the tile's rows as far as this
  // stage's accelerations allow, one slice each, after their pair loops: not
  // before the pair loop of the first wave (it would hold every SM's FMA pipes
  // idle while its FP64 loads return), not in the last chunks (their CTAs end
  // the launch).  At the last stage every chunk's slot of the partial sums is
  // written (zero outside those CTAs).  Measured at N = 16384 (RKF78 stage):
  // slices in chunks [nc/4, nc/2) 0.1316 ms, in [nc/2, 3nc/4) 0.1361 ms.
  {
    const int c0 = nc / 4, npre = max(1, nc / 4);
    const int slice = chunk - c0;
    double sq_pos = 0.0;
    if (slice >= 0 && slice < npre) {
      const int rpc = (BI + npre - 1) / npre;
      const int rb = slice * rpc;
      const int cnt = max(0, min(b_hi, rb + rpc) - rb);
      split_pre_rows<T>(tab, P, C, s, i0, rb, cnt, sh_pos, sq_pos);
    }
    if (last) {
      const double v = block_sum(sq_pos, red);
      if (threadIdx.x == 0) P.partials[itile * (nc + 1) + chunk] = v;
    }
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) sh_last = atomicAdd(P.tile_count + itile, 1u) == (unsigned)(nc - 1);
  __syncthreads();
  if (!sh_last) return;
  __threadfence();
  // What the tile's velocity elements need is loaded first, so its latency
  // overlaps the chunk sums: element e = threadIdx.x + 128 r of the tile's 3 x
  // 128 acceleration components, its state index, x0, the earlier stages'
  // sums, and the box input (the tile's new packed positions).
  const int k0slot = C->k0slot;
  const double dt = C->dt;
  const int cur = C->cur;
  const double* x0 = P.ring + (long long)cur * n_var;
  double* ks_s = P.ks + (long long)kslot(s, S, k0slot) * n_var;
  const int ne = 3 * b_hi;
  long long wv[3];
  double x0v[3], p1[3], p2[3];
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    const int e = (int)threadIdx.x + r * T;
    wv[r] = e < ne ? 3 * (long long)P.perm[i0 + e / 3] + e % 3 : 0;
  }
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    const int e = (int)threadIdx.x + r * T;
    if (e < ne) {
      x0v[r] = x0[3 * n + wv[r]];
      p1[r] = P.pre[wv[r]];
      p2[r] = last ? P.pre[3 * n + wv[r]] : 0.0;
    }
  }
  const float4 bx = box_load(pnext + i0, b_hi);
  // chunks added in chunk order in double-single FP32 arithmetic (the FP64
  // pipe runs at 1/64 of the FP32 rate), eight loads in flight at a time,
  // one conversion per component
  const float2* g0 = reinterpret_cast<const float2*>(P.chunk_sums) + itile * nc * BW;
  double* pw = &part[0][0];
  double acc[3];
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    const int e = (int)threadIdx.x + r * T;
    float hs = 0.f, ls = 0.f;
    for (int c0 = 0; c0 < nc; c0 += 8) {
      float2 vv[8];
#pragma unroll
      for (int c = 0; c < 8; ++c)
        if (c0 + c < nc) vv[c] = __ldcg(g0 + (long long)(c0 + c) * BW + e);
#pragma unroll
      for (int c = 0; c < 8; ++c)
        if (c0 + c < nc) ds_add(hs, ls, vv[c].x, vv[c].y);
    }
    acc[r] = dadd((double)hs, (double)ls);
    pw[e] = acc[r];
  }
  if (threadIdx.x == 0) P.tile_count[itile] = 0u;
  // the velocity elements: k_s = m a, plus the last term of each sum
  double sq_acc = 0.0;
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    const int e = (int)threadIdx.x + r * T;
    if (e >= ne) continue;
    const long long idx = 3 * n + wv[r];
    const double k = dmul(acc[r], P.mass);
    ks_s[idx] = k;
    if (!last) {
      double v = p1[r];
      if ((tab.anz[s] >> s) & 1u) v = dadd(v, dmul(tab.a[s][s], k));
      P.Y[(long long)((s + 1) & 1) * n_var + idx] = dadd(x0v[r], dmul(v, dt));
    } else {
      double xv = p1[r], ev = p2[r];
      if ((tab.bnz >> s) & 1u) xv = dadd(xv, dmul(tab.b[s], k));
      if ((tab.dbnz >> s) & 1u) ev = dadd(ev, dmul(tab.db[s], k));
      const double xn = dadd(x0v[r], dmul(xv, dt));
      const double er = dmul(ev, dt);
      P.ring[(long long)((cur + 1) % P.R) * n_var + idx] = xn;
      const double at = P.atol ? P.atol[idx] : P.atol_s;
      const double rt = P.rtol ? P.rtol[idx] : P.rtol_s;
      const double ax = fabs(xn), ax0 = fabs(x0v[r]);
      const double tg = dadd(at, dmul(rt, ax < ax0 ? ax0 : ax));
      const double q = __ddiv_rn(er, tg);
      sq_acc = dadd(sq_acc, dmul(q, q));
    }
  }
  box_write(bx, b_hi, box_next + 2 * itile, reinterpret_cast<float*>(red));
  if (!last) return;
  double amax = 0.0;
  for (int b = threadIdx.x; b < b_hi; b += T) {
    const double k0 = dmul(pw[3 * b], P.mass), k1 = dmul(pw[3 * b + 1], P.mass),
                 k2 = dmul(pw[3 * b + 2], P.mass);
    amax = fmax(amax, sqrt(k0 * k0 + k1 * k1 + k2 * k2));
  }
  const double m = block_max(amax, red);
  const double tile_sum = block_sum(sq_acc, red);
  if (threadIdx.x == 0) {
    P.aux[itile] = m;
    P.partials[itile * (nc + 1) + nc] = tile_sum;
  }
}

// The mixed-precision stage on Morton-sorted tiles: i-tile = 128 consecutive
// sorted bodies, far j-tiles through the tile-centroid records, the epilogue
// repacks the CTA's own tile (centroid, radius, near and far records) for
// the next stage.
template <int T, int L, int BPT, bool UNIFORM>
__global__ void __launch_bounds__(T, 768 / T)
    fused_sorted_kernel(const __grid_constant__ DevTableau tab,
                        const __grid_constant__ FusedParams P, int s) {
  constexpr int BI = (T / L) * BPT;
  static_assert(BI == T, "one body per thread in the epilogue");
  __shared__ __align__(16) PackedBody sh[T];
  __shared__ double part[BI][3];
  __shared__ double red[T];
  Ctrl* C = P.ctrl;
  if (C->done) return;
  const int cur = C->cur;
  const double dt = C->dt;
  const int k0_valid = C->k0_valid;
  const int k0slot = C->k0slot;
  const int px = C->px;
  const int S = tab.n_stages;
  const long long n = P.n, n_var = P.n_var, nt = P.n_itiles;
  const double* x0 = P.ring + (long long)cur * n_var;
  const double* ysrc = (s == 0) ? x0 : P.Y + (long long)(s & 1) * n_var;
  const ClusterInfo ci = cluster_info();
  const long long i0 = ci.itile * BI;
  const bool skip_force = (s == 0 && k0_valid);
  if (!skip_force) {
    long long jb, je;
    j_chunk(n, ci.rank, ci.size, T, jb, je);
    const PackedBody* near = (s == 0) ? P.PX + (long long)px * n : P.PY + (long long)(s & 1) * n;
    const float4* far = (s == 0) ? P.PXF + (long long)px * n : P.PYF + (long long)(s & 1) * n;
    const TileMeta* meta = (s == 0) ? P.MX + (long long)px * nt : P.MY + (long long)(s & 1) * nt;
    force_mixed_sorted_cta<T, L, BPT, UNIFORM>(near, far, meta, n, ci.itile, jb, je, P.eps2f, sh,
                                               part);
    cluster_combine<BI>(part, ci.rank, ci.size);
  }
  if (ci.rank != 0) return;
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
  E.ks = P.ks;
  E.kstride = n_var;
  E.ynext = P.Y + (long long)((s + 1) & 1) * n_var;
  E.xnew = P.ring + (long long)((cur + 1) % P.R) * n_var;
  E.pnext = nullptr;
  E.atol = P.atol;
  E.rtol = P.rtol;
  E.atol_s = P.atol_s;
  E.rtol_s = P.rtol_s;
  E.masses = P.masses;
  E.mass = P.mass;
  E.cref = P.cref;
  E.sq = nullptr;
  const long long nb = min((long long)BI, n - i0);
  const int b = threadIdx.x;
  const bool valid = b < nb;
  double np[3] = {0.0, 0.0, 0.0};
  double sq_acc = 0.0, amax = 0.0;
  long long id = 0;
  if (valid) {
    id = P.perm[i0 + b];
    body_epilogue<GB_PREC_MIXED>(E, id, part[b], sq_acc, amax, np);
  }
  const long long po = last ? (long long)(px ^ 1) : (long long)((s + 1) & 1);
  PackedBody* near_out = (last ? P.PX : P.PY) + po * n + i0 + b;
  float4* far_out = (last ? P.PXF : P.PYF) + po * n + i0 + b;
  TileMeta* meta_out = (last ? P.MX : P.MY) + po * nt + ci.itile;
  const float w = valid ? (P.masses ? (float)P.masses[id] : 1.0f) : 0.f;
  pack_sorted_tile(np, valid, (int)nb, w, P.cref, near_out, far_out, meta_out, red);
  if (last) {
    const double m = block_max(amax, red);
    if (threadIdx.x == 0) P.aux[ci.itile * ci.size] = m;
  }
  if (!last) return;
  const double tile_sum = block_sum(sq_acc, red);
  if (threadIdx.x == 0) P.partials[ci.itile * ci.size] = tile_sum;
}

// Dense output of DOPRI5 (the continuous extension of Dormand & Prince as
// in Hairer, Norsett & Wanner and NumericalRecipes/StepperDopr5.hpp:179-219):
// for each output time in the step just accepted, theta = (t_out - t_old)/h
// and x(theta) = r1 + theta (r2 + (1-theta) (r3 + theta (r4 + (1-theta) r5)))
// with r1 = y0, r2 = y1 - y0, r3 = h k1 - r2, r4 = r2 - h k7 - r3,
// r5 = h (d1 k1 + d3 k3 + d4 k4 + d5 k5 + d6 k6 + d7 k7).
__global__ void dense_kernel(const __grid_constant__ FusedParams P) {
  const Ctrl* C = P.ctrl;
  const long long lo = C->dense_lo, hi = C->dense_hi;
  if (hi <= lo) return;
  const long long nv = P.n_var;
  const int R = P.R;
  const double* y1 = P.ring + (long long)C->cur * nv;
  const double* y0 = P.ring + (long long)((C->cur + R - 1) % R) * nv;
  const double h = C->dt_hist[0];
  const double t_old = C->t - h;
  const double* k1 = P.ks + (long long)C->dense_k0 * nv;
  const double* k7 = P.ks + (long long)C->dense_klast * nv;
  const double* k3 = P.ks + 2 * nv;
  const double* k4 = P.ks + 3 * nv;
  const double* k5 = P.ks + 4 * nv;
  const double* k6 = P.ks + 5 * nv;
  const double d1 = -12715105075.0 / 11282082432.0, d3 = 87487479700.0 / 32700410799.0,
               d4 = -10690763975.0 / 1880347072.0, d5 = 701980252875.0 / 199316789632.0,
               d6 = -1453857185.0 / 822651844.0, d7 = 69997945.0 / 29380423.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nv;
       i += (long long)gridDim.x * blockDim.x) {
    const double r1 = y0[i];
    const double r2 = y1[i] - y0[i];
    const double r3 = h * k1[i] - r2;
    const double r4 = r2 - h * k7[i] - r3;
    const double r5 =
        h * (d1 * k1[i] + d3 * k3[i] + d4 * k4[i] + d5 * k5[i] + d6 * k6[i] + d7 * k7[i]);
    for (long long j = lo; j < hi; ++j) {
      const double th = (P.dense_t[j] - t_old) / h;
      const double s1 = 1.0 - th;
      P.dense_out[j * nv + i] = r1 + th * (r2 + s1 * (r3 + th * (r4 + s1 * r5)));
    }
  }
}

// End of an attempt: one CTA reduces the per-tile partial sums in tile
// order (or, in exact mode, the per-element squares in element order, as the
// reference's serial executor adds them), forms err = sqrt(sum / n_var)
// (rk_norm, RKEmbeddedParallel.hpp:141-149) and runs the controller.  The
// learned proposal is evaluated cooperatively by the whole CTA with BF16
// weights and FP32 accumulation.
__global__ void __launch_bounds__(256)
    control_kernel(const __grid_constant__ DevTableau tab, const __grid_constant__ FusedParams P) {
  constexpr int T = 256;
  __shared__ double red[T];
  __shared__ float feat[kIn];
  __shared__ float h1[kHid];
  __shared__ float outv;
  __shared__ int sh_flag;
  Ctrl* C = P.ctrl;
  if (C->done) return;
  const int S = tab.n_stages;
  const long long n_var = P.n_var;
  double total;
  if (P.exact) {
    if (threadIdx.x == 0) {
      double v = 0.0;
      for (long long e = 0; e < n_var; ++e) v = dadd(v, P.sq[e]);
      red[0] = v;
    }
    __syncthreads();
    total = red[0];
    __syncthreads();
  } else {
    double v = 0.0;
    for (long long k = threadIdx.x; k < P.n_parts; k += T) v = dadd(v, P.partials[k]);
    total = block_sum(v, red);
  }
  const int k0_valid = C->k0_valid;
  double amax_all = 0.0;
  {
    double v = 0.0;
    for (long long k = threadIdx.x; k < P.n_parts; k += T) v = fmax(v, P.aux[k]);
    amax_all = block_max(v, red);
  }
  const double err = sqrt(total / (double)n_var);
  // Learned proposal: features of the post-attempt state (thread 0), then
  // the 16 -> 64 -> 64 -> 1 network across the CTA.
  if (threadIdx.x == 0) {
    Ctrl c = *C;
    c.max_abs_acc = amax_all;
    const bool want = P.mlp && c.controller == GB_CTRL_LEARNED && isfinite(err) && err <= 1.0;
    sh_flag = want ? 1 : 0;
    if (want) {
      Ctrl pre = c;
      preview_history(pre, err, true);
      make_features(pre, tab, P.n, feat);
    }
  }
  __syncthreads();
  if (sh_flag) {
    mlp_infer_block(P.mlp, feat, h1, &outv);
  }
  if (threadIdx.x == 0) {
    Ctrl c = *C;
    c.max_abs_acc = amax_all;
    c.n_rhs += k0_valid ? S - 1 : S;
    if (k0_valid) c.n_rhs_saved += 1;
    const CtrlEnv env{P.log, P.log_capacity, P.times_ring, P.R, P.n};
    finish_attempt(tab, env, c, err, sh_flag ? (double)outv : 0.0, sh_flag != 0);
    c.dense_lo = c.dense_hi = c.dense_next;
    if (P.dense_t && c.last_accepted) {
      long long j = c.dense_next;
      while (j < P.n_dense && P.dense_t[j] <= c.t) ++j;
      c.dense_hi = j;
      c.dense_next = j;
    }
    *C = c;
  }
}

// ---------------------------------------------------------------------------
// Start-up kernels: initial step (estimate_initial_step, :170-200).
// ---------------------------------------------------------------------------
__global__ void target0_kernel(const double* __restrict__ x0, const double* __restrict__ atol,
                               const double* __restrict__ rtol, double atol_s, double rtol_s,
                               double* __restrict__ tg, long long n) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double a = atol ? atol[i] : atol_s;
  const double r = rtol ? rtol[i] : rtol_s;
  tg[i] = dadd(dmul(fabs(x0[i]), r), a);  // compute_error_target_kernel (:151-156)
}

__device__ __forceinline__ double initial_dt0(double d0, double d1) {
  return (d0 < 1.0e-5 || d1 < 1.0e-5) ? 1.0e-6 : 0.01 * (d0 / d1);
}

__global__ void euler_kernel(const double* __restrict__ x0, const double* __restrict__ f0,
                             const double* __restrict__ d, double* __restrict__ x1, long long n) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double dt0 = initial_dt0(d[0], d[1]);
  x1[i] = dadd(x0[i], dmul(f0[i], dt0));  // euler_step_kernel (:158-162)
}

__global__ void diff_kernel(double* __restrict__ df, const double* __restrict__ f0, long long n) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) df[i] = dsub(df[i], f0[i]);  // difference_kernel (:164-167)
}

__global__ void pack_state_kernel(const double* __restrict__ x, const double* __restrict__ masses,
                                  const double* __restrict__ c, long long n, PackedBody* out) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float w = masses ? (float)masses[i] : 1.0f;
  out[i] = pack_body(x[3 * i], x[3 * i + 1], x[3 * i + 2], c[0], c[1], c[2], w);
}

__global__ void serial_norm_kernel(const double* __restrict__ v, const double* __restrict__ s,
                                   long long n, double* out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double acc = 0.0;
  for (long long i = 0; i < n; ++i) {
    const double q = __ddiv_rn(v[i], s[i]);
    acc = dadd(acc, dmul(q, q));
  }
  *out = sqrt(acc / (double)n);
}

__global__ void centroid_state_kernel(const double* __restrict__ x, long long n, double* c_out) {
  __shared__ double sh[3][256];
  double s0 = 0.0, s1 = 0.0, s2 = 0.0;
  for (long long i = threadIdx.x; i < n; i += blockDim.x) {
    s0 += x[3 * i];
    s1 += x[3 * i + 1];
    s2 += x[3 * i + 2];
  }
  sh[0][threadIdx.x] = s0;
  sh[1][threadIdx.x] = s1;
  sh[2][threadIdx.x] = s2;
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st /= 2) {
    if ((int)threadIdx.x < st) {
      for (int c = 0; c < 3; ++c) sh[c][threadIdx.x] += sh[c][threadIdx.x + st];
    }
    __syncthreads();
  }
  if (threadIdx.x < 3) c_out[threadIdx.x] = sh[threadIdx.x][0] / (double)n;
}

__global__ void init_ctrl_kernel(Ctrl* C, const double* __restrict__ d, double t0, double tf,
                                 double* times_ring, int p, int q, double safety,
                                 int controller, double pi_beta, int fsal,
                                 long long max_attempts, int exact, double log_tol,
                                 long long n) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const double d0 = d[0], d1 = d[1];
  const double dt0 = initial_dt0(d0, d1);
  const double d2 = d[2] / dt0;
  const double dmax = d1 < d2 ? d2 : d1;
  double dt1;
  if (dmax <= 1.0e-15) {
    const double alt = dt0 * 1.0e-3;
    dt1 = alt < 1.0e-6 ? 1.0e-6 : alt;
  } else {
    dt1 = exact ? dd_pow(0.01 / dmax, 1.0 / (1.0 + p)) : pow(0.01 / dmax, 1.0 / (1.0 + p));
  }
  const double big = 100.0 * dt0;
  Ctrl c;
  memset(&c, 0, sizeof c);
  c.exact_pow = exact;
  c.t = t0;
  c.t0 = t0;
  c.tf = tf;
  c.dt = dt1 < big ? dt1 : big;
  c.dt_initial = c.dt;
  c.safety = safety;
  c.q = q;
  c.controller = controller;
  c.pi_beta = pi_beta;
  c.pi_alpha = 1.0 / (1.0 + q) - 0.75 * pi_beta;
  c.err_prev = 1.0e-4;
  c.log_tol = log_tol;
  c.fsal = fsal;
  c.k0_valid = 1;  // f(x0) computed for the estimate is k_0 of the first attempt
  c.k0slot = 0;
  c.cur = 0;
  c.px = 0;
  c.n_rhs = 2;
  c.max_attempts = max_attempts;
  for (int k = 0; k < 3; ++k) {
    c.dt_hist[k] = c.dt;
    c.err_hist[k] = 1.0;
  }
  init_log_cache(c, n);
  c.done = (t0 < tf) ? 0 : 1;
  times_ring[0] = t0;
  *C = c;
}

__global__ void max_acc_kernel(const double* __restrict__ f, long long n, Ctrl* C) {
  __shared__ double red[256];
  double m = 0.0;
  for (long long i = threadIdx.x; i < n; i += blockDim.x) {
    const double ax = f[3 * n + 3 * i], ay = f[3 * n + 3 * i + 1], az = f[3 * n + 3 * i + 2];
    m = fmax(m, sqrt(ax * ax + ay * ay + az * az));
  }
  red[threadIdx.x] = m;
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st /= 2) {
    if ((int)threadIdx.x < st) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + st]);
    __syncthreads();
  }
  if (threadIdx.x == 0) C->max_abs_acc = red[0];
}

unsigned blocks256(long long n) { return (unsigned)((n + 255) / 256); }

// Kernel table ----------------------------------------------------------------
template <int PREC, int T, int BPT>
const void* pick_L(int L) {
  switch (L) {
    case 1: return (const void*)fused_stage_kernel<PREC, T, 1, BPT>;
    case 2: return (const void*)fused_stage_kernel<PREC, T, 2, BPT>;
    case 4: return (const void*)fused_stage_kernel<PREC, T, 4, BPT>;
    case 8: return (const void*)fused_stage_kernel<PREC, T, 8, BPT>;
    default: return nullptr;
  }
}

template <int T, int BPT>
const void* pick_packed(int L) {
  switch (L) {
    case 1: return (const void*)fused_stage_kernel<GB_PREC_MIXED, T, 1, BPT, true>;
    case 2: return (const void*)fused_stage_kernel<GB_PREC_MIXED, T, 2, BPT, true>;
    case 4: return (const void*)fused_stage_kernel<GB_PREC_MIXED, T, 4, BPT, true>;
    default: return nullptr;
  }
}

template <int BPT>
const void* pick_split(int L) {
  return L == 1 ? (const void*)fused_split_kernel<128, 1, BPT> : nullptr;
}

const void* pick_fused(int prec, int T, int L, int BPT, bool packed = false) {
  if (prec == GB_PREC_MIXED && packed) {
    if (T == 128 && BPT == 1) return pick_packed<128, 1>(L);
    if (T == 128 && BPT == 2) return pick_packed<128, 2>(L);
    return nullptr;
  }
  if (prec == GB_PREC_F64) {
    if (BPT != 1) return nullptr;
    switch (T) {
      case 64: return pick_L<GB_PREC_F64, 64, 1>(L);
      case 128: return pick_L<GB_PREC_F64, 128, 1>(L);
      case 256: return pick_L<GB_PREC_F64, 256, 1>(L);
    }
    return nullptr;
  }
  switch (T) {
    case 128:
      if (BPT == 1) return pick_L<GB_PREC_MIXED, 128, 1>(L);
      if (BPT == 2) return pick_L<GB_PREC_MIXED, 128, 2>(L);
      return nullptr;
    case 256:
      if (BPT == 1) return pick_L<GB_PREC_MIXED, 256, 1>(L);
      if (BPT == 2) return pick_L<GB_PREC_MIXED, 256, 2>(L);
      return nullptr;
  }
  return nullptr;
}

template <int T, int L, bool U>
const void* sorted_ptr() {
  return (const void*)fused_sorted_kernel<T, L, L, U>;
}

const void* pick_sorted(int T, int L, bool uniform) {
#define GB_SK(T_, L_)                                                        \
  if (T == T_ && L == L_) return uniform ? sorted_ptr<T_, L_, true>() : sorted_ptr<T_, L_, false>();
  GB_SK(128, 1) GB_SK(128, 2) GB_SK(256, 1) GB_SK(256, 2)
#undef GB_SK
  return nullptr;
}

}  // namespace

// Standalone RHS used by the start-up (initial step) path.
int rhs_for_start(int prec, const double* x, double* dxdt, long long n, double softening,
                  double mass, const double* masses, const PackedBody* packed, int exact,
                  const gb_force_tiling* tiling, cudaStream_t s);

}  // namespace gb

// ---------------------------------------------------------------------------
// Host object
// ---------------------------------------------------------------------------
struct gb_integrator_s {
  gb::DevTableau tab;
  gb_tableau htab;
  gb_nbody_system sys;
  gb_integrate_opts opts;
  gb::ForceGeom geom;
  const void* kernel = nullptr;
  bool split = false;               // packed mixed stage as independent partner chunks
  std::vector<long long> chunks;    // partner chunk boundaries of the split stage
  gb_force_tiling start_tiling{};   // right-hand sides of the initial step
  cudaStream_t user_stream = nullptr;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  cudaEvent_t ev = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  long long n = 0, n_var = 0;
  int S = 0, R = 0, A = 0;
  // device buffers
  gb::Ctrl* ctrl = nullptr;
  double* ring = nullptr;
  double* times_ring = nullptr;
  double* ks = nullptr;
  double* Y = nullptr;
  gb::PackedBody* PX = nullptr;
  gb::PackedBody* PY = nullptr;
  double* atol = nullptr;
  double* rtol = nullptr;
  double* cref = nullptr;
  double* partials = nullptr;
  double* aux = nullptr;
  double* sq = nullptr;
  double* dscal = nullptr;  // initial-step norms
  double* norm_work = nullptr;
  double* masses = nullptr;
  gb::StepLog* log = nullptr;
  long long log_capacity = 0;
  // spatially sorted mixed path
  bool sorted = false;
  int* perm = nullptr;
  int* vals = nullptr;
  unsigned long long* keys = nullptr;
  unsigned long long* keys_alt = nullptr;
  void* cub_temp = nullptr;
  size_t cub_bytes = 0;
  double* bbox = nullptr;
  float4* PXF = nullptr;
  float4* PYF = nullptr;
  gb::TileMeta* MX = nullptr;
  gb::TileMeta* MY = nullptr;
  double* dense_t = nullptr;
  double* dense_out = nullptr;
  long long n_dense = 0;
  void* mlp_dev = nullptr;
  double* chunk_sums = nullptr;
  unsigned* tile_count = nullptr;
  double* pre = nullptr;
  float4* BX = nullptr;
  float4* BY = nullptr;
  bool split_sort = false;          // split stage on Morton-sorted bodies
  // host
  gb::Ctrl* hctrl = nullptr;  // pinned
  double* hstage = nullptr;   // pinned R * n_var (recording)
  double* htimes = nullptr;   // pinned R
  std::vector<double> hstate;
  long long delivered = 0;    // accepted states handed to the save callback
  bool started = false;
  double atol_s = 0.0, rtol_s = 0.0;
  gb::FusedParams params;
};

namespace gb {
namespace {

int wait_event(cudaEvent_t ev, double timeout_s) {
  const auto t0 = std::chrono::steady_clock::now();
  for (;;) {
    cudaError_t e = cudaEventQuery(ev);
    if (e == cudaSuccess) return GB_OK;
    if (e != cudaErrorNotReady) {
      note_cuda_error(e);
      return GB_ERR_CUDA;
    }
    const double el =
        std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (el > timeout_s) return GB_ERR_TIMEOUT;
    std::this_thread::sleep_for(std::chrono::microseconds(el < 0.01 ? 5 : 200));
  }
}

void free_all(gb_integrator_s* it) {
  if (it->exec) cudaGraphExecDestroy(it->exec);
  if (it->graph) cudaGraphDestroy(it->graph);
  void* bufs[] = {it->ctrl,  it->ring, it->times_ring, it->ks,     it->Y,        it->PX,
                  it->PY,    it->atol, it->rtol,       it->cref,   it->partials, it->aux,
                  it->sq,    it->dscal, it->norm_work, it->masses, it->log,      it->mlp_dev,
                  it->perm,  it->vals, it->keys,     it->keys_alt, it->cub_temp, it->bbox,
                  it->PXF,   it->PYF,  it->MX,       it->MY,       it->dense_t, it->dense_out,
                  it->chunk_sums, it->tile_count, it->pre, it->BX, it->BY};
  for (void* p : bufs)
    if (p) cudaFree(p);
  if (it->hctrl) cudaFreeHost(it->hctrl);
  if (it->hstage) cudaFreeHost(it->hstage);
  if (it->htimes) cudaFreeHost(it->htimes);
  if (it->ev) cudaEventDestroy(it->ev);
  if (it->stream && it->own_stream) cudaStreamDestroy(it->stream);
}

// Partner chunk boundaries of the split stage kernel, each a multiple of 128
// partners (a tile of the box test; the packed loop takes any run of pairs).
// CTAs are dispatched chunk-major, so the last chunks are the last work of
// the launch: their lengths fall off, in the weights 6 (first half of the
// chunks), 4, 2 (an eighth each) and 1 (the rest), so that the SMs drain on
// short CTAs (measured at N = 16384, 16 chunks: 0.1350 ms per RKF78 stage
// against 0.1384 ms for equal chunks; 8 or 32 chunks, equal or falling, were
// no faster).
std::vector<long long> split_schedule(long long n, int nc) {
  const long long tiles = (n + 127) / 128;
  std::vector<long long> w((size_t)nc), b;
  const int h = nc / 2, e = nc / 8;
  long long total = 0;
  for (int c = 0; c < nc; ++c) {
    w[c] = c < h ? 6 : (c < h + e ? 4 : (c < h + 2 * e ? 2 : 1));
    total += w[c];
  }
  long long acc = 0;
  for (int c = 0; c < nc; ++c) {
    b.push_back(std::min(n, 128 * (tiles * acc / total)));
    acc += w[c];
  }
  b.push_back(n);
  return b;
}

int launch_stage_kernel(gb_integrator_s* it, void** args) {
  if (!it->split) return launch_cluster(it->kernel, it->geom, 0, it->stream, args);
  const dim3 grid((unsigned)(it->geom.n_itiles * it->geom.P)), block((unsigned)it->geom.T);
  GB_CUDA_TRY(cudaLaunchKernel(it->kernel, grid, block, args, 0, it->stream));
  return GB_OK;
}

int launch_fused(gb_integrator_s* it, int s) {
  void* args[] = {(void*)&it->tab, (void*)&it->params, (void*)&s};
  GB_TRY(launch_stage_kernel(it, args));
  if (s == it->S - 1) {
    control_kernel<<<1, 256, 0, it->stream>>>(it->tab, it->params);
    GB_CUDA_TRY(cudaGetLastError());
    if (it->params.dense_t) {
      dense_kernel<<<(unsigned)std::min<long long>((it->n_var + 255) / 256, 1024), 256, 0,
                     it->stream>>>(it->params);
      GB_CUDA_TRY(cudaGetLastError());
    }
  }
  return GB_OK;
}

// Re-sorts the bodies of x0 along a Morton curve and repacks x0's tiles (and
// their boxes, split stage).
int launch_resort(gb_integrator_s* it) {
  if (it->split) {
    cudaStream_t s = it->stream;
    const int* cur = reinterpret_cast<const int*>(reinterpret_cast<const char*>(it->ctrl) +
                                                  offsetof(Ctrl, cur));
    const int* px = reinterpret_cast<const int*>(reinterpret_cast<const char*>(it->ctrl) +
                                                 offsetof(Ctrl, px));
    if (it->split_sort) {
      SortBuffers sb{it->perm, it->vals, it->keys, it->keys_alt, it->cub_temp, it->cub_bytes,
                     it->bbox};
      GB_TRY(sort_bodies(it->ring, cur, it->n_var, it->n, sb, s));
    }
    pack_boxes_kernel<<<(unsigned)it->geom.n_itiles, 128, 0, s>>>(
        it->ring, cur, it->n_var, it->n, it->perm, it->cref, it->PX, px, it->BX,
        2 * it->geom.n_itiles);
    GB_CUDA_TRY(cudaGetLastError());
    return GB_OK;
  }
  if (!it->sorted) return GB_OK;
  cudaStream_t s = it->stream;
  const long long n = it->n;
  const int* cur = reinterpret_cast<const int*>(reinterpret_cast<const char*>(it->ctrl) +
                                                offsetof(Ctrl, cur));
  const int* px = reinterpret_cast<const int*>(reinterpret_cast<const char*>(it->ctrl) +
                                               offsetof(Ctrl, px));
  SortBuffers sb{it->perm, it->vals, it->keys, it->keys_alt, it->cub_temp, it->cub_bytes,
                 it->bbox};
  return sort_and_pack(it->ring, cur, it->n_var, n, sb, it->masses, it->cref, it->PX, it->PXF,
                       it->MX, px, it->geom.n_itiles, it->geom.T, s);
}

int build_graph(gb_integrator_s* it) {
  GB_CUDA_TRY(cudaStreamBeginCapture(it->stream, cudaStreamCaptureModeThreadLocal));
  int rc = launch_resort(it);
  for (int a = 0; a < it->A && rc == GB_OK; ++a)
    for (int s = 0; s < it->S && rc == GB_OK; ++s) rc = launch_fused(it, s);
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(it->stream, &g);
  if (rc != GB_OK) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  GB_CUDA_TRY(e);
  it->graph = g;
  GB_CUDA_TRY(cudaGraphInstantiate(&it->exec, g, 0));
  return GB_OK;
}

int read_ctrl(gb_integrator_s* it) {
  GB_CUDA_TRY(cudaMemcpyAsync(it->hctrl, it->ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost,
                              it->stream));
  GB_CUDA_TRY(cudaEventRecord(it->ev, it->stream));
  return wait_event(it->ev, it->opts.host_wait_timeout_s);
}

// Hands newly accepted states to the callback, in order (ring slots
// delivered+1 .. n_accepted): each contiguous run of slots is copied to
// pinned staging in one transfer, then delivered state by state.
int drain(gb_integrator_s* it, gb_save_fn save, void* user) {
  if (!save || !it->opts.record) {
    it->delivered = it->hctrl->n_accepted;
    return GB_OK;
  }
  const long long upto = it->hctrl->n_accepted;
  long long k = it->delivered + 1;
  while (k <= upto) {
    const int slot0 = (int)(k % it->R);
    const long long run = std::min<long long>(upto - k + 1, it->R - slot0);
    GB_CUDA_TRY(cudaMemcpyAsync(it->hstage, it->ring + (long long)slot0 * it->n_var,
                                (size_t)run * it->n_var * sizeof(double),
                                cudaMemcpyDeviceToHost, it->stream));
    GB_CUDA_TRY(cudaMemcpyAsync(it->htimes, it->times_ring + slot0, (size_t)run * sizeof(double),
                                cudaMemcpyDeviceToHost, it->stream));
    GB_CUDA_TRY(cudaStreamSynchronize(it->stream));
    for (long long j = 0; j < run; ++j)
      save(user, it->htimes[j], it->hstage + j * it->n_var, it->n_var);
    k += run;
  }
  it->delivered = upto;
  return GB_OK;
}

}  // namespace

}  // namespace gb

using namespace gb;

extern "C" int gb_integrator_create(const gb_tableau* tab, const gb_nbody_system* sys,
                                    const gb_integrate_opts* opts_in, gb_stream_t stream,
                                    gb_integrator* out) {
  if (!out) return GB_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  GB_TRY(check_tableau(tab));
  if (!sys || sys->n_particles < 1 || !(sys->softening >= 0.0)) return GB_ERR_INVALID_ARGUMENT;
  if (!sys->masses_dev && !(sys->mass > 0.0)) return GB_ERR_INVALID_ARGUMENT;
  gb_integrate_opts opts;
  std::memset(&opts, 0, sizeof opts);
  if (opts_in) opts = *opts_in;
  if (opts.precision != GB_PREC_F64 && opts.precision != GB_PREC_MIXED)
    return GB_ERR_INVALID_ARGUMENT;
  if (opts.precision == GB_PREC_MIXED && !(sys->softening > 0.0)) return GB_ERR_INVALID_ARGUMENT;
  if (opts.precision == GB_PREC_MIXED && opts.exact) return GB_ERR_INVALID_ARGUMENT;
  if (opts.controller < GB_CTRL_REFERENCE || opts.controller > GB_CTRL_LEARNED)
    return GB_ERR_INVALID_ARGUMENT;
  if (opts.controller == GB_CTRL_LEARNED && !opts.mlp) return GB_ERR_INVALID_ARGUMENT;
  if (opts.attempts_per_sync <= 0) opts.attempts_per_sync = 16;
  if (opts.attempts_per_sync > 4096) opts.attempts_per_sync = 4096;
  if (opts.host_wait_timeout_s <= 0.0) opts.host_wait_timeout_s = 600.0;
  if (opts.pi_beta <= 0.0) opts.pi_beta = 0.04;

  auto* it = new gb_integrator_s();
  it->htab = *tab;
  it->tab = make_dev_tableau(*tab);
  if (!opts.fsal) it->tab.fsal = 0;
  it->sys = *sys;
  it->opts = opts;
  it->n = sys->n_particles;
  it->n_var = 6 * it->n;
  it->S = tab->n_stages;
  it->A = opts.attempts_per_sync;
  it->R = opts.record ? it->A + 2 : 2;
  it->user_stream = as_cuda(stream);
  it->geom = choose_geom(it->n, opts.precision, &opts.tiling, opts.exact,
                         sys->masses_dev == nullptr);
  if (opts.precision == GB_PREC_F64) it->geom.BPT = 1;
  if (opts.precision == GB_PREC_MIXED && it->geom.T < 128) it->geom.T = 128;
  // spatially sorted tiles (mixed precision): on unless switched off
  it->sorted = opts.precision == GB_PREC_MIXED && opts.spatial_sort == 1;
  if (it->sorted) {
    if (it->geom.L > 2) it->geom.L = 2;
    it->geom.BPT = it->geom.L;  // i-tile = j-tile = T bodies
  }
  // One-lane packed mixed stages run as independent partner chunks
  // (fused_split_kernel); from N = 8192 one lane per body with chunks of about
  // 1024 partners, at most 32 per tile (measured per RKF78 stage: N = 8192
  // 0.0563 ms against 0.0594 ms for clusters of 8 x 2 lanes; 16384 0.142
  // against 0.155; 32768 0.470 against 0.513; 131072 6.88 against 7.37).
  if (!it->sorted && opts.precision == GB_PREC_MIXED && it->geom.variant == 3 && !opts.exact) {
    if (it->n >= 8192) {
      if (opts.tiling.lanes <= 0) it->geom.L = 1;
      if (it->geom.L == 1 && opts.tiling.j_split <= 0) {
        int P = 8;
        while (P < 32 && (long long)P * 2 * 1024 <= it->n) P *= 2;
        it->geom.P = P;
      }
    }
    it->split = it->geom.L == 1 && it->geom.P > 1 && it->geom.T == 128 && it->geom.BPT == 1;
    if (it->split) {
      it->chunks = split_schedule(it->n, std::min(it->geom.P, kMaxChunks));
      it->geom.P = (int)it->chunks.size() - 1;
      // spatial_sort 3: bodies in their own order (no Morton sort)
      it->split_sort = opts.spatial_sort != 3;
    }
  }
  it->geom.n_itiles = (it->n + it->geom.bodies_per_cta() - 1) / it->geom.bodies_per_cta();
  it->kernel = it->sorted ? pick_sorted(it->geom.T, it->geom.L, sys->masses_dev == nullptr)
                          : pick_fused(opts.precision, it->geom.T, it->geom.L, it->geom.BPT,
                                       it->geom.variant != 1);
  if (it->split) it->kernel = pick_split<1>(it->geom.L);
  it->start_tiling = opts.tiling;
  if (it->start_tiling.j_split > 8) it->start_tiling.j_split = 8;
  int rc = GB_OK;
  auto fail = [&](int code) {
    free_all(it);
    delete it;
    return code;
  };
  if (!it->kernel) return fail(GB_ERR_UNSUPPORTED);
  if (!it->split && it->geom.P > 8 &&
      cudaFuncSetAttribute(it->kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) !=
          cudaSuccess)
    return fail(GB_ERR_UNSUPPORTED);  // 16-CTA clusters opt-in before any graph capture
  const long long n = it->n, nv = it->n_var;
  cudaError_t e = cudaSuccess;
#define GB_ALLOC(ptr, bytes)                                        \
  do {                                                              \
    e = cudaMalloc((void**)&(ptr), (bytes));                        \
    if (e != cudaSuccess) {                                         \
      note_cuda_error(e);                                           \
      return fail(GB_ERR_CUDA);                                     \
    }                                                               \
  } while (0)
  GB_ALLOC(it->ctrl, sizeof(Ctrl));
  GB_ALLOC(it->ring, (size_t)it->R * nv * sizeof(double));
  GB_ALLOC(it->times_ring, (size_t)it->R * sizeof(double));
  GB_ALLOC(it->ks, (size_t)it->S * nv * sizeof(double));
  GB_ALLOC(it->Y, (size_t)2 * nv * sizeof(double));
  GB_ALLOC(it->cref, 4 * sizeof(double));
  // one partial per (i-tile, cluster rank), or per (i-tile, chunk) plus one
  // per i-tile in the split stage; entries a kernel does not write stay 0
  const size_t n_parts = (size_t)it->geom.n_itiles * (it->geom.P + (it->split ? 1 : 0));
  GB_ALLOC(it->partials, n_parts * sizeof(double));
  GB_ALLOC(it->aux, n_parts * sizeof(double));
  e = cudaMemset(it->partials, 0, n_parts * sizeof(double));
  if (e == cudaSuccess) e = cudaMemset(it->aux, 0, n_parts * sizeof(double));
  if (e == cudaSuccess && it->split) {
    GB_ALLOC(it->chunk_sums, n_parts * 3 * (size_t)it->geom.bodies_per_cta() * sizeof(double));
    GB_ALLOC(it->tile_count, (size_t)it->geom.n_itiles * sizeof(unsigned));
    e = cudaMemset(it->tile_count, 0, (size_t)it->geom.n_itiles * sizeof(unsigned));
    GB_ALLOC(it->pre, (size_t)nv * sizeof(double));
    GB_ALLOC(it->BX, (size_t)4 * it->geom.n_itiles * sizeof(float4));  // 2 buffers x 2 per tile
    GB_ALLOC(it->BY, (size_t)4 * it->geom.n_itiles * sizeof(float4));
    GB_ALLOC(it->perm, (size_t)n * sizeof(int));
    if (e == cudaSuccess) {
      iota_kernel<<<(unsigned)((n + 255) / 256), 256>>>(it->perm, n);
      e = cudaGetLastError();
    }
    if (it->split_sort) {
      GB_ALLOC(it->vals, (size_t)n * sizeof(int));
      GB_ALLOC(it->keys, (size_t)n * sizeof(unsigned long long));
      GB_ALLOC(it->keys_alt, (size_t)n * sizeof(unsigned long long));
      GB_ALLOC(it->bbox, 8 * sizeof(double));
      it->cub_bytes = sort_temp_bytes(n);
      GB_ALLOC(it->cub_temp, it->cub_bytes);
    }
  }
  if (e != cudaSuccess) {
    note_cuda_error(e);
    return fail(GB_ERR_CUDA);
  }
  GB_ALLOC(it->dscal, 8 * sizeof(double));
  GB_ALLOC(it->norm_work, norm_workspace_bytes(nv));
  if (opts.exact) GB_ALLOC(it->sq, (size_t)nv * sizeof(double));
  if (opts.precision == GB_PREC_MIXED) {
    GB_ALLOC(it->PX, (size_t)2 * n * sizeof(PackedBody));
    GB_ALLOC(it->PY, (size_t)2 * n * sizeof(PackedBody));
  }
  if (sys->masses_dev) {
    GB_ALLOC(it->masses, (size_t)n * sizeof(double));
    e = cudaMemcpy(it->masses, sys->masses_dev, n * sizeof(double), cudaMemcpyDeviceToDevice);
    if (e != cudaSuccess) {
      note_cuda_error(e);
      return fail(GB_ERR_CUDA);
    }
  }
  if (it->sorted) {
    GB_ALLOC(it->perm, (size_t)n * sizeof(int));
    GB_ALLOC(it->vals, (size_t)n * sizeof(int));
    GB_ALLOC(it->keys, (size_t)n * sizeof(unsigned long long));
    GB_ALLOC(it->keys_alt, (size_t)n * sizeof(unsigned long long));
    GB_ALLOC(it->bbox, 8 * sizeof(double));
    GB_ALLOC(it->PXF, (size_t)2 * n * sizeof(float4));
    GB_ALLOC(it->PYF, (size_t)2 * n * sizeof(float4));
    GB_ALLOC(it->MX, (size_t)2 * it->geom.n_itiles * sizeof(TileMeta));
    GB_ALLOC(it->MY, (size_t)2 * it->geom.n_itiles * sizeof(TileMeta));
    it->cub_bytes = sort_temp_bytes(n);
    GB_ALLOC(it->cub_temp, it->cub_bytes);
  }
  if (opts.log_steps > 0) {
    it->log_capacity = opts.log_steps;
    GB_ALLOC(it->log, (size_t)it->log_capacity * sizeof(StepLog));
  }
  if (opts.controller == GB_CTRL_LEARNED) {
    it->mlp_dev = mlp_upload(opts.mlp, &rc);
    if (!it->mlp_dev) return fail(rc == GB_OK ? GB_ERR_INVALID_ARGUMENT : rc);
  }
#undef GB_ALLOC
  e = cudaMallocHost((void**)&it->hctrl, sizeof(Ctrl));
  if (e == cudaSuccess && opts.record)
    e = cudaMallocHost((void**)&it->hstage, (size_t)it->R * nv * sizeof(double));
  if (e == cudaSuccess && opts.record)
    e = cudaMallocHost((void**)&it->htimes, (size_t)it->R * sizeof(double));
  if (e == cudaSuccess) {
    // Graphs cannot be captured on the legacy default stream: run on the
    // caller's stream when it is a real stream, else on an owned one.
    if (it->user_stream) {
      it->stream = it->user_stream;
    } else {
      e = cudaStreamCreateWithFlags(&it->stream, cudaStreamNonBlocking);
      it->own_stream = true;
    }
  }
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&it->ev, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaMemset(it->ctrl, 0, sizeof(Ctrl));
  if (e != cudaSuccess) {
    note_cuda_error(e);
    return fail(GB_ERR_CUDA);
  }
  std::memset(it->hctrl, 0, sizeof(Ctrl));
  it->hstate.resize((size_t)nv);

  FusedParams& P = it->params;
  std::memset(&P, 0, sizeof P);
  P.ctrl = it->ctrl;
  P.ring = it->ring;
  P.times_ring = it->times_ring;
  P.ks = it->ks;
  P.Y = it->Y;
  P.PX = it->PX;
  P.PY = it->PY;
  P.masses = it->masses;
  P.mass = sys->mass;
  P.eps2 = sys->softening * sys->softening;
  P.eps2f = (float)P.eps2;
  P.R = it->R;
  P.cref = it->cref;
  P.partials = it->partials;
  P.sq = it->sq;
  P.aux = it->aux;
  P.log = it->log;
  P.log_capacity = it->log_capacity;
  P.mlp = it->mlp_dev;
  P.n = n;
  P.n_var = nv;
  P.n_itiles = it->geom.n_itiles;
  P.n_parts = (long long)n_parts;
  P.pre = it->pre;
  P.BX = it->BX;
  P.BY = it->BY;
  P.cull = opts.spatial_sort == 2 ? 0 : 1;
  P.n_chunks = it->split ? it->geom.P : 1;
  for (int c = 0; c <= kMaxChunks; ++c)
    P.chunk_start[c] = c < (int)it->chunks.size() ? it->chunks[c] : n;
  P.chunk_sums = it->chunk_sums;
  P.tile_count = it->tile_count;
  P.exact = opts.exact;
  P.f64_fast = (opts.precision == GB_PREC_F64 && !opts.exact && opts.tiling.f64_pair != 2) ? 1 : 0;
  P.S = it->S;
  P.perm = it->perm;
  P.PXF = it->PXF;
  P.PYF = it->PYF;
  P.MX = it->MX;
  P.MY = it->MY;
  *out = it;
  return GB_OK;
}

extern "C" int gb_integrator_start(gb_integrator it, const double* x0, double t0, double tf,
                                   const double* atol_dev, const double* rtol_dev,
                                   double atol_s, double rtol_s, gb_save_fn save, void* user) {
  if (!it || !x0) return GB_ERR_INVALID_ARGUMENT;
  if (!std::isfinite(t0) || !std::isfinite(tf)) return GB_ERR_INVALID_ARGUMENT;
  if ((!atol_dev && !(atol_s >= 0.0)) || (!rtol_dev && !(rtol_s >= 0.0)))
    return GB_ERR_INVALID_ARGUMENT;
  const long long n = it->n, nv = it->n_var;
  cudaStream_t s = it->stream;
  // order after the caller's prior work on its stream
  GB_CUDA_TRY(cudaEventRecord(it->ev, it->user_stream));
  GB_CUDA_TRY(cudaStreamWaitEvent(s, it->ev, 0));
  FusedParams& P = it->params;
  if (atol_dev) {
    if (!it->atol) GB_CUDA_TRY(cudaMalloc((void**)&it->atol, nv * sizeof(double)));
    GB_CUDA_TRY(cudaMemcpyAsync(it->atol, atol_dev, nv * sizeof(double),
                                cudaMemcpyDeviceToDevice, s));
  }
  if (rtol_dev) {
    if (!it->rtol) GB_CUDA_TRY(cudaMalloc((void**)&it->rtol, nv * sizeof(double)));
    GB_CUDA_TRY(cudaMemcpyAsync(it->rtol, rtol_dev, nv * sizeof(double),
                                cudaMemcpyDeviceToDevice, s));
  }
  P.atol = atol_dev ? it->atol : nullptr;
  P.rtol = rtol_dev ? it->rtol : nullptr;
  P.atol_s = atol_s;
  P.rtol_s = rtol_s;
  // x0 -> ring slot 0
  GB_CUDA_TRY(cudaMemcpyAsync(it->ring, x0, nv * sizeof(double), cudaMemcpyDeviceToDevice, s));
  const int prec = it->opts.precision;
  if (prec == GB_PREC_MIXED) {
    centroid_state_kernel<<<1, 256, 0, s>>>(it->ring, n, it->cref);
    GB_CUDA_TRY(cudaGetLastError());
    pack_state_kernel<<<blocks256(n), 256, 0, s>>>(it->ring, it->masses, it->cref, n, it->PX);
    GB_CUDA_TRY(cudaGetLastError());
  }
  // estimate_initial_step: target -> Y[0], f0 -> ks slot 0, x1 -> Y[1],
  // df -> ks slot 1.
  double* tg = it->Y;
  double* x1 = it->Y + nv;
  double* f0 = it->ks;
  double* df = it->ks + nv;
  target0_kernel<<<blocks256(nv), 256, 0, s>>>(it->ring, P.atol, P.rtol, atol_s, rtol_s, tg, nv);
  GB_CUDA_TRY(cudaGetLastError());
  const gb_nbody_system& sys = it->sys;
  GB_TRY(rhs_for_start(prec, it->ring, f0, n, sys.softening, sys.mass, it->masses, it->PX,
                       it->opts.exact, &it->start_tiling, s));
  double* d = it->dscal;
  if (it->opts.exact) {
    serial_norm_kernel<<<1, 32, 0, s>>>(it->ring, tg, nv, d + 0);
    serial_norm_kernel<<<1, 32, 0, s>>>(f0, tg, nv, d + 1);
  } else {
    GB_TRY(launch_norm(it->ring, tg, nv, it->norm_work, d + 0, 1, s));
    GB_TRY(launch_norm(f0, tg, nv, it->norm_work, d + 1, 1, s));
  }
  GB_CUDA_TRY(cudaGetLastError());
  euler_kernel<<<blocks256(nv), 256, 0, s>>>(it->ring, f0, d, x1, nv);
  GB_CUDA_TRY(cudaGetLastError());
  if (prec == GB_PREC_MIXED) {
    pack_state_kernel<<<blocks256(n), 256, 0, s>>>(x1, it->masses, it->cref, n, it->PY);
    GB_CUDA_TRY(cudaGetLastError());
  }
  GB_TRY(rhs_for_start(prec, x1, df, n, sys.softening, sys.mass, it->masses, it->PY,
                       it->opts.exact, &it->start_tiling, s));
  diff_kernel<<<blocks256(nv), 256, 0, s>>>(df, f0, nv);
  GB_CUDA_TRY(cudaGetLastError());
  if (it->opts.exact) {
    serial_norm_kernel<<<1, 32, 0, s>>>(df, tg, nv, d + 2);
  } else {
    GB_TRY(launch_norm(df, tg, nv, it->norm_work, d + 2, 1, s));
  }
  GB_CUDA_TRY(cudaGetLastError());
  const int q = it->htab.p < it->htab.pt ? it->htab.p : it->htab.pt;
  const double safety = std::pow(0.38, (1.0 / (1.0 + q)));
  // the learned proposer's tolerance feature: scalar tolerances only
  const double tol_scale = std::max(atol_s, rtol_s);
  const double log_tol =
      (atol_dev || rtol_dev || !(tol_scale > 0.0)) ? 0.0 : std::log(tol_scale);
  init_ctrl_kernel<<<1, 32, 0, s>>>(it->ctrl, d, t0, tf, it->times_ring, it->htab.p, q, safety,
                                    it->opts.controller, it->opts.pi_beta, it->tab.fsal,
                                    it->opts.max_attempts, it->opts.exact, log_tol, n);
  GB_CUDA_TRY(cudaGetLastError());
  max_acc_kernel<<<1, 256, 0, s>>>(f0, n, it->ctrl);
  GB_CUDA_TRY(cudaGetLastError());
  GB_TRY(launch_resort(it));
  if (!it->exec) GB_TRY(build_graph(it));
  GB_TRY(read_ctrl(it));
  it->delivered = 0;
  it->started = true;
  if (save && it->opts.record) {
    GB_CUDA_TRY(cudaMemcpyAsync(it->hstate.data(), it->ring, nv * sizeof(double),
                                cudaMemcpyDeviceToHost, s));
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    save(user, t0, it->hstate.data(), nv);
  }
  return GB_OK;
}

extern "C" int gb_integrator_enqueue(gb_integrator it, int64_t n_replays) {
  if (!it || !it->started || n_replays < 0) return GB_ERR_INVALID_ARGUMENT;
  for (int64_t r = 0; r < n_replays; ++r) GB_CUDA_TRY(cudaGraphLaunch(it->exec, it->stream));
  return GB_OK;
}

extern "C" int gb_integrator_sync(gb_integrator it) {
  if (!it) return GB_ERR_INVALID_ARGUMENT;
  GB_TRY(read_ctrl(it));
  GB_CUDA_TRY(cudaEventRecord(it->ev, it->stream));
  GB_CUDA_TRY(cudaStreamWaitEvent(it->user_stream, it->ev, 0));
  return GB_OK;
}

extern "C" int gb_integrator_advance(gb_integrator it, int64_t max_attempts, gb_save_fn save,
                                     void* user) {
  if (!it || !it->started) return GB_ERR_INVALID_ARGUMENT;
  const long long start_attempts = it->hctrl->n_attempts;
  while (!it->hctrl->done) {
    if (max_attempts > 0 && it->hctrl->n_attempts - start_attempts >= max_attempts) break;
    GB_CUDA_TRY(cudaGraphLaunch(it->exec, it->stream));
    GB_TRY(read_ctrl(it));
    GB_TRY(drain(it, save, user));
  }
  GB_TRY(drain(it, save, user));
  GB_CUDA_TRY(cudaEventRecord(it->ev, it->stream));
  GB_CUDA_TRY(cudaStreamWaitEvent(it->user_stream, it->ev, 0));
  return it->hctrl->status;
}

// Output at the given times (ascending, within (t0, tf]) by the DOPRI5 dense
// formula after every accepted step.  Call after create and before start;
// the graph is rebuilt.
extern "C" int gb_integrator_set_dense_output(gb_integrator it, const double* times_host,
                                              int64_t n_times) {
  if (!it || n_times < 0 || (n_times > 0 && !times_host)) return GB_ERR_INVALID_ARGUMENT;
  gb_tableau dp;
  gb_tableau_builtin(GB_DOPRI5, &dp);
  if (std::memcmp(&dp, &it->htab, sizeof dp) != 0) return GB_ERR_UNSUPPORTED;
  for (int64_t j = 1; j < n_times; ++j)
    if (!(times_host[j] >= times_host[j - 1])) return GB_ERR_INVALID_ARGUMENT;
  if (it->dense_t) cudaFree(it->dense_t);
  if (it->dense_out) cudaFree(it->dense_out);
  it->dense_t = nullptr;
  it->dense_out = nullptr;
  it->n_dense = n_times;
  if (n_times > 0) {
    GB_CUDA_TRY(cudaMalloc((void**)&it->dense_t, n_times * sizeof(double)));
    GB_CUDA_TRY(cudaMalloc((void**)&it->dense_out, (size_t)n_times * it->n_var * sizeof(double)));
    GB_CUDA_TRY(cudaMemcpy(it->dense_t, times_host, n_times * sizeof(double),
                           cudaMemcpyHostToDevice));
  }
  it->params.dense_t = it->dense_t;
  it->params.dense_out = it->dense_out;
  it->params.n_dense = n_times;
  if (it->exec) {
    cudaGraphExecDestroy(it->exec);
    cudaGraphDestroy(it->graph);
    it->exec = nullptr;
    it->graph = nullptr;
  }
  return GB_OK;
}

// Copies the dense outputs computed so far (count = outputs whose time has
// been passed) to x_host [count][n_var].
extern "C" int gb_integrator_dense_output(gb_integrator it, double* x_host, int64_t capacity,
                                          int64_t* count) {
  if (!it || !count) return GB_ERR_INVALID_ARGUMENT;
  GB_TRY(read_ctrl(it));
  const long long c = std::min<long long>(it->hctrl->dense_next, it->n_dense);
  *count = c;
  if (x_host && capacity > 0 && c > 0) {
    const long long m = std::min<long long>(c, capacity);
    GB_CUDA_TRY(cudaMemcpy(x_host, it->dense_out, (size_t)m * it->n_var * sizeof(double),
                           cudaMemcpyDeviceToHost));
  }
  return GB_OK;
}

extern "C" int gb_integrator_launch_stage(gb_integrator it, int32_t stage) {
  if (!it || !it->started || stage < 0 || stage >= it->S) return GB_ERR_INVALID_ARGUMENT;
  void* args[] = {(void*)&it->tab, (void*)&it->params, (void*)&stage};
  return launch_stage_kernel(it, args);
}

extern "C" int gb_integrator_geometry(gb_integrator it, gb_force_tiling* out, int64_t* n_ctas) {
  if (!it || !out) return GB_ERR_INVALID_ARGUMENT;
  out->j_split = it->geom.P;
  out->lanes = it->geom.L;
  out->bodies_per_cta = it->geom.bodies_per_cta();
  out->mixed_variant = it->geom.variant;
  if (n_ctas) *n_ctas = it->geom.n_itiles * it->geom.P;
  return GB_OK;
}

extern "C" int gb_integrator_stats(gb_integrator it, gb_integrate_stats* o) {
  if (!it || !o) return GB_ERR_INVALID_ARGUMENT;
  const Ctrl& c = *it->hctrl;
  std::memset(o, 0, sizeof *o);
  o->n_accepted = c.n_accepted;
  o->n_rejected = c.n_rejected;
  o->n_attempts = c.n_attempts;
  o->n_rhs = c.n_rhs;
  o->n_rhs_saved = c.n_rhs_saved;
  o->t = c.t;
  o->dt = c.dt;
  o->dt_initial = c.dt_initial;
  o->err_last = c.err;
  o->interactions = (double)c.n_rhs * (double)it->n * (double)(it->n - 1);
  o->status = c.status;
  o->done = c.done;
  o->n_learned_proposals = c.n_learned;
  o->n_learned_rejected = c.n_learned_rejected;
  return GB_OK;
}

extern "C" int gb_integrator_state(gb_integrator it, double* x_dev, double* t_host) {
  if (!it || !it->started) return GB_ERR_INVALID_ARGUMENT;
  GB_TRY(read_ctrl(it));
  if (x_dev) {
    GB_CUDA_TRY(cudaMemcpyAsync(x_dev, it->ring + (long long)it->hctrl->cur * it->n_var,
                                it->n_var * sizeof(double), cudaMemcpyDeviceToDevice, it->stream));
    GB_CUDA_TRY(cudaStreamSynchronize(it->stream));
  }
  if (t_host) *t_host = it->hctrl->t;
  return GB_OK;
}

extern "C" int gb_integrator_destroy(gb_integrator it) {
  if (!it) return GB_OK;
  cudaStreamSynchronize(it->stream);
  free_all(it);
  delete it;
  return GB_OK;
}

// Step log access for the learned controller's training set.
extern "C" int gb_integrator_log(gb_integrator it, gb_step_log* host_records, int64_t capacity,
                                 int64_t* count) {
  if (!it || !count) return GB_ERR_INVALID_ARGUMENT;
  GB_TRY(read_ctrl(it));
  long long c = it->hctrl->log_count;
  if (c > it->log_capacity) c = it->log_capacity;
  *count = c;
  if (host_records && capacity > 0) {
    long long m = c < capacity ? c : capacity;
    if (m > 0) {
      GB_CUDA_TRY(cudaMemcpyAsync(host_records, it->log, (size_t)m * sizeof(StepLog),
                                  cudaMemcpyDeviceToHost, it->stream));
      GB_CUDA_TRY(cudaStreamSynchronize(it->stream));
    }
  }
  return GB_OK;
}

extern "C" int gb_integrate_nbody(const gb_tableau* tab, const gb_nbody_system* sys,
                                  const gb_integrate_opts* opts, const double* x0, double t0,
                                  double tf, const double* atol_dev, const double* rtol_dev,
                                  double atol_s, double rtol_s, gb_save_fn save, void* user,
                                  double* x_final, gb_integrate_stats* stats, gb_stream_t stream) {
  gb_integrator it = nullptr;
  GB_TRY(gb_integrator_create(tab, sys, opts, stream, &it));
  int rc = gb_integrator_start(it, x0, t0, tf, atol_dev, rtol_dev, atol_s, rtol_s, save, user);
  if (rc == GB_OK) rc = gb_integrator_advance(it, 0, save, user);
  if (rc == GB_OK || rc == GB_ERR_BUDGET || rc == GB_ERR_NOT_FINITE) {
    if (stats) gb_integrator_stats(it, stats);
    if (x_final) {
      int rc2 = gb_integrator_state(it, x_final, nullptr);
      if (rc == GB_OK) rc = rc2;
    }
  }
  gb_integrator_destroy(it);
  return rc;
}
