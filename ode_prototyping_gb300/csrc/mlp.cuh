// mlp.cuh -- the learned step-size proposer: a 16 -> 64 -> 64 -> 1 MLP with
// SiLU activations.  The controller runs it with BF16 weights and FP32
// accumulation; training (mlp.cu) keeps FP32 master weights.
#pragma once

#include <cuda_bf16.h>

#include "integrator.cuh"

namespace gb {

constexpr int kIn = GB_MLP_IN;
constexpr int kHid = GB_MLP_HIDDEN;

// Inference copy resident on the device.
struct MlpDev {
  __nv_bfloat16 w1[kHid * kIn];
  __nv_bfloat16 w2[kHid * kHid];
  __nv_bfloat16 w3[kHid];
  float b1[kHid];
  float b2[kHid];
  float b3;
  float in_mean[kIn];
  float in_scale[kIn];
  float out_scale;
  float out_bias;
};

__device__ __forceinline__ float silu(float x) { return x / (1.0f + __expf(-x)); }

// Feature vector of the controller state after an attempt (16 entries):
//  0-2  log of the last three attempted steps
//  3-5  log of the last three scaled error norms
//  6    log max |a| over bodies (first stage of the last attempt)
//  7    log of a closest-approach proxy sqrt(m / max|a|)
//  8    log N
//  9    order q = min(p, pt) of the tableau
//  10   log of the step relative to the integration interval
//  11   1 if the last attempt was accepted
//  12   log(dt_{n} / dt_{n-1})
//  13   log of the PI memory (the last accepted error)
//  14   log max(atol, rtol) (scalar tolerances; 0 for vector ones).  Networks
//       trained at one tolerance saw a constant here and carry in_scale 0
//       for it, so they ignore it; a network trained over several
//       tolerances uses it.
//  15   zero
__device__ __forceinline__ void make_features(const Ctrl& c, const DevTableau& tab, long long n,
                                              float* f) {
  const double tiny = 1e-300;
  // the learned controller keeps these logs from attempt to attempt
  // (Ctrl::lg_*, the same values); a log of another controller computes them
  double ldt[3], lerr[3], lprev, ln;
  if (c.lg_valid) {
    for (int k = 0; k < 3; ++k) {
      ldt[k] = c.lg_dt[k];
      lerr[k] = c.lg_err[k];
    }
    lprev = c.lg_err_prev;
    ln = c.lg_n;
  } else {
    for (int k = 0; k < 3; ++k) {
      ldt[k] = log(fmax(c.dt_hist[k], tiny));
      lerr[k] = log(fmax(c.err_hist[k], 1e-30));
    }
    lprev = log(fmax(c.err_prev, 1e-30));
    ln = log((double)n);
  }
  for (int k = 0; k < 3; ++k) {
    f[k] = (float)ldt[k];
    f[3 + k] = (float)lerr[k];
  }
  const double amax = fmax(c.max_abs_acc, 1e-30);
  f[6] = (float)log(amax);
  const double m = 1.0 / (double)n;
  f[7] = (float)(0.5 * log(m / amax));
  f[8] = (float)ln;
  f[9] = (float)(tab.p < tab.pt ? tab.p : tab.pt);
  f[10] = (float)log(fmax(c.dt_hist[0] / fmax(c.tf - c.t0, tiny), tiny));
  f[11] = (float)c.last_accepted;
  f[12] = (float)(ldt[0] - ldt[1]);
  f[13] = (float)lprev;  // PI memory: last accepted error
  f[14] = (float)c.log_tol;  // log max(atol, rtol): one network for several tolerances
  f[15] = 0.f;
}

// Single-thread BF16-weight / FP32-accumulate forward pass.
__device__ __forceinline__ float mlp_infer(const void* mlp_v, const float* feat) {
  const MlpDev* M = reinterpret_cast<const MlpDev*>(mlp_v);
  float x[kIn];
#pragma unroll
  for (int k = 0; k < kIn; ++k) x[k] = (feat[k] - M->in_mean[k]) * M->in_scale[k];
  float h1[kHid];
  for (int o = 0; o < kHid; ++o) {
    float acc = M->b1[o];
#pragma unroll
    for (int k = 0; k < kIn; ++k) acc = fmaf(__bfloat162float(M->w1[o * kIn + k]), x[k], acc);
    h1[o] = silu(acc);
  }
  float out = M->b3;
  for (int o = 0; o < kHid; ++o) {
    float acc = M->b2[o];
    for (int k = 0; k < kHid; ++k) acc = fmaf(__bfloat162float(M->w2[o * kHid + k]), h1[k], acc);
    out = fmaf(__bfloat162float(M->w3[o]), silu(acc), out);
  }
  return M->out_scale * out + M->out_bias;
}

// CTA-cooperative forward pass (same arithmetic as mlp_infer): thread o < 64
// owns hidden unit o.  All threads of the block must call it; `feat` and
// `h1` are shared arrays, the result lands in *out (shared).
__device__ __forceinline__ void mlp_infer_block(const void* mlp_v, const float* feat, float* h1,
                                                float* out) {
  const MlpDev* M = reinterpret_cast<const MlpDev*>(mlp_v);
  const int o = threadIdx.x;
  if (o < kHid) {
    float acc = M->b1[o];
#pragma unroll
    for (int k = 0; k < kIn; ++k)
      acc = fmaf(__bfloat162float(M->w1[o * kIn + k]), (feat[k] - M->in_mean[k]) * M->in_scale[k],
                 acc);
    h1[o] = silu(acc);
  }
  __syncthreads();
  float contrib = 0.f;
  if (o < kHid) {
    float acc = M->b2[o];
    // unrolled so that the row's weight loads are in flight together (the
    // sum keeps its order)
#pragma unroll
    for (int k = 0; k < kHid; ++k) acc = fmaf(__bfloat162float(M->w2[o * kHid + k]), h1[k], acc);
    contrib = __bfloat162float(M->w3[o]) * silu(acc);
  }
  // fixed-order sum of the 64 contributions over two warps
  if (o < kHid) {
#pragma unroll
    for (int off = 16; off >= 1; off /= 2) contrib += __shfl_down_sync(0xffffffffu, contrib, off);
  }
  __syncthreads();
  if (o == 0) h1[0] = contrib;
  if (o == 32) h1[1] = contrib;
  __syncthreads();
  if (o == 0) *out = M->out_scale * (M->b3 + h1[0] + h1[1]) + M->out_bias;
  __syncthreads();
}

// Warp-cooperative forward pass (one warp, lane u owns hidden units u and
// u + 32); the hidden activations move between lanes by shuffles.  All 32
// lanes must call it; returns the network output on every lane.
__device__ __forceinline__ float mlp_infer_warp(const void* mlp_v, const float* feat) {
  const MlpDev* M = reinterpret_cast<const MlpDev*>(mlp_v);
  const int lane = threadIdx.x & 31;
  float x[kIn];
#pragma unroll
  for (int k = 0; k < kIn; ++k) x[k] = (feat[k] - M->in_mean[k]) * M->in_scale[k];
  float h1[2];
#pragma unroll
  for (int r = 0; r < 2; ++r) {
    const int u = lane + 32 * r;
    float acc = M->b1[u];
#pragma unroll
    for (int k = 0; k < kIn; ++k) acc = fmaf(__bfloat162float(M->w1[u * kIn + k]), x[k], acc);
    h1[r] = silu(acc);
  }
  float contrib = 0.f;
#pragma unroll
  for (int r = 0; r < 2; ++r) {
    const int u = lane + 32 * r;
    float acc = M->b2[u];
#pragma unroll
    for (int k = 0; k < kHid; ++k) {
      const float hk = __shfl_sync(0xffffffffu, k < 32 ? h1[0] : h1[1], k & 31);
      acc = fmaf(__bfloat162float(M->w2[u * kHid + k]), hk, acc);
    }
    contrib = fmaf(__bfloat162float(M->w3[u]), silu(acc), contrib);
  }
#pragma unroll
  for (int off = 16; off >= 1; off /= 2) contrib += __shfl_xor_sync(0xffffffffu, contrib, off);
  return M->out_scale * (M->b3 + contrib) + M->out_bias;
}

// Allocates the device inference copy of a host gb_mlp (rounded to BF16).
void* mlp_upload(const void* host_mlp, int* rc);

}  // namespace gb
