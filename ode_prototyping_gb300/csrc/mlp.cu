// mlp.cu -- training and inference kernels of the learned step-size proposer
// (16 -> 64 -> 64 -> 1, SiLU).  No counterpart in the reference.
//
// Training keeps FP32 master weights in a gb_mlp struct in device memory:
//   forward  : one thread per sample, weights staged in shared memory, the
//              pre-activations z1, z2 saved for the backward pass;
//   backward : per-sample deltas (dz1, dz2, h1, h2) in one pass, then one
//              thread per parameter sums its gradient over the batch in
//              sample order (deterministic, no atomics);
//   adam     : one thread per parameter.
// Inference in the controller uses BF16-rounded weights with FP32
// accumulation (mlp.cuh); gb_mlp_infer_bf16 exposes the same arithmetic.
#include <cstring>
#include <vector>

#include "mlp.cuh"

namespace gb {

namespace {

constexpr int kParamsW1 = kHid * kIn;
constexpr int kParamsW2 = kHid * kHid;
// trainable parameters in gb_mlp order: w1, b1, w2, b2, w3, b3
constexpr int kTrainable = kParamsW1 + kHid + kParamsW2 + kHid + kHid + 1;
constexpr int kActPerSample = 2 * kHid;         // z1, z2
constexpr int kDeltaPerSample = 4 * kHid;       // h1, dz1, h2, dz2

static_assert(offsetof(gb_mlp, b1) == sizeof(float) * kParamsW1, "layout");
static_assert(offsetof(gb_mlp, w2) == sizeof(float) * (kParamsW1 + kHid), "layout");

__device__ __forceinline__ float dsilu(float z) {
  const float s = 1.0f / (1.0f + __expf(-z));
  return s * (1.0f + z * (1.0f - s));
}

__device__ __forceinline__ float* param_ptr(gb_mlp* m, int p) {
  return reinterpret_cast<float*>(m) + p;  // w1..b3 are contiguous floats
}

__global__ void forward_kernel(const gb_mlp* __restrict__ W, const float* __restrict__ x,
                               float* __restrict__ y, long long B, float* __restrict__ act,
                               int bf16) {
  __shared__ float w1[kHid * kIn];
  __shared__ float w2[kHid * kHid];
  __shared__ float w3[kHid], b1[kHid], b2[kHid];
  __shared__ float mean[kIn], scl[kIn];
  for (int k = threadIdx.x; k < kHid * kIn; k += blockDim.x) {
    float v = (&W->w1[0][0])[k];
    w1[k] = bf16 ? __bfloat162float(__float2bfloat16_rn(v)) : v;
  }
  for (int k = threadIdx.x; k < kHid * kHid; k += blockDim.x) {
    float v = (&W->w2[0][0])[k];
    w2[k] = bf16 ? __bfloat162float(__float2bfloat16_rn(v)) : v;
  }
  for (int k = threadIdx.x; k < kHid; k += blockDim.x) {
    float v = W->w3[k];
    w3[k] = bf16 ? __bfloat162float(__float2bfloat16_rn(v)) : v;
    b1[k] = W->b1[k];
    b2[k] = W->b2[k];
  }
  for (int k = threadIdx.x; k < kIn; k += blockDim.x) {
    mean[k] = W->in_mean[k];
    scl[k] = W->in_scale[k];
  }
  __syncthreads();
  const long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (s >= B) return;
  float xin[kIn];
#pragma unroll
  for (int k = 0; k < kIn; ++k) xin[k] = (x[s * kIn + k] - mean[k]) * scl[k];
  float h1[kHid];
  for (int o = 0; o < kHid; ++o) {
    float acc = b1[o];
#pragma unroll
    for (int k = 0; k < kIn; ++k) acc = fmaf(w1[o * kIn + k], xin[k], acc);
    if (act) act[s * kActPerSample + o] = acc;
    h1[o] = silu(acc);
  }
  float out = W->b3;
  for (int o = 0; o < kHid; ++o) {
    float acc = b2[o];
    for (int k = 0; k < kHid; ++k) acc = fmaf(w2[o * kHid + k], h1[k], acc);
    if (act) act[s * kActPerSample + kHid + o] = acc;
    out = fmaf(w3[o], silu(acc), out);
  }
  y[s] = W->out_scale * out + W->out_bias;
}

// Per-sample deltas: h1, dz1, h2, dz2.
__global__ void delta_kernel(const gb_mlp* __restrict__ W, const float* __restrict__ act,
                             const float* __restrict__ dy, long long B,
                             float* __restrict__ delta) {
  __shared__ float w2[kHid * kHid];
  __shared__ float w3[kHid];
  for (int k = threadIdx.x; k < kHid * kHid; k += blockDim.x) w2[k] = (&W->w2[0][0])[k];
  for (int k = threadIdx.x; k < kHid; k += blockDim.x) w3[k] = W->w3[k];
  __syncthreads();
  const long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (s >= B) return;
  const float g = dy[s] * W->out_scale;
  const float* z1 = act + s * kActPerSample;
  const float* z2 = z1 + kHid;
  float* d = delta + s * kDeltaPerSample;
  float dz2[kHid];
  for (int o = 0; o < kHid; ++o) {
    dz2[o] = g * w3[o] * dsilu(z2[o]);
    d[2 * kHid + o] = silu(z2[o]);
    d[3 * kHid + o] = dz2[o];
  }
  for (int k = 0; k < kHid; ++k) {
    float acc = 0.f;
    for (int o = 0; o < kHid; ++o) acc = fmaf(w2[o * kHid + k], dz2[o], acc);
    d[k] = silu(z1[k]);
    d[kHid + k] = acc * dsilu(z1[k]);
  }
}

// One thread per trainable parameter; sums over samples in order.
__global__ void grad_kernel(const gb_mlp* __restrict__ W, const float* __restrict__ x,
                            const float* __restrict__ delta, const float* __restrict__ dy,
                            long long B, gb_mlp* __restrict__ G) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= kTrainable) return;
  double acc = 0.0;  // FP64 accumulation keeps the batch sum order-stable
  if (p < kParamsW1) {
    const int o = p / kIn, k = p % kIn;
    const float mean = W->in_mean[k], scl = W->in_scale[k];
    for (long long s = 0; s < B; ++s)
      acc += (double)delta[s * kDeltaPerSample + kHid + o] * ((x[s * kIn + k] - mean) * scl);
  } else if (p < kParamsW1 + kHid) {
    const int o = p - kParamsW1;
    for (long long s = 0; s < B; ++s) acc += delta[s * kDeltaPerSample + kHid + o];
  } else if (p < kParamsW1 + kHid + kParamsW2) {
    const int q = p - kParamsW1 - kHid;
    const int o = q / kHid, k = q % kHid;
    for (long long s = 0; s < B; ++s)
      acc += (double)delta[s * kDeltaPerSample + 3 * kHid + o] * delta[s * kDeltaPerSample + k];
  } else if (p < kParamsW1 + 2 * kHid + kParamsW2) {
    const int o = p - kParamsW1 - kHid - kParamsW2;
    for (long long s = 0; s < B; ++s) acc += delta[s * kDeltaPerSample + 3 * kHid + o];
  } else if (p < kTrainable - 1) {
    const int o = p - kParamsW1 - 2 * kHid - kParamsW2;
    const float os = W->out_scale;
    for (long long s = 0; s < B; ++s)
      acc += (double)(dy[s] * os) * delta[s * kDeltaPerSample + 2 * kHid + o];
  } else {
    const float os = W->out_scale;
    for (long long s = 0; s < B; ++s) acc += (double)(dy[s] * os);
  }
  *param_ptr(G, p) = (float)acc;
}

__global__ void zero_nontrainable_kernel(gb_mlp* G) {
  const int k = threadIdx.x;
  if (k < kIn) {
    G->in_mean[k] = 0.f;
    G->in_scale[k] = 0.f;
  }
  if (k == 0) {
    G->out_scale = 0.f;
    G->out_bias = 0.f;
  }
}

__global__ void adam_kernel(gb_mlp* W, const gb_mlp* G, gb_mlp* M, gb_mlp* V, float lr,
                            float b1, float b2, float eps, float c1, float c2) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= kTrainable) return;
  const float g = *param_ptr(const_cast<gb_mlp*>(G), p);
  float& m = *param_ptr(M, p);
  float& v = *param_ptr(V, p);
  m = b1 * m + (1.f - b1) * g;
  v = b2 * v + (1.f - b2) * g * g;
  const float mh = m / c1, vh = v / c2;
  *param_ptr(W, p) -= lr * mh / (sqrtf(vh) + eps);
}

// Asymmetric squared error: w (y - t)^2 with w = over_weight when y > t.
__global__ void loss_kernel(const float* __restrict__ y, const float* __restrict__ t, long long B,
                            float over_w, float* __restrict__ dy, float* __restrict__ lsample) {
  const long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (s >= B) return;
  const float r = y[s] - t[s];
  const float w = r > 0.f ? over_w : 1.f;
  dy[s] = 2.f * w * r / (float)B;
  lsample[s] = w * r * r;
}

__global__ void mean_kernel(const float* __restrict__ v, long long B, float* out) {
  __shared__ double sh[256];
  double acc = 0.0;
  for (long long s = threadIdx.x; s < B; s += 256) acc += v[s];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int st = 128; st > 0; st /= 2) {
    if ((int)threadIdx.x < st) sh[threadIdx.x] += sh[threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = (float)(sh[0] / (double)B);
}

unsigned nblk(long long n, int b) { return (unsigned)((n + b - 1) / b); }

uint64_t splitmix64(uint64_t& s) {
  uint64_t z = (s += 0x9e3779b97f4a7c15ULL);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
  return z ^ (z >> 31);
}

}  // namespace

void* mlp_upload(const void* host_mlp, int* rc) {
  *rc = GB_OK;
  if (!host_mlp) {
    *rc = GB_ERR_INVALID_ARGUMENT;
    return nullptr;
  }
  const gb_mlp& m = *reinterpret_cast<const gb_mlp*>(host_mlp);
  MlpDev d;
  for (int o = 0; o < kHid; ++o) {
    for (int k = 0; k < kIn; ++k) d.w1[o * kIn + k] = __float2bfloat16_rn(m.w1[o][k]);
    for (int k = 0; k < kHid; ++k) d.w2[o * kHid + k] = __float2bfloat16_rn(m.w2[o][k]);
    d.w3[o] = __float2bfloat16_rn(m.w3[o]);
    d.b1[o] = m.b1[o];
    d.b2[o] = m.b2[o];
  }
  d.b3 = m.b3;
  for (int k = 0; k < kIn; ++k) {
    d.in_mean[k] = m.in_mean[k];
    d.in_scale[k] = m.in_scale[k];
  }
  d.out_scale = m.out_scale;
  d.out_bias = m.out_bias;
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, sizeof(MlpDev));
  if (e == cudaSuccess) e = cudaMemcpy(p, &d, sizeof(MlpDev), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    note_cuda_error(e);
    if (p) cudaFree(p);
    *rc = GB_ERR_CUDA;
    return nullptr;
  }
  return p;
}

}  // namespace gb

using namespace gb;

extern "C" int gb_mlp_init(gb_mlp* m, uint64_t seed) {
  if (!m) return GB_ERR_INVALID_ARGUMENT;
  std::memset(m, 0, sizeof *m);
  uint64_t s = seed;
  auto uni = [&s](float lim) {
    const double u = (double)(splitmix64(s) >> 11) * (1.0 / 9007199254740992.0);
    return (float)((2.0 * u - 1.0) * lim);
  };
  const float l1 = std::sqrt(6.0f / (kIn + kHid));
  const float l2 = std::sqrt(6.0f / (kHid + kHid));
  const float l3 = std::sqrt(6.0f / (kHid + 1));
  for (int o = 0; o < kHid; ++o)
    for (int k = 0; k < kIn; ++k) m->w1[o][k] = uni(l1);
  for (int o = 0; o < kHid; ++o)
    for (int k = 0; k < kHid; ++k) m->w2[o][k] = uni(l2);
  for (int o = 0; o < kHid; ++o) m->w3[o] = uni(l3);
  for (int k = 0; k < kIn; ++k) m->in_scale[k] = 1.f;
  m->out_scale = 1.f;
  return GB_OK;
}

extern "C" int64_t gb_mlp_act_floats(int64_t B) { return B < 0 ? 0 : B * kActPerSample; }

extern "C" int gb_mlp_forward_f32(const gb_mlp* W, const float* x, float* y, int64_t B,
                                  float* act, gb_stream_t stream) {
  if (!W || !x || !y || B < 1) return GB_ERR_INVALID_ARGUMENT;
  forward_kernel<<<nblk(B, 128), 128, 0, as_cuda(stream)>>>(W, x, y, B, act, 0);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

extern "C" int gb_mlp_infer_bf16(const gb_mlp* W, const float* x, float* y, int64_t B,
                                 gb_stream_t stream) {
  if (!W || !x || !y || B < 1) return GB_ERR_INVALID_ARGUMENT;
  forward_kernel<<<nblk(B, 128), 128, 0, as_cuda(stream)>>>(W, x, y, B, nullptr, 1);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

extern "C" size_t gb_mlp_backward_workspace_bytes(int64_t B) {
  return B < 1 ? 0 : (size_t)B * kDeltaPerSample * sizeof(float);
}

extern "C" int gb_mlp_backward_f32(const gb_mlp* W, const float* x, const float* act,
                                   const float* dy, gb_mlp* G, int64_t B, void* work,
                                   gb_stream_t stream) {
  if (!W || !x || !act || !dy || !G || !work || B < 1) return GB_ERR_INVALID_ARGUMENT;
  cudaStream_t s = as_cuda(stream);
  float* delta = reinterpret_cast<float*>(work);
  delta_kernel<<<nblk(B, 128), 128, 0, s>>>(W, act, dy, B, delta);
  GB_CUDA_TRY(cudaGetLastError());
  grad_kernel<<<nblk(kTrainable, 128), 128, 0, s>>>(W, x, delta, dy, B, G);
  GB_CUDA_TRY(cudaGetLastError());
  zero_nontrainable_kernel<<<1, 32, 0, s>>>(G);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

extern "C" int gb_mlp_adam_step(gb_mlp* W, const gb_mlp* G, gb_mlp* M, gb_mlp* V, float lr,
                                float b1, float b2, float eps, int32_t step, gb_stream_t stream) {
  if (!W || !G || !M || !V || step < 1) return GB_ERR_INVALID_ARGUMENT;
  const float c1 = 1.f - std::pow(b1, (float)step);
  const float c2 = 1.f - std::pow(b2, (float)step);
  adam_kernel<<<nblk(kTrainable, 256), 256, 0, as_cuda(stream)>>>(W, G, M, V, lr, b1, b2, eps,
                                                                   c1, c2);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

extern "C" int gb_mlp_train(gb_mlp* W, const float* x, const float* target, int64_t B,
                            int32_t epochs, float lr, float over_w, float* loss_host,
                            gb_stream_t stream) {
  if (!W || !x || !target || B < 1 || epochs < 0) return GB_ERR_INVALID_ARGUMENT;
  cudaStream_t s = as_cuda(stream);
  float *act = nullptr, *y = nullptr, *dy = nullptr, *ls = nullptr, *loss = nullptr;
  void* work = nullptr;
  gb_mlp *G = nullptr, *M = nullptr, *V = nullptr;
  int rc = GB_OK;
  cudaError_t e = cudaSuccess;
  auto alloc = [&](void** p, size_t b) {
    if (e == cudaSuccess) e = cudaMalloc(p, b);
  };
  alloc((void**)&act, (size_t)B * kActPerSample * sizeof(float));
  alloc((void**)&y, (size_t)B * sizeof(float));
  alloc((void**)&dy, (size_t)B * sizeof(float));
  alloc((void**)&ls, (size_t)B * sizeof(float));
  alloc((void**)&loss, sizeof(float));
  alloc(&work, gb_mlp_backward_workspace_bytes(B));
  alloc((void**)&G, sizeof(gb_mlp));
  alloc((void**)&M, sizeof(gb_mlp));
  alloc((void**)&V, sizeof(gb_mlp));
  if (e == cudaSuccess) e = cudaMemsetAsync(M, 0, sizeof(gb_mlp), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(V, 0, sizeof(gb_mlp), s);
  if (e != cudaSuccess) {
    note_cuda_error(e);
    rc = GB_ERR_CUDA;
  }
  for (int ep = 1; ep <= epochs && rc == GB_OK; ++ep) {
    rc = gb_mlp_forward_f32(W, x, y, B, act, stream);
    if (rc != GB_OK) break;
    loss_kernel<<<nblk(B, 256), 256, 0, s>>>(y, target, B, over_w, dy, ls);
    rc = gb_mlp_backward_f32(W, x, act, dy, G, B, work, stream);
    if (rc != GB_OK) break;
    rc = gb_mlp_adam_step(W, G, M, V, lr, 0.9f, 0.999f, 1e-8f, ep, stream);
  }
  if (rc == GB_OK) {
    rc = gb_mlp_forward_f32(W, x, y, B, act, stream);
    if (rc == GB_OK) {
      loss_kernel<<<nblk(B, 256), 256, 0, s>>>(y, target, B, over_w, dy, ls);
      mean_kernel<<<1, 256, 0, s>>>(ls, B, loss);
      float hl = 0.f;
      e = cudaMemcpyAsync(&hl, loss, sizeof(float), cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);
      if (e != cudaSuccess) {
        note_cuda_error(e);
        rc = GB_ERR_CUDA;
      } else if (loss_host) {
        *loss_host = hl;
      }
    }
  }
  cudaStreamSynchronize(s);
  void* bufs[] = {act, y, dy, ls, loss, work, G, M, V};
  for (void* p : bufs)
    if (p) cudaFree(p);
  return rc;
}
