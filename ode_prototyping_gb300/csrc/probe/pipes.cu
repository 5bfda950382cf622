// pipes.cu -- throughput probe for the force kernel's roofline (a standalone
// program, not part of libgbode; bench.py --workload pipes builds and runs it).
//
// Measures on the GPU it runs on: the FP32 FMA pipe with scalar fma and with
// packed fma.rn.f32x2 (independent accumulators, no memory traffic), the SFU
// reciprocal square root (rsqrt.approx.ftz.f32), and the mixed-precision pair
// loop alone -- the body of the force kernel's path without the close-pair
// test (records in shared memory, no barriers, no tails or epilogue) -- so the
// stage kernel's fraction of the nominal FP32 peak can be read against the
// ceiling of its own instruction mix.  Prints one JSON object.
#include <cstdio>
#include <cuda_runtime.h>

namespace {

typedef unsigned long long f2_t;
__device__ __forceinline__ f2_t pk(float a, float b) {
  f2_t r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ void upk(f2_t r, float& a, float& b) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(r));
}
__device__ __forceinline__ f2_t sub2(f2_t a, f2_t b) {
  f2_t r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ f2_t mul2(f2_t a, f2_t b) {
  f2_t r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ f2_t fma2(f2_t a, f2_t b, f2_t c) {
  f2_t r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
  return r;
}
__device__ __forceinline__ float rsq(float x) {
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__global__ void ffma_kernel(float* out, int iters, float b, float c) {
  float a[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) a[i] = threadIdx.x * 0.001f + i;
  for (int k = 0; k < iters; ++k)
#pragma unroll
    for (int i = 0; i < 8; ++i) a[i] = fmaf(a[i], b, c);
  float s = 0.f;
#pragma unroll
  for (int i = 0; i < 8; ++i) s += a[i];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void ffma2_kernel(float* out, int iters, float b, float c) {
  f2_t a[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) a[i] = pk(threadIdx.x * 0.001f + i, i * 0.5f);
  const f2_t B = pk(b, b), Cc = pk(c, c);
  for (int k = 0; k < iters; ++k)
#pragma unroll
    for (int i = 0; i < 8; ++i) a[i] = fma2(a[i], B, Cc);
  float s = 0.f;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    float x, y;
    upk(a[i], x, y);
    s += x + y;
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void rsqrt_kernel(float* out, int iters) {
  float a[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) a[i] = 1.0f + threadIdx.x * 0.001f + i;
  for (int k = 0; k < iters; ++k)
#pragma unroll
    for (int i = 0; i < 8; ++i) a[i] = rsq(a[i]);
  float s = 0.f;
#pragma unroll
  for (int i = 0; i < 8; ++i) s += a[i];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

struct __align__(16) Rec {
  ulonglong2 xy, zl, yz;  // the force kernel's 48-byte partner-pair record
};

// The pair loop without the close-pair test: one body per thread, partners j
// and j + 1 per f32x2 instruction, unrolled 4, NR records in shared memory
// swept `reps` times.
template <int NR>
__global__ void __launch_bounds__(128) pair_loop_kernel(float* out, int reps, float eps2) {
  __shared__ Rec rec[NR];
  for (int r = threadIdx.x; r < NR; r += blockDim.x) {
    const float a = 0.37f * r, b = 0.11f * r;
    rec[r].xy = make_ulonglong2(pk(sinf(a), sinf(b)), pk(cosf(a), cosf(b)));
    rec[r].zl = make_ulonglong2(pk(sinf(2 * a), sinf(2 * b)), 0ULL);
    rec[r].yz = make_ulonglong2(0ULL, 0ULL);
  }
  __syncthreads();
  const float hx = 0.01f * threadIdx.x, hy = 0.02f * blockIdx.x, hz = 0.3f;
  const f2_t HX = pk(hx, hx), HY = pk(hy, hy), HZ = pk(hz, hz), E2 = pk(eps2, eps2);
  f2_t TX = 0ULL, TY = 0ULL, TZ = 0ULL;
  for (int rp = 0; rp < reps; ++rp) {
#pragma unroll 4
    for (int jj = 0; jj < NR; ++jj) {
      const ulonglong2 xy = rec[jj].xy;
      const f2_t z = rec[jj].zl.x;
      const f2_t dx = sub2(xy.x, HX), dy = sub2(xy.y, HY), dz = sub2(z, HZ);
      const f2_t r2 = fma2(dz, dz, fma2(dy, dy, fma2(dx, dx, E2)));
      float ra, rb;
      upk(r2, ra, rb);
      const f2_t ri = pk(rsq(ra), rsq(rb));
      const f2_t sc = mul2(ri, mul2(ri, ri));
      TX = fma2(sc, dx, TX);
      TY = fma2(sc, dy, TY);
      TZ = fma2(sc, dz, TZ);
    }
  }
  float a, b, c, d, e, f;
  upk(TX, a, b);
  upk(TY, c, d);
  upk(TZ, e, f);
  out[blockIdx.x * blockDim.x + threadIdx.x] = a + b + c + d + e + f;
}

template <class F>
float time_ms(F f) {
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  f();  // warm-up
  cudaDeviceSynchronize();
  cudaEventRecord(e0);
  for (int r = 0; r < 5; ++r) f();
  cudaEventRecord(e1);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return ms / 5;
}

}  // namespace

int main() {
  int sms = 0, clk_khz = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
  cudaDeviceGetAttribute(&clk_khz, cudaDevAttrClockRate, 0);
  const double hz = clk_khz * 1e3;
  const double peak = sms * 128.0 * 2.0 * hz;  // nominal FP32 FLOP/s
  const int tpb = 256, cps = 8, grid = sms * cps, iters = 20000;
  float* out = nullptr;
  if (cudaMalloc(&out, sizeof(float) * grid * tpb) != cudaSuccess) return 1;
  const double fl1 = 2.0 * 8 * iters * (double)grid * tpb;
  const float t1 = time_ms([&] { ffma_kernel<<<grid, tpb>>>(out, iters, 0.999f, 0.001f); });
  const double fl2 = 4.0 * 8 * iters * (double)grid * tpb;
  const float t2 = time_ms([&] { ffma2_kernel<<<grid, tpb>>>(out, iters, 0.999f, 0.001f); });
  const double ops3 = 8.0 * (iters / 4) * (double)grid * tpb;
  const float t3 = time_ms([&] { rsqrt_kernel<<<grid, tpb>>>(out, iters / 4); });
  const int lgrid = sms * 6, reps = 200;  // six 128-thread CTAs per SM, as the stage kernel
  const double inter = 2.0 * 512 * reps * (double)lgrid * 128;
  const float t4 = time_ms([&] { pair_loop_kernel<512><<<lgrid, 128>>>(out, reps, 2.5e-5f); });
  const cudaError_t e = cudaDeviceSynchronize();
  cudaFree(out);
  printf("{\"sms\": %d, \"clock_mhz\": %.0f, \"fp32_nominal_tflops\": %.2f, "
         "\"ffma_tflops\": %.2f, \"ffma_frac\": %.4f, \"ffma2_tflops\": %.2f, \"ffma2_frac\": %.4f, "
         "\"rsqrt_per_sm_per_clock\": %.2f, \"pair_loop_interactions_per_s\": %.4e, "
         "\"pair_loop_frac_20flop\": %.4f, \"status\": \"%s\"}\n",
         sms, hz / 1e6, peak / 1e12, fl1 / (t1 / 1e3) / 1e12, fl1 / (t1 / 1e3) / peak,
         fl2 / (t2 / 1e3) / 1e12, fl2 / (t2 / 1e3) / peak, ops3 / (t3 / 1e3) / sms / hz,
         inter / (t4 / 1e3), 20.0 * inter / (t4 / 1e3) / peak, cudaGetErrorString(e));
  return e == cudaSuccess ? 0 : 1;
}
