// sortpack.cuh -- Morton ordering of the bodies and packing of the sorted
// tiles for the mixed-precision far-field path (host launch helper + kernels).
#pragma once

#include <cub/device/device_radix_sort.cuh>

#include "epilogue.cuh"

namespace gb {

struct SortBuffers {
  int* perm;                       // n: sorted position -> body
  int* vals;                       // n: body ids (sort input)
  unsigned long long* keys;        // n
  unsigned long long* keys_alt;    // n
  void* cub_temp;
  size_t cub_bytes;
  double* bbox;                    // 6
};

namespace {  // kernels get internal linkage in every translation unit

// Positions are read from base + (*slot) * stride (slot null: 0), so a
// graph-captured launch follows the integrator's current ring slot.
__device__ __forceinline__ const double* slot_ptr(const double* base, const int* slot,
                                                  long long stride) {
  return base + (slot ? (long long)*slot : 0LL) * stride;
}

__global__ void sort_bbox_kernel(const double* base, const int* slot, long long stride,
                                 long long n, double* bbox) {
  __shared__ double lo[3][256], hi[3][256];
  const double* x = slot_ptr(base, slot, stride);
  double l[3] = {1e300, 1e300, 1e300}, h[3] = {-1e300, -1e300, -1e300};
  for (long long i = threadIdx.x; i < n; i += blockDim.x)
    for (int d = 0; d < 3; ++d) {
      l[d] = fmin(l[d], x[3 * i + d]);
      h[d] = fmax(h[d], x[3 * i + d]);
    }
  for (int d = 0; d < 3; ++d) {
    lo[d][threadIdx.x] = l[d];
    hi[d][threadIdx.x] = h[d];
  }
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st /= 2) {
    if ((int)threadIdx.x < st)
      for (int d = 0; d < 3; ++d) {
        lo[d][threadIdx.x] = fmin(lo[d][threadIdx.x], lo[d][threadIdx.x + st]);
        hi[d][threadIdx.x] = fmax(hi[d][threadIdx.x], hi[d][threadIdx.x + st]);
      }
    __syncthreads();
  }
  if (threadIdx.x < 3) {
    bbox[threadIdx.x] = lo[threadIdx.x][0];
    bbox[3 + threadIdx.x] = hi[threadIdx.x][0];
  }
}

__device__ __forceinline__ unsigned long long spread3(unsigned long long v) {
  v &= 0x1fffffULL;
  v = (v | v << 32) & 0x1f00000000ffffULL;
  v = (v | v << 16) & 0x1f0000ff0000ffULL;
  v = (v | v << 8) & 0x100f00f00f00f00fULL;
  v = (v | v << 4) & 0x10c30c30c30c30c3ULL;
  v = (v | v << 2) & 0x1249249249249249ULL;
  return v;
}

// 63-bit Morton key of each body in the bounding box; value = body id.
__global__ void morton_kernel(const double* base, const int* slot, long long stride, long long n,
                              const double* bbox, unsigned long long* keys, int* vals) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double* x = slot_ptr(base, slot, stride);
  unsigned long long q[3];
  for (int d = 0; d < 3; ++d) {
    const double span = fmax(bbox[3 + d] - bbox[d], 1e-300);
    double u = (x[3 * i + d] - bbox[d]) / span;
    u = fmin(fmax(u, 0.0), 1.0);
    q[d] = (unsigned long long)(u * 2097151.0);
  }
  keys[i] = spread3(q[0]) | (spread3(q[1]) << 1) | (spread3(q[2]) << 2);
  vals[i] = (int)i;
}

// One CTA per sorted tile of T bodies: near / far records and metadata,
// written at (*out_slot) * n (records) and (*out_slot) * n_tiles (metadata).
template <int T>
__global__ void __launch_bounds__(T)
    pack_tiles_kernel(const double* base, const int* slot, long long stride, long long n,
                      const int* perm, const double* masses, const double* cref,
                      PackedBody* near, float4* far, TileMeta* meta, const int* out_slot,
                      long long n_tiles) {
  __shared__ double red[T];
  const double* x = slot_ptr(base, slot, stride);
  const long long o = out_slot ? (long long)*out_slot : 0LL;
  const long long i = blockIdx.x * (long long)T + threadIdx.x;
  const bool valid = i < n;
  double p[3] = {0.0, 0.0, 0.0};
  float w = 0.f;
  if (valid) {
    const long long id = perm[i];
    for (int d = 0; d < 3; ++d) p[d] = x[3 * id + d];
    w = masses ? (float)masses[id] : 1.0f;
  }
  const long long cnt = min((long long)T, n - blockIdx.x * (long long)T);
  pack_sorted_tile(p, valid, (int)cnt, w, cref, near + o * n + i, far + o * n + i,
                   meta + o * n_tiles + blockIdx.x, red);
}

}  // namespace

inline size_t sort_temp_bytes(long long n) {
  size_t bytes = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, bytes, (unsigned long long*)nullptr,
                                  (unsigned long long*)nullptr, (int*)nullptr, (int*)nullptr,
                                  (int)n, 0, 63);
  return bytes;
}

// Bounding box, Morton keys and the radix sort: perm = bodies in Morton order.
inline int sort_bodies(const double* base, const int* slot, long long stride, long long n,
                       const SortBuffers& sb, cudaStream_t s) {
  sort_bbox_kernel<<<1, 256, 0, s>>>(base, slot, stride, n, sb.bbox);
  morton_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(base, slot, stride, n, sb.bbox,
                                                             sb.keys, sb.vals);
  GB_CUDA_TRY(cudaGetLastError());
  size_t bytes = sb.cub_bytes;
  GB_CUDA_TRY(cub::DeviceRadixSort::SortPairs(sb.cub_temp, bytes, sb.keys, sb.keys_alt, sb.vals,
                                              sb.perm, (int)n, 0, 63, s));
  return GB_OK;
}

// Bounding box, Morton keys, radix sort (perm), then the tile packing.
inline int sort_and_pack(const double* base, const int* slot, long long stride, long long n,
                         const SortBuffers& sb, const double* masses, const double* cref,
                         PackedBody* near, float4* far, TileMeta* meta, const int* out_slot,
                         long long n_tiles, int T, cudaStream_t s) {
  sort_bbox_kernel<<<1, 256, 0, s>>>(base, slot, stride, n, sb.bbox);
  morton_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(base, slot, stride, n, sb.bbox,
                                                             sb.keys, sb.vals);
  GB_CUDA_TRY(cudaGetLastError());
  size_t bytes = sb.cub_bytes;
  GB_CUDA_TRY(cub::DeviceRadixSort::SortPairs(sb.cub_temp, bytes, sb.keys, sb.keys_alt, sb.vals,
                                              sb.perm, (int)n, 0, 63, s));
  if (T == 256) {
    pack_tiles_kernel<256><<<(unsigned)n_tiles, 256, 0, s>>>(base, slot, stride, n, sb.perm,
                                                             masses, cref, near, far, meta,
                                                             out_slot, n_tiles);
  } else {
    pack_tiles_kernel<128><<<(unsigned)n_tiles, 128, 0, s>>>(base, slot, stride, n, sb.perm,
                                                             masses, cref, near, far, meta,
                                                             out_slot, n_tiles);
  }
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

}  // namespace gb
