// noalloc.cu -- the mixed-precision N-body right-hand side for callers that
// must not allocate device memory.
//
// gb_nbody_rhs_mixed needs 32 bytes of scratch per body (the packed hi/lo
// FP32 positions) plus the reference point; its caller passes that workspace.
// Some callers cannot obtain one: a host that hands the library a fixed,
// pre-reserved slice of device memory and rejects any further cudaMalloc, or
// an executor-style caller that evaluates the right-hand side once per stage
// and cannot afford cudaMalloc/cudaFree per call (cudaFree waits for the whole
// device; the reference's CUDA executor pays that price on every reduction,
// src/par_exec/CudaExecutor.cuh:103-122).  This entry point takes the scratch
// from a fixed device array compiled into the library instead.
#include <mutex>

#include "force.cuh"

namespace gb {
int validate_nbody(const void* a, const void* b, long long n, double softening, double mass,
                   const double* masses);
int mixed_rhs_into(const double* x, double* dxdt, long long n, double softening, double mass,
                   const double* masses, PackedBody* packed, double* c,
                   const gb_force_tiling* tiling, cudaStream_t s);
}  // namespace gb

namespace {

constexpr long long kNoAllocMaxBodies = 65536;
constexpr size_t kPackedBytes = (size_t)kNoAllocMaxBodies * sizeof(gb::PackedBody);

// 2 MiB of packed bodies followed by the reference point (3 doubles).  Every
// GPU that loads the library holds this array until the process exits.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kPackedBytes + 256];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_scratch_ptr[kMaxDevices] = {};

// Device address of the scratch array on the current device, looked up once
// per device (the host-side name of a __device__ array is only a stand-in).
// The cached address belongs to the device's current context: after
// cudaDeviceReset the module is loaded again and the address may change, so
// this entry point must not be called after a reset in the same process.
int scratch_for_current_device(unsigned char** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    gb::note_cuda_error(e);
    return GB_ERR_CUDA;
  }
  if (dev < 0 || dev >= kMaxDevices) return GB_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      gb::note_cuda_error(e);
      return GB_ERR_CUDA;
    }
    g_scratch_ptr[dev] = p;
  }
  *out = static_cast<unsigned char*>(g_scratch_ptr[dev]);
  return GB_OK;
}

}  // namespace

extern "C" int64_t gb_nbody_rhs_mixed_noalloc_max_bodies(void) { return kNoAllocMaxBodies; }

extern "C" int gb_nbody_rhs_mixed_noalloc(const double* x, double* dxdt, int64_t n,
                                          double softening, double mass, const double* masses,
                                          const gb_force_tiling* tiling, gb_stream_t stream) {
  // the same argument checks as gb_nbody_rhs_mixed
  GB_TRY(gb::validate_nbody(x, dxdt, n, softening, mass, masses));
  if (!(softening > 0.0)) return GB_ERR_INVALID_ARGUMENT;
  if (n > kNoAllocMaxBodies) return GB_ERR_CAPACITY;
  unsigned char* base = nullptr;
  int rc = scratch_for_current_device(&base);
  if (rc != GB_OK) return rc;
  auto* packed = reinterpret_cast<gb::PackedBody*>(base);
  auto* c = reinterpret_cast<double*>(base + kPackedBytes);
  return gb::mixed_rhs_into(x, dxdt, n, softening, mass, masses, packed, c, tiling,
                            gb::as_cuda(stream));
}
