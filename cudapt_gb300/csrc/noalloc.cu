// Allocation-free variant of the device-array bilateral filter.
//
// gbpt_bilateral() copies the caller's spatial weight table into a small
// device buffer that it cudaMalloc's and cudaFree's on every call.  Some
// callers cannot do that: code that runs while a custom allocator or a
// pre-reserved memory pool owns the device heap (serving processes that
// forbid driver allocations after start-up), or callers on latency-critical
// paths where a cudaMalloc/cudaFree pair (which can synchronize the device)
// is not acceptable.  gbpt_bilateral_noalloc() keeps that weight table in a
// file-scope device array instead, so it never allocates or frees memory.
//
// Limits and sharing:
//   * the table holds at most kMaxWeights = 64 floats, so radius <= 31
//     (2*radius+1 weights); larger radii are rejected before any arithmetic
//     on the radius;
//   * the array is one per device and lives until the process exits; every
//     call overwrites the first 2*radius+1 entries before its kernel reads
//     them, so nothing has to start at zero;
//   * calls whose work overlaps on the GPU (different streams or threads)
//     race on that array and must be serialized by the caller;
//   * the first call in a device's context looks up the array's device
//     address with cudaGetSymbolAddress (with that device current) and keeps
//     it for that context; a call in a new context of the same device (after
//     cudaDeviceReset, for instance) looks it up again;
//   * each call copies the table from host memory and then synchronizes the
//     caller's stream (all work queued on it so far, not only the filter), so
//     it is refused (GBPT_ERR_STATE) while that stream is being captured.
#include <cuda.h>
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "gbpt_internal.h"
#include "launch.h"

namespace {

constexpr uint32_t kMaxWeights = 64;
constexpr int kMaxDevices = 64;

// Host code must not take the address of this array directly: on the host
// the name is only a stand-in for the device symbol.
static __device__ __align__(256) float g_weights[kMaxWeights];

std::mutex g_mu;
struct Cached {
  unsigned long long ctx_id = 0;  // cuCtxGetId of the context the address belongs to (0: none yet)
  float* ptr = nullptr;
};
Cached g_cache[kMaxDevices];

// Driver entry points resolved through the runtime (the library does not link
// libcuda): the current context and its process-unique id.
typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long*);

bool current_context_id(unsigned long long* id) {
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  static bool resolved = false;
  if (!resolved) {
    cudaDriverEntryPointQueryResult q1 = cudaDriverEntryPointSymbolNotFound, q2 = cudaDriverEntryPointSymbolNotFound;
    void* f1 = nullptr;
    void* f2 = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) == cudaSuccess &&
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) == cudaSuccess &&
        q1 == cudaDriverEntryPointSuccess && q2 == cudaDriverEntryPointSuccess) {
      get_current = (CtxGetCurrentFn)f1;
      get_id = (CtxGetIdFn)f2;
    }
    resolved = true;
  }
  CUcontext ctx = nullptr;
  if (!get_current || !get_id || get_current(&ctx) != CUDA_SUCCESS || !ctx) return false;
  return get_id(ctx, id) == CUDA_SUCCESS;
}

gbpt_status weights_address(float** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return gbpt::fail(GBPT_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return gbpt::fail(GBPT_ERR_INVALID_ARG, "device ordinal out of range");
  // the caller's earlier runtime call (cudaStreamIsCapturing) has made the
  // device's context current; without an id the address is looked up anew
  unsigned long long ctx_id = 0;
  const bool have_id = current_context_id(&ctx_id);
  std::lock_guard<std::mutex> lock(g_mu);
  Cached& c = g_cache[dev];
  if (!have_id || !c.ptr || c.ctx_id != ctx_id) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_weights);
    if (e != cudaSuccess || !p)
      return gbpt::fail(GBPT_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    c.ptr = (float*)p;
    c.ctx_id = have_id ? ctx_id : 0;
  }
  *out = c.ptr;
  return GBPT_OK;
}

}  // namespace

extern "C" gbpt_status gbpt_bilateral_noalloc(const float* color, const float* pos, const float* norm,
                                              const float* emit, uint32_t width, uint32_t height, float color_eud,
                                              float pos_eud, float norm_eud, float emit_eud, uint32_t radius,
                                              const float* g, float* out, void* stream) {
  if (!color || !pos || !norm || !g || !out) return gbpt::fail(GBPT_ERR_INVALID_ARG, "NULL argument");
  if (width == 0 || height == 0) return gbpt::fail(GBPT_ERR_INVALID_ARG, "empty image");
  // compared before any arithmetic on radius, which could wrap
  if (radius > (kMaxWeights - 1) / 2)
    return gbpt::fail(GBPT_ERR_INVALID_ARG, "radius " + std::to_string(radius) +
                                                " exceeds the allocation-free limit of 31 (64-entry weight table)");
  cudaStream_t s = (cudaStream_t)stream;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  cudaError_t e = cudaStreamIsCapturing(s, &cap);
  if (e != cudaSuccess || cap != cudaStreamCaptureStatusNone)
    return gbpt::fail(GBPT_ERR_STATE, "gbpt_bilateral_noalloc copies from host memory and synchronizes its stream: "
                                      "it cannot be called while the stream is being captured");
  float* table = nullptr;
  gbpt_status st = weights_address(&table);
  if (st != GBPT_OK) return st;
  e = cudaMemcpyAsync(table, g, (2 * radius + 1) * sizeof(float), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess)
    e = gbpt::launch_bilateral(color, pos, norm, emit, width, height, color_eud, pos_eud, norm_eud, emit_eud, radius,
                               table, out, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return gbpt::fail(GBPT_ERR_CUDA, std::string("bilateral_noalloc: ") + cudaGetErrorString(e));
  return GBPT_OK;
}
