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
//     (2*radius+1 weights); larger radii are rejected;
//   * the array is one per device and lives until the process exits; every
//     call overwrites the first 2*radius+1 entries before its kernel reads
//     them, so nothing has to start at zero;
//   * calls whose work overlaps on the GPU (different streams or threads)
//     race on that array and must be serialized by the caller;
//   * the first call on a device looks up the array's device address with
//     cudaGetSymbolAddress (with that device current); make that first call
//     before any stream capture on that device.
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
float* g_weights_dev[kMaxDevices] = {nullptr};

gbpt_status weights_address(float** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return gbpt::fail(GBPT_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return gbpt::fail(GBPT_ERR_INVALID_ARG, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_weights_dev[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_weights);
    if (e != cudaSuccess || !p)
      return gbpt::fail(GBPT_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    g_weights_dev[dev] = (float*)p;
  }
  *out = g_weights_dev[dev];
  return GBPT_OK;
}

}  // namespace

extern "C" gbpt_status gbpt_bilateral_noalloc(const float* color, const float* pos, const float* norm,
                                              const float* emit, uint32_t width, uint32_t height, float color_eud,
                                              float pos_eud, float norm_eud, float emit_eud, uint32_t radius,
                                              const float* g, float* out, void* stream) {
  if (!color || !pos || !norm || !g || !out) return gbpt::fail(GBPT_ERR_INVALID_ARG, "NULL argument");
  if (width == 0 || height == 0) return gbpt::fail(GBPT_ERR_INVALID_ARG, "empty image");
  if (2 * radius + 1 > kMaxWeights)
    return gbpt::fail(GBPT_ERR_INVALID_ARG, "radius " + std::to_string(radius) +
                                                " exceeds the allocation-free limit of 31 (64-entry weight table)");
  float* table = nullptr;
  gbpt_status st = weights_address(&table);
  if (st != GBPT_OK) return st;
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = cudaMemcpyAsync(table, g, (2 * radius + 1) * sizeof(float), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess)
    e = gbpt::launch_bilateral(color, pos, norm, emit, width, height, color_eud, pos_eud, norm_eud, emit_eud, radius,
                               table, out, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return gbpt::fail(GBPT_ERR_CUDA, std::string("bilateral_noalloc: ") + cudaGetErrorString(e));
  return GBPT_OK;
}
