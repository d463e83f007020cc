// Image export and the RMSE measurement of the RMSE-vs-time experiments.
//
// CUDAPTWindow saves results as 8-bit images and scores them against a
// captured converged image (src/cudapt.cpp:482-619, 867-896, 951-966):
//   * result PNG: clamp to [0,1], x = 1 - exp(-x * exposure), x = x^(1/2.2),
//     byte = (unsigned char)(x * 255), RGBA with alpha 255, top row first
//     (the result buffer has row 0 at the bottom);
//   * MSE PNG: per-pixel mean over RGB of (result - converged)^2, clamped to
//     [0,1], written to all three channels;
//   * converged BMP: clamp to [0,1] times 255;
//   * RMSE: sqrt(sum (converged - result)^2 / (3 W H)).  The reference sums in
//     float, in index order, on the host; here the sum runs on the device in
//     double (a different but far more accurate order-independent sum).
#include <cuda_runtime.h>

#include <cmath>
#include <string>

#include "gbpt_internal.h"
#include "launch.h"

namespace gbpt {
namespace {

constexpr int kBlock = 256;

__device__ __forceinline__ float clamp01(float x) { return fmaxf(0.f, fminf(x, 1.0f)); }
__device__ __forceinline__ unsigned char to_byte(float x) { return (unsigned char)(x * 255.f); }

__global__ void k_tonemap(const float* __restrict__ rgb, const float* __restrict__ ref, uint32_t w, uint32_t h,
                          float exposure, int kind, uchar4* __restrict__ out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= w * h) return;
  const uint32_t y = i / w, x = i - y * w;
  const size_t ind = ((size_t)(h - y - 1) * w + x) * 3;
  float c[3];
  if (kind == 1) {
    const float d0 = rgb[ind] - ref[ind], d1 = rgb[ind + 1] - ref[ind + 1], d2 = rgb[ind + 2] - ref[ind + 2];
    const float m = clamp01((d0 * d0 + d1 * d1 + d2 * d2) / 3.f);
    c[0] = c[1] = c[2] = m;
  } else {
    for (int k = 0; k < 3; k++) {
      float v = clamp01(rgb[ind + k]);
      if (kind == 0) {
        v = 1.0f - expf(-v * exposure);
        v = powf(v, 1.0f / 2.2f);
      }
      c[k] = v;
    }
  }
  out[i] = make_uchar4(to_byte(c[0]), to_byte(c[1]), to_byte(c[2]), 255);
}

__global__ void k_sqdiff(const float* __restrict__ a, const float* __restrict__ b, uint64_t n, double* acc) {
  __shared__ double part[kBlock / 32];
  double s = 0.0;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const double d = (double)a[i] - (double)b[i];
    s += d * d;
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int k = 0; k < kBlock / 32; k++) t += part[k];
    atomicAdd(acc, t);
  }
}

template <typename T>
struct DevBuf {
  T* p = nullptr;
  ~DevBuf() {
    if (p) cudaFree(p);
  }
};

#define CKI(x)                                                                              \
  do {                                                                                      \
    cudaError_t e_ = (x);                                                                   \
    if (e_ != cudaSuccess) return fail(GBPT_ERR_CUDA, std::string(#x ": ") + cudaGetErrorString(e_)); \
  } while (0)

}  // namespace

gbpt_status rmse_device(const float* a, const float* b, uint64_t n, double* out, void* stream) {
  cudaStream_t st = (cudaStream_t)stream;
  DevBuf<double> acc;
  CKI(cudaMalloc(&acc.p, sizeof(double)));
  CKI(cudaMemsetAsync(acc.p, 0, sizeof(double), st));
  if (n) {
    const uint64_t want = (n + kBlock - 1) / kBlock;
    const uint32_t grid = (uint32_t)(want < (uint64_t)sm_count() * 8 ? want : (uint64_t)sm_count() * 8);
    k_sqdiff<<<grid, kBlock, 0, st>>>(a, b, n, acc.p);
    note_launches(1);
    CKI(cudaGetLastError());
  }
  double s = 0.0;
  CKI(cudaMemcpyAsync(&s, acc.p, sizeof(double), cudaMemcpyDeviceToHost, st));
  CKI(cudaStreamSynchronize(st));
  *out = n ? std::sqrt(s / (double)n) : 0.0;
  return GBPT_OK;
}

}  // namespace gbpt

using gbpt::DevBuf;
using gbpt::fail;

extern "C" {

gbpt_status gbpt_rmse(const float* a, const float* b, uint64_t n, int32_t is_device, double* out) {
  if (!a || !b || !out) return fail(GBPT_ERR_INVALID_ARG, "NULL argument");
  if (is_device) return gbpt::rmse_device(a, b, n, out, nullptr);
  DevBuf<float> da, db;
  CKI(cudaMalloc(&da.p, n * 4 + 4));
  CKI(cudaMalloc(&db.p, n * 4 + 4));
  CKI(cudaMemcpy(da.p, a, n * 4, cudaMemcpyHostToDevice));
  CKI(cudaMemcpy(db.p, b, n * 4, cudaMemcpyHostToDevice));
  return gbpt::rmse_device(da.p, db.p, n, out, nullptr);
}

gbpt_status gbpt_tonemap_rgba8(const float* rgb, const float* ref, uint32_t width, uint32_t height, float exposure,
                               int32_t kind, uint8_t* out_rgba, int32_t is_device) {
  if (!rgb || !out_rgba || (kind == 1 && !ref)) return fail(GBPT_ERR_INVALID_ARG, "NULL argument");
  if (kind < 0 || kind > 2) return fail(GBPT_ERR_INVALID_ARG, "kind is 0 (result), 1 (MSE) or 2 (clamped)");
  const size_t np = (size_t)width * height;
  if (np == 0) return GBPT_OK;
  const uint32_t grid = (uint32_t)((np + 255) / 256);
  if (is_device) {
    gbpt::k_tonemap<<<grid, 256>>>(rgb, ref, width, height, exposure, kind, (uchar4*)out_rgba);
    gbpt::note_launches(1);
    CKI(cudaGetLastError());
    CKI(cudaDeviceSynchronize());
    return GBPT_OK;
  }
  DevBuf<float> dc, dr;
  DevBuf<uchar4> dout;
  CKI(cudaMalloc(&dc.p, np * 12));
  CKI(cudaMalloc(&dout.p, np * 4));
  CKI(cudaMemcpy(dc.p, rgb, np * 12, cudaMemcpyHostToDevice));
  if (kind == 1) {
    CKI(cudaMalloc(&dr.p, np * 12));
    CKI(cudaMemcpy(dr.p, ref, np * 12, cudaMemcpyHostToDevice));
  }
  gbpt::k_tonemap<<<grid, 256>>>(dc.p, dr.p, width, height, exposure, kind, dout.p);
  gbpt::note_launches(1);
  CKI(cudaGetLastError());
  CKI(cudaMemcpy(out_rgba, dout.p, np * 4, cudaMemcpyDeviceToHost));
  return GBPT_OK;
}

}  // extern "C"
