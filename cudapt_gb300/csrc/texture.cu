// Texture filter checks: the kernels' software filter (texture.cuh) and the
// texture unit the reference sampled through (a texture object over a CUDA
// array with the descriptor of CreateCURTTexture, src/cudaRTCommon.cu:418-448),
// evaluated at the same coordinates.  Test entry point only: it allocates.
#include <cuda_runtime.h>

#include <string>

#include "gbpt_internal.h"
#include "texture.cuh"

namespace gbpt {
namespace {

__global__ void k_tex_hw(cudaTextureObject_t obj, const float2* uv, uint32_t n, float4* out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = tex2D<float4>(obj, uv[i].x, uv[i].y);
}

__global__ void k_tex_sw(const float4* texels, uint4 info, const float2* uv, uint32_t n, float4* out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = tex_bilinear(texels, info, uv[i].x, uv[i].y);
}

}  // namespace
}  // namespace gbpt

extern "C" gbpt_status gbpt_texture_sample(const float* rgba, uint32_t width, uint32_t height, const float* uv,
                                           uint32_t n, int32_t hardware, float* out) {
  using namespace gbpt;
  if (!rgba || !uv || !out || width == 0 || height == 0) return fail(GBPT_ERR_INVALID_ARG, "NULL or empty argument");
  if (width > 16384 || height > 16384) return fail(GBPT_ERR_INVALID_ARG, "texture larger than 16384 x 16384");
  if (n == 0) return GBPT_OK;
  const size_t texN = (size_t)width * height;
  float4* dTex = nullptr;
  float2* dUv = nullptr;
  float4* dOut = nullptr;
  cudaArray_t arr = nullptr;
  cudaTextureObject_t obj = 0;
  cudaError_t e = cudaMalloc(&dUv, n * sizeof(float2));
  if (e == cudaSuccess) e = cudaMalloc(&dOut, n * sizeof(float4));
  if (e == cudaSuccess) e = cudaMemcpy(dUv, uv, n * sizeof(float2), cudaMemcpyHostToDevice);
  const uint32_t grid = (n + 255) / 256;
  if (e == cudaSuccess && hardware) {
    cudaChannelFormatDesc cd = cudaCreateChannelDesc(32, 32, 32, 32, cudaChannelFormatKindFloat);
    e = cudaMallocArray(&arr, &cd, width, height);
    if (e == cudaSuccess)
      e = cudaMemcpy2DToArray(arr, 0, 0, rgba, width * sizeof(float4), width * sizeof(float4), height,
                              cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
      cudaResourceDesc rd{};
      rd.resType = cudaResourceTypeArray;
      rd.res.array.array = arr;
      cudaTextureDesc td{};
      td.addressMode[0] = cudaAddressModeWrap;
      td.addressMode[1] = cudaAddressModeWrap;
      td.filterMode = cudaFilterModeLinear;
      td.readMode = cudaReadModeElementType;
      td.normalizedCoords = 1;
      e = cudaCreateTextureObject(&obj, &rd, &td, nullptr);
    }
    if (e == cudaSuccess) {
      k_tex_hw<<<grid, 256>>>(obj, dUv, n, dOut);
      e = cudaGetLastError();
    }
  } else if (e == cudaSuccess) {
    e = cudaMalloc(&dTex, texN * sizeof(float4));
    if (e == cudaSuccess) e = cudaMemcpy(dTex, rgba, texN * sizeof(float4), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
      k_tex_sw<<<grid, 256>>>(dTex, make_uint4(0u, width, height, 0u), dUv, n, dOut);
      e = cudaGetLastError();
    }
  }
  if (e == cudaSuccess) e = cudaMemcpy(out, dOut, n * sizeof(float4), cudaMemcpyDeviceToHost);
  if (obj) cudaDestroyTextureObject(obj);
  if (arr) cudaFreeArray(arr);
  cudaFree(dTex);
  cudaFree(dUv);
  cudaFree(dOut);
  if (e != cudaSuccess) return fail(GBPT_ERR_CUDA, std::string("texture sample: ") + cudaGetErrorString(e));
  return GBPT_OK;
}
