// Material textures of GetMaterialColors (src/cudaRTCommon.cu:369-406).
//
// The reference samples float4 textures through texture objects created by
// CreateCURTTexture (:418-448): normalized coordinates, wrap addressing on
// both axes, linear filtering.  Here textures are plain float4 arrays in HBM
// (all textures of a scene in one array, a {first texel, width, height}
// record each) and the filter runs in the kernel, so that every bit of a
// textured frame is reproducible by the CPU oracle.  It follows the texture
// unit's documented linear filter: x = frac(u) * W - 0.5, i = floor(x), the
// weight a = frac(x) kept with 8 fractional bits (rounded to the nearest
// 1/256), the same in y, texels (i, j), (i+1, j), (i, j+1), (i+1, j+1)
// wrapped around the edges and blended with (1-a)(1-b), a(1-b), (1-a)b, ab.
// The hardware's own blend arithmetic is not documented to the bit; a GPU
// test bounds the difference to the texture unit's result.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace gbpt {

__device__ __forceinline__ float tex_frac_coord(float u) {
  float f = u - floorf(u);
  return (f >= 0.f && f <= 1.f) ? f : 0.f;  // NaN / infinite coordinates read texel (0, 0)'s corner
}

__device__ __forceinline__ int tex_wrap(int i, int n) {
  int r = i % n;
  return r < 0 ? r + n : r;
}

// texel record: {first texel index, width, height, 0} (uint bits)
__device__ __forceinline__ float4 tex_bilinear(const float4* __restrict__ texels, uint4 info, float u, float v) {
  const int W = (int)info.y, H = (int)info.z;
  const float x = tex_frac_coord(u) * (float)W - 0.5f;
  const float y = tex_frac_coord(v) * (float)H - 0.5f;
  const float xf = floorf(x), yf = floorf(y);
  const float a = rintf((x - xf) * 256.0f) * (1.0f / 256.0f);
  const float b = rintf((y - yf) * 256.0f) * (1.0f / 256.0f);
  const int i0 = tex_wrap((int)xf, W), i1 = tex_wrap((int)xf + 1, W);
  const int j0 = tex_wrap((int)yf, H), j1 = tex_wrap((int)yf + 1, H);
  const float4* t = texels + info.x;
  const float4 t00 = __ldg(t + (size_t)j0 * W + i0), t10 = __ldg(t + (size_t)j0 * W + i1);
  const float4 t01 = __ldg(t + (size_t)j1 * W + i0), t11 = __ldg(t + (size_t)j1 * W + i1);
  const float w00 = (1.f - a) * (1.f - b), w10 = a * (1.f - b), w01 = (1.f - a) * b, w11 = a * b;
  float4 r;
  r.x = ((w00 * t00.x + w10 * t10.x) + w01 * t01.x) + w11 * t11.x;
  r.y = ((w00 * t00.y + w10 * t10.y) + w01 * t01.y) + w11 * t11.y;
  r.z = ((w00 * t00.z + w10 * t10.z) + w01 * t01.z) + w11 * t11.z;
  r.w = ((w00 * t00.w + w10 * t10.w) + w01 * t01.w) + w11 * t11.w;
  return r;
}

}  // namespace gbpt
