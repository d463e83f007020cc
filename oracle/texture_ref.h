// TEST INFRASTRUCTURE ONLY -- CPU oracle: the material texture fetch of
// GetMaterialColors (src/cudaRTCommon.cu:369-406) through a texture with the
// descriptor of CreateCURTTexture (:418-448: float4 texels, normalized
// coordinates, wrap addressing, linear filtering).  The filter is the texture
// unit's documented one: x = frac(u) * W - 0.5, i = floor(x), the weight
// a = frac(x) kept with 8 fractional bits (rounded to the nearest 1/256),
// the same in y, texels (i, j), (i+1, j), (i, j+1), (i+1, j+1) wrapped and
// blended with (1-a)(1-b), a(1-b), (1-a)b, ab in that order.  R = float is
// the kernels' arithmetic to the bit; R = double serves the FP64 image.
#pragma once
#include <cmath>
#include <cstdint>
#include <vector>

namespace orc {

struct Texture {
  uint32_t w = 0, h = 0;
  std::vector<float> rgba;  // w * h * 4, row-major, row 0 first
};

template <typename R>
inline R tex_frac_coord(R u) {
  R f = u - std::floor(u);
  return (f >= (R)0 && f <= (R)1) ? f : (R)0;
}

inline int tex_wrap(long long i, int n) {
  long long r = i % n;
  return (int)(r < 0 ? r + n : r);
}

template <typename R>
inline void tex_bilinear(const Texture& t, R u, R v, R out[4]) {
  const int W = (int)t.w, H = (int)t.h;
  const R x = tex_frac_coord<R>(u) * (R)W - (R)0.5;
  const R y = tex_frac_coord<R>(v) * (R)H - (R)0.5;
  const R xf = std::floor(x), yf = std::floor(y);
  const R a = std::nearbyint((x - xf) * (R)256) * ((R)1 / (R)256);
  const R b = std::nearbyint((y - yf) * (R)256) * ((R)1 / (R)256);
  const int i0 = tex_wrap((long long)xf, W), i1 = tex_wrap((long long)xf + 1, W);
  const int j0 = tex_wrap((long long)yf, H), j1 = tex_wrap((long long)yf + 1, H);
  const float* t00 = &t.rgba[((size_t)j0 * W + i0) * 4];
  const float* t10 = &t.rgba[((size_t)j0 * W + i1) * 4];
  const float* t01 = &t.rgba[((size_t)j1 * W + i0) * 4];
  const float* t11 = &t.rgba[((size_t)j1 * W + i1) * 4];
  const R w00 = ((R)1 - a) * ((R)1 - b), w10 = a * ((R)1 - b), w01 = ((R)1 - a) * b, w11 = a * b;
  for (int k = 0; k < 4; k++)
    out[k] = ((w00 * (R)t00[k] + w10 * (R)t10[k]) + w01 * (R)t01[k]) + w11 * (R)t11[k];
}

}  // namespace orc
