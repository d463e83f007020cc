// Pre-included stand-ins that let two of the reference's own sources build
// on the host, unmodified, for the oracle pin -- TEST INFRASTRUCTURE ONLY.
//
//   src/bvhhelper.cpp   (CreateBVH / CompactBVH, the binned-SAH builder)
//   src/cudaRTCommon.cu (CURay::IntersectAABB / IntersectTri, TracePrimitive,
//                        GetMaterialColors), compiled as host C++
//
// What is stood in, and why:
//   * include/mathhelper.h cannot be compiled by g++: its Vec2/Vec3/Vec4
//     unions hold anonymous structs whose members have constructors (an MSVC
//     extension).  This file defines the header's include guard and supplies
//     the NPMathHelper::Vec2 / Vec3 members, operators and macros that the two
//     sources and the headers they include use, each with the header's own
//     arithmetic (component-wise float operations, fmin/fmax, float sqrt,
//     normalize = v / length(v)).  Nothing of the builder or the traversal
//     is restated.
//   * MSVC's __int32 is given on the command line (-D__int32=int).
//   * cudaRTCommon.cu is compiled as host code with the device branch of
//     include/cudahelper.h selected (__CUDA_ARCH__ defined after the CUDA
//     headers), so IntersectAABB / IntersectTri / TracePrimitive run with the
//     arithmetic the reference's GPU executed: the IEEE single-precision
//     intrinsics __fadd_rn, __fsub_rn, __fmul_rn, __fdiv_rn, __frcp_rn (all
//     correctly rounded to nearest: the host's float operators), __fmaf_rn
//     (fused multiply-add: std::fma on floats) and __fsqrt_rd (square root
//     rounded towards zero, from the correctly rounded sqrtf and an exact
//     double-precision check of its square).
//   * The legacy texture references that CUDA 12 removed (texture<>,
//     tex1Dfetch, cudaBindTexture) become a plain array view; a fetch beyond
//     the bound range returns zeros as a texture reference did.
//   * tex2D on a texture object (GetMaterialColors) reads a host texture
//     registered by the pin library (refpin_capi.cpp) through the oracle's
//     restatement of the descriptor's filter (oracle/texture_ref.h:
//     normalized coordinates, wrap, linear filtering with 8-bit weights).
//   * curand_kernel.h, warp intrinsics and atomics are declared only so that
//     the file compiles; the pin library never calls the functions that use
//     them.
#ifndef GBREF_PRELUDE_H
#define GBREF_PRELUDE_H

#include <math.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <string>
#include <vector>

// ---------------------------------------------------------------- math stand-in
#define MATHHELPER_H
#define M_EPSILON 1E-9
#define M_FLT_EPSILON 1E-5
#define M_FLT_BIAS_EPSILON 1E-4
#define M_INF 1E20
#define M_MIN_INF -1E20
#define XORSWAP(a, b) ((a) ^= (b), (b) ^= (a), (a) ^= (b))
#define MAT_COLUMN_MAJOR

typedef unsigned int uint32;
typedef int int32;

namespace NPMathHelper {

class Vec2 {
 public:
  union {
    float _e[2];
    struct {
      float _x, _y;
    };
  };
  Vec2(const float x = 0.f, const float y = 0.f) {
    _x = x;
    _y = y;
  }
};

class Vec3 {
 public:
  union {
    float _e[3];
    struct {
      float _x, _y, _z;
    };
  };
  Vec3(const float x = 0.f, const float y = 0.f, const float z = 0.f) {
    _x = x;
    _y = y;
    _z = z;
  }
  Vec3(const Vec3& o) {
    _x = o._x;
    _y = o._y;
    _z = o._z;
  }
  Vec3& operator=(const Vec3& o) {
    _x = o._x;
    _y = o._y;
    _z = o._z;
    return *this;
  }
  static Vec3 cross(const Vec3& a, const Vec3& b) {
    return Vec3(a._y * b._z - a._z * b._y, a._z * b._x - a._x * b._z, a._x * b._y - a._y * b._x);
  }
  static float dot(const Vec3& a, const Vec3& b) { return a._x * b._x + a._y * b._y + a._z * b._z; }
  static float length(const Vec3& a) { return std::sqrt(a._x * a._x + a._y * a._y + a._z * a._z); }
  static Vec3 normalize(const Vec3& a);
  static Vec3 min(const Vec3& a, const Vec3& b) {
    return Vec3(std::fmin(a._x, b._x), std::fmin(a._y, b._y), std::fmin(a._z, b._z));
  }
  static Vec3 max(const Vec3& a, const Vec3& b) {
    return Vec3(std::fmax(a._x, b._x), std::fmax(a._y, b._y), std::fmax(a._z, b._z));
  }
  Vec3 cross(const Vec3& o) const { return cross(*this, o); }
  float dot(const Vec3& o) const { return dot(*this, o); }
  float length() const { return length(*this); }
  Vec3 normalize() const { return normalize(*this); }
  Vec3 min(const Vec3& o) const { return min(*this, o); }
  Vec3 max(const Vec3& o) const { return max(*this, o); }
  bool operator==(const Vec3& o) const { return _x == o._x && _y == o._y && _z == o._z; }
  bool operator!=(const Vec3& o) const { return !(*this == o); }
};

inline const Vec3 operator*(const Vec3& l, const float v) { return Vec3(l._x * v, l._y * v, l._z * v); }
inline const Vec3 operator*(const float v, const Vec3& r) { return r * v; }
inline const Vec3 operator/(const Vec3& l, const float v) { return Vec3(l._x / v, l._y / v, l._z / v); }
inline const Vec3 operator/(const Vec3& l, const Vec3& r) { return Vec3(l._x / r._x, l._y / r._y, l._z / r._z); }
inline const Vec3 operator+(const Vec3& l, const Vec3& r) { return Vec3(l._x + r._x, l._y + r._y, l._z + r._z); }
inline const Vec3 operator-(const Vec3& l, const Vec3& r) { return Vec3(l._x - r._x, l._y - r._y, l._z - r._z); }
inline Vec3 Vec3::normalize(const Vec3& a) {
  float l = length(a);
  return Vec3(a) / l;
}

}  // namespace NPMathHelper

#ifdef GBREF_CUDA_SHIMS
// ---------------------------------------------------------------- CUDA host shims
#include <cuda.h>
#include <cuda_runtime.h>
#include <device_launch_parameters.h>

// include/cudahelper.h defines host fminf/fmaxf/rsqrtf for compilers whose
// math library lacked them; glibc declares them, so its definitions are
// renamed (they keep the header's own semantics).
#define fminf gbref_fminf
#define fmaxf gbref_fmaxf
#define rsqrtf gbref_rsqrtf

// the device branch of include/cudahelper.h
#define __CUDA_ARCH__ 1000

inline float __fadd_rn(float a, float b) { return a + b; }
inline float __fsub_rn(float a, float b) { return a - b; }
inline float __fmul_rn(float a, float b) { return a * b; }
inline float __fdiv_rn(float a, float b) { return a / b; }
inline float __frcp_rn(float a) { return 1.0f / a; }
inline float __fmaf_rn(float a, float b, float c) { return std::fma(a, b, c); }
inline float __fsqrt_rd(float x) {
  float r = std::sqrt(x);
  if (std::isfinite(r) && r > 0.0f && (double)r * (double)r > (double)x) r = std::nextafter(r, 0.0f);
  return r;
}

// legacy texture references
template <class T, int dim = 1, enum cudaTextureReadMode mode = cudaReadModeElementType>
struct texture {
  const T* data = nullptr;
  size_t count = 0;
  int normalized = 0;
  cudaTextureFilterMode filterMode = cudaFilterModePoint;
  cudaTextureAddressMode addressMode[3] = {cudaAddressModeWrap, cudaAddressModeWrap, cudaAddressModeWrap};
};
template <class T, int dim, enum cudaTextureReadMode mode>
inline T tex1Dfetch(const texture<T, dim, mode>& t, int i) {
  T z;
  std::memset(&z, 0, sizeof(z));
  if (i < 0 || (size_t)i >= t.count || !t.data) return z;
  return t.data[i];
}
template <class T, int dim, enum cudaTextureReadMode mode>
inline cudaError_t cudaBindTexture(size_t*, const texture<T, dim, mode>& t, const void* p, const cudaChannelFormatDesc&,
                                   size_t size) {
  texture<T, dim, mode>& w = const_cast<texture<T, dim, mode>&>(t);
  w.data = (const T*)p;
  w.count = size / sizeof(T);
  return cudaSuccess;
}
template <class T, int dim, enum cudaTextureReadMode mode>
inline cudaError_t cudaUnbindTexture(const texture<T, dim, mode>& t) {
  texture<T, dim, mode>& w = const_cast<texture<T, dim, mode>&>(t);
  w.data = nullptr;
  w.count = 0;
  return cudaSuccess;
}

// texture objects: filtered fetch from a host texture registered by the pin library
float4 gbref_tex2D_float4(cudaTextureObject_t obj, float u, float v);
template <class T>
inline T tex2D(cudaTextureObject_t obj, float u, float v);
template <>
inline float4 tex2D<float4>(cudaTextureObject_t obj, float u, float v) {
  return gbref_tex2D_float4(obj, u, v);
}

// curand_kernel.h: the state type only (nothing here draws random numbers)
#define CURAND_KERNEL_H_
struct curandStateXORWOW {
  unsigned int d, v[5];
  int boxmuller_flag, boxmuller_flag_double;
  float boxmuller_extra;
  double boxmuller_extra_double;
};
typedef struct curandStateXORWOW curandState;
float curand_uniform(curandState*);

// warp intrinsics and atomics of atomicAggInc (never called on the host)
unsigned int __ballot(int);
int __ffs(int);
int __popc(unsigned int);
int atomicAdd(int*, int);
int __shfl(int, int);
#endif  // GBREF_CUDA_SHIMS

#endif  // GBREF_PRELUDE_H
