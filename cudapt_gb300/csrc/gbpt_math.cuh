// Device float helpers of the GB300 BDPT kernels.
//
// Arithmetic contract.  CudaPT builds its float3 algebra from explicit
// round-to-nearest intrinsics (include/cudahelper.h:119-310): vecCross and
// vecDot use __fmaf_rn, the component operators __fadd_rn/__fmul_rn/__fdiv_rn,
// rcpf __frcp_rn and `length` the round-down square root __fsqrt_rd.  The
// kernels keep exactly that, and every other expression is a chain of single
// IEEE operations: this translation unit is compiled with -fmad=false, so no
// a*b+c is ever contracted behind our back.  Double-precision literals of the
// reference (1e-9, 0.1, 1e-4) that it compares floats against are replaced by
// the float thresholds giving the same answer for every float input.
//
// Transcendentals are the project's own (Cody & Waite argument reduction with
// a two-constant split, Taylor polynomials with coefficients 1/n!), so results
// do not depend on the CUDA math library version.
#pragma once
#include <cstdint>

#ifndef __CUDACC__
#include <cmath>
#endif

#if defined(__CUDACC__)
#define GB_HD __host__ __device__ __forceinline__
#else
#define GB_HD inline
#endif

namespace gb {

// ---- thresholds equivalent to the reference's double comparisons ----------
// (double)|x| < 1e-9        <=> |x| < kLtEps9
// (double)x   > 1e-9        <=> x   > kGtEps9
// (double)p   < 1e-4        <=> p   < kLtEps4           (ProbabilityRand)
// (double)p + 1e-4 > 1.0    <=> p   >= kProbOne         (ProbabilityRand)
// (double)|x| > 0.1         <=> |x| >= kPointOne        (tangent-frame switch)
constexpr float kEps9f = 0x1.12e0bep-30f;  // (float)1e-9, the float M_EPSILON argument
constexpr float kLtEps9 = 0x1.12e0c0p-30f;
constexpr float kGtEps9 = 0x1.12e0bep-30f;
constexpr float kLtEps4 = 0x1.a36e30p-14f;
constexpr float kProbOne = 0x1.fff2e6p-1f;
constexpr float kPointOne = 0x1.99999ap-4f;
constexpr float kInf = 0x1.5af1d8p+66f;    // (float)1e20, M_INF
constexpr float kBias = 0x1.a36e2ep-14f;   // (float)1e-4, M_FLT_BIAS_EPSILON
constexpr float kFltEps = 0x1.4f8b58p-17f; // (float)1e-5, M_FLT_EPSILON
constexpr float kPi = 0x1.921fb6p+1f;      // (float)M_PI
constexpr float kInvPi = 0x1.45f306p-2f;   // (float)(1/M_PI)
constexpr float kTwoPi = 0x1.921fb6p+2f;   // (float)(2*M_PI)
constexpr float kF0Spec = 0x1.47ae14p-4f;  // (float)0.08

struct f3 {
  float x, y, z;
};
GB_HD f3 mk(float x, float y, float z) { return f3{x, y, z}; }

#if defined(__CUDA_ARCH__)
GB_HD float fma_(float a, float b, float c) { return __fmaf_rn(a, b, c); }
GB_HD float rcp_(float a) { return __frcp_rn(a); }
GB_HD float sqrt_rd_(float a) { return __fsqrt_rd(a); }
GB_HD float rint_(float a) { return rintf(a); }
GB_HD float bits_f(uint32_t b) { return __uint_as_float(b); }
#else
inline float fma_(float a, float b, float c) { return std::fmaf(a, b, c); }
inline float rcp_(float a) { return 1.f / a; }
inline float sqrt_rd_(float x) {
  float s = std::sqrt(x);
  if (!(x > 0.f) || std::isinf(x)) return s;
  if ((double)s * (double)s > (double)x) s = std::nextafter(s, 0.f);
  return s;
}
inline float rint_(float a) { return std::nearbyint(a); }
inline float bits_f(uint32_t b) {
  float f;
  __builtin_memcpy(&f, &b, 4);
  return f;
}
#endif

GB_HD f3 operator+(f3 a, f3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
GB_HD f3 operator-(f3 a, f3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
GB_HD f3 operator*(f3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
GB_HD f3 operator*(float s, f3 a) { return mk(a.x * s, a.y * s, a.z * s); }
GB_HD f3 operator/(f3 a, float s) { return mk(a.x / s, a.y / s, a.z / s); }
GB_HD f3 vmul(f3 a, f3 b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }
GB_HD f3 vmax0(f3 a) { return mk(fmaxf(0.f, a.x), fmaxf(0.f, a.y), fmaxf(0.f, a.z)); }
GB_HD f3 neg(f3 a) { return mk(-a.x, -a.y, -a.z); }
GB_HD float dot(f3 l, f3 r) { return fma_(l.x, r.x, fma_(l.y, r.y, l.z * r.z)); }
GB_HD f3 cross(f3 l, f3 r) {
  return mk(fma_(l.y, r.z, -(l.z * r.y)), fma_(l.z, r.x, -(l.x * r.z)), fma_(l.x, r.y, -(l.y * r.x)));
}
GB_HD float length(f3 a) { return sqrt_rd_(a.x * a.x + a.y * a.y + a.z * a.z); }
GB_HD f3 normalize(f3 a) { return a / length(a); }
GB_HD f3 vlerp(f3 x, f3 y, float d) { return x + (y - x) * d; }
GB_HD float lerp(float x, float y, float d) { return x + (y - x) * d; }
GB_HD float escape_zero(float v) {
  float r = v;
  if (fabsf(r) < kEps9f) r = (r > 0) ? r + kEps9f : r - kEps9f;
  return r;
}

// sin and cos of x (|x| up to a few thousand): k = rint(x * 2/pi),
// r = x - k*pi/2 with pi/2 = hi + lo, Taylor degree 9 / 10 on |r| <= pi/4.
GB_HD void sincos_p(float x, float* s, float* c) {
  const float two_over_pi = 0x1.45f306p-1f;
  const float pio2_hi = 0x1.921fb6p+0f;
  const float pio2_lo = -0x1.777a5cp-25f;
  float kf = rint_(x * two_over_pi);
  float r = fma_(-kf, pio2_hi, x);
  r = fma_(-kf, pio2_lo, r);
  float r2 = r * r;
  float ps = fma_(r2, 2.75573192e-06f, -1.98412698e-04f);
  ps = fma_(r2, ps, 8.33333333e-03f);
  ps = fma_(r2, ps, -1.66666667e-01f);
  float sn = fma_(r * r2, ps, r);
  float pc = fma_(r2, -2.75573192e-07f, 2.48015873e-05f);
  pc = fma_(r2, pc, -1.38888889e-03f);
  pc = fma_(r2, pc, 4.16666667e-02f);
  pc = fma_(r2, pc, -0.5f);
  float cs = fma_(r2, pc, 1.0f);
  int q = ((int)kf) & 3;
  float so = (q & 1) ? cs : sn;
  float co = (q & 1) ? sn : cs;
  if (q == 1 || q == 2) co = -co;
  if (q >= 2) so = -so;
  *s = so;
  *c = co;
}

// exp(x): k = rint(x / ln2), r = x - k*ln2 (hi + lo), Taylor degree 7,
// times 2^k applied as two exact power-of-two factors.  x < -87 gives 0.
GB_HD float exp_p(float x) {
  if (x < -87.0f) return 0.0f;
  if (x > 88.0f) return bits_f(0x7f800000u);
  const float log2e = 0x1.715476p+0f;
  const float ln2_hi = 0x1.62e430p-1f;
  const float ln2_lo = -0x1.05c610p-29f;
  float kf = rint_(x * log2e);
  float r = fma_(-kf, ln2_hi, x);
  r = fma_(-kf, ln2_lo, r);
  float p = fma_(r, 1.98412698e-04f, 1.38888889e-03f);
  p = fma_(r, p, 8.33333333e-03f);
  p = fma_(r, p, 4.16666667e-02f);
  p = fma_(r, p, 1.66666667e-01f);
  p = fma_(r, p, 0.5f);
  p = fma_(r, p, 1.0f);
  p = fma_(r, p, 1.0f);
  int k = (int)kf;
  int k1 = k / 2, k2 = k - k1;
  return (p * bits_f((uint32_t)(k1 + 127) << 23)) * bits_f((uint32_t)(k2 + 127) << 23);
}

GB_HD float pow5(float x) {
  float x2 = x * x;
  return (x2 * x2) * x;
}

// ---- Philox4x32-10 (Salmon et al., SC'11) ----------------------------------
struct u4 {
  uint32_t a, b, c, d;
};
GB_HD u4 philox(u4 ctr, uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; r++) {
#if defined(__CUDA_ARCH__)
    uint32_t lo0 = 0xD2511F53u * ctr.a, hi0 = __umulhi(0xD2511F53u, ctr.a);
    uint32_t lo1 = 0xCD9E8D57u * ctr.c, hi1 = __umulhi(0xCD9E8D57u, ctr.c);
#else
    uint64_t p0 = (uint64_t)0xD2511F53u * ctr.a, p1 = (uint64_t)0xCD9E8D57u * ctr.c;
    uint32_t lo0 = (uint32_t)p0, hi0 = (uint32_t)(p0 >> 32), lo1 = (uint32_t)p1, hi1 = (uint32_t)(p1 >> 32);
#endif
    ctr = u4{hi1 ^ ctr.b ^ k0, lo1, hi0 ^ ctr.d ^ k1, lo0};
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return ctr;
}
// 23 random bits -> (2m+1) * 2^-24 in (0, 1), exact
GB_HD float u01(uint32_t x) { return (float)(x >> 9) * 0x1p-23f + 0x1p-24f; }

enum Stream : uint32_t { kCamera = 0, kEyeBounce = 1, kLightGen = 2, kLightBounce = 3, kBinaryAccept = 4 };

// Eight uniforms for one (path, frame, stream, depth, sample): two Philox blocks.
GB_HD void draw8(uint32_t k0, uint32_t k1, uint32_t path, uint32_t frame, uint32_t stream, uint32_t depth,
                 uint32_t sample, float u[8]) {
  u4 a = philox(u4{path, frame, (stream << 24) | (depth << 8) | 0u, sample}, k0, k1);
  u4 b = philox(u4{path, frame, (stream << 24) | (depth << 8) | 1u, sample}, k0, k1);
  u[0] = u01(a.a); u[1] = u01(a.b); u[2] = u01(a.c); u[3] = u01(a.d);
  u[4] = u01(b.a); u[5] = u01(b.b); u[6] = u01(b.c); u[7] = u01(b.d);
}
GB_HD void draw4(uint32_t k0, uint32_t k1, uint32_t path, uint32_t frame, uint32_t stream, uint32_t depth,
                 uint32_t sample, uint32_t block, float u[4]) {
  u4 a = philox(u4{path, frame, (stream << 24) | (depth << 8) | block, sample}, k0, k1);
  u[0] = u01(a.a); u[1] = u01(a.b); u[2] = u01(a.c); u[3] = u01(a.d);
}

}  // namespace gb
