// TEST INFRASTRUCTURE ONLY -- part of the CPU oracle. Nothing in the shipped
// library may include this file; only tests/, the smoke check and the CPU
// baseline of bench.py load the oracle.
//
// Float semantics of the CudaPT device helpers, restated for the host.
//
// include/cudahelper.h:119-310 builds every float3 operator from explicit
// round-to-nearest intrinsics (__fadd_rn, __fmul_rn, __fmaf_rn, __frcp_rn,
// __fdiv_rn) and `length` from the round-down square root __fsqrt_rd.  On the
// host those map to single IEEE operations, provided the compiler does not
// contract a*b+c into an FMA: the oracle is always compiled with
// -ffp-contract=off and calls fmaf() exactly where the reference calls
// __fmaf_rn (vecCross, vecDot).
//
// Transcendentals: the reference calls CUDA's cosf/sinf/powf/expf, whose last
// bits are not pinned by anything in the reference.  The oracle and the CUDA
// kernels both use the functions below, written from the mathematics
// (Cody & Waite two-constant argument reduction, Taylor polynomials with
// coefficients 1/n!), so that a path traced on the GPU and on the CPU with the
// same random numbers gives the same bits.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

namespace orc {

struct f3 {
  float x, y, z;
};
static inline f3 mk(float x, float y, float z) { return f3{x, y, z}; }

// ---- include/cudahelper.h:119-125 escapeZero --------------------------------
static inline float escapeZero(float v, float eps) {
  float r = v;
  if (std::fabs(r) < eps) r = (r > 0) ? r + eps : r - eps;
  return r;
}
// ---- cudahelper.h:127-134, 170-177: __frcp_rn == IEEE 1/x -------------------
static inline float rcpf(float x) { return 1.f / x; }
// ---- cudahelper.h:142-150 vecMin/vecMax (fminf/fmaxf) -----------------------
static inline f3 vmin(f3 a, f3 b) { return mk(std::fmin(a.x, b.x), std::fmin(a.y, b.y), std::fmin(a.z, b.z)); }
static inline f3 vmax(f3 a, f3 b) { return mk(std::fmax(a.x, b.x), std::fmax(a.y, b.y), std::fmax(a.z, b.z)); }
// ---- cudahelper.h:152-159 vecMul -------------------------------------------
static inline f3 vmul(f3 a, f3 b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline f3 vrcp(f3 a) { return mk(1.f / a.x, 1.f / a.y, 1.f / a.z); }
// ---- cudahelper.h:179-189 vecCross with __fmaf_rn ---------------------------
static inline f3 cross(f3 l, f3 r) {
  return mk(std::fmaf(l.y, r.z, -(l.z * r.y)), std::fmaf(l.z, r.x, -(l.x * r.z)),
            std::fmaf(l.x, r.y, -(l.y * r.x)));
}
// ---- cudahelper.h:191-198 vecDot with __fmaf_rn -----------------------------
static inline float dot(f3 l, f3 r) { return std::fmaf(l.x, r.x, std::fmaf(l.y, r.y, l.z * r.z)); }
// ---- cudahelper.h:200-280 component operators --------------------------------
static inline f3 operator+(f3 a, f3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline f3 operator-(f3 a, f3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline f3 operator*(f3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
static inline f3 operator*(float s, f3 a) { return a * s; }
static inline f3 operator/(f3 a, float s) { return mk(a.x / s, a.y / s, a.z / s); }

// round-toward-zero square root of a non-negative float, from the IEEE
// round-to-nearest one: s*s is exact in double, so one comparison decides.
static inline float sqrt_rd(float x) {
  float s = std::sqrt(x);
  if (!(x > 0.f) || std::isinf(x)) return s;
  if ((double)s * (double)s > (double)x) s = std::nextafter(s, 0.f);
  return s;
}
// ---- cudahelper.h:292-304 length (__fsqrt_rd of an uncontracted sum) --------
static inline float length(f3 a) { return sqrt_rd(a.x * a.x + a.y * a.y + a.z * a.z); }
static inline f3 normalize(f3 a) { return a / length(a); }
// ---- cudahelper.h:306-309 vecLerp; :136-139 lerp ----------------------------
static inline f3 vlerp(f3 x, f3 y, float d) { return x + (y - x) * d; }
static inline float lerp(float x, float y, float d) { return x + (y - x) * d; }

// ---------------------------------------------------------------------------
// Project transcendentals (same algorithm as the CUDA kernels).
// sin/cos: Cody & Waite reduction by pi/2 split into a float head and tail,
// then Taylor polynomials of degree 9 (sin) and 10 (cos) on |r| <= pi/4.
static inline void sincos_p(float x, float* s, float* c) {
  const float two_over_pi = 0x1.45f306p-1f;
  const float pio2_hi = 0x1.921fb6p+0f;
  const float pio2_lo = -0x1.777a5cp-25f;
  float kf = std::nearbyint(x * two_over_pi);
  float r = std::fmaf(-kf, pio2_hi, x);
  r = std::fmaf(-kf, pio2_lo, r);
  float r2 = r * r;
  float ps = std::fmaf(r2, 2.75573192e-06f, -1.98412698e-04f);  // 1/9!, -1/7!
  ps = std::fmaf(r2, ps, 8.33333333e-03f);                        // 1/5!
  ps = std::fmaf(r2, ps, -1.66666667e-01f);                       // -1/3!
  float sn = std::fmaf(r * r2, ps, r);
  float pc = std::fmaf(r2, -2.75573192e-07f, 2.48015873e-05f);   // -1/10!, 1/8!
  pc = std::fmaf(r2, pc, -1.38888889e-03f);                       // -1/6!
  pc = std::fmaf(r2, pc, 4.16666667e-02f);                        // 1/4!
  pc = std::fmaf(r2, pc, -0.5f);                                  // -1/2!
  float cs = std::fmaf(r2, pc, 1.0f);
  int q = ((int)kf) & 3;
  float so, co;
  switch (q) {
    case 0: so = sn; co = cs; break;
    case 1: so = cs; co = -sn; break;
    case 2: so = -sn; co = -cs; break;
    default: so = -cs; co = sn; break;
  }
  *s = so;
  *c = co;
}
// exp: Cody & Waite reduction by ln2 (head/tail), Taylor degree 7 on
// |r| <= ln2/2, exact scaling by 2^k.  Arguments below -87 return 0.
static inline float exp_p(float x) {
  if (x < -87.0f) return 0.0f;
  if (x > 88.0f) return INFINITY;
  const float log2e = 0x1.715476p+0f;
  const float ln2_hi = 0x1.62e430p-1f;
  const float ln2_lo = -0x1.05c610p-29f;
  float kf = std::nearbyint(x * log2e);
  float r = std::fmaf(-kf, ln2_hi, x);
  r = std::fmaf(-kf, ln2_lo, r);
  float p = std::fmaf(r, 1.98412698e-04f, 1.38888889e-03f);  // 1/7!, 1/6!
  p = std::fmaf(r, p, 8.33333333e-03f);                        // 1/5!
  p = std::fmaf(r, p, 4.16666667e-02f);                        // 1/4!
  p = std::fmaf(r, p, 1.66666667e-01f);                        // 1/3!
  p = std::fmaf(r, p, 0.5f);                                   // 1/2!
  p = std::fmaf(r, p, 1.0f);
  p = std::fmaf(r, p, 1.0f);
  int k = (int)kf;
  // 2^k as two factors so that k down to -126 stays exact
  int k1 = k / 2, k2 = k - k1;
  uint32_t b1 = (uint32_t)(k1 + 127) << 23, b2 = (uint32_t)(k2 + 127) << 23;
  float s1, s2;
  std::memcpy(&s1, &b1, 4);
  std::memcpy(&s2, &b2, 4);
  return (p * s1) * s2;
}
// pow(x, 5) as ((x*x)*(x*x))*x
static inline float pow5(float x) {
  float x2 = x * x;
  return (x2 * x2) * x;
}

}  // namespace orc
