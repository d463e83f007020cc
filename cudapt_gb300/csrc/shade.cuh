// Shading helpers of the GB300 BDPT kernels: the reference's UE4-style GGX +
// Lambert model (src/cudaRTCommon.cu:284-365) and GetShadingResult
// (src/cudaRTBDPTStream.cu:642-663), in the float contract of gbpt_math.cuh.
#pragma once
#include "gbpt_math.cuh"

namespace gbpt {
using gb::f3;
using gb::mk;

// ProbabilityRand (src/cudaRTCommon.cu:284-291); u is this decision's uniform.
__device__ __forceinline__ bool prob_rand(float prob, float u) {
  if (prob < gb::kLtEps4) return false;
  if (prob >= gb::kProbOne) return true;
  return u < prob;
}

// Vis_SmithJointApprox with k = r^2/2 (:299-307)
__device__ __forceinline__ float vis_smith(float r, float NoV, float NoL) {
  float k = (r * r) / 2.0f;
  return (NoV / (NoV * (1.f - k) + k)) * (NoL / (NoL * (1.f - k) + k));
}

// D_GGX with m = r^2 (:309-315)
__device__ __forceinline__ float d_ggx(float r, float NoH) {
  float m = r * r;
  float m2 = m * m;
  float d = (NoH * m2 - NoH) * NoH + 1.f;
  return m2 / ((gb::kPi * d) * d);
}

// F_Schlick with the saturate(50 * F0.z) term (:317-322)
__device__ __forceinline__ f3 f_schlick(f3 s, float VoH) {
  float Fc = gb::pow5(1.f - VoH);
  float x = 50.f * s.z;
  float first = ((x < 0.f) ? 0.f : (x > 1.f) ? 1.f : x) * Fc;
  return mk(first, first, first) + (1.f - Fc) * s;
}

// Tangent frame used by ImportanceSampleGGX (:338-341) and the cosine lobe.
__device__ __forceinline__ void frame(f3 w, f3& u, f3& v) {
  f3 a = (fabsf(w.x) >= gb::kPointOne) ? mk(0.f, 1.f, 0.f) : mk(1.f, 0.f, 0.f);
  u = gb::normalize(gb::cross(a, w));
  v = gb::cross(w, u);
  u = gb::cross(v, w);
}

// ImportanceSampleGGX (:324-345); the angle 2*pi*xi is a float product.
__device__ __forceinline__ f3 ggx_sample(float xi0, float xi1, float r, f3 N) {
  float a = r * r;
  float phi = gb::kTwoPi * xi0;
  float cosT = sqrtf((1.f - xi1) / (1.f + (a * a - 1.f) * xi1));
  float sinT = sqrtf(1.f - cosT * cosT);
  float sp, cp;
  gb::sincos_p(phi, &sp, &cp);
  f3 u, v;
  frame(N, u, v);
  return (u * (sinT * cp) + v * (sinT * sp)) + N * cosT;
}

// Diffuse lobe of pt_traceSample_kernel (src/cudaRTBDPTStream.cu:481-489):
// r2sin = 1 - r2cos^2 as in the reference.
__device__ __forceinline__ f3 cos_dir(float u4, float u5, f3 w) {
  f3 u, v;
  frame(w, u, v);
  float r1 = gb::kTwoPi * u4;
  float r2cos = sqrtf(u5);
  float r2sin = 1.f - r2cos * r2cos;
  float sp, cp;
  gb::sincos_p(r1, &sp, &cp);
  return gb::normalize((w * r2cos + (u * r2sin) * cp) + (v * r2sin) * sp);
}

// GetShadingResult (src/cudaRTBDPTStream.cu:642-663)
__device__ __forceinline__ f3 shading(f3 V, f3 L, f3 irrad, f3 N, f3 diff, float metallic, float rough, float specular,
                                      float dsx, float dsy) {
  using namespace gb;
  if (dot(N, L) <= 0.f) return mk(0.f, 0.f, 0.f);
  f3 h = normalize(V + L);
  float voH = dot(V, h);
  float noV = dot(N, V);
  float noH = dot(N, h);
  float noL = dot(N, L);
  float s = kF0Spec * specular;
  f3 f0 = vlerp(mk(s, s, s), diff, metallic);
  f3 F = f_schlick(f0, voH);
  float dd = d_ggx(rough, noH);
  float vis = vis_smith(rough, noV, noL);
  f3 specI = F * (dd * vis);
  f3 diffI = vmul(mk(1.f, 1.f, 1.f) - F, diff * kInvPi);
  return vmul(irrad * noL, specI * dsy + diffI * dsx);
}

}  // namespace gbpt
