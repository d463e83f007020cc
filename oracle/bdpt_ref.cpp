// TEST INFRASTRUCTURE ONLY -- CPU oracle: CudaPT's streaming BDPT estimator,
// one path at a time.
//
//   src/cudaRTBDPTStream.cu:180-363   pt_traceLight_kernel   -> light_bounce
//   src/cudaRTBDPTStream.cu:365-543   pt_traceSample_kernel  -> eye_path (loop)
//   src/cudaRTBDPTStream.cu:545-617   pt_genLightPathQueue_kernel -> light_pass
//   src/cudaRTBDPTStream.cu:619-640   pt_genPathQueue_kernel -> camera_ray
//   src/cudaRTBDPTStream.cu:642-723   GetShadingResult / connection
//   src/cudaRTBDPTStream.cu:741-778   pt_applyPathQueueResult_kernel -> apply
//   src/cudaRTBDPTStream.cu:816-951   Render (frame counter, light pass every 3rd frame)
//   src/cudaRTCommon.cu:284-365       ProbabilityRand and the shading helpers
//   src/cudaRTBDPTStreamAdapBilatAtomic.cu:583, 650-655, 817-842, 1041-1156, 1253-1554
//                                     adaptive variant (spec push, G-buffer, budget)
//
// The wavefront order of the reference (stream compaction between bounces)
// does not change any path's result: every path owns its random numbers and
// the light-vertex cache is fixed during the eye pass.  Only the light pass
// depends on compaction order (cache slots are handed out in stream order
// after a stable remove_if), and that order is reproduced here.
//
// Random numbers: Philox4x32-10 with the counter layout of philox_ref.h in
// place of curand XORWOW (which cannot be reproduced bit for bit anyway).
// Per eye bounce: u0,u1 GGX sample, u2 reflect choice, u3 transmit choice,
// u4,u5 diffuse direction, u6 Russian roulette, u7 light-vertex pick.
//
// FP32 follows the float contract of fmath_ref.h.  Double literals of the
// reference's shading code (M_PI, 0.08, M_FLT_BIAS_EPSILON ...) are rounded
// to float first, and the one double-precision expression the reference
// evaluates per sample (2*M_PI*xi) is evaluated as float(2*pi)*xi.
#include "bdpt_ref.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <thread>

#include "fmath_ref.h"
#include "philox_ref.h"

namespace orc {

namespace {

enum RayType : uint32_t { kEye = 0, kDiff = 1, kSpec = 2, kLight = 3 };

template <typename R>
struct V {
  R x, y, z;
};
template <typename R>
static inline V<R> mkv(R x, R y, R z) {
  return V<R>{x, y, z};
}
template <typename R>
static inline V<R> ld(const float* p) {
  return mkv<R>((R)p[0], (R)p[1], (R)p[2]);
}
template <typename R>
static inline void st(float* p, V<R> a) {
  p[0] = (float)a.x;
  p[1] = (float)a.y;
  p[2] = (float)a.z;
}
template <typename R>
static inline V<R> operator+(V<R> a, V<R> b) {
  return mkv<R>(a.x + b.x, a.y + b.y, a.z + b.z);
}
template <typename R>
static inline V<R> operator-(V<R> a, V<R> b) {
  return mkv<R>(a.x - b.x, a.y - b.y, a.z - b.z);
}
template <typename R>
static inline V<R> operator*(V<R> a, R s) {
  return mkv<R>(a.x * s, a.y * s, a.z * s);
}
template <typename R>
static inline V<R> operator*(R s, V<R> a) {
  return a * s;
}
template <typename R>
static inline V<R> operator/(V<R> a, R s) {
  return mkv<R>(a.x / s, a.y / s, a.z / s);
}
template <typename R>
static inline V<R> operator/(V<R> a, V<R> b) {
  return mkv<R>(a.x / b.x, a.y / b.y, a.z / b.z);
}
template <typename R>
static inline V<R> vmulv(V<R> a, V<R> b) {
  return mkv<R>(a.x * b.x, a.y * b.y, a.z * b.z);
}
template <typename R>
static inline V<R> vmaxv(V<R> a, V<R> b) {
  return mkv<R>(std::fmax(a.x, b.x), std::fmax(a.y, b.y), std::fmax(a.z, b.z));
}
template <typename R>
static inline R dotv(V<R> l, V<R> r) {
  return std::fma(l.x, r.x, std::fma(l.y, r.y, l.z * r.z));
}
template <typename R>
static inline V<R> crossv(V<R> l, V<R> r) {
  return mkv<R>(std::fma(l.y, r.z, -(l.z * r.y)), std::fma(l.z, r.x, -(l.x * r.z)), std::fma(l.x, r.y, -(l.y * r.x)));
}
static inline float lenR(V<float> a) { return sqrt_rd(a.x * a.x + a.y * a.y + a.z * a.z); }
static inline double lenR(V<double> a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
template <typename R>
static inline V<R> normv(V<R> a) {
  return a / lenR(a);
}
template <typename R>
static inline V<R> lerpv(V<R> x, V<R> y, R d) {
  return x + (y - x) * d;
}
template <typename R>
static inline R lerpR(R x, R y, R d) {
  return x + (y - x) * d;
}
static inline void sincosR(float x, float* s, float* c) { sincos_p(x, s, c); }
static inline void sincosR(double x, double* s, double* c) {
  *s = std::sin(x);
  *c = std::cos(x);
}
static inline float pow5R(float x) { return pow5(x); }
static inline double pow5R(double x) { return std::pow(x, 5.0); }
template <typename R>
static inline R sat(R x) {
  return (x < (R)0) ? (R)0 : (x > (R)1) ? (R)1 : x;
}

template <typename R>
struct K {
  static constexpr R pi = (R)3.14159265358979323846264338327950288;
  static constexpr R inv_pi = (R)(1.0 / 3.14159265358979323846264338327950288);
  static constexpr R two_pi = (R)(2.0 * 3.14159265358979323846264338327950288);
  static constexpr R bias = (R)1E-4;  // M_FLT_BIAS_EPSILON
  static constexpr R fltEps = (R)1E-5;  // M_FLT_EPSILON
  static constexpr R f0s = (R)0.08;
  static constexpr R inf = (R)1E20;
};

// ---- shading helpers, src/cudaRTCommon.cu:284-365 -------------------------
template <typename R>
static inline bool prob_rand(R prob, float u) {  // ProbabilityRand, :284-291
  if ((double)prob < 1E-4) return false;
  if ((double)prob + 1E-4 > 1.0) return true;
  return (R)u < prob;
}
template <typename R>
static inline R vis_smith(R rough, R NoV, R NoL) {  // :299-307
  R k = (rough * rough) / (R)2;
  return (NoV / (NoV * ((R)1 - k) + k)) * (NoL / (NoL * ((R)1 - k) + k));
}
template <typename R>
static inline R d_ggx(R rough, R NoH) {  // :309-315
  R m = rough * rough;
  R m2 = m * m;
  R d = (NoH * m2 - NoH) * NoH + (R)1;
  return m2 / ((K<R>::pi * d) * d);
}
template <typename R>
static inline V<R> f_schlick(V<R> s, R VoH) {  // :317-322
  R Fc = pow5R((R)1 - VoH);
  R first = sat((R)50 * s.z) * Fc;
  return mkv<R>(first, first, first) + ((R)1 - Fc) * s;
}
// |w.x| > .1 with the double literal: for floats this is |w.x| >= 0.1f.
template <typename R>
static inline void basis(V<R> w, V<R>* u, V<R>* v) {
  V<R> a = ((double)std::fabs(w.x) > 0.1) ? mkv<R>(0, 1, 0) : mkv<R>(1, 0, 0);
  *u = normv(crossv(a, w));
  *v = crossv(w, *u);
  *u = crossv(*v, w);
}
template <typename R>
static inline V<R> ggx_sample(R xi0, R xi1, R rough, V<R> N) {  // :324-345
  R a = rough * rough;
  R phi = K<R>::two_pi * xi0;
  R cosT = std::sqrt(((R)1 - xi1) / ((R)1 + (a * a - (R)1) * xi1));
  R sinT = std::sqrt((R)1 - cosT * cosT);
  R sp, cp;
  sincosR(phi, &sp, &cp);
  V<R> H = mkv<R>(sinT * cp, sinT * sp, cosT);
  V<R> u, v;
  basis(N, &u, &v);
  return (u * H.x + v * H.y) + N * H.z;
}
template <typename R>
static inline V<R> cos_dir(R u4, R u5, V<R> w) {
  V<R> u, v;
  basis(w, &u, &v);
  R r1 = K<R>::two_pi * u4;
  R r2cos = std::sqrt(u5);
  R r2sin = (R)1 - r2cos * r2cos;
  R sp, cp;
  sincosR(r1, &sp, &cp);
  return normv((w * r2cos + (u * r2sin) * cp) + (v * r2sin) * sp);
}

// GetShadingResult, src/cudaRTBDPTStream.cu:642-663
template <typename R>
static inline V<R> shading(V<R> Vd, V<R> L, V<R> irrad, V<R> N, V<R> diff, R metallic, R rough, R specular, R dsx,
                           R dsy) {
  if (dotv(N, L) <= (R)0) return mkv<R>(0, 0, 0);
  V<R> h = normv(Vd + L);
  R voH = dotv(Vd, h);
  R noV = dotv(N, Vd);
  R noH = dotv(N, h);
  R noL = dotv(N, L);
  R s = K<R>::f0s * specular;
  V<R> f0 = lerpv(mkv<R>(s, s, s), diff, metallic);
  V<R> F = f_schlick(f0, voH);
  R d = d_ggx(rough, noH);
  R vis = vis_smith(rough, noV, noL);
  V<R> specI = F * (d * vis);
  V<R> diffI = vmulv(mkv<R>(1, 1, 1) - F, diff * K<R>::inv_pi);
  return vmulv(irrad * noL, specI * dsy + diffI * dsx);
}

struct MatV {
  const RTMaterial* m;
};

// diff / emissive / trans: GetMaterialColors (src/cudaRTCommon.cu:369-406)
// at the hit's uv = ((uv0*w) + (uv1*u)) + uv2*v (the reference's float2
// operators, src/cudaRTBDPTStream.cu:379-382): a diffuse texture replaces the
// diffuse colour and scales the transparency by its alpha, an emissive
// texture replaces the emissive colour (texture_ref.h).
template <typename R>
struct HitShade {
  V<R> norm, triPos;
  const RTMaterial* mat;
  V<R> diff, emissive;
  R trans;
};

template <typename R>
static inline void mat_colors(const std::vector<Texture>& texs, const RTMaterial& m, R tu, R tv, V<R>& diff,
                              V<R>& emissive, R& trans) {
  diff = ld<R>(m.diffuse);
  emissive = ld<R>(m.emissive);
  trans = (R)m.transparency;
  R tx[4];
  if (m.diffuseTexId >= 0 && (size_t)m.diffuseTexId < texs.size()) {
    tex_bilinear<R>(texs[(size_t)m.diffuseTexId], tu, tv, tx);
    diff = mkv<R>(tx[0], tx[1], tx[2]);
    trans = tx[3] * trans;
  }
  if (m.emissiveTexId >= 0 && (size_t)m.emissiveTexId < texs.size()) {
    tex_bilinear<R>(texs[(size_t)m.emissiveTexId], tu, tv, tx);
    emissive = mkv<R>(tx[0], tx[1], tx[2]);
  }
}

template <typename R>
static inline HitShade<R> hit_shade(const Scene& s, int32_t triId, R w, R u, R v) {
  const RTTriangle& t = s.tris[(uint32_t)triId];
  const RTVertex& a = s.verts[t.v0];
  const RTVertex& b = s.verts[t.v1];
  const RTVertex& c = s.verts[t.v2];
  HitShade<R> h;
  h.norm = (ld<R>(a.norm) * w + ld<R>(b.norm) * u) + ld<R>(c.norm) * v;
  h.triPos = (ld<R>(a.pos) * w + ld<R>(b.pos) * u) + ld<R>(c.pos) * v;
  h.mat = &s.mats[t.mat];
  const RTMaterial& m = *h.mat;
  R tu = 0, tv = 0;
  if (m.diffuseTexId >= 0 || m.emissiveTexId >= 0) {
    tu = ((R)a.tex[0] * w + (R)b.tex[0] * u) + (R)c.tex[0] * v;
    tv = ((R)a.tex[1] * w + (R)b.tex[1] * u) + (R)c.tex[1] * v;
  }
  mat_colors<R>(s.textures, m, tu, tv, h.diff, h.emissive, h.trans);
  return h;
}

}  // namespace

// GetMaterialColors' colour outputs for one material at n uvs: 8 floats each
// (diffuse rgb, emissive rgb, transparency, 0).
void material_colors(const std::vector<Texture>& texs, const RTMaterial& m, const float* uv, uint32_t n, float* out) {
  for (uint32_t i = 0; i < n; i++) {
    V<float> d, e;
    float tr;
    mat_colors<float>(texs, m, uv[2 * i], uv[2 * i + 1], d, e, tr);
    float* o = out + 8 * (size_t)i;
    o[0] = d.x; o[1] = d.y; o[2] = d.z;
    o[3] = e.x; o[4] = e.y; o[5] = e.z;
    o[6] = tr;
    o[7] = 0.f;
  }
}

namespace {

// double-precision walk of the same tree (FP64 mode only)
struct HitD {
  double dist, w, u, v;
  int32_t triId;
};
static bool trace_d(const Scene& s, V<double> o, V<double> d, double maxDist, double eps, HitD* hit, bool anyHit) {
  auto ez = [](double x) {
    double r = x;
    if (std::fabs(r) < 1E-9) r = (r > 0) ? r + 1E-9 : r - 1E-9;
    return r;
  };
  V<double> inv = mkv<double>(1.0 / ez(d.x), 1.0 / ez(d.y), 1.0 / ez(d.z));
  double best = maxDist;
  int32_t bestId = -1;
  double bw = 0, bu = 0, bv = 0;
  uint32_t stack[32];
  stack[0] = 0;
  int sp = 0;
  uint32_t steps = 0;
  const uint32_t nodeN = s.bvh.nodeN, triN = (uint32_t)s.tris.size();
  while (sp >= 0 && steps++ < 2048) {
    uint32_t cur = stack[sp--];
    double mn[3] = {0, 0, 0}, mx[3] = {0, 0, 0};
    uint32_t off = 0, tn = 0;
    if (cur < nodeN) {
      for (int k = 0; k < 3; k++) {
        mn[k] = s.bvh.bounds[(size_t)cur * 6 + k];
        mx[k] = s.bvh.bounds[(size_t)cur * 6 + 3 + k];
      }
      off = s.bvh.offOrTSTN[(size_t)cur * 2];
      tn = s.bvh.offOrTSTN[(size_t)cur * 2 + 1];
    }
    double o3[3] = {o.x, o.y, o.z}, i3[3] = {inv.x, inv.y, inv.z};
    double tmin = -1e300, tmax = 1e300;
    for (int k = 0; k < 3; k++) {
      double a = (mn[k] - o3[k]) * i3[k], b = (mx[k] - o3[k]) * i3[k];
      tmin = std::max(tmin, std::min(a, b));
      tmax = std::min(tmax, std::max(a, b));
    }
    double tb = 1E20;
    if (tmax >= tmin && (tmax > 0 || tmin > 0)) tb = (tmin > 1E-9) ? tmin : 0;
    if (!(tb >= 0 && tb < best)) continue;
    if (tn == 0) {
      if (sp < 29) {
        stack[++sp] = cur + 1;
        stack[++sp] = cur + off;
      }
      continue;
    }
    for (uint32_t i = off; i < off + tn; i++) {
      if (i >= triN) continue;
      const float* q = &s.isect[(size_t)i * 9];
      V<double> p0 = ld<double>(q), e0 = ld<double>(q + 3), e1 = ld<double>(q + 6);
      V<double> de2 = crossv(d, e1);
      double div = dotv(de2, e0);
      if (std::fabs(div) < 1E-9) continue;
      div = 1.0 / div;
      V<double> t = (o + d * eps) - p0;
      V<double> te1 = crossv(t, e0);
      double rT = dotv(te1, e1) * div;
      if (rT < 0) continue;
      double u = dotv(de2, t) * div;
      if (u < 0 || u > 1) continue;
      double v = dotv(te1, d) * div;
      if (v < 0 || u + v > 1) continue;
      if (rT < best) {
        best = rT;
        bestId = (int32_t)i;
        bw = 1 - u - v;
        bu = u;
        bv = v;
        if (anyHit) {
          hit->dist = best;
          return true;
        }
      }
    }
  }
  if (best < maxDist && bestId >= 0) {
    hit->dist = best;
    hit->triId = bestId;
    hit->w = bw;
    hit->u = bu;
    hit->v = bv;
    return true;
  }
  return false;
}

template <typename R>
struct HitR {
  R dist, w, u, v;
  int32_t triId;
};
static bool traceR(const Scene& s, V<float> o, V<float> d, float maxDist, HitR<float>* h, bool anyHit,
                   TraceCount* cnt) {
  (void)anyHit;  // closest-hit walk gives the same visibility answer (same walk up to the first hit)
  float of[3] = {o.x, o.y, o.z}, df[3] = {d.x, d.y, d.z};
  Hit hh;
  bool r = trace_primitive(s, of, df, maxDist, K<float>::bias, false, &hh, cnt);
  if (r) {
    h->dist = hh.dist;
    h->w = hh.w;
    h->u = hh.u;
    h->v = hh.v;
    h->triId = hh.triId;
  }
  return r;
}
static bool traceR(const Scene& s, V<double> o, V<double> d, double maxDist, HitR<double>* h, bool anyHit,
                   TraceCount* cnt) {
  (void)cnt;
  HitD hd;
  bool r = trace_d(s, o, d, maxDist, 1E-4, &hd, anyHit);
  if (r) {
    h->dist = hd.dist;
    h->w = hd.w;
    h->u = hd.u;
    h->v = hd.v;
    h->triId = hd.triId;
  }
  return r;
}

// ---- eye path: pt_traceSample_kernel loop + connections ---------------------
template <typename R>
//
// bilat: the filter-only variant's extra per-path outputs
// (src/cudaRTBDPTStreamBilat.cu:472-671, :884-915): the sampling density
// product ("path potential", :515-518 and per branch :560/:575/:599, :627),
// the direct-light sample (pathSample added at bounces 0 and 1, :628-631; the
// bounce-0 connection's light L turns it into (direct + L)/5, or L/4 when no
// channel is positive, :907-913) and the first-hit emissive (:636).
//
// pt: the unidirectional "PTSC" path of src/cudaRTPTStream.cu:91-258 -- no
// connections, total internal reflection reflects (cos2t < 0 sets reflProb =
// 1, :153-160), depth cap pt_depth_max.
static void eye_path(const Scene& s, const Params& p, const LightVertex* cache, uint32_t cacheSize, V<R> orig,
                     V<R> dir, uint32_t pathId, uint32_t frame, uint32_t sample, bool specPush, bool bilat,
                     bool pt, PathResult* out) {
  V<R> outMul = mkv<R>(1, 1, 1), pathSample = mkv<R>(0, 0, 0), acc = mkv<R>(0, 0, 0);
  V<R> direct = mkv<R>(0, 0, 0);
  R pot = (R)1;
  uint32_t n = 0, depth = 0;
  TraceCount cnt, cntS;  // extension walks, connection (shadow) walks
  uint32_t rays = 0, extRays = 0;
  for (int k = 0; k < 3; k++) out->gpos[k] = out->gnorm[k] = out->gdiff[k] = out->gemis[k] = 0;
  const R bias = K<R>::bias;
  while (true) {
    HitR<R> hit;
    rays++;
    extRays++;
    if (!traceR(s, orig, dir, K<R>::inf, &hit, false, &cnt)) {
      // miss: optional constant environment, then accumulate and stop
      if (p.env[0] != 0.f || p.env[1] != 0.f || p.env[2] != 0.f)
        pathSample = pathSample + vmulv(mkv<R>((R)p.env[0], (R)p.env[1], (R)p.env[2]), outMul);
      acc = acc + pathSample;
      n++;
      out->pot = (double)pot;
      break;
    }
    float u[8];
    draw8(p.seed, p.request_id, pathId, frame, kEyeBounce, depth, sample, u);
    HitShade<R> hs = hit_shade<R>(s, hit.triId, hit.w, hit.u, hit.v);
    const RTMaterial& m = *hs.mat;
    V<R> diff = hs.diff, emissive = hs.emissive;
    R trans = hs.trans, specular = (R)m.specular, metallic = (R)m.metallic, rough = (R)m.roughness;
    V<R> norm = hs.norm;
    V<R> nl = dotv(norm, dir) < (R)0 ? norm : (R)-1 * norm;
    V<R> hDir = ggx_sample<R>((R)u[0], (R)u[1], rough, nl);
    V<R> ndir = (R)-1 * dir;
    R voH = dotv(ndir, hDir);
    V<R> f0 = lerpv(K<R>::f0s * mkv<R>(specular, specular, specular), diff, metallic);
    V<R> F = f_schlick(f0, voH);
    R pdf = (R)1;
    if (bilat) {
      R NoH0 = dotv(nl, hDir);
      pdf = (d_ggx(rough, NoH0) * NoH0) / ((R)4 * voH);
    }
    R reflProb = lerpR(lenR(F), (R)1, metallic);
    R refrProb = trans;
    V<R> reflDir = mkv<R>(0, 0, 0), refrDir = mkv<R>(0, 0, 0);
    if (refrProb > (R)0) {
      bool into = dotv(nl, norm) > (R)0;
      R nt = specular * (R)0.8 + (R)1;
      R nc = (R)1;
      R nnt = into ? nc / nt : nt / nc;
      R ddn = dotv(hDir, dir);
      R cos2t = (R)1 - (nnt * nnt) * ((R)1 - ddn * ddn);
      if (pt && cos2t < (R)0)
        reflProb = (R)1;
      else
        refrDir = normv(dir * nnt - hDir * (ddn * nnt + std::sqrt(cos2t)));
    }
    if (reflProb > (R)0) {
      reflDir = normv(dir - (hDir * (R)2) * dotv(hDir, dir));
      if (dotv(reflDir, nl) < (R)0) reflProb = (R)0;
    }
    V<R> nOrig, nDir, lmt;
    uint32_t nType;
    if (prob_rand(reflProb, u[2])) {
      nOrig = orig + (hit.dist - bias) * dir;
      if (specPush) nOrig = nOrig + reflDir * bias;
      nDir = reflDir;
      R VoH = dotv(ndir, hDir);
      R NoV = dotv(nl, ndir);
      R NoH = dotv(nl, hDir);
      R NoL = dotv(nl, reflDir);
      R G = vis_smith(rough, NoV, NoL);
      lmt = ((F * G) * VoH) / ((NoV * NoH) * reflProb);
      nType = kSpec;
      pdf = pdf * reflProb;
    } else if (prob_rand(refrProb, u[3])) {
      nOrig = (orig + (hit.dist + bias) * dir) + refrDir * bias;
      nDir = refrDir;
      R cosine = dotv((R)-1 * nl, refrDir);
      lmt = (cosine * diff) / (refrProb * ((R)1 - reflProb));
      nType = kSpec;
      pdf = pdf * (refrProb * ((R)1 - reflProb));
    } else {
      V<R> dd = cos_dir<R>((R)u[4], (R)u[5], nl);
      nOrig = (orig + hit.dist * dir) + dd * bias;
      nDir = dd;
      lmt = (K<R>::pi * (diff * K<R>::inv_pi)) / (((R)1 - refrProb) * ((R)1 - reflProb));
      nType = kDiff;
      pdf = pdf * ((((R)1 - refrProb) * ((R)1 - reflProb)) * dotv(dd, nl));
    }
    pathSample = pathSample + vmulv(emissive, outMul);
    if (depth == 0) {  // G-buffer, AdapBilatAtomic.cu:471-476
      out->gpos[0] = (double)hs.triPos.x;
      out->gpos[1] = (double)hs.triPos.y;
      out->gpos[2] = (double)hs.triPos.z;
      out->gnorm[0] = (double)nl.x;
      out->gnorm[1] = (double)nl.y;
      out->gnorm[2] = (double)nl.z;
      out->gdiff[0] = (double)diff.x;
      out->gdiff[1] = (double)diff.y;
      out->gdiff[2] = (double)diff.z;
      out->gemis[0] = (double)emissive.x;
      out->gemis[1] = (double)emissive.y;
      out->gemis[2] = (double)emissive.z;
    }
    if (bilat) {
      pot = pot * pdf;
      if (depth < 2) direct = direct + pathSample;
    }
    V<R> inMul = outMul;
    R contrib = lenR(outMul) * lenR(lmt);
    if (lenR(emissive) > (R)0) contrib = (R)0;
    if ((R)u[6] > contrib || depth + 1 >= (pt ? p.pt_depth_max : p.eye_depth_max)) {
      acc = acc + pathSample;
      n++;
      out->pot = (double)pot;
      break;
    }
    outMul = vmulv(outMul, lmt);
    dir = nDir;
    depth++;
    orig = nOrig;
    if (nType != kDiff || pt) continue;
    // ---- connection to a cached light vertex (:665-723) ----
    if (cacheSize == 0) continue;
    V<R> pos = orig + nl * bias;
    uint32_t li = (uint32_t)(u[7] * (float)cacheSize);
    if (li >= cacheSize) li = cacheSize - 1;
    const LightVertex& lv = cache[li];
    V<R> lpos = ld<R>(lv.pos);
    V<R> toDir = normv(lpos - pos);
    R toDist = lenR(lpos - pos);
    V<R> irrad = mkv<R>(0, 0, 0), irradDir = mkv<R>(0, 0, 0);
    if (lenR(ld<R>(lv.irrad)) > (R)0 && dotv(nl, toDir) > (R)0) {
      HitR<R> sh;
      rays++;
      if (!traceR(s, pos, toDir, toDist - bias, &sh, true, &cntS)) {
        if (toDist > K<R>::fltEps) {
          irrad = shading<R>((R)-1 * toDir, ld<R>(lv.irradDir), ld<R>(lv.irrad), ld<R>(lv.norm), ld<R>(lv.diff),
                             (R)lv.metallic, (R)lv.roughness, (R)lv.specular, (R)1, (R)1) +
                  ld<R>(lv.emissive);
          irradDir = toDir;
        } else {
          irrad = ld<R>(lv.irrad);
          irradDir = (R)-1 * ld<R>(lv.irradDir);
        }
      }
    }
    V<R> c = vmaxv(mkv<R>(0, 0, 0), shading<R>(ndir, irradDir, irrad, nl, diff, metallic, rough, specular,
                                                  (R)1 - trans, (R)1));
    if (lenR(c) > (R)0) {
      acc = acc + vmulv(c, inMul);
      n += 4;
      if (bilat && depth <= 1) {
        V<R> L = vmulv(c, inMul);
        direct = (direct.x > (R)0 || direct.y > (R)0 || direct.z > (R)0) ? (direct + L) / (R)5 : L / (R)4;
      }
    }
  }
  out->direct[0] = (double)direct.x;
  out->direct[1] = (double)direct.y;
  out->direct[2] = (double)direct.z;
  out->acc[0] = (double)acc.x;
  out->acc[1] = (double)acc.y;
  out->acc[2] = (double)acc.z;
  out->n = n;
  out->rays = rays;
  out->nodes = cnt.nodes + cntS.nodes;
  out->tris = cnt.tris + cntS.tris;
  out->extRays = extRays;
  out->extNodes = cnt.nodes;
  out->extTris = cnt.tris;
}

// ---- light pass: pt_genLightPathQueue_kernel + pt_traceLight_kernel --------
struct LPath {
  V<float> orig, dir, outMul, sample;
  uint32_t home, depth, type, id;
};

static void light_pass_f(const Scene& s, const Params& p, uint32_t frame, std::vector<LightVertex>& cache,
                         uint32_t* cacheSize) {
  const uint32_t NL = p.light_paths;
  cache.assign((size_t)NL * (1 + p.light_depth_max), LightVertex{});
  *cacheSize = 0;
  if (s.lightTri.empty() || NL == 0) return;
  const uint32_t nLight = (uint32_t)s.lightTri.size();
  std::vector<LPath> stream;
  for (uint32_t x = 0; x < NL; x++) {
    float u[8];
    draw8(p.seed, p.request_id, x, frame, kLightGen, 0, 0, u);
    uint32_t id = (uint32_t)(u[0] * (float)nLight);
    if (id >= nLight) id = nLight - 1;
    float lw = u[1], lu = u[2];
    if (lw + lu > 1.0f) {
      lw = 1.f - lw;
      lu = 1.f - lu;
    }
    float lvv = 1.f - lw - lu;
    HitShade<float> hs = hit_shade<float>(s, (int32_t)s.lightTri[id], lw, lu, lvv);
    const RTMaterial& m = *hs.mat;
    V<float> dd = cos_dir<float>(u[3], u[4], hs.norm);
    LPath lp;
    lp.orig = hs.triPos + K<float>::bias * hs.norm;
    lp.dir = dd;
    lp.outMul = mkv<float>(1, 1, 1);
    lp.sample = hs.emissive;
    lp.home = x;
    lp.depth = 0;
    lp.type = kLight;
    lp.id = x;
    stream.push_back(lp);
    LightVertex& lv = cache[x];
    st(lv.irrad, hs.emissive);
    st(lv.irradDir, mkv<float>(0, 0, 0));
    st(lv.norm, hs.norm);
    st(lv.pos, hs.triPos);
    st(lv.diff, hs.diff);
    st(lv.emissive, hs.emissive);
    lv.specular = m.specular;
    lv.metallic = m.metallic;
    lv.roughness = m.roughness;
  }
  uint32_t size = NL;
  const float bias = K<float>::bias;
  while (!stream.empty()) {
    std::vector<LPath> next;
    for (uint32_t x = 0; x < stream.size(); x++) {
      LPath& lp = stream[x];
      LightVertex& slot = cache[size + x];
      HitR<float> hit;
      if (!traceR(s, lp.orig, lp.dir, K<float>::inf, &hit, false, nullptr)) {
        slot = cache[lp.home];  // :358-362
        continue;
      }
      float u[8];
      draw8(p.seed, p.request_id, lp.id, frame, kLightBounce, lp.depth, 0, u);
      HitShade<float> hs = hit_shade<float>(s, hit.triId, hit.w, hit.u, hit.v);
      const RTMaterial& m = *hs.mat;
      V<float> diff = hs.diff, emissive = hs.emissive;
      float trans = hs.trans, specular = m.specular, metallic = m.metallic, rough = m.roughness;
      V<float> norm = hs.norm, dir = lp.dir;
      V<float> nl = dotv(norm, dir) < 0.f ? norm : -1.f * norm;
      st(slot.irrad, lp.sample);
      st(slot.irradDir, -1.f * dir);
      st(slot.norm, nl);
      st(slot.pos, hs.triPos);
      st(slot.diff, diff);
      st(slot.emissive, emissive);
      slot.specular = specular;
      slot.metallic = metallic;
      slot.roughness = rough;
      V<float> hDir = ggx_sample<float>(u[0], u[1], rough, nl);
      V<float> ndir = -1.f * dir;
      float voH = dotv(ndir, hDir);
      V<float> f0 = lerpv(K<float>::f0s * mkv<float>(specular, specular, specular), diff, metallic);
      V<float> F = f_schlick(f0, voH);
      float reflProb = lerpR(lenR(F), 1.0f, metallic);
      float refrProb = trans;
      V<float> reflDir = mkv<float>(0, 0, 0), refrDir = mkv<float>(0, 0, 0);
      if (refrProb > 0.f) {
        bool into = dotv(nl, norm) > 0.f;
        float nt = specular * 0.8f + 1.f;
        float nnt = into ? 1.0f / nt : nt / 1.0f;
        float ddn = dotv(hDir, dir);
        float cos2t = 1.f - (nnt * nnt) * (1.f - ddn * ddn);
        refrDir = normv(dir * nnt - hDir * (ddn * nnt + std::sqrt(cos2t)));
      }
      if (reflProb > 0.f) {
        reflDir = normv(dir - (hDir * 2.f) * dotv(hDir, dir));
        if (dotv(reflDir, nl) < 0.f) reflProb = 0.f;
      }
      V<float> nOrig, nDir, lmt;
      uint32_t nType;
      if (prob_rand(reflProb, u[2])) {
        nOrig = lp.orig + (hit.dist - bias) * dir;
        nDir = reflDir;
        float VoH = dotv(ndir, hDir), NoV = dotv(nl, ndir), NoH = dotv(nl, hDir), NoL = dotv(nl, reflDir);
        float G = vis_smith(rough, NoV, NoL);
        lmt = ((F * G) * VoH) / ((NoV * NoH) * reflProb);
        nType = kSpec;
      } else if (prob_rand(refrProb, u[3])) {
        nOrig = (lp.orig + (hit.dist + bias) * dir) + refrDir * bias;
        nDir = refrDir;
        float cosine = dotv(-1.f * nl, refrDir);
        lmt = (cosine * diff) / (refrProb * (1.f - reflProb));
        nType = kSpec;
      } else {
        V<float> dd = cos_dir<float>(u[4], u[5], nl);
        nOrig = (lp.orig + hit.dist * dir) + dd * bias;
        nDir = dd;
        lmt = (K<float>::pi * (diff * K<float>::inv_pi)) / ((1.f - refrProb) * (1.f - reflProb));
        nType = kDiff;
      }
      if (nType != kDiff) st(slot.irrad, mkv<float>(0, 0, 0));
      if (dotv(nDir, nl) < 0.f) st(slot.norm, -1.f * nl);
      lp.sample = emissive + vmulv(lp.sample, lmt);
      float contrib = lenR(lp.outMul) * lenR(lmt);
      if (lenR(emissive) > 0.f) contrib = 0.f;
      if (u[6] > contrib || lp.depth + 1 >= p.light_depth_max) continue;
      lp.outMul = vmulv(lp.outMul, lmt);
      lp.dir = nDir;
      lp.orig = nOrig;
      lp.type = nType;
      lp.depth++;
      next.push_back(lp);  // stable compaction, as thrust::remove_if
    }
    size += (uint32_t)stream.size();
    stream.swap(next);
  }
  *cacheSize = size;
}

template <typename F>
static void parallel_rows(uint32_t H, uint32_t threads, F fn) {
  if (threads <= 1) {
    for (uint32_t y = 0; y < H; y++) fn(y);
    return;
  }
  std::vector<std::thread> th;
  std::atomic<uint32_t> next{0};
  for (uint32_t t = 0; t < threads; t++)
    th.emplace_back([&]() {
      for (;;) {
        uint32_t y = next.fetch_add(1);
        if (y >= H) break;
        fn(y);
      }
    });
  for (auto& t : th) t.join();
}

// host camera basis, src/cudaRTBDPTStream.cu:823-824 (Vec3 ops, no FMA)
static void cam_basis(const Camera& c, float right[3], float up[3]) {
  const float* d = c.dir;
  const float* u = c.up;
  float r[3] = {d[1] * u[2] - d[2] * u[1], d[2] * u[0] - d[0] * u[2], d[0] * u[1] - d[1] * u[0]};
  float l = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
  for (int k = 0; k < 3; k++) right[k] = r[k] / l;
  float q[3] = {right[1] * d[2] - right[2] * d[1], right[2] * d[0] - right[0] * d[2],
                right[0] * d[1] - right[1] * d[0]};
  l = std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2]);
  for (int k = 0; k < 3; k++) up[k] = q[k] / l;
}

struct CamF {
  float pos[3], dir[3], up[3], right[3], tanHalf, W, H;
};

// pt_genPathQueue_kernel, :619-640
template <typename R>
static void camera_ray(const CamF& c, uint32_t x, uint32_t y, float j0, float j1, V<R>* o, V<R>* d) {
  R W = (R)c.W, H = (R)c.H, th = (R)c.tanHalf;
  R u = (((((R)2 * ((R)x + (R)0.5)) / W) - (R)1) * th * W) / H;
  R v = ((((R)2 * ((R)y + (R)0.5)) / H) - (R)1) * th;
  R au = u + (((R)j0 - (R)0.5) / H) * th;
  R av = v + (((R)j1 - (R)0.5) / H) * th;
  *d = normv((ld<R>(c.right) * au + ld<R>(c.up) * av) + ld<R>(c.dir));
  *o = ld<R>(c.pos);
}

// running mean, pt_applyPathQueueResult_kernel :754-777 (float)
static void apply_mean(float* res, uint32_t* N, uint32_t ind, const double acc[3], uint32_t n, bool frame0,
                       float* g3[3], const double* gsrc[3]) {
  if (n == 0) return;
  if (frame0) N[ind] = 0;
  uint32_t nn = N[ind] + n;
  if (!(nn > N[ind])) return;
  float a[3] = {(float)acc[0], (float)acc[1], (float)acc[2]};
  if (std::isinf(a[0]) || std::isinf(a[1]) || std::isinf(a[2])) return;
  float rInf = 1.f / (float)nn;
  float oInf = (float)N[ind] * rInf;
  for (int k = 0; k < 3; k++) res[ind * 3 + k] = std::fmax(rInf * a[k] + oInf * res[ind * 3 + k], 0.f);
  N[ind] = nn;
  if (g3) {  // G-buffer running means weighted by the path's count (AdapBilatAtomic.cu:951-964)
    for (int b = 0; b < 3; b++)
      for (int k = 0; k < 3; k++) {
        float sv = (float)gsrc[b][k] * (float)n;
        g3[b][ind * 3 + k] = rInf * sv + oInf * g3[b][ind * 3 + k];
      }
  }
}

}  // namespace

void default_params(Params* p) {
  p->seed = 1234;
  p->eye_depth_max = 5;
  p->light_depth_max = 5;
  p->light_paths = 128;
  p->light_every = 3;
  p->env[0] = p->env[1] = p->env[2] = 0.f;
  p->warmup_frames = 5;
  p->desired_n = 5;
  p->filter_color_eud = 50.f;
  p->filter_pos_eud = 1.f;
  p->filter_norm_eud = 0.25f;
  p->filter_diff_eud = 0.1f;
  p->filter_radius = 5;
  p->filter_diffuse = 0;
  p->filter_sigma_spatial = 0.f;
  p->request_id = 0;
  p->min_trace_prob = 0.f;
  p->bilat_color_eud = 1.f;
  p->bilat_pos_eud = 1.f;
  p->bilat_norm_eud = 1.f;
  p->bilat_emit_eud = 0.5f;
  p->bilat_diff_eud = 0.5f;
  p->bilat_radius = 5;
  p->filter_iterations = 1;
  p->render_iterations = 5;
  p->pt_depth_max = 10;
}

void renderer_init(Renderer* r, uint32_t W, uint32_t H, int32_t mode, const Params& p, bool fp64, uint32_t threads) {
  r->W = W;
  r->H = H;
  r->mode = mode;
  r->p = p;
  r->fp64 = fp64;
  r->threads = threads ? threads : 1;
  r->frame = 0;
  r->started = false;
  size_t np = (size_t)W * H;
  r->result.assign(np * 3, 0.f);
  r->gpos.assign(np * 3, 0.f);
  r->gnorm.assign(np * 3, 0.f);
  r->gdiff.assign(np * 3, 0.f);
  r->filtered.assign(np * 3, 0.f);
  r->err.assign(np, 0.f);
  r->gemis.assign(np * 3, 0.f);
  r->direct.assign(np * 3, 0.f);
  r->pot.assign(np, 0.f);
  r->out.assign(np * 3, 0.f);
  r->sampleN.assign(np, 0u);
  r->counts.assign(np, 0u);
  r->cache.clear();
  r->cacheSize = 0;
}

void light_pass(Renderer* r, const Scene& s, uint32_t frame) { light_pass_f(s, r->p, frame, r->cache, &r->cacheSize); }

void gaussian_table(float delta, uint32_t radius, float* g) {  // src/cudaBilateralFilter.cu:5-24
  for (uint32_t i = 0; i < 2 * radius + 1; i++) {
    int x = (int)i - (int)radius;
    g[i] = exp_p((float)(-(x * x)) / (2 * delta * delta));
  }
}

// src/cudaBilateralFilter.cu:26-33
static inline float eucl(const float* a, const float* b, float d) {
  float dx = b[0] - a[0], dy = b[1] - a[1], dz = b[2] - a[2];
  float mod = dx * dx + dy * dy + dz * dz;
  return exp_p(-mod / (2.f * d * d));
}

// src/cudaBilateralFilter.cu:66-142.  Neighbour index uses the reference's
// unsigned arithmetic: x + j wraps for negative offsets, so umin/umax send
// taps left of column 0 (below row 0) to the last column (row).
void bilateral(const float* color, const float* pos, const float* norm, const float* emit, uint32_t W, uint32_t H,
               float colorEuD, float posEuD, float normEuD, float emitEuD, uint32_t radius, const float* g,
               float* out) {
  for (uint32_t y = 0; y < H; y++)
    for (uint32_t x = 0; x < W; x++) {
      uint32_t ind = x + y * W;
      float sum = 0.f;
      float t[3] = {0.f, 0.f, 0.f};
      const float* cc = color + ind * 3;
      const float* cp = pos + ind * 3;
      const float* cn = norm + ind * 3;
      const float* ce = emit ? emit + ind * 3 : nullptr;
      for (int i = -(int)radius; i <= (int)radius; i++)
        for (int j = -(int)radius; j <= (int)radius; j++) {
          uint32_t xx = std::min(W - 1, std::max(0u, x + (uint32_t)j));
          uint32_t yy = std::min(H - 1, std::max(0u, y + (uint32_t)i));
          uint32_t ci = xx + yy * W;
          const float* px = color + ci * 3;
          float f = g[i + radius] * g[j + radius] * eucl(px, cc, colorEuD) * eucl(pos + ci * 3, cp, posEuD) *
                    eucl(norm + ci * 3, cn, normEuD);
          if (ce) f = f * eucl(emit + ci * 3, ce, emitEuD);
          for (int k = 0; k < 3; k++) t[k] = t[k] + f * px[k];
          sum = sum + f;
        }
      for (int k = 0; k < 3; k++) out[ind * 3 + k] = t[k] / sum;
    }
}

template <typename R>
static void trace_pixels(Renderer* r, const Scene& s, const CamF& c, const std::vector<uint32_t>& pixOf,
                         const std::vector<uint32_t>& sampleOf, std::vector<PathResult>& res, bool specPush,
                         bool bilat = false, bool pt = false) {
  const uint32_t n = (uint32_t)pixOf.size();
  res.assign(n, PathResult{});
  const uint32_t W = r->W;
  // ~8 chunks per thread: small samples still use every core
  const uint32_t chunk = std::max<uint32_t>(64u, (n + r->threads * 8 - 1) / (r->threads * 8));
  uint32_t nchunks = (n + chunk - 1) / chunk;
  parallel_rows(nchunks, r->threads, [&](uint32_t ck) {
    uint32_t e = std::min(n, (ck + 1) * chunk);
    for (uint32_t i = ck * chunk; i < e; i++) {
      uint32_t smp = sampleOf[i];
      uint32_t x = pixOf[i] % W + r->x0, y = pixOf[i] / W + r->y0;
      uint32_t pix = y * (r->fullW ? r->fullW : W) + x;  // global pixel id (RNG stream)
      float u[8];
      draw8(r->p.seed, r->p.request_id, pix, r->frame, kCamera, 0, smp, u);
      V<R> o, d;
      camera_ray<R>(c, x, y, u[0], u[1], &o, &d);
      eye_path<R>(s, r->p, r->cache.data(), r->cacheSize, o, d, pix, r->frame, smp, specPush, bilat, pt, &res[i]);
    }
  });
}

// Filter-only mode ("BDPTSC Bilaterial", src/cudaRTBDPTStreamBilat.cu:1160-1461):
// while frame < "Render Iteration" (0: always) one path per pixel with the
// running means of pt_applyPathQueueResult_kernel (:989-1051: no inf test;
// direct light and 1 - potential as running means; first-hit planes are the
// frame's own), then the posnormemit filter with the diffuse plane as the
// third feature, "Filter Iteration" passes, and the debug view.  The "Prob"
// views filter max(minProb, mean potential) without overwriting the result
// (the reference writes that view into its accumulator, :933-940).
static void render_bilat(Renderer* r, const Scene& s, const CamF& c) {
  const uint32_t np = r->W * r->H;
  const uint32_t RI = r->p.render_iterations;
  r->lastPaths = r->lastRays = r->lastNodes = r->lastTris = 0;
  r->lastExt[0] = r->lastExt[1] = r->lastExt[2] = 0;
  if (RI == 0 || r->frame < RI) {
    if (r->frame % r->p.light_every == 0) light_pass(r, s, r->frame);
    std::vector<uint32_t> pixOf(np), sampleOf(np, 0u);
    for (uint32_t i = 0; i < np; i++) pixOf[i] = i;
    std::vector<PathResult> res;
    trace_pixels<float>(r, s, c, pixOf, sampleOf, res, false, true);
    r->lastPaths = res.size();
    for (auto& q : res) {
      r->lastRays += q.rays;
      r->lastNodes += q.nodes;
      r->lastTris += q.tris;
      r->lastExt[0] += q.extRays;
      r->lastExt[1] += q.extNodes;
      r->lastExt[2] += q.extTris;
    }
    const bool frame0 = r->frame == 0;
    for (uint32_t i = 0; i < np; i++) {
      const PathResult& q = res[i];
      if (q.n == 0) continue;
      if (frame0) r->sampleN[i] = 0;
      const uint32_t old = r->sampleN[i], nn = old + q.n;
      if (!(nn > old)) continue;
      const float rInf = 1.f / (float)nn, oInf = (float)old * rInf;
      for (int k = 0; k < 3; k++)
        r->result[i * 3 + k] = std::fmax(rInf * (float)q.acc[k] + oInf * r->result[i * 3 + k], 0.f);
      r->pot[i] = std::fmax(rInf * (1.f - (float)q.pot) + oInf * r->pot[i], 0.f);
      r->sampleN[i] = nn;
      for (int k = 0; k < 3; k++) {
        r->direct[i * 3 + k] = rInf * (float)q.direct[k] + oInf * r->direct[i * 3 + k];
        r->gpos[i * 3 + k] = (float)q.gpos[k];
        r->gnorm[i * 3 + k] = (float)q.gnorm[k];
        r->gemis[i * 3 + k] = (float)q.gemis[k];
        r->gdiff[i * 3 + k] = (float)q.gdiff[k];
      }
    }
  }
  float gt[64];
  const float delta = r->p.filter_sigma_spatial > 0.f ? r->p.filter_sigma_spatial : r->p.bilat_color_eud;
  gaussian_table(delta, r->p.bilat_radius, gt);
  std::vector<float> view;
  const float* src = r->result.data();
  const uint32_t dm = r->debug_mode;
  if (dm == 2 || dm == 3) {
    const float mp = dm == 3 ? r->p.min_trace_prob : 0.f;
    view.resize((size_t)np * 3);
    for (uint32_t i = 0; i < np; i++) view[i * 3] = view[i * 3 + 1] = view[i * 3 + 2] = std::fmax(mp, r->pot[i]);
    src = view.data();
  }
  const Params& p = r->p;
  bilateral(src, r->gpos.data(), r->gnorm.data(), r->gdiff.data(), r->W, r->H, p.bilat_color_eud, p.bilat_pos_eud,
            p.bilat_norm_eud, p.bilat_diff_eud, p.bilat_radius, gt, r->filtered.data());
  std::vector<float> tmp((size_t)np * 3);
  for (uint32_t it = 1; it < p.filter_iterations; it++) {
    bilateral(r->filtered.data(), r->gpos.data(), r->gnorm.data(), r->gdiff.data(), r->W, r->H, p.bilat_color_eud,
              p.bilat_pos_eud, p.bilat_norm_eud, p.bilat_diff_eud, p.bilat_radius, gt, tmp.data());
    r->filtered.swap(tmp);
  }
  const std::vector<float>& o = dm == 4 ? r->direct : dm == 5 ? r->gpos : dm == 6 ? r->gnorm
                                : dm == 7 ? r->result : r->filtered;
  r->out = o;
}

void render_frame(Renderer* r, const Scene& s, const Camera& cam) {
  CamF c;
  float right[3], up[3];
  cam_basis(cam, right, up);
  for (int k = 0; k < 3; k++) {
    c.pos[k] = cam.pos[k];
    c.dir[k] = cam.dir[k];
    c.up[k] = up[k];
    c.right[k] = right[k];
  }
  c.tanHalf = (float)std::tan((double)(cam.fov * 0.5f));
  c.W = (float)(r->fullW ? r->fullW : r->W);
  c.H = (float)(r->fullH ? r->fullH : r->H);
  float basis9[9] = {cam.pos[0], cam.pos[1], cam.pos[2], cam.dir[0], cam.dir[1], cam.dir[2], up[0], up[1], up[2]};
  bool same = r->started && std::equal(basis9, basis9 + 9, r->camBasis);
  r->frame = same ? r->frame + 1 : 0;
  std::copy(basis9, basis9 + 9, r->camBasis);
  r->started = true;
  const uint32_t np = r->W * r->H;
  if (r->mode == kModeBilat) {
    render_bilat(r, s, c);
    return;
  }
  if (r->mode == kModePT) {  // cudaRTPTStream::Render (src/cudaRTPTStream.cu:380-431): no light pass
    std::vector<uint32_t> pixOf(np), sampleOf(np, 0u);
    for (uint32_t i = 0; i < np; i++) pixOf[i] = i;
    std::vector<PathResult> res;
    trace_pixels<float>(r, s, c, pixOf, sampleOf, res, false, false, true);
    r->lastPaths = res.size();
    r->lastRays = r->lastNodes = r->lastTris = 0;
    r->lastExt[0] = r->lastExt[1] = r->lastExt[2] = 0;
    for (auto& q : res) {
      r->lastRays += q.rays;
      r->lastNodes += q.nodes;
      r->lastTris += q.tris;
      r->lastExt[0] += q.extRays;
      r->lastExt[1] += q.extNodes;
      r->lastExt[2] += q.extTris;
    }
    // pt_applyPathQueueResult_kernel (:335-358): frame-count weights, no inf test
    const float rInf = 1.f / (float)(r->frame + 1), oInf = 1.f - rInf;
    for (uint32_t i = 0; i < np; i++) {
      if (res[i].n == 0) continue;
      for (int k = 0; k < 3; k++) {
        const float smp = (float)res[i].acc[k] / (float)res[i].n;
        r->result[i * 3 + k] = std::fmax(rInf * smp + oInf * r->result[i * 3 + k], 0.f);
      }
      r->sampleN[i] = r->frame + 1;
    }
    return;
  }
  if (r->frame % r->p.light_every == 0) light_pass(r, s, r->frame);

  const bool adaptive = r->mode == kModeAdaptive || r->mode == kModeAdaptiveBinary;
  const bool binary = r->mode == kModeAdaptiveBinary;
  const bool frame0 = r->frame == 0;
  std::vector<uint32_t> pixOf, sampleOf;
  bool uniform = !adaptive || r->frame < r->p.warmup_frames;
  if (uniform) {
    pixOf.resize(np);
    sampleOf.assign(np, 0u);
    for (uint32_t i = 0; i < np; i++) pixOf[i] = i;
  } else {
    // filter -> per-pixel error -> budget (AdapBilatAtomic.cu:1409-1483)
    float gt[64];
    float delta = r->p.filter_sigma_spatial > 0.f ? r->p.filter_sigma_spatial : r->p.filter_color_eud;
    gaussian_table(delta, r->p.filter_radius, gt);
    bilateral(r->result.data(), r->gpos.data(), r->gnorm.data(), r->p.filter_diffuse ? r->gdiff.data() : nullptr,
              r->W, r->H, r->p.filter_color_eud, r->p.filter_pos_eud, r->p.filter_norm_eud, r->p.filter_diff_eud,
              r->p.filter_radius, gt, r->filtered.data());
    double sum = 0.0;
    const uint32_t D = r->p.desired_n;
    for (uint32_t i = 0; i < np; i++) {  // pt_calculateSquareError_kernel :1143-1156
      uint32_t sn = r->sampleN[i];
      float rf = (float)D / (float)(D + sn);
      if (D + sn < sn) rf = 0;
      const float* a = &r->filtered[i * 3];
      const float* b = &r->result[i * 3];
      float d0 = a[0] - b[0], d1 = a[1] - b[1], d2 = a[2] - b[2];
      r->err[i] = (rf * ((d0 * d0 + d1 * d1) + d2 * d2)) / 3.f;
      sum += (double)r->err[i];
    }
    float sumF = (float)sum;
    const uint32_t gen = np;
    uint64_t total = 0;
    if (binary) {
      // binary search of an acceptance scale (AdapBilatBinary.cu:1316-1384):
      // each pass accepts pixel p when u * mid <= max(e_p, minTraceProb),
      // appends the accepted pixels in pixel order, and halves the window
      // towards W*H/D accepted paths; leftover slots get pixel ids 0, 1, ...
      float maxE = 0.f;
      for (uint32_t i = 0; i < np; i++) maxE = (maxE < r->err[i]) ? r->err[i] : maxE;  // thrust::maximum
      float left = 0.f, right = maxE * 2.f;
      const float desired = (float)np / (float)D;
      uint32_t accum = 0;
      r->chunks.clear();
      for (uint32_t pass = 0; accum < gen && pass < 64; pass++) {
        const float mid = (left + right) * 0.5f;
        uint32_t take = 0;
        for (uint32_t i = 0; i < np && accum + take < gen; i++) {
          U4 rr = philox4x32_10(U4{{i, r->frame, (uint32_t)kBinaryAccept << 24, pass}}, r->p.seed, r->p.request_id);
          float th = std::fmax(r->err[i], r->p.min_trace_prob);
          if (!(u01(rr.v[0]) * mid > th)) {
            pixOf.push_back(i);
            sampleOf.push_back(pass);
            take++;
          }
        }
        r->chunks.push_back(take);
        accum += take;
        if (take == 0) break;
        if ((float)take < desired)
          right = mid;
        else if ((float)take > desired)
          left = mid;
      }
      if (accum < gen) {
        uint32_t fill = gen - accum;
        for (uint32_t k = 0; k < fill; k++) {
          pixOf.push_back(k);
          sampleOf.push_back((uint32_t)r->chunks.size());
        }
        r->chunks.push_back(fill);
      }
    }
    for (uint32_t i = 0; i < np && !binary; i++) {  // pt_genAdapPathQueue_kernel :817-842
      float ratio = r->err[i] / sumF;
      float v = (float)gen * ratio;
      uint32_t cnt = (v >= 1.f && v < 4294967040.f) ? (uint32_t)v : 0u;
      if (total + cnt > gen) cnt = (uint32_t)(gen - total);
      r->counts[i] = cnt;
      total += cnt;
      for (uint32_t k = 0; k < cnt; k++) {
        pixOf.push_back(i);
        sampleOf.push_back(k);
      }
    }
  }

  std::vector<PathResult> res;
  trace_pixels<float>(r, s, c, pixOf, sampleOf, res, r->mode == kModeAdaptive);  // spec push: PLL variant only
  r->lastPaths = res.size();
  r->lastRays = r->lastNodes = r->lastTris = 0;
  r->lastExt[0] = r->lastExt[1] = r->lastExt[2] = 0;
  for (auto& q : res) {
    r->lastRays += q.rays;
    r->lastNodes += q.nodes;
    r->lastTris += q.tris;
    r->lastExt[0] += q.extRays;
    r->lastExt[1] += q.extNodes;
    r->lastExt[2] += q.extTris;
  }
  float* g3[3] = {r->gpos.data(), r->gnorm.data(), r->gdiff.data()};
  if (!uniform && binary) {  // pt_applyPathQueueResult_kernel per pass, in pass order (:1396-1418)
    for (size_t k = 0; k < pixOf.size(); k++) {
      const double* gs[3] = {res[k].gpos, res[k].gnorm, res[k].gdiff};
      apply_mean(r->result.data(), r->sampleN.data(), pixOf[k], res[k].acc, res[k].n, frame0, g3, gs);
    }
    return;
  }
  if (uniform) {
    for (uint32_t i = 0; i < np; i++) {
      const double* gs[3] = {res[i].gpos, res[i].gnorm, res[i].gdiff};
      apply_mean(r->result.data(), r->sampleN.data(), i, res[i].acc, res[i].n, frame0, adaptive ? g3 : nullptr, gs);
    }
    return;
  }
  // per-pixel sums (pt_atomicApplyPathQueueResult_kernel :1041-1085, then
  // pt_accumTempResultToResult_kernel :1088-1141) in the library's fixed
  // order: P partials (partial l adds samples l, l+P, ...; P = 8 for up to 64
  // samples, 32 for up to 4096, 1024 above), then a butterfly
  // x[l] = x[l] + x[l^m] for m = P/2, ..., 1.
  size_t q = 0;
  std::vector<float> part, nxt;
  std::vector<uint32_t> pn, nn2;
  for (uint32_t i = 0; i < np; i++) {
    const uint32_t cnt = r->counts[i];
    const uint32_t P = cnt <= 64 ? 8u : cnt <= 4096 ? 32u : 1024u;
    part.assign((size_t)P * 12, 0.f);
    pn.assign(P, 0u);
    for (uint32_t k = 0; k < cnt; k++) {
      const PathResult& pr = res[q + k];
      float a[3] = {(float)pr.acc[0], (float)pr.acc[1], (float)pr.acc[2]};
      if (std::isinf(a[0]) || std::isinf(a[1]) || std::isinf(a[2])) continue;
      float* v = &part[(size_t)(k % P) * 12];
      float fn = (float)pr.n;
      for (int c3 = 0; c3 < 3; c3++) {
        v[c3] = v[c3] + a[c3];
        v[3 + c3] = v[3 + c3] + (float)pr.gpos[c3] * fn;
        v[6 + c3] = v[6 + c3] + (float)pr.gnorm[c3] * fn;
        v[9 + c3] = v[9 + c3] + (float)pr.gdiff[c3] * fn;
      }
      pn[k % P] += pr.n;
    }
    q += cnt;
    for (uint32_t m = P / 2; m > 0; m >>= 1) {
      nxt.assign((size_t)P * 12, 0.f);
      nn2.assign(P, 0u);
      for (uint32_t l = 0; l < P; l++) {
        for (int k = 0; k < 12; k++) nxt[(size_t)l * 12 + k] = part[(size_t)l * 12 + k] + part[(size_t)(l ^ m) * 12 + k];
        nn2[l] = pn[l] + pn[l ^ m];
      }
      part.swap(nxt);
      pn.swap(nn2);
    }
    float tr[3], tp[3], tn[3], td[3];
    for (int c3 = 0; c3 < 3; c3++) {
      tr[c3] = part[c3];
      tp[c3] = part[3 + c3];
      tn[c3] = part[6 + c3];
      td[c3] = part[9 + c3];
    }
    uint32_t tN = pn[0];
    uint32_t N = r->sampleN[i];
    if (frame0) {
      N = 0;
      for (int c3 = 0; c3 < 3; c3++) r->result[i * 3 + c3] = g3[0][i * 3 + c3] = g3[1][i * 3 + c3] = g3[2][i * 3 + c3] = 0.f;
    }
    uint32_t nn = tN + N;
    if (nn > N) {
      float rInf = 1.f / (float)nn, oInf = (float)N * rInf;
      for (int c3 = 0; c3 < 3; c3++) {
        r->result[i * 3 + c3] = std::fmax(rInf * tr[c3] + oInf * r->result[i * 3 + c3], 0.f);
        g3[0][i * 3 + c3] = rInf * tp[c3] + oInf * g3[0][i * 3 + c3];
        g3[1][i * 3 + c3] = rInf * tn[c3] + oInf * g3[1][i * 3 + c3];
        g3[2][i * 3 + c3] = rInf * td[c3] + oInf * g3[2][i * 3 + c3];
      }
      N = nn;
    }
    r->sampleN[i] = N;
  }
}

// FP64 mode: the same estimator in double, plain BDPT only; returns the
// per-pixel ratio sum(acc)/sum(n) over `frames` frames (light cache from the
// FP32 light pass, which the FP64 paths then read in double).
void render_fp64(const Scene& s, const Params& p, uint32_t W, uint32_t H, const Camera& cam, uint32_t frames,
                 uint32_t threads, double* out) {
  Renderer r;
  renderer_init(&r, W, H, kModeBDPT, p, true, threads);
  CamF c;
  float right[3], up[3];
  cam_basis(cam, right, up);
  for (int k = 0; k < 3; k++) {
    c.pos[k] = cam.pos[k];
    c.dir[k] = cam.dir[k];
    c.up[k] = up[k];
    c.right[k] = right[k];
  }
  c.tanHalf = (float)std::tan((double)(cam.fov * 0.5f));
  c.W = (float)W;
  c.H = (float)H;
  const uint32_t np = W * H;
  std::vector<double> sum((size_t)np * 3, 0.0), cnt(np, 0.0);
  std::vector<uint32_t> pixOf(np), sampleOf(np, 0u);
  for (uint32_t i = 0; i < np; i++) pixOf[i] = i;
  for (uint32_t f = 0; f < frames; f++) {
    r.frame = f;
    if (f % p.light_every == 0) light_pass(&r, s, f);
    std::vector<PathResult> res;
    trace_pixels<double>(&r, s, c, pixOf, sampleOf, res, false);
    for (uint32_t i = 0; i < np; i++) {
      if (std::isinf(res[i].acc[0]) || std::isinf(res[i].acc[1]) || std::isinf(res[i].acc[2])) continue;
      for (int k = 0; k < 3; k++) sum[(size_t)i * 3 + k] += res[i].acc[k];
      cnt[i] += res[i].n;
    }
  }
  for (uint32_t i = 0; i < np; i++)
    for (int k = 0; k < 3; k++) out[(size_t)i * 3 + k] = cnt[i] > 0 ? std::max(sum[(size_t)i * 3 + k] / cnt[i], 0.0) : 0.0;
}

}  // namespace orc
