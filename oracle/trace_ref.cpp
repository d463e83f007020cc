// TEST INFRASTRUCTURE ONLY -- CPU oracle: ray/box, ray/triangle and the
// closest-hit BVH walk, restated from the reference.
//
//   src/cudaRTCommon.cu:24-40   CURay::IntersectAABB
//   src/cudaRTCommon.cu:42-64   CURay::IntersectTri (Moller-Trumbore variant)
//   src/cudaRTCommon.cu:66-127  TracePrimitive (32-entry stack, 2048 steps)
//   include/cudaRTCommon.h:13-14 BVH_DEPTH_MAX / BVH_TRACE_MAX
//
// Float semantics follow include/cudahelper.h (see fmath_ref.h).  The two
// comparisons against the double literal M_EPSILON (1e-9) are evaluated in
// double, as the reference does.  Node and triangle fetches outside the
// arrays return zeros, like tex1Dfetch on linear memory; only degenerate
// trees (a split that leaves one child empty) ever reach them.
#include <cmath>

#include "fmath_ref.h"
#include "oracle.h"

namespace orc {

namespace {
constexpr float kInf = (float)1E20;                 // M_INF as a float
constexpr float kEpsF = (float)1E-9;                // M_EPSILON passed as float
constexpr uint32_t kStack = 32, kMaxSteps = 2048;  // BVH_DEPTH_MAX, BVH_TRACE_MAX
}  // namespace

struct RayPre {
  f3 o, d, inv;
};

static inline float aabb(const RayPre& r, f3 mn, f3 mx) {
  f3 tmin = vmul(mn - r.o, r.inv);
  f3 tmax = vmul(mx - r.o, r.inv);
  f3 rmin = vmin(tmin, tmax);
  f3 rmax = vmax(tmin, tmax);
  float minmax = std::fmin(std::fmin(rmax.x, rmax.y), rmax.z);
  float maxmin = std::fmax(std::fmax(rmin.x, rmin.y), rmin.z);
  if (minmax >= maxmin && (minmax > 0.f || maxmin > 0.f)) return ((double)maxmin > 1E-9) ? maxmin : 0;
  return kInf;
}

static inline float tri_isect(const RayPre& r, f3 p0, f3 e0, f3 e1, float eps, bool cullback, float& w, float& u,
                              float& v) {
  if (cullback && dot(cross(e0, e1), r.d) > 0.f) return kInf;
  f3 de2 = cross(r.d, e1);
  float divisor = dot(de2, e0);
  if ((double)std::fabs(divisor) < 1E-9) return kInf;
  divisor = rcpf(divisor);
  f3 t = (r.o + eps * r.d) - p0;
  f3 te1 = cross(t, e0);
  float rT = dot(te1, e1) * divisor;
  if (rT < 0.f) return kInf;
  u = dot(de2, t) * divisor;
  if (u < 0.f || u > 1.f) return kInf;
  v = dot(te1, r.d) * divisor;
  if (v < 0.f || (u + v) > 1.f) return kInf;
  w = 1 - u - v;
  return rT;
}

bool trace_primitive(const Scene& s, const float o[3], const float d[3], float maxDist, float eps, bool cullback,
                     Hit* hit, TraceCount* cnt) {
  RayPre r;
  r.o = mk(o[0], o[1], o[2]);
  r.d = mk(d[0], d[1], d[2]);
  f3 md = mk(escapeZero(r.d.x, kEpsF), escapeZero(r.d.y, kEpsF), escapeZero(r.d.z, kEpsF));
  r.inv = vrcp(md);
  const uint32_t nodeN = s.bvh.nodeN;
  const uint32_t triN = (uint32_t)s.tris.size();
  float minIntersect = maxDist;
  uint32_t tracedTriId = 0;
  float w = 0, u = 0, v = 0;
  uint32_t stack[kStack];
  stack[0] = 0;
  int32_t sp = 0;
  uint32_t steps = 0;
  while (sp >= 0 && steps++ < kMaxSteps) {
    uint32_t cur = stack[sp--];
    f3 mn = mk(0, 0, 0), mx = mk(0, 0, 0);
    uint32_t off = 0, tn = 0;
    if (cur < nodeN) {
      const float* b = &s.bvh.bounds[(size_t)cur * 6];
      mn = mk(b[0], b[1], b[2]);
      mx = mk(b[3], b[4], b[5]);
    }
    if (cnt) cnt->nodes++;
    float tb = aabb(r, mn, mx);
    if (tb >= 0 && tb < minIntersect) {
      if (cur < nodeN) {
        off = s.bvh.offOrTSTN[(size_t)cur * 2];
        tn = s.bvh.offOrTSTN[(size_t)cur * 2 + 1];
      }
      if (tn == 0) {
        if (sp < (int32_t)kStack - 3) {
          stack[++sp] = cur + 1;
          stack[++sp] = cur + off;
        }
      } else {
        for (uint32_t i = off; i < off + tn; i++) {
          f3 p0 = mk(0, 0, 0), e0 = p0, e1 = p0;
          if (i < triN) {
            const float* q = &s.isect[(size_t)i * 9];
            p0 = mk(q[0], q[1], q[2]);
            e0 = mk(q[3], q[4], q[5]);
            e1 = mk(q[6], q[7], q[8]);
          }
          if (cnt) cnt->tris++;
          float tw = 0, tu = 0, tv = 0;
          float ti = tri_isect(r, p0, e0, e1, eps, cullback, tw, tu, tv);
          if (ti >= 0 && ti < minIntersect) {
            minIntersect = ti;
            tracedTriId = i;
            w = tw;
            u = tu;
            v = tv;
          }
        }
      }
    }
  }
  if (minIntersect < maxDist) {
    hit->dist = minIntersect;
    hit->triId = (int32_t)tracedTriId;
    hit->w = w;
    hit->u = u;
    hit->v = v;
    return true;
  }
  return false;
}

// The two intersection routines alone, for case-by-case comparison with
// the reference's CURay functions.
float intersect_aabb(const float o[3], const float d[3], const float mn[3], const float mx[3]) {
  RayPre r;
  r.o = mk(o[0], o[1], o[2]);
  r.d = mk(d[0], d[1], d[2]);
  r.inv = vrcp(mk(escapeZero(r.d.x, kEpsF), escapeZero(r.d.y, kEpsF), escapeZero(r.d.z, kEpsF)));
  return aabb(r, mk(mn[0], mn[1], mn[2]), mk(mx[0], mx[1], mx[2]));
}

float intersect_tri(const float o[3], const float d[3], const float p0[3], const float e0[3], const float e1[3],
                    float eps, bool cullback, float wuv[3]) {
  RayPre r;
  r.o = mk(o[0], o[1], o[2]);
  r.d = mk(d[0], d[1], d[2]);
  float w = 0.f, u = 0.f, v = 0.f;
  float t = tri_isect(r, mk(p0[0], p0[1], p0[2]), mk(e0[0], e0[1], e0[2]), mk(e1[0], e1[1], e1[2]), eps, cullback, w,
                      u, v);
  wuv[0] = w;
  wuv[1] = u;
  wuv[2] = v;
  return t;
}

bool make_scene(const RTVertex* v, uint32_t nv, const RTTriangle* t, uint32_t nt, const RTMaterial* m, uint32_t nm,
                Scene* s) {
  s->verts.assign(v, v + nv);
  s->mats.assign(m, m + nm);
  std::vector<float> pos((size_t)nv * 3);
  for (uint32_t i = 0; i < nv; i++)
    for (int k = 0; k < 3; k++) pos[(size_t)i * 3 + k] = v[i].pos[k];
  std::vector<uint32_t> idx((size_t)nt * 3);
  for (uint32_t i = 0; i < nt; i++) {
    idx[(size_t)i * 3] = t[i].v0;
    idx[(size_t)i * 3 + 1] = t[i].v1;
    idx[(size_t)i * 3 + 2] = t[i].v2;
  }
  if (!build_bvh(pos.data(), nv, idx.data(), nt, 32, &s->bvh)) return false;
  // src/raytracer.cpp:268-280 reorder; src/cudaRTCommon.cu:503-513 p0, p1-p0, p2-p0
  s->tris.resize(nt);
  s->isect.resize((size_t)nt * 9);
  for (uint32_t i = 0; i < nt; i++) {
    s->tris[i] = t[s->bvh.order[i]];
    const float* a = v[s->tris[i].v0].pos;
    const float* b = v[s->tris[i].v1].pos;
    const float* c = v[s->tris[i].v2].pos;
    for (int k = 0; k < 3; k++) {
      s->isect[(size_t)i * 9 + k] = a[k];
      s->isect[(size_t)i * 9 + 3 + k] = b[k] - a[k];
      s->isect[(size_t)i * 9 + 6 + k] = c[k] - a[k];
    }
  }
  refresh_lights(s);
  return true;
}

// src/cudaRTBDPTStream.cu:57-77: a triangle is a light when the host length
// of its material's emissive colour is > 0.
void refresh_lights(Scene* s) {
  s->lightTri.clear();
  for (uint32_t i = 0; i < s->tris.size(); i++) {
    const RTMaterial& mm = s->mats[s->tris[i].mat];
    const float* e = mm.emissive;
    float l = std::sqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]);
    if (l > 0.f) s->lightTri.push_back(i);
  }
}

}  // namespace orc
