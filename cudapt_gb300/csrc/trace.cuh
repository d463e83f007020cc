// BVH walk of the GB300 BDPT kernels.
//
// Same visiting order and arithmetic as the reference's TracePrimitive
// (src/cudaRTCommon.cu:66-127) so hit ids are bit-exact:
//   * stack of 32 node ids; an inner node whose box is hit pushes i+1 (left)
//     then i+offset (right), so the right child is popped first (:88-92);
//     pushes are skipped once the stack pointer reaches BVH_DEPTH_MAX-3 (:88);
//   * at most BVH_TRACE_MAX = 2048 pops (include/cudaRTCommon.h:14);
//   * box test of CURay::IntersectAABB (:24-40): entry distance, 0 when the
//     origin is inside, M_INF on a miss; accepted when 0 <= t < closest;
//   * CURay::IntersectTri (:42-64) with the origin pushed by eps*dir, strict
//     `<` against the closest hit (first triangle wins ties).
// The per-ray constants of those two tests (1/escapeZero(dir), o + eps*dir)
// are hoisted out of the loop; they are the same values every iteration.
// Node and triangle fetches are read-only 16-byte __ldg loads (one 32-byte
// sector per node); an out-of-range id reads zeros like the reference's
// texture fetch.
#pragma once
#include "gbpt_math.cuh"
#include "launch.h"

namespace gbpt {

struct TraceHit {
  float t, w, u, v;
  uint32_t tri;
};

template <bool kAnyHit, bool kCount>
__device__ __forceinline__ bool trace_ref(const DevScene& S, gb::f3 o, gb::f3 d, float maxDist, float eps,
                                          bool cullback, TraceHit& h, uint32_t& nNodes, uint32_t& nTris) {
  using namespace gb;
  const f3 inv = mk(rcp_(escape_zero(d.x)), rcp_(escape_zero(d.y)), rcp_(escape_zero(d.z)));
  const f3 oe = o + eps * d;
  float minT = maxDist;
  uint32_t best = 0;
  float bw = 0.f, bu = 0.f, bv = 0.f;
  uint32_t stack[32];
  stack[0] = 0;
  int sp = 0;
  uint32_t steps = 0;
  const float4* __restrict__ nodes = S.nodes;
  const float4* __restrict__ tris = S.tris;
  while (sp >= 0 && steps++ < 2048u) {
    const uint32_t cur = stack[sp--];
    float4 a = make_float4(0.f, 0.f, 0.f, 0.f), b = a;
    if (cur < S.nodeN) {
      a = __ldg(nodes + 2 * (size_t)cur);
      b = __ldg(nodes + 2 * (size_t)cur + 1);
    }
    if (kCount) nNodes++;
    const float t0x = (a.x - o.x) * inv.x, t1x = (b.x - o.x) * inv.x;
    const float t0y = (a.y - o.y) * inv.y, t1y = (b.y - o.y) * inv.y;
    const float t0z = (a.z - o.z) * inv.z, t1z = (b.z - o.z) * inv.z;
    const float minmax = fminf(fminf(fmaxf(t0x, t1x), fmaxf(t0y, t1y)), fmaxf(t0z, t1z));
    const float maxmin = fmaxf(fmaxf(fminf(t0x, t1x), fminf(t0y, t1y)), fminf(t0z, t1z));
    float tb = kInf;
    if (minmax >= maxmin && (minmax > 0.f || maxmin > 0.f)) tb = (maxmin > kGtEps9) ? maxmin : 0.f;
    if (!(tb >= 0.f && tb < minT)) continue;
    const uint32_t off = __float_as_uint(a.w);
    const uint32_t tn = __float_as_uint(b.w);
    if (tn == 0) {
      if (sp < 29) {
        stack[++sp] = cur + 1;
        stack[++sp] = cur + off;
      }
      continue;
    }
    for (uint32_t i = off; i < off + tn; i++) {
      float4 p0 = make_float4(0.f, 0.f, 0.f, 0.f), e0 = p0, e1 = p0;
      if (i < S.triN) {
        p0 = __ldg(tris + 3 * (size_t)i);
        e0 = __ldg(tris + 3 * (size_t)i + 1);
        e1 = __ldg(tris + 3 * (size_t)i + 2);
      }
      if (kCount) nTris++;
      const f3 E0 = mk(e0.x, e0.y, e0.z), E1 = mk(e1.x, e1.y, e1.z);
      if (cullback && dot(cross(E0, E1), d) > 0.f) continue;
      const f3 de2 = cross(d, E1);
      float div = dot(de2, E0);
      if (fabsf(div) < kLtEps9) continue;
      div = rcp_(div);
      const f3 t = oe - mk(p0.x, p0.y, p0.z);
      const f3 te1 = cross(t, E0);
      const float rT = dot(te1, E1) * div;
      if (rT < 0.f) continue;
      const float u = dot(de2, t) * div;
      if (u < 0.f || u > 1.f) continue;
      const float v = dot(te1, d) * div;
      if (v < 0.f || (u + v) > 1.f) continue;
      if (rT >= 0.f && rT < minT) {
        minT = rT;
        best = i;
        bw = 1.f - u - v;
        bu = u;
        bv = v;
        if (kAnyHit) {
          h.t = rT;
          h.tri = i;
          return true;
        }
      }
    }
  }
  if (minT < maxDist) {
    h.t = minT;
    h.tri = best;
    h.w = bw;
    h.u = bu;
    h.v = bv;
    return true;
  }
  return false;
}

// The same walk as trace_ref, one node per step(), so that a persistent
// kernel can hand a new ray to a lane as soon as its current ray is done
// without changing the order in which any single ray visits nodes.
//
// Latency: the top stack entry is kept in a register (tos), so the next
// node id is known without a memory round trip and the reload of the new top
// overlaps the node fetch.
struct Walk {
  gb::f3 o, d, inv, oe;
  float minT, maxDist, eps;
  float bw, bu, bv;
  uint32_t best, steps, tos;
  int sp;  // index of the top entry (entries below it live in the stack array)

  // the node stack lives outside the struct (it is indexed dynamically and
  // goes to local memory; the other members stay in registers)
  __device__ __forceinline__ void init(gb::f3 o_, gb::f3 d_, float maxDist_, float eps_, uint32_t* stack) {
    using namespace gb;
    (void)stack;
    o = o_;
    d = d_;
    inv = mk(rcp_(escape_zero(d.x)), rcp_(escape_zero(d.y)), rcp_(escape_zero(d.z)));
    eps = eps_;
    oe = o + eps * d;
    maxDist = maxDist_;
    minT = maxDist_;
    best = 0;
    bw = bu = bv = 0.f;
    steps = 0;
    sp = 0;
    tos = 0;  // root
  }

  // One pop of TracePrimitive's loop.  Returns true when the walk is over:
  // stack empty, 2048 pops done, or (anyHit) a hit closer than maxDist found.
  template <bool kCount>
  __device__ __forceinline__ bool step(const DevScene& S, uint32_t* stack, bool anyHit, uint32_t& nNodes,
                                       uint32_t& nTris) {
    using namespace gb;
    if (sp < 0 || steps >= 2048u) return true;
    steps++;
    const uint32_t cur = tos;
    sp--;
    if (sp >= 0) tos = stack[sp];
    float4 a = make_float4(0.f, 0.f, 0.f, 0.f), b = a;
    if (cur < S.nodeN) {
      a = __ldg(S.nodes + 2 * (size_t)cur);
      b = __ldg(S.nodes + 2 * (size_t)cur + 1);
    }
    if (kCount) nNodes++;
    const float t0x = (a.x - o.x) * inv.x, t1x = (b.x - o.x) * inv.x;
    const float t0y = (a.y - o.y) * inv.y, t1y = (b.y - o.y) * inv.y;
    const float t0z = (a.z - o.z) * inv.z, t1z = (b.z - o.z) * inv.z;
    const float minmax = fminf(fminf(fmaxf(t0x, t1x), fmaxf(t0y, t1y)), fmaxf(t0z, t1z));
    const float maxmin = fmaxf(fmaxf(fminf(t0x, t1x), fminf(t0y, t1y)), fminf(t0z, t1z));
    float tb = kInf;
    if (minmax >= maxmin && (minmax > 0.f || maxmin > 0.f)) tb = (maxmin > kGtEps9) ? maxmin : 0.f;
    if (!(tb >= 0.f && tb < minT)) return sp < 0 || steps >= 2048u;
    const uint32_t off = __float_as_uint(a.w);
    const uint32_t tn = __float_as_uint(b.w);
    if (tn == 0) {
      if (sp < 29) {  // push cur+1 then cur+off (the reference's order); cur+off becomes tos
        // (stack[sp] already holds the current tos: it was just reloaded from there)
        stack[sp + 1] = cur + 1;
        sp += 2;
        tos = cur + off;
      }
      return sp < 0 || steps >= 2048u;
    }
    for (uint32_t i = off; i < off + tn; i++) {
      float4 p0 = make_float4(0.f, 0.f, 0.f, 0.f), e0 = p0, e1 = p0;
      if (i < S.triN) {
        p0 = __ldg(S.tris + 3 * (size_t)i);
        e0 = __ldg(S.tris + 3 * (size_t)i + 1);
        e1 = __ldg(S.tris + 3 * (size_t)i + 2);
      }
      if (kCount) nTris++;
      const f3 E0 = mk(e0.x, e0.y, e0.z), E1 = mk(e1.x, e1.y, e1.z);
      const f3 de2 = cross(d, E1);
      float div = dot(de2, E0);
      if (fabsf(div) < kLtEps9) continue;
      div = rcp_(div);
      const f3 t = oe - mk(p0.x, p0.y, p0.z);
      const f3 te1 = cross(t, E0);
      const float rT = dot(te1, E1) * div;
      if (rT < 0.f) continue;
      const float u = dot(de2, t) * div;
      if (u < 0.f || u > 1.f) continue;
      const float v = dot(te1, d) * div;
      if (v < 0.f || (u + v) > 1.f) continue;
      if (rT >= 0.f && rT < minT) {
        minT = rT;
        best = i;
        bw = 1.f - u - v;
        bu = u;
        bv = v;
        if (anyHit) return true;
      }
    }
    return sp < 0 || steps >= 2048u;
  }

  __device__ __forceinline__ bool hit() const { return minT < maxDist; }
};

}  // namespace gbpt
