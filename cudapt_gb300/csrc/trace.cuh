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
// A node is fetched with one 32-byte non-coherent load (ld.global.nc.v8, one
// sector; sm_100 and later), a triangle (64-byte record) with one 32-byte and
// one 16-byte load; an
// out-of-range id reads zeros like the reference's texture fetch: ids are
// clamped to one all-zero record stored after each array.
#pragma once
#include "gbpt_math.cuh"
#include "launch.h"

namespace gbpt {

// Both halves of a 32-byte node record (min.xyz + word, max.xyz + word).
// `p` is 32-byte aligned: node arrays start on cudaMalloc's 256-byte
// boundary and a record is 32 bytes.
__device__ __forceinline__ void ldg_node(const float4* p, float4& a, float4& b) {
  asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
      : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
      : "l"(p));
}

// Three-input min / max (PTX ISA 8.8, sm_100 and later): one instruction each
// for fminf(fminf(a, b), c) and fmaxf(fmaxf(a, b), c), NaN inputs ignored the
// same way.
__device__ __forceinline__ float fmin3_(float a, float b, float c) {
  float d;
  asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
  return d;
}
__device__ __forceinline__ float fmax3_(float a, float b, float c) {
  float d;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
  return d;
}

// CURay::IntersectAABB (src/cudaRTCommon.cu:24-40) on the slab distances of
// one box: true, with the entry distance tb (0 when the origin is inside),
// when the box is hit and tb < limit.  The reference's test
// `minmax >= maxmin && (minmax > 0 || maxmin > 0)` is written
// `minmax >= maxmin && minmax > 0` (once maxmin <= minmax, maxmin > 0 implies
// minmax > 0), and its walk's `0 <= tb` holds for every hit.
__device__ __forceinline__ bool slab_hit(float t0x, float t1x, float t0y, float t1y, float t0z, float t1z,
                                         float limit, float& tb) {
  const float minmax = fmin3_(fmaxf(t0x, t1x), fmaxf(t0y, t1y), fmaxf(t0z, t1z));
  const float maxmin = fmax3_(fminf(t0x, t1x), fminf(t0y, t1y), fminf(t0z, t1z));
  tb = (maxmin > gb::kGtEps9) ? maxmin : 0.f;
  return minmax >= maxmin && minmax > 0.f && tb < limit;
}

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
    float4 a, b;  // an id past the tree reads the zero record after it
    ldg_node(nodes + 2 * (size_t)min(cur, S.nodeN), a, b);
    if (kCount) nNodes++;
    const float t0x = (a.x - o.x) * inv.x, t1x = (b.x - o.x) * inv.x;
    const float t0y = (a.y - o.y) * inv.y, t1y = (b.y - o.y) * inv.y;
    const float t0z = (a.z - o.z) * inv.z, t1z = (b.z - o.z) * inv.z;
    float tb;
    if (!slab_hit(t0x, t1x, t0y, t1y, t0z, t1z, minT, tb)) continue;
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
      const size_t ti = 4 * (size_t)min(i, S.triN);  // past the end: the zero record
      float4 p0, e0;
      ldg_node(tris + ti, p0, e0);
      const float4 e1 = __ldg(tris + ti + 2);
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
      if (!(rT >= 0.f && rT < minT)) continue;  // the acceptance test's bound, checked before u and v
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
  // (anyHit) a hit closer than maxDist found, or -- at the start of the call
  // after the last pop -- stack empty or 2048 pops done (testing that once per
  // call instead of after every pop costs one more call per ray).
  template <bool kCount>
  __device__ __forceinline__ bool step(const DevScene& S, uint32_t* stack, bool anyHit, uint32_t& nNodes,
                                       uint32_t& nTris) {
    using namespace gb;
    if (sp < 0 || steps >= 2048u) return true;
    steps++;
    const uint32_t cur = tos;
    sp--;
    if (sp >= 0) tos = stack[sp];
    float4 a, b;  // an id past the tree reads the zero record after it
    ldg_node(S.nodes + 2 * (size_t)min(cur, S.nodeN), a, b);
    if (kCount) nNodes++;
    const float t0x = (a.x - o.x) * inv.x, t1x = (b.x - o.x) * inv.x;
    const float t0y = (a.y - o.y) * inv.y, t1y = (b.y - o.y) * inv.y;
    const float t0z = (a.z - o.z) * inv.z, t1z = (b.z - o.z) * inv.z;
    float tb;
    if (!slab_hit(t0x, t1x, t0y, t1y, t0z, t1z, minT, tb)) return false;
    const uint32_t off = __float_as_uint(a.w);
    const uint32_t tn = __float_as_uint(b.w);
    if (tn == 0) {
      if (sp < 29) {  // push cur+1 then cur+off (the reference's order); cur+off becomes tos
        // (stack[sp] already holds the current tos: it was just reloaded from there)
        stack[sp + 1] = cur + 1;
        sp += 2;
        tos = cur + off;
      }
      return false;
    }
    for (uint32_t i = off; i < off + tn; i++) {
      const size_t ti = 4 * (size_t)min(i, S.triN);  // past the end: the zero record
      float4 p0, e0;
      ldg_node(S.tris + ti, p0, e0);
      const float4 e1 = __ldg(S.tris + ti + 2);
      if (kCount) nTris++;
      const f3 E0 = mk(e0.x, e0.y, e0.z), E1 = mk(e1.x, e1.y, e1.z);
      const f3 de2 = cross(d, E1);
      float div = dot(de2, E0);
      if (fabsf(div) < kLtEps9) continue;
      div = rcp_(div);
      const f3 t = oe - mk(p0.x, p0.y, p0.z);
      const f3 te1 = cross(t, E0);
      const float rT = dot(te1, E1) * div;
      if (!(rT >= 0.f && rT < minT)) continue;  // the acceptance test's bound, checked before u and v
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
    return false;
  }

  __device__ __forceinline__ bool hit() const { return minT < maxDist; }
};

// Wide walk (DevScene::traversal == 1): the collapsed 4-ary tree, one wide
// node per step -- one 112-byte fetch and four box tests (the reference's
// IntersectAABB arithmetic) -- children accepted when their entry distance
// is at most the closest hit so far, pushed far to near so the nearest is
// walked next.  The closest hit is the reference's: a triangle is accepted
// when strictly closer, or equally close with a larger index (the
// reference's right-first order reaches larger indices first and keeps the
// first of equal distances; inside one leaf it walks triangles in index
// order, so there the smaller index wins).  Stack entries are {code, entry
// distance}.
constexpr uint32_t kWideDepth = 56;      // >= 3 * (binary depth cap 32) / 2 + 1
constexpr uint32_t kWideStepCap = 8192;  // pops; a wide pop replaces up to three binary ones
struct Walk4 {
  gb::f3 o, d, inv, oe;
  float minT, maxDist, eps;
  float bw, bu, bv;
  uint32_t best, bestLeaf, steps;  // bestLeaf: first triangle of the leaf holding best
  uint2 tos;
  int sp;

  __device__ __forceinline__ void init(gb::f3 o_, gb::f3 d_, float maxDist_, float eps_, uint2* stack) {
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
    bestLeaf = 0;
    bw = bu = bv = 0.f;
    steps = 0;
    sp = 0;
    tos = make_uint2(0u, 0u);  // wide root, entry distance 0
  }

  __device__ __forceinline__ float box(float lx, float ly, float lz, float hx, float hy, float hz) const {
    using namespace gb;
    const float t0x = (lx - o.x) * inv.x, t1x = (hx - o.x) * inv.x;
    const float t0y = (ly - o.y) * inv.y, t1y = (hy - o.y) * inv.y;
    const float t0z = (lz - o.z) * inv.z, t1z = (hz - o.z) * inv.z;
    float tb;
    return slab_hit(t0x, t1x, t0y, t1y, t0z, t1z, kInf, tb) ? tb : kInf;
  }

  template <bool kCount>
  __device__ __forceinline__ bool step(const DevScene& S, uint2* stack, bool anyHit, uint32_t& nNodes,
                                       uint32_t& nTris) {
    using namespace gb;
    if (sp < 0 || steps >= kWideStepCap) return true;
    steps++;
    const uint2 e = tos;
    sp--;
    if (sp >= 0) tos = stack[sp];
    if (!(__uint_as_float(e.y) <= minT)) return sp < 0;
    const uint32_t code = e.x;
    if (code & kWideLeaf) {
      uint32_t first, cnt;
      if (code & 0x40000000u) {
        first = code & 0x3FFFFFFFu;
        cnt = 1;
      } else {
        const uint32_t nid = code & 0x7FFFFFFFu;
        first = __float_as_uint(__ldg(S.nodes + 2 * (size_t)nid).w);
        cnt = __float_as_uint(__ldg(S.nodes + 2 * (size_t)nid + 1).w);
      }
      for (uint32_t i = first; i < first + cnt; i++) {
        const size_t ti = 4 * (size_t)min(i, S.triN);  // past the end: the zero record
        float4 p0, e0;
        ldg_node(S.tris + ti, p0, e0);
        const float4 e1 = __ldg(S.tris + ti + 2);
        if (kCount) nTris++;
        const f3 E0 = mk(e0.x, e0.y, e0.z), E1 = mk(e1.x, e1.y, e1.z);
        const f3 de2 = cross(d, E1);
        float div = dot(de2, E0);
        if (fabsf(div) < kLtEps9) continue;
        div = rcp_(div);
        const f3 t = oe - mk(p0.x, p0.y, p0.z);
        const f3 te1 = cross(t, E0);
        const float rT = dot(te1, E1) * div;
        if (!(rT >= 0.f && rT <= minT)) continue;  // the acceptance test's bound, checked before u and v
        const float u = dot(de2, t) * div;
        if (u < 0.f || u > 1.f) continue;
        const float v = dot(te1, d) * div;
        if (v < 0.f || (u + v) > 1.f) continue;
        if (rT < minT || (rT == minT && minT < maxDist && first > bestLeaf)) {
          minT = rT;
          best = i;
          bestLeaf = first;
          bw = 1.f - u - v;
          bu = u;
          bv = v;
          if (anyHit) return true;
        }
      }
      return sp < 0;
    }
    if (kCount) nNodes++;
    const float4* r = S.wide + 8 * (size_t)code;
    float4 lx, ly, lz, hx, hy, hz;
    ldg_node(r, lx, ly);
    ldg_node(r + 2, lz, hx);
    ldg_node(r + 4, hy, hz);
    const uint4 cd = __ldg(reinterpret_cast<const uint4*>(r + 6));
    float t[4] = {box(lx.x, ly.x, lz.x, hx.x, hy.x, hz.x), box(lx.y, ly.y, lz.y, hx.y, hy.y, hz.y),
                  box(lx.z, ly.z, lz.z, hx.z, hy.z, hz.z), box(lx.w, ly.w, lz.w, hx.w, hy.w, hz.w)};
    uint32_t c[4] = {cd.x, cd.y, cd.z, cd.w};
    uint32_t m = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const bool ok = c[k] != kWideEmpty && t[k] < kInf && t[k] <= minT;
      if (!ok) t[k] = __uint_as_float(0x7f800000u);  // +inf sorts last
      m += ok ? 1u : 0u;
    }
    // sort the four (distance, code) pairs, nearest first
#define GB_CSWAP(a, b)                   \
  if (t[b] < t[a]) {                     \
    const float tt = t[a];               \
    t[a] = t[b];                         \
    t[b] = tt;                           \
    const uint32_t cc = c[a];            \
    c[a] = c[b];                         \
    c[b] = cc;                           \
  }
    GB_CSWAP(0, 1) GB_CSWAP(2, 3) GB_CSWAP(0, 2) GB_CSWAP(1, 3) GB_CSWAP(1, 2)
#undef GB_CSWAP
    if (m == 0) return sp < 0;
    if (sp + (int)m >= (int)kWideDepth) m = (uint32_t)((int)kWideDepth - 1 - sp);  // keep the nearest
    // far to near below the new top; the nearest becomes the top (stack[sp] keeps the old top)
    for (uint32_t j = m - 1; j >= 1; j--) stack[sp + (int)(m - j)] = make_uint2(c[j], __float_as_uint(t[j]));
    sp += (int)m;
    tos = make_uint2(c[0], __float_as_uint(t[0]));
    return false;
  }

  __device__ __forceinline__ bool hit() const { return minT < maxDist; }
};

// walk type, stack entry type and stack depth of the two traversal orders
template <bool kWide>
struct WalkOf {
  using type = Walk;
  using Entry = uint32_t;
  static constexpr int kDepth = 32;
};
template <>
struct WalkOf<true> {
  using type = Walk4;
  using Entry = uint2;
  static constexpr int kDepth = (int)kWideDepth;
};

}  // namespace gbpt
