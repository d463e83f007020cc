// Wavefront BDPT kernels for GB300 (sm_103a).
//
// One frame of the reference's streaming BDPT (src/cudaRTBDPTStream.cu:816-951)
// runs as a fixed sequence of launches with no host round trip:
//
//   light pass (1 CTA)          pt_genLightPathQueue_kernel + pt_traceLight_kernel
//                               loop with stable compaction (:875-906)
//   camera                      pt_genPathQueue_kernel (:619-640)
//   per bounce launch d (k_walk, then k_shade):
//     shadow (any hit)          the visibility test of GetLightFromRandLightVertices
//                               (:665-700) for bounce d-1's connections
//     trace  (closest hit)      the TracePrimitive half of pt_traceSample_kernel,
//                               for the walks launch d-1 carried and wave d
//     shade                     the rest of pt_traceSample_kernel (:365-543);
//                               survivors are appended to the other wave
//                               buffer with one atomic per warp (replaces
//                               thrust::remove_if, :930), connection requests
//                               likewise (replaces thrust::copy_if, :934)
//   tail (k_tail)               the remaining bounces of the paths still alive,
//                               one lane per path, and the last launch's carried walks
//   fold (k_fold)               the accumulate of pt_connectEyeLightPath_kernel
//                               (:703-723) and of the path's end, in bounce order
//   apply                       pt_applyPathQueueResult_kernel (:741-778)
//
// Queue lengths live in device memory (DevCounters) and every kernel runs a
// grid-stride loop or a persistent fetch loop over them, so the host never
// waits on a count.
#include <algorithm>
#include <atomic>
#include <cuda_runtime.h>

#include <cstdlib>

#include "launch.h"
#include "shade.cuh"
#include "texture.cuh"
#include "trace.cuh"

namespace gbpt {

using gb::f3;
using gb::mk;

namespace {

constexpr int kBlock = 256;

__device__ __forceinline__ f3 ld3(float4 v) { return mk(v.x, v.y, v.z); }
__device__ __forceinline__ float4 st4(f3 v, float w) { return make_float4(v.x, v.y, v.z, w); }
__device__ __forceinline__ float4 st4u(f3 v, uint32_t w) { return make_float4(v.x, v.y, v.z, __uint_as_float(w)); }
__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

struct Mat {
  f3 diff, emis;
  float trans, spec, metal, rough;
  int32_t texD, texE;  // diffuseTexId, emissiveTexId (-1: none)
};
__device__ __forceinline__ Mat load_mat(const DevScene& S, uint32_t id) {
  float4 a = __ldg(S.mats + 3 * (size_t)id), b = __ldg(S.mats + 3 * (size_t)id + 1),
         c = __ldg(S.mats + 3 * (size_t)id + 2);
  Mat m;
  m.diff = ld3(a);
  m.trans = a.w;
  m.emis = ld3(b);
  m.spec = b.w;
  m.metal = c.x;
  m.rough = c.y;
  m.texD = __float_as_int(c.z);
  m.texE = __float_as_int(c.w);
  return m;
}

// The texture half of GetMaterialColors (src/cudaRTCommon.cu:369-406) at the
// barycentrics (w, u, v) of triangle `tri`: uv = ((uv0*w) + (uv1*u)) + uv2*v
// (the float2 operators of the reference's kernels, e.g.
// src/cudaRTBDPTStream.cu:379-382); a diffuse texture gives the diffuse
// colour and scales the transparency by its alpha, an emissive texture gives
// the emissive colour.
__device__ __forceinline__ void apply_textures(const DevScene& S, Mat& m, uint32_t tri, float w, float u, float v) {
  const float2* q = S.uvs + 3 * (size_t)tri;
  const float2 a = __ldg(q), b = __ldg(q + 1), c = __ldg(q + 2);
  const float tu = (a.x * w + b.x * u) + c.x * v;
  const float tv = (a.y * w + b.y * u) + c.y * v;
  if (m.texD >= 0) {
    const float4 t = tex_bilinear(S.texels, __ldg(S.texInfo + m.texD), tu, tv);
    m.diff = mk(t.x, t.y, t.z);
    m.trans = t.w * m.trans;
  }
  if (m.texE >= 0) {
    const float4 t = tex_bilinear(S.texels, __ldg(S.texInfo + m.texE), tu, tv);
    m.emis = mk(t.x, t.y, t.z);
  }
}
__device__ __forceinline__ Mat load_mat_at(const DevScene& S, uint32_t matId, uint32_t tri, float w, float u,
                                           float v) {
  Mat m = load_mat(S, matId);
  if (m.texD >= 0 || m.texE >= 0) apply_textures(S, m, tri, w, u, v);
  return m;
}

// interpolated normal, position and material id of a triangle at (w,u,v):
// ((x0*w) + (x1*u)) + (x2*v) as the reference's float3 operators.
struct Surf {
  f3 norm, pos;
  uint32_t mat;
};
__device__ __forceinline__ Surf load_surf(const DevScene& S, uint32_t tri, float w, float u, float v, bool wantPos) {
  const float4* r = S.shade + 5 * (size_t)tri;
  float4 a = __ldg(r), b = __ldg(r + 1), c = __ldg(r + 2), d = __ldg(r + 3);
  Surf s;
  s.norm = (ld3(a) * w + ld3(b) * u) + ld3(c) * v;
  s.mat = __float_as_uint(d.w);
  if (wantPos) {
    float4 e = __ldg(r + 4);
    s.pos = (mk(a.w, b.w, c.w) * w + ld3(d) * u) + ld3(e) * v;
  } else {
    s.pos = mk(0.f, 0.f, 0.f);
  }
  return s;
}

enum : uint32_t { kTypeEye = 0, kTypeDiff = 1, kTypeSpec = 2, kTypeLight = 3 };

// The bounce decision shared by eye and light paths (reflect / transmit /
// diffuse, src/cudaRTBDPTStream.cu:400-493 and :223-323).
// With wantPdf, also the sampling density of the filter-only variant
// (src/cudaRTBDPTStreamBilat.cu:515-518, :560, :575, :599): D*NoH/(4 VoH)
// times the probability of the branch taken.
struct Bounce {
  f3 nl, nOrig, nDir, lmt, F;
  uint32_t type;
  float pdf;
};
//
// ptTir: the unidirectional variant reflects on total internal reflection
// (src/cudaRTPTStream.cu:153-160: cos2t < 0 sets reflProb = 1); the BDPT
// variants compute the refracted direction regardless (the test is commented
// out there).  The refracted direction stays zero when it is not computed
// (uninitialised in the reference).
__device__ __forceinline__ void sample_bounce(f3 orig, f3 dir, float dist, f3 norm, const Mat& m, const float* u,
                                              bool specPush, bool wantPdf, bool ptTir, Bounce& B) {
  using namespace gb;
  B.nl = dot(norm, dir) < 0.f ? norm : -1.f * norm;
  const f3 nl = B.nl;
  f3 hDir = ggx_sample(u[0], u[1], m.rough, nl);
  f3 ndir = -1.f * dir;
  float voH = dot(ndir, hDir);
  f3 f0 = vlerp(kF0Spec * mk(m.spec, m.spec, m.spec), m.diff, m.metal);
  f3 F = f_schlick(f0, voH);
  B.F = F;
  B.pdf = 1.f;
  if (wantPdf) {
    const float NoH0 = dot(nl, hDir);
    B.pdf = (d_ggx(m.rough, NoH0) * NoH0) / (4.f * voH);
  }
  float reflProb = lerp(length(F), 1.0f, m.metal);
  float refrProb = m.trans;
  f3 reflDir = mk(0.f, 0.f, 0.f), refrDir = reflDir;
  if (refrProb > 0.f) {
    bool into = dot(nl, norm) > 0.f;
    float nt = m.spec * 0.8f + 1.f;
    float nnt = into ? 1.0f / nt : nt / 1.0f;
    float ddn = dot(hDir, dir);
    float cos2t = 1.f - (nnt * nnt) * (1.f - ddn * ddn);
    if (ptTir && cos2t < 0.f)
      reflProb = 1.0f;
    else
      refrDir = normalize(dir * nnt - hDir * (ddn * nnt + sqrtf(cos2t)));
  }
  if (reflProb > 0.f) {
    reflDir = normalize(dir - (hDir * 2.f) * dot(hDir, dir));
    if (dot(reflDir, nl) < 0.f) reflProb = 0.f;
  }
  if (prob_rand(reflProb, u[2])) {
    B.nOrig = orig + (dist - kBias) * dir;
    if (specPush) B.nOrig = B.nOrig + reflDir * kBias;
    B.nDir = reflDir;
    float VoH = dot(ndir, hDir), NoV = dot(nl, ndir), NoH = dot(nl, hDir), NoL = dot(nl, reflDir);
    float G = vis_smith(m.rough, NoV, NoL);
    B.lmt = ((F * G) * VoH) / ((NoV * NoH) * reflProb);
    B.type = kTypeSpec;
    B.pdf = B.pdf * reflProb;
  } else if (prob_rand(refrProb, u[3])) {
    B.nOrig = (orig + (dist + kBias) * dir) + refrDir * kBias;
    B.nDir = refrDir;
    float cosine = dot(-1.f * nl, refrDir);
    B.lmt = (cosine * m.diff) / (refrProb * (1.f - reflProb));
    B.type = kTypeSpec;
    B.pdf = B.pdf * (refrProb * (1.f - reflProb));
  } else {
    f3 dd = cos_dir(u[4], u[5], nl);
    B.nOrig = (orig + dist * dir) + dd * kBias;
    B.nDir = dd;
    B.lmt = (kPi * (m.diff * kInvPi)) / ((1.f - refrProb) * (1.f - reflProb));
    B.type = kTypeDiff;
    B.pdf = B.pdf * (((1.f - refrProb) * (1.f - reflProb)) * dot(dd, nl));
  }
}

// light-vertex cache record: 6 float4
//   {pos, specular} {norm, metallic} {irrad, roughness} {irradDir, 0} {diff, 0} {emissive, 0}
struct LV {
  f3 pos, norm, irrad, irradDir, diff, emis;
  float spec, metal, rough;
};
__device__ __forceinline__ void store_lv(float4* c, const LV& v) {
  c[0] = st4(v.pos, v.spec);
  c[1] = st4(v.norm, v.metal);
  c[2] = st4(v.irrad, v.rough);
  c[3] = st4(v.irradDir, 0.f);
  c[4] = st4(v.diff, 0.f);
  c[5] = st4(v.emis, 0.f);
}
__device__ __forceinline__ LV load_lv(const float4* c) {
  LV v;
  float4 a = c[0], b = c[1], d = c[2], e = c[3], f = c[4], g = c[5];
  v.pos = ld3(a);
  v.spec = a.w;
  v.norm = ld3(b);
  v.metal = b.w;
  v.irrad = ld3(d);
  v.rough = d.w;
  v.irradDir = ld3(e);
  v.diff = ld3(f);
  v.emis = ld3(g);
  return v;
}

// ---------------------------------------------------------------------------
// Light pass: one CTA, one thread per light subpath.  Cache slots are handed
// out exactly as the reference's stable remove_if does: a surviving path's
// position in the stream equals the number of surviving paths with a lower
// index, i.e. an exclusive scan of the "alive" flags.
__global__ void __launch_bounds__(1024) k_light(DevScene S, FrameArgs a, float4* cache, uint32_t cacheCap,
                                                DevCounters* ctr) {
  using namespace gb;
  __shared__ uint32_t warpCnt[32];
  const uint32_t x = threadIdx.x;
  const uint32_t NL = a.lightPaths;
  const uint32_t lane = x & 31, warp = x >> 5, nWarps = (blockDim.x + 31) >> 5;
  bool alive = (x < NL) && (S.lightN > 0);
  f3 orig = mk(0.f, 0.f, 0.f), dir = orig, outMul = mk(1.f, 1.f, 1.f), sample = orig;
  uint32_t depth = 0;
  if (alive) {
    float u[8];
    draw8(a.key0, a.key1, x, a.frame, kLightGen, 0, 0, u);
    uint32_t id = (uint32_t)(u[0] * (float)S.lightN);
    if (id >= S.lightN) id = S.lightN - 1;
    float lw = u[1], lu = u[2];
    if (lw + lu > 1.0f) {
      lw = 1.f - lw;
      lu = 1.f - lu;
    }
    float lvv = 1.f - lw - lu;
    Surf sf = load_surf(S, S.lightTri[id], lw, lu, lvv, true);
    Mat m = load_mat_at(S, sf.mat, S.lightTri[id], lw, lu, lvv);
    dir = cos_dir(u[3], u[4], sf.norm);
    orig = sf.pos + kBias * sf.norm;
    sample = m.emis;
    LV v;
    v.pos = sf.pos;
    v.norm = sf.norm;
    v.irrad = m.emis;
    v.irradDir = mk(0.f, 0.f, 0.f);
    v.diff = m.diff;
    v.emis = m.emis;
    v.spec = m.spec;
    v.metal = m.metal;
    v.rough = m.rough;
    store_lv(cache + 6 * (size_t)x, v);
  }
  uint32_t size = (S.lightN > 0) ? NL : 0;
  __syncthreads();
  for (;;) {
    uint32_t bal = __ballot_sync(0xffffffffu, alive);
    if (lane == 0) warpCnt[warp] = __popc(bal);
    __syncthreads();
    uint32_t before = 0, total = 0;
    for (uint32_t w = 0; w < nWarps; w++) {
      uint32_t c = warpCnt[w];
      if (w < warp) before += c;
      total += c;
    }
    __syncthreads();
    if (total == 0) break;
    if (alive) {
      uint32_t slot = size + before + __popc(bal & lanemask_lt());
      if (slot >= cacheCap) {
        atomicOr(&ctr->errFlags, 1u);
        alive = false;
      } else {
        float4* cs = cache + 6 * (size_t)slot;
        TraceHit h;
        uint32_t nn = 0, nt = 0;
        if (!trace_ref<false, false>(S, orig, dir, kInf, kBias, false, h, nn, nt)) {
          const float4* home = cache + 6 * (size_t)x;  // :358-362
          for (int k = 0; k < 6; k++) cs[k] = home[k];
          alive = false;
        } else {
          float u[8];
          draw8(a.key0, a.key1, x, a.frame, kLightBounce, depth, 0, u);
          float hw = 1.f - h.u - h.v;
          Surf sf = load_surf(S, h.tri, hw, h.u, h.v, true);
          Mat m = load_mat_at(S, sf.mat, h.tri, hw, h.u, h.v);
          Bounce B;
          sample_bounce(orig, dir, h.t, sf.norm, m, u, false, false, false, B);
          LV v;
          v.irrad = (B.type != kTypeDiff) ? mk(0.f, 0.f, 0.f) : sample;
          v.irradDir = -1.f * dir;
          v.norm = (dot(B.nDir, B.nl) < 0.f) ? -1.f * B.nl : B.nl;
          v.pos = sf.pos;
          v.diff = m.diff;
          v.emis = m.emis;
          v.spec = m.spec;
          v.metal = m.metal;
          v.rough = m.rough;
          store_lv(cs, v);
          sample = m.emis + vmul(sample, B.lmt);
          float contrib = length(outMul) * length(B.lmt);
          if (length(m.emis) > 0.f) contrib = 0.f;
          if (u[6] > contrib || depth + 1 >= a.lightDepth) {
            alive = false;
          } else {
            outMul = vmul(outMul, B.lmt);
            dir = B.nDir;
            orig = B.nOrig;
            depth++;
          }
        }
      }
    }
    size += total;
    __syncthreads();
  }
  if (x == 0) ctr->cacheSize[a.cacheSel] = size;
}

// ---------------------------------------------------------------------------
// Camera rays, one per pixel (pt_genPathQueue_kernel, :619-640), for the
// band's pixels b.base .. b.base + b.count - 1; a ray's wave index is its
// index inside the band.
// Wave item i of a whole-image wavefront -> its pixel: 4x8-pixel tiles, one
// warp's 32 camera rays per tile, tiles in row-major order, then the pixels
// right of and below the whole tiles in row-major order (a bijection for any
// width and height).  Camera rays of a compact tile walk more of the same
// nodes than a 32-pixel row: hall 1280x720 188.0 -> 190.1 Mpaths/s (8x4
// tiles 189.2, 16x2 187.8), interior even, Cornell 256x256 190.1 -> 187.2
// (cheap walks: its first-bounce slot writes in 4-pixel runs show).  Results
// do not depend on it: every path's random numbers and its slot follow from
// its pixel.
__device__ __forceinline__ uint32_t tiled_pixel(uint32_t i, uint32_t w, uint32_t h) {
  constexpr uint32_t TW = 4u, TH = 8u;
  const uint32_t tx = w / TW, ty = h / TH, nFull = tx * ty * TW * TH;
  if (i < nFull) {
    const uint32_t t = i / (TW * TH), k = i % (TW * TH);
    return ((t / tx) * TH + k / TW) * w + (t % tx) * TW + k % TW;
  }
  uint32_t j = i - nFull;
  const uint32_t rw = w - tx * TW, rightN = rw * ty * TH;
  if (j < rightN) return (j / rw) * w + tx * TW + j % rw;
  j -= rightN;
  return (ty * TH + j / w) * w + j % w;
}

__global__ void k_camera(FrameArgs a, RenderBuffers b) {
  using namespace gb;
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) {
    b.ctr->wave[0] = b.count;
    b.ctr->paths = b.count;
    b.ctr->fetchT = 0;
    b.ctr->carryN[0] = b.ctr->carryN[1] = b.ctr->carryN[2] = 0;
    b.ctr->fetchTail = 0;
    b.ctr->tailAt = 0xFFFFFFFFu;
  }
  if (i >= b.count) return;
  // local pixel (the band's range in row-major order when the frame is split)
  const uint32_t p = b.count == a.width * a.height ? tiled_pixel(i, a.width, a.height) : b.base + i;
  // pixel of the full image: its coordinates place the ray and its id keys
  // every random number of the path, so a window renders as in the full image
  const uint32_t x = a.winX0 + p % a.width, y = a.winY0 + p / a.width;
  const uint32_t gp = y * a.fullW + x;
  float u[4];
  draw4(a.key0, a.key1, gp, a.frame, kCamera, 0, 0, 0, u);
  const float W = a.W, H = a.H, th = a.tanHalf;
  float cu = ((((2.f * ((float)x + 0.5f)) / W) - 1.f) * th * W) / H;
  float cv = (((2.f * ((float)y + 0.5f)) / H) - 1.f) * th;
  float au = cu + ((u[0] - 0.5f) / H) * th;
  float av = cv + ((u[1] - 0.5f) / H) * th;
  f3 R = mk(a.camRight[0], a.camRight[1], a.camRight[2]);
  f3 U = mk(a.camUp[0], a.camUp[1], a.camUp[2]);
  f3 D = mk(a.camDir[0], a.camDir[1], a.camDir[2]);
  f3 dir = normalize((R * au + U * av) + D);
  Wave w = b.wave[0];
  w.o[i] = make_float4(a.camPos[0], a.camPos[1], a.camPos[2], __uint_as_float(p));
  w.d[i] = st4u(dir, gp);
  w.thr[i] = make_float4(1.f, 1.f, 1.f, 1.f);  // .w: path potential (filter-only mode)
  w.smp[i] = make_float4(0.f, 0.f, 0.f, 0.f);
  b.res[p] = make_float4(0.f, 0.f, 0.f, __uint_as_float(0u));
  b.slotPix[p] = p;
  b.slotSmp[p] = 0;
  if (a.gbuffer) {
    b.gbuf[3 * (size_t)p] = make_float4(0.f, 0.f, 0.f, 0.f);
    b.gbuf[3 * (size_t)p + 1] = make_float4(0.f, 0.f, 0.f, 0.f);
    b.gbuf[3 * (size_t)p + 2] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  if (a.bilat) b.dsm[p] = make_float4(0.f, 0.f, 0.f, 0.f);
}

// Direct-light sample of a bounce-0 connection that reached its light vertex
// (pt_connectEyeLightPath_kernel, src/cudaRTBDPTStreamBilat.cu:905-913):
// (direct + L) / 5 when any channel is positive, else L / 4.
__device__ __forceinline__ void direct_connect(float4* dsm, uint32_t slot, float4 C) {
  using namespace gb;
  const float4 q = dsm[slot];
  const f3 L = ld3(C);
  const f3 d = (q.x > 0.f || q.y > 0.f || q.z > 0.f) ? (ld3(q) + L) / 5.f : L / 4.f;
  dsm[slot] = st4(d, q.w);
}

__device__ __forceinline__ void warp_add_u64(unsigned long long* dst, uint32_t v) {
  uint32_t s = v;
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0 && s) atomicAdd(dst, (unsigned long long)s);
}

// ---------------------------------------------------------------------------
// One persistent kernel walks the BVH for the extension rays of bounce d
// (closest hit) and the shadow rays of bounce d-1 (any hit): the two sets
// are independent, so running them in one launch removes one kernel tail per
// bounce.  A lane takes a new ray as soon as its ray is finished (refill when
// at least kRefill lanes of the warp are idle), so warps stay full while rays
// last.  Shadow rays are handed out first: they cannot be carried to the next
// launch (a path's connection contributions are summed in bounce order), so
// the long ones must start early; then the walks the previous launch carried,
// then the extension rays (hall 1280x720: 181.4 -> 187.9 Mpaths/s against
// extension rays first; interior 169.0 -> 168.2).
// Every ray still visits nodes exactly in TracePrimitive's order, so per-ray
// results do not depend on this scheduling.  The any-hit walk stops at the
// first hit closer than maxDist: that is exactly when the reference's
// closest-hit walk with the same maxDist would report a hit.
// 4 resident CTAs per SM (64 registers, no spill) for both orders.  The
// reference order measured 1-2% faster at 5 (48 registers) than at 4 or 6
// before walks were carried and before 16-step batches; now (hall / interior
// / Cornell / hall adaptive, Mpaths/s) 3: 173.2 / 160.6 / 204.5 / 137.8, 4:
// 198.7 / 179.9 / 198.5 / 153.8, 5: 196.0 / 178.5 / 190.4 / 151.6, 6: 180.9 /
// 168.0 / 187.3 / 141.1.
// walk steps per refill check (measured in Mpaths/s on interior / hall /
// Cornell): reference order before carrying 1: 148.4 / 167.6 / 140.7, 2:
// 152.2 / 171.7 / 144.5, 4: 154.9 / 174.3 / 143.1, 6: 156.0 / 176.2 / 141.9,
// 8: 155.5 / 176.6 / 142.7; with carrying (a launch's end no longer waits on
// idle lanes) and refill at 2 idle lanes: hall / interior / hall adaptive 6
// (refill 8): 190.0 / 172.3 / 147.4, 12: 195.1 / 177.8 / 150.9, 16: 196.5 /
// 178.1 / 151.3, 24 (refill 4): 195.2 / 178.3 / 151.4; wide order 2: 170.0 /
// 180.7 / 159.2, 4: 171.2 / 181.8 / 157.4
template <bool kWide>
__host__ __device__ constexpr int walk_steps() {
  return kWide ? 2 : 16;
}

// Word 3.w of a carry record: the path's depth for an extension walk, this
// tag for a connection (shadow) walk, whose record holds the connection
// {origin, slot} {direction, maxDist} {contribution, bounce} instead of the path.
constexpr uint32_t kShadowRec = 0xFFFFFFFFu;

// One carried walk to carry record r (out of line: it runs for a few walks
// per launch, and keeping it out of the walk loop keeps that loop's
// registers): three float4 of the walk's ray at src, src + stride, src +
// 2 * stride (the path of a wave, or a connection record), the fourth at src
// + 3 * stride (the path's carried emission and depth) or the connection tag,
// then the walk's state and its node stack.
__device__ __noinline__ void save_carry(float4* r, const float4* src, size_t stride, bool shadow, float minT,
                                        uint32_t best, float bu, float bv, float bw, uint32_t steps, uint32_t tos,
                                        int sp, const uint32_t* stack) {
  r[0] = src[0];
  r[1] = src[stride];
  r[2] = src[2 * stride];
  r[3] = shadow ? make_float4(0.f, 0.f, 0.f, __uint_as_float(kShadowRec)) : src[3 * stride];
  r[4] = make_float4(minT, __uint_as_float(best), bu, bv);
  r[5] = make_float4(bw, __uint_as_float(steps), __uint_as_float(tos), __int_as_float(sp));
  for (int k = 0; k < 8; k++)
    r[6 + k] = make_float4(__uint_as_float(stack[4 * k]), __uint_as_float(stack[4 * k + 1]),
                           __uint_as_float(stack[4 * k + 2]), __uint_as_float(stack[4 * k + 3]));
}

// The walk of carry record r, resumed at the step where it stopped; true for
// a connection walk (any hit up to its maxDist).
__device__ __forceinline__ bool resume_walk(const float4* r, Walk& w, uint32_t* stack) {
  const float4 r1 = r[1];
  const bool shadow = __float_as_uint(r[3].w) == kShadowRec;
  w.init(ld3(r[0]), ld3(r1), shadow ? r1.w : gb::kInf, gb::kBias, stack);
  const float4 q = r[4], z = r[5];
  w.minT = q.x;
  w.best = __float_as_uint(q.y);
  w.bu = q.z;
  w.bv = q.w;
  w.bw = z.x;
  w.steps = __float_as_uint(z.y);
  w.tos = __float_as_uint(z.z);
  w.sp = __float_as_int(z.w);
#pragma unroll
  for (int k = 0; k < 8; k++) {
    const float4 e = r[6 + k];
    stack[4 * k] = __float_as_uint(e.x);
    stack[4 * k + 1] = __float_as_uint(e.y);
    stack[4 * k + 2] = __float_as_uint(e.z);
    stack[4 * k + 3] = __float_as_uint(e.w);
  }
  return shadow;
}

// An unoccluded connection: its contribution into the slot's entry for the
// bounce that made it (summed with the path's other connections, in bounce
// order, by k_fold once every walk of the frame is done).
__device__ __forceinline__ void connection_reached(const RenderBuffers& b, uint32_t bilat, float4 A, float4 C) {
  const uint32_t slot = __float_as_uint(A.w), bounce = __float_as_uint(C.w);
  b.conn[(size_t)bounce * b.cap + slot] = make_float4(C.x, C.y, C.z, 1.f);
  if (bilat && bounce == 0u) direct_connect(b.dsm, slot, C);
}

// walks carried out of bounce launch L (buffer L & 1, counter L % 3; the
// counter of launch L + 1 is reset by launch L, after its last reader)
__device__ __forceinline__ uint32_t carried_of(const RenderBuffers& b, uint32_t launch) {
  return b.carry[0] ? min(b.ctr->carryN[launch % 3u], b.carryCap) : 0u;
}

// Carrying (reference order only): once the launch's ray queue is empty, a
// warp keeps stepping its walks for carrySteps more steps; walks still
// unfinished then are written, with their path (or connection) and complete
// walk state, to the launch's carry buffer, an extension walk's hit word
// marked -2 (k_shade skips it).  The next bounce launch resumes them after its
// shadow rays (items nS .. nS+nC-1; their hit words after its own extension
// rays' at nE + k, -2 for a connection) and its shading kernel shades the
// extension walks at their own depth, one bounce behind the paths around
// them; the tail kernel takes those of the last bounce launch.  Results are
// unchanged: every random number is keyed by the path's own depth, and
// connections do not add to the slot when their walk ends but store their
// contribution per bounce, summed in bounce order by k_fold (a path's
// connections may now finish out of order).  The filter-only mode's bounce-0
// connections, whose direct-light sample is read by the next bounce's
// shading, are never carried.
template <bool kCount, bool kWide>
__global__ void __launch_bounds__(kBlock, 4) k_walk(DevScene S, RenderBuffers b, int in, int shIn,
                                                              int shReset, uint32_t bilat, uint32_t kRefill,
                                                              uint32_t launch, uint32_t carrySteps) {
  if (b.ctr->tailAt <= launch) return;  // the frame's tail kernel carries this bounce
  const uint32_t nC = (!kWide && in >= 0 && launch > 0) ? carried_of(b, launch - 1) : 0u;
  const uint32_t nE = (in >= 0) ? b.ctr->wave[in] : 0u;
  const uint32_t nS = (shIn >= 0) ? b.ctr->shadow[shIn] : 0u;
  const uint32_t nCE = nC + nE;
  const uint32_t n = nCE + nS;
  uint32_t* fetch = &b.ctr->fetchT;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    atomicAdd(&b.ctr->rays, (unsigned long long)nS);
    atomicAdd(&b.ctr->shadowRays, (unsigned long long)nS);
    if (in >= 0) b.ctr->wave[in ^ 1] = 0;
    b.ctr->shadow[shReset] = 0;
    b.ctr->carryN[(launch + 1) % 3u] = 0;
  }
  const Wave wv = b.wave[in >= 0 ? in : 0];
  const float4* __restrict__ sh = b.sh[shIn >= 0 ? shIn : 0];
  const float4* prev = b.carry[(launch + 1) & 1u];  // launch - 1's carried walks
  const uint32_t lane = threadIdx.x & 31;
  typename WalkOf<kWide>::type w;
  typename WalkOf<kWide>::Entry stack[WalkOf<kWide>::kDepth];
  bool has = false, drained = false, any = false, res = false;
  uint32_t item = 0, nnE = 0, ntE = 0, nnS = 0, ntS = 0;
  uint32_t dryFor = 0;  // walk steps since this warp found the queue empty
  for (;;) {
    const uint32_t idle = __ballot_sync(0xffffffffu, !has);
    if (idle == 0xffffffffu && drained) break;
    if constexpr (!kWide) {
      if (carrySteps && drained && in >= 0) {
        // once per warp, carrySteps steps after it found the queue empty: its
        // walks still running take carry records with one atomic for the warp
        // (walks that find the buffer full finish here)
        if (dryFor >= carrySteps && dryFor < carrySteps + walk_steps<kWide>()) {
          const float4* src = res ? prev + (size_t)item * kCarryF4 : (any ? sh + 3 * (size_t)item : wv.o + item);
          const bool want = has && !(any && bilat && __float_as_uint(src[2].w) == 0u);
          const uint32_t m = __ballot_sync(0xffffffffu, want);
          uint32_t c0 = 0;
          if (m && lane == 0) c0 = atomicAdd(&b.ctr->carryN[launch % 3u], (uint32_t)__popc(m));
          c0 = __shfl_sync(0xffffffffu, c0, 0) + __popc(m & lanemask_lt());
          if (want && c0 < b.carryCap) {
            save_carry(b.carry[launch & 1u] + (size_t)c0 * kCarryF4, src, (res || any) ? 1 : (size_t)(wv.d - wv.o),
                       any && !res, w.minT, w.best, w.bu, w.bv, w.bw, w.steps, w.tos, w.sp, stack);
            if (res || !any) b.hit[res ? nE + item : item] = make_float4(-2.f, 0.f, 0.f, 0.f);
            has = false;
          }
        }
        dryFor += walk_steps<kWide>();
      }
    }
    if (!drained && (idle == 0xffffffffu || __popc(idle) >= kRefill)) {
      const uint32_t cnt = __popc(idle);
      uint32_t base = 0;
      if (lane == 0) base = atomicAdd(fetch, cnt);
      base = __shfl_sync(0xffffffffu, base, 0);
      if (base + cnt >= n) drained = true;
      if (!has) {
        const uint32_t k = base + __popc(idle & lanemask_lt());
        if (k < n) {
          has = true;
          any = k < nS;
          res = !any && k < nS + nC;
          item = any ? k : (res ? k - nS : k - nS - nC);
          if (res) {
            if constexpr (!kWide) any = resume_walk(prev + (size_t)item * kCarryF4, w, stack);
          } else if (any) {
            const float4 A = sh[3 * (size_t)item], B = sh[3 * (size_t)item + 1];
            w.init(ld3(A), ld3(B), B.w, gb::kBias, stack);
          } else {
            w.init(ld3(wv.o[item]), ld3(wv.d[item]), gb::kInf, gb::kBias, stack);
          }
        }
      }
    }
    // walk_steps() steps per refill check: the ballot and refill test are paid
    // once for them (a lane whose walk ends in the first waits out the rest)
#pragma unroll 1
    for (int u = 0; u < walk_steps<kWide>(); u++) {
      // one inlined walk step for both ray kinds (a runtime any-hit flag), so a
      // warp holding extension and shadow rays does not run two copies of it;
      // the counting variant keeps separate counters per kind
      bool fin = false;
      if (has) {
        if (kCount)
          fin = any ? w.template step<kCount>(S, stack, true, nnS, ntS) : w.template step<kCount>(S, stack, false, nnE, ntE);
        else
          fin = w.template step<kCount>(S, stack, any, nnE, ntE);
      }
      if (fin) {
        has = false;
        if (any) {
          const float4* q = res ? prev + (size_t)item * kCarryF4 : sh + 3 * (size_t)item;
          if (!w.hit()) connection_reached(b, bilat, q[0], q[2]);  // unoccluded: it counts (:716-721)
          if (res) b.hit[nE + item] = make_float4(-2.f, 0.f, 0.f, 0.f);
        } else {
          b.hit[res ? nE + item : item] = w.hit() ? make_float4(w.minT, __uint_as_float(w.best), w.bu, w.bv)
                                                  : make_float4(-1.f, 0.f, 0.f, 0.f);
        }
      }
    }
  }
  if (kCount) {
    warp_add_u64(&b.ctr->nodes, nnE);
    warp_add_u64(&b.ctr->tris, ntE);
    warp_add_u64(&b.ctr->nodesS, nnS);
    warp_add_u64(&b.ctr->trisS, ntS);
  }
}

// ---------------------------------------------------------------------------
// Shading of one path after its closest-hit walk (pt_traceSample_kernel after
// TracePrimitive, src/cudaRTBDPTStream.cu:381-543) and the connection set-up
// of GetLightFromRandLightVertices / pt_connectEyeLightPath_kernel
// (:665-723): everything but the visibility test, which the shadow walk does.
// io holds the path (origin+slot, direction+pixel, throughput, carried
// emission) on entry and the next ray's state on exit when cont is set.
struct PathIO {
  float4 o, d, t, s;
  bool cont, conn;
  float4 shA, shB, shC;
};

// learned allocator statistics: a finished path of pixel `pix` after `hits`
// surface hits, counted in its 8x8 tile's path-length histogram
__device__ __forceinline__ void count_path_length(const FrameArgs& a, const RenderBuffers& b, uint32_t pix,
                                                  uint32_t hits) {
  const uint32_t px = pix % a.width, py = pix / a.width;
  const uint32_t tile = (py >> 3) * a.tilesX + (px >> 3);
  atomicAdd(&b.hist[tile * 8u + (hits < 7u ? hits : 7u)], 1u);
}

__device__ __forceinline__ void shade_path(const DevScene& S, const FrameArgs& a, const RenderBuffers& b,
                                           const float4* __restrict__ cache, uint32_t cacheSize, uint32_t depth,
                                           float4 h4, PathIO& io) {
  using namespace gb;
  io.cont = false;
  io.conn = false;
  const uint32_t slot = __float_as_uint(io.o.w);
  const uint32_t pix = __float_as_uint(io.d.w);
  f3 orig = ld3(io.o), dir = ld3(io.d), outMul = ld3(io.t), pathSample = ld3(io.s);
  float pot = io.t.w;  // path potential (filter-only mode)
  if (h4.x < 0.f) {  // miss (:537-542), plus the optional environment term
    if (a.useEnv) pathSample = pathSample + vmul(mk(a.env[0], a.env[1], a.env[2]), outMul);
    // the path's end: its emission and how many bounces' connections k_fold sums before it
    b.res[slot] = make_float4(pathSample.x, pathSample.y, pathSample.z, __uint_as_float(depth));
    if (a.bilat) reinterpret_cast<float*>(b.dsm + slot)[3] = pot;
    if (a.moments) count_path_length(a, b, pix, depth);
    return;
  }
  const uint32_t smp = b.slotSmp[slot];
  float u[8];
  draw8(a.key0, a.key1, pix, a.frame, kEyeBounce, depth, smp, u);
  const float hu = h4.z, hv = h4.w, hw = 1.f - hu - hv;
  Surf sf = load_surf(S, __float_as_uint(h4.y), hw, hu, hv, a.gbuffer && depth == 0);
  Mat m = load_mat_at(S, sf.mat, __float_as_uint(h4.y), hw, hu, hv);
  Bounce B;
  sample_bounce(orig, dir, h4.x, sf.norm, m, u, a.specPush != 0, a.bilat != 0, a.ptsc != 0, B);
  pathSample = pathSample + vmul(m.emis, outMul);
  if (a.gbuffer && depth == 0) {  // AdapBilatAtomic.cu:471-476, Bilat.cu:632-638
    const bool be = a.bilat != 0;
    b.gbuf[3 * (size_t)slot] = st4(sf.pos, be ? m.emis.x : 0.f);
    b.gbuf[3 * (size_t)slot + 1] = st4(B.nl, be ? m.emis.y : 0.f);
    b.gbuf[3 * (size_t)slot + 2] = st4(m.diff, be ? m.emis.z : 0.f);
  }
  if (a.bilat) {  // Bilat.cu:628-631
    pot = pot * B.pdf;
    if (depth < 2) {
      const float4 q = b.dsm[slot];
      b.dsm[slot] = make_float4(q.x + pathSample.x, q.y + pathSample.y, q.z + pathSample.z, q.w);
    }
  }
  const f3 inMul = outMul;
  float contrib = length(outMul) * length(B.lmt);
  if (length(m.emis) > 0.f) contrib = 0.f;
  if (u[6] > contrib || depth + 1 >= a.eyeDepth) {
    b.res[slot] = make_float4(pathSample.x, pathSample.y, pathSample.z, __uint_as_float(depth));
    if (a.bilat) reinterpret_cast<float*>(b.dsm + slot)[3] = pot;
    if (a.moments) count_path_length(a, b, pix, depth + 1);
    return;
  }
  io.cont = true;
  b.conn[(size_t)depth * b.cap + slot] = make_float4(0.f, 0.f, 0.f, 0.f);  // none, until a connection walk says
  outMul = vmul(outMul, B.lmt);
  io.o = st4u(B.nOrig, slot);
  io.d = st4u(B.nDir, pix);
  io.t = st4(outMul, pot);
  io.s = make_float4(pathSample.x, pathSample.y, pathSample.z, __uint_as_float(depth + 1));
  if (B.type != kTypeDiff || cacheSize == 0 || a.ptsc) return;
  // connection: pick a cached light vertex, shade both ends (:665-723)
  f3 pos = B.nOrig + B.nl * kBias;
  uint32_t li = (uint32_t)(u[7] * (float)cacheSize);
  if (li >= cacheSize) li = cacheSize - 1;
  LV lv = load_lv(cache + 6 * (size_t)li);
  f3 toDir = normalize(lv.pos - pos);
  float toDist = length(lv.pos - pos);
  if (!(length(lv.irrad) > 0.f && dot(B.nl, toDir) > 0.f)) return;
  f3 irrad, irradDir;
  if (toDist > kFltEps) {
    irrad = shading(-1.f * toDir, lv.irradDir, lv.irrad, lv.norm, lv.diff, lv.metal, lv.rough, lv.spec, 1.f, 1.f) +
            lv.emis;
    irradDir = toDir;
  } else {
    irrad = lv.irrad;
    irradDir = -1.f * lv.irradDir;
  }
  f3 c = vmax0(shading(-1.f * dir, irradDir, irrad, B.nl, m.diff, m.metal, m.rough, m.spec, 1.f - m.trans, 1.f));
  if (length(c) > 0.f) {
    io.conn = true;
    io.shA = st4u(pos, slot);
    io.shB = st4(toDir, toDist - kBias);
    const f3 cw = vmul(c, inMul);
    io.shC = make_float4(cw.x, cw.y, cw.z, __uint_as_float(depth));  // .w: the bounce that made it
  }
}

// Shading of bounce launch L: the paths of its wave, then the walks it
// resumed for launch L - 1 (carry records, their hits after the wave's), each
// at its own depth; survivors are appended to the other wave buffer and
// connection requests to queue L & 1, one atomic per warp each.
// attach != 0 (the last bounce launch before the tail kernel): each continuing
// path's connection record is stored at the path's own index j of queue
// L & 1 (slot word 0xffffffff when it has none), so that the tail kernel
// walks it on the path's lane before the path's next bounce.  Three CTAs per
// SM (80 registers, a few bytes of spill) beat two at 96 registers: shading
// time -10 to -12% on the interior and hall walks.
__global__ void __launch_bounds__(kBlock, 3) k_shade(DevScene S, FrameArgs a, RenderBuffers b, int in, uint32_t launch,
                                                     uint32_t attach) {
  if (b.ctr->tailAt <= launch) return;  // the frame's tail kernel carries this bounce
  const uint32_t n = b.ctr->wave[in];
  const uint32_t nC = launch > 0 ? carried_of(b, launch - 1) : 0u;
  const uint32_t total = n + nC;
  // the switch decided on the device: with fewer than tailBelow x the band's
  // camera paths alive at this launch, the paths that continue go to the tail
  // kernel from the next launch (every CTA reads the same counts and decides alike)
  if (!attach && a.tailBelow > 0.f && launch + 1 < a.eyeDepth && (float)total < a.tailBelow * (float)b.ctr->paths)
    attach = 2u;
  const uint32_t cacheSize = b.lctr->cacheSize[a.cacheSel];
  const float4* __restrict__ cache = b.cache[a.cacheSel];
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    atomicAdd(&b.ctr->rays, (unsigned long long)n);  // resumed walks were counted by their own launch
    b.ctr->fetchT = 0;  // for the next walk (next bounce's rays + this bounce's shadow rays)
    if (attach == 2u) b.ctr->tailAt = launch + 1;
  }
  const Wave w = b.wave[in];
  const Wave wo = b.wave[in ^ 1];
  const float4* prev = b.carry[(launch + 1) & 1u];
  const uint32_t stride = gridDim.x * blockDim.x;
  const uint32_t lane = threadIdx.x & 31;
  float4* shq = b.sh[launch & 1u];
  for (uint32_t base = blockIdx.x * blockDim.x; base < total; base += stride) {
    const uint32_t i = base + threadIdx.x;
    PathIO io;
    io.cont = io.conn = false;
    if (i < total) {
      const float4 h = b.hit[i];
      if (h.x != -2.f) {  // -2: the walk was carried on, to the next launch or the tail kernel
        if (i < n) {
          io.o = w.o[i];
          io.d = w.d[i];
          io.t = w.thr[i];
          io.s = w.smp[i];
        } else {
          const float4* r = prev + (size_t)(i - n) * kCarryF4;
          io.o = r[0];
          io.d = r[1];
          io.t = r[2];
          io.s = r[3];
        }
        shade_path(S, a, b, cache, cacheSize, __float_as_uint(io.s.w), h, io);
      }
    }
    const uint32_t mc = __ballot_sync(0xffffffffu, io.cont);
    if (mc) {
      uint32_t basej = 0;
      if (lane == 0) basej = atomicAdd(&b.ctr->wave[in ^ 1], __popc(mc));
      basej = __shfl_sync(0xffffffffu, basej, 0);
      if (io.cont) {
        const uint32_t j = basej + __popc(mc & lanemask_lt());
        wo.o[j] = io.o;
        wo.d[j] = io.d;
        wo.thr[j] = io.t;
        wo.smp[j] = io.s;
        if (attach) {
          shq[3 * (size_t)j] = io.conn ? io.shA : make_float4(0.f, 0.f, 0.f, __uint_as_float(0xffffffffu));
          shq[3 * (size_t)j + 1] = io.shB;
          shq[3 * (size_t)j + 2] = io.shC;
        }
      }
    }
    if (attach) continue;
    const uint32_t ms = __ballot_sync(0xffffffffu, io.conn);
    if (ms) {
      uint32_t basej = 0;
      if (lane == 0) basej = atomicAdd(&b.ctr->shadow[launch & 1u], __popc(ms));
      basej = __shfl_sync(0xffffffffu, basej, 0);
      if (io.conn) {
        const uint32_t j = basej + __popc(ms & lanemask_lt());
        shq[3 * (size_t)j] = io.shA;
        shq[3 * (size_t)j + 1] = io.shB;
        shq[3 * (size_t)j + 2] = io.shC;
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Tail of a frame: once few paths are left, per-bounce launches are bounded
// by their slowest ray.  This persistent kernel instead carries every path
// of the wave left by the last bounce launch run (t, the switch bounce or K)
// through all its remaining bounces on one lane, each at its own depth: the
// connection attached to it by that launch (queue (t - 1) & 1, same index;
// slot word 0xffffffff: none), then closest-hit walk, shading, connection and
// shadow walk bounce after bounce; then the walks that launch carried,
// resumed where they stopped.  A path executes exactly the operations of the
// wavefront kernels in the same order (a connection is applied before the
// next bounce is shaded), so results are identical.
enum : uint32_t { kIdle = 0, kPathExt = 1, kPathShadow = 2 };

// walk steps of the tail kernel between two refill checks: a lane whose walk
// ends early waits for the others, and the warp then shades its finished
// paths together.  Measured in Mpaths/s on interior / Cornell before walks
// were carried (the hall then ran no tail kernel): 1: 154.4 / 144.2, 4:
// 157.5 / 158.7, 16: 161.1 / 171.4, 64: 162.3 / 189.1, 512: 156.7 / 197.4;
// with carrying and 16-step walk batches (hall / interior / Cornell): 32:
// 194.3 / 175.4 / 171.6, 64: 195.9 / 178.8 / 190.4, 128: 195.2 / 178.1 /
// 192.7.  Three CTAs per SM (80 registers, some spill) against two (116
// registers): interior 167.0 -> 170.0, Cornell 195.6 -> 193.6 Mpaths/s; four
// (64 registers): hall 195.9 -> 194.6, Cornell 190.4 -> 183.1.
__host__ __device__ constexpr int tail_steps() { return 64; }

template <bool kCount, bool kWide>
__global__ void __launch_bounds__(kBlock, 3) k_tail(DevScene S, FrameArgs a, RenderBuffers b, uint32_t K,
                                                   uint32_t kRefill) {
  // t: the launch the bounce launches stopped before (the device switch or K)
  const uint32_t t = min(b.ctr->tailAt, K);
  const int in = (int)(t & 1u);
  const int shIn = t > 0 ? (int)((t - 1) & 1u) : -1;
  const uint32_t n = b.ctr->wave[in];
  const uint32_t nCarry = t > 0 ? carried_of(b, t - 1) : 0u;
  const float4* carried = b.carry[(t + 1) & 1u];  // launch t - 1's
  const uint32_t total = n + nCarry;
  const uint32_t cacheSize = b.lctr->cacheSize[a.cacheSel];
  const float4* __restrict__ cache = b.cache[a.cacheSel];
  const float4* __restrict__ sh = b.sh[shIn >= 0 ? shIn : 0];
  const Wave wv = b.wave[in];
  const uint32_t lane = threadIdx.x & 31;
  typename WalkOf<kWide>::type w;
  typename WalkOf<kWide>::Entry stack[WalkOf<kWide>::kDepth];
  PathIO io;
  uint32_t mode = kIdle;
  bool drained = false, resumed = false;
  uint32_t extRays = 0, shRays = 0, nnE = 0, ntE = 0, nnS = 0, ntS = 0;
  for (;;) {
    const uint32_t idle = __ballot_sync(0xffffffffu, mode == kIdle);
    if (idle == 0xffffffffu && drained) break;
    if (!drained && (idle == 0xffffffffu || __popc(idle) >= kRefill)) {
      const uint32_t cnt = __popc(idle);
      uint32_t base = 0;
      if (lane == 0) base = atomicAdd(&b.ctr->fetchTail, cnt);
      base = __shfl_sync(0xffffffffu, base, 0);
      if (base + cnt >= total) drained = true;
      if (mode == kIdle) {
        const uint32_t j = base + __popc(idle & lanemask_lt());
        if (j >= n && j < total) {  // a carried walk: resume it where it stopped
          const float4* r = carried + (size_t)(j - n) * kCarryF4;
          resumed = true;
          if constexpr (!kWide) {
            if (resume_walk(r, w, stack)) {  // a connection alone, without its path
              io.shA = r[0];
              io.shB = r[1];
              io.shC = r[2];
              mode = kPathShadow;
            } else {
              io.o = r[0];
              io.d = r[1];
              io.t = r[2];
              io.s = r[3];
              mode = kPathExt;
            }
          }
        } else if (j < n) {
          io.o = wv.o[j];
          io.d = wv.d[j];
          io.t = wv.thr[j];
          io.s = wv.smp[j];
          const float4 A = (shIn >= 0) ? sh[3 * (size_t)j] : make_float4(0.f, 0.f, 0.f, __uint_as_float(0xffffffffu));
          if (__float_as_uint(A.w) != 0xffffffffu) {
            io.shA = A;
            io.shB = sh[3 * (size_t)j + 1];
            io.shC = sh[3 * (size_t)j + 2];
            mode = kPathShadow;
            w.init(ld3(io.shA), ld3(io.shB), io.shB.w, gb::kBias, stack);
          } else {
            mode = kPathExt;
            w.init(ld3(io.o), ld3(io.d), gb::kInf, gb::kBias, stack);
          }
        }
      }
    }
    if (mode == kIdle) continue;
    const bool anyHit = mode == kPathShadow;
    bool done = false;
#pragma unroll 1
    for (int u = 0; u < tail_steps() && !done; u++)
      done = kCount ? (anyHit ? w.template step<kCount>(S, stack, true, nnS, ntS)
                              : w.template step<kCount>(S, stack, false, nnE, ntE))
                    : w.template step<kCount>(S, stack, anyHit, nnE, ntE);
    if (!done) continue;
    if (anyHit) {
      if (!w.hit()) connection_reached(b, a.bilat, io.shA, io.shC);  // unoccluded connection (:716-721)
      if (resumed) {  // a carried connection alone (counted by its launch): done
        resumed = false;
        mode = kIdle;
        continue;
      }
      shRays++;
      mode = kPathExt;  // the path's next extension ray
      w.init(ld3(io.o), ld3(io.d), gb::kInf, gb::kBias, stack);
      continue;
    }
    // closest hit of the path's current ray: shade it (a resumed walk was
    // counted by the bounce launch's shading kernel)
    if (!resumed) extRays++;
    resumed = false;
    const float4 h4 = w.hit() ? make_float4(w.minT, __uint_as_float(w.best), w.bu, w.bv)
                              : make_float4(-1.f, 0.f, 0.f, 0.f);
    shade_path(S, a, b, cache, cacheSize, __float_as_uint(io.s.w), h4, io);
    if (!io.cont) {
      mode = kIdle;
    } else {
      if (io.conn) {
        mode = kPathShadow;
        w.init(ld3(io.shA), ld3(io.shB), io.shB.w, gb::kBias, stack);
      } else {
        w.init(ld3(io.o), ld3(io.d), gb::kInf, gb::kBias, stack);
      }
    }
  }
  warp_add_u64(&b.ctr->rays, extRays + shRays);
  warp_add_u64(&b.ctr->shadowRays, shRays);
  if (kCount) {
    warp_add_u64(&b.ctr->nodes, nnE);
    warp_add_u64(&b.ctr->tris, ntE);
    warp_add_u64(&b.ctr->nodesS, nnS);
    warp_add_u64(&b.ctr->trisS, ntS);
  }
}

// ---------------------------------------------------------------------------
// Sum of each path of the band, once all its walks are done: the unoccluded
// connections of bounces 0 .. k-1 in bounce order, then the path's emission
// at its end (bounce k), with the count word the accumulation kernels read
// (4 per connection, 1 for the end): the additions the reference makes into
// the path's result as each connection and the end happen (:716-721,
// :520-542), in the same order, so the sums are equal to the bit.
__global__ void k_fold(RenderBuffers b) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= b.ctr->paths) return;
  const uint32_t s = b.base + i;
  const float4 e = b.res[s];
  const uint32_t k = min(__float_as_uint(e.w), b.connDepth);
  float x = 0.f, y = 0.f, z = 0.f;
  uint32_t n = 0;
  for (uint32_t d = 0; d < k; d++) {
    const float4 c = b.conn[(size_t)d * b.cap + s];
    if (c.w != 0.f) {
      x = x + c.x;
      y = y + c.y;
      z = z + c.z;
      n += 4u;
    }
  }
  b.res[s] = make_float4(x + e.x, y + e.y, z + e.z, __uint_as_float(n + 1u));
}

// ---------------------------------------------------------------------------
// Running mean of one path per pixel (pt_applyPathQueueResult_kernel :741-778);
// with G-buffer planes, also the count-weighted first-hit means
// (AdapBilatAtomic.cu:929-966).
__global__ void k_apply(FrameArgs a, RenderBuffers b, float* result, uint32_t* sampleN, float* gpos, float* gnorm,
                        float* gdiff) {
  const uint32_t np = a.width * a.height;
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= np) return;
  const float4 r = b.res[p];
  const uint32_t n = __float_as_uint(r.w);
  if (n == 0) return;
  uint32_t old = (a.frame == 0) ? 0u : sampleN[p];
  if (a.frame == 0) sampleN[p] = 0;
  const uint32_t nn = old + n;
  if (!(nn > old)) return;
  if (isinf(r.x) || isinf(r.y) || isinf(r.z)) return;
  const float rInf = 1.f / (float)nn;
  const float oInf = (float)old * rInf;
  float* q = result + 3 * (size_t)p;
  q[0] = fmaxf(rInf * r.x + oInf * q[0], 0.f);
  q[1] = fmaxf(rInf * r.y + oInf * q[1], 0.f);
  q[2] = fmaxf(rInf * r.z + oInf * q[2], 0.f);
  sampleN[p] = nn;
  if (a.moments) {  // running mean of acc^2 / n (the path's second moment weighted like its mean)
    const float fn = (float)n;
    float* m = b.m2 + 3 * (size_t)p;
    const float s0 = (r.x * r.x) / fn, s1 = (r.y * r.y) / fn, s2 = (r.z * r.z) / fn;
    m[0] = old ? rInf * s0 + oInf * m[0] : rInf * s0;
    m[1] = old ? rInf * s1 + oInf * m[1] : rInf * s1;
    m[2] = old ? rInf * s2 + oInf * m[2] : rInf * s2;
  }
  if (gpos) {
    float* planes[3] = {gpos, gnorm, gdiff};
    const float fn = (float)n;
    for (int k = 0; k < 3; k++) {
      float4 g = b.gbuf[3 * (size_t)p + k];
      float* o = planes[k] + 3 * (size_t)p;
      o[0] = rInf * (g.x * fn) + oInf * o[0];
      o[1] = rInf * (g.y * fn) + oInf * o[1];
      o[2] = rInf * (g.z * fn) + oInf * o[2];
    }
  }
}

// Filter-only mode (pt_applyPathQueueResult_kernel of
// src/cudaRTBDPTStreamBilat.cu:989-1051): the running means have no inf test
// here; direct light and 1 - potential are running means too; the first-hit
// planes hold this frame's values.
__global__ void k_apply_bilat(FrameArgs a, RenderBuffers b, float* result, uint32_t* sampleN, float* gpos,
                              float* gnorm, float* gdiff, float* gemis, float* direct, float* pot) {
  const uint32_t np = a.width * a.height;
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= np) return;
  const float4 r = b.res[p];
  const uint32_t n = __float_as_uint(r.w);
  if (n == 0) return;
  uint32_t old = (a.frame == 0) ? 0u : sampleN[p];
  if (a.frame == 0) sampleN[p] = 0;
  const uint32_t nn = old + n;
  if (!(nn > old)) return;
  const float rInf = 1.f / (float)nn;
  const float oInf = (float)old * rInf;
  const float4 ds = b.dsm[p];
  float* q = result + 3 * (size_t)p;
  q[0] = fmaxf(rInf * r.x + oInf * q[0], 0.f);
  q[1] = fmaxf(rInf * r.y + oInf * q[1], 0.f);
  q[2] = fmaxf(rInf * r.z + oInf * q[2], 0.f);
  pot[p] = fmaxf(rInf * (1.f - ds.w) + oInf * pot[p], 0.f);
  sampleN[p] = nn;
  float* dq = direct + 3 * (size_t)p;
  dq[0] = rInf * ds.x + oInf * dq[0];
  dq[1] = rInf * ds.y + oInf * dq[1];
  dq[2] = rInf * ds.z + oInf * dq[2];
  const float4 g0 = b.gbuf[3 * (size_t)p], g1 = b.gbuf[3 * (size_t)p + 1], g2 = b.gbuf[3 * (size_t)p + 2];
  const size_t o = 3 * (size_t)p;
  gpos[o] = g0.x, gpos[o + 1] = g0.y, gpos[o + 2] = g0.z;
  gnorm[o] = g1.x, gnorm[o + 1] = g1.y, gnorm[o + 2] = g1.z;
  gemis[o] = g0.w, gemis[o + 1] = g1.w, gemis[o + 2] = g2.w;
  gdiff[o] = g2.x, gdiff[o + 1] = g2.y, gdiff[o + 2] = g2.z;
}

// Unidirectional mode: one path per pixel, weights of the frame index.
__global__ void k_apply_pt(FrameArgs a, RenderBuffers b, float* result, uint32_t* sampleN) {
  using namespace gb;
  const uint32_t np = a.width * a.height;
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= np) return;
  const float4 r = b.res[p];
  const uint32_t n = __float_as_uint(r.w);
  if (n == 0) return;
  const f3 smp = ld3(r) / (float)n;
  const float rInf = 1.f / (float)(a.frame + 1);
  const float oInf = 1.f - rInf;
  float* q = result + 3 * (size_t)p;
  q[0] = fmaxf(rInf * smp.x + oInf * q[0], 0.f);
  q[1] = fmaxf(rInf * smp.y + oInf * q[1], 0.f);
  q[2] = fmaxf(rInf * smp.z + oInf * q[2], 0.f);
  sampleN[p] = a.frame + 1;  // frames so far (the reference keeps no count in this mode)
}

__global__ void k_prob_view(const float* pot, uint32_t np, float minProb, float* out) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= np) return;
  const float v = fmaxf(minProb, pot[p]);
  out[3 * (size_t)p] = v;
  out[3 * (size_t)p + 1] = v;
  out[3 * (size_t)p + 2] = v;
}

// ---------------------------------------------------------------------------
// Stand-alone TracePrimitive for caller-supplied rays.
template <bool kCount>
__global__ void k_trace_rays(DevScene S, const float* rays, uint32_t n, float maxDist, float eps, int cullback,
                             float* t, int32_t* tri, float* w, float* u, float* v, uint32_t* nodes,
                             uint32_t* trisTested) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float* r = rays + 6 * (size_t)i;
  TraceHit h;
  uint32_t nn = 0, nt = 0;
  bool hit;
  if (S.traversal == 1 && S.wide && !cullback) {  // wide order (no back-face culling there)
    Walk4 wk;
    uint2 stack[kWideDepth];
    wk.init(mk(r[0], r[1], r[2]), mk(r[3], r[4], r[5]), maxDist, eps, stack);
    while (!wk.step<kCount>(S, stack, false, nn, nt)) {
    }
    hit = wk.hit();
    h.t = wk.minT;
    h.tri = wk.best;
    h.w = wk.bw;
    h.u = wk.bu;
    h.v = wk.bv;
  } else {
    hit = trace_ref<false, kCount>(S, mk(r[0], r[1], r[2]), mk(r[3], r[4], r[5]), maxDist, eps, cullback != 0, h,
                                   nn, nt);
  }
  t[i] = hit ? h.t : -1.f;
  tri[i] = hit ? (int32_t)h.tri : -1;
  w[i] = hit ? h.w : 0.f;
  u[i] = hit ? h.u : 0.f;
  v[i] = hit ? h.v : 0.f;
  if (kCount) {
    nodes[i] = nn;
    trisTested[i] = nt;
  }
}

int g_sm = 0;

// Idle lanes of a warp that trigger a refill in k_walk / k_tail (tuning
// knob, GBPT_WALK_REFILL, 1..32; 0 when unset).  Defaults, measured on the
// interior, hall and Cornell workloads: 8 for the reference order (4-10
// within 1%, 20 3-4% slower), 20 for the wide order (10-20 within 1%, 4 2-3%
// slower).
uint32_t walk_refill_env() {
  static uint32_t v = [] {
    const char* e = std::getenv("GBPT_WALK_REFILL");
    if (!e) return 0u;
    int x = std::atoi(e);
    return (uint32_t)(x < 1 ? 1 : x > 32 ? 32 : x);
  }();
  return v;
}

uint32_t grid_for(const void* kernel, size_t smem = 0) {
  int per = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, kBlock, smem);
  if (per < 1) per = 1;
  return (uint32_t)(sm_count() * per);
}

}  // namespace

static std::atomic<uint64_t> g_launches{0};
void note_launches(uint32_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
uint64_t launch_count() { return g_launches.load(std::memory_order_relaxed); }

int sm_count() {
  if (!g_sm) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_sm, cudaDevAttrMultiProcessorCount, dev);
    if (g_sm <= 0) g_sm = 1;
  }
  return g_sm;
}

cudaError_t launch_light_pass(const DevScene& S, const FrameArgs& a, const RenderBuffers& b, cudaStream_t st) {
  uint32_t threads = ((a.lightPaths + 31) / 32) * 32;
  if (threads == 0) threads = 32;
  k_light<<<1, threads, 0, st>>>(S, a, b.cache[a.cacheSel], b.cacheCap, b.ctr);
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_camera(const FrameArgs& a, const RenderBuffers& b, cudaStream_t st) {
  k_camera<<<(b.count + kBlock - 1) / kBlock, kBlock, 0, st>>>(a, b);
  note_launches(1);
  return cudaGetLastError();
}

// launch shapes, queried once per kernel
template <bool kCount, bool kWide>
uint32_t walk_grid() {
  static uint32_t g = grid_for((const void*)k_walk<kCount, kWide>);
  return g;
}

template <bool kCount, bool kWide>
uint32_t tail_grid() {
  static uint32_t g = grid_for((const void*)k_tail<kCount, kWide>);
  return g;
}

uint32_t shade_grid() {
  static uint32_t g = grid_for((const void*)k_shade);
  return g;
}

// persistent grid: every CTA that fits, or `ctasPerSm` per SM when that is
// fewer (requests that share the GPU leave SMs to each other)
uint32_t persistent_grid(uint32_t full, uint32_t ctasPerSm) {
  if (ctasPerSm == 0) return full;
  return std::min(full, (uint32_t)sm_count() * ctasPerSm);
}

template <bool kCount, bool kWide>
void walk_variant(const DevScene& S, const RenderBuffers& b, int in, int shIn, int shReset, uint32_t bilat,
                  uint32_t refill, uint32_t ctas, uint32_t launch, uint32_t carrySteps, cudaStream_t st) {
  const uint32_t g = persistent_grid(walk_grid<kCount, kWide>(), ctas);
  k_walk<kCount, kWide><<<g, kBlock, 0, st>>>(S, b, in, shIn, shReset, bilat, refill, launch, carrySteps);
}

template <bool kCount, bool kWide>
void tail_variant(const DevScene& S, const FrameArgs& a, const RenderBuffers& b, uint32_t K, cudaStream_t st) {
  const uint32_t g = persistent_grid(tail_grid<kCount, kWide>(), a.walkCtas);
  k_tail<kCount, kWide><<<g, kBlock, 0, st>>>(S, a, b, K, walk_refill_for(a.refill, kWide));
}

cudaError_t launch_walk(const DevScene& S, const FrameArgs& a, const RenderBuffers& b, int in, int shIn,
                        int shReset, uint32_t launch, cudaStream_t st) {
  const uint32_t sd = a.bilat ? 1u : 0u;
  const bool wide = S.traversal == 1 && S.wide;
  const uint32_t rf = walk_refill_for(a.refill, wide);
  const uint32_t cs = b.carry[0] ? a.carrySteps : 0u;
  if (a.counting) {
    if (wide) walk_variant<true, true>(S, b, in, shIn, shReset, sd, rf, a.walkCtas, launch, 0u, st);
    else walk_variant<true, false>(S, b, in, shIn, shReset, sd, rf, a.walkCtas, launch, cs, st);
  } else {
    if (wide) walk_variant<false, true>(S, b, in, shIn, shReset, sd, rf, a.walkCtas, launch, 0u, st);
    else walk_variant<false, false>(S, b, in, shIn, shReset, sd, rf, a.walkCtas, launch, cs, st);
  }
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_tail(const DevScene& S, const FrameArgs& a, const RenderBuffers& b, uint32_t K, cudaStream_t st) {
  const bool wide = S.traversal == 1 && S.wide;
  if (a.counting) {
    if (wide) tail_variant<true, true>(S, a, b, K, st);
    else tail_variant<true, false>(S, a, b, K, st);
  } else {
    if (wide) tail_variant<false, true>(S, a, b, K, st);
    else tail_variant<false, false>(S, a, b, K, st);
  }
  note_launches(1);
  return cudaGetLastError();
}

uint32_t walk_lanes() { return walk_grid<false, false>() * (uint32_t)kBlock; }

void prepare_launches() {
  walk_grid<false, false>();
  walk_grid<false, true>();
  walk_grid<true, false>();
  walk_grid<true, true>();
  tail_grid<false, false>();
  tail_grid<false, true>();
  tail_grid<true, false>();
  tail_grid<true, true>();
  shade_grid();
}

uint32_t tail_from(uint32_t eyeDepth, bool wide, int32_t requested, size_t paths, bool carrying) {
  // default while carrying (reference order): a frame with fewer camera paths
  // than the walk grid has lanes hands its paths to the tail kernel from bounce
  // 2 on, a larger one from bounce D/2 when D > 6, else never.  Measured with
  // carrying (Mpaths/s; the walk grid then had 194,560 lanes, now 155,648):
  // Cornell 256x256 (65,536 paths),
  // D = 8: from 2 204.6, 3 193.6, 4 180.6, 5 168.2; interior 1024x768, D = 10:
  // from 3 163.0, 4 167.5, 5 170.6, 6 169.7; hall 1280x720, D = 5: none 188.1
  // (launches past the cap: worse).  Against the rule without carrying: interior
  // 168.4 -> 172.3, Cornell 188.9 -> 194.6, hall and hall adaptive even.  The
  // same choice on the device (a shading launch switching once the live paths
  // fall below 1-3 x the lanes) cost Cornell 14 %: the host still issues the
  // skipped launches.
  // default without carrying, D > 6: from bounce D/2 - 1 in the reference
  // order, D/2 in the wide order; per-bounce launches throughout for D <= 6.
  // Measured in Mpaths/s (reference / wide order), tail kernel at three CTAs
  // per SM: interior, D = 10: from 4 174.3 / 169.6, from 5 170.6 / 174.8,
  // from 6 161.4 / 173.7; Cornell, D = 8: from 3 199.3 / 173.7, from 4 194.3
  // / 173.5; hall, D = 5: no tail 176.7 / 180.5, from 4 171.1 / 175.8, from 3
  // 158.9 (once few paths are alive the tail kernel's per-path schedule wins;
  // while many are, per-bounce launches keep more of them resident).
  static int v = [] {
    const char* e = std::getenv("GBPT_TAIL_FROM");
    return e ? std::atoi(e) : -2;
  }();
  if (requested >= 0) return (uint32_t)requested;
  if (v == -2 && carrying) {
    if (paths < walk_lanes()) return std::min(eyeDepth, 2u);
    return eyeDepth > 6 ? eyeDepth / 2 : eyeDepth;
  }
  if (v == -2) return eyeDepth > 6 ? eyeDepth / 2 - (wide ? 0u : 1u) : eyeDepth;
  return v < 0 ? eyeDepth : (uint32_t)v;
}

uint32_t walk_refill_for(uint32_t requested, bool wide) {
  if (requested >= 1 && requested <= 32) return requested;
  if (walk_refill_env()) return walk_refill_env();
  return wide ? 20u : 2u;
}

cudaError_t launch_shade(const DevScene& S, const FrameArgs& a, const RenderBuffers& b, int in, uint32_t launch,
                         bool attach, cudaStream_t st) {
  const uint32_t g = shade_grid();
  k_shade<<<g, kBlock, 0, st>>>(S, a, b, in, launch, attach ? 1u : 0u);
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_fold(const RenderBuffers& b, cudaStream_t st) {
  const uint32_t n = b.count ? b.count : b.cap;
  k_fold<<<(n + kBlock - 1) / kBlock, kBlock, 0, st>>>(b);
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_apply(const FrameArgs& a, const RenderBuffers& b, float* result, uint32_t* sampleN, float* gpos,
                         float* gnorm, float* gdiff, cudaStream_t st) {
  const uint32_t np = a.width * a.height;
  k_apply<<<(np + kBlock - 1) / kBlock, kBlock, 0, st>>>(a, b, result, sampleN, gpos, gnorm, gdiff);
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_apply_bilat(const FrameArgs& a, const RenderBuffers& b, float* result, uint32_t* sampleN,
                               float* gpos, float* gnorm, float* gdiff, float* gemis, float* direct, float* pot,
                               cudaStream_t st) {
  const uint32_t np = a.width * a.height;
  k_apply_bilat<<<(np + kBlock - 1) / kBlock, kBlock, 0, st>>>(a, b, result, sampleN, gpos, gnorm, gdiff, gemis,
                                                               direct, pot);
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_apply_pt(const FrameArgs& a, const RenderBuffers& b, float* result, uint32_t* sampleN,
                            cudaStream_t st) {
  const uint32_t np = a.width * a.height;
  k_apply_pt<<<(np + kBlock - 1) / kBlock, kBlock, 0, st>>>(a, b, result, sampleN);
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_prob_view(const float* pot, uint32_t np, float minProb, float* out, cudaStream_t st) {
  if (np == 0) return cudaSuccess;
  k_prob_view<<<(np + kBlock - 1) / kBlock, kBlock, 0, st>>>(pot, np, minProb, out);
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_trace_rays(const DevScene& S, const float* rays, uint32_t n, float maxDist, float eps, int cullback,
                              float* t, int32_t* tri, float* w, float* u, float* v, uint32_t* nodes,
                              uint32_t* trisTested, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  uint32_t grid = (n + kBlock - 1) / kBlock;
  if (nodes && trisTested)
    k_trace_rays<true><<<grid, kBlock, 0, st>>>(S, rays, n, maxDist, eps, cullback, t, tri, w, u, v, nodes,
                                                  trisTested);
  else
    k_trace_rays<false><<<grid, kBlock, 0, st>>>(S, rays, n, maxDist, eps, cullback, t, tri, w, u, v, nodes,
                                                   trisTested);
  note_launches(1);
  return cudaGetLastError();
}

}  // namespace gbpt
