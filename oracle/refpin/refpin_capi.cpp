// C ABI over the reference's own BVH builder and traversal, compiled from
// the reference sources (src/bvhhelper.cpp, src/cudaRTCommon.cu) with the
// stand-ins of prelude.h -- TEST INFRASTRUCTURE ONLY.  It pins the oracle:
// tests compare the oracle's restatement against these functions and the
// golden fixtures are generated from them.
//
// The scene set-up follows the reference's call sites: RTScene::AddModel
// (src/raytracer.cpp:255-281: index and position lists, CreateBVH, the
// triangle reorder, the intersection data, InitialCompactBVH) and
// initAllSceneCudaMem (src/cudaRTCommon.cu:529-566: float4 node bounds,
// uint1 child/leaf words, float4 triangle records p0, p1-p0, p2-p0, bound to
// the three texture references).  One scene is bound at a time.
#include "bvhhelper.h"
#include "cudaRTCommon.h"
#include "texture_ref.h"

#include <cmath>
#include <cstdint>
#include <map>
#include <vector>

extern const uint3 threadIdx = {0, 0, 0};
float curand_uniform(curandState*) { std::abort(); }
unsigned int __ballot(int) { std::abort(); }
int __ffs(int) { std::abort(); }
int __popc(unsigned int) { std::abort(); }
int atomicAdd(int*, int) { std::abort(); }
int __shfl(int, int) { std::abort(); }

namespace {

struct RefScene {
  NPBVHHelper::BVHNode root;
  NPBVHHelper::CompactBVH compact;
  std::vector<uint32> order;
  std::vector<float4> bounds;    // 2 per node: min, max (w = 0)
  std::vector<uint1> offs;       // 2 per node: offOrTs, triN
  std::vector<float4> isect;     // 3 per triangle: p0, p1 - p0, p2 - p0
  ~RefScene() {
    root.Clear();
    delete[] compact.bounds;
    delete[] compact.offOrTSTN;
  }
};

RefScene* g_bound = nullptr;

void bind(RefScene* s) {
  cudaChannelFormatDesc d{};
  cudaBindTexture(nullptr, g_bvhMinMaxBounds, s->bounds.data(), d, s->bounds.size() * sizeof(float4));
  cudaBindTexture(nullptr, g_bvhOffsetTriStartN, s->offs.data(), d, s->offs.size() * sizeof(uint1));
  cudaBindTexture(nullptr, g_triIntersectionData, s->isect.data(), d, s->isect.size() * sizeof(float4));
  g_bound = s;
}

// host textures for tex2D on texture objects (ids start at 1)
std::map<unsigned long long, orc::Texture> g_tex;

}  // namespace

// tex2D stand-in: the oracle's restatement of the linear, wrapped fetch
// (texture_ref.h), so that the pin compares GetMaterialColors' own logic
// (which texture, transparency times alpha, the emissive override).
float4 gbref_tex2D_float4(cudaTextureObject_t obj, float u, float v) {
  auto it = g_tex.find(obj);
  if (it == g_tex.end() || it->second.w == 0 || it->second.h == 0) return make_float4(0.f, 0.f, 0.f, 0.f);
  float r[4];
  orc::tex_bilinear<float>(it->second, u, v, r);
  return make_float4(r[0], r[1], r[2], r[3]);
}

extern "C" {

// Builds the reference BVH of nt triangles (idx: 3 vertex ids each) over nv
// positions (pos: 3 floats each); returns a handle and its node count.
void* refpin_scene_create(const float* pos, uint32_t nv, const uint32_t* idx, uint32_t nt, uint32_t* node_n) {
  if (!pos || !idx || nt == 0) return nullptr;
  RefScene* s = new RefScene();
  std::vector<uint32> tris(idx, idx + 3 * (size_t)nt);
  std::vector<NPMathHelper::Vec3> verts;
  verts.reserve(nv);
  for (uint32_t i = 0; i < nv; i++) verts.push_back(NPMathHelper::Vec3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]));
  s->root.Clear();
  s->order = NPBVHHelper::CreateBVH(&s->root, tris, verts);
  std::vector<NPMathHelper::Vec3> tdata(s->order.size() * 3);
  for (size_t i = 0; i < s->order.size(); i++) {
    const uint32 t = s->order[i];
    tdata[i * 3] = verts[tris[3 * t]];
    tdata[i * 3 + 1] = verts[tris[3 * t + 1]];
    tdata[i * 3 + 2] = verts[tris[3 * t + 2]];
  }
  if (!s->compact.InitialCompactBVH(&s->root)) {
    delete s;
    return nullptr;
  }
  const uint32 n = s->compact.nodeN;
  s->bounds.resize(2 * (size_t)n);
  s->offs.resize(2 * (size_t)n);
  for (uint32 i = 0; i < n; i++) {
    s->bounds[2 * i] = V32F4(s->compact.bounds[i].minPoint);
    s->bounds[2 * i + 1] = V32F4(s->compact.bounds[i].maxPoint);
    s->offs[2 * i].x = s->compact.offOrTSTN[2 * i];
    s->offs[2 * i + 1].x = s->compact.offOrTSTN[2 * i + 1];
  }
  s->isect.resize(tdata.size());
  for (size_t i = 0; i < s->order.size(); i++) {
    s->isect[i * 3] = V32F4(tdata[i * 3]);
    s->isect[i * 3 + 1] = V32F4(tdata[i * 3 + 1] - tdata[i * 3]);
    s->isect[i * 3 + 2] = V32F4(tdata[i * 3 + 2] - tdata[i * 3]);
  }
  if (node_n) *node_n = n;
  return s;
}

void refpin_scene_destroy(void* h) {
  RefScene* s = (RefScene*)h;
  if (g_bound == s) g_bound = nullptr;
  delete s;
}

// bounds: 6 floats per node (min, max); offs: 2 words per node; order: the
// reordered triangle ids; isect: 9 floats per triangle (p0, p1-p0, p2-p0).
void refpin_scene_export(void* h, float* bounds, uint32_t* offs, uint32_t* order, float* isect) {
  RefScene* s = (RefScene*)h;
  const size_t n = s->compact.nodeN;
  for (size_t i = 0; i < n; i++) {
    const float4 a = s->bounds[2 * i], b = s->bounds[2 * i + 1];
    float* o = bounds + 6 * i;
    o[0] = a.x; o[1] = a.y; o[2] = a.z; o[3] = b.x; o[4] = b.y; o[5] = b.z;
    offs[2 * i] = s->offs[2 * i].x;
    offs[2 * i + 1] = s->offs[2 * i + 1].x;
  }
  for (size_t i = 0; i < s->order.size(); i++) {
    order[i] = s->order[i];
    for (int k = 0; k < 3; k++) {
      const float4 p = s->isect[3 * i + k];
      isect[9 * i + 3 * k] = p.x;
      isect[9 * i + 3 * k + 1] = p.y;
      isect[9 * i + 3 * k + 2] = p.z;
    }
  }
}

// TracePrimitive (src/cudaRTCommon.cu:66-127) over n rays (6 floats each:
// origin, direction); hit[i] = 1 on a hit, and then t, triangle (in the
// reordered order), w, u, v; a miss gives t = -1, triangle -1, w = u = v = 0.
void refpin_trace(void* h, const float* rays, uint32_t n, float max_dist, float eps, int32_t cullback, uint8_t* hit,
                  float* t, int32_t* tri, float* w, float* u, float* v) {
  bind((RefScene*)h);
  for (uint32_t i = 0; i < n; i++) {
    const float* r = rays + 6 * (size_t)i;
    CURay ray(make_float3(r[0], r[1], r[2]), make_float3(r[3], r[4], r[5]));
    TracePrimitiveResult res{};
    const bool ok = TracePrimitive(ray, res, max_dist, eps, cullback != 0);
    hit[i] = ok ? 1 : 0;
    t[i] = ok ? res.dist : -1.f;
    tri[i] = ok ? res.triId : -1;
    w[i] = ok ? res.w : 0.f;
    u[i] = ok ? res.u : 0.f;
    v[i] = ok ? res.v : 0.f;
  }
}

// CURay::IntersectAABB (:24-40) for n (origin, direction, min, max) cases,
// 12 floats each.
void refpin_intersect_aabb(const float* cases, uint32_t n, float* out) {
  for (uint32_t i = 0; i < n; i++) {
    const float* c = cases + 12 * (size_t)i;
    CURay ray(make_float3(c[0], c[1], c[2]), make_float3(c[3], c[4], c[5]));
    out[i] = ray.IntersectAABB(make_float3(c[6], c[7], c[8]), make_float3(c[9], c[10], c[11]));
  }
}

// CURay::IntersectTri (:42-64) for n (origin, direction, p0, e0, e1) cases,
// 15 floats each; out: 4 floats per case (t, w, u, v; w, u, v are left at
// 0 where the function returns before setting them).
void refpin_intersect_tri(const float* cases, uint32_t n, float eps, int32_t cullback, float* out) {
  for (uint32_t i = 0; i < n; i++) {
    const float* c = cases + 15 * (size_t)i;
    CURay ray(make_float3(c[0], c[1], c[2]), make_float3(c[3], c[4], c[5]));
    float w = 0.f, u = 0.f, v = 0.f;
    const float t = ray.IntersectTri(make_float3(c[6], c[7], c[8]), make_float3(c[9], c[10], c[11]),
                                     make_float3(c[12], c[13], c[14]), w, u, v, eps, cullback != 0);
    out[4 * i] = t;
    out[4 * i + 1] = w;
    out[4 * i + 2] = u;
    out[4 * i + 3] = v;
  }
}

// Registers a W x H float4 texture (row-major, RGBA) under id (>= 1) for
// the tex2D stand-in.
void refpin_texture_set(uint64_t id, const float* rgba, int32_t w, int32_t h) {
  orc::Texture t;
  t.w = (uint32_t)w;
  t.h = (uint32_t)h;
  t.rgba.assign(rgba, rgba + (size_t)w * h * 4);
  g_tex[id] = std::move(t);
}

// GetMaterialColors (:369-406) of one 80-byte RTMaterial at n uv
// coordinates; textures: texture object ids indexed by the material's
// texture ids; out: 8 floats per uv (diffuse rgb, emissive rgb, trans, spare).
void refpin_material_colors(const void* mat, const float* uv, uint32_t n, const uint64_t* tex_ids, uint32_t ntex,
                            float* out) {
  std::vector<CURTTexture> texs(ntex);
  for (uint32_t i = 0; i < ntex; i++) texs[i].texObj = tex_ids[i];
  const RTMaterial* m = (const RTMaterial*)mat;
  for (uint32_t i = 0; i < n; i++) {
    float3 diff, normal = make_float3(0.f, 0.f, 0.f), emis;
    float trans, spec, metal, rough, aniso, sheen, sheenTint, cc, ccg;
    GetMaterialColors(m, make_float2(uv[2 * i], uv[2 * i + 1]), texs.data(), diff, normal, emis, trans, spec, metal,
                      rough, aniso, sheen, sheenTint, cc, ccg);
    float* o = out + 8 * (size_t)i;
    o[0] = diff.x; o[1] = diff.y; o[2] = diff.z;
    o[3] = emis.x; o[4] = emis.y; o[5] = emis.z;
    o[6] = trans; o[7] = 0.f;
  }
}

}  // extern "C"
