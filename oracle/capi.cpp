// TEST INFRASTRUCTURE ONLY -- flat C entry points of the CPU oracle, loaded
// with ctypes by tests/, the smoke check and bench.py's CPU baseline.
#include <chrono>
#include <cstring>

#include "bdpt_ref.h"
#include "fmath_ref.h"
#include "oracle.h"
#include "philox_ref.h"

using namespace orc;

extern "C" {

void* orc_scene_create(const void* verts, uint32_t nv, const void* tris, uint32_t nt, const void* mats, uint32_t nm,
                       double* build_seconds) {
  Scene* s = new Scene();
  auto t0 = std::chrono::steady_clock::now();
  bool ok = make_scene((const RTVertex*)verts, nv, (const RTTriangle*)tris, nt, (const RTMaterial*)mats, nm, s);
  auto t1 = std::chrono::steady_clock::now();
  if (build_seconds) *build_seconds = std::chrono::duration<double>(t1 - t0).count();
  if (!ok) {
    delete s;
    return nullptr;
  }
  return s;
}

void orc_scene_destroy(void* s) { delete (Scene*)s; }

uint32_t orc_scene_node_count(void* s) { return ((Scene*)s)->bvh.nodeN; }
uint32_t orc_scene_empty_children(void* s) { return ((Scene*)s)->bvh.stats.empty_children; }
uint32_t orc_scene_light_count(void* s) { return (uint32_t)((Scene*)s)->lightTri.size(); }

void orc_scene_export(void* sp, float* bounds, uint32_t* offOrTSTN, uint32_t* order, float* isect) {
  Scene* s = (Scene*)sp;
  if (bounds) std::memcpy(bounds, s->bvh.bounds.data(), s->bvh.bounds.size() * 4);
  if (offOrTSTN) std::memcpy(offOrTSTN, s->bvh.offOrTSTN.data(), s->bvh.offOrTSTN.size() * 4);
  if (order) std::memcpy(order, s->bvh.order.data(), s->bvh.order.size() * 4);
  if (isect) std::memcpy(isect, s->isect.data(), s->isect.size() * 4);
}

void orc_update_materials(void* sp, const void* mats, uint32_t nm) {
  Scene* s = (Scene*)sp;
  s->mats.assign((const RTMaterial*)mats, (const RTMaterial*)mats + nm);
  refresh_lights(s);
}

// n textures: widths / heights, texels of all of them concatenated (4 floats each).
void orc_scene_set_textures(void* sp, uint32_t n, const uint32_t* w, const uint32_t* h, const float* rgba) {
  Scene* s = (Scene*)sp;
  s->textures.assign(n, Texture{});
  size_t off = 0;
  for (uint32_t i = 0; i < n; i++) {
    Texture& t = s->textures[i];
    t.w = w[i];
    t.h = h[i];
    const size_t cnt = (size_t)w[i] * h[i] * 4;
    t.rgba.assign(rgba + off, rgba + off + cnt);
    off += cnt;
  }
}

// n texture samples (u, v) of one texture -> 4 floats each (texture_ref.h)
void orc_texture_sample(const float* rgba, uint32_t w, uint32_t h, const float* uv, uint32_t n, float* out) {
  Texture t;
  t.w = w;
  t.h = h;
  t.rgba.assign(rgba, rgba + (size_t)w * h * 4);
  for (uint32_t i = 0; i < n; i++) tex_bilinear<float>(t, uv[2 * i], uv[2 * i + 1], out + 4 * (size_t)i);
}

// GetMaterialColors of one material at n uvs with the given textures
// (widths / heights / concatenated texels as orc_scene_set_textures).
void orc_material_colors(const void* mat, const float* uv, uint32_t n, uint32_t ntex, const uint32_t* w,
                         const uint32_t* h, const float* rgba, float* out) {
  std::vector<Texture> texs(ntex);
  size_t off = 0;
  for (uint32_t i = 0; i < ntex; i++) {
    texs[i].w = w[i];
    texs[i].h = h[i];
    const size_t cnt = (size_t)w[i] * h[i] * 4;
    texs[i].rgba.assign(rgba + off, rgba + off + cnt);
    off += cnt;
  }
  material_colors(texs, *(const RTMaterial*)mat, uv, n, out);
}

// rays: 6 floats each (origin, direction).  Outputs per ray.
// IntersectAABB over n cases of 12 floats (origin, direction, min, max).
void orc_intersect_aabb(const float* c, uint32_t n, float* out) {
  for (uint32_t i = 0; i < n; i++) {
    const float* q = c + (size_t)i * 12;
    out[i] = intersect_aabb(q, q + 3, q + 6, q + 9);
  }
}

// IntersectTri over n cases of 15 floats (origin, direction, p0, e0, e1); 4 floats out each (t, w, u, v).
void orc_intersect_tri(const float* c, uint32_t n, float eps, int32_t cullback, float* out) {
  for (uint32_t i = 0; i < n; i++) {
    const float* q = c + (size_t)i * 15;
    out[(size_t)i * 4] = intersect_tri(q, q + 3, q + 6, q + 9, q + 12, eps, cullback != 0, out + (size_t)i * 4 + 1);
  }
}

void orc_trace(void* sp, const float* rays, uint32_t n, float maxDist, float eps, int32_t cullback, float* t,
               int32_t* triId, float* w, float* u, float* v, uint32_t* nodes, uint32_t* trisTested) {
  Scene* s = (Scene*)sp;
  for (uint32_t i = 0; i < n; i++) {
    Hit h;
    TraceCount c;
    bool r = trace_primitive(*s, rays + i * 6, rays + i * 6 + 3, maxDist, eps, cullback != 0, &h, &c);
    t[i] = r ? h.dist : -1.f;
    triId[i] = r ? h.triId : -1;
    w[i] = r ? h.w : 0.f;
    u[i] = r ? h.u : 0.f;
    v[i] = r ? h.v : 0.f;
    if (nodes) nodes[i] = c.nodes;
    if (trisTested) trisTested[i] = c.tris;
  }
}

void orc_default_params(void* p) { default_params((Params*)p); }

void* orc_renderer_create(uint32_t W, uint32_t H, int32_t mode, const void* params, uint32_t threads) {
  Renderer* r = new Renderer();
  renderer_init(r, W, H, mode, *(const Params*)params, false, threads);
  return r;
}
void orc_renderer_destroy(void* r) { delete (Renderer*)r; }
void orc_renderer_set_window(void* rp, uint32_t x0, uint32_t y0, uint32_t fullW, uint32_t fullH) {
  Renderer* r = (Renderer*)rp;
  r->x0 = x0;
  r->y0 = y0;
  r->fullW = fullW;
  r->fullH = fullH;
}
void orc_renderer_set_params(void* r, const void* params) { ((Renderer*)r)->p = *(const Params*)params; }

// camera: pos[3], dir[3], up[3], fov
void orc_render(void* rp, void* sp, const float* cam, uint32_t frames) {
  Renderer* r = (Renderer*)rp;
  Camera c;
  std::memcpy(c.pos, cam, 3 * 4);
  std::memcpy(c.dir, cam + 3, 3 * 4);
  std::memcpy(c.up, cam + 6, 3 * 4);
  c.fov = cam[9];
  for (uint32_t f = 0; f < frames; f++) render_frame(r, *(Scene*)sp, c);
}

// which: 0 result, 1 position, 2 normal, 3 diffuse, 4 filtered, 5 error (W*H),
// filter-only mode: 8 direct, 9 first-hit emissive, 10 mean 1 - potential (W*H), 11 the debug view
void orc_renderer_get(void* rp, int32_t which, float* out) {
  Renderer* r = (Renderer*)rp;
  const std::vector<float>* src = nullptr;
  switch (which) {
    case 0: src = &r->result; break;
    case 1: src = &r->gpos; break;
    case 2: src = &r->gnorm; break;
    case 3: src = &r->gdiff; break;
    case 4: src = &r->filtered; break;
    case 5: src = &r->err; break;
    case 8: src = &r->direct; break;
    case 9: src = &r->gemis; break;
    case 10: src = &r->pot; break;
    case 11: src = &r->out; break;
    default: return;
  }
  std::memcpy(out, src->data(), src->size() * 4);
}
void orc_renderer_set_debug(void* rp, uint32_t mode) { ((Renderer*)rp)->debug_mode = mode; }
void orc_renderer_counts(void* rp, uint32_t* sampleN, uint32_t* counts) {
  Renderer* r = (Renderer*)rp;
  if (sampleN) std::memcpy(sampleN, r->sampleN.data(), r->sampleN.size() * 4);
  if (counts) std::memcpy(counts, r->counts.data(), r->counts.size() * 4);
}
uint32_t orc_renderer_frame(void* rp) { return ((Renderer*)rp)->frame; }
void orc_renderer_stats(void* rp, uint64_t* out4) {
  Renderer* r = (Renderer*)rp;
  out4[0] = r->lastPaths;
  out4[1] = r->lastRays;
  out4[2] = r->lastNodes;
  out4[3] = r->lastTris;
}
void orc_renderer_ext_stats(void* rp, uint64_t* out3) {
  Renderer* r = (Renderer*)rp;
  for (int k = 0; k < 3; k++) out3[k] = r->lastExt[k];
}
uint32_t orc_renderer_light_cache(void* rp, float* out) {  // 21 floats per vertex
  Renderer* r = (Renderer*)rp;
  if (out) std::memcpy(out, r->cache.data(), r->cacheSize * sizeof(LightVertex));
  return r->cacheSize;
}

void orc_render_fp64(void* sp, const void* params, uint32_t W, uint32_t H, const float* cam, uint32_t frames,
                     uint32_t threads, double* out) {
  Camera c;
  std::memcpy(c.pos, cam, 3 * 4);
  std::memcpy(c.dir, cam + 3, 3 * 4);
  std::memcpy(c.up, cam + 6, 3 * 4);
  c.fov = cam[9];
  render_fp64(*(Scene*)sp, *(const Params*)params, W, H, c, frames, threads, out);
}

void orc_gaussian(float delta, uint32_t radius, float* g) { gaussian_table(delta, radius, g); }

void orc_bilateral(const float* color, const float* pos, const float* norm, const float* emit, uint32_t W, uint32_t H,
                   float colorEuD, float posEuD, float normEuD, float emitEuD, uint32_t radius, const float* g,
                   float* out) {
  bilateral(color, pos, norm, emit, W, H, colorEuD, posEuD, normEuD, emitEuD, radius, g, out);
}

void orc_philox(const uint32_t* ctr4, uint32_t k0, uint32_t k1, uint32_t* out4) {
  U4 c{{ctr4[0], ctr4[1], ctr4[2], ctr4[3]}};
  U4 r = philox4x32_10(c, k0, k1);
  std::memcpy(out4, r.v, 16);
}

void orc_fmath(int32_t which, const float* x, uint32_t n, float* out) {
  for (uint32_t i = 0; i < n; i++) {
    float s, c;
    switch (which) {
      case 0: sincos_p(x[i], &s, &c); out[i] = s; break;
      case 1: sincos_p(x[i], &s, &c); out[i] = c; break;
      case 2: out[i] = exp_p(x[i]); break;
      case 3: out[i] = sqrt_rd(x[i]); break;
      case 4: out[i] = pow5(x[i]); break;
      default: out[i] = 0.f;
    }
  }
}

}  // extern "C"
