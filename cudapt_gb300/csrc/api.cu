// C ABI of libgbpt: scenes, renderers and the per-frame launch sequence.
//
// Replaces RTScene / RTRenderer (include/raytracer.h:228-323) and the
// per-renderer Render functions (src/cudaRTBDPTStream.cu:816-951,
// src/cudaRTBDPTStreamAdapBilatAtomic.cu:1253-1554) for the BDPT modes.
// Unlike the reference there is no process-global device state: every scene
// and renderer owns its buffers, and a renderer owns its CUDA stream.
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "gbpt_internal.h"
#include "gbpt_math.cuh"
#include "launch.h"

using namespace gbpt;

namespace gbpt {
static thread_local std::string g_err;
void set_error(const std::string& s) { g_err = s; }
gbpt_status fail(gbpt_status st, const std::string& s) {
  g_err = s;
  return st;
}
}  // namespace gbpt

#define CK(call)                                                                                 \
  do {                                                                                           \
    cudaError_t e_ = (call);                                                                     \
    if (e_ != cudaSuccess)                                                                       \
      return fail(e_ == cudaErrorMemoryAllocation ? GBPT_ERR_OOM : GBPT_ERR_CUDA,                \
                  std::string(#call) + ": " + cudaGetErrorString(e_));                           \
  } while (0)

namespace {

// host-side fault injection for tests (gbpt_test_fail_allocations): when
// >= 0, the device allocations of this file fail once this many more have
// succeeded
std::atomic<int64_t> g_failAfter{-1};

template <typename T>
cudaError_t dalloc(T** p, size_t n) {
  *p = nullptr;
  if (n == 0) n = 1;
  if (g_failAfter.load(std::memory_order_relaxed) >= 0 && g_failAfter.fetch_sub(1) <= 0) {
    g_failAfter.store(0);
    return cudaErrorMemoryAllocation;
  }
  return cudaMalloc((void**)p, n * sizeof(T));
}
template <typename T>
void dfree(T*& p) {
  if (p) cudaFree((void*)p);
  p = nullptr;
}

uint64_t g_sceneVersion = 1;
std::mutex g_versionMu;
uint64_t next_version() {
  std::lock_guard<std::mutex> l(g_versionMu);
  return ++g_sceneVersion;
}

}  // namespace

struct gbpt_scene {
  std::vector<gbpt_vertex> verts;
  std::vector<gbpt_triangle> tris;  // caller order
  std::vector<gbpt_material> mats;
  HostBVH bvh;
  bool built = false;
  std::vector<gbpt_triangle> trisOrdered;
  std::vector<uint32_t> lightTri;
  struct Texture {
    std::vector<float4> texels;
    uint32_t w = 0, h = 0;
  };
  std::vector<Texture> textures;  // RTScene::m_pTextures
  float4 *dNodes = nullptr, *dTris = nullptr, *dShade = nullptr, *dMats = nullptr, *dWide = nullptr;
  float4* dTexels = nullptr;
  uint4* dTexInfo = nullptr;
  float2* dUvs = nullptr;
  uint32_t traversal = 0;  // 0: the reference's order, 1: wide (collapsed 4-ary tree)
  uint32_t* dLight = nullptr;
  DevScene dev;
  uint64_t version = 0;
  bool uploaded = false;
  std::mutex upload;  // renderers on several threads (a server's workers) may upload it first

  void free_dev() {
    dfree(dNodes);
    dfree(dTris);
    dfree(dShade);
    dfree(dMats);
    dfree(dLight);
    dfree(dWide);
    dfree(dTexels);
    dfree(dTexInfo);
    dfree(dUvs);
    dev = DevScene{};
  }
  ~gbpt_scene() { free_dev(); }
};

namespace {

// src/cudaRTBDPTStream.cu:57-77 -- host length of the emissive colour > 0
void scan_lights(gbpt_scene* s) {
  s->lightTri.clear();
  for (uint32_t i = 0; i < s->trisOrdered.size(); i++) {
    const float* e = s->mats[s->trisOrdered[i].mat].emissive;
    if (std::sqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]) > 0.f) s->lightTri.push_back(i);
  }
}

float as_f(uint32_t u) {
  float f;
  std::memcpy(&f, &u, 4);
  return f;
}

// material texture ids must index the scene's textures (negative: none)
gbpt_status check_texture_ids(const std::vector<gbpt_material>& mats, size_t ntex) {
  for (size_t i = 0; i < mats.size(); i++) {
    const gbpt_material& a = mats[i];
    for (int32_t id : {a.diffuseTexId, a.normalTexId, a.emissiveTexId})
      if (id >= 0 && (size_t)id >= ntex)
        return fail(GBPT_ERR_INVALID_ARG, "material " + std::to_string(i) + " names texture " + std::to_string(id) +
                                              " but the scene has " + std::to_string(ntex) +
                                              " (gbpt_scene_set_textures)");
  }
  return GBPT_OK;
}

std::vector<float4> pack_materials(const std::vector<gbpt_material>& mats) {
  std::vector<float4> m(mats.size() * 3);
  for (size_t i = 0; i < mats.size(); i++) {
    const gbpt_material& a = mats[i];
    m[3 * i] = make_float4(a.diffuse[0], a.diffuse[1], a.diffuse[2], a.transparency);
    m[3 * i + 1] = make_float4(a.emissive[0], a.emissive[1], a.emissive[2], a.specular);
    m[3 * i + 2] = make_float4(a.metallic, a.roughness, as_f((uint32_t)(a.diffuseTexId < 0 ? -1 : a.diffuseTexId)),
                               as_f((uint32_t)(a.emissiveTexId < 0 ? -1 : a.emissiveTexId)));
  }
  return m;
}

// texels of every texture in one array, a {first texel, width, height} record
// each, and the vertex uvs of every triangle in BVH order
gbpt_status upload_textures(gbpt_scene* s) {
  dfree(s->dTexels);
  dfree(s->dTexInfo);
  dfree(s->dUvs);
  s->dev.texels = nullptr;
  s->dev.texInfo = nullptr;
  s->dev.uvs = nullptr;
  if (s->textures.empty()) return GBPT_OK;
  size_t total = 0;
  std::vector<uint4> info(s->textures.size());
  for (size_t i = 0; i < s->textures.size(); i++) {
    info[i] = make_uint4((uint32_t)total, s->textures[i].w, s->textures[i].h, 0u);
    total += s->textures[i].texels.size();
  }
  if (total >= 0xFFFFFFFFull) return fail(GBPT_ERR_INVALID_ARG, "textures exceed 2^32 texels in total");
  const uint32_t nt = (uint32_t)s->trisOrdered.size();
  std::vector<float2> uvs((size_t)nt * 3);
  for (uint32_t i = 0; i < nt; i++) {
    const gbpt_triangle& t = s->trisOrdered[i];
    const gbpt_vertex* v[3] = {&s->verts[t.v0], &s->verts[t.v1], &s->verts[t.v2]};
    for (int k = 0; k < 3; k++) uvs[3 * (size_t)i + k] = make_float2(v[k]->tex[0], v[k]->tex[1]);
  }
  CK(dalloc(&s->dTexels, total));
  CK(dalloc(&s->dTexInfo, info.size()));
  CK(dalloc(&s->dUvs, uvs.size()));
  size_t off = 0;
  for (const auto& t : s->textures) {
    CK(cudaMemcpy(s->dTexels + off, t.texels.data(), t.texels.size() * 16, cudaMemcpyHostToDevice));
    off += t.texels.size();
  }
  CK(cudaMemcpy(s->dTexInfo, info.data(), info.size() * 16, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(s->dUvs, uvs.data(), uvs.size() * 8, cudaMemcpyHostToDevice));
  s->dev.texels = s->dTexels;
  s->dev.texInfo = s->dTexInfo;
  s->dev.uvs = s->dUvs;
  return GBPT_OK;
}

gbpt_status upload_wide(gbpt_scene* s) {
  dfree(s->dWide);
  std::vector<float> w = collapse_wide(s->bvh);
  CK(dalloc(&s->dWide, w.size() / 4));
  CK(cudaMemcpy(s->dWide, w.data(), w.size() * 4, cudaMemcpyHostToDevice));
  s->dev.wide = s->dWide;
  s->dev.wideN = (uint32_t)(w.size() / 32);
  return GBPT_OK;
}

gbpt_status upload_scene(gbpt_scene* s) {
  gbpt_status ids = check_texture_ids(s->mats, s->textures.size());
  if (ids != GBPT_OK) return ids;
  s->free_dev();
  const uint32_t nt = (uint32_t)s->trisOrdered.size(), nn = s->bvh.nodeN;
  // one all-zero node record and one all-zero triangle record after the
  // arrays: a walk reads them for ids past the end (the reference's texture
  // fetches return zeros there) without a bounds-checked load
  std::vector<float4> nodes((size_t)(nn + 1) * 2), tris((size_t)(nt + 1) * 4), shade((size_t)nt * 5);
  for (uint32_t i = 0; i < nn; i++) {
    const float* b = &s->bvh.bounds[(size_t)i * 6];
    nodes[2 * i] = make_float4(b[0], b[1], b[2], as_f(s->bvh.offOrTSTN[2 * i]));
    nodes[2 * i + 1] = make_float4(b[3], b[4], b[5], as_f(s->bvh.offOrTSTN[2 * i + 1]));
  }
  for (uint32_t i = 0; i < nt; i++) {
    const gbpt_triangle& t = s->trisOrdered[i];
    const gbpt_vertex &a = s->verts[t.v0], &b = s->verts[t.v1], &c = s->verts[t.v2];
    // src/cudaRTCommon.cu:507-509: p0, p1 - p0, p2 - p0 (host float subtraction)
    tris[4 * i] = make_float4(a.pos[0], a.pos[1], a.pos[2], 0.f);
    tris[4 * i + 1] = make_float4(b.pos[0] - a.pos[0], b.pos[1] - a.pos[1], b.pos[2] - a.pos[2], 0.f);
    tris[4 * i + 2] = make_float4(c.pos[0] - a.pos[0], c.pos[1] - a.pos[1], c.pos[2] - a.pos[2], 0.f);
    shade[5 * i] = make_float4(a.norm[0], a.norm[1], a.norm[2], a.pos[0]);
    shade[5 * i + 1] = make_float4(b.norm[0], b.norm[1], b.norm[2], a.pos[1]);
    shade[5 * i + 2] = make_float4(c.norm[0], c.norm[1], c.norm[2], a.pos[2]);
    shade[5 * i + 3] = make_float4(b.pos[0], b.pos[1], b.pos[2], as_f(t.mat));
    shade[5 * i + 4] = make_float4(c.pos[0], c.pos[1], c.pos[2], 0.f);
  }
  std::vector<float4> mats = pack_materials(s->mats);
  CK(dalloc(&s->dNodes, nodes.size()));
  CK(dalloc(&s->dTris, tris.size()));
  CK(dalloc(&s->dShade, shade.size()));
  CK(dalloc(&s->dMats, mats.size()));
  CK(dalloc(&s->dLight, s->lightTri.size()));
  CK(cudaMemcpy(s->dNodes, nodes.data(), nodes.size() * 16, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(s->dTris, tris.data(), tris.size() * 16, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(s->dShade, shade.data(), shade.size() * 16, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(s->dMats, mats.data(), mats.size() * 16, cudaMemcpyHostToDevice));
  if (!s->lightTri.empty())
    CK(cudaMemcpy(s->dLight, s->lightTri.data(), s->lightTri.size() * 4, cudaMemcpyHostToDevice));
  s->dev.nodes = s->dNodes;
  s->dev.tris = s->dTris;
  s->dev.shade = s->dShade;
  s->dev.mats = s->dMats;
  s->dev.lightTri = s->dLight;
  s->dev.nodeN = nn;
  s->dev.triN = nt;
  s->dev.lightN = (uint32_t)s->lightTri.size();
  s->dev.matN = (uint32_t)s->mats.size();
  s->dev.traversal = s->traversal;
  if (s->traversal == 1) {
    gbpt_status w = upload_wide(s);
    if (w != GBPT_OK) return w;
  }
  gbpt_status tx = upload_textures(s);
  if (tx != GBPT_OK) return tx;
  s->uploaded = true;
  return GBPT_OK;
}

gbpt_status ensure_uploaded(gbpt_scene* s) {
  if (!s->built) return fail(GBPT_ERR_STATE, "scene has no BVH (call gbpt_scene_build_bvh)");
  std::lock_guard<std::mutex> lock(s->upload);
  if (s->uploaded) return GBPT_OK;
  return upload_scene(s);
}

enum Phase { kPhLight = 0, kPhTrace, kPhShade, kPhShadow, kPhFilter, kPhAdapt, kPhOther, kPhN };

}  // namespace

struct gbpt_renderer {
  uint32_t W = 0, H = 0;
  int32_t mode = GBPT_MODE_BDPT_SC;
  gbpt_params p{};
  float debugMode = 0.f;
  cudaStream_t st = nullptr;
  bool alloc = false;
  RenderBuffers rb{};
  AdaptBuffers ab{};
  float *result = nullptr, *gpos = nullptr, *gnorm = nullptr, *gdiff = nullptr, *gauss = nullptr;
  // filter-only mode: first-hit emissive, direct-light and 1 - potential means,
  // the second ping-pong filter plane and the "Prob" view scratch plane
  float *gemis = nullptr, *direct = nullptr, *pot = nullptr, *filtered2 = nullptr, *probView = nullptr;
  // learned allocator: the attached network (not owned), whether statistics are kept without one
  gbpt_mlp* mlp = nullptr;
  bool collect = false;
  // work stream: the renderer's own (ownSt) unless the caller supplied one
  bool userStream = false;
  cudaStream_t ownSt = nullptr;
  const float* bilatOut = nullptr;  // filter plane holding the last filtered image
  uint32_t* sampleN = nullptr;
  float4* waveMem = nullptr;
  float* hostResult = nullptr;  // page-locked copy of the current view (gbpt_result)
  size_t hostResultN = 0;
  uint32_t frame = 0;
  bool started = false;
  float camBasis[9] = {0};
  uint64_t sceneVersion = 0;
  bool counting = false;
  float gaussKey[2] = {-1.f, -1.f};
  std::vector<std::pair<int, cudaEvent_t>> evs;
  std::vector<cudaEvent_t> evPool;
  // light passes run one group ahead on a side stream into the cache the
  // current frames do not read; tag = (epoch, frame) the cache was made for
  cudaStream_t stLight = nullptr;
  cudaEvent_t evMain = nullptr, evLight[2] = {nullptr, nullptr};
  // bands: a frame's camera paths split into bands, one wavefront each on its
  // own stream, forked from and joined to the work stream by events, so that
  // one band's last long walks overlap the others' work
  cudaStream_t stBand[kMaxBands] = {};
  cudaEvent_t evFork = nullptr, evJoin[kMaxBands] = {};
  uint32_t lastBands = 1;
  // window of a larger image (gbpt_renderer_set_window); the whole image by default
  uint32_t winX0 = 0, winY0 = 0, fullW = 0, fullH = 0;
  // frames issued as CUDA graphs (plain and PTSC modes): executable graphs
  // without / with an inline light pass
  bool graphs = false, graphWarm = false;
  cudaGraphExec_t gexec[2] = {nullptr, nullptr};
  bool lightPending[2] = {false, false};
  uint64_t epoch = 0;
  // a restored checkpoint adopts the next frame's scene when it has the
  // checkpoint's triangle and node counts (scene handles do not outlive a process)
  bool resumeScene = false;
  uint32_t resumeTriN = 0, resumeNodeN = 0;
  uint32_t lastTriN = 0, lastNodeN = 0;  // the scene of the last frame (checkpoint check)
  uint64_t cacheEpoch[2] = {~0ull, ~0ull};
  uint32_t cacheFrame[2] = {0, 0};
  uint32_t lastSel = 0;
  bool lastTraced = true;  // the last frame traced camera paths (filter-only mode may only filter)

  void free_dev() {
    for (int k = 0; k < 2; k++) rb.wave[k] = Wave{};
    dfree(waveMem);
    dfree(rb.hit);
    dfree(rb.sh[0]);
    dfree(rb.sh[1]);
    dfree(rb.res);
    dfree(rb.gbuf);
    dfree(rb.dsm);
    dfree(rb.slotPix);
    dfree(rb.slotSmp);
    if (stLight) cudaStreamSynchronize(stLight);
    dfree(rb.cache[0]);
    dfree(rb.cache[1]);
    cacheEpoch[0] = cacheEpoch[1] = ~0ull;
    lightPending[0] = lightPending[1] = false;
    dfree(rb.ctr);
    dfree(rb.carry[0]);
    dfree(rb.carry[1]);
    dfree(rb.conn);
    rb.connDepth = 0;
    dfree(ab.err);
    dfree(ab.cnt);
    dfree(ab.off);
    dfree(ab.blockSum);
    dfree(ab.partial);
    dfree(ab.filtered);
    dfree(ab.coop);
    dfree(ab.heavy);
    dfree(ab.list8);
    dfree(result);
    dfree(gpos);
    dfree(gnorm);
    dfree(gdiff);
    dfree(gemis);
    dfree(direct);
    dfree(pot);
    dfree(filtered2);
    dfree(probView);
    dfree(rb.m2);
    dfree(rb.hist);
    dfree(ab.feat);
    dfree(ab.pred);
    dfree(ab.tileErr);
    bilatOut = nullptr;
    dfree(gauss);
    dfree(sampleN);
    if (hostResult) cudaFreeHost(hostResult);
    hostResult = nullptr;
    hostResultN = 0;
    alloc = false;
  }
  ~gbpt_renderer() {
    if (st) cudaStreamSynchronize(st);
    free_dev();
    for (auto e : evPool) cudaEventDestroy(e);
    for (cudaGraphExec_t& x : gexec)
      if (x) cudaGraphExecDestroy(x);
    for (cudaEvent_t e : {evMain, evLight[0], evLight[1], evFork})
      if (e) cudaEventDestroy(e);
    for (uint32_t b = 0; b < kMaxBands; b++) {
      if (evJoin[b]) cudaEventDestroy(evJoin[b]);
      if (stBand[b]) {
        cudaStreamSynchronize(stBand[b]);
        cudaStreamDestroy(stBand[b]);
      }
    }
    if (stLight) cudaStreamDestroy(stLight);
    if (st && !userStream) cudaStreamDestroy(st);
    if (ownSt && ownSt != st) cudaStreamDestroy(ownSt);
  }
};

namespace {

gbpt_status check_params(const gbpt_params* p) {
  if (!p) return fail(GBPT_ERR_INVALID_ARG, "params is NULL");
  if (p->eye_depth_max < 1 || p->eye_depth_max > 64) return fail(GBPT_ERR_INVALID_ARG, "eye_depth_max must be 1..64");
  if (p->light_depth_max < 1 || p->light_depth_max > 64)
    return fail(GBPT_ERR_INVALID_ARG, "light_depth_max must be 1..64");
  if (p->light_paths > 1024) return fail(GBPT_ERR_INVALID_ARG, "light_paths must be <= 1024");
  if (p->light_every < 1) return fail(GBPT_ERR_INVALID_ARG, "light_every must be >= 1");
  if (p->filter_radius > 31) return fail(GBPT_ERR_INVALID_ARG, "filter_radius must be <= 31");
  if (p->bilat_radius > 31) return fail(GBPT_ERR_INVALID_ARG, "bilat_radius must be <= 31");
  if (p->pt_depth_max < 1 || p->pt_depth_max > 64) return fail(GBPT_ERR_INVALID_ARG, "pt_depth_max must be 1..64");
  if (p->walk_refill > 32) return fail(GBPT_ERR_INVALID_ARG, "walk_refill must be 0..32");
  if (p->tail_from < -1) return fail(GBPT_ERR_INVALID_ARG, "tail_from must be >= -1");
  if (p->bands > kMaxBands) return fail(GBPT_ERR_INVALID_ARG, "bands must be 0..8");
  if (p->walk_ctas > 32) return fail(GBPT_ERR_INVALID_ARG, "walk_ctas must be 0..32");
  if (p->carry_steps > (1u << 20)) return fail(GBPT_ERR_INVALID_ARG, "carry_steps must be <= 2^20");
  if (!(p->tail_below >= 0.f && p->tail_below <= 1.f))
    return fail(GBPT_ERR_INVALID_ARG, "tail_below must be in [0, 1]");
  return GBPT_OK;
}

// Bands of a frame: `requested` when set, else 1 when the bounce launches
// carry their last walks on (carrying removes the per-launch wait that bands
// partly overlap; carrying with 2 bands measured 127-164 against 173 Mpaths/s
// with 1 on the hall), else 2 from 512K camera paths.  Measured on GB300
// (Mpaths/s, 1 / 2 / 3 / 4 bands, no carrying): hall 1280x720 175.6 / 180.9 /
// 176.4 / 165.3, interior 1024x768 154.7 / 157.4 / 144.8 / 137.1, Cornell
// 256x256 206.3 / 188.6 (1 / 2).  A band's persistent walk holds its SMs
// until its queue drains, so the bands of one frame stay nearly in step.
uint32_t bands_for(uint32_t requested, size_t paths, bool carrying) {
  if (requested) return std::min<uint32_t>(requested, kMaxBands);
  if (carrying) return 1;
  return paths >= (1u << 19) ? 2u : 1u;
}

// The buffers of band b of k: pixels [b*np/k, (b+1)*np/k); the wave, hit and
// connection-queue arrays start at the band's first pixel, the counters are
// the band's own.
RenderBuffers band_buffers(const RenderBuffers& rb, uint32_t b, uint32_t k, size_t np) {
  RenderBuffers x = rb;
  const size_t p0 = np * b / k, p1 = np * (b + 1) / k;
  x.base = (uint32_t)p0;
  x.count = (uint32_t)(p1 - p0);
  for (int w = 0; w < 2; w++) {
    x.wave[w].o += p0;
    x.wave[w].d += p0;
    x.wave[w].thr += p0;
    x.wave[w].smp += p0;
  }
  const size_t c0 = (size_t)rb.carryCap * b / k, c1 = (size_t)rb.carryCap * (b + 1) / k;
  x.hit += p0 + c0;  // the band's paths and the walks it resumes: count + its carry records
  x.sh[0] += 3 * p0;
  x.sh[1] += 3 * p0;
  x.ctr = rb.ctr + b;
  x.lctr = rb.ctr;
  x.carry[0] = rb.carry[0] + c0 * kCarryF4;
  x.carry[1] = rb.carry[1] + c0 * kCarryF4;
  x.carryCap = (uint32_t)(c1 - c0);
  return x;
}

}  // namespace

uint64_t gbpt::renderer_bytes(uint32_t W, uint32_t H, const gbpt_params& p) {
  const size_t np = (size_t)W * H;
  const uint32_t cacheCap = std::max(1u, p.light_paths * (1 + p.light_depth_max));
  return np * (128 + 16 + 96 + 16 + 48 + 16 + 8) + np * (12 * 10 + 4 * 2 + 4 * 5) + (size_t)cacheCap * 192 +
         std::max<size_t>(std::min<size_t>(np, walk_lanes()), 256) * (2 * kCarryF4 + 1) * 16 +
         np * 16 * (std::max(std::max(p.eye_depth_max, p.pt_depth_max), 2u) - 1);
}

namespace {

gbpt_status ensure_alloc(gbpt_renderer* r) {
  if (r->alloc) return GBPT_OK;
  const size_t np = (size_t)r->W * r->H;
  const size_t cap = np;
  const uint32_t cacheCap = std::max(1u, r->p.light_paths * (1 + r->p.light_depth_max));
  // admission: refuse when the buffers cannot fit in free HBM
  const size_t need = renderer_bytes(r->W, r->H, r->p);
  size_t freeB = 0, totB = 0;
  CK(cudaMemGetInfo(&freeB, &totB));
  if (need + (64ull << 20) > freeB)
    return fail(GBPT_ERR_OOM, "renderer needs " + std::to_string(need) + " bytes, " + std::to_string(freeB) +
                                  " free");
  CK(dalloc(&r->waveMem, cap * 8));
  for (int k = 0; k < 2; k++) {
    float4* b = r->waveMem + (size_t)k * 4 * cap;
    r->rb.wave[k] = Wave{b, b + cap, b + 2 * cap, b + 3 * cap};
  }
  // carry records: as many as the walk grid has lanes (a launch carries at
  // most one walk per lane), but no more than paths.  Hit words: one per live
  // path of the wave, plus one per walk a launch resumes (carried connection
  // walks are not paths: they take words past the paths').
  r->rb.carryCap = (uint32_t)std::max<size_t>(std::min<size_t>(cap, walk_lanes()), 256);
  CK(dalloc(&r->rb.hit, cap + r->rb.carryCap));
  CK(dalloc(&r->rb.sh[0], cap * 3));
  CK(dalloc(&r->rb.sh[1], cap * 3));
  CK(dalloc(&r->rb.res, cap));
  CK(dalloc(&r->rb.gbuf, cap * 3));
  CK(dalloc(&r->rb.dsm, cap));
  CK(dalloc(&r->rb.slotPix, cap));
  CK(dalloc(&r->rb.slotSmp, cap));
  CK(dalloc(&r->rb.cache[0], (size_t)cacheCap * 6));
  CK(dalloc(&r->rb.cache[1], (size_t)cacheCap * 6));
  CK(dalloc(&r->rb.carry[0], (size_t)r->rb.carryCap * kCarryF4));
  CK(dalloc(&r->rb.carry[1], (size_t)r->rb.carryCap * kCarryF4));
  CK(dalloc(&r->rb.ctr, kMaxBands));
  CK(cudaMemsetAsync(r->rb.ctr, 0, sizeof(DevCounters) * kMaxBands, r->st));
  r->rb.lctr = r->rb.ctr;
  r->rb.base = 0;
  r->rb.count = (uint32_t)np;
  CK(cudaMemsetAsync(r->rb.cache[0], 0, (size_t)cacheCap * 96, r->st));
  CK(cudaMemsetAsync(r->rb.cache[1], 0, (size_t)cacheCap * 96, r->st));
  r->rb.cap = (uint32_t)cap;
  r->rb.cacheCap = cacheCap;
  CK(dalloc(&r->result, np * 3));
  CK(dalloc(&r->gpos, np * 3));
  CK(dalloc(&r->gnorm, np * 3));
  CK(dalloc(&r->gdiff, np * 3));
  CK(dalloc(&r->gemis, np * 3));
  CK(dalloc(&r->direct, np * 3));
  CK(dalloc(&r->pot, np));
  CK(dalloc(&r->filtered2, np * 3));
  CK(dalloc(&r->probView, np * 3));
  const size_t nTiles = (size_t)((r->W + 7) / 8) * ((r->H + 7) / 8);
  CK(dalloc(&r->rb.m2, np * 3));
  CK(dalloc(&r->rb.hist, nTiles * 8));
  CK(dalloc(&r->ab.feat, nTiles * kFeatures));
  CK(dalloc(&r->ab.pred, nTiles));
  CK(dalloc(&r->ab.tileErr, nTiles));
  CK(cudaMemsetAsync(r->rb.m2, 0, np * 12, r->st));
  CK(cudaMemsetAsync(r->rb.hist, 0, nTiles * 32, r->st));
  CK(dalloc(&r->sampleN, np));
  CK(dalloc(&r->gauss, 64));
  CK(dalloc(&r->ab.err, np));
  CK(dalloc(&r->ab.cnt, np));
  CK(dalloc(&r->ab.off, np));
  CK(dalloc(&r->ab.blockSum, adapt_scan_blocks((uint32_t)np)));
  CK(dalloc(&r->ab.partial, adapt_reduce_blocks((uint32_t)np)));
  CK(dalloc(&r->ab.filtered, np * 3));
  CK(dalloc(&r->ab.coop, kCoopWords));
  CK(dalloc(&r->ab.heavy, np));
  CK(dalloc(&r->ab.list8, np));
  CK(cudaMemsetAsync(r->ab.coop, 0, kCoopWords * 4, r->st));
  for (float* b : {r->result, r->gpos, r->gnorm, r->gdiff, r->ab.filtered, r->gemis, r->direct, r->filtered2,
                   r->probView})
    CK(cudaMemsetAsync(b, 0, np * 12, r->st));
  CK(cudaMemsetAsync(r->pot, 0, np * 4, r->st));
  r->bilatOut = r->ab.filtered;
  CK(cudaMemsetAsync(r->sampleN, 0, np * 4, r->st));
  CK(cudaMemsetAsync(r->ab.err, 0, np * 4, r->st));
  CK(cudaMallocHost((void**)&r->hostResult, np * 12));
  std::memset(r->hostResult, 0, np * 12);
  r->hostResultN = np * 3;
  r->alloc = true;
  r->gaussKey[0] = r->gaussKey[1] = -1.f;
  return GBPT_OK;
}

// host camera basis, src/cudaRTBDPTStream.cu:823-824 (host Vec3 algebra)
void cam_basis(const gbpt_camera& c, float right[3], float up[3]) {
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

void gaussian_table_host(float delta, uint32_t radius, float* g) {  // src/cudaBilateralFilter.cu:5-24
  for (uint32_t i = 0; i < 2 * radius + 1; i++) {
    int x = (int)i - (int)radius;
    g[i] = gb::exp_p((float)(-(x * x)) / (2 * delta * delta));
  }
}

cudaEvent_t mark(gbpt_renderer* r, int phase, bool timing) {
  if (!timing) return nullptr;
  cudaEvent_t e;
  size_t used = r->evs.size();
  if (used < r->evPool.size()) {
    e = r->evPool[used];
  } else {
    cudaEventCreate(&e);
    r->evPool.push_back(e);
  }
  cudaEventRecord(e, r->st);
  r->evs.push_back({phase, e});
  return e;
}

gbpt_status ensure_gauss(gbpt_renderer* r, float delta, uint32_t radius, cudaStream_t st) {
  if (r->gaussKey[0] != delta || r->gaussKey[1] != (float)radius) {
    float g[64] = {0};
    gaussian_table_host(delta, radius, g);
    CK(cudaMemcpyAsync(r->gauss, g, sizeof(g), cudaMemcpyHostToDevice, st));
    r->gaussKey[0] = delta;
    r->gaussKey[1] = (float)radius;
  }
  return GBPT_OK;
}

// Filter stage of the filter-only mode (src/cudaRTBDPTStreamBilat.cu:1418-1432):
// posnormemit with the first-hit diffuse plane as the third feature, then
// "Filter Iteration" - 1 more passes ping-ponging between two planes.  Debug
// modes 2/3 filter the path-potential view instead of the result (the
// reference overwrites its accumulator with that view; here it stays intact).
gbpt_status bilat_filter(gbpt_renderer* r, cudaStream_t st, bool timing) {
  const gbpt_params& p = r->p;
  const float delta = p.filter_sigma_spatial > 0.f ? p.filter_sigma_spatial : p.bilat_color_eud;
  gbpt_status e = ensure_gauss(r, delta, p.bilat_radius, st);
  if (e != GBPT_OK) return e;
  const float* src = r->result;
  const int dm = (int)r->debugMode;
  if (dm == 2 || dm == 3) {
    CK(launch_prob_view(r->pot, r->W * r->H, dm == 3 ? p.min_trace_prob : 0.f, r->probView, st));
    src = r->probView;
  }
  float* planes[2] = {r->ab.filtered, r->filtered2};
  int cur = 0;
  CK(launch_bilateral(src, r->gpos, r->gnorm, r->gdiff, r->W, r->H, p.bilat_color_eud, p.bilat_pos_eud,
                      p.bilat_norm_eud, p.bilat_diff_eud, p.bilat_radius, r->gauss, planes[cur], st));
  for (uint32_t i = 1; i < p.filter_iterations; i++) {
    CK(launch_bilateral(planes[cur], r->gpos, r->gnorm, r->gdiff, r->W, r->H, p.bilat_color_eud, p.bilat_pos_eud,
                        p.bilat_norm_eud, p.bilat_diff_eud, p.bilat_radius, r->gauss, planes[cur ^ 1], st));
    cur ^= 1;
  }
  r->bilatOut = planes[cur];
  mark(r, kPhFilter, timing);
  return GBPT_OK;
}

gbpt_status frame_once(gbpt_renderer* r, gbpt_scene* s, const gbpt_camera* cam, bool timing) {
  float right[3], up[3];
  cam_basis(*cam, right, up);
  float basis9[9] = {cam->pos[0], cam->pos[1], cam->pos[2], cam->dir[0], cam->dir[1],
                     cam->dir[2], up[0],       up[1],       up[2]};
  if (r->resumeScene) {
    if (s->dev.triN != r->resumeTriN || s->bvh.nodeN != r->resumeNodeN)
      return fail(GBPT_ERR_STATE, "the checkpoint was made with another scene");
    r->sceneVersion = s->version;
    r->resumeScene = false;
  }
  bool same = r->started && r->sceneVersion == s->version && std::memcmp(basis9, r->camBasis, sizeof(basis9)) == 0;
  r->frame = same ? r->frame + 1 : 0;
  if (!same) r->epoch++;  // light passes made ahead for the old sequence are stale
  std::memcpy(r->camBasis, basis9, sizeof(basis9));
  r->started = true;
  r->sceneVersion = s->version;
  r->lastTriN = s->dev.triN;
  r->lastNodeN = s->bvh.nodeN;

  FrameArgs a{};
  for (int k = 0; k < 3; k++) {
    a.camPos[k] = cam->pos[k];
    a.camDir[k] = cam->dir[k];
    a.camUp[k] = up[k];
    a.camRight[k] = right[k];
  }
  a.tanHalf = (float)std::tan((double)(cam->fov * 0.5f));
  const uint32_t fullW = r->fullW ? r->fullW : r->W, fullH = r->fullH ? r->fullH : r->H;
  a.W = (float)fullW;
  a.H = (float)fullH;
  a.width = r->W;
  a.height = r->H;
  a.winX0 = r->winX0;
  a.winY0 = r->winY0;
  a.fullW = fullW;
  a.frame = r->frame;
  a.key0 = r->p.seed;
  a.key1 = r->p.request_id;
  const bool pt = r->mode == GBPT_MODE_PT_SC;  // unidirectional: no light pass, no connections
  a.ptsc = pt ? 1u : 0u;
  a.eyeDepth = pt ? r->p.pt_depth_max : r->p.eye_depth_max;
  a.lightDepth = r->p.light_depth_max;
  a.lightPaths = r->p.light_paths;
  for (int k = 0; k < 3; k++) a.env[k] = r->p.env[k];
  a.useEnv = (r->p.env[0] != 0.f || r->p.env[1] != 0.f || r->p.env[2] != 0.f) ? 1u : 0u;
  const bool adaptive = r->mode == GBPT_MODE_BDPT_SC_ADAP_BILAT || r->mode == GBPT_MODE_BDPT_SC_ADAP_BILAT_BINARY;
  const bool binary = r->mode == GBPT_MODE_BDPT_SC_ADAP_BILAT_BINARY;
  if (adaptive && (fullW != r->W || fullH != r->H))
    return fail(GBPT_ERR_STATE, "the adaptive modes render whole images only: their sample budget and filter "
                                "couple every pixel of the image");
  // the PLL variant pushes the specular origin along reflDir (AdapBilatAtomic.cu:583); the others do not
  a.specPush = r->mode == GBPT_MODE_BDPT_SC_ADAP_BILAT ? 1u : 0u;
  const bool bilat = r->mode == GBPT_MODE_BDPT_SC_BILAT;
  a.gbuffer = (adaptive || bilat) ? 1u : 0u;
  a.bilat = bilat ? 1u : 0u;
  // learned allocator (PLL adaptive mode): second moments and path-length counts
  const bool learned = r->mlp != nullptr && r->mode == GBPT_MODE_BDPT_SC_ADAP_BILAT;
  a.moments = (learned || (r->collect && adaptive)) ? 1u : 0u;
  a.tilesX = (r->W + 7) / 8;
  a.refill = r->p.walk_refill;
  a.walkCtas = r->p.walk_ctas;
  a.carrySteps = r->p.carry_steps;
  a.tailBelow = r->p.tail_below;
  if (a.moments && r->frame == 0)
    CK(cudaMemsetAsync(r->rb.hist, 0, (size_t)a.tilesX * ((r->H + 7) / 8) * 32, r->st));
  a.counting = r->counting ? 1u : 0u;
  const DevScene& S = s->dev;
  cudaStream_t st = r->st;
  // filter-only mode: frames past "Render Iteration" trace nothing and only
  // filter again (src/cudaRTBDPTStreamBilat.cu:1278)
  const uint32_t RI = r->p.render_iterations;
  auto traces = [&](uint32_t f) { return !bilat || RI == 0 || f < RI; };
  r->lastTraced = traces(r->frame);
  if (!r->lastTraced) return bilat_filter(r, st, timing);

  // plain and PTSC frames can be issued as one CUDA graph (gbpt_renderer_set_graphs)
  const bool useGraph = r->graphs && !a.counting && (r->mode == GBPT_MODE_BDPT_SC || pt);
  mark(r, kPhOther, timing);
  // light pass (src/cudaRTBDPTStream.cu:875-906): group g = frame / light_every
  // reads cache g % 2.  Its light pass normally ran ahead on the side stream;
  // if not (first group, camera change), it runs here on the main stream.
  const uint32_t k = r->p.light_every;
  const uint32_t g = r->frame / k;
  const uint32_t sel = g & 1u;
  const uint32_t nsel = sel ^ 1u;
  a.cacheSel = sel;
  r->lastSel = sel;
  bool inlineLight = false, ahead = false;
  // the group's first frame: its light pass (a frame inside a group whose
  // cache is not there -- after a restored checkpoint -- makes it too)
  const uint32_t g0 = r->frame - r->frame % k;
  FrameArgs al = a;
  al.frame = g0;
  if (!pt && (r->frame == g0 || r->cacheEpoch[sel] != r->epoch || r->cacheFrame[sel] != g0)) {
    const bool ready = r->cacheEpoch[sel] == r->epoch && r->cacheFrame[sel] == g0;
    if (r->lightPending[sel]) CK(cudaStreamWaitEvent(st, r->evLight[sel], 0));
    r->lightPending[sel] = false;
    inlineLight = !ready;
    if (!ready) {
      r->cacheEpoch[sel] = r->epoch;
      r->cacheFrame[sel] = g0;
    }
    ahead = r->frame == g0 && traces(r->frame + k);
  }
  // the next group's light pass, ahead, into the other cache: it waits for
  // everything queued so far (earlier frames that read that cache)
  auto launch_ahead = [&]() -> gbpt_status {
    CK(cudaEventRecord(r->evMain, st));
    CK(cudaStreamWaitEvent(r->stLight, r->evMain, 0));
    FrameArgs an = a;
    an.frame = r->frame + k;
    an.cacheSel = nsel;
    CK(launch_light_pass(S, an, r->rb, r->stLight));
    CK(cudaEventRecord(r->evLight[nsel], r->stLight));
    r->lightPending[nsel] = true;
    r->cacheEpoch[nsel] = r->epoch;
    r->cacheFrame[nsel] = r->frame + k;
    return GBPT_OK;
  };
  // camera rays (or the adaptive budget), the bounce loop, accumulation;
  // tm: phase events between the launches
  auto body = [&](bool tm) -> gbpt_status {
    const bool budgeted = adaptive && r->frame >= r->p.warmup_frames;
    if (budgeted) {
      float delta = r->p.filter_sigma_spatial > 0.f ? r->p.filter_sigma_spatial : r->p.filter_color_eud;
      gbpt_status ge = ensure_gauss(r, delta, r->p.filter_radius, st);
      if (ge != GBPT_OK) return ge;
      CK(launch_bilateral(r->result, r->gpos, r->gnorm, r->p.filter_diffuse ? r->gdiff : nullptr, r->W, r->H,
                          r->p.filter_color_eud, r->p.filter_pos_eud, r->p.filter_norm_eud, r->p.filter_diff_eud,
                          r->p.filter_radius, r->gauss, r->ab.filtered, st));
      mark(r, kPhFilter, tm);
      if (binary)
        CK(launch_binary_budget(a, r->rb, r->ab, r->result, r->sampleN, r->p.desired_n, r->p.min_trace_prob, st));
      else if (learned) {  // heuristic error -> tile features -> MLP -> per-pixel weights -> budget
        CK(launch_adapt_error(a, r->ab, r->result, r->sampleN, r->p.desired_n, st));
        CK(launch_tile_features(a, r->rb, r->ab, r->result, r->sampleN, r->gpos, r->gnorm, r->gdiff, st));
        const uint32_t nTiles = a.tilesX * ((r->H + 7) / 8);
        gbpt_status ms = mlp_forward_async(r->mlp, r->ab.feat, nTiles, r->ab.pred, &r->rb.ctr->errFlags,
                                           kErrMlpTimeout, st);
        if (ms != GBPT_OK) return ms;
        CK(launch_mlp_alloc(a, r->ab, st));
        CK(launch_adapt_alloc(a, r->rb, r->ab, st));
      } else
        CK(launch_adapt_budget(a, r->rb, r->ab, r->result, r->sampleN, r->p.desired_n, st));
      mark(r, kPhAdapt, tm);
    }
    // bounce launch d < K: walk (the walks launch d - 1 carried, the extension
    // rays of its wave, the shadow rays of launch d - 1), then shade, one launch
    // each; from K (or the bounce a shading launch switched at): one persistent
    // kernel per frame carries every remaining path to its end (few paths are
    // left by then, and per-bounce launches would each wait for their slowest
    // ray).  Without carrying or a switch on the device and with K = D, the
    // last launch walks the final connections instead of the tail kernel.
    const uint32_t D = a.eyeDepth;
    const bool wideT = S.traversal == 1 && S.wide;
    const bool carrying = a.carrySteps && !wideT;
    const size_t np = (size_t)r->W * r->H;
    const uint32_t nb = adaptive ? 1u : bands_for(r->p.bands, np, carrying);
    const uint32_t K = std::min(tail_from(D, wideT, r->p.tail_from, np / nb, carrying), D);
    const bool tailRun = K < D || carrying || a.tailBelow > 0.f;
    auto bounces = [&](const RenderBuffers& rbx, cudaStream_t sx, bool mk) -> gbpt_status {
      int in = 0;
      for (uint32_t d = 0; d < K; d++) {
        CK(launch_walk(S, a, rbx, in, d > 0 ? (int)((d - 1) & 1u) : -1, (int)(d & 1u), d, sx));
        if (mk) mark(r, kPhTrace, tm);
        CK(launch_shade(S, a, rbx, in, d, tailRun && d + 1 == K, sx));
        if (mk) mark(r, kPhShade, tm);
        in ^= 1;
      }
      if (tailRun) {
        CK(launch_tail(S, a, rbx, K, sx));
      } else {
        // shadow rays of the last bounce (none in practice: paths at the depth cap
        // terminate without connecting; kept so the sequence needs no special case)
        CK(launch_walk(S, a, rbx, -1, (int)((D - 1) & 1u), (int)(D & 1u), D, sx));
      }
      CK(launch_fold(rbx, sx));
      return GBPT_OK;
    };
    r->lastBands = nb;
    if (budgeted || nb == 1) {
      if (!budgeted) {
        CK(launch_camera(a, r->rb, st));
        mark(r, kPhOther, tm);
      }
      gbpt_status be = bounces(r->rb, st, true);
      if (be != GBPT_OK) return be;
    } else {
      // one wavefront per band: camera rays and every bounce of the band on its
      // own stream; the apply below waits for all of them.  Results do not
      // depend on the split: every path's random numbers follow from its pixel.
      CK(cudaEventRecord(r->evFork, st));
      for (uint32_t b = 0; b < nb; b++) {
        cudaStream_t sb = r->stBand[b];
        CK(cudaStreamWaitEvent(sb, r->evFork, 0));
        const RenderBuffers rbb = band_buffers(r->rb, b, nb, np);
        CK(launch_camera(a, rbb, sb));
        gbpt_status be = bounces(rbb, sb, false);
        if (be != GBPT_OK) return be;
        CK(cudaEventRecord(r->evJoin[b], sb));
      }
      for (uint32_t b = 0; b < nb; b++) CK(cudaStreamWaitEvent(st, r->evJoin[b], 0));
    }
    mark(r, kPhTrace, tm);
    if (budgeted) {
      if (binary)
        CK(launch_binary_apply(a, r->rb, r->ab, r->result, r->sampleN, r->gpos, r->gnorm, r->gdiff, st));
      else
        CK(launch_adapt_accum(a, r->rb, r->ab, r->result, r->sampleN, r->gpos, r->gnorm, r->gdiff, st));
      mark(r, kPhAdapt, tm);
    } else if (pt) {
      CK(launch_apply_pt(a, r->rb, r->result, r->sampleN, st));
      mark(r, kPhOther, tm);
    } else if (bilat) {
      CK(launch_apply_bilat(a, r->rb, r->result, r->sampleN, r->gpos, r->gnorm, r->gdiff, r->gemis, r->direct, r->pot,
                            st));
      mark(r, kPhOther, tm);
      return bilat_filter(r, st, tm);
    } else {
      CK(launch_apply(a, r->rb, r->result, r->sampleN, adaptive ? r->gpos : nullptr, r->gnorm, r->gdiff, st));
      mark(r, kPhOther, tm);
    }
    return GBPT_OK;
  };

  if (!useGraph || !r->graphWarm) {
    if (inlineLight) {
      CK(launch_light_pass(S, al, r->rb, st));
      mark(r, kPhLight, timing);
    }
    if (ahead) {
      gbpt_status e = launch_ahead();
      if (e != GBPT_OK) return e;
    }
    if (useGraph) {  // kernels load and launch shapes are queried on first use: outside any capture
      prepare_launches();
      r->graphWarm = true;
    }
    return body(timing);
  }
  // One graph per frame: captured, then applied to the renderer's executable
  // graph of the same shape (with or without an inline light pass) by
  // cudaGraphExecUpdate, which keeps the instantiation when only kernel
  // arguments changed.  The light pass ahead is issued after the frame.
  CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  gbpt_status bs = GBPT_OK;
  if (inlineLight) {
    const cudaError_t le = launch_light_pass(S, al, r->rb, st);
    if (le != cudaSuccess) bs = fail(GBPT_ERR_CUDA, std::string("light pass: ") + cudaGetErrorString(le));
  }
  if (bs == GBPT_OK) bs = body(false);
  cudaGraph_t graph = nullptr;
  const cudaError_t ce = cudaStreamEndCapture(st, &graph);
  if (bs != GBPT_OK || ce != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    if (bs != GBPT_OK) return bs;
    return fail(GBPT_ERR_CUDA, std::string("cudaStreamEndCapture: ") + cudaGetErrorString(ce));
  }
  cudaGraphExec_t& ex = r->gexec[inlineLight ? 1 : 0];
  if (ex) {
    cudaGraphExecUpdateResultInfo info;
    if (cudaGraphExecUpdate(ex, graph, &info) != cudaSuccess) {
      cudaGetLastError();
      cudaGraphExecDestroy(ex);
      ex = nullptr;
    }
  }
  cudaError_t ie = cudaSuccess;
  if (!ex) ie = cudaGraphInstantiate(&ex, graph, 0);
  cudaGraphDestroy(graph);
  if (ie != cudaSuccess) {
    ex = nullptr;
    return fail(GBPT_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(ie));
  }
  CK(cudaGraphLaunch(ex, st));
  mark(r, kPhTrace, timing);
  if (ahead) return launch_ahead();
  return GBPT_OK;
}

struct CtrSnap {
  unsigned long long rays, nodes, tris;
};

// The renderer's counters with the bands' work counters, paths and error
// words added into the first band's.
gbpt_status read_ctr(gbpt_renderer* r, DevCounters* out) {
  DevCounters c[kMaxBands];
  CK(cudaMemcpyAsync(c, r->rb.ctr, sizeof(c), cudaMemcpyDeviceToHost, r->st));
  CK(cudaStreamSynchronize(r->st));
  *out = c[0];
  for (uint32_t b = 1; b < kMaxBands; b++) {
    out->rays += c[b].rays;
    out->nodes += c[b].nodes;
    out->tris += c[b].tris;
    out->shadowRays += c[b].shadowRays;
    out->nodesS += c[b].nodesS;
    out->trisS += c[b].trisS;
    out->errFlags |= c[b].errFlags;
    if (b < r->lastBands) out->paths += c[b].paths;
  }
  return GBPT_OK;
}

// The image gbpt_render copies out: the result, or the mode's debug view.
const float* output_view(const gbpt_renderer* r) {
  if (r->mode == GBPT_MODE_BDPT_SC_BILAT) {  // src/cudaRTBDPTStreamBilat.cu:1440-1459
    const int dm = (int)r->debugMode;
    return dm == 4 ? r->direct : dm == 5 ? r->gpos : dm == 6 ? r->gnorm : dm == 7 ? r->result : r->bilatOut;
  }
  return (r->debugMode == 4.f && r->mode != GBPT_MODE_BDPT_SC) ? r->ab.filtered : r->result;
}

// The per-bounce connection entries for the renderer's depth caps, grown when
// a cap grows (D - 1 bounces make connections: paths end at the cap).
gbpt_status ensure_conn(gbpt_renderer* r) {
  const uint32_t need = std::max(std::max(r->p.eye_depth_max, r->p.pt_depth_max), 2u) - 1;
  if (r->rb.conn && r->rb.connDepth >= need) return GBPT_OK;
  if (r->rb.conn) {
    CK(cudaStreamSynchronize(r->st));
    dfree(r->rb.conn);
  }
  r->rb.connDepth = 0;
  CK(dalloc(&r->rb.conn, (size_t)r->rb.cap * need));
  r->rb.connDepth = need;
  return GBPT_OK;
}

gbpt_status render_impl(gbpt_renderer* r, gbpt_scene* s, const gbpt_camera* cam, uint32_t frames, float* out,
                        int32_t outDev, gbpt_stats* stats) {
  if (!r || !s || !cam) return fail(GBPT_ERR_INVALID_ARG, "NULL renderer, scene or camera");
  gbpt_status stt = ensure_uploaded(s);
  if (stt != GBPT_OK) return stt;
  stt = ensure_alloc(r);
  if (stt != GBPT_OK) return stt;
  stt = ensure_conn(r);
  if (stt != GBPT_OK) return stt;
  DevCounters before{};
  const bool timing = stats != nullptr;
  if (timing) {
    stt = read_ctr(r, &before);
    if (stt != GBPT_OK) return stt;
  }
  const uint64_t launches0 = launch_count();
  r->evs.clear();
  for (uint32_t f = 0; f < frames; f++) {
    // NVTX range per frame (free without a profiler attached; ncu --nvtx can filter on it)
    nvtxRangePushA("gbpt frame");
    stt = frame_once(r, s, cam, timing);
    nvtxRangePop();
    if (stt != GBPT_OK) return stt;
  }
  const size_t np = (size_t)r->W * r->H;
  if (out) CK(cudaMemcpyAsync(out, output_view(r), np * 12, outDev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                             r->st));
  CK(cudaStreamSynchronize(r->st));
  CK(cudaGetLastError());
  {  // device-side error words (bounded waits, bounds checks) of every band: report once, then clear
    uint32_t flags = 0;
    DevCounters c{};
    stt = read_ctr(r, &c);
    if (stt != GBPT_OK) return stt;
    flags = c.errFlags;
    if (flags) {
      for (uint32_t b = 0; b < kMaxBands; b++) CK(cudaMemsetAsync(&r->rb.ctr[b].errFlags, 0, 4, r->st));
      CK(cudaStreamSynchronize(r->st));
      if (flags & 4u) return fail(GBPT_ERR_TIMEOUT, "grid barrier of the binary allocator timed out");
      if (flags & kErrMlpTimeout) return fail(GBPT_ERR_TIMEOUT, "learned allocator: tensor-core wait timed out");
      return fail(GBPT_ERR_BOUNDS, "device bounds check tripped (light cache)");
    }
  }
  if (timing) {
    DevCounters after{};
    stt = read_ctr(r, &after);
    if (stt != GBPT_OK) return stt;
    std::memset(stats, 0, sizeof(*stats));
    stats->frame = r->frame;
    stats->light_vertices = r->mode == GBPT_MODE_PT_SC ? 0u : after.cacheSize[r->lastSel];
    stats->paths = r->lastTraced ? after.paths : 0;
    stats->rays = after.rays - before.rays;
    stats->nodes = after.nodes - before.nodes;
    stats->tris = after.tris - before.tris;
    stats->shadow_rays = after.shadowRays - before.shadowRays;
    stats->shadow_nodes = after.nodesS - before.nodesS;
    stats->shadow_tris = after.trisS - before.trisS;
    float ph[kPhN] = {0};
    for (size_t i = 1; i < r->evs.size(); i++) {
      float ms = 0.f;
      cudaEventElapsedTime(&ms, r->evs[i - 1].second, r->evs[i].second);
      ph[r->evs[i].first] += ms;
    }
    if (r->evs.size() > 1) cudaEventElapsedTime(&stats->ms_total, r->evs.front().second, r->evs.back().second);
    stats->ms_light = ph[kPhLight];
    stats->ms_trace = ph[kPhTrace];
    stats->ms_shade = ph[kPhShade];
    stats->ms_shadow = ph[kPhShadow];
    stats->ms_filter = ph[kPhFilter];
    stats->ms_adapt = ph[kPhAdapt];
    stats->launches = (uint32_t)(launch_count() - launches0);
  }
  return GBPT_OK;
}

struct AttrDef {
  const char* name;
  int kind;  // 0 float, 1 uint, 2 the renderer's debug view
  size_t off;
};
// reference attribute names first (src/cudaRTBDPTStreamAdapBilatAtomic.cu:48-60)
const AttrDef kAttrs[] = {
    {"Desired Max Sampling", 1, offsetof(gbpt_params, desired_n)},
    {"Filter Color EuD", 0, offsetof(gbpt_params, filter_color_eud)},
    {"Filter Pos EuD", 0, offsetof(gbpt_params, filter_pos_eud)},
    {"Filter Norm EuD", 0, offsetof(gbpt_params, filter_norm_eud)},
    {"Filter Diff EuD", 0, offsetof(gbpt_params, filter_diff_eud)},
    {"Filter Radius", 1, offsetof(gbpt_params, filter_radius)},
    {"Filter Diffuse Flag", 1, offsetof(gbpt_params, filter_diffuse)},
    {"Eye Depth Max", 1, offsetof(gbpt_params, eye_depth_max)},
    {"Light Depth Max", 1, offsetof(gbpt_params, light_depth_max)},
    {"Light Paths", 1, offsetof(gbpt_params, light_paths)},
    {"Light Pass Every", 1, offsetof(gbpt_params, light_every)},
    {"Warmup Frames", 1, offsetof(gbpt_params, warmup_frames)},
    {"Filter Sigma Spatial", 0, offsetof(gbpt_params, filter_sigma_spatial)},
    {"Seed", 1, offsetof(gbpt_params, seed)},
    {"Min Trace Probability", 0, offsetof(gbpt_params, min_trace_prob)},
    {"Debug Mode", 2, 0},
};
constexpr uint32_t kAttrN = sizeof(kAttrs) / sizeof(kAttrs[0]);
// "BDPTSC Bilaterial" (src/cudaRTBDPTStreamBilat.cu:40-50), then the defines
const AttrDef kAttrsBilat[] = {
    {"Filter Color E Delta", 0, offsetof(gbpt_params, bilat_color_eud)},
    {"Filter Pos E Delta", 0, offsetof(gbpt_params, bilat_pos_eud)},
    {"Filter Norm E Delta", 0, offsetof(gbpt_params, bilat_norm_eud)},
    {"Filter Emit E Delta", 0, offsetof(gbpt_params, bilat_emit_eud)},
    {"Filter Diff E Delta", 0, offsetof(gbpt_params, bilat_diff_eud)},
    {"Filter Radius", 1, offsetof(gbpt_params, bilat_radius)},
    {"Filter Iteration", 1, offsetof(gbpt_params, filter_iterations)},
    {"Debug Mode", 2, 0},
    {"Render Iteration", 1, offsetof(gbpt_params, render_iterations)},
    {"Eye Depth Max", 1, offsetof(gbpt_params, eye_depth_max)},
    {"Light Depth Max", 1, offsetof(gbpt_params, light_depth_max)},
    {"Light Paths", 1, offsetof(gbpt_params, light_paths)},
    {"Light Pass Every", 1, offsetof(gbpt_params, light_every)},
    {"Filter Sigma Spatial", 0, offsetof(gbpt_params, filter_sigma_spatial)},
    {"Seed", 1, offsetof(gbpt_params, seed)},
    {"MinTraceProb", 0, offsetof(gbpt_params, min_trace_prob)},
};
constexpr uint32_t kAttrBilatN = sizeof(kAttrsBilat) / sizeof(kAttrsBilat[0]);
// "PTSC" has no attributes in the reference (src/cudaRTPTStream.cu:10); its define and the seed
const AttrDef kAttrsPT[] = {
    {"PT Depth Max", 1, offsetof(gbpt_params, pt_depth_max)},
    {"Seed", 1, offsetof(gbpt_params, seed)},
};
constexpr uint32_t kAttrPTN = sizeof(kAttrsPT) / sizeof(kAttrsPT[0]);

const AttrDef* attr_table(const gbpt_renderer* r, uint32_t* n) {
  if (r->mode == GBPT_MODE_BDPT_SC_BILAT) {
    *n = kAttrBilatN;
    return kAttrsBilat;
  }
  if (r->mode == GBPT_MODE_PT_SC) {
    *n = kAttrPTN;
    return kAttrsPT;
  }
  *n = kAttrN;
  return kAttrs;
}

}  // namespace

extern "C" {

const char* gbpt_last_error_string(void) { return g_err.c_str(); }

gbpt_status gbpt_device_check(int32_t* ok) {
  if (!ok) return fail(GBPT_ERR_INVALID_ARG, "ok is NULL");
  *ok = 0;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) return fail(GBPT_ERR_NO_DEVICE, "no CUDA device");
  float x = 1.f, y = 0.f;
  float* d = nullptr;
  if (cudaMalloc(&d, 8) != cudaSuccess) return fail(GBPT_ERR_NO_DEVICE, "cudaMalloc failed");
  cudaMemcpy(d, &x, 4, cudaMemcpyHostToDevice);
  e = launch_fmath(4, d, 1, d + 1, nullptr);
  if (e == cudaSuccess) e = cudaMemcpy(&y, d + 1, 4, cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return fail(GBPT_ERR_NO_DEVICE, std::string("kernel launch failed: ") + cudaGetErrorString(e));
  *ok = (y == 1.f) ? 1 : 0;
  return GBPT_OK;
}

gbpt_status gbpt_params_default(gbpt_params* p) {
  if (!p) return fail(GBPT_ERR_INVALID_ARG, "params is NULL");
  std::memset(p, 0, sizeof(*p));
  p->seed = 1234;
  p->eye_depth_max = 5;
  p->light_depth_max = 5;
  p->light_paths = 128;
  p->light_every = 3;
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
  p->walk_refill = 0;
  p->tail_from = -1;
  p->bands = 0;
  p->walk_ctas = 0;
  p->carry_steps = 64;
  p->tail_below = 0.f;
  return GBPT_OK;
}

gbpt_status gbpt_scene_create(const gbpt_vertex* verts, uint32_t nv, const gbpt_triangle* tris, uint32_t nt,
                              const gbpt_material* mats, uint32_t nm, gbpt_scene** out) {
  if (!out) return fail(GBPT_ERR_INVALID_ARG, "out is NULL");
  *out = nullptr;
  if ((nv && !verts) || (nt && !tris) || (nm && !mats)) return fail(GBPT_ERR_INVALID_ARG, "NULL array");
  for (uint32_t i = 0; i < nt; i++) {
    if (tris[i].v0 >= nv || tris[i].v1 >= nv || tris[i].v2 >= nv)
      return fail(GBPT_ERR_INVALID_ARG, "triangle " + std::to_string(i) + " has a vertex index out of range");
    if (tris[i].mat >= nm)
      return fail(GBPT_ERR_INVALID_ARG, "triangle " + std::to_string(i) + " has a material index out of range");
  }
  for (uint32_t i = 0; i < nv; i++)
    for (int k = 0; k < 3; k++)
      if (!std::isfinite(verts[i].pos[k]))
        return fail(GBPT_ERR_INVALID_ARG, "vertex " + std::to_string(i) + " has a non-finite position");
  gbpt_scene* s = new (std::nothrow) gbpt_scene();
  if (!s) return fail(GBPT_ERR_OOM, "host allocation failed");
  s->verts.assign(verts, verts + nv);
  s->tris.assign(tris, tris + nt);
  s->mats.assign(mats, mats + nm);
  *out = s;
  return GBPT_OK;
}

gbpt_status gbpt_scene_destroy(gbpt_scene* s) {
  delete s;
  return GBPT_OK;
}

gbpt_status gbpt_scene_build_bvh(gbpt_scene* s, uint32_t max_depth, uint32_t threads, double* build_seconds) {
  if (!s) return fail(GBPT_ERR_INVALID_ARG, "scene is NULL");
  if (s->tris.empty()) return fail(GBPT_ERR_STATE, "scene has no triangles");
  if (max_depth == 0) max_depth = 32;
  if (threads == 0) threads = std::max(1u, std::thread::hardware_concurrency());
  auto t0 = std::chrono::steady_clock::now();
  if (!build_bvh(s->verts.data(), s->tris.data(), (uint32_t)s->tris.size(), max_depth, threads, &s->bvh))
    return fail(GBPT_ERR_STATE, "BVH compaction failed");
  s->trisOrdered.resize(s->tris.size());
  for (size_t i = 0; i < s->tris.size(); i++) s->trisOrdered[i] = s->tris[s->bvh.order[i]];
  auto t1 = std::chrono::steady_clock::now();
  if (build_seconds) *build_seconds = std::chrono::duration<double>(t1 - t0).count();
  scan_lights(s);
  s->free_dev();  // uploaded on first use (the reference uploads lazily in Render, :830-838)
  s->uploaded = false;
  s->built = true;
  s->version = next_version();
  return GBPT_OK;
}

gbpt_status gbpt_scene_set_traversal(gbpt_scene* s, int32_t traversal) {
  if (!s) return fail(GBPT_ERR_INVALID_ARG, "scene is NULL");
  if (traversal != 0 && traversal != 1) return fail(GBPT_ERR_INVALID_ARG, "traversal is 0 (reference) or 1 (wide)");
  if ((uint32_t)traversal == s->traversal) return GBPT_OK;
  s->traversal = (uint32_t)traversal;
  s->version = next_version();  // progressive accumulation restarts
  if (!s->uploaded) return GBPT_OK;
  if (traversal == 1 && !s->dWide) {
    gbpt_status w = upload_wide(s);
    if (w != GBPT_OK) return w;
  }
  s->dev.traversal = s->traversal;
  return GBPT_OK;
}

gbpt_status gbpt_scene_update_materials(gbpt_scene* s, const gbpt_material* mats, uint32_t nm) {
  if (!s || !mats) return fail(GBPT_ERR_INVALID_ARG, "NULL argument");
  if (nm != s->mats.size()) return fail(GBPT_ERR_INVALID_ARG, "material count differs from the scene's");
  s->mats.assign(mats, mats + nm);
  if (!s->built) return GBPT_OK;
  scan_lights(s);
  s->version = next_version();  // progressive accumulation restarts (src/cudaRTBDPTStream.cu:845-850)
  if (!s->uploaded) return GBPT_OK;
  gbpt_status ids = check_texture_ids(s->mats, s->textures.size());
  if (ids != GBPT_OK) {
    s->uploaded = false;  // the next use uploads again and reports the bad id
    return ids;
  }
  std::vector<float4> m = pack_materials(s->mats);
  CK(cudaMemcpy(s->dMats, m.data(), m.size() * 16, cudaMemcpyHostToDevice));
  dfree(s->dLight);
  CK(dalloc(&s->dLight, s->lightTri.size()));
  if (!s->lightTri.empty())
    CK(cudaMemcpy(s->dLight, s->lightTri.data(), s->lightTri.size() * 4, cudaMemcpyHostToDevice));
  s->dev.lightTri = s->dLight;
  s->dev.lightN = (uint32_t)s->lightTri.size();
  return GBPT_OK;
}

gbpt_status gbpt_scene_set_textures(gbpt_scene* s, const gbpt_texture* tex, uint32_t n) {
  if (!s || (n && !tex)) return fail(GBPT_ERR_INVALID_ARG, "NULL argument");
  std::vector<gbpt_scene::Texture> t(n);
  for (uint32_t i = 0; i < n; i++) {
    if (!tex[i].rgba || tex[i].width == 0 || tex[i].height == 0 || tex[i].width > 65536 || tex[i].height > 65536)
      return fail(GBPT_ERR_INVALID_ARG, "texture " + std::to_string(i) + " is empty, NULL or above 65536 texels a side");
    t[i].w = tex[i].width;
    t[i].h = tex[i].height;
    t[i].texels.resize((size_t)tex[i].width * tex[i].height);
    std::memcpy(t[i].texels.data(), tex[i].rgba, t[i].texels.size() * 16);
  }
  std::lock_guard<std::mutex> lock(s->upload);
  s->textures.swap(t);
  s->version = next_version();  // progressive accumulation restarts
  s->uploaded = false;          // the next use uploads the scene with its textures
  return GBPT_OK;
}

gbpt_status gbpt_scene_bvh_info(const gbpt_scene* s, uint32_t* node_count, uint32_t* tri_count,
                                uint32_t* light_count) {
  if (!s) return fail(GBPT_ERR_INVALID_ARG, "scene is NULL");
  if (node_count) *node_count = s->built ? s->bvh.nodeN : 0;
  if (tri_count) *tri_count = (uint32_t)s->tris.size();
  if (light_count) *light_count = (uint32_t)s->lightTri.size();
  return GBPT_OK;
}

gbpt_status gbpt_scene_bvh_export(const gbpt_scene* s, float* bounds, uint32_t* off_or_tstn, uint32_t* tri_order) {
  if (!s) return fail(GBPT_ERR_INVALID_ARG, "scene is NULL");
  if (!s->built) return fail(GBPT_ERR_STATE, "scene has no BVH");
  if (bounds) std::memcpy(bounds, s->bvh.bounds.data(), s->bvh.bounds.size() * 4);
  if (off_or_tstn) std::memcpy(off_or_tstn, s->bvh.offOrTSTN.data(), s->bvh.offOrTSTN.size() * 4);
  if (tri_order) std::memcpy(tri_order, s->bvh.order.data(), s->bvh.order.size() * 4);
  return GBPT_OK;
}

gbpt_status gbpt_trace_rays(gbpt_scene* s, const float* rays, uint32_t n, float max_dist, float eps, int32_t cullback,
                            float* t, int32_t* tri, float* w, float* u, float* v, uint32_t* nodes,
                            uint32_t* tris_tested, int32_t is_device) {
  if (!s || !rays || !t || !tri || !w || !u || !v) return fail(GBPT_ERR_INVALID_ARG, "NULL argument");
  gbpt_status up = ensure_uploaded(s);
  if (up != GBPT_OK) return up;
  if (n == 0) return GBPT_OK;
  const bool counts = nodes && tris_tested;
  if (is_device) {
    CK(launch_trace_rays(s->dev, rays, n, max_dist, eps, cullback, t, tri, w, u, v, counts ? nodes : nullptr,
                         counts ? tris_tested : nullptr, nullptr));
    CK(cudaDeviceSynchronize());
    return GBPT_OK;
  }
  float *dr = nullptr, *dt = nullptr, *dw = nullptr, *du = nullptr, *dv = nullptr;
  int32_t* di = nullptr;
  uint32_t *dn = nullptr, *dq = nullptr;
  gbpt_status st = GBPT_OK;
  auto cleanup = [&]() {
    dfree(dr); dfree(dt); dfree(dw); dfree(du); dfree(dv); dfree(di); dfree(dn); dfree(dq);
  };
  do {
    if (dalloc(&dr, (size_t)n * 6) || dalloc(&dt, n) || dalloc(&dw, n) || dalloc(&du, n) || dalloc(&dv, n) ||
        dalloc(&di, n) || dalloc(&dn, n) || dalloc(&dq, n)) {
      st = fail(GBPT_ERR_OOM, "device allocation for rays failed");
      break;
    }
    cudaError_t e = cudaMemcpy(dr, rays, (size_t)n * 24, cudaMemcpyHostToDevice);
    if (!e) e = launch_trace_rays(s->dev, dr, n, max_dist, eps, cullback, dt, di, dw, du, dv, counts ? dn : nullptr,
                                  counts ? dq : nullptr, nullptr);
    if (!e) e = cudaMemcpy(t, dt, (size_t)n * 4, cudaMemcpyDeviceToHost);
    if (!e) e = cudaMemcpy(tri, di, (size_t)n * 4, cudaMemcpyDeviceToHost);
    if (!e) e = cudaMemcpy(w, dw, (size_t)n * 4, cudaMemcpyDeviceToHost);
    if (!e) e = cudaMemcpy(u, du, (size_t)n * 4, cudaMemcpyDeviceToHost);
    if (!e) e = cudaMemcpy(v, dv, (size_t)n * 4, cudaMemcpyDeviceToHost);
    if (!e && counts) e = cudaMemcpy(nodes, dn, (size_t)n * 4, cudaMemcpyDeviceToHost);
    if (!e && counts) e = cudaMemcpy(tris_tested, dq, (size_t)n * 4, cudaMemcpyDeviceToHost);
    if (e) st = fail(GBPT_ERR_CUDA, std::string("trace_rays: ") + cudaGetErrorString(e));
  } while (0);
  cleanup();
  return st;
}

gbpt_status gbpt_renderer_create(uint32_t width, uint32_t height, int32_t mode, const gbpt_params* params,
                                 gbpt_renderer** out) {
  if (!out) return fail(GBPT_ERR_INVALID_ARG, "out is NULL");
  *out = nullptr;
  if (width == 0 || height == 0 || (uint64_t)width * height > (1ull << 26))
    return fail(GBPT_ERR_INVALID_ARG, "image size must be 1..2^26 pixels");
  if (mode < GBPT_MODE_BDPT_SC || mode > GBPT_MODE_PT_SC)
    return fail(GBPT_ERR_INVALID_ARG, "unknown renderer mode");
  gbpt_params p;
  if (params) {
    gbpt_status st = check_params(params);
    if (st != GBPT_OK) return st;
    p = *params;
  } else {
    gbpt_params_default(&p);
  }
  gbpt_renderer* r = new (std::nothrow) gbpt_renderer();
  if (!r) return fail(GBPT_ERR_OOM, "host allocation failed");
  r->W = width;
  r->H = height;
  r->mode = mode;
  r->p = p;
  int prLow = 0, prHigh = 0;
  cudaDeviceGetStreamPriorityRange(&prLow, &prHigh);
  cudaError_t e = cudaStreamCreateWithFlags(&r->st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&r->stLight, cudaStreamNonBlocking, prLow);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&r->evMain, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&r->evLight[0], cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&r->evLight[1], cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&r->evFork, cudaEventDisableTiming);
  // band b's stream has the b-th highest priority: the first band takes the
  // SMs whenever it has work and the others fill what its walks leave idle,
  // so the bands run out of phase
  for (uint32_t b = 0; b < kMaxBands && e == cudaSuccess; b++) {
    e = cudaEventCreateWithFlags(&r->evJoin[b], cudaEventDisableTiming);
    const int pr = std::min(prHigh + (int)b, prLow);
    if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&r->stBand[b], cudaStreamNonBlocking, pr);
  }
  if (e != cudaSuccess) {
    delete r;
    return fail(GBPT_ERR_CUDA, std::string("cudaStreamCreate: ") + cudaGetErrorString(e));
  }
  *out = r;
  return GBPT_OK;
}

gbpt_status gbpt_renderer_destroy(gbpt_renderer* r) {
  delete r;
  return GBPT_OK;
}

gbpt_status gbpt_set_mode(gbpt_renderer* r, int32_t mode) {
  if (!r) return fail(GBPT_ERR_INVALID_ARG, "renderer is NULL");
  if (mode < GBPT_MODE_BDPT_SC || mode > GBPT_MODE_PT_SC) return fail(GBPT_ERR_INVALID_ARG, "unknown renderer mode");
  if (mode != r->mode) {
    r->mode = mode;
    r->started = false;  // RTRenderer::SetRendererMode starts the new renderer from scratch
  }
  return GBPT_OK;
}

gbpt_status gbpt_set_params(gbpt_renderer* r, const gbpt_params* params) {
  if (!r) return fail(GBPT_ERR_INVALID_ARG, "renderer is NULL");
  gbpt_status st = check_params(params);
  if (st != GBPT_OK) return st;
  bool realloc = params->light_paths * (1 + params->light_depth_max) > r->rb.cacheCap;
  if (realloc && r->alloc) {
    cudaStreamSynchronize(r->st);
    r->free_dev();
  }
  r->p = *params;
  r->started = false;
  return GBPT_OK;
}

gbpt_status gbpt_get_params(const gbpt_renderer* r, gbpt_params* params) {
  if (!r || !params) return fail(GBPT_ERR_INVALID_ARG, "NULL argument");
  *params = r->p;
  return GBPT_OK;
}

gbpt_status gbpt_render(gbpt_renderer* r, gbpt_scene* s, const gbpt_camera* cam, float* out_rgb,
                        int32_t out_is_device, gbpt_stats* stats) {
  return render_impl(r, s, cam, 1, out_rgb, out_is_device, stats);
}

gbpt_status gbpt_render_frames(gbpt_renderer* r, gbpt_scene* s, const gbpt_camera* cam, uint32_t frames,
                               gbpt_stats* stats) {
  return render_impl(r, s, cam, frames, nullptr, 0, stats);
}

const float* gbpt_result(gbpt_renderer* r) {
  if (!r || !r->alloc) return nullptr;
  // the image gbpt_render copies out (the mode's current view), as the reference's GetResult returns
  if (cudaStreamSynchronize(r->st) != cudaSuccess ||
      cudaMemcpy(r->hostResult, output_view(r), r->hostResultN * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
    return nullptr;
  return r->hostResult;
}

gbpt_status gbpt_host_register(void* p, size_t bytes) {
  if (!p || bytes == 0) return fail(GBPT_ERR_INVALID_ARG, "NULL or empty host range");
  CK(cudaHostRegister(p, bytes, cudaHostRegisterDefault));
  return GBPT_OK;
}

gbpt_status gbpt_host_unregister(void* p) {
  if (!p) return fail(GBPT_ERR_INVALID_ARG, "NULL host pointer");
  CK(cudaHostUnregister(p));
  return GBPT_OK;
}

gbpt_status gbpt_read_buffer(gbpt_renderer* r, int32_t which, void* dst, size_t bytes, int32_t dst_is_device) {
  if (!r || !dst) return fail(GBPT_ERR_INVALID_ARG, "NULL argument");
  if (!r->alloc) return fail(GBPT_ERR_STATE, "renderer has not rendered yet");
  const size_t np = (size_t)r->W * r->H;
  const void* src = nullptr;
  size_t need = np * 12;
  switch (which) {
    case 0: src = r->result; break;
    case 1: src = r->gpos; break;
    case 2: src = r->gnorm; break;
    case 3: src = r->gdiff; break;
    case 4: src = r->mode == GBPT_MODE_BDPT_SC_BILAT ? r->bilatOut : r->ab.filtered; break;
    case 5: src = r->ab.err; need = np * 4; break;
    case 6: src = r->sampleN; need = np * 4; break;
    case 8: src = r->direct; break;
    case 9: src = r->gemis; break;
    case 10: src = r->pot; need = np * 4; break;
    case 11: src = r->rb.m2; break;
    case 12: src = r->rb.hist; need = (size_t)((r->W + 7) / 8) * ((r->H + 7) / 8) * 32; break;
    case 7: {  // light-vertex cache in the 21-float layout of the reference's LightVertex
      DevCounters c{};
      gbpt_status st = read_ctr(r, &c);
      if (st != GBPT_OK) return st;
      const uint32_t cs = c.cacheSize[r->lastSel];
      need = (size_t)cs * 21 * 4;
      if (bytes < need) return fail(GBPT_ERR_INVALID_ARG, "destination too small");
      std::vector<float4> raw((size_t)cs * 6);
      if (cs) CK(cudaMemcpy(raw.data(), r->rb.cache[r->lastSel], raw.size() * 16, cudaMemcpyDeviceToHost));
      std::vector<float> o((size_t)cs * 21);
      for (uint32_t i = 0; i < cs; i++) {
        const float4* q = &raw[(size_t)i * 6];
        float* d = &o[(size_t)i * 21];
        const float4* fields[6] = {&q[0], &q[1], &q[2], &q[3], &q[4], &q[5]};
        for (int f = 0; f < 6; f++) {
          d[f * 3] = fields[f]->x;
          d[f * 3 + 1] = fields[f]->y;
          d[f * 3 + 2] = fields[f]->z;
        }
        d[18] = q[0].w;  // specular
        d[19] = q[1].w;  // metallic
        d[20] = q[2].w;  // roughness
      }
      CK(cudaMemcpy(dst, o.data(), need, dst_is_device ? cudaMemcpyHostToDevice : cudaMemcpyHostToHost));
      return GBPT_OK;
    }
    default: return fail(GBPT_ERR_INVALID_ARG, "unknown buffer id");
  }
  if (bytes < need) return fail(GBPT_ERR_INVALID_ARG, "destination too small");
  CK(cudaStreamSynchronize(r->st));
  CK(cudaMemcpy(dst, src, need, dst_is_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost));
  return GBPT_OK;
}

gbpt_status gbpt_renderer_rmse(gbpt_renderer* r, const float* converged, int32_t converged_is_device, double* out) {
  if (!r || !converged || !out) return fail(GBPT_ERR_INVALID_ARG, "NULL argument");
  if (!r->alloc) return fail(GBPT_ERR_STATE, "renderer has not rendered yet");
  const size_t n = (size_t)r->W * r->H * 3;
  if (converged_is_device) return rmse_device(output_view(r), converged, n, out, r->st);
  float* d = nullptr;
  CK(dalloc(&d, n));
  cudaError_t e = cudaMemcpyAsync(d, converged, n * 4, cudaMemcpyHostToDevice, r->st);
  gbpt_status st = e == cudaSuccess ? rmse_device(output_view(r), d, n, out, r->st)
                                    : fail(GBPT_ERR_CUDA, std::string("cudaMemcpyAsync: ") + cudaGetErrorString(e));
  cudaStreamSynchronize(r->st);
  dfree(d);
  return st;
}

gbpt_status gbpt_renderer_set_stream(gbpt_renderer* r, void* stream) {
  if (!r) return fail(GBPT_ERR_INVALID_ARG, "renderer is NULL");
  CK(cudaStreamSynchronize(r->st));
  if (!r->ownSt) r->ownSt = r->st;
  r->st = stream ? (cudaStream_t)stream : r->ownSt;
  r->userStream = stream != nullptr;
  return GBPT_OK;
}

gbpt_status gbpt_renderer_set_window(gbpt_renderer* r, uint32_t x0, uint32_t y0, uint32_t full_w, uint32_t full_h) {
  if (!r) return fail(GBPT_ERR_INVALID_ARG, "renderer is NULL");
  if (full_w == 0 || full_h == 0 || (uint64_t)full_w * full_h > (1ull << 32) - 1 || x0 > full_w ||
      y0 > full_h || r->W > full_w - x0 || r->H > full_h - y0)
    return fail(GBPT_ERR_INVALID_ARG, "the renderer's " + std::to_string(r->W) + "x" + std::to_string(r->H) +
                                          " window at (" + std::to_string(x0) + ", " + std::to_string(y0) +
                                          ") does not fit a " + std::to_string(full_w) + "x" +
                                          std::to_string(full_h) + " image");
  r->winX0 = x0;
  r->winY0 = y0;
  r->fullW = full_w;
  r->fullH = full_h;
  r->started = false;  // progressive accumulation restarts
  return GBPT_OK;
}

gbpt_status gbpt_renderer_set_graphs(gbpt_renderer* r, int32_t on) {
  if (!r) return fail(GBPT_ERR_INVALID_ARG, "renderer is NULL");
  r->graphs = on != 0;
  return GBPT_OK;
}

gbpt_status gbpt_renderer_set_mlp(gbpt_renderer* r, gbpt_mlp* mlp, int32_t collect) {
  if (!r) return fail(GBPT_ERR_INVALID_ARG, "renderer is NULL");
  r->mlp = mlp;
  r->collect = collect != 0;
  return GBPT_OK;
}

gbpt_status gbpt_renderer_features(gbpt_renderer* r, float* out, uint32_t capacity, int32_t out_is_device,
                                   uint32_t* n_tiles) {
  if (!r) return fail(GBPT_ERR_INVALID_ARG, "renderer is NULL");
  const uint32_t tilesX = (r->W + 7) / 8, nTiles = tilesX * ((r->H + 7) / 8);
  if (n_tiles) *n_tiles = nTiles;
  if (!out) return GBPT_OK;
  if (capacity < nTiles) return fail(GBPT_ERR_INVALID_ARG, "feature buffer too small");
  if (!r->alloc || !r->started) return fail(GBPT_ERR_STATE, "renderer has not rendered yet");
  if (r->mode != GBPT_MODE_BDPT_SC_ADAP_BILAT && r->mode != GBPT_MODE_BDPT_SC_ADAP_BILAT_BINARY)
    return fail(GBPT_ERR_STATE, "features need an adaptive mode (first-hit planes)");
  cudaStream_t st = r->st;
  FrameArgs a{};
  a.width = r->W;
  a.height = r->H;
  a.tilesX = tilesX;
  a.moments = 1;
  for (int k = 0; k < 3; k++) a.camPos[k] = r->camBasis[k];
  const float delta = r->p.filter_sigma_spatial > 0.f ? r->p.filter_sigma_spatial : r->p.filter_color_eud;
  gbpt_status ge = ensure_gauss(r, delta, r->p.filter_radius, st);
  if (ge != GBPT_OK) return ge;
  CK(launch_bilateral(r->result, r->gpos, r->gnorm, r->p.filter_diffuse ? r->gdiff : nullptr, r->W, r->H,
                      r->p.filter_color_eud, r->p.filter_pos_eud, r->p.filter_norm_eud, r->p.filter_diff_eud,
                      r->p.filter_radius, r->gauss, r->ab.filtered, st));
  CK(launch_adapt_error(a, r->ab, r->result, r->sampleN, r->p.desired_n, st));
  CK(launch_tile_features(a, r->rb, r->ab, r->result, r->sampleN, r->gpos, r->gnorm, r->gdiff, st));
  CK(cudaMemcpyAsync(out, r->ab.feat, (size_t)nTiles * kFeatures * 4,
                     out_is_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  return GBPT_OK;
}

// ---- checkpoint / resume ---------------------------------------------------
// Layout: CkHeader, then the device planes of ck_planes() in order.  Every
// random number of a frame follows from (seed, request id, frame, pixel,
// sample), so the accumulators, the sample counts and the frame counter are
// the whole state: a restored renderer continues the interrupted sequence to
// the bit (the light cache of the current group is made again on the next
// frame).
namespace {

struct CkHeader {
  char magic[8];  // "GBPTCKP1"
  uint32_t version, W, H;
  int32_t mode;
  uint32_t frame, started, bilatIs2, triN, nodeN;
  float camBasis[9];
  float debugMode;
  gbpt_params p;
};

struct CkPlane {
  void* dev;
  size_t bytes;
};

std::vector<CkPlane> ck_planes(gbpt_renderer* r) {
  const size_t np = (size_t)r->W * r->H;
  const size_t nTiles = (size_t)((r->W + 7) / 8) * ((r->H + 7) / 8);
  return {{r->result, np * 12},     {r->sampleN, np * 4},   {r->gpos, np * 12},        {r->gnorm, np * 12},
          {r->gdiff, np * 12},      {r->gemis, np * 12},    {r->direct, np * 12},      {r->pot, np * 4},
          {r->filtered2, np * 12},  {r->probView, np * 12}, {r->ab.filtered, np * 12}, {r->rb.m2, np * 12},
          {r->rb.hist, nTiles * 32}};
}

size_t ck_bytes(gbpt_renderer* r) {
  size_t n = sizeof(CkHeader);
  const size_t np = (size_t)r->W * r->H;
  const size_t nTiles = (size_t)((r->W + 7) / 8) * ((r->H + 7) / 8);
  n += np * (12 * 11 + 4 * 2) + nTiles * 32;
  return n;
}

}  // namespace

gbpt_status gbpt_renderer_checkpoint_size(gbpt_renderer* r, size_t* bytes) {
  if (!r || !bytes) return fail(GBPT_ERR_INVALID_ARG, "NULL argument");
  *bytes = ck_bytes(r);
  return GBPT_OK;
}

gbpt_status gbpt_renderer_checkpoint(gbpt_renderer* r, void* buf, size_t bytes) {
  if (!r || !buf) return fail(GBPT_ERR_INVALID_ARG, "NULL argument");
  if (bytes < ck_bytes(r)) return fail(GBPT_ERR_INVALID_ARG, "checkpoint buffer too small");
  if (!r->alloc || !r->started) return fail(GBPT_ERR_STATE, "renderer has not rendered yet");
  CkHeader h{};
  std::memcpy(h.magic, "GBPTCKP1", 8);
  h.version = 1;
  h.W = r->W;
  h.H = r->H;
  h.mode = r->mode;
  h.frame = r->frame;
  h.started = r->started ? 1u : 0u;
  h.bilatIs2 = r->bilatOut == r->filtered2 ? 1u : 0u;
  h.triN = r->lastTriN;
  h.nodeN = r->lastNodeN;
  std::memcpy(h.camBasis, r->camBasis, sizeof(h.camBasis));
  h.debugMode = r->debugMode;
  h.p = r->p;
  char* out = static_cast<char*>(buf);
  std::memcpy(out, &h, sizeof(h));
  size_t at = sizeof(h);
  for (const CkPlane& c : ck_planes(r)) {
    CK(cudaMemcpyAsync(out + at, c.dev, c.bytes, cudaMemcpyDeviceToHost, r->st));
    at += c.bytes;
  }
  CK(cudaStreamSynchronize(r->st));
  return GBPT_OK;
}

gbpt_status gbpt_renderer_restore(gbpt_renderer* r, const void* buf, size_t bytes) {
  if (!r || !buf) return fail(GBPT_ERR_INVALID_ARG, "NULL argument");
  if (bytes < sizeof(CkHeader)) return fail(GBPT_ERR_INVALID_ARG, "checkpoint truncated");
  CkHeader h;
  std::memcpy(&h, buf, sizeof(h));
  if (std::memcmp(h.magic, "GBPTCKP1", 8) != 0 || h.version != 1)
    return fail(GBPT_ERR_INVALID_ARG, "not a gbpt checkpoint");
  if (h.W != r->W || h.H != r->H) return fail(GBPT_ERR_INVALID_ARG, "checkpoint image size differs");
  if (bytes < ck_bytes(r)) return fail(GBPT_ERR_INVALID_ARG, "checkpoint truncated");
  gbpt_status st = gbpt_set_params(r, &h.p);
  if (st == GBPT_OK) st = gbpt_set_mode(r, h.mode);
  if (st != GBPT_OK) return st;
  st = ensure_alloc(r);
  if (st != GBPT_OK) return st;
  if (r->stLight) CK(cudaStreamSynchronize(r->stLight));  // no light pass still writes a cache
  const char* in = static_cast<const char*>(buf);
  size_t at = sizeof(h);
  for (const CkPlane& c : ck_planes(r)) {
    CK(cudaMemcpyAsync(c.dev, in + at, c.bytes, cudaMemcpyHostToDevice, r->st));
    at += c.bytes;
  }
  CK(cudaStreamSynchronize(r->st));
  r->frame = h.frame;
  r->started = h.started != 0;
  std::memcpy(r->camBasis, h.camBasis, sizeof(h.camBasis));
  r->debugMode = h.debugMode;
  r->bilatOut = h.bilatIs2 ? r->filtered2 : r->ab.filtered;
  r->lastTraced = true;
  r->epoch++;  // the light caches are made again
  r->lightPending[0] = r->lightPending[1] = false;
  r->resumeScene = true;
  r->resumeTriN = h.triN;
  r->resumeNodeN = h.nodeN;
  return GBPT_OK;
}

gbpt_status gbpt_test_fail_allocations(int64_t after) {
  g_failAfter.store(after < 0 ? -1 : after);
  return GBPT_OK;
}

gbpt_status gbpt_selftest_wait_timeout(double* elapsed_ms) {
  uint32_t* coop = nullptr;
  DevCounters* ctr = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  gbpt_status st = GBPT_OK;
  uint32_t flags = 0;
  float ms = 0.f;
  cudaError_t e = dalloc(&coop, 4);
  if (!e) e = dalloc(&ctr, 1);
  if (!e) e = cudaMemset(coop, 0, 16);
  if (!e) e = cudaMemset(ctr, 0, sizeof(DevCounters));
  if (!e) e = cudaEventCreate(&e0);
  if (!e) e = cudaEventCreate(&e1);
  if (!e) e = cudaEventRecord(e0, nullptr);
  if (!e) e = launch_barrier_selftest(coop, ctr, 2, nullptr);
  if (!e) e = cudaEventRecord(e1, nullptr);
  if (!e) e = cudaEventSynchronize(e1);
  if (!e) e = cudaEventElapsedTime(&ms, e0, e1);
  if (!e) e = cudaMemcpy(&flags, &ctr->errFlags, 4, cudaMemcpyDeviceToHost);
  if (e) st = fail(GBPT_ERR_CUDA, std::string("wait self-test: ") + cudaGetErrorString(e));
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  dfree(coop);
  dfree(ctr);
  if (st != GBPT_OK) return st;
  if (elapsed_ms) *elapsed_ms = ms;
  if (flags & 4u) return fail(GBPT_ERR_TIMEOUT, "grid barrier wait ran out (self-test)");
  return GBPT_OK;
}

gbpt_status gbpt_reset(gbpt_renderer* r) {
  if (!r) return fail(GBPT_ERR_INVALID_ARG, "renderer is NULL");
  r->started = false;
  return GBPT_OK;
}

gbpt_status gbpt_clean(gbpt_renderer* r) {
  if (!r) return fail(GBPT_ERR_INVALID_ARG, "renderer is NULL");
  cudaStreamSynchronize(r->st);
  r->free_dev();
  r->started = false;
  return GBPT_OK;
}

gbpt_status gbpt_set_counting(gbpt_renderer* r, int32_t on) {
  if (!r) return fail(GBPT_ERR_INVALID_ARG, "renderer is NULL");
  r->counting = on != 0;
  return GBPT_OK;
}

gbpt_status gbpt_attr_count(const gbpt_renderer* r, uint32_t* n) {
  if (!r || !n) return fail(GBPT_ERR_INVALID_ARG, "NULL argument");
  attr_table(r, n);
  return GBPT_OK;
}

gbpt_status gbpt_attr_name(const gbpt_renderer* r, uint32_t index, char* name, size_t cap) {
  if (!r || !name || cap == 0) return fail(GBPT_ERR_INVALID_ARG, "NULL argument");
  uint32_t n = 0;
  const AttrDef* t = attr_table(r, &n);
  if (index >= n) return fail(GBPT_ERR_INVALID_ARG, "attribute index out of range");
  std::strncpy(name, t[index].name, cap - 1);
  name[cap - 1] = 0;
  return GBPT_OK;
}

gbpt_status gbpt_attr_get(const gbpt_renderer* r, const char* name, float* value) {
  if (!r || !name || !value) return fail(GBPT_ERR_INVALID_ARG, "NULL argument");
  uint32_t n = 0;
  const AttrDef* t = attr_table(r, &n);
  for (uint32_t i = 0; i < n; i++)
    if (std::strcmp(name, t[i].name) == 0) {
      const char* base = (const char*)&r->p;
      if (t[i].kind == 2) {
        *value = r->debugMode;
      } else if (t[i].kind == 0) {
        std::memcpy(value, base + t[i].off, 4);
      } else {
        uint32_t u;
        std::memcpy(&u, base + t[i].off, 4);
        *value = (float)u;
      }
      return GBPT_OK;
    }
  return fail(GBPT_ERR_INVALID_ARG, std::string("unknown attribute '") + name + "'");
}

gbpt_status gbpt_attr_set(gbpt_renderer* r, const char* name, float value) {
  if (!r || !name) return fail(GBPT_ERR_INVALID_ARG, "NULL argument");
  uint32_t n = 0;
  const AttrDef* t = attr_table(r, &n);
  for (uint32_t i = 0; i < n; i++)
    if (std::strcmp(name, t[i].name) == 0) {
      if (t[i].kind == 2) {
        if (r->mode == GBPT_MODE_BDPT_SC_BILAT) {
          // None, Traced, Prob, Prob With Limit, Direct, Position, Normal, Non-Filter (:27)
          if (!(value >= 0.f && value <= 7.f) || value != (float)(int)value)
            return fail(GBPT_ERR_INVALID_ARG, "Debug Mode is 0..7 in BDPTSC Bilaterial");
        } else if (value != 0.f && value != 4.f) {
          return fail(GBPT_ERR_INVALID_ARG, "Debug Mode supports 0 (None) and 4 (Filtered)");
        }
        r->debugMode = value;
        return GBPT_OK;
      }
      gbpt_params p = r->p;
      char* base = (char*)&p;
      if (t[i].kind == 0) {
        std::memcpy(base + t[i].off, &value, 4);
      } else {
        if (!(value >= 0.f) || value > 4294967295.f) return fail(GBPT_ERR_INVALID_ARG, "value out of range");
        uint32_t u = (uint32_t)value;
        std::memcpy(base + t[i].off, &u, 4);
      }
      return gbpt_set_params(r, &p);
    }
  return fail(GBPT_ERR_INVALID_ARG, std::string("unknown attribute '") + name + "'");
}

gbpt_status gbpt_gaussian_table(float delta, uint32_t radius, float* g) {
  if (!g) return fail(GBPT_ERR_INVALID_ARG, "g is NULL");
  if (radius > 31) return fail(GBPT_ERR_INVALID_ARG, "radius must be <= 31");
  gaussian_table_host(delta, radius, g);
  return GBPT_OK;
}

gbpt_status gbpt_bilateral(const float* color, const float* pos, const float* norm, const float* emit,
                           uint32_t width, uint32_t height, float color_eud, float pos_eud, float norm_eud,
                           float emit_eud, uint32_t radius, const float* g, float* out, int32_t is_device) {
  if (!color || !pos || !norm || !g || !out) return fail(GBPT_ERR_INVALID_ARG, "NULL argument");
  if (radius > 31 || width == 0 || height == 0) return fail(GBPT_ERR_INVALID_ARG, "bad size or radius");
  const size_t n = (size_t)width * height * 3;
  float* dg = nullptr;
  CK(dalloc(&dg, 2 * radius + 1));
  CK(cudaMemcpy(dg, g, (2 * radius + 1) * 4, cudaMemcpyHostToDevice));
  gbpt_status st = GBPT_OK;
  if (is_device) {
    cudaError_t e = launch_bilateral(color, pos, norm, emit, width, height, color_eud, pos_eud, norm_eud, emit_eud,
                                     radius, dg, out, nullptr);
    if (!e) e = cudaDeviceSynchronize();
    if (e) st = fail(GBPT_ERR_CUDA, std::string("bilateral: ") + cudaGetErrorString(e));
  } else {
    float* d[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    const float* src[4] = {color, pos, norm, emit};
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < 5 && !e; k++) {
      if (k < 4 && !src[k]) continue;
      e = dalloc(&d[k], n);
      if (!e && k < 4) e = cudaMemcpy(d[k], src[k], n * 4, cudaMemcpyHostToDevice);
    }
    if (!e)
      e = launch_bilateral(d[0], d[1], d[2], d[3], width, height, color_eud, pos_eud, norm_eud, emit_eud, radius, dg,
                           d[4], nullptr);
    if (!e) e = cudaMemcpy(out, d[4], n * 4, cudaMemcpyDeviceToHost);
    for (int k = 0; k < 5; k++) dfree(d[k]);
    if (e) st = fail(GBPT_ERR_CUDA, std::string("bilateral: ") + cudaGetErrorString(e));
  }
  dfree(dg);
  return st;
}

gbpt_status gbpt_fmath(int32_t which, const float* x, uint32_t n, float* out) {
  if (!x || !out || which < 0 || which > 5) return fail(GBPT_ERR_INVALID_ARG, "bad argument");
  if (n == 0) return GBPT_OK;
  float *dx = nullptr, *dy = nullptr;
  CK(dalloc(&dx, n));
  CK(dalloc(&dy, n));
  cudaError_t e = cudaMemcpy(dx, x, (size_t)n * 4, cudaMemcpyHostToDevice);
  if (!e) e = launch_fmath(which, dx, n, dy, nullptr);
  if (!e) e = cudaMemcpy(out, dy, (size_t)n * 4, cudaMemcpyDeviceToHost);
  dfree(dx);
  dfree(dy);
  if (e) return fail(GBPT_ERR_CUDA, std::string("fmath: ") + cudaGetErrorString(e));
  return GBPT_OK;
}

gbpt_status gbpt_philox(const uint32_t* ctr, uint32_t n, uint32_t k0, uint32_t k1, uint32_t* out) {
  if (!ctr || !out) return fail(GBPT_ERR_INVALID_ARG, "bad argument");
  if (n == 0) return GBPT_OK;
  uint32_t *dc = nullptr, *dout = nullptr;
  CK(dalloc(&dc, (size_t)n * 4));
  CK(dalloc(&dout, (size_t)n * 4));
  cudaError_t e = cudaMemcpy(dc, ctr, (size_t)n * 16, cudaMemcpyHostToDevice);
  if (!e) e = launch_philox(dc, n, k0, k1, dout, nullptr);
  if (!e) e = cudaMemcpy(out, dout, (size_t)n * 16, cudaMemcpyDeviceToHost);
  dfree(dc);
  dfree(dout);
  if (e) return fail(GBPT_ERR_CUDA, std::string("philox: ") + cudaGetErrorString(e));
  return GBPT_OK;
}

}  // extern "C"
