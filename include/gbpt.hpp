// C++ shim over the gbpt C ABI with the shape of CudaPT's RTScene /
// RTRenderer (include/raytracer.h:228-323), for host code that was written
// against those classes.  Header-only; link libgbpt.so.
//
//   gbpt::RTScene scene;                       // RTScene
//   scene.m_pVertices = ...; scene.m_pTriangles = ...; scene.m_pMaterials = ...;
//   scene.UpdateBVH();                         // AddModel's BVH build (src/raytracer.cpp:264-281)
//   gbpt::RTRenderer r;
//   r.Init(w, h);                              // RTRenderer::Init
//   r.SetRendererMode(GBPT_MODE_BDPT_SC);      // RTRenderer::SetRendererMode
//   r.Render(camPos, camDir, camUp, fov, scene);  // one progressive pass
//   const float* rgb = r.GetResult();          // RTRenderer::GetResult
//
// Errors throw gbpt::Error carrying the gbpt_status and the library's message
// (the reference printed and continued, include/cudahelper.h:65-75).
#ifndef GBPT_HPP
#define GBPT_HPP

#include <stdexcept>
#include <string>
#include <vector>

#include "gbpt.h"

namespace gbpt {

struct Error : std::runtime_error {
  gbpt_status status;
  Error(gbpt_status s, const std::string& what) : std::runtime_error(what), status(s) {}
};

inline void check(gbpt_status s) {
  if (s != GBPT_OK) {
    const char* m = gbpt_last_error_string();
    throw Error(s, m ? m : "gbpt error");
  }
}

struct Vec3 {
  float x, y, z;
};

class RTScene {
 public:
  std::vector<gbpt_vertex> m_pVertices;
  std::vector<gbpt_triangle> m_pTriangles;
  std::vector<gbpt_material> m_pMaterials;

  RTScene() = default;
  RTScene(const RTScene&) = delete;
  RTScene& operator=(const RTScene&) = delete;
  ~RTScene() { release(); }

  // Uploads the vectors and builds the BVH (the reference's AddModel + CreateBVH).
  void UpdateBVH(uint32_t maxDepth = 32) {
    release();
    check(gbpt_scene_create(m_pVertices.data(), (uint32_t)m_pVertices.size(), m_pTriangles.data(),
                            (uint32_t)m_pTriangles.size(), m_pMaterials.data(), (uint32_t)m_pMaterials.size(),
                            &scene_));
    check(gbpt_scene_build_bvh(scene_, maxDepth, 0, nullptr));
  }
  // GetIsCudaMaterialDirty -> updateAllSceneMaterialsCudaMem (src/cudaRTCommon.cu:580-599)
  void UpdateMaterials() {
    check(gbpt_scene_update_materials(scene_, m_pMaterials.data(), (uint32_t)m_pMaterials.size()));
  }
  gbpt_scene* handle() const { return scene_; }

 private:
  void release() {
    if (scene_) gbpt_scene_destroy(scene_);
    scene_ = nullptr;
  }
  gbpt_scene* scene_ = nullptr;
};

class RTRenderer {
 public:
  RTRenderer() { check(gbpt_params_default(&params_)); }
  RTRenderer(const RTRenderer&) = delete;
  RTRenderer& operator=(const RTRenderer&) = delete;
  ~RTRenderer() { release(); }

  bool Init(uint32_t w, uint32_t h) {
    release();
    w_ = w;
    h_ = h;
    check(gbpt_renderer_create(w, h, mode_, &params_, &r_));
    return true;
  }
  void SetRendererMode(int32_t mode) {
    mode_ = mode;
    if (r_) check(gbpt_set_mode(r_, mode));
  }
  int32_t GetRendererMode() const { return mode_; }
  // One progressive pass; the result stays available from GetResult().
  bool Render(Vec3 camPos, Vec3 camDir, Vec3 camUp, float fov, RTScene& scene) {
    if (!r_) return false;
    gbpt_camera cam = {{camPos.x, camPos.y, camPos.z}, {camDir.x, camDir.y, camDir.z}, {camUp.x, camUp.y, camUp.z},
                       fov};
    check(gbpt_render(r_, scene.handle(), &cam, nullptr, 0, &stats_));
    return true;
  }
  const float* GetResult() { return r_ ? gbpt_result(r_) : nullptr; }
  const gbpt_stats& LastStats() const { return stats_; }

  // GetAttribsN / GetAttribute (src/raytracer.cpp:19-31), by name
  uint32_t GetAttribsN() const {
    uint32_t n = 0;
    if (r_) check(gbpt_attr_count(r_, &n));
    return n;
  }
  std::string GetAttribName(uint32_t i) const {
    char buf[64] = {0};
    check(gbpt_attr_name(r_, i, buf, sizeof(buf)));
    return buf;
  }
  float GetAttrib(const std::string& name) const {
    float v = 0.f;
    check(gbpt_attr_get(r_, name.c_str(), &v));
    return v;
  }
  void SetAttrib(const std::string& name, float v) { check(gbpt_attr_set(r_, name.c_str(), v)); }
  void CleanMem() {
    if (r_) check(gbpt_clean(r_));
  }
  gbpt_renderer* handle() const { return r_; }

 private:
  void release() {
    if (r_) gbpt_renderer_destroy(r_);
    r_ = nullptr;
  }
  gbpt_renderer* r_ = nullptr;
  gbpt_params params_{};
  gbpt_stats stats_{};
  int32_t mode_ = GBPT_MODE_BDPT_SC;
  uint32_t w_ = 0, h_ = 0;
};

}  // namespace gbpt

#endif  // GBPT_HPP
