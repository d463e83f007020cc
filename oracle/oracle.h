// TEST INFRASTRUCTURE ONLY -- CPU oracle for the GB300 BDPT library.
//
// A plain C++ restatement of CudaPT's BDPT hot path (see each .cpp for the
// reference file:line it follows).  It is the checker for the CUDA kernels:
// tests/, the smoke check and the CPU baseline of bench.py load it; the
// shipped library never does.
#pragma once
#include <cstdint>
#include <vector>

#include "texture_ref.h"

namespace orc {

struct BuildStats {
  uint32_t empty_children = 0;  // splits that left one child without triangles
};

// CompactBVH (include/bvhhelper.h:45-54) plus the triangle order CreateBVH
// returns.  bounds: 6 floats per node (min xyz, max xyz); offOrTSTN: 2 words
// per node ({right offset, 0} for an inner node, {triStart, triN} for a leaf).
struct BVH {
  uint32_t nodeN = 0;
  std::vector<float> bounds;
  std::vector<uint32_t> offOrTSTN;
  std::vector<uint32_t> order;
  BuildStats stats;
};

bool build_bvh(const float* pos, uint32_t nv, const uint32_t* tri, uint32_t nt, uint32_t maxDepth, BVH* out);

// Reference data layouts (include/raytracer.h:58-101)
struct RTVertex {  // 44 bytes
  float pos[3], norm[3], tan[3], tex[2];
};
struct RTTriangle {  // 16 bytes
  uint32_t v0, v1, v2, mat;
};
struct RTMaterial {  // 80 bytes
  float diffuse[3], emissive[3];
  int32_t diffuseTexId, normalTexId, emissiveTexId, matType;
  float transparency, subsurface, specular, metallic, roughness, anisotropic, sheen, sheenTint, clearcoat,
      clearcoatGloss;
};
static_assert(sizeof(RTVertex) == 44, "RTVertex");
static_assert(sizeof(RTTriangle) == 16, "RTTriangle");
static_assert(sizeof(RTMaterial) == 80, "RTMaterial");

// A scene after RTScene::AddModel (src/raytracer.cpp:238-282): triangles in
// BVH order, intersect data p0 / p1-p0 / p2-p0 (src/cudaRTCommon.cu:503-513),
// and the emissive-triangle list (src/cudaRTBDPTStream.cu:57-77).
struct Scene {
  std::vector<RTVertex> verts;
  std::vector<RTTriangle> tris;  // reordered
  std::vector<RTMaterial> mats;
  BVH bvh;
  std::vector<float> isect;  // 9 floats per triangle: p0, e0, e1
  std::vector<uint32_t> lightTri;
  std::vector<Texture> textures;  // RTScene::m_pTextures
};

bool make_scene(const RTVertex* v, uint32_t nv, const RTTriangle* t, uint32_t nt, const RTMaterial* m, uint32_t nm,
                Scene* s);
void refresh_lights(Scene* s);

struct Hit {
  float dist;
  int32_t triId;
  float w, u, v;
};
struct TraceCount {
  uint32_t nodes = 0, tris = 0;
};

// src/cudaRTCommon.cu:66-127 TracePrimitive
float intersect_aabb(const float o[3], const float d[3], const float mn[3], const float mx[3]);
float intersect_tri(const float o[3], const float d[3], const float p0[3], const float e0[3], const float e1[3],
                    float eps, bool cullback, float wuv[3]);
bool trace_primitive(const Scene& s, const float o[3], const float d[3], float maxDist, float eps, bool cullback,
                     Hit* hit, TraceCount* cnt);

}  // namespace orc
