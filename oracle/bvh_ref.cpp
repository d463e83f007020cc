// TEST INFRASTRUCTURE ONLY -- CPU oracle.  Restates the reference's host BVH
// builder and compactor, single threaded, operation for operation.
//
//   src/bvhhelper.cpp:33-39    AABBSurfaceArea
//   src/bvhhelper.cpp:41-53    InitialBVHLeafNode
//   src/bvhhelper.cpp:55-237   InitialBVHNode (binned SAH, 16 bins)
//   src/bvhhelper.cpp:239-283  CreateBVH
//   src/bvhhelper.cpp:285-313  InitialCompactBVH(OnNode)
//   src/raytracer.cpp:264-281  AddModel: triangle reorder + intersect data
//
// Host float semantics of the reference (MSVC x64, /fp:precise): every float
// operation is a single IEEE float operation; mixed float/double expressions
// (M_EPSILON, M_FLT_BIAS_EPSILON are double literals) are evaluated in double
// and rounded on assignment, as written below.
#include <cmath>
#include <cstdint>
#include <vector>

#include "oracle.h"

namespace orc {

namespace {

constexpr uint32_t kBins = 16;  // BVH_SAH_BIN_N, src/bvhhelper.cpp:9
constexpr double kEps = 1E-9;   // M_EPSILON
constexpr double kBias = 1E-4;  // M_FLT_BIAS_EPSILON

struct V3 {
  float e[3];
};
static inline V3 v3(float x, float y, float z) { return V3{{x, y, z}}; }
static inline V3 vmin3(V3 a, V3 b) {
  return v3(std::fmin(a.e[0], b.e[0]), std::fmin(a.e[1], b.e[1]), std::fmin(a.e[2], b.e[2]));
}
static inline V3 vmax3(V3 a, V3 b) {
  return v3(std::fmax(a.e[0], b.e[0]), std::fmax(a.e[1], b.e[1]), std::fmax(a.e[2], b.e[2]));
}
static inline float vlen(V3 a) {  // Vec3::length: sqrt of the float sum
  return std::sqrt(a.e[0] * a.e[0] + a.e[1] * a.e[1] + a.e[2] * a.e[2]);
}

struct Box {
  V3 mn, mx;
};
static inline Box empty_box() {
  const float inf = (float)1E20, minf = (float)-1E20;
  return Box{v3(inf, inf, inf), v3(minf, minf, minf)};
}
static inline Box merge(Box a, Box b) { return Box{vmin3(a.mn, b.mn), vmax3(a.mx, b.mx)}; }
static inline Box merge(Box a, V3 p) { return Box{vmin3(a.mn, p), vmax3(a.mx, p)}; }

// src/bvhhelper.cpp:33-39
static float surface_area(const Box& b) {
  V3 d = v3(b.mx.e[0] - b.mn.e[0], b.mx.e[1] - b.mn.e[1], b.mx.e[2] - b.mn.e[2]);
  if (d.e[0] < 0 || d.e[1] < 0 || d.e[2] < 0 || (double)vlen(d) < kEps) return 0;
  return d.e[0] * d.e[1] + d.e[0] * d.e[2] + d.e[1] * d.e[2];
}

struct BTri {
  V3 centroid;
  Box bound;
};

struct Node {
  Node* child[2] = {nullptr, nullptr};
  Box bound = empty_box();
  uint32_t triStart = 0, triN = 0, desN = 0;
  ~Node() {
    delete child[0];
    delete child[1];
  }
};

struct Bin {
  uint32_t triN = 0;
  Box cb = empty_box();
};

// src/bvhhelper.cpp:55-237
static void build_node(Node* node, const BTri* tris, uint32_t* order, uint32_t triStart, uint32_t triN,
                       uint32_t depthBudget, BuildStats* st) {
  if (triN <= 0) return;
  Box centroidBound = empty_box();
  for (uint32_t i = 0; i < triN; i++) {
    uint32_t ind = order[triStart + i];
    node->bound = merge(node->bound, tris[ind].bound);
    centroidBound = merge(centroidBound, tris[ind].centroid);
  }
  V3 dia = v3(centroidBound.mx.e[0] - centroidBound.mn.e[0], centroidBound.mx.e[1] - centroidBound.mn.e[1],
              centroidBound.mx.e[2] - centroidBound.mn.e[2]);
  if (dia.e[0] < 0 || dia.e[1] < 0 || dia.e[2] < 0) return;
  if (triN == 1 || depthBudget <= 1 || (double)vlen(dia) < kEps) {
    node->triStart = triStart;  // InitialBVHLeafNode, :41-53
    node->triN = triN;
    node->desN = 0;
    return;
  }
  uint32_t axis = 0;
  if (std::fabs(dia.e[1]) > std::fabs(dia.e[0])) axis = 1;
  if (std::fabs(dia.e[2]) > std::fabs(dia.e[1]) && std::fabs(dia.e[2]) > std::fabs(dia.e[0])) axis = 2;
  float L = std::fabs(dia.e[axis]);

  // :87-111 -- bin i takes centroids in [start_i, end_i); the last bin's end
  // is (double)max + 1e-4 rounded to float.
  Bin bins[kBins];
  for (uint32_t i = 0; i < kBins; i++) {
    float bs = centroidBound.mn.e[axis] + (float)i * L / (float)kBins;
    float be = centroidBound.mn.e[axis] + (float)(i + 1) * L / (float)kBins;
    if (i + 1 == kBins) be = (float)((double)centroidBound.mx.e[axis] + kBias);
    for (uint32_t j = 0; j < triN; j++) {
      uint32_t ind = order[triStart + j];
      float p = tris[ind].centroid.e[axis];
      if (p >= bs && p < be) {
        bins[i].triN++;
        bins[i].cb = merge(bins[i].cb, tris[ind].centroid);
      }
    }
  }

  // :120-164 -- two sweeps; the second one runs j = 16 .. 9 with an unsigned
  // step of -1 and writes binHeu[j-1].  Counts are converted to float.
  float nodeSA = surface_area(node->bound);
  float heu[kBins];
  for (int pass = 0; pass < 2; pass++) {
    uint32_t startBin = 0, endBin = kBins / 2, step = 1;
    if (pass == 1) {
      startBin = kBins;
      endBin = kBins / 2;
      step = (uint32_t)-1;
    }
    uint32_t mainN = 0;
    Box mainB = empty_box();
    for (uint32_t j = startBin; j != endBin; j += step) {
      if (j < kBins) {
        mainN += bins[j].triN;
        mainB = merge(mainB, bins[j].cb);
      }
      uint32_t opN = 0;
      Box opB = empty_box();
      for (uint32_t k = j + step; k < kBins; k += step) {
        opN += bins[k].triN;
        opB = merge(opB, bins[k].cb);
      }
      float h = 0.125f + ((float)mainN * surface_area(mainB) + (float)opN * surface_area(opB)) / nodeSA;
      if (pass == 0)
        heu[j] = h;
      else
        heu[j - 1] = h;
    }
  }
  // :173-182 -- the winning bin index is held in a float
  float minCost = (float)1E20;
  float minBin = kBins - 1;
  for (uint32_t i = 0; i < kBins; i++) {
    if (heu[i] < minCost) {
      minCost = heu[i];
      minBin = (float)i;
    }
  }
  if (minBin >= kBins) {
    node->triStart = triStart;
    node->triN = triN;
    return;
  }
  // :190-211 -- in-place partition around the split plane
  uint32_t mid;
  {
    float split = centroidBound.mn.e[axis] + (float)(minBin + 1) * L / (float)kBins;
    uint32_t left = triStart, right = triStart + triN - 1;
    while (left < right) {
      while (tris[order[left]].centroid.e[axis] <= split && left < right) left++;
      while (tris[order[right]].centroid.e[axis] > split && left < right) right--;
      if (left < right) {
        uint32_t t = order[left];
        order[left] = order[right];
        order[right] = t;
        left++;
        right--;
      }
    }
    if (tris[order[left]].centroid.e[axis] <= split)
      mid = left;
    else
      mid = left - 1;
  }
  Node* l = new Node();
  Node* r = new Node();
  node->child[0] = l;
  node->child[1] = r;
  uint32_t nl = mid - triStart + 1;  // unsigned: mid may be triStart-1
  build_node(l, tris, order, triStart, nl, depthBudget - 1, st);
  build_node(r, tris, order, mid + 1, triN - nl, depthBudget - 1, st);
  if (nl == 0 || triN - nl == 0) st->empty_children++;
  node->desN = 2 + l->desN + r->desN;
}

// src/bvhhelper.cpp:285-298
static uint32_t compact_node(const Node* node, float* bounds, uint32_t* oot, uint32_t cur) {
  for (int k = 0; k < 3; k++) {
    bounds[cur * 6 + k] = node->bound.mn.e[k];
    bounds[cur * 6 + 3 + k] = node->bound.mx.e[k];
  }
  if (!node->child[0] || !node->child[1]) {
    oot[cur * 2] = node->triStart;
    oot[cur * 2 + 1] = node->triN;
    return 1;
  }
  oot[cur * 2 + 1] = 0;
  uint32_t first = compact_node(node->child[0], bounds, oot, cur + 1);
  oot[cur * 2] = first + 1;
  return compact_node(node->child[1], bounds, oot, cur + first + 1) + first + 1;
}

}  // namespace

bool build_bvh(const float* pos, uint32_t nv, const uint32_t* tri, uint32_t nt, uint32_t maxDepth, BVH* out) {
  (void)nv;
  out->nodeN = 0;
  out->bounds.clear();
  out->offOrTSTN.clear();
  out->order.clear();
  out->stats = BuildStats{};
  if (nt == 0) return false;
  std::vector<uint32_t> order(nt);
  std::vector<BTri> tris(nt);
  for (uint32_t i = 0; i < nt; i++) {  // :248-260
    order[i] = i;
    const float* a = pos + 3 * tri[i * 3];
    const float* b = pos + 3 * tri[i * 3 + 1];
    const float* c = pos + 3 * tri[i * 3 + 2];
    for (int k = 0; k < 3; k++) {
      tris[i].centroid.e[k] = ((a[k] + b[k]) + c[k]) / 3.f;
      tris[i].bound.mn.e[k] = std::fmin(c[k], std::fmin(b[k], a[k]));
      tris[i].bound.mx.e[k] = std::fmax(c[k], std::fmax(b[k], a[k]));
    }
  }
  Node root;
  build_node(&root, tris.data(), order.data(), 0, nt, maxDepth, &out->stats);
  uint32_t nodeN = root.desN + 1;
  out->bounds.assign((size_t)nodeN * 6, 0.f);
  out->offOrTSTN.assign((size_t)nodeN * 2, 0u);
  uint32_t got = compact_node(&root, out->bounds.data(), out->offOrTSTN.data(), 0);
  out->nodeN = nodeN;
  out->order = order;
  return got == nodeN;
}

}  // namespace orc
