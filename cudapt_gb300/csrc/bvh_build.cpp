// Host BVH builder of the GB300 BDPT library.
//
// Produces, bit for bit, the tree of CudaPT's binned-SAH builder
// (src/bvhhelper.cpp:33-313) and its depth-first compaction:
//   * 16 bins over the centroid bounds on the longest centroid axis; bin i
//     holds centroids in [lo + i*L/16, lo + (i+1)*L/16), the last bin ends at
//     (float)(hi + 1e-4) (:87-111);
//   * split cost 0.125 + (nL*SA(cL) + nR*SA(cR)) / SA(node) with the
//     *centroid* bounds of the bins (:120-164), first minimum wins (:173-182);
//   * in-place two-pointer partition around the split plane (:190-211);
//   * leaf when one triangle, depth budget <= 1 or degenerate centroid box
//     (:76-77); empty children are kept as (0, 0) leaves (:58-59, :288-293).
//
// Differences that do not change the result: every centroid is binned in one
// pass (binary search over the 16 bin starts, then the reference's interval
// test) instead of 16 passes, and the two children of large nodes are built
// on separate threads (they own disjoint slices of the triangle order).
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <thread>
#include <vector>

#include "gbpt_internal.h"

namespace gbpt {

namespace {

constexpr uint32_t kBins = 16;

struct Box {
  float mn[3], mx[3];
};
inline Box empty_box() {
  const float inf = (float)1E20;
  return Box{{inf, inf, inf}, {-inf, -inf, -inf}};
}
inline void grow(Box& b, const Box& o) {
  for (int k = 0; k < 3; k++) {
    b.mn[k] = std::fmin(b.mn[k], o.mn[k]);
    b.mx[k] = std::fmax(b.mx[k], o.mx[k]);
  }
}
inline void grow(Box& b, const float* p) {
  for (int k = 0; k < 3; k++) {
    b.mn[k] = std::fmin(b.mn[k], p[k]);
    b.mx[k] = std::fmax(b.mx[k], p[k]);
  }
}
inline float area(const Box& b) {
  float d0 = b.mx[0] - b.mn[0], d1 = b.mx[1] - b.mn[1], d2 = b.mx[2] - b.mn[2];
  if (d0 < 0 || d1 < 0 || d2 < 0 || (double)std::sqrt(d0 * d0 + d1 * d1 + d2 * d2) < 1E-9) return 0;
  return d0 * d1 + d0 * d2 + d1 * d2;
}

struct Node {
  Box bound = empty_box();
  uint32_t triStart = 0, triN = 0, desN = 0;
  std::unique_ptr<Node> child[2];
};

struct Ctx {
  const float* centroid;  // 3 per triangle
  const Box* tbox;
  uint32_t* order;
  uint32_t parallelMin;
  std::atomic<uint32_t> emptyChildren{0};
};

void build(Ctx& c, Node* node, uint32_t triStart, uint32_t triN, uint32_t depthBudget) {
  if (triN == 0) return;
  Box cb = empty_box();
  for (uint32_t i = 0; i < triN; i++) {
    uint32_t ind = c.order[triStart + i];
    grow(node->bound, c.tbox[ind]);
    grow(cb, c.centroid + 3 * (size_t)ind);
  }
  float dia[3] = {cb.mx[0] - cb.mn[0], cb.mx[1] - cb.mn[1], cb.mx[2] - cb.mn[2]};
  if (dia[0] < 0 || dia[1] < 0 || dia[2] < 0) return;
  if (triN == 1 || depthBudget <= 1 ||
      (double)std::sqrt(dia[0] * dia[0] + dia[1] * dia[1] + dia[2] * dia[2]) < 1E-9) {
    node->triStart = triStart;
    node->triN = triN;
    return;
  }
  uint32_t axis = 0;
  if (std::fabs(dia[1]) > std::fabs(dia[0])) axis = 1;
  if (std::fabs(dia[2]) > std::fabs(dia[1]) && std::fabs(dia[2]) > std::fabs(dia[0])) axis = 2;
  const float L = std::fabs(dia[axis]);
  const float lo = cb.mn[axis];
  float start[kBins + 1];
  for (uint32_t i = 0; i <= kBins; i++) start[i] = lo + (float)i * L / (float)kBins;
  const float lastEnd = (float)((double)cb.mx[axis] + 1E-4);

  uint32_t binN[kBins] = {0};
  Box binB[kBins];
  for (uint32_t i = 0; i < kBins; i++) binB[i] = empty_box();
  for (uint32_t j = 0; j < triN; j++) {
    uint32_t ind = c.order[triStart + j];
    const float* cp = c.centroid + 3 * (size_t)ind;
    float p = cp[axis];
    // largest i in [0,15] with start[i] <= p
    int i = (int)(std::upper_bound(start, start + kBins, p) - start) - 1;
    if (i < 0) continue;
    float end = (i + 1 == (int)kBins) ? lastEnd : start[i + 1];
    if (p >= start[i] && p < end) {
      binN[i]++;
      grow(binB[i], cp);
    }
  }
  // prefix (left) and suffix (right) sweeps
  const float nodeSA = area(node->bound);
  uint32_t leftN[kBins], rightN[kBins];
  float leftA[kBins], rightA[kBins];
  {
    Box acc = empty_box();
    uint32_t n = 0;
    for (uint32_t j = 0; j < kBins; j++) {
      n += binN[j];
      grow(acc, binB[j]);
      leftN[j] = n;
      leftA[j] = area(acc);
    }
    acc = empty_box();
    n = 0;
    for (int j = (int)kBins - 1; j >= 0; j--) {
      rightN[j] = n;  // bins j+1 .. 15
      rightA[j] = area(acc);
      n += binN[j];
      grow(acc, binB[j]);
    }
  }
  float heu[kBins];
  for (uint32_t j = 0; j < kBins; j++) {
    // the reference's first sweep (j < 8) adds left + right, the second (j >= 8)
    // right + left; float addition is commutative so both equal this sum.
    heu[j] = 0.125f + ((float)leftN[j] * leftA[j] + (float)rightN[j] * rightA[j]) / nodeSA;
  }
  // heu[15] is the reference's second sweep at j = 16 (all bins on one side,
  // empty other side): the same value as the formula above.
  float minCost = (float)1E20;
  float minBin = kBins - 1;
  for (uint32_t i = 0; i < kBins; i++)
    if (heu[i] < minCost) {
      minCost = heu[i];
      minBin = (float)i;
    }
  const float split = lo + (float)(minBin + 1) * L / (float)kBins;
  uint32_t left = triStart, right = triStart + triN - 1;
  uint32_t* ord = c.order;
  auto cen = [&](uint32_t k) { return c.centroid[3 * (size_t)ord[k] + axis]; };
  while (left < right) {
    while (cen(left) <= split && left < right) left++;
    while (cen(right) > split && left < right) right--;
    if (left < right) {
      std::swap(ord[left], ord[right]);
      left++;
      right--;
    }
  }
  uint32_t mid = (cen(left) <= split) ? left : left - 1;
  node->child[0].reset(new Node());
  node->child[1].reset(new Node());
  uint32_t nl = mid - triStart + 1;
  uint32_t nr = triN - nl;
  if (nl == 0 || nr == 0) c.emptyChildren++;
  Node* L0 = node->child[0].get();
  Node* R0 = node->child[1].get();
  if (triN >= c.parallelMin && nl > 1024 && nr > 1024) {
    std::thread t([&]() { build(c, L0, triStart, nl, depthBudget - 1); });
    build(c, R0, mid + 1, nr, depthBudget - 1);
    t.join();
  } else {
    build(c, L0, triStart, nl, depthBudget - 1);
    build(c, R0, mid + 1, nr, depthBudget - 1);
  }
  node->desN = 2 + L0->desN + R0->desN;
}

uint32_t compact(const Node* node, HostBVH& out, uint32_t cur) {
  for (int k = 0; k < 3; k++) {
    out.bounds[cur * 6 + k] = node->bound.mn[k];
    out.bounds[cur * 6 + 3 + k] = node->bound.mx[k];
  }
  if (!node->child[0] || !node->child[1]) {
    out.offOrTSTN[cur * 2] = node->triStart;
    out.offOrTSTN[cur * 2 + 1] = node->triN;
    return 1;
  }
  out.offOrTSTN[cur * 2 + 1] = 0;
  uint32_t first = compact(node->child[0].get(), out, cur + 1);
  out.offOrTSTN[cur * 2] = first + 1;
  return compact(node->child[1].get(), out, cur + first + 1) + first + 1;
}

}  // namespace

bool build_bvh(const gbpt_vertex* verts, const gbpt_triangle* tris, uint32_t nt, uint32_t maxDepth, uint32_t threads,
               HostBVH* out) {
  out->nodeN = 0;
  if (nt == 0) return false;
  std::vector<float> centroid((size_t)nt * 3);
  std::vector<Box> tbox(nt);
  out->order.resize(nt);
  for (uint32_t i = 0; i < nt; i++) {  // src/bvhhelper.cpp:248-260
    out->order[i] = i;
    const float* a = verts[tris[i].v0].pos;
    const float* b = verts[tris[i].v1].pos;
    const float* cc = verts[tris[i].v2].pos;
    for (int k = 0; k < 3; k++) {
      centroid[(size_t)i * 3 + k] = ((a[k] + b[k]) + cc[k]) / 3.f;
      tbox[i].mn[k] = std::fmin(cc[k], std::fmin(b[k], a[k]));
      tbox[i].mx[k] = std::fmax(cc[k], std::fmax(b[k], a[k]));
    }
  }
  Ctx c;
  c.centroid = centroid.data();
  c.tbox = tbox.data();
  c.order = out->order.data();
  c.parallelMin = threads > 1 ? 8192u : 0xFFFFFFFFu;
  Node root;
  build(c, &root, 0, nt, maxDepth);
  out->nodeN = root.desN + 1;
  out->bounds.assign((size_t)out->nodeN * 6, 0.f);
  out->offOrTSTN.assign((size_t)out->nodeN * 2, 0u);
  out->emptyChildren = c.emptyChildren.load();
  return compact(&root, *out, 0) == out->nodeN;
}

std::vector<float> collapse_wide(const HostBVH& bvh) {
  constexpr uint32_t kEmpty = 0xFFFFFFFFu, kLeaf = 0x80000000u, kTri = 0xC0000000u;
  const uint32_t n = bvh.nodeN;
  auto emptyBox = [&](uint32_t i) { return bvh.bounds[6 * (size_t)i] > bvh.bounds[6 * (size_t)i + 3]; };
  // an inner node has a zero triangle count and a non-empty box (an empty leaf
  // also stores a zero count, but its box is empty)
  auto inner = [&](uint32_t i) { return bvh.offOrTSTN[2 * (size_t)i + 1] == 0 && !emptyBox(i); };
  std::vector<float> out;
  std::vector<uint32_t> src;  // binary node each wide node was made from
  auto add = [&](uint32_t b) {
    src.push_back(b);
    out.resize(out.size() + 32, 0.f);
    return (uint32_t)(src.size() - 1);
  };
  if (n == 0) return out;
  add(0);
  for (size_t w = 0; w < src.size(); w++) {
    const uint32_t b = src[w];
    uint32_t slot[4], ns = 0;
    if (!inner(b)) {
      slot[ns++] = b;  // a leaf root
    } else {
      const uint32_t kids[2] = {b + 1, b + bvh.offOrTSTN[2 * (size_t)b]};
      for (uint32_t c : kids) {
        if (c >= n) continue;
        if (inner(c)) {
          slot[ns++] = c + 1;
          slot[ns++] = c + bvh.offOrTSTN[2 * (size_t)c];
        } else {
          slot[ns++] = c;
        }
      }
    }
    float lo[3][4], hi[3][4];
    uint32_t code[4];
    for (int k = 0; k < 4; k++) {
      code[k] = kEmpty;
      for (int a = 0; a < 3; a++) {
        lo[a][k] = 1e20f;
        hi[a][k] = -1e20f;
      }
    }
    for (uint32_t k = 0; k < ns; k++) {
      const uint32_t s = slot[k];
      if (s >= n || emptyBox(s)) continue;
      for (int a = 0; a < 3; a++) {
        lo[a][k] = bvh.bounds[6 * (size_t)s + a];
        hi[a][k] = bvh.bounds[6 * (size_t)s + 3 + a];
      }
      const uint32_t tn = bvh.offOrTSTN[2 * (size_t)s + 1];
      if (inner(s))
        code[k] = add(s);
      else if (tn == 1)
        code[k] = kTri | bvh.offOrTSTN[2 * (size_t)s];
      else
        code[k] = kLeaf | s;
    }
    float* r = &out[w * 32];
    for (int k = 0; k < 4; k++) {
      for (int a = 0; a < 3; a++) {
        r[a * 4 + k] = lo[a][k];
        r[12 + a * 4 + k] = hi[a][k];
      }
      std::memcpy(&r[24 + k], &code[k], 4);
    }
  }
  return out;
}

}  // namespace gbpt
