// Internal declarations shared by the translation units of libgbpt.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/gbpt.h"

namespace gbpt {

// CompactBVH in host memory (include/bvhhelper.h:45-54) + CreateBVH's order.
struct HostBVH {
  uint32_t nodeN = 0;
  std::vector<float> bounds;        // 6 per node
  std::vector<uint32_t> offOrTSTN;  // 2 per node
  std::vector<uint32_t> order;      // triangle order
  uint32_t emptyChildren = 0;
};

bool build_bvh(const gbpt_vertex* verts, const gbpt_triangle* tris, uint32_t nt, uint32_t maxDepth, uint32_t threads,
               HostBVH* out);

// The binary tree collapsed to 4-wide nodes for the wide traversal: 32 floats
// per node (lo.x[4], lo.y[4], lo.z[4], hi.x[4], hi.y[4], hi.z[4], code[4] as
// uint bits, 4 zeros); see DevScene in launch.h for the child codes.
std::vector<float> collapse_wide(const HostBVH& bvh);

// sqrt(mean((a - b)^2)) over n floats in device memory, summed in double on
// `stream` (a cudaStream_t); image.cu
gbpt_status rmse_device(const float* a, const float* b, uint64_t n, double* out, void* stream);

// MLP inference on device arrays on `stream` (mlp.cu); a tensor-core wait that
// runs out ORs errBit into *err
gbpt_status mlp_forward_async(gbpt_mlp* m, const float* x, uint32_t n, float* y, uint32_t* err, uint32_t errBit,
                              void* stream);

// device bytes a renderer of this size allocates (its admission figure)
uint64_t renderer_bytes(uint32_t W, uint32_t H, const gbpt_params& p);
// the walks' refill threshold for a requested value (0: the library's default)
uint32_t walk_refill_for(uint32_t requested, bool wide);

// thread-local error text (gbpt_last_error_string)
void set_error(const std::string& s);
gbpt_status fail(gbpt_status st, const std::string& s);

}  // namespace gbpt
