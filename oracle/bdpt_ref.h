// TEST INFRASTRUCTURE ONLY -- CPU oracle: the reference's streaming BDPT
// estimator and its adaptive/bilateral variants, per path, in FP32 (bit
// contract shared with the CUDA kernels) or FP64 (the "FP64 host-rendered
// reference" of the same estimator).
#pragma once
#include <cstdint>
#include <vector>

#include "oracle.h"

namespace orc {

// Mirrors gbpt_params in include/gbpt.h (same field order).
struct Params {
  uint32_t seed;
  uint32_t eye_depth_max;    // NORMALRAY_BOUND_MAX (src/cudaRTBDPTStream.cu:7)
  uint32_t light_depth_max;  // LIGHTRAY_BOUND_MAX (:10)
  uint32_t light_paths;      // min(PATHSTREAM_SIZE, LIGHTVERTEX_N / LIGHTRAY_BOUND_MAX) = 128 (:877)
  uint32_t light_every;      // light pass when frame % light_every == 0 (:875)
  float env[3];              // constant environment radiance (0 in the reference)
  uint32_t warmup_frames;    // uniform frames before adaptive sampling (AdapBilatAtomic.cu:1372)
  uint32_t desired_n;        // "Desired Max Sampling" (AdapBilatAtomic.cu:27)
  float filter_color_eud;    // "Filter Color EuD" 50
  float filter_pos_eud;      // "Filter Pos EuD" 1
  float filter_norm_eud;     // "Filter Norm EuD" 0.25
  float filter_diff_eud;     // "Filter Diff EuD" 0.1
  uint32_t filter_radius;    // "Filter Radius" 5
  uint32_t filter_diffuse;   // "Filter Diffuse Flag" 0
  float filter_sigma_spatial;  // <= 0: the reference's quirk (spatial table from the colour delta)
  uint32_t request_id;       // Philox key word 1
  float min_trace_prob;      // "Min Trace Probability" (AdapBilatBinary.cu:28), binary allocator
  // filter-only mode, src/cudaRTBDPTStreamBilat.cu:29-37
  float bilat_color_eud;     // "Filter Color E Delta" 1
  float bilat_pos_eud;       // "Filter Pos E Delta" 1
  float bilat_norm_eud;      // "Filter Norm E Delta" 1
  float bilat_emit_eud;      // "Filter Emit E Delta" 0.5 (not read by the filter call)
  float bilat_diff_eud;      // "Filter Diff E Delta" 0.5
  uint32_t bilat_radius;     // "Filter Radius" 5
  uint32_t filter_iterations;  // "Filter Iteration" 1
  uint32_t render_iterations;  // "Render Iteration" 5 (0: no limit)
  uint32_t pt_depth_max;       // PTSC NORMALRAY_BOUND_MAX (src/cudaRTPTStream.cu:6) 10
};

enum Mode : int32_t { kModeBDPT = 0, kModeAdaptive = 1, kModeAdaptiveBinary = 2, kModeBilat = 3, kModePT = 4 };

struct Camera {
  float pos[3], dir[3], up[3];
  float fov;
};

struct LightVertex {
  float pos[3], norm[3], irrad[3], irradDir[3], diff[3], emissive[3];
  float specular, metallic, roughness;
};

struct PathResult {  // per finished camera path
  double acc[3];
  uint32_t n;
  double gpos[3], gnorm[3], gdiff[3];  // first-hit G-buffer (adaptive variant)
  double gemis[3];                     // first-hit emissive (filter-only mode)
  double direct[3];                    // direct-light sample (filter-only mode)
  double pot;                          // path potential at termination (filter-only mode)
  uint32_t rays;                       // extension + shadow rays traced
  uint64_t nodes, tris;                // traversal work (algorithmic byte count)
  uint32_t extRays;                    // of which extension (closest-hit) walks
  uint64_t extNodes, extTris;
};

struct Renderer {
  uint32_t W = 0, H = 0;
  int32_t mode = kModeBDPT;
  bool fp64 = false;
  Params p{};
  uint32_t frame = 0;
  bool started = false;
  float camBasis[9] = {0};  // pos, dir, up after orthonormalisation
  std::vector<float> result, gpos, gnorm, gdiff, filtered, err;
  std::vector<float> gemis, direct, pot, out;  // filter-only mode; `out` = the view gbpt_render copies
  uint32_t debug_mode = 0;                     // filter-only mode "Debug Mode" (0..7)
  std::vector<uint32_t> sampleN, counts;
  std::vector<uint32_t> chunks;  // binary allocator: paths per pass (last = fill)
  std::vector<LightVertex> cache;
  uint32_t cacheSize = 0;
  uint32_t threads = 1;
  // sub-window of a larger image (row-band sharding): global pixel = (x+x0, y+y0) of fullW x fullH
  uint32_t x0 = 0, y0 = 0, fullW = 0, fullH = 0;
  // statistics of the last frame
  uint64_t lastPaths = 0, lastRays = 0, lastNodes = 0, lastTris = 0;
  uint64_t lastExt[3] = {0, 0, 0};  // extension rays, node visits, triangle tests
};

void default_params(Params* p);
void renderer_init(Renderer* r, uint32_t W, uint32_t H, int32_t mode, const Params& p, bool fp64, uint32_t threads);
void render_frame(Renderer* r, const Scene& s, const Camera& cam);
void light_pass(Renderer* r, const Scene& s, uint32_t frame);
void render_fp64(const Scene& s, const Params& p, uint32_t W, uint32_t H, const Camera& cam, uint32_t frames,
                 uint32_t threads, double* out);

// GetMaterialColors (src/cudaRTCommon.cu:369-406), colour outputs at n uvs:
// 8 floats each (diffuse rgb, emissive rgb, transparency, 0)
void material_colors(const std::vector<Texture>& texs, const RTMaterial& m, const float* uv, uint32_t n, float* out);

// src/cudaBilateralFilter.cu:5-24 and :66-142 (posnorm / posnormemit)
void gaussian_table(float delta, uint32_t radius, float* g);
void bilateral(const float* color, const float* pos, const float* norm, const float* emit, uint32_t W, uint32_t H,
               float colorEuD, float posEuD, float normEuD, float emitEuD, uint32_t radius, const float* g, float* out);

}  // namespace orc
