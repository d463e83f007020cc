/*
 * gbpt -- GB300-native streaming bidirectional path tracer, C ABI.
 *
 * Drop-in boundary for the BDPT hot path of CudaPT.  Every entry point below
 * names the reference interface it replaces (paths are relative to the
 * CudaPT repository).  Plain pointers and sizes only; no C++ or framework
 * types cross this boundary.  All functions return a gbpt_status; the text of
 * the last error of the calling thread is available from
 * gbpt_last_error_string().
 *
 * Threading: a scene or renderer handle is used by one host thread at a time;
 * different handles may be driven from different threads.  Each renderer owns
 * a CUDA stream; gbpt_render() returns when the frame is complete and, if an
 * output pointer is given, copied.
 */
#ifndef GBPT_H
#define GBPT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum gbpt_status {
  GBPT_OK = 0,
  GBPT_ERR_INVALID_ARG = 1, /* bad handle, size or pointer */
  GBPT_ERR_OOM = 2,         /* device or host allocation failed / admission refused */
  GBPT_ERR_CUDA = 3,        /* a CUDA runtime call failed */
  GBPT_ERR_TIMEOUT = 4,     /* a bounded device wait ran out */
  GBPT_ERR_BOUNDS = 5,      /* a device-side bounds check tripped */
  GBPT_ERR_STATE = 6,       /* call not valid in the current state (e.g. no BVH) */
  GBPT_ERR_NO_DEVICE = 7    /* no CUDA device or the kernels were not built for it */
} gbpt_status;

/* Scene records, byte-compatible with the reference (include/raytracer.h:58-101). */
typedef struct gbpt_vertex { /* RTVertex, 44 bytes */
  float pos[3], norm[3], tan[3], tex[2];
} gbpt_vertex;

typedef struct gbpt_triangle { /* RTTriangle, 16 bytes */
  uint32_t v0, v1, v2, mat;
} gbpt_triangle;

typedef struct gbpt_material { /* RTMaterial (no FULLSPECTRAL), 80 bytes */
  float diffuse[3], emissive[3];
  int32_t diffuseTexId, normalTexId, emissiveTexId, matType;
  float transparency, subsurface, specular, metallic, roughness;
  float anisotropic, sheen, sheenTint, clearcoat, clearcoatGloss;
} gbpt_material;

/* RTTexture (include/raytracer.h:219-226): width*height texels of 4 floats
 * (RGBA), row-major, row 0 first. */
typedef struct gbpt_texture {
  const float* rgba;
  uint32_t width, height;
} gbpt_texture;

/* Camera of RTRenderer::Render(camPos, camDir, camUp, fov, scene)
 * (include/raytracer.h:310); fov in radians. */
typedef struct gbpt_camera {
  float pos[3], dir[3], up[3];
  float fov;
} gbpt_camera;

/* Renderer knobs.  The reference kept these as compile-time defines and GUI
 * attributes: NORMALRAY_BOUND_MAX / LIGHTRAY_BOUND_MAX
 * (src/cudaRTBDPTStream.cu:7,10), the 128-path light pass every 3rd frame
 * (:875-877), and the adaptive attributes of
 * src/cudaRTBDPTStreamAdapBilatAtomic.cu:26-37.  gbpt_params_default() gives
 * the reference values. */
typedef struct gbpt_params {
  uint32_t seed;            /* Philox4x32-10 key word 0 (default 1234) */
  uint32_t eye_depth_max;   /* camera-path bounce cap (5) */
  uint32_t light_depth_max; /* light-path bounce cap (5) */
  uint32_t light_paths;     /* light subpaths per light pass (128, <= 1024) */
  uint32_t light_every;     /* light pass when frame % light_every == 0 (3) */
  float env[3];             /* constant environment radiance on a miss (0) */
  uint32_t warmup_frames;   /* uniform frames before adaptive sampling (5) */
  uint32_t desired_n;       /* "Desired Max Sampling" (5) */
  float filter_color_eud;   /* "Filter Color EuD" (50) */
  float filter_pos_eud;     /* "Filter Pos EuD" (1) */
  float filter_norm_eud;    /* "Filter Norm EuD" (0.25) */
  float filter_diff_eud;    /* "Filter Diff EuD" (0.1) */
  uint32_t filter_radius;   /* "Filter Radius" (5, <= 31) */
  uint32_t filter_diffuse;  /* "Filter Diffuse Flag" (0) */
  float filter_sigma_spatial; /* spatial Gaussian sigma in pixels; <= 0 keeps the
                                 reference's table built from the colour delta */
  uint32_t request_id;      /* Philox key word 1 (0) */
  float min_trace_prob;     /* "Min Trace Probability" of the binary allocator (0) */
  /* "BDPTSC Bilaterial" (filter-only mode, src/cudaRTBDPTStreamBilat.cu:26-52):
   * its own filter deltas, pass counts and frame limit */
  float bilat_color_eud;    /* "Filter Color E Delta" (1) */
  float bilat_pos_eud;      /* "Filter Pos E Delta" (1) */
  float bilat_norm_eud;     /* "Filter Norm E Delta" (1) */
  float bilat_emit_eud;     /* "Filter Emit E Delta" (0.5; kept, the reference's filter call does not read it) */
  float bilat_diff_eud;     /* "Filter Diff E Delta" (0.5): the first-hit diffuse plane's delta */
  uint32_t bilat_radius;    /* "Filter Radius" (5, <= 31) */
  uint32_t filter_iterations; /* "Filter Iteration" (1): filter passes per frame, ping-pong */
  uint32_t render_iterations; /* "Render Iteration" (5): frames that trace paths; 0 = no limit */
  uint32_t pt_depth_max;    /* "PTSC" bounce cap, NORMALRAY_BOUND_MAX of src/cudaRTPTStream.cu:6 (10) */
  /* scheduling of the wavefront (results do not depend on either) */
  uint32_t walk_refill;     /* idle lanes of a warp that make a persistent walk fetch new rays
                               (1..32; 0: 2 in the reference order, 20 in the wide order) */
  int32_t tail_from;        /* first bounce the per-path tail kernel carries (>= the depth cap: none;
                               -1: while carrying, bounce 2 for a frame with fewer camera paths than the
                               walk grid has lanes, else depth / 2 when the cap exceeds 6, else none;
                               without carrying depth / 2 - 1 (wide order: depth / 2) when the cap
                               exceeds 6, else none) */
  uint32_t bands;           /* wavefronts a frame's camera paths are split into, each on its own stream
                               (1..8; 0: 1 while carry_steps is on, else 2 from 512K paths, else 1); the
                               adaptive modes use 1 */
  uint32_t walk_ctas;       /* CTAs per SM of the persistent walk and tail grids (0: as many as fit, 1..32);
                               fewer leave SMs to other requests that share the GPU */
  uint32_t carry_steps;     /* walk steps a bounce launch keeps stepping its last extension walks after
                               its ray queue ran dry before handing the unfinished ones, mid-walk, to the
                               next bounce launch (or the tail kernel), where they finish and are shaded one
                               bounce behind (0: never; default 64; <= 2^20; the reference-order walk only) */
  float tail_below;         /* live paths, as a fraction of the frame's (band's) camera paths, below which a
                               bounce's shading launch hands the remaining bounces to the tail kernel,
                               decided on the device from the bounce's path count ([0, 1]; 0: tail_from
                               alone); the switch comes at tail_from at the latest */
} gbpt_params;

/* Renderer modes: the BDPT entries of the X-macro registry
 * (include/raytracer.h:13-23). */
typedef enum gbpt_mode {
  GBPT_MODE_BDPT_SC = 0,                  /* "BDPTSC"                    cudaRTBDPTStream */
  GBPT_MODE_BDPT_SC_ADAP_BILAT = 1,       /* "BDPTSC Adap Bilat PLL"     cudaRTBDPTStreamAdapBilatAtomic */
  GBPT_MODE_BDPT_SC_ADAP_BILAT_BINARY = 2, /* "BDPTSC Adap Bilat Binary"  cudaRTBDPTStreamAdapBilatBinary */
  GBPT_MODE_BDPT_SC_BILAT = 3,            /* "BDPTSC Bilaterial"          cudaRTBDPTStreamBilat */
  GBPT_MODE_PT_SC = 4                     /* "PTSC" (unidirectional)     cudaRTPTStream */
} gbpt_mode;

/* Per-frame statistics (the reference's PERFBREAKDOWN timers,
 * src/cudaRTBDPTStreamAdapBilatAtomic.cu:1409-1536, plus work counters). */
typedef struct gbpt_stats {
  uint32_t frame;          /* progressive frame index after this call */
  uint32_t light_vertices; /* light-vertex cache size used by this frame */
  uint64_t paths;          /* camera paths traced this frame */
  uint64_t rays;           /* extension + shadow rays this frame */
  uint64_t shadow_rays;    /* of which shadow (connection) rays */
  uint64_t nodes;          /* closest-hit BVH node visits (only with gbpt_set_counting(r, 1)) */
  uint64_t tris;           /* closest-hit triangle tests (only with counting on) */
  uint64_t shadow_nodes;   /* any-hit node visits (counting on) */
  uint64_t shadow_tris;    /* any-hit triangle tests (counting on) */
  float ms_total;          /* device time of the frame */
  float ms_light;          /* light pass */
  float ms_trace;          /* BVH walks: extension rays and, in the same launches, shadow rays */
  float ms_shade;          /* shading / compaction kernels */
  float ms_shadow;         /* 0: shadow rays are walked together with the next bounce's rays */
  float ms_filter;         /* bilateral filter */
  float ms_adapt;          /* error, budget and accumulation kernels */
  uint32_t launches;       /* kernels this library launched during the call (all streams) */
} gbpt_stats;

typedef struct gbpt_scene gbpt_scene;
typedef struct gbpt_renderer gbpt_renderer;

/* ---- library ------------------------------------------------------------ */
const char* gbpt_last_error_string(void);
/* 1 when a usable sm_103 device is present and the kernels load on it. */
gbpt_status gbpt_device_check(int32_t* ok);
gbpt_status gbpt_params_default(gbpt_params* p);

/* ---- scene: RTScene (include/raytracer.h:228-290) ------------------------- */
/* Copies the arrays (RTScene::m_pVertices / m_pTriangles / m_pMaterials).
 * Replaces RTScene::AddModel's Assimp import (src/raytracer.cpp:238-263):
 * the caller passes the imported geometry directly. */
gbpt_status gbpt_scene_create(const gbpt_vertex* verts, uint32_t nv, const gbpt_triangle* tris, uint32_t nt,
                              const gbpt_material* mats, uint32_t nm, gbpt_scene** out);
gbpt_status gbpt_scene_destroy(gbpt_scene* s);
/* NPBVHHelper::CreateBVH + CompactBVH::InitialCompactBVH
 * (src/bvhhelper.cpp:239-313) and AddModel's triangle reorder
 * (src/raytracer.cpp:264-281); then the device upload of initAllSceneCudaMem
 * (src/cudaRTCommon.cu:472-578).  max_depth 32 is the reference default.
 * build_seconds (optional) receives the host build time. */
gbpt_status gbpt_scene_build_bvh(gbpt_scene* s, uint32_t max_depth, uint32_t threads, double* build_seconds);
/* updateAllSceneMaterialsCudaMem (src/cudaRTCommon.cu:580-599) and the
 * light-triangle rescan updateLightTriCudaMem (src/cudaRTBDPTStream.cu:57-77). */
/* BVH walk order.  0 (default): the reference's TracePrimitive order
 * (src/cudaRTCommon.cu:66-127): hits, node and triangle counts bit-exact.
 * 1: wide -- the same tree collapsed to 4 children per node, nearest child
 * first, boxes culled against the closest hit so far; the closest hit is the
 * same triangle (ties go to the one the reference reaches first, the larger
 * triangle index) except where the reference's limits cut its walk short
 * (2048 pops, 29-deep stack) or surfaces lie closer together than the 1e-4
 * origin push; node counts differ.  Restarts progressive accumulation. */
gbpt_status gbpt_scene_set_traversal(gbpt_scene* s, int32_t traversal);
gbpt_status gbpt_scene_update_materials(gbpt_scene* s, const gbpt_material* mats, uint32_t nm);
/* The scene's textures, RTScene::m_pTextures (include/raytracer.h:228-290,
 * filled by AssimpProcessSceneMaterial's texture loader, src/raytracer.cpp:
 * 180-195), copied; they replace any set before.  A material's
 * diffuseTexId / emissiveTexId index them: GetMaterialColors
 * (src/cudaRTCommon.cu:369-406) then takes the diffuse colour from the
 * texture's RGB and multiplies the transparency by its alpha, or takes the
 * emissive colour from the texture's RGB, at the hit's interpolated vertex
 * uv.  Sampling follows the reference's texture descriptor
 * (src/cudaRTCommon.cu:418-448: normalized coordinates, wrap, linear
 * filtering with 8-bit weights), evaluated in the kernels.  normalTexId is
 * fetched but unused by the reference and is ignored here.  A material whose
 * texture id is not below the texture count makes the next upload (first
 * render or trace) fail with GBPT_ERR_INVALID_ARG.  Restarts progressive
 * accumulation. */
gbpt_status gbpt_scene_set_textures(gbpt_scene* s, const gbpt_texture* tex, uint32_t n);
/* CompactBVH export (include/bvhhelper.h:45-54): node count first (pass NULL
 * arrays), then bounds[6*nodeN] (min xyz, max xyz), offOrTSTN[2*nodeN],
 * tri_order[nt] (CreateBVH's return value). */
gbpt_status gbpt_scene_bvh_info(const gbpt_scene* s, uint32_t* node_count, uint32_t* tri_count,
                                uint32_t* light_count);
gbpt_status gbpt_scene_bvh_export(const gbpt_scene* s, float* bounds, uint32_t* off_or_tstn, uint32_t* tri_order);

/* ---- traversal: TracePrimitive (src/cudaRTCommon.cu:66-127) ---------------
 * Closest hit for n rays given as 6 floats (origin, direction).  rays and the
 * outputs may be host or device pointers (is_device = 0/1).  t = -1 and
 * tri = -1 on a miss.  nodes/tris_tested are optional per-ray work counters. */
gbpt_status gbpt_trace_rays(gbpt_scene* s, const float* rays, uint32_t n, float max_dist, float eps, int32_t cullback,
                            float* t, int32_t* tri, float* w, float* u, float* v, uint32_t* nodes,
                            uint32_t* tris_tested, int32_t is_device);

/* ---- renderer: RTRenderer (include/raytracer.h:292-323) -------------------- */
/* RTRenderer::Init(width, height) + SetRendererMode(mode). */
gbpt_status gbpt_renderer_create(uint32_t width, uint32_t height, int32_t mode, const gbpt_params* params,
                                 gbpt_renderer** out);
gbpt_status gbpt_renderer_destroy(gbpt_renderer* r);
gbpt_status gbpt_set_mode(gbpt_renderer* r, int32_t mode);
/* No counterpart in the reference (one image per process there).  The
 * renderer's width x height pixels become the window at (x0, y0) of a
 * full_w x full_h image: camera rays are those of the full image's pixels and
 * every path's random numbers follow from its full-image pixel id, so the
 * windows of one image rendered apart (by separate renderers, processes or
 * GPUs) reproduce the whole image's running means and sample counts to the
 * bit.  (0, 0, width, height) is the whole image again.  Plain, filter-only
 * (its unfiltered planes; the filter sees only the window) and PTSC modes;
 * the adaptive modes, whose budget and filter couple every pixel, refuse a
 * window with GBPT_ERR_STATE at render time.  Restarts accumulation. */
gbpt_status gbpt_renderer_set_window(gbpt_renderer* r, uint32_t x0, uint32_t y0, uint32_t full_w, uint32_t full_h);
gbpt_status gbpt_set_params(gbpt_renderer* r, const gbpt_params* params);
gbpt_status gbpt_get_params(const gbpt_renderer* r, gbpt_params* params);
/* RTRenderer::Render -> <codename>::Render(camPos, camDir, camUp, fov, scene,
 * width, height, result) (src/raytracer.cpp:19-31, 610-625;
 * src/cudaRTBDPTStream.cu:816-951).  Adds one progressive pass; the frame
 * counter restarts when the camera changes.  out_rgb (may be NULL) receives
 * width*height*3 floats, row 0 at the bottom; out_is_device selects a device
 * or host destination.  stats may be NULL. */
gbpt_status gbpt_render(gbpt_renderer* r, gbpt_scene* s, const gbpt_camera* cam, float* out_rgb,
                        int32_t out_is_device, gbpt_stats* stats);
/* Adds `frames` passes without copying (benchmarks / progressive runs). */
gbpt_status gbpt_render_frames(gbpt_renderer* r, gbpt_scene* s, const gbpt_camera* cam, uint32_t frames,
                               gbpt_stats* stats);
/* RTRenderer::GetResult (include/raytracer.h:311): library-owned, page-locked
 * host copy of the current result view, read from the device on each call
 * (NULL before the first pass or on a CUDA error). */
const float* gbpt_result(gbpt_renderer* r);
/* Page-lock (cudaHostRegister) / release a caller-owned host range, so that
 * gbpt_render's out_rgb copy into it runs at link speed rather than through a
 * staging buffer.  Optional: unregistered host memory works, more slowly.
 * Ranges must not overlap a registered page of another range. */
gbpt_status gbpt_host_register(void* p, size_t bytes);
gbpt_status gbpt_host_unregister(void* p);
/* Copies a renderer buffer: 0 result RGB, 1 first-hit position, 2 normal,
 * 3 diffuse (G-buffer: count-weighted means in the adaptive modes, the last
 * frame's first hit in BDPT_SC_BILAT), 4 filtered RGB, 5 per-pixel error
 * (W*H floats), 6 per-pixel sample count (W*H uint32), 7 light-vertex cache
 * (21 floats per vertex), and in BDPT_SC_BILAT: 8 direct-light running mean
 * RGB, 9 first-hit emissive RGB, 10 running mean of 1 - path potential
 * (W*H floats; the "Prob" debug view); with learned-allocator statistics on:
 * 11 per-pixel second moments RGB, 12 per-tile path-length counts (8 uint32
 * per 8x8 tile). */
gbpt_status gbpt_read_buffer(gbpt_renderer* r, int32_t which, void* dst, size_t bytes, int32_t dst_is_device);
/* Restart progressive accumulation (next frame is frame 0). */
gbpt_status gbpt_reset(gbpt_renderer* r);
/* Checkpoint / resume (the reference keeps only .NPRTENV presets with an
 * optional converged image, src/cudapt.cpp:735-836).  A checkpoint holds the
 * frame counter, camera, mode, parameters and every per-pixel accumulator; a
 * renderer of the same size restored from it and given the same scene (same
 * triangle and node counts) and camera continues the interrupted sequence to
 * the bit.  gbpt_renderer_checkpoint_size gives the bytes the host buffer
 * needs (about 150 per pixel). */
gbpt_status gbpt_renderer_checkpoint_size(gbpt_renderer* r, size_t* bytes);
gbpt_status gbpt_renderer_checkpoint(gbpt_renderer* r, void* buf, size_t bytes);
gbpt_status gbpt_renderer_restore(gbpt_renderer* r, const void* buf, size_t bytes);
/* CleanMem (src/cudaRTBDPTStream.cu:780-789): release device buffers now;
 * they are re-created on the next render. */
gbpt_status gbpt_clean(gbpt_renderer* r);
/* Enable per-frame node/triangle counters (costs one atomic per warp and step). */
gbpt_status gbpt_set_counting(gbpt_renderer* r, int32_t on);

/* ---- attributes: GetAttribute / GetAttribsN (src/raytracer.cpp:19-31) -----
 * The names are the current mode's: the adaptive modes list the reference's
 * "Desired Max Sampling", "Filter Color EuD", ... (AdapBilatAtomic.cu:48-60);
 * BDPT_SC_BILAT lists "Filter Color E Delta" ... "Render Iteration"
 * (src/cudaRTBDPTStreamBilat.cu:40-50).  Both add the knobs the reference kept
 * as defines (depth caps, light paths, seed).  "Debug Mode" selects the view
 * gbpt_render copies out: adaptive modes 0 result, 4 filtered; BDPT_SC_BILAT
 * 0/1 filtered, 2/3 filtered path-potential view, 4 direct light, 5 position,
 * 6 normal, 7 unfiltered result. */
gbpt_status gbpt_attr_count(const gbpt_renderer* r, uint32_t* n);
gbpt_status gbpt_attr_name(const gbpt_renderer* r, uint32_t index, char* name, size_t cap);
gbpt_status gbpt_attr_get(const gbpt_renderer* r, const char* name, float* value);
gbpt_status gbpt_attr_set(gbpt_renderer* r, const char* name, float value);

/* ---- bilateral filter: cudaBilateralFilter (src/cudaBilateralFilter.cu) ----
 * updateGaussian (:5-24) into g[2*radius+1]. */
gbpt_status gbpt_gaussian_table(float delta, uint32_t radius, float* g);
/* bilaterial_posnorm_kernel (:66-101) when emit == NULL, else
 * bilaterial_posnormemit_kernel (:103-142).  All planes are W*H*3 floats, on
 * the device when is_device = 1, else on the host; g is a host table of
 * 2*radius+1 floats. */
gbpt_status gbpt_bilateral(const float* color, const float* pos, const float* norm, const float* emit,
                           uint32_t width, uint32_t height, float color_eud, float pos_eud, float norm_eud,
                           float emit_eud, uint32_t radius, const float* g, float* out, int32_t is_device);
/* No counterpart in the reference.  Same filter as gbpt_bilateral on device
 * arrays, for callers that must not allocate device memory (a process whose
 * device heap is owned by its own pool, or a latency-critical caller that
 * cannot afford a cudaMalloc/cudaFree pair): the weight table g (host,
 * 2*radius+1 floats) is staged in a file-scope device array of 64 floats
 * instead of a per-call allocation, so radius must be <= 31.  The array is
 * shared by all calls on a device (calls that overlap on the GPU race on it).
 * The first call in a device's context resolves the array's address (again
 * after cudaDeviceReset).  Each call copies g from host memory and then
 * synchronizes the whole stream (all work queued on it, not only the
 * filter), so it must not be made while the stream is being captured: it
 * returns GBPT_ERR_STATE then.  stream may be NULL (default stream). */
gbpt_status gbpt_bilateral_noalloc(const float* color, const float* pos, const float* norm, const float* emit,
                                   uint32_t width, uint32_t height, float color_eud, float pos_eud, float norm_eud,
                                   float emit_eud, uint32_t radius, const float* g, float* out, void* stream);

/* ---- RMSE experiments and image export (src/cudapt.cpp:482-619, 867-997) ---
 * RMSE = sqrt(sum((a - b)^2) / n) over n floats, summed in double on the
 * device (the reference sums in float on the host). */
gbpt_status gbpt_rmse(const float* a, const float* b, uint64_t n, int32_t is_device, double* out);
/* RMSE of the image gbpt_render would copy out (the current view) against a
 * converged W*H*3 image (CUDAPTWindow::CalculateRMSE), without copying the
 * view to the host. */
gbpt_status gbpt_renderer_rmse(gbpt_renderer* r, const float* converged, int32_t converged_is_device, double* out);
/* 8-bit RGBA export, top row first (the float image has row 0 at the bottom):
 * kind 0 the tone-mapped result of BrowseAndSaveResult (clamp to [0,1],
 * 1 - exp(-x * exposure), x^(1/2.2)); kind 1 the per-pixel MSE against ref of
 * BrowseAndSaveMSEResult; kind 2 clamp to [0,1] (ExportConvergedResult).
 * bytes = (unsigned char)(x * 255); alpha 255.  Device arrays (is_device) must
 * be 4-byte aligned. */
gbpt_status gbpt_tonemap_rgba8(const float* rgb, const float* ref, uint32_t width, uint32_t height, float exposure,
                               int32_t kind, uint8_t* out_rgba, int32_t is_device);

/* ---- learned sample allocator (no reference counterpart: CudaPT links FANN
 * but never calls it) -------------------------------------------------------
 * A 24 -> 64 -> 64 -> 1 GELU MLP with BF16 weights and FP32 accumulation on
 * the tensor cores (tcgen05), trained with Adam on mean squared error.
 * Parameters: an FP32 vector of gbpt_mlp_param_count() = 5825 values laid out
 * W1[64][24], b1[64], W2[64][64], b2[64], w3[64], b3.  Inputs: n rows of 24
 * FP32 features; targets / outputs: n FP32 values. */
typedef struct gbpt_mlp gbpt_mlp;
uint32_t gbpt_mlp_param_count(void);
/* He-uniform weights from Philox draws of `seed`, zero biases. */
gbpt_status gbpt_mlp_create(uint32_t seed, gbpt_mlp** out);
gbpt_status gbpt_mlp_destroy(gbpt_mlp* m);
gbpt_status gbpt_mlp_get_params(gbpt_mlp* m, float* params);
/* Also resets the Adam moments and step. */
gbpt_status gbpt_mlp_set_params(gbpt_mlp* m, const float* params);
gbpt_status gbpt_mlp_forward(gbpt_mlp* m, const float* x, uint32_t n, float* y, int32_t is_device);
/* Gradient of mean((y - t)^2) (param_count values) and the loss; no update. */
gbpt_status gbpt_mlp_gradients(gbpt_mlp* m, const float* x, const float* t, uint32_t n, int32_t is_device,
                               float* grad, float* loss);
/* One Adam step (beta 0.9 / 0.999, eps 1e-8, bias-corrected) on a batch. */
gbpt_status gbpt_mlp_train_step(gbpt_mlp* m, const float* x, const float* t, uint32_t n, float lr,
                                int32_t is_device, float* loss);

/* Run the renderer's work on the caller's cudaStream_t (NULL: back to its own
 * stream), so that several renderers can be batched on streams the caller
 * schedules.  Every call still returns when its frame is complete. */
gbpt_status gbpt_renderer_set_stream(gbpt_renderer* r, void* stream);
/* on != 0: in the plain (BDPT_SC) and PTSC modes each frame's launches are
 * captured and issued as one CUDA graph (updated in place from frame to
 * frame); the image is the same.  With stats, only ms_total is broken down
 * (into the trace phase).  Off by default. */
gbpt_status gbpt_renderer_set_graphs(gbpt_renderer* r, int32_t on);

/* Learned allocation in GBPT_MODE_BDPT_SC_ADAP_BILAT: with mlp != NULL every
 * budgeted frame turns the heuristic per-pixel error into per-tile weights
 * exp(mlp(features)) spread over each 8x8 tile in proportion to the heuristic
 * (the network is not owned; keep it alive while attached).  collect != 0
 * keeps the statistics the features need (per-pixel second moments, per-tile
 * path-length counts) without changing the allocation.  NULL, 0: plain. */
gbpt_status gbpt_renderer_set_mlp(gbpt_renderer* r, gbpt_mlp* mlp, int32_t collect);
/* The 24 features of every 8x8 tile (row-major tiles, ceil(W/8) per row) of
 * the current statistics (adaptive modes, after frames rendered with the
 * statistics on): 0-2 log(1 + mean colour), 3-5 log(1 + 100 * mean variance of
 * the pixel means), 6-8 mean albedo, 9-11 mean normal, 12 log(1 + mean
 * first-hit distance), 13-20 fraction of paths ending after 0..7+ hits,
 * 21 log2(1 + mean spp), 22/23 log(1 + 1000 * mean / max heuristic error).
 * out == NULL: only *n_tiles. */
gbpt_status gbpt_renderer_features(gbpt_renderer* r, float* out, uint32_t capacity, int32_t out_is_device,
                                   uint32_t* n_tiles);

/* ---- batched render serving ----------------------------------------------
 * The reference renders one scene per process, synchronously
 * (src/cudaRTBDPTStream.cu:134-169, 816-951).  A server takes render requests
 * of uneven size from any thread and runs up to `workers` of them at once,
 * each on its own renderer and CUDA stream, so that small requests fill the
 * SMs together; scenes stay resident on the device.  A request is admitted
 * when its renderer's buffers fit in free HBM minus `hbm_reserve_bytes`
 * (otherwise it waits for running requests to free memory, and fails with
 * GBPT_ERR_OOM only when nothing else runs).  Requests whose params leave
 * walk_refill = 0 and tail_from = -1 get those scheduling knobs from the
 * server's autotuner, which times whole requests per class (mode, depth cap,
 * image size) and keeps the fastest candidate; the knobs change only speed,
 * never the image. */
typedef struct gbpt_server gbpt_server;
typedef struct gbpt_request {
  gbpt_scene* scene;         /* BVH built; shared by any number of requests */
  gbpt_camera camera;
  uint32_t width, height;
  uint32_t frames;           /* progressive passes (samples per pixel in BDPT_SC) */
  int32_t mode;              /* gbpt_mode */
  const gbpt_params* params; /* NULL: defaults; copied at submission */
  float* out_rgb;            /* NULL or a host buffer of width*height*3 floats, written on completion */
} gbpt_request;
typedef struct gbpt_request_status {
  uint64_t id;
  int32_t status;            /* GBPT_OK or the error the request ended with */
  uint32_t done;             /* 1 once finished */
  double queued_ms;          /* submission to start */
  double run_ms;             /* start to completion (image on the host) */
  double latency_ms;         /* submission to completion */
  uint64_t paths;            /* camera paths traced */
  uint32_t walk_refill;      /* the scheduling knobs it ran with */
  int32_t tail_from;
} gbpt_request_status;
gbpt_status gbpt_server_create(uint32_t workers, uint64_t hbm_reserve_bytes, gbpt_server** out);
/* Queue order: GBPT_SERVE_FIFO, or GBPT_SERVE_SHORTEST_FIRST (default): the
 * queued request with the least estimated run time (its camera paths at
 * 1e5 paths per ms) minus the time it has waited starts next. */
enum { GBPT_SERVE_FIFO = 0, GBPT_SERVE_SHORTEST_FIRST = 1 };
gbpt_status gbpt_server_set_policy(gbpt_server* s, int32_t policy);
/* on != 0 (default): the server's renderers issue plain / PTSC frames as
 * CUDA graphs (gbpt_renderer_set_graphs). */
gbpt_status gbpt_server_set_graphs(gbpt_server* s, int32_t on);
/* Finishes the queued and running requests, then frees every renderer. */
gbpt_status gbpt_server_destroy(gbpt_server* s);
gbpt_status gbpt_server_submit(gbpt_server* s, const gbpt_request* req, uint64_t* id);
/* Waits up to timeout_ms (0: poll) for request `id`; GBPT_ERR_TIMEOUT if it
 * is still queued or running (out->done = 0).  A finished request's status
 * stays readable until the server is destroyed. */
gbpt_status gbpt_server_wait(gbpt_server* s, uint64_t id, uint32_t timeout_ms, gbpt_request_status* out);
/* Forgets a finished request's status (a long-running server otherwise keeps
 * every status until it is destroyed); GBPT_ERR_STATE while it runs. */
gbpt_status gbpt_server_release(gbpt_server* s, uint64_t id);
/* All knobs the autotuner holds for a request class: walk_refill, tail_from,
 * bands and walk_ctas of *knobs (the other fields are the defaults); the
 * class's first candidate when it has no samples yet; *samples requests
 * timed so far. */
gbpt_status gbpt_server_tuned_params(gbpt_server* s, int32_t mode, uint32_t depth, uint32_t width, uint32_t height,
                                     gbpt_params* knobs, uint32_t* samples);
/* The autotuner's choice for a class (its refill and tail knobs only):
 * *samples requests timed so far. */
gbpt_status gbpt_server_tuned(gbpt_server* s, int32_t mode, uint32_t depth, uint32_t width, uint32_t height,
                              uint32_t* walk_refill, int32_t* tail_from, uint32_t* samples);

/* ---- failure detection ------------------------------------------------------
 * Device waits (the binary allocator's grid barrier, the learned allocator's
 * tensor-core completions) are bounded: one that runs out sets a bit of the
 * renderer's device error word and its kernel returns, and the next host call
 * reports GBPT_ERR_TIMEOUT with the context still usable.  This self-test
 * runs the grid barrier with one block missing, so its wait runs out (about
 * a second); it returns GBPT_ERR_TIMEOUT, and *elapsed_ms the wait's length. */
gbpt_status gbpt_selftest_wait_timeout(double* elapsed_ms);
/* Host-side fault injection for tests: after `after` more successful device
 * allocations of the renderer / scene code, the following ones fail (as an
 * out-of-memory device would) until called again with after < 0. */
gbpt_status gbpt_test_fail_allocations(int64_t after);

/* ---- device math, exposed for verification -------------------------------
 * Evaluated by a kernel on host arrays x/out (copied in and out).
 * which: 0 sin, 1 cos, 2 exp, 3 round-down sqrt, 4 x^5, 5 exp of an argument <= 0 as the
 * bilateral filter's tile kernel evaluates it (equal to 2 there). */
gbpt_status gbpt_fmath(int32_t which, const float* x, uint32_t n, float* out);
/* Test utility (allocates): n float4 samples of one RGBA float texture at the
 * n (u, v) pairs of uv, either through the texture unit (hardware = 1: a
 * texture object with CreateCURTTexture's descriptor, src/cudaRTCommon.cu:
 * 418-448) or through the kernels' software filter (hardware = 0); host
 * arrays. */
gbpt_status gbpt_texture_sample(const float* rgba, uint32_t width, uint32_t height, const float* uv, uint32_t n,
                                int32_t hardware, float* out);
/* Philox4x32-10 by a kernel: n counters (4 words each) -> 4 words each, host arrays. */
gbpt_status gbpt_philox(const uint32_t* ctr, uint32_t n, uint32_t k0, uint32_t k1, uint32_t* out);

#ifdef __cplusplus
}
#endif
#endif /* GBPT_H */
