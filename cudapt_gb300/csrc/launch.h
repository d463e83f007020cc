// Device data layouts and kernel launchers of libgbpt (host-visible part).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace gbpt {

// Scene in HBM.  The BVH node keeps the reference's compact layout
// (src/cudaRTCommon.cu:527-541: float4 min/max + two uint words) folded into
// one 32-byte record: {min.xyz, offOrTs}, {max.xyz, triN}.  Intersection data
// is the reference's p0 / p1-p0 / p2-p0 (:503-513), 48 bytes per triangle.
// Shading data is gathered per triangle in BVH order (5 float4, 80 bytes):
//   {n0.xyz, p0.x} {n1.xyz, p0.y} {n2.xyz, p0.z} {p1.xyz, mat} {p2.xyz, 0}
// so a hit reads one contiguous record instead of RTTriangle + 3 RTVertex.
// Materials: {diffuse.xyz, transparency} {emissive.xyz, specular}
//            {metallic, roughness, diffuseTexId, emissiveTexId} (ids as int
//            bits, -1: none).
//
// Wide traversal (opt-in, gbpt_scene_set_traversal): the same tree collapsed
// to 4 children per node (each node's children are its binary grandchildren,
// or its binary children where those are leaves); 8 float4 per node:
//   {lo.x[4]} {lo.y[4]} {lo.z[4]} {hi.x[4]} {hi.y[4]} {hi.z[4]} {code[4]} {0}
// code: kWideEmpty, kWideTri | first triangle (a one-triangle leaf),
// kWideLeaf | binary node id (other leaves), or a wide node index.
constexpr uint32_t kWideEmpty = 0xFFFFFFFFu, kWideLeaf = 0x80000000u, kWideTri = 0xC0000000u;
struct DevScene {
  const float4* nodes = nullptr;  // nodeN + 1 records of 2 float4, the last all zeros
  const float4* tris = nullptr;   // triN + 1 records of 4 float4 (p0, p1 - p0, p2 - p0, 0), the last all zeros
  const float4* shade = nullptr;
  const float4* mats = nullptr;
  const uint32_t* lightTri = nullptr;
  const float4* wide = nullptr;  // collapsed 4-wide tree (wide traversal only)
  // material textures (only when the scene has any): texels of every texture,
  // one {first texel, width, height, 0} record per texture, and the three
  // vertex uvs of each triangle in BVH order
  const float4* texels = nullptr;
  const uint4* texInfo = nullptr;
  const float2* uvs = nullptr;
  uint32_t nodeN = 0, triN = 0, lightN = 0, matN = 0;
  uint32_t wideN = 0;
  uint32_t traversal = 0;        // 0: the reference's order (default), 1: wide
};

// Counters shared by the kernels of one renderer (device memory).
struct DevCounters {
  uint32_t wave[2];       // paths in the two ping-pong wave buffers
  uint32_t shadow[2];     // connection (shadow) rays queued by bounce d in queue d & 1
  uint32_t cacheSize[2];  // entries of the two light-vertex caches
  uint32_t paths;         // camera paths of the current frame
  uint32_t errFlags;      // bit 0: light cache overflow, bit 1: bounds
  uint32_t fetchT;        // next ray handed to a lane by the persistent walk kernel
  uint32_t heavyMid;      // adaptive accumulation: pixels listed for the warp-per-pixel pass
  uint32_t heavyHuge;     // ... and for the CTA-per-pixel pass
  uint32_t heavySmall;    // ... and for the eight-lanes-per-pixel pass (9..64 samples)
  unsigned long long rays, nodes, tris;  // cumulative work counters (closest-hit walks)
  unsigned long long shadowRays, nodesS, trisS;  // any-hit (shadow) walks
  double errSum;          // adaptive: sum of per-pixel errors
  uint32_t carryN[3];     // extension walks carried out of bounce launch L, in counter L % 3
  uint32_t fetchTail;     // next item handed to a lane by the tail kernel
  uint32_t tailAt;        // bounce from which the tail kernel carries the frame's paths, when a shading
                          // launch found fewer live paths than FrameArgs::tailBelow (~0u: no switch)
};

// Path state of one wavefront (structure of arrays, float4-packed).
struct Wave {
  float4* o;    // origin.xyz, slot (uint bits)
  float4* d;    // direction.xyz, pixel id (uint bits)
  float4* thr;  // throughput (pathOutMulTerm).xyz, path potential (filter-only mode)
  float4* smp;  // carried emission (pathSample).xyz, the path's depth (uint bits): waves mix
                // depths once carried walks rejoin a launch one bounce behind
};

struct FrameArgs {
  float camPos[3], camDir[3], camUp[3], camRight[3];
  float tanHalf, W, H;
  uint32_t width, height, frame;
  uint32_t key0, key1;
  uint32_t eyeDepth, lightDepth, lightPaths;
  float env[3];
  uint32_t specPush;    // adaptive variant: spec reflection origin pushed along reflDir
  uint32_t gbuffer;     // record first-hit position/normal/diffuse
  uint32_t counting;    // node/triangle counters
  uint32_t useEnv;      // env != 0: add env * throughput on a miss
  uint32_t cacheSel;    // light-vertex cache (0/1) this frame reads or the light pass writes
  uint32_t bilat;       // filter-only mode: direct-light sample, path potential, first-hit emissive
  uint32_t ptsc;        // unidirectional mode: no connections, total internal reflection reflects
  uint32_t moments;     // learned allocator: per-pixel second moments and per-tile path-length counts
  uint32_t tilesX;      // 8x8 tiles per image row
  uint32_t refill;      // idle lanes of a warp that trigger a refill in the persistent walks
  uint32_t walkCtas;    // CTAs per SM of the persistent walk and tail grids (0: as many as fit)
  // window of a larger image this renderer covers (gbpt_renderer_set_window):
  // local pixel (x, y) is pixel (winX0 + x, winY0 + y) of a fullW-wide image;
  // W and H above are the full image's for the camera projection, width and
  // height the window's
  uint32_t winX0, winY0, fullW;
  // walk steps a warp keeps stepping its extension walks after the launch's
  // ray queue ran dry before it carries the unfinished ones to the next
  // launch (0: never; the reference-order walk only)
  uint32_t carrySteps;
  // live paths, as a fraction of the band's camera paths, below which the
  // shading launch of a bounce hands the remaining bounces to the tail kernel
  // (decided on the device from the bounce's path count; 0: the fixed switch
  // bounce alone)
  float tailBelow;
};

struct RenderBuffers {
  Wave wave[2];
  float4* hit;          // t, tri bits, u, v (t -1: miss, -2: the walk was carried on); one per wave
                        // path, then one per walk resumed from the previous launch's carry records
  float4* sh[2];        // connection queues (bounce parity), 3 float4 per entry:
                        // {origin, slot} {dir, maxDist} {weighted contribution}
  float4* res;          // per slot: acc.xyz, n bits
  float4* gbuf;         // per slot: 3 float4 (pos, normal, diffuse) when gbuffer; with bilat the
                        // three .w words hold the first-hit emissive
  float4* dsm;          // bilat, per slot: direct-light sample .xyz, path potential at termination .w
  float* m2;            // moments: per-pixel running mean of (path sum)^2 / path count, RGB
  uint32_t* hist;       // moments: per 8x8 tile, paths ended after 0..7+ surface hits (8 counts)
  uint32_t* slotPix;    // per slot pixel id
  uint32_t* slotSmp;    // per slot sample id
  float4* cache[2];     // two light-vertex caches (6 float4 per vertex): one is read by the
                        // current frames while the next light pass fills the other
  DevCounters* ctr;     // this band's queue counters (the renderer's first counters without bands)
  DevCounters* lctr;    // the counters the light pass writes the cache sizes to (the renderer's first)
  uint32_t cap;         // slots
  uint32_t cacheCap;    // light vertices
  // Band of camera paths this wavefront carries: pixels base .. base+count-1.
  // A frame split into bands runs one wavefront per band on its own stream;
  // wave, hit and connection-queue pointers then point at the band's part of
  // the renderer's buffers, and per-slot arrays stay indexed by pixel.
  uint32_t base;
  uint32_t count;
  // extension walks still running when a bounce launch's other work is done
  // are handed over (carried) to the next bounce launch, or the tail kernel,
  // instead of being waited for: kCarryF4 float4 per walk (the path with its
  // depth, the walk's state and stack), up to carryCap walks per launch and
  // band, launch L's in buffer L & 1
  float4* carry[2];
  uint32_t carryCap;
  // per bounce d < connDepth and slot (index d * cap + slot): the connection
  // the path made at bounce d, contribution.xyz and .w = 1 when its walk found
  // it unoccluded, 0 when occluded or none was made; k_fold sums them into the
  // slot's result in bounce order once the frame's walks are done.  Until
  // then a slot's res word holds the path's emission at its end and, in .w,
  // the bounce it ended at.
  float4* conn;
  uint32_t connDepth;
};
constexpr uint32_t kMaxBands = 8;
constexpr uint32_t kCarryF4 = 14;

// wavefront kernels (kernels_wave.cu)
cudaError_t launch_light_pass(const DevScene& S, const FrameArgs& a, const RenderBuffers& b, cudaStream_t st);
cudaError_t launch_camera(const FrameArgs& a, const RenderBuffers& b, cudaStream_t st);
// bounce launch L's persistent walk: the walks launch L - 1 carried (when it
// has a wave), the extension rays of wave `in` (in < 0: none), then the
// shadow rays of connection queue `shIn` (shIn < 0: none); resets the
// counters of wave in^1 and of connection queue `shReset`
cudaError_t launch_walk(const DevScene& S, const FrameArgs& a, const RenderBuffers& b, int in, int shIn,
                        int shReset, uint32_t launch, cudaStream_t st);
// attach: store each continuing path's connection at the path's index (for the tail kernel)
cudaError_t launch_shade(const DevScene& S, const FrameArgs& a, const RenderBuffers& b, int in, uint32_t launch,
                         bool attach, cudaStream_t st);
// threads of the persistent walk grid (the most walks one launch can carry)
uint32_t walk_lanes();
// the sum of every path of the band (connections, then its end): after the
// band's last walk, before the accumulation
cudaError_t launch_fold(const RenderBuffers& b, cudaStream_t st);
// remaining bounces of every path alive at bounce t = min(switch bounce the
// shading launches recorded, K) when t is below the depth cap (wave t & 1,
// starting with the connection attached to each path in queue (t - 1) & 1),
// then of every walk the bounce launches carried; one lane per path
cudaError_t launch_tail(const DevScene& S, const FrameArgs& a, const RenderBuffers& b, uint32_t K, cudaStream_t st);
// first bounce handled by the tail kernel: `requested` when >= 0 (>= D: none),
// else GBPT_TAIL_FROM when set, else D/2 - 1 (wide order: D/2) for D > 6 and
// none for D <= 6
// first bounce the tail kernel carries (requested >= 0, the GBPT_TAIL_FROM
// override, or the default for the depth cap, the paths of one wavefront and
// whether the bounce launches carry walks)
uint32_t tail_from(uint32_t eyeDepth, bool wide, int32_t requested, size_t paths, bool carrying);
// refill threshold of the persistent walks: `requested` when 1..32, else
// GBPT_WALK_REFILL when set, else 8 (reference order) or 20 (wide order)
uint32_t walk_refill_for(uint32_t requested, bool wide);
// Queries (once) the launch shapes of the wavefront kernels, which also loads
// them: call before the first stream capture.
void prepare_launches();
// `blocks` CTAs wait at a grid barrier sized for blocks + 1 (failure-detection self-test)
cudaError_t launch_barrier_selftest(uint32_t* coop, DevCounters* ctr, uint32_t blocks, cudaStream_t st);
cudaError_t launch_apply(const FrameArgs& a, const RenderBuffers& b, float* result, uint32_t* sampleN, float* gpos,
                         float* gnorm, float* gdiff, cudaStream_t st);
// filter-only mode (src/cudaRTBDPTStreamBilat.cu:989-1051): running means of
// the result (no inf filter), the direct-light sample and 1 - path potential;
// the first-hit planes are overwritten with this frame's values
cudaError_t launch_apply_bilat(const FrameArgs& a, const RenderBuffers& b, float* result, uint32_t* sampleN,
                               float* gpos, float* gnorm, float* gdiff, float* gemis, float* direct, float* pot,
                               cudaStream_t st);
// unidirectional mode (pt_applyPathQueueResult_kernel of src/cudaRTPTStream.cu:335-358):
// result = max(acc/n / (frame+1) + (1 - 1/(frame+1)) * result, 0)
cudaError_t launch_apply_pt(const FrameArgs& a, const RenderBuffers& b, float* result, uint32_t* sampleN,
                            cudaStream_t st);
// "Prob" debug views (pt_applyPixelProbToResult_kernel, :933-940): RGB = max(minProb, pot)
cudaError_t launch_prob_view(const float* pot, uint32_t np, float minProb, float* out, cudaStream_t st);
cudaError_t launch_trace_rays(const DevScene& S, const float* rays, uint32_t n, float maxDist, float eps, int cullback,
                              float* t, int32_t* tri, float* w, float* u, float* v, uint32_t* nodes,
                              uint32_t* trisTested, cudaStream_t st);

// adaptive sampling and filter kernels (kernels_adapt.cu)
struct AdaptBuffers {
  float* err;          // W*H
  uint32_t* cnt;       // W*H sample counts
  uint32_t* off;       // W*H exclusive offsets
  uint32_t* blockSum;  // per scan block
  double* partial;     // per reduce block
  float* filtered;     // W*H*3
  uint32_t* coop;      // binary allocator: barrier words, per-block counts, pass table
  float* feat;         // learned allocator: 24 features per 8x8 tile
  float* pred;         // learned allocator: log budget weight per tile
  float* tileErr;      // learned allocator: sum of the heuristic error over each tile
  uint32_t* heavy;     // W*H: pixels with many budgeted samples (medium ones from the front, heaviest from the back)
  uint32_t* list8;     // W*H: pixels with 9..64 budgeted samples
};
constexpr uint32_t kFeatures = 24;
constexpr uint32_t kErrMlpTimeout = 256u;  // DevCounters::errFlags bit: an MLP tensor-core wait ran out
constexpr uint32_t kCoopWords = 8192;  // coop buffer size (uint32 words)
cudaError_t launch_bilateral(const float* color, const float* pos, const float* norm, const float* emit, uint32_t W,
                             uint32_t H, float ceud, float peud, float neud, float eeud, uint32_t radius,
                             const float* g, float* out, cudaStream_t st);
cudaError_t launch_adapt_budget(const FrameArgs& a, const RenderBuffers& b, const AdaptBuffers& ab,
                                const float* result, const uint32_t* sampleN, uint32_t desired, cudaStream_t st);
// the two halves of launch_adapt_budget: per-pixel error (+ partial sums), then
// sum, counts, offsets and camera paths from ab.err
cudaError_t launch_adapt_error(const FrameArgs& a, const AdaptBuffers& ab, const float* result,
                               const uint32_t* sampleN, uint32_t desired, cudaStream_t st);
cudaError_t launch_adapt_alloc(const FrameArgs& a, const RenderBuffers& b, const AdaptBuffers& ab, cudaStream_t st);
// learned allocator: 24 features per 8x8 tile of the current statistics (needs ab.err)
cudaError_t launch_tile_features(const FrameArgs& a, const RenderBuffers& b, const AdaptBuffers& ab,
                                 const float* result, const uint32_t* sampleN, const float* gpos, const float* gnorm,
                                 const float* gdiff, cudaStream_t st);
// learned allocator: per-pixel weights exp(pred[tile]) * err / tile sum; rewrites ab.err and its partial sums
cudaError_t launch_mlp_alloc(const FrameArgs& a, const AdaptBuffers& ab, cudaStream_t st);
cudaError_t launch_adapt_accum(const FrameArgs& a, const RenderBuffers& b, const AdaptBuffers& ab, float* result,
                               uint32_t* sampleN, float* gpos, float* gnorm, float* gdiff, cudaStream_t st);
// binary allocator (src/cudaRTBDPTStreamAdapBilatBinary.cu:1316-1418):
// error, cooperative window search + queue, camera paths for the queue
cudaError_t launch_binary_budget(const FrameArgs& a, const RenderBuffers& b, const AdaptBuffers& ab,
                                 const float* result, const uint32_t* sampleN, uint32_t desired, float minProb,
                                 cudaStream_t st);
// running means of the queue, pass by pass (pt_applyPathQueueResult_kernel per pass)
cudaError_t launch_binary_apply(const FrameArgs& a, const RenderBuffers& b, const AdaptBuffers& ab, float* result,
                                uint32_t* sampleN, float* gpos, float* gnorm, float* gdiff, cudaStream_t st);
uint32_t adapt_scan_blocks(uint32_t np);
uint32_t adapt_reduce_blocks(uint32_t np);
cudaError_t launch_fmath(int which, const float* x, uint32_t n, float* out, cudaStream_t st);
cudaError_t launch_philox(const uint32_t* ctr, uint32_t n, uint32_t k0, uint32_t k1, uint32_t* out, cudaStream_t st);

int sm_count();
// Kernels this library has launched so far (every launcher adds its count).
void note_launches(uint32_t n);
uint64_t launch_count();

}  // namespace gbpt
