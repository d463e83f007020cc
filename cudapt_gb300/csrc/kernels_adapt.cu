// Adaptive sampling and bilateral-filter kernels for GB300 (sm_103a).
//
//   bilateral   bilaterial_posnorm_kernel / bilaterial_posnormemit_kernel
//               (src/cudaBilateralFilter.cu:66-142), shared-memory tiles
//   error       pt_calculateSquareError_kernel (src/cudaRTBDPTStreamAdapBilatAtomic.cu:1143-1156)
//               fused with a per-block FP64 partial sum (replaces thrust::reduce, :1444)
//   budget      pt_genAdapPathQueue_kernel (:817-842): floor(W*H * e_p / sum e)
//               samples per pixel, laid out pixel-major by an exclusive scan
//               (replaces the warp-aggregated atomic append, src/cudaRTCommon.cu:620-628)
//   accumulate  pt_atomicApplyPathQueueResult_kernel + pt_accumTempResultToResult_kernel
//               (:1041-1141): each pixel sums its own samples in sample order
//               instead of float atomics, so the result does not depend on timing.
#include <cuda_runtime.h>

#include <cmath>

#include <cstddef>

#include "gbpt_math.cuh"
#include "launch.h"

namespace gbpt {

namespace {

constexpr int kTile = 16;
constexpr int kScanBlock = 1024;
constexpr int kReduceBlock = 256;

// -mod / c2, the exponent of src/cudaBilateralFilter.cu:26-33.  A negative c2
// stands for -1/c2' of a power of two c2' (bilateral_c2 on the host): then
// mod * c2 is the same correctly rounded value as -mod / c2' (the exact
// quotient is the exact product), one multiply instead of a divide.
__device__ __forceinline__ float neg_ratio(float mod, float c2) { return c2 < 0.f ? mod * c2 : -mod / c2; }

__device__ __forceinline__ float eucl(float ax, float ay, float az, float bx, float by, float bz, float c2) {
  // src/cudaBilateralFilter.cu:26-33: exp(-|b-a|^2 / (2 d d)), c2 = (2*d)*d
  float dx = bx - ax, dy = by - ay, dz = bz - az;
  float mod = (dx * dx + dy * dy) + dz * dz;
  return gb::exp_p(neg_ratio(mod, c2));
}

// gb::exp_p for arguments x <= 0 (or NaN), to the bit: the same reduction and
// polynomial, with 2^k applied as one factor and the x < -87 case as a
// select instead of a branch.  For -87 <= x <= 0, k = rint(x log2 e) lies in
// [-126, 0], so 2^k is a normal number; exp_p's p * 2^k1 is then a normal
// number (exact) and its second product p * 2^k1 * 2^k2 rounds exactly as
// the single product p * 2^k does.
__device__ __forceinline__ float exp_nonpos_p(float x) {
  using namespace gb;
  const float log2e = 0x1.715476p+0f;
  const float ln2_hi = 0x1.62e430p-1f;
  const float ln2_lo = -0x1.05c610p-29f;
  const float kf = rint_(x * log2e);
  float r = fma_(-kf, ln2_hi, x);
  r = fma_(-kf, ln2_lo, r);
  float p = fma_(r, 1.98412698e-04f, 1.38888889e-03f);
  p = fma_(r, p, 8.33333333e-03f);
  p = fma_(r, p, 4.16666667e-02f);
  p = fma_(r, p, 1.66666667e-01f);
  p = fma_(r, p, 0.5f);
  p = fma_(r, p, 1.0f);
  p = fma_(r, p, 1.0f);
  const float res = p * bits_f((uint32_t)((int)kf + 127) << 23);
  return (x < -87.0f) ? 0.0f : res;
}

// eucl() for the tile kernel: -mod / c2 <= 0 (or NaN) for c2 >= 0
__device__ __forceinline__ float eucl_nonpos(float ax, float ay, float az, float bx, float by, float bz, float c2) {
  float dx = bx - ax, dy = by - ay, dz = bz - az;
  float mod = (dx * dx + dy * dy) + dz * dz;
  return exp_nonpos_p(neg_ratio(mod, c2));
}

// Tap (x+j, y+i) with the reference's unsigned arithmetic: a coordinate left
// of column 0 wraps to a huge value and min() sends it to the last column.
__device__ __forceinline__ uint32_t wrapc(int g, uint32_t n) { return ((uint32_t)g < n) ? (uint32_t)g : n - 1; }

// One 16x16 output tile; the (16+2r)^2 input window is staged in shared
// memory as one 48-byte record per texel -- colour, position, normal and (the
// filter-only mode's fourth plane) emission packed into three float4 -- so a
// tap is three 16-byte shared loads.  A quarter warp's eight consecutive
// records start 12 words apart and cover all 32 banks once: no conflicts.
// kR > 0 fixes the radius at compile time (the tap row is unrolled and its
// weights live in registers); kR == 0 takes r at run time.
template <bool kEmit, int kR>
__global__ void __launch_bounds__(kTile* kTile) k_bilateral_tile(const float* __restrict__ color,
                                                                  const float* __restrict__ pos,
                                                                  const float* __restrict__ norm,
                                                                  const float* __restrict__ emit, uint32_t W,
                                                                  uint32_t H, float cc2, float pc2, float nc2,
                                                                  float ec2, int rArg, const float* __restrict__ g,
                                                                  float* __restrict__ out) {
  extern __shared__ float4 smv[];
  const int r = kR > 0 ? kR : rArg;
  const int T = kTile + 2 * r;
  float* sg = reinterpret_cast<float*>(smv);  // 2r+1 gaussian weights, padded to whole float4
  float4* tile = smv + (2 * r + 1 + 3) / 4;
  const int x0 = blockIdx.x * kTile - r, y0 = blockIdx.y * kTile - r;
  const int tid = threadIdx.y * kTile + threadIdx.x;
  for (int k = tid; k < 2 * r + 1; k += kTile * kTile) sg[k] = g[k];
  for (int k = tid; k < T * T; k += kTile * kTile) {
    int ty = k / T, tx = k - ty * T;
    uint32_t gx = wrapc(x0 + tx, W), gy = wrapc(y0 + ty, H);
    size_t src = 3 * ((size_t)gy * W + gx);
    float4* dst = tile + 3 * (size_t)k;
    const float n2 = norm[src + 2];
    dst[0] = make_float4(color[src], color[src + 1], color[src + 2], pos[src]);
    dst[1] = make_float4(pos[src + 1], pos[src + 2], norm[src], norm[src + 1]);
    dst[2] = kEmit ? make_float4(n2, emit[src], emit[src + 1], emit[src + 2]) : make_float4(n2, 0.f, 0.f, 0.f);
  }
  __syncthreads();
  const uint32_t x = blockIdx.x * kTile + threadIdx.x, y = blockIdx.y * kTile + threadIdx.y;
  if (x >= W || y >= H) return;
  const float4* c4 = tile + 3 * (size_t)((threadIdx.y + r) * T + threadIdx.x + r);
  const float4 cA = c4[0], cB = c4[1], cC = c4[2];
  float sum = 0.f, tx = 0.f, ty = 0.f, tz = 0.f;
  // one tap, in the reference's order of products and sums
  auto tap = [&](const float4* q, float f) {
    const float4 A = q[0], B = q[1], C = q[2];
    f = f * eucl_nonpos(A.x, A.y, A.z, cA.x, cA.y, cA.z, cc2);
    f = f * eucl_nonpos(A.w, B.x, B.y, cA.w, cB.x, cB.y, pc2);
    f = f * eucl_nonpos(B.z, B.w, C.x, cB.z, cB.w, cC.x, nc2);
    if (kEmit) f = f * eucl_nonpos(C.y, C.z, C.w, cC.y, cC.z, cC.w, ec2);
    tx = tx + f * A.x;
    ty = ty + f * A.y;
    tz = tz + f * A.z;
    sum = sum + f;
  };
  if constexpr (kR > 0) {
    float gw[2 * kR + 1];
#pragma unroll
    for (int j = 0; j <= 2 * kR; j++) gw[j] = sg[j];
#pragma unroll 1
    for (int i = 0; i <= 2 * kR; i++) {
      const float gi = sg[i];
      const float4* row = tile + 3 * (size_t)((threadIdx.y + i) * T + threadIdx.x);
#pragma unroll
      for (int j = 0; j <= 2 * kR; j++) tap(row + 3 * j, gi * gw[j]);
    }
  } else {
    for (int i = 0; i <= 2 * r; i++) {
      const float gi = sg[i];
      const float4* row = tile + 3 * (size_t)((threadIdx.y + i) * T + threadIdx.x);
      for (int j = 0; j <= 2 * r; j++) tap(row + 3 * j, gi * sg[j]);
    }
  }
  float* o = out + 3 * ((size_t)y * W + x);
  o[0] = tx / sum;
  o[1] = ty / sum;
  o[2] = tz / sum;
}

// Same arithmetic, reading global memory directly (large radii).
template <bool kEmit>
__global__ void k_bilateral_direct(const float* __restrict__ color, const float* __restrict__ pos,
                                   const float* __restrict__ norm, const float* __restrict__ emit, uint32_t W,
                                   uint32_t H, float cc2, float pc2, float nc2, float ec2, int r,
                                   const float* __restrict__ g, float* __restrict__ out) {
  const uint32_t x = blockIdx.x * kTile + threadIdx.x, y = blockIdx.y * kTile + threadIdx.y;
  if (x >= W || y >= H) return;
  const size_t c = 3 * ((size_t)y * W + x);
  float sum = 0.f, tx = 0.f, ty = 0.f, tz = 0.f;
  for (int i = -r; i <= r; i++)
    for (int j = -r; j <= r; j++) {
      size_t q = 3 * ((size_t)wrapc((int)y + i, H) * W + wrapc((int)x + j, W));
      float f = g[i + r] * g[j + r];
      f = f * eucl(color[q], color[q + 1], color[q + 2], color[c], color[c + 1], color[c + 2], cc2);
      f = f * eucl(pos[q], pos[q + 1], pos[q + 2], pos[c], pos[c + 1], pos[c + 2], pc2);
      f = f * eucl(norm[q], norm[q + 1], norm[q + 2], norm[c], norm[c + 1], norm[c + 2], nc2);
      if (kEmit) f = f * eucl(emit[q], emit[q + 1], emit[q + 2], emit[c], emit[c + 1], emit[c + 2], ec2);
      tx = tx + f * color[q];
      ty = ty + f * color[q + 1];
      tz = tz + f * color[q + 2];
      sum = sum + f;
    }
  out[c] = tx / sum;
  out[c + 1] = ty / sum;
  out[c + 2] = tz / sum;
}

// per-pixel error and per-block FP64 partial sums
__global__ void __launch_bounds__(kReduceBlock) k_error(const float* __restrict__ filtered,
                                                        const float* __restrict__ result,
                                                        const uint32_t* __restrict__ sampleN, uint32_t np,
                                                        uint32_t D, float* __restrict__ err,
                                                        double* __restrict__ partial) {
  __shared__ double ws[kReduceBlock / 32];
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  double v = 0.0;
  if (p < np) {
    uint32_t sn = sampleN[p];
    float rf = (float)D / (float)(D + sn);
    if (D + sn < sn) rf = 0.f;
    const float* a = filtered + 3 * (size_t)p;
    const float* b = result + 3 * (size_t)p;
    float d0 = a[0] - b[0], d1 = a[1] - b[1], d2 = a[2] - b[2];
    float e = (rf * ((d0 * d0 + d1 * d1) + d2 * d2)) / 3.f;
    err[p] = e;
    v = (double)e;
  }
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < kReduceBlock / 32; w++) s += ws[w];
    partial[blockIdx.x] = s;
  }
}

__global__ void k_reduce_final(const double* __restrict__ partial, uint32_t n, DevCounters* ctr) {
  __shared__ double ws[32];
  double v = 0.0;
  for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) v += partial[i];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (uint32_t w = 0; w < (blockDim.x + 31) / 32; w++) s += ws[w];
    ctr->errSum = s;
  }
}

// counts and block-local exclusive scan
__global__ void __launch_bounds__(kScanBlock) k_budget(const float* __restrict__ err, uint32_t np,
                                                       const DevCounters* __restrict__ ctr, uint32_t* cnt,
                                                       uint32_t* off, uint32_t* blockSum) {
  __shared__ uint32_t ws[kScanBlock / 32];
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  const float sumF = (float)ctr->errSum;
  uint32_t c = 0;
  if (p < np) {
    float ratio = err[p] / sumF;
    float v = (float)np * ratio;
    c = (v >= 1.f && v < 4294967040.f) ? (uint32_t)v : 0u;
    cnt[p] = c;
  }
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t incl = c;
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= (uint32_t)o) incl += t;
  }
  if (lane == 31) ws[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    uint32_t s = (lane < kScanBlock / 32) ? ws[lane] : 0u;
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t t = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= (uint32_t)o) s += t;
    }
    if (lane < kScanBlock / 32) ws[lane] = s;
  }
  __syncthreads();
  uint32_t before = (warp > 0) ? ws[warp - 1] : 0u;
  if (p < np) off[p] = before + incl - c;
  if (threadIdx.x == blockDim.x - 1) blockSum[blockIdx.x] = ws[kScanBlock / 32 - 1];
}

// exclusive scan of the block sums (one CTA; 64-bit running total)
__global__ void k_scan_blocks(uint32_t* blockSum, uint32_t nb, uint32_t gen, DevCounters* ctr) {
  __shared__ unsigned long long carry;
  __shared__ uint32_t ws[32];
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (uint32_t base = 0; base < nb; base += blockDim.x) {
    uint32_t i = base + threadIdx.x;
    uint32_t v = (i < nb) ? blockSum[i] : 0u;
    uint32_t incl = v;
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= (uint32_t)o) incl += t;
    }
    if (lane == 31) ws[warp] = incl;
    __syncthreads();
    if (warp == 0) {
      uint32_t s = (lane < nw) ? ws[lane] : 0u;
      for (int o = 1; o < 32; o <<= 1) {
        uint32_t t = __shfl_up_sync(0xffffffffu, s, o);
        if (lane >= (uint32_t)o) s += t;
      }
      if (lane < nw) ws[lane] = s;
    }
    __syncthreads();
    unsigned long long c0 = carry;
    unsigned long long ex = c0 + ((warp > 0) ? ws[warp - 1] : 0u) + incl - v;
    if (i < nb) blockSum[i] = (uint32_t)(ex < gen ? ex : gen);
    __syncthreads();
    if (threadIdx.x == 0) carry = c0 + ws[nw - 1];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    unsigned long long tot = carry < gen ? carry : gen;
    ctr->wave[0] = (uint32_t)tot;
    ctr->paths = (uint32_t)tot;
    ctr->fetchT = 0;
    ctr->carryN[0] = ctr->carryN[1] = ctr->carryN[2] = 0;
    ctr->fetchTail = 0;
    ctr->tailAt = 0xFFFFFFFFu;
  }
}

// global clamped offsets: off_c = min(prefix, gen), cnt_c = min(prefix+cnt, gen) - off_c
__global__ void k_offsets(uint32_t* off, uint32_t* cnt, const uint32_t* blockSum, uint32_t np, uint32_t gen) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= np) return;
  unsigned long long pre = (unsigned long long)blockSum[p / kScanBlock] + off[p];
  unsigned long long a = pre < gen ? pre : gen;
  unsigned long long e = pre + cnt[p];
  unsigned long long b = e < gen ? e : gen;
  off[p] = (uint32_t)a;
  cnt[p] = (uint32_t)(b - a);
}

// one camera path per budgeted sample; slot s belongs to the last pixel whose
// offset is <= s (pixels without samples share their successor's offset).
__global__ void k_gen_adapt(FrameArgs a, RenderBuffers b, const uint32_t* __restrict__ off,
                            const uint32_t* __restrict__ cnt) {
  using namespace gb;
  const uint32_t total = b.ctr->wave[0];
  const uint32_t np = a.width * a.height;
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < total; s += stride) {
    uint32_t lo = 0, hi = np;  // first index with off > s
    while (lo < hi) {
      uint32_t mid = (lo + hi) >> 1;
      if (off[mid] <= s)
        lo = mid + 1;
      else
        hi = mid;
    }
    const uint32_t p = lo - 1;
    const uint32_t k = s - off[p];
    const uint32_t x = p % a.width, y = p / a.width;
    float u[4];
    draw4(a.key0, a.key1, p, a.frame, kCamera, 0, k, 0, u);
    const float W = a.W, H = a.H, th = a.tanHalf;
    float cu = ((((2.f * ((float)x + 0.5f)) / W) - 1.f) * th * W) / H;
    float cv = (((2.f * ((float)y + 0.5f)) / H) - 1.f) * th;
    float au = cu + ((u[0] - 0.5f) / H) * th;
    float av = cv + ((u[1] - 0.5f) / H) * th;
    f3 R = mk(a.camRight[0], a.camRight[1], a.camRight[2]);
    f3 U = mk(a.camUp[0], a.camUp[1], a.camUp[2]);
    f3 D = mk(a.camDir[0], a.camDir[1], a.camDir[2]);
    f3 dir = normalize((R * au + U * av) + D);
    Wave w = b.wave[0];
    w.o[s] = make_float4(a.camPos[0], a.camPos[1], a.camPos[2], __uint_as_float(s));
    w.d[s] = make_float4(dir.x, dir.y, dir.z, __uint_as_float(p));
    w.thr[s] = make_float4(1.f, 1.f, 1.f, 0.f);
    w.smp[s] = make_float4(0.f, 0.f, 0.f, 0.f);
    b.res[s] = make_float4(0.f, 0.f, 0.f, 0.f);
    b.slotPix[s] = p;
    b.slotSmp[s] = k;
    b.gbuf[3 * (size_t)s] = make_float4(0.f, 0.f, 0.f, 0.f);
    b.gbuf[3 * (size_t)s + 1] = make_float4(0.f, 0.f, 0.f, 0.f);
    b.gbuf[3 * (size_t)s + 2] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
}

// Per-pixel sums of the budgeted samples, then the running means.  The sum
// order is a fixed function of the pixel's sample count c, so results do not
// depend on timing (the reference adds with float atomics in arbitrary
// order): P(c) partial sums -- partial l adds samples l, l+P, l+2P, ... in
// slot order -- combined by a butterfly (x[l] += x[l ^ m] for m = P/2 .. 1),
// with P = 8 for c <= 64, 32 for c <= 4096 and 1024 above.  The budget
// spreads one frame's W*H samples very unevenly (a firefly pixel can take
// tens of thousands), so each range has its own kernel: one thread per pixel
// for c <= 8 (the same eight partials, combined in the butterfly's order),
// eight lanes per pixel for c <= 64, a warp per pixel for the medium ones, a
// 1024-thread CTA per pixel for the heaviest; the last three take their
// pixels from lists the first kernel appends to.
constexpr uint32_t kAccumSmall = 64, kAccumMid = 4096;
constexpr uint32_t kHugeThreads = 1024;

template <bool kMoments>
__device__ __forceinline__ void accum_sample(float4 r, float4 g0, float4 g1, float4 g2, float* v, uint32_t& tN) {
  if (isinf(r.x) || isinf(r.y) || isinf(r.z)) return;
  uint32_t n = __float_as_uint(r.w);
  float fn = (float)n;
  v[0] = v[0] + r.x; v[1] = v[1] + r.y; v[2] = v[2] + r.z;
  v[3] = v[3] + g0.x * fn; v[4] = v[4] + g0.y * fn; v[5] = v[5] + g0.z * fn;
  v[6] = v[6] + g1.x * fn; v[7] = v[7] + g1.y * fn; v[8] = v[8] + g1.z * fn;
  v[9] = v[9] + g2.x * fn; v[10] = v[10] + g2.y * fn; v[11] = v[11] + g2.z * fn;
  if (kMoments) {  // second moments for the learned allocator's features
    v[12] = v[12] + (r.x * r.x) / fn; v[13] = v[13] + (r.y * r.y) / fn; v[14] = v[14] + (r.z * r.z) / fn;
  }
  tN += n;
}

// Partial l of pixel samples [o, o + c): samples l, l + P, l + 2P, ... added
// one after another in that order.  The loads of kBatch samples are issued
// before their additions (the order of the additions is unchanged), so a
// lane with a long run -- a heavy pixel's warp or CTA lanes walk up to a few
// hundred samples each -- keeps kBatch loads in flight instead of one (2 in
// the 1024-thread kernel, whose 64 registers a thread do not hold four).
template <bool kMoments, int kBatch = 4>
__device__ __forceinline__ void accum_partials(const RenderBuffers& b, uint32_t o, uint32_t c, uint32_t l, uint32_t P,
                                               float* v, uint32_t& tN) {
  const uint32_t end = o + c;
  uint32_t s = o + l;
  for (; s + (kBatch - 1) * P < end; s += kBatch * P) {
    float4 r[kBatch], g0[kBatch], g1[kBatch], g2[kBatch];
#pragma unroll
    for (int j = 0; j < kBatch; j++) {
      const size_t q = (size_t)s + (size_t)j * P;
      r[j] = b.res[q];
      g0[j] = b.gbuf[3 * q];
      g1[j] = b.gbuf[3 * q + 1];
      g2[j] = b.gbuf[3 * q + 2];
    }
#pragma unroll
    for (int j = 0; j < kBatch; j++) accum_sample<kMoments>(r[j], g0[j], g1[j], g2[j], v, tN);
  }
  for (; s < end; s += P)
    accum_sample<kMoments>(b.res[s], b.gbuf[3 * (size_t)s], b.gbuf[3 * (size_t)s + 1], b.gbuf[3 * (size_t)s + 2], v,
                           tN);
}

// running means of pixel p from its summed samples (one thread)
template <bool kMoments>
__device__ __forceinline__ void accum_write(const FrameArgs& a, const RenderBuffers& b, uint32_t p, const float* v,
                                            uint32_t tN, float* result, uint32_t* sampleN, float* gpos,
                                            float* gnorm, float* gdiff) {
  float* q = result + 3 * (size_t)p;
  float* P = gpos + 3 * (size_t)p;
  float* Nn = gnorm + 3 * (size_t)p;
  float* Dd = gdiff + 3 * (size_t)p;
  uint32_t N = sampleN[p];
  if (a.frame == 0) {
    N = 0;
    for (int k = 0; k < 3; k++) q[k] = P[k] = Nn[k] = Dd[k] = 0.f;
  }
  const uint32_t nn = tN + N;
  if (nn > N) {
    const float rInf = 1.f / (float)nn, oInf = (float)N * rInf;
    if (kMoments) {
      float* m = b.m2 + 3 * (size_t)p;
      for (int k = 0; k < 3; k++) m[k] = N ? rInf * v[12 + k] + oInf * m[k] : rInf * v[12 + k];
    }
    for (int k = 0; k < 3; k++) {
      q[k] = fmaxf(rInf * v[k] + oInf * q[k], 0.f);
      P[k] = rInf * v[3 + k] + oInf * P[k];
      Nn[k] = rInf * v[6 + k] + oInf * Nn[k];
      Dd[k] = rInf * v[9 + k] + oInf * Dd[k];
    }
    N = nn;
  }
  sampleN[p] = N;
}

// The eight-lane partial of one sample (lane l holds sample l when c <= 8):
// 0 + its contribution, or 0 when absent or infinite (accum_partials' terms)
template <bool kMoments>
__device__ __forceinline__ void accum_lane(const RenderBuffers& b, uint32_t s, bool present, float* v,
                                           uint32_t& tN) {
  for (int k = 0; k < (kMoments ? 15 : 12); k++) v[k] = 0.f;
  if (present)
    accum_sample<kMoments>(b.res[s], b.gbuf[3 * (size_t)s], b.gbuf[3 * (size_t)s + 1], b.gbuf[3 * (size_t)s + 2], v,
                           tN);
}

template <int N>
__device__ __forceinline__ void add_into(float* x, const float* y) {
#pragma unroll
  for (int k = 0; k < N; k++) x[k] = x[k] + y[k];
}

// Pixels with at most 8 samples, one thread each (most pixels of a budgeted
// frame hold 0-2): the sum of the eight lane partials x_0..x_7 in the
// eight-lane butterfly's order, ((x0 + x4) + (x2 + x6)) + ((x1 + x5) + (x3 +
// x7)), so the result is that pass's to the bit.  Pixels with more samples
// are listed for the eight-lane, warp and CTA passes.
template <bool kMoments>
__global__ void k_accum_one(FrameArgs a, RenderBuffers b, AdaptBuffers ab, float* result, uint32_t* sampleN,
                            float* gpos, float* gnorm, float* gdiff) {
  constexpr int NV = kMoments ? 15 : 12;
  const uint32_t np = a.width * a.height;
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= np) return;
  const uint32_t c = ab.cnt[p];
  if (c > 8u) {
    if (c <= kAccumSmall)
      ab.list8[atomicAdd(&b.ctr->heavySmall, 1u)] = p;
    else if (c <= kAccumMid)
      ab.heavy[atomicAdd(&b.ctr->heavyMid, 1u)] = p;
    else
      ab.heavy[np - 1u - atomicAdd(&b.ctr->heavyHuge, 1u)] = p;
    return;
  }
  const uint32_t o = c ? ab.off[p] : 0u;
  uint32_t tN = 0;
  float v[15], hi[NV], t[NV], u[NV];
  // lanes {0,4} + {2,6} -> v; lanes {1,5} + {3,7} -> hi
  const uint32_t order[2][4] = {{0u, 4u, 2u, 6u}, {1u, 5u, 3u, 7u}};
#pragma unroll
  for (int h = 0; h < 2; h++) {
    float* dst = h ? hi : v;
    accum_lane<kMoments>(b, o + order[h][0], order[h][0] < c, dst, tN);
    accum_lane<kMoments>(b, o + order[h][1], order[h][1] < c, t, tN);
    add_into<NV>(dst, t);
    accum_lane<kMoments>(b, o + order[h][2], order[h][2] < c, t, tN);
    accum_lane<kMoments>(b, o + order[h][3], order[h][3] < c, u, tN);
    add_into<NV>(t, u);
    add_into<NV>(dst, t);
  }
  add_into<NV>(v, hi);
  accum_write<kMoments>(a, b, p, v, tN, result, sampleN, gpos, gnorm, gdiff);
}

// listed pixels with 9..64 samples, eight lanes each
template <bool kMoments>
__global__ void k_accum(FrameArgs a, RenderBuffers b, AdaptBuffers ab, float* result, uint32_t* sampleN, float* gpos,
                        float* gnorm, float* gdiff) {
  const uint32_t n = b.ctr->heavySmall;
  const uint32_t gid = blockIdx.x * blockDim.x + threadIdx.x, l = gid & 7u;
  const uint32_t groups = (gridDim.x * blockDim.x) >> 3;
  // every lane of a warp runs the same number of rounds (the shuffles need all 32)
  const uint32_t rounds = (n + groups - 1) / groups;
  for (uint32_t k = 0; k < rounds; k++) {
    const uint32_t i = (gid >> 3) + k * groups;
    const uint32_t p = i < n ? ab.list8[i] : 0u;
    const uint32_t c = i < n ? ab.cnt[p] : 0u;
    float v[15] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    uint32_t tN = 0;
    if (c) accum_partials<kMoments>(b, ab.off[p], c, l, 8, v, tN);
    for (int q = 0; q < (kMoments ? 15 : 12); q++)
      for (int m = 4; m > 0; m >>= 1) v[q] = v[q] + __shfl_xor_sync(0xffffffffu, v[q], m);
    for (int m = 4; m > 0; m >>= 1) tN += __shfl_xor_sync(0xffffffffu, tN, m);
    if (l == 0 && i < n) accum_write<kMoments>(a, b, p, v, tN, result, sampleN, gpos, gnorm, gdiff);
  }
}

// medium pixels: a warp each, 32 partials
template <bool kMoments>
__global__ void k_accum_mid(FrameArgs a, RenderBuffers b, AdaptBuffers ab, float* result, uint32_t* sampleN,
                            float* gpos, float* gnorm, float* gdiff) {
  const uint32_t nMid = b.ctr->heavyMid;
  const uint32_t lane = threadIdx.x & 31u;
  for (uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < nMid; w += (gridDim.x * blockDim.x) >> 5) {
    const uint32_t p = ab.heavy[w];
    float v[15] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    uint32_t tN = 0;
    accum_partials<kMoments>(b, ab.off[p], ab.cnt[p], lane, 32, v, tN);
    for (int k = 0; k < (kMoments ? 15 : 12); k++)
      for (int m = 16; m > 0; m >>= 1) v[k] = v[k] + __shfl_xor_sync(0xffffffffu, v[k], m);
    for (int m = 16; m > 0; m >>= 1) tN += __shfl_xor_sync(0xffffffffu, tN, m);
    if (lane == 0) accum_write<kMoments>(a, b, p, v, tN, result, sampleN, gpos, gnorm, gdiff);
  }
}

// the heaviest pixels: a 1024-thread CTA each, 1024 partials; butterfly steps
// m >= 32 exchange through shared memory, the rest through shuffles
template <bool kMoments>
__global__ void __launch_bounds__(kHugeThreads) k_accum_huge(FrameArgs a, RenderBuffers b, AdaptBuffers ab,
                                                             float* result, uint32_t* sampleN, float* gpos,
                                                             float* gnorm, float* gdiff) {
  __shared__ float xs[kHugeThreads];
  __shared__ uint32_t ns[kHugeThreads];
  const uint32_t np = a.width * a.height;
  const uint32_t nHuge = b.ctr->heavyHuge;
  const uint32_t t = threadIdx.x;
  for (uint32_t h = blockIdx.x; h < nHuge; h += gridDim.x) {
    const uint32_t p = ab.heavy[np - 1u - h];
    float v[15] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    uint32_t tN = 0;
    accum_partials<kMoments, 2>(b, ab.off[p], ab.cnt[p], t, kHugeThreads, v, tN);
    for (int k = 0; k < (kMoments ? 15 : 12); k++) {
      float x = v[k];
      for (uint32_t m = kHugeThreads / 2; m >= 32; m >>= 1) {
        xs[t] = x;
        __syncthreads();
        const float y = xs[t ^ m];
        __syncthreads();
        x = x + y;
      }
      for (int m = 16; m > 0; m >>= 1) x = x + __shfl_xor_sync(0xffffffffu, x, m);
      v[k] = x;
    }
    ns[t] = tN;
    __syncthreads();
    if (t == 0) {
      uint32_t total = 0;
      for (uint32_t i = 0; i < kHugeThreads; i++) total += ns[i];
      accum_write<kMoments>(a, b, p, v, total, result, sampleN, gpos, gnorm, gdiff);
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Binary allocator.  The reference runs its window search as a host loop
// with a D2H count per pass; here one cooperative kernel (all blocks
// resident) runs every pass, separated by a grid barrier.  The barrier spins
// on a generation word with an iteration limit: on timeout it sets bit 2 of
// DevCounters::errFlags and the kernel returns (the host reports
// GBPT_ERR_TIMEOUT).
// coop layout: [0] barrier count, [1] barrier generation, [2] passes,
// [16, 16+G) per-block values, [4096, 4096+80) paths per pass.
constexpr uint32_t kCoopBlocks = 16, kCoopPass = 4096, kMaxPasses = 64;
constexpr unsigned long long kBarrierSpins = 1ull << 24;

__device__ __forceinline__ bool grid_barrier(uint32_t* coop, uint32_t nblocks, DevCounters* ctr) {
  __shared__ uint32_t ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile uint32_t* gen = coop + 1;
    const uint32_t g = *gen;
    __threadfence();
    const uint32_t arrived = atomicAdd(coop, 1u);
    ok = 1u;
    if (arrived == nblocks - 1) {
      coop[0] = 0;
      __threadfence();
      atomicAdd(coop + 1, 1u);
    } else {
      unsigned long long spins = 0;
      while (*gen == g) {
        if (++spins > kBarrierSpins) {
          atomicOr(&ctr->errFlags, 4u);
          ok = 0u;
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return ok != 0u;
}

// Failure-detection self-test: a grid barrier that waits for one block more
// than are launched, so nobody releases it and every block's bounded wait
// runs out (errFlags bit 2, as in the binary allocator).
__global__ void k_barrier_selftest(uint32_t* coop, uint32_t nblocks, DevCounters* ctr) {
  grid_barrier(coop, nblocks + 1u, ctr);
}

__device__ __forceinline__ uint32_t block_sum(uint32_t v, uint32_t* ws) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = v;
  __syncthreads();
  uint32_t t = 0;
  for (uint32_t w = 0; w < (blockDim.x + 31) / 32; w++) t += ws[w];
  return t;
}

__device__ __forceinline__ bool bin_accept(const FrameArgs& a, const float* err, uint32_t p, uint32_t pass, float mid,
                                           float minProb) {
  gb::u4 r = gb::philox(gb::u4{p, a.frame, (uint32_t)gb::kBinaryAccept << 24, pass}, a.key0, a.key1);
  return !(gb::u01(r.a) * mid > fmaxf(err[p], minProb));
}

__global__ void __launch_bounds__(256) k_bin_search(FrameArgs a, RenderBuffers b, const float* __restrict__ err,
                                                    uint32_t np, uint32_t D, float minProb, uint32_t* coop) {
  __shared__ uint32_t ws[32];
  __shared__ float wf[32];
  const uint32_t G = gridDim.x;
  const uint32_t per = (np + G - 1) / G;
  const uint32_t lo = min(np, blockIdx.x * per), hi = min(np, lo + per);
  uint32_t* blockVal = coop + kCoopBlocks;
  uint32_t* passLen = coop + kCoopPass;
  // max error (NaN ignored, as the reference's thrust::maximum from 0)
  float m = 0.f;
  for (uint32_t p = lo + threadIdx.x; p < hi; p += blockDim.x) m = fmaxf(m, err[p]);
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) wf[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.f;
    for (uint32_t w = 0; w < (blockDim.x + 31) / 32; w++) t = fmaxf(t, wf[w]);
    blockVal[blockIdx.x] = __float_as_uint(t);
  }
  if (!grid_barrier(coop, G, b.ctr)) return;
  float maxE = 0.f;
  for (uint32_t k = 0; k < G; k++) maxE = fmaxf(maxE, __uint_as_float(((volatile uint32_t*)blockVal)[k]));
  float left = 0.f, right = maxE * 2.f;
  const float desired = (float)np / (float)D;
  uint32_t accum = 0, passes = 0;
  if (!grid_barrier(coop, G, b.ctr)) return;  // every block has read blockVal
  for (uint32_t pass = 0; accum < np && pass < kMaxPasses; pass++) {
    const float mid = (left + right) * 0.5f;
    uint32_t c = 0;
    for (uint32_t p = lo + threadIdx.x; p < hi; p += blockDim.x) c += bin_accept(a, err, p, pass, mid, minProb) ? 1u : 0u;
    c = block_sum(c, ws);
    if (threadIdx.x == 0) blockVal[blockIdx.x] = c;
    if (!grid_barrier(coop, G, b.ctr)) return;
    uint32_t total = 0, before = 0;
    for (uint32_t k = 0; k < G; k++) {
      const uint32_t v = ((volatile uint32_t*)blockVal)[k];
      if (k < blockIdx.x) before += v;
      total += v;
    }
    const uint32_t take = min(np - accum, total);
    // write accepted pixels of this block in pixel order (stable compaction)
    uint32_t rank = before;
    for (uint32_t base = lo; base < hi; base += blockDim.x) {
      const uint32_t p = base + threadIdx.x;
      const bool acc = p < hi && bin_accept(a, err, p, pass, mid, minProb);
      const uint32_t bal = __ballot_sync(0xffffffffu, acc);
      uint32_t lm;
      asm("mov.u32 %0, %%lanemask_lt;" : "=r"(lm));
      __syncthreads();
      if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = __popc(bal);
      __syncthreads();
      uint32_t wbefore = 0, tile = 0;
      for (uint32_t w = 0; w < (blockDim.x + 31) / 32; w++) {
        if (w < (threadIdx.x >> 5)) wbefore += ws[w];
        tile += ws[w];
      }
      if (acc) {
        const uint32_t r = rank + wbefore + __popc(bal & lm);
        if (r < take) {
          b.slotPix[accum + r] = p;
          b.slotSmp[accum + r] = pass;
        }
      }
      rank += tile;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) passLen[pass] = take;
    accum += take;
    passes = pass + 1;
    if (!grid_barrier(coop, G, b.ctr)) return;  // blockVal is reused by the next pass
    if (take == 0) break;
    if ((float)take < desired)
      right = mid;
    else if ((float)take > desired)
      left = mid;
  }
  if (accum < np) {  // leftover slots: pixel ids 0, 1, ... (pt_fillTempAdapPathQueue_kernel)
    const uint32_t fill = np - accum;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < fill; k += G * blockDim.x) {
      b.slotPix[accum + k] = k;
      b.slotSmp[accum + k] = passes;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) passLen[passes] = fill;
    passes++;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    coop[2] = passes;
    b.ctr->wave[0] = np;
    b.ctr->paths = np;
    b.ctr->fetchT = 0;
    b.ctr->carryN[0] = b.ctr->carryN[1] = b.ctr->carryN[2] = 0;
    b.ctr->fetchTail = 0;
    b.ctr->tailAt = 0xFFFFFFFFu;
  }
}

// camera path for queue entry s (pixel slotPix[s], sample slotSmp[s])
__global__ void k_gen_queue(FrameArgs a, RenderBuffers b, uint32_t np) {
  using namespace gb;
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= np) return;
  const uint32_t p = b.slotPix[s], k = b.slotSmp[s];
  const uint32_t x = p % a.width, y = p / a.width;
  float u[4];
  draw4(a.key0, a.key1, p, a.frame, kCamera, 0, k, 0, u);
  const float W = a.W, H = a.H, th = a.tanHalf;
  float cu = ((((2.f * ((float)x + 0.5f)) / W) - 1.f) * th * W) / H;
  float cv = (((2.f * ((float)y + 0.5f)) / H) - 1.f) * th;
  float au = cu + ((u[0] - 0.5f) / H) * th;
  float av = cv + ((u[1] - 0.5f) / H) * th;
  f3 dir = normalize((mk(a.camRight[0], a.camRight[1], a.camRight[2]) * au +
                      mk(a.camUp[0], a.camUp[1], a.camUp[2]) * av) +
                     mk(a.camDir[0], a.camDir[1], a.camDir[2]));
  Wave w = b.wave[0];
  w.o[s] = make_float4(a.camPos[0], a.camPos[1], a.camPos[2], __uint_as_float(s));
  w.d[s] = make_float4(dir.x, dir.y, dir.z, __uint_as_float(p));
  w.thr[s] = make_float4(1.f, 1.f, 1.f, 0.f);
  w.smp[s] = make_float4(0.f, 0.f, 0.f, 0.f);
  b.res[s] = make_float4(0.f, 0.f, 0.f, 0.f);
  b.gbuf[3 * (size_t)s] = make_float4(0.f, 0.f, 0.f, 0.f);
  b.gbuf[3 * (size_t)s + 1] = make_float4(0.f, 0.f, 0.f, 0.f);
  b.gbuf[3 * (size_t)s + 2] = make_float4(0.f, 0.f, 0.f, 0.f);
}

// running means, pass by pass (a pixel appears at most once per pass)
__global__ void __launch_bounds__(256) k_bin_apply(FrameArgs a, RenderBuffers b, uint32_t* coop, float* result,
                                                   uint32_t* sampleN, float* gpos, float* gnorm, float* gdiff) {
  const uint32_t G = gridDim.x;
  const uint32_t passes = coop[2];
  const uint32_t* passLen = coop + kCoopPass;
  float* planes[3] = {gpos, gnorm, gdiff};
  uint32_t start = 0;
  for (uint32_t c = 0; c < passes; c++) {
    const uint32_t len = passLen[c];
    for (uint32_t s = start + blockIdx.x * blockDim.x + threadIdx.x; s < start + len; s += G * blockDim.x) {
      const uint32_t p = b.slotPix[s];
      const float4 r = b.res[s];
      const uint32_t n = __float_as_uint(r.w);
      if (n == 0) continue;
      if (a.frame == 0) sampleN[p] = 0;
      const uint32_t old = sampleN[p];
      const uint32_t nn = old + n;
      if (!(nn > old)) continue;
      if (isinf(r.x) || isinf(r.y) || isinf(r.z)) continue;
      const float rInf = 1.f / (float)nn, oInf = (float)old * rInf;
      float* q = result + 3 * (size_t)p;
      q[0] = fmaxf(rInf * r.x + oInf * q[0], 0.f);
      q[1] = fmaxf(rInf * r.y + oInf * q[1], 0.f);
      q[2] = fmaxf(rInf * r.z + oInf * q[2], 0.f);
      sampleN[p] = nn;
      const float fn = (float)n;
      for (int k = 0; k < 3; k++) {
        const float4 g = b.gbuf[3 * (size_t)s + k];
        float* o = planes[k] + 3 * (size_t)p;
        o[0] = rInf * (g.x * fn) + oInf * o[0];
        o[1] = rInf * (g.y * fn) + oInf * o[1];
        o[2] = rInf * (g.z * fn) + oInf * o[2];
      }
    }
    start += len;
    if (!grid_barrier(coop, G, b.ctr)) return;
  }
}

__global__ void k_fmath(int which, const float* x, uint32_t n, float* out) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float s, c, v = x[i], r = 0.f;
  switch (which) {
    case 0: gb::sincos_p(v, &s, &c); r = s; break;
    case 1: gb::sincos_p(v, &s, &c); r = c; break;
    case 2: r = gb::exp_p(v); break;
    case 3: r = gb::sqrt_rd_(v); break;
    case 4: r = gb::pow5(v); break;
    case 5: r = exp_nonpos_p(v); break;
  }
  out[i] = r;
}

__global__ void k_philox(const uint32_t* ctr, uint32_t n, uint32_t k0, uint32_t k1, uint32_t* out) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  gb::u4 r = gb::philox(gb::u4{ctr[4 * i], ctr[4 * i + 1], ctr[4 * i + 2], ctr[4 * i + 3]}, k0, k1);
  out[4 * i] = r.a;
  out[4 * i + 1] = r.b;
  out[4 * i + 2] = r.c;
  out[4 * i + 3] = r.d;
}

}  // namespace

uint32_t adapt_scan_blocks(uint32_t np) { return (np + kScanBlock - 1) / kScanBlock; }
uint32_t adapt_reduce_blocks(uint32_t np) { return (np + kReduceBlock - 1) / kReduceBlock; }

// 2 d d, the divisor of a feature plane's weight; when it is a power of two
// whose reciprocal is a normal float, -1 / (2 d d) instead (neg_ratio then
// multiplies; the default position and normal deltas, 1 and 0.25, give 2 and
// 1/8).  Measured on the hall's 1280x720 radius-4 filter: 0.381 -> 0.310 ms per pass.
float bilateral_c2(float d) {
  const float c2 = (2.f * d) * d;
  int e = 0;
  const float m = std::frexp(c2, &e);
  if (m == 0.5f && e - 1 >= -126 && e - 1 <= 126) return -1.f / c2;
  return c2;
}

cudaError_t launch_bilateral(const float* color, const float* pos, const float* norm, const float* emit, uint32_t W,
                             uint32_t H, float ceud, float peud, float neud, float eeud, uint32_t radius,
                             const float* g, float* out, cudaStream_t st) {
  const float cc2 = bilateral_c2(ceud), pc2 = bilateral_c2(peud), nc2 = bilateral_c2(neud), ec2 = bilateral_c2(eeud);
  dim3 grid((W + kTile - 1) / kTile, (H + kTile - 1) / kTile), block(kTile, kTile);
  const int r = (int)radius;
  const int T = kTile + 2 * r;
  const size_t smem = ((size_t)(2 * r + 1 + 3) / 4 + 3 * (size_t)T * T) * sizeof(float4);
  if (smem <= 200 * 1024) {
    auto tile = [&](auto kern) {
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      kern<<<grid, block, smem, st>>>(color, pos, norm, emit, W, H, cc2, pc2, nc2, ec2, r, g, out);
    };
    if (emit) {
      if (r == 4) tile(k_bilateral_tile<true, 4>);
      else if (r == 5) tile(k_bilateral_tile<true, 5>);
      else tile(k_bilateral_tile<true, 0>);
    } else {
      if (r == 4) tile(k_bilateral_tile<false, 4>);
      else if (r == 5) tile(k_bilateral_tile<false, 5>);
      else tile(k_bilateral_tile<false, 0>);
    }
  } else if (emit) {
    k_bilateral_direct<true><<<grid, block, 0, st>>>(color, pos, norm, emit, W, H, cc2, pc2, nc2, ec2, r, g, out);
  } else {
    k_bilateral_direct<false><<<grid, block, 0, st>>>(color, pos, norm, emit, W, H, cc2, pc2, nc2, ec2, r, g, out);
  }
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_adapt_error(const FrameArgs& a, const AdaptBuffers& ab, const float* result,
                               const uint32_t* sampleN, uint32_t desired, cudaStream_t st) {
  const uint32_t np = a.width * a.height;
  k_error<<<adapt_reduce_blocks(np), kReduceBlock, 0, st>>>(ab.filtered, result, sampleN, np, desired, ab.err,
                                                             ab.partial);
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_adapt_alloc(const FrameArgs& a, const RenderBuffers& b, const AdaptBuffers& ab, cudaStream_t st) {
  const uint32_t np = a.width * a.height;
  const uint32_t nr = adapt_reduce_blocks(np), ns = adapt_scan_blocks(np);
  k_reduce_final<<<1, 1024, 0, st>>>(ab.partial, nr, b.ctr);
  k_budget<<<ns, kScanBlock, 0, st>>>(ab.err, np, b.ctr, ab.cnt, ab.off, ab.blockSum);
  k_scan_blocks<<<1, 1024, 0, st>>>(ab.blockSum, ns, np, b.ctr);
  k_offsets<<<(np + 255) / 256, 256, 0, st>>>(ab.off, ab.cnt, ab.blockSum, np, np);
  k_gen_adapt<<<sm_count() * 8, 256, 0, st>>>(a, b, ab.off, ab.cnt);
  note_launches(5);
  return cudaGetLastError();
}

cudaError_t launch_adapt_budget(const FrameArgs& a, const RenderBuffers& b, const AdaptBuffers& ab,
                                const float* result, const uint32_t* sampleN, uint32_t desired, cudaStream_t st) {
  cudaError_t e = launch_adapt_error(a, ab, result, sampleN, desired, st);
  return e == cudaSuccess ? launch_adapt_alloc(a, b, ab, st) : e;
}

// ---------------------------------------------------------------------------
// Learned allocator.  Features of one 8x8 tile (edge tiles: the pixels that
// exist), one warp per tile, lane l covering pixels l and l + 32:
//   0-2   log(1 + mean colour)             3-5   log(1 + 100 * mean variance of the pixel means)
//   6-8   mean first-hit albedo            9-11  mean first-hit normal
//   12    log(1 + mean first-hit distance) 13-20 fraction of paths that ended after 0..7+ hits
//   21    log2(1 + mean samples per pixel) 22/23 log(1 + 1000 * mean / max heuristic error)
// The variance of a pixel mean is max(m2 - mean^2, 0) / n with m2 the running
// mean of (path sum)^2 / (path count).
__global__ void k_tile_features(FrameArgs a, RenderBuffers b, AdaptBuffers ab, const float* __restrict__ result,
                                const uint32_t* __restrict__ sampleN, const float* __restrict__ gpos,
                                const float* __restrict__ gnorm, const float* __restrict__ gdiff,
                                uint32_t nTiles) {
  const uint32_t tile = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t lane = threadIdx.x & 31;
  if (tile >= nTiles) return;  // warp-uniform
  const uint32_t tx = tile % a.tilesX, ty = tile / a.tilesX;
  float s[16];
  for (int k = 0; k < 16; k++) s[k] = 0.f;
  float emax = 0.f;
  for (uint32_t h = 0; h < 2; h++) {
    const uint32_t k = lane + 32u * h;
    const uint32_t x = tx * 8u + (k & 7u), y = ty * 8u + (k >> 3);
    if (x >= a.width || y >= a.height) continue;
    const size_t p = (size_t)y * a.width + x;
    const float n = (float)sampleN[p];
    for (int c = 0; c < 3; c++) {
      const float mu = result[3 * p + c];
      const float var = n > 0.f ? fmaxf(b.m2[3 * p + c] - mu * mu, 0.f) / n : 0.f;
      s[c] += mu;
      s[3 + c] += var;
      s[6 + c] += gdiff[3 * p + c];
      s[9 + c] += gnorm[3 * p + c];
    }
    const float dx = gpos[3 * p] - a.camPos[0], dy = gpos[3 * p + 1] - a.camPos[1], dz = gpos[3 * p + 2] - a.camPos[2];
    s[12] += sqrtf(dx * dx + dy * dy + dz * dz);
    s[13] += n;
    const float e = ab.err[p];
    s[14] += e;
    emax = fmaxf(emax, e);
    s[15] += 1.f;
  }
  for (int k = 0; k < 16; k++)
    for (int o = 16; o > 0; o >>= 1) s[k] += __shfl_xor_sync(0xffffffffu, s[k], o);
  for (int o = 16; o > 0; o >>= 1) emax = fmaxf(emax, __shfl_xor_sync(0xffffffffu, emax, o));
  if (lane >= 8) return;
  const uint32_t* hp = b.hist + tile * 8u;
  uint32_t hsum = 0;
  for (int k = 0; k < 8; k++) hsum += hp[k];
  float* f = ab.feat + (size_t)tile * kFeatures;
  const float inv = 1.f / fmaxf(s[15], 1.f);
  if (lane == 0) {
    for (int c = 0; c < 3; c++) {
      f[c] = log1pf(fmaxf(s[c] * inv, 0.f));
      f[3 + c] = log1pf(100.f * s[3 + c] * inv);
      f[6 + c] = s[6 + c] * inv;
      f[9 + c] = s[9 + c] * inv;
    }
    f[12] = log1pf(s[12] * inv);
    f[21] = log2f(1.f + s[13] * inv);
    f[22] = log1pf(1000.f * s[14] * inv);
    f[23] = log1pf(1000.f * emax);
    ab.tileErr[tile] = s[14];
  }
  f[13 + lane] = hsum ? (float)hp[lane] / (float)hsum : 0.f;
}

// The network predicts pred = 1/2 log(MSE_t) of the tile's current image
// (up to a constant); one more sample per pixel lowers the tile's error
// V_t / n by about V_t / n^2 = MSE_t / n, so the tile's weight this frame is
// w = exp(2 pred) / n (n: the tile's mean samples per pixel, from feature 21).
// e'_p = w * e_p / (sum of e over the tile), or w / pixels when the tile's
// heuristic error is zero; FP64 partial sums as k_error's.
__global__ void __launch_bounds__(kReduceBlock) k_mlp_alloc(FrameArgs a, AdaptBuffers ab, uint32_t np) {
  __shared__ double ws[kReduceBlock / 32];
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  double v = 0.0;
  if (p < np) {
    const uint32_t x = p % a.width, y = p / a.width;
    const uint32_t tile = (y >> 3) * a.tilesX + (x >> 3);
    const float nMean = exp2f(ab.feat[(size_t)tile * kFeatures + 21]) - 1.f;
    const float w = expf(fminf(fmaxf(2.f * ab.pred[tile], -60.f), 60.f)) / fmaxf(nMean, 1.f);
    const float S = ab.tileErr[tile];
    const uint32_t tw = min(8u, a.width - (x & ~7u)), th = min(8u, a.height - (y & ~7u));
    const float e = S > 0.f ? w * (ab.err[p] / S) : w / (float)(tw * th);
    ab.err[p] = e;
    v = (double)e;
  }
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s2 = 0.0;
    for (int w = 0; w < kReduceBlock / 32; w++) s2 += ws[w];
    ab.partial[blockIdx.x] = s2;
  }
}

cudaError_t launch_tile_features(const FrameArgs& a, const RenderBuffers& b, const AdaptBuffers& ab,
                                 const float* result, const uint32_t* sampleN, const float* gpos, const float* gnorm,
                                 const float* gdiff, cudaStream_t st) {
  const uint32_t nTiles = a.tilesX * ((a.height + 7) / 8);
  k_tile_features<<<(nTiles * 32 + 255) / 256, 256, 0, st>>>(a, b, ab, result, sampleN, gpos, gnorm, gdiff, nTiles);
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_mlp_alloc(const FrameArgs& a, const AdaptBuffers& ab, cudaStream_t st) {
  const uint32_t np = a.width * a.height;
  k_mlp_alloc<<<adapt_reduce_blocks(np), kReduceBlock, 0, st>>>(a, ab, np);
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_adapt_accum(const FrameArgs& a, const RenderBuffers& b, const AdaptBuffers& ab, float* result,
                               uint32_t* sampleN, float* gpos, float* gnorm, float* gdiff, cudaStream_t st) {
  const uint32_t np = a.width * a.height;
  const uint32_t g = (np + 255) / 256;
  static_assert(offsetof(DevCounters, heavySmall) == offsetof(DevCounters, heavyMid) + 8, "list counters");
  cudaError_t e = cudaMemsetAsync(&b.ctr->heavyMid, 0, 3 * sizeof(uint32_t), st);
  if (e != cudaSuccess) return e;
  const uint32_t gm = (uint32_t)sm_count() * 8, gh = (uint32_t)sm_count();
  if (a.moments) {
    k_accum_one<true><<<g, 256, 0, st>>>(a, b, ab, result, sampleN, gpos, gnorm, gdiff);
    k_accum<true><<<gm, 256, 0, st>>>(a, b, ab, result, sampleN, gpos, gnorm, gdiff);
    k_accum_mid<true><<<gm, 256, 0, st>>>(a, b, ab, result, sampleN, gpos, gnorm, gdiff);
    k_accum_huge<true><<<gh, kHugeThreads, 0, st>>>(a, b, ab, result, sampleN, gpos, gnorm, gdiff);
  } else {
    k_accum_one<false><<<g, 256, 0, st>>>(a, b, ab, result, sampleN, gpos, gnorm, gdiff);
    k_accum<false><<<gm, 256, 0, st>>>(a, b, ab, result, sampleN, gpos, gnorm, gdiff);
    k_accum_mid<false><<<gm, 256, 0, st>>>(a, b, ab, result, sampleN, gpos, gnorm, gdiff);
    k_accum_huge<false><<<gh, kHugeThreads, 0, st>>>(a, b, ab, result, sampleN, gpos, gnorm, gdiff);
  }
  note_launches(4);
  return cudaGetLastError();
}

cudaError_t launch_barrier_selftest(uint32_t* coop, DevCounters* ctr, uint32_t blocks, cudaStream_t st) {
  k_barrier_selftest<<<blocks, 32, 0, st>>>(coop, blocks, ctr);
  note_launches(1);
  return cudaGetLastError();
}

static uint32_t coop_grid(const void* kernel) {
  int per = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, 256, 0);
  if (per < 1) per = 1;
  uint32_t g = (uint32_t)(sm_count() * per);
  return g > kCoopPass - kCoopBlocks ? kCoopPass - kCoopBlocks : g;
}

cudaError_t launch_binary_budget(const FrameArgs& a, const RenderBuffers& b, const AdaptBuffers& ab,
                                 const float* result, const uint32_t* sampleN, uint32_t desired, float minProb,
                                 cudaStream_t st) {
  const uint32_t np = a.width * a.height;
  const uint32_t nr = adapt_reduce_blocks(np);
  k_error<<<nr, kReduceBlock, 0, st>>>(ab.filtered, result, sampleN, np, desired, ab.err, ab.partial);
  cudaError_t e = cudaMemsetAsync(ab.coop, 0, 16 * sizeof(uint32_t), st);
  if (e != cudaSuccess) return e;
  static uint32_t g = coop_grid((const void*)k_bin_search);
  FrameArgs aa = a;
  RenderBuffers bb = b;
  const float* errp = ab.err;
  uint32_t npv = np, Dv = desired;
  float mp = minProb;
  uint32_t* coop = ab.coop;
  void* args[] = {&aa, &bb, &errp, &npv, &Dv, &mp, &coop};
  e = cudaLaunchCooperativeKernel((const void*)k_bin_search, dim3(g), dim3(256), args, 0, st);
  if (e != cudaSuccess) return e;
  k_gen_queue<<<(np + 255) / 256, 256, 0, st>>>(a, b, np);
  note_launches(3);
  return cudaGetLastError();
}

cudaError_t launch_binary_apply(const FrameArgs& a, const RenderBuffers& b, const AdaptBuffers& ab, float* result,
                                uint32_t* sampleN, float* gpos, float* gnorm, float* gdiff, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(ab.coop, 0, 2 * sizeof(uint32_t), st);
  if (e != cudaSuccess) return e;
  static uint32_t g = coop_grid((const void*)k_bin_apply);
  FrameArgs aa = a;
  RenderBuffers bb = b;
  uint32_t* coop = ab.coop;
  void* args[] = {&aa, &bb, &coop, &result, &sampleN, &gpos, &gnorm, &gdiff};
  note_launches(1);
  return cudaLaunchCooperativeKernel((const void*)k_bin_apply, dim3(g), dim3(256), args, 0, st);
}

cudaError_t launch_fmath(int which, const float* x, uint32_t n, float* out, cudaStream_t st) {
  if (n) k_fmath<<<(n + 255) / 256, 256, 0, st>>>(which, x, n, out);
  if (n) note_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_philox(const uint32_t* ctr, uint32_t n, uint32_t k0, uint32_t k1, uint32_t* out, cudaStream_t st) {
  if (n) k_philox<<<(n + 255) / 256, 256, 0, st>>>(ctr, n, k0, k1, out);
  if (n) note_launches(1);
  return cudaGetLastError();
}

}  // namespace gbpt
