// Learned sample allocator: a 24 -> 64 -> 64 -> 1 GELU MLP trained and run
// on the 5th-generation tensor cores.
//
// The reference links FANN but never calls it; the allocator is new (its
// features and use are in kernels_adapt.cu / api.cu).  Everything here is
// written for sm_103a:
//   * BF16 operands staged in shared memory in the canonical K-major,
//     no-swizzle layout (8-row x 16-byte core matrices; LBO = 128 B between
//     core matrices along K, SBO = 16 * K bytes between 8-row groups);
//   * tcgen05.mma (kind::f16, BF16 x BF16 -> FP32, M = 128, cta_group::1)
//     issued by one thread, accumulators in tensor memory (TMEM), completion
//     signalled by tcgen05.commit on an mbarrier, results read back with
//     tcgen05.ld (32x32b: warp w sees TMEM lanes 32w..32w+31 = rows);
//   * every mbarrier wait is bounded (1 s on %globaltimer): on expiry the
//     kernel sets an error bit, waits once more (bounded) for its own MMAs,
//     frees its TMEM and returns.
// One CTA of 128 threads owns 128 rows (samples); thread r owns row r in
// every epilogue.  Training: forward, loss, backward through both layers and
// the weight gradients as tensor-core products over the CTA's rows
// (dW2 = dZ2^T H1, dW1 = dZ1^T X, with the 64 output rows padded to M = 128
// by zero rows), accumulated across CTAs with FP32 atomics; then Adam.
// Rounding points (matched by the CPU oracle): X, W1, W2, w3, H1, dZ2, dZ1
// are BF16; biases, pre-activations, H2, y and all sums are FP32.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "gbpt_internal.h"
#include "gbpt_math.cuh"
#include "launch.h"

namespace gbpt {
namespace mlp {

constexpr int kIn = 24, kInPad = 32, kHid = 64, kRows = 128, kThreads = 128;
constexpr int oW1 = 0, oB1 = kHid * kIn, oW2 = oB1 + kHid, oB2 = oW2 + kHid * kHid, oW3 = oB2 + kHid,
              oB3 = oW3 + kHid, kParams = oB3 + 1;  // 5825
static_assert(kParams == 5825, "parameter layout");

constexpr uint32_t kErrTimeout = 1u;  // an mbarrier wait ran out

// ---- shared-memory tile layout ------------------------------------------------
// byte offset of element (row, k) of a K-major tile whose rows hold kTot elements
__host__ __device__ constexpr uint32_t kmaj(uint32_t row, uint32_t k, uint32_t kTot) {
  return (row >> 3) * (kTot * 16u) + (k >> 3) * 128u + (row & 7u) * 16u + (k & 7u) * 2u;
}
__host__ __device__ constexpr uint32_t tile_bytes(uint32_t rows, uint32_t kTot) { return rows * kTot * 2u; }

// training-kernel shared memory (bytes, all offsets 1024-aligned)
constexpr uint32_t sAx = 0;                                   // X       128 x 32
constexpr uint32_t sBw1 = sAx + tile_bytes(128, 32);          // W1       64 x 32
constexpr uint32_t sAh1 = sBw1 + tile_bytes(64, 32);          // H1      128 x 64
constexpr uint32_t sBw2 = sAh1 + tile_bytes(128, 64);         // W2       64 x 64
constexpr uint32_t sBw2t = sBw2 + tile_bytes(64, 64);         // W2^T     64 x 64
constexpr uint32_t sAdz2 = sBw2t + tile_bytes(64, 64);        // dZ2     128 x 64
constexpr uint32_t sAdz2t = sAdz2 + tile_bytes(128, 64);      // dZ2^T   128 x 128 (rows 64.. zero)
constexpr uint32_t sBh1t = sAdz2t + tile_bytes(128, 128);     // H1^T     64 x 128
constexpr uint32_t sAdz1t = sBh1t + tile_bytes(64, 128);      // dZ1^T   128 x 128 (rows 64.. zero)
constexpr uint32_t sBxt = sAdz1t + tile_bytes(128, 128);      // X^T      32 x 128
constexpr uint32_t sVec = sBxt + tile_bytes(32, 128);         // fp32: b1, b2, w3, sums
constexpr uint32_t kVecFloats = 64 * 3 + 64 * 3 + 64 + 4;     // b1 b2 w3 | db1 db2 dw3 | pad | db3 loss
constexpr uint32_t sBar = sVec + kVecFloats * 4;              // mbarrier (8 B) + TMEM slot (4 B)
constexpr uint32_t kTrainSmem = sBar + 64;
constexpr uint32_t kInferSmem = sBw2 + tile_bytes(64, 64) + kVecFloats * 4 + 64;
// the inference kernel requests this much so that at most 4 CTAs (4 x 128
// TMEM columns = the SM's 512) are resident per SM: tcgen05.alloc never waits
constexpr uint32_t kInferSmemLaunch = 56 * 1024;
static_assert(kInferSmem <= kInferSmemLaunch, "inference tile fits");
static_assert(kTrainSmem <= 200 * 1024, "training tile fits in shared memory");

// TMEM columns (fp32 accumulators, one column per output element)
constexpr uint32_t tD1 = 0, tD2 = 64, tD3 = 128, tD4 = 192, tD5 = 64;  // D5 reuses D2 after it is read
constexpr uint32_t kTmemCols = 256;

__host__ __device__ constexpr uint32_t idesc_bf16(uint32_t n) {
  // kind::f16 instruction descriptor: D FP32 (bit 4), A BF16 (bits 7-9 = 1),
  // B BF16 (bits 10-12 = 1), both K-major, N >> 3 at bit 17, M >> 4 at bit 24
  return (1u << 4) | (1u << 7) | (1u << 10) | ((n >> 3) << 17) | ((128u >> 4) << 24);
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t kTot) {
  // start >> 4 | LBO (128 B) >> 4 << 16 | SBO (16 * kTot B) >> 4 << 32 | version 1 << 46; no swizzle
  return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(128u >> 4) << 16) |
         ((uint64_t)((16u * kTot) >> 4) << 32) | (1ull << 46);
}

__device__ __forceinline__ uint64_t now_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t phase) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(phase)
      : "memory");
  return ok != 0;
}

// bounded wait for the mbarrier phase; false after ~1 s
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t phase) {
  const uint64_t t0 = now_ns();
  while (!mbar_try(bar, phase)) {
    if (now_ns() - t0 > 1000000000ull) return false;
  }
  return true;
}

__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// D[tmem] (+)= A (128 x 16*ksteps, K-major at aAddr) x B (n x 16*ksteps, K-major at bAddr)^T
__device__ __forceinline__ void mma_issue(uint32_t dTmem, uint32_t aAddr, uint32_t aKtot, uint32_t bAddr,
                                          uint32_t bKtot, uint32_t n, uint32_t ksteps) {
  const uint32_t id = idesc_bf16(n);
  for (uint32_t s = 0; s < ksteps; s++) {
    const uint64_t da = sdesc(aAddr + s * 256u, aKtot);
    const uint64_t db = sdesc(bAddr + s * 256u, bKtot);
    const uint32_t acc = s > 0 ? 1u : 0u;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
        :
        : "r"(dTmem), "l"(da), "l"(db), "r"(id), "r"(acc)
        : "memory");
  }
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
               : "memory");
}

// 16 consecutive FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
  for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void st_bf16(uint8_t* base, uint32_t off, float x) {
  *reinterpret_cast<__nv_bfloat16*>(base + off) = __float2bfloat16_rn(x);
}

__device__ __forceinline__ float warp_sum(float v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.f + erff(z * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float z) {
  return 0.5f * (1.f + erff(z * 0.70710678118654752f)) + z * expf(-0.5f * z * z) * 0.39894228040143268f;
}

// TMEM allocation by warp 0; returns the base address through the smem slot
__device__ __forceinline__ void tmem_alloc(uint32_t slotAddr, uint32_t cols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slotAddr), "r"(cols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_free(uint32_t base, uint32_t cols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(base), "r"(cols) : "memory");
}

// Stage the weights of both MMA layers (and their biases, w3) from the FP32 master vector.
__device__ void stage_weights(uint8_t* sm, const float* __restrict__ theta, bool transposeW2) {
  const uint32_t t = threadIdx.x;
  for (uint32_t e = t; e < 64u * 32u; e += kThreads) {  // W1 (64 x 32, K 24..31 zero)
    const uint32_t o = e >> 5, k = e & 31u;
    st_bf16(sm + sBw1, kmaj(o, k, 32), k < (uint32_t)kIn ? theta[oW1 + o * kIn + k] : 0.f);
  }
  for (uint32_t e = t; e < 64u * 64u; e += kThreads) {  // W2 (o, i) and W2^T (i, o)
    const uint32_t o = e >> 6, i = e & 63u;
    const float w = theta[oW2 + e];
    st_bf16(sm + sBw2, kmaj(o, i, 64), w);
    if (transposeW2) st_bf16(sm + sBw2t, kmaj(i, o, 64), w);
  }
  float* vec = reinterpret_cast<float*>(sm + (transposeW2 ? sVec : kInferSmem - kVecFloats * 4 - 64));
  if (t < 64) {
    vec[t] = theta[oB1 + t];
    vec[64 + t] = theta[oB2 + t];
    vec[128 + t] = __bfloat162float(__float2bfloat16_rn(theta[oW3 + t]));
  }
}

}  // namespace mlp

namespace {
using namespace mlp;

// ---------------------------------------------------------------------------
// Inference: y[r] = MLP(x[r]) for n rows of 24 FP32 features.
__global__ void __launch_bounds__(kThreads, 1) k_mlp_forward(const float* __restrict__ x, uint32_t n,
                                                            const float* __restrict__ theta, float* __restrict__ y,
                                                            uint32_t* err, uint32_t errBit) {
  extern __shared__ __align__(1024) uint8_t sm[];
  const uint32_t t = threadIdx.x, warp = t >> 5;
  const uint32_t row = blockIdx.x * kRows + t;
  float* vec = reinterpret_cast<float*>(sm + kInferSmem - kVecFloats * 4 - 64);
  uint32_t* slot = reinterpret_cast<uint32_t*>(sm + kInferSmem - 64);
  const uint32_t bar = smem_u32(sm + kInferSmem - 56);
  if (warp == 0) tmem_alloc(smem_u32(slot), 128);
  if (t == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  stage_weights(sm, theta, false);
  {  // X tile
    for (int k = 0; k < kInPad; k++) {
      const float v = (row < n && k < kIn) ? x[(size_t)row * kIn + k] : 0.f;
      st_bf16(sm + sAx, kmaj(t, k, 32), v);
    }
  }
  fence_async_smem();
  tc_before();
  __syncthreads();
  tc_after();
  const uint32_t tmem = *slot;
  bool ok = true;
  uint32_t phase = 0;
  if (t == 0) {
    mma_issue(tmem + tD1, smem_u32(sm + sAx), 32, smem_u32(sm + sBw1), 32, 64, 2);
    mma_commit(bar);
  }
  ok = __syncthreads_and(mbar_wait(bar, phase) ? 1 : 0) != 0;  // block-uniform
  if (ok) phase ^= 1u;
  tc_after();
  const uint32_t lane0 = (warp * 32u) << 16;
  if (ok) {
    for (int c = 0; c < 64; c += 16) {
      float z[16];
      tmem_ld16(tmem + lane0 + tD1 + c, z);
      for (int j = 0; j < 16; j++) st_bf16(sm + sAh1, kmaj(t, c + j, 64), gelu(z[j] + vec[c + j]));
    }
    fence_async_smem();
  }
  tc_before();
  __syncthreads();
  tc_after();
  if (ok && t == 0) {
    mma_issue(tmem + tD2, smem_u32(sm + sAh1), 64, smem_u32(sm + sBw2), 64, 64, 4);
    mma_commit(bar);
  }
  if (ok) {
    ok = __syncthreads_and(mbar_wait(bar, phase) ? 1 : 0) != 0;  // block-uniform
    if (ok) phase ^= 1u;
    tc_after();
  }
  if (ok) {
    float acc = theta[oB3];
    for (int c = 0; c < 64; c += 16) {
      float z[16];
      tmem_ld16(tmem + lane0 + tD2 + c, z);
      for (int j = 0; j < 16; j++) acc += gelu(z[j] + vec[64 + c + j]) * vec[128 + c + j];
    }
    if (row < n) y[row] = acc;
  } else if (t == 0) {
    atomicOr(err, errBit);
  }
  if (!ok) mbar_wait(bar, phase);  // bounded second wait for MMAs still in flight
  tc_before();
  __syncthreads();
  if (warp == 0) {
    tc_after();
    tmem_free(tmem, 128);
  }
}

// ---------------------------------------------------------------------------
// Training: loss, and the gradient of the mean squared error over n rows
// accumulated into grad (FP32, kParams).  lossSum receives sum (y - t)^2.
__global__ void __launch_bounds__(kThreads, 1) k_mlp_train(const float* __restrict__ x, const float* __restrict__ tgt,
                                                          uint32_t n, const float* __restrict__ theta,
                                                          float* __restrict__ grad, float* lossSum, uint32_t* err) {
  extern __shared__ __align__(1024) uint8_t sm[];
  const uint32_t t = threadIdx.x, warp = t >> 5;
  const uint32_t row = blockIdx.x * kRows + t;
  const bool valid = row < n;
  float* vec = reinterpret_cast<float*>(sm + sVec);
  float* sdb1 = vec + 192;
  float* sdb2 = vec + 256;
  float* sdw3 = vec + 320;
  float* sscal = vec + 448;  // [0] db3, [1] loss
  uint32_t* slot = reinterpret_cast<uint32_t*>(sm + sBar + 8);
  const uint32_t bar = smem_u32(sm + sBar);
  if (warp == 0) tmem_alloc(smem_u32(slot), kTmemCols);
  if (t == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  stage_weights(sm, theta, true);
  if (t < 64) sdb1[t] = sdb2[t] = sdw3[t] = 0.f;
  if (t < 2) sscal[t] = 0.f;
  // zero the padding rows (64..127) of the two transposed gradient tiles
  for (uint32_t e = t; e < 64u * 128u / 8u; e += kThreads) {
    const uint32_t r = 64u + (e >> 4), k8 = (e & 15u) * 8u;
    *reinterpret_cast<uint4*>(sm + sAdz2t + kmaj(r, k8, 128)) = make_uint4(0, 0, 0, 0);
    *reinterpret_cast<uint4*>(sm + sAdz1t + kmaj(r, k8, 128)) = make_uint4(0, 0, 0, 0);
  }
  for (int k = 0; k < kInPad; k++) {  // X tile (row-major) and X^T
    const float v = (valid && k < kIn) ? x[(size_t)row * kIn + k] : 0.f;
    st_bf16(sm + sAx, kmaj(t, k, 32), v);
    st_bf16(sm + sBxt, kmaj(k, t, 128), v);
  }
  const float target = valid ? tgt[row] : 0.f;
  fence_async_smem();
  tc_before();
  __syncthreads();
  tc_after();
  const uint32_t tmem = *slot;
  const uint32_t lane0 = (warp * 32u) << 16;
  uint32_t phase = 0;
  bool ok = true;

  // ---- layer 1: D1 = X W1^T
  if (t == 0) {
    mma_issue(tmem + tD1, smem_u32(sm + sAx), 32, smem_u32(sm + sBw1), 32, 64, 2);
    mma_commit(bar);
  }
  ok = __syncthreads_and(mbar_wait(bar, phase) ? 1 : 0) != 0;  // block-uniform
  if (ok) phase ^= 1u;
  tc_after();
  if (ok) {
    for (int c = 0; c < 64; c += 16) {
      float z[16];
      tmem_ld16(tmem + lane0 + tD1 + c, z);
      for (int j = 0; j < 16; j++) {
        const float h = gelu(z[j] + vec[c + j]);
        st_bf16(sm + sAh1, kmaj(t, c + j, 64), h);
        st_bf16(sm + sBh1t, kmaj(c + j, t, 128), h);
      }
    }
    fence_async_smem();
  }
  tc_before();
  __syncthreads();
  tc_after();
  // ---- layer 2: D2 = H1 W2^T
  if (ok && t == 0) {
    mma_issue(tmem + tD2, smem_u32(sm + sAh1), 64, smem_u32(sm + sBw2), 64, 64, 4);
    mma_commit(bar);
  }
  if (ok) {
    ok = __syncthreads_and(mbar_wait(bar, phase) ? 1 : 0) != 0;  // block-uniform
    if (ok) phase ^= 1u;
    tc_after();
  }
  if (ok) {
    float z2[64];
    for (int c = 0; c < 64; c += 16) tmem_ld16(tmem + lane0 + tD2 + c, z2 + c);
    float yv = theta[oB3];
    for (int j = 0; j < 64; j++) {
      z2[j] += vec[64 + j];
      yv += gelu(z2[j]) * vec[128 + j];
    }
    const float dy = valid ? 2.f * (yv - target) / (float)n : 0.f;
    // column sums over the CTA's rows: a warp butterfly, then one shared atomic per warp
    const float l2 = warp_sum(valid ? (yv - target) * (yv - target) : 0.f), sdy = warp_sum(dy);
    if ((t & 31) == 0) {
      atomicAdd(&sscal[1], l2);
      atomicAdd(&sscal[0], sdy);
    }
    for (int j = 0; j < 64; j++) {
      const float g3 = warp_sum(dy * gelu(z2[j]));
      const float dz = dy * vec[128 + j] * gelu_grad(z2[j]);
      const float g2 = warp_sum(dz);
      if ((t & 31) == 0) {
        atomicAdd(&sdw3[j], g3);
        atomicAdd(&sdb2[j], g2);
      }
      st_bf16(sm + sAdz2, kmaj(t, j, 64), dz);
      st_bf16(sm + sAdz2t, kmaj(j, t, 128), dz);
    }
    fence_async_smem();
  }
  tc_before();
  __syncthreads();
  tc_after();
  // ---- backward: D3 = dZ2 W2 (dH1), D4 = dZ2^T H1 (dW2)
  if (ok && t == 0) {
    mma_issue(tmem + tD3, smem_u32(sm + sAdz2), 64, smem_u32(sm + sBw2t), 64, 64, 4);
    mma_issue(tmem + tD4, smem_u32(sm + sAdz2t), 128, smem_u32(sm + sBh1t), 128, 64, 8);
    mma_commit(bar);
  }
  if (ok) {
    ok = __syncthreads_and(mbar_wait(bar, phase) ? 1 : 0) != 0;  // block-uniform
    if (ok) phase ^= 1u;
    tc_after();
  }
  if (ok) {
    for (int c = 0; c < 64; c += 16) {
      float dh[16], z1[16];
      tmem_ld16(tmem + lane0 + tD3 + c, dh);
      tmem_ld16(tmem + lane0 + tD1 + c, z1);
      for (int j = 0; j < 16; j++) {
        const float dz = dh[j] * gelu_grad(z1[j] + vec[c + j]);
        const float g1 = warp_sum(dz);
        if ((t & 31) == 0) atomicAdd(&sdb1[c + j], g1);
        st_bf16(sm + sAdz1t, kmaj(c + j, t, 128), dz);
      }
    }
    if (warp < 2) {  // rows 0..63 of D4 = dW2[o = t][i] (warps 2-3 hold the zero padding rows)
      for (int c = 0; c < 64; c += 16) {
        float g[16];
        tmem_ld16(tmem + lane0 + tD4 + c, g);
        for (int j = 0; j < 16; j++) atomicAdd(&grad[oW2 + t * 64 + c + j], g[j]);
      }
    }
    fence_async_smem();
  }
  tc_before();
  __syncthreads();
  tc_after();
  // ---- D5 = dZ1^T X (dW1), into the columns D2 used
  if (ok && t == 0) {
    mma_issue(tmem + tD5, smem_u32(sm + sAdz1t), 128, smem_u32(sm + sBxt), 128, 32, 8);
    mma_commit(bar);
  }
  if (ok) {
    ok = __syncthreads_and(mbar_wait(bar, phase) ? 1 : 0) != 0;  // block-uniform
    if (ok) phase ^= 1u;
    tc_after();
  }
  if (ok && warp < 2) {  // rows 0..63 of D5 = dW1[o = t][i], i < 24
    for (int c = 0; c < 32; c += 16) {
      float g[16];
      tmem_ld16(tmem + lane0 + tD5 + c, g);
      for (int j = 0; j < 16; j++)
        if (c + j < kIn) atomicAdd(&grad[oW1 + t * kIn + c + j], g[j]);
    }
  }
  if (!ok) {
    if (t == 0) atomicOr(err, kErrTimeout);
    mbar_wait(bar, phase);  // bounded second wait for MMAs still in flight
  }
  tc_before();
  __syncthreads();
  if (ok && t < 64) {
    atomicAdd(&grad[oB1 + t], sdb1[t]);
    atomicAdd(&grad[oB2 + t], sdb2[t]);
    atomicAdd(&grad[oW3 + t], sdw3[t]);
  }
  if (ok && t == 0) {
    atomicAdd(&grad[oB3], sscal[0]);
    atomicAdd(lossSum, sscal[1]);
  }
  if (warp == 0) {
    tc_after();
    tmem_free(tmem, kTmemCols);
  }
}

// Adam (Kingma & Ba): bias-corrected first and second moments.
__global__ void k_adam(float* __restrict__ theta, float* __restrict__ m, float* __restrict__ v,
                       const float* __restrict__ g, uint32_t n, float lr, float c1, float c2) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = 0.9f * m[i] + 0.1f * gi;
  const float vi = 0.999f * v[i] + 0.001f * gi * gi;
  m[i] = mi;
  v[i] = vi;
  theta[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + 1e-8f);
}

}  // namespace
}  // namespace gbpt

// ---------------------------------------------------------------------------
// C ABI
struct gbpt_mlp {
  float* theta = nullptr;  // device: parameters, Adam moments, gradient, loss, error word
  float* m = nullptr;
  float* v = nullptr;
  float* grad = nullptr;
  float* loss = nullptr;
  uint32_t* err = nullptr;
  uint32_t step = 0;
  cudaStream_t st = nullptr;
  ~gbpt_mlp() {
    if (st) cudaStreamSynchronize(st);
    for (void* p : {(void*)theta, (void*)m, (void*)v, (void*)grad, (void*)loss, (void*)err})
      if (p) cudaFree(p);
    if (st) cudaStreamDestroy(st);
  }
};

namespace {
using gbpt::fail;
using namespace gbpt::mlp;

#define CKM(x)                                                                                      \
  do {                                                                                              \
    cudaError_t e_ = (x);                                                                           \
    if (e_ != cudaSuccess) return fail(GBPT_ERR_CUDA, std::string(#x ": ") + cudaGetErrorString(e_)); \
  } while (0)

gbpt_status check_err(gbpt_mlp* m) {
  uint32_t e = 0;
  CKM(cudaMemcpyAsync(&e, m->err, 4, cudaMemcpyDeviceToHost, m->st));
  CKM(cudaStreamSynchronize(m->st));
  if (e) {
    CKM(cudaMemsetAsync(m->err, 0, 4, m->st));
    return fail(GBPT_ERR_TIMEOUT, "MLP kernel: tensor-core completion wait timed out");
  }
  return GBPT_OK;
}

struct Staged {
  const float* p = nullptr;
  float* own = nullptr;
  ~Staged() {
    if (own) cudaFree(own);
  }
};
cudaError_t stage(const float* src, size_t n, int32_t isDev, cudaStream_t st, Staged* out) {
  if (isDev || n == 0) {
    out->p = src;
    return cudaSuccess;
  }
  cudaError_t e = cudaMalloc(&out->own, n * 4);
  if (e != cudaSuccess) return e;
  out->p = out->own;
  return cudaMemcpyAsync(out->own, src, n * 4, cudaMemcpyHostToDevice, st);
}

gbpt_status forward_attr() {
  static bool attr = false;
  if (!attr) {
    CKM(cudaFuncSetAttribute(gbpt::k_mlp_forward, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)kInferSmemLaunch));
    attr = true;
  }
  return GBPT_OK;
}

gbpt_status gradients_impl(gbpt_mlp* m, const float* x, const float* t, uint32_t n, int32_t isDev, float* lossOut) {
  Staged sx, stg;
  CKM(stage(x, (size_t)n * kIn, isDev, m->st, &sx));
  CKM(stage(t, n, isDev, m->st, &stg));
  CKM(cudaMemsetAsync(m->grad, 0, kParams * 4, m->st));
  CKM(cudaMemsetAsync(m->loss, 0, 4, m->st));
  static bool attr = false;
  if (!attr) {
    CKM(cudaFuncSetAttribute(gbpt::k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTrainSmem));
    attr = true;
  }
  const uint32_t grid = (n + kRows - 1) / kRows;
  if (grid) {
    gbpt::k_mlp_train<<<grid, kThreads, kTrainSmem, m->st>>>(sx.p, stg.p, n, m->theta, m->grad, m->loss, m->err);
    gbpt::note_launches(1);
    CKM(cudaGetLastError());
  }
  gbpt_status s = check_err(m);
  if (s != GBPT_OK) return s;
  if (lossOut) {
    float l = 0.f;
    CKM(cudaMemcpy(&l, m->loss, 4, cudaMemcpyDeviceToHost));
    *lossOut = n ? l / (float)n : 0.f;
  }
  return GBPT_OK;
}

}  // namespace

gbpt_status gbpt::mlp_forward_async(gbpt_mlp* m, const float* x, uint32_t n, float* y, uint32_t* err,
                                    uint32_t errBit, void* stream) {
  gbpt_status sa = forward_attr();
  if (sa != GBPT_OK) return sa;
  const uint32_t grid = (n + kRows - 1) / kRows;
  if (grid) {
    gbpt::k_mlp_forward<<<grid, kThreads, kInferSmemLaunch, (cudaStream_t)stream>>>(x, n, m->theta, y, err, errBit);
    gbpt::note_launches(1);
    CKM(cudaGetLastError());
  }
  return GBPT_OK;
}

extern "C" {

gbpt_status gbpt_mlp_create(uint32_t seed, gbpt_mlp** out) {
  if (!out) return fail(GBPT_ERR_INVALID_ARG, "out is NULL");
  *out = nullptr;
  gbpt_mlp* m = new (std::nothrow) gbpt_mlp();
  if (!m) return fail(GBPT_ERR_OOM, "host allocation failed");
  cudaError_t e = cudaStreamCreateWithFlags(&m->st, cudaStreamNonBlocking);
  for (float** p : {&m->theta, &m->m, &m->v, &m->grad})
    if (e == cudaSuccess) e = cudaMalloc(p, kParams * 4);
  if (e == cudaSuccess) e = cudaMalloc(&m->loss, 4);
  if (e == cudaSuccess) e = cudaMalloc(&m->err, 4);
  if (e != cudaSuccess) {
    delete m;
    return fail(GBPT_ERR_OOM, std::string("MLP buffers: ") + cudaGetErrorString(e));
  }
  // He-uniform weights (bound sqrt(6 / fan_in)) from Philox4x32-10 draws, zero biases
  std::vector<float> w(kParams, 0.f);
  uint32_t k0 = seed, k1 = 0x4d4c5021u;
  for (int i = 0; i < kParams; i++) {
    gb::u4 r = gb::philox(gb::u4{(uint32_t)i, 0u, 0u, 0u}, k0, k1);
    float u = gb::u01(r.a) * 2.f - 1.f;
    float fan = (i < oB1) ? (float)kIn : (i >= oW2 && i < oB2) ? (float)kHid : (i >= oW3 && i < oB3) ? (float)kHid : 0.f;
    w[i] = fan > 0.f ? u * std::sqrt(6.f / fan) : 0.f;
  }
  e = cudaMemcpy(m->theta, w.data(), kParams * 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(m->m, 0, kParams * 4);
  if (e == cudaSuccess) e = cudaMemset(m->v, 0, kParams * 4);
  if (e == cudaSuccess) e = cudaMemset(m->err, 0, 4);
  if (e != cudaSuccess) {
    delete m;
    return fail(GBPT_ERR_CUDA, std::string("MLP init: ") + cudaGetErrorString(e));
  }
  *out = m;
  return GBPT_OK;
}

gbpt_status gbpt_mlp_destroy(gbpt_mlp* m) {
  delete m;
  return GBPT_OK;
}

uint32_t gbpt_mlp_param_count(void) { return kParams; }

gbpt_status gbpt_mlp_get_params(gbpt_mlp* m, float* w) {
  if (!m || !w) return fail(GBPT_ERR_INVALID_ARG, "NULL argument");
  CKM(cudaMemcpyAsync(w, m->theta, kParams * 4, cudaMemcpyDeviceToHost, m->st));
  CKM(cudaStreamSynchronize(m->st));
  return GBPT_OK;
}

gbpt_status gbpt_mlp_set_params(gbpt_mlp* m, const float* w) {
  if (!m || !w) return fail(GBPT_ERR_INVALID_ARG, "NULL argument");
  CKM(cudaMemcpyAsync(m->theta, w, kParams * 4, cudaMemcpyHostToDevice, m->st));
  CKM(cudaMemsetAsync(m->m, 0, kParams * 4, m->st));
  CKM(cudaMemsetAsync(m->v, 0, kParams * 4, m->st));
  CKM(cudaStreamSynchronize(m->st));
  m->step = 0;
  return GBPT_OK;
}

gbpt_status gbpt_mlp_forward(gbpt_mlp* m, const float* x, uint32_t n, float* y, int32_t is_device) {
  if (!m || (n && (!x || !y))) return fail(GBPT_ERR_INVALID_ARG, "NULL argument");
  Staged sx;
  CKM(stage(x, (size_t)n * kIn, is_device, m->st, &sx));
  float* dy = y;
  float* own = nullptr;
  if (!is_device && n) {
    CKM(cudaMalloc(&own, (size_t)n * 4));
    dy = own;
  }
  gbpt_status sa = forward_attr();
  if (sa != GBPT_OK) return sa;
  const uint32_t grid = (n + kRows - 1) / kRows;
  if (grid) {
    gbpt::k_mlp_forward<<<grid, kThreads, kInferSmemLaunch, m->st>>>(sx.p, n, m->theta, dy, m->err, kErrTimeout);
    gbpt::note_launches(1);
  }
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess && own) e = cudaMemcpyAsync(y, own, (size_t)n * 4, cudaMemcpyDeviceToHost, m->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(m->st);
  if (own) cudaFree(own);
  if (e != cudaSuccess) return fail(GBPT_ERR_CUDA, std::string("MLP forward: ") + cudaGetErrorString(e));
  return check_err(m);
}

gbpt_status gbpt_mlp_gradients(gbpt_mlp* m, const float* x, const float* t, uint32_t n, int32_t is_device,
                               float* grad_out, float* loss_out) {
  if (!m || (n && (!x || !t))) return fail(GBPT_ERR_INVALID_ARG, "NULL argument");
  gbpt_status s = gradients_impl(m, x, t, n, is_device, loss_out);
  if (s != GBPT_OK) return s;
  if (grad_out) {
    CKM(cudaMemcpy(grad_out, m->grad, kParams * 4, cudaMemcpyDeviceToHost));
  }
  return GBPT_OK;
}

gbpt_status gbpt_mlp_train_step(gbpt_mlp* m, const float* x, const float* t, uint32_t n, float lr, int32_t is_device,
                                float* loss_out) {
  if (!m || (n && (!x || !t))) return fail(GBPT_ERR_INVALID_ARG, "NULL argument");
  gbpt_status s = gradients_impl(m, x, t, n, is_device, loss_out);
  if (s != GBPT_OK) return s;
  m->step++;
  const float c1 = 1.f - std::pow(0.9f, (float)m->step), c2 = 1.f - std::pow(0.999f, (float)m->step);
  gbpt::k_adam<<<(kParams + 255) / 256, 256, 0, m->st>>>(m->theta, m->m, m->v, m->grad, kParams, lr, c1, c2);
  gbpt::note_launches(1);
  CKM(cudaGetLastError());
  CKM(cudaStreamSynchronize(m->st));
  return GBPT_OK;
}

}  // extern "C"
