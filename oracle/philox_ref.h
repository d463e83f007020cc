// TEST INFRASTRUCTURE ONLY -- CPU oracle: Philox4x32-10 counter-based RNG.
//
// Restated from the published description: J. K. Salmon, M. A. Moraes,
// R. O. Dror, D. E. Shaw, "Parallel Random Numbers: As Easy as 1, 2, 3",
// SC'11 (the Random123 family).  Ten rounds of
//   (c0,c1,c2,c3) <- (hi(M1*c2) ^ c1 ^ k0, lo(M1*c2), hi(M0*c0) ^ c3 ^ k1, lo(M0*c0))
// with the Weyl key schedule k0 += W0, k1 += W1 between rounds.
//
// The reference seeds curand XORWOW per path (src/cudaRTBDPTStream.cu:632-633,
// :552); a counter-based generator replaces it so that any path's random
// numbers can be recomputed anywhere from (path, frame, bounce, purpose).
#pragma once
#include <cstdint>

namespace orc {

struct U4 {
  uint32_t v[4];
};

static inline U4 philox4x32_10(U4 c, uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
  for (int r = 0; r < 10; r++) {
    uint64_t p0 = (uint64_t)M0 * c.v[0];
    uint64_t p1 = (uint64_t)M1 * c.v[2];
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    U4 n;
    n.v[0] = hi1 ^ c.v[1] ^ k0;
    n.v[1] = lo1;
    n.v[2] = hi0 ^ c.v[3] ^ k1;
    n.v[3] = lo0;
    c = n;
    k0 += W0;
    k1 += W1;
  }
  return c;
}

// 23 random bits mapped to the open interval (0, 1): (2m+1) * 2^-24, exact.
static inline float u01(uint32_t x) { return (float)(x >> 9) * 0x1p-23f + 0x1p-24f; }

// Counter layout shared with the CUDA kernels.
enum Stream : uint32_t { kCamera = 0, kEyeBounce = 1, kLightGen = 2, kLightBounce = 3, kBinaryAccept = 4 };

static inline void draw8(uint32_t key0, uint32_t key1, uint32_t pathId, uint32_t frame, uint32_t stream, uint32_t depth,
                         uint32_t sample, float u[8]) {
  for (uint32_t b = 0; b < 2; b++) {
    U4 c{{pathId, frame, (stream << 24) | (depth << 8) | b, sample}};
    U4 r = philox4x32_10(c, key0, key1);
    for (int k = 0; k < 4; k++) u[b * 4 + k] = u01(r.v[k]);
  }
}

}  // namespace orc
