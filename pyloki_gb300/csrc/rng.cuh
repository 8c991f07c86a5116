// Counter-based Gaussian draws shared by the Monte-Carlo kernels.
//
// Philox-4x32-10 (Salmon, Moraes, Dror and Shaw, "Parallel random numbers: as
// easy as 1, 2, 3", SC 2011) keyed by a 64-bit seed, followed by the
// Box-Muller transform. A draw depends only on (seed, counter), never on the
// launch shape, so a kernel can regenerate the same noise in a later pass.
#pragma once

#include <cstdint>

namespace loki {

__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k) {
  // round multipliers and Weyl key increments of the published Philox-4x32
#pragma unroll
  for (int i = 0; i < 10; ++i) {
    const uint32_t hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
    const uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
    c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
    k.x += 0x9E3779B9u;
    k.y += 0xBB67AE85u;
  }
  return c;
}

// One standard normal for counter (row, col) in stream `domain`: Box-Muller
// on two 32-bit uniforms in (0, 1).
__device__ __forceinline__ float normal_at(uint64_t seed, int64_t row, int col,
                                           uint32_t domain = 0x5A17u) {
  const uint4 r = philox4x32_10(
      make_uint4((uint32_t)row, (uint32_t)((uint64_t)row >> 32), (uint32_t)col, domain),
      make_uint2((uint32_t)seed, (uint32_t)(seed >> 32)));
  const float u1 = ((float)r.x + 0.5f) * 2.3283064365386963e-10f;  // 2^-32
  const float u2 = ((float)r.y + 0.5f) * 2.3283064365386963e-10f;
  float s, c;
  sincospif(2.0f * u2, &s, &c);
  return sqrtf(-2.0f * logf(u1)) * c;
}

}  // namespace loki
