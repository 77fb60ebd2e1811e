// Philox4x32-10 counter-based generator (Salmon, Moraes, Dror, Shaw,
// "Parallel random numbers: as easy as 1, 2, 3", SC'11): ten rounds of two
// 32x32->64-bit multiplies with the published multipliers and Weyl key
// increments.  Used by the basis-state sampler and the projector shots.
#pragma once
#include <stdint.h>

namespace qg {

static __device__ __forceinline__ void philox_round(uint32_t* c, uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t lo0 = M0 * c[0], hi0 = __umulhi(M0, c[0]);
  const uint32_t lo1 = M1 * c[2], hi1 = __umulhi(M1, c[2]);
  const uint32_t n0 = hi1 ^ c[1] ^ k0, n1 = lo1, n2 = hi0 ^ c[3] ^ k1, n3 = lo0;
  c[0] = n0;
  c[1] = n1;
  c[2] = n2;
  c[3] = n3;
}

static __device__ __forceinline__ void philox4x32_10(uint32_t* c, uint32_t k0, uint32_t k1) {
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    philox_round(c, k0, k1);
    k0 += W0;
    k1 += W1;
  }
}

// 53 random bits -> a double in [0, 1)
static __device__ __forceinline__ double u01_from(uint32_t a, uint32_t b) {
  const uint64_t m = ((uint64_t)(a >> 5) << 26) | (uint64_t)(b >> 6);
  return (double)m * (1.0 / 9007199254740992.0);
}

}  // namespace qg
