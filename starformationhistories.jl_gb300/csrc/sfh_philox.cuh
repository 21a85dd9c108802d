// sfh_philox.cuh -- counter-based random numbers shared by the samplers and the mock
// observation: Philox4x32-10 (Salmon, Moraes, Dror and Shaw, SC'11) and its conversions.
#pragma once
#include <stdint.h>

namespace sfh_rng {

struct u4 {
    uint32_t x, y, z, w;
};

// Philox4x32 with 10 rounds (multipliers 0xD2511F53 / 0xCD9E8D57, Weyl key increments
// 0x9E3779B9 / 0xBB67AE85), as published by Salmon, Moraes, Dror and Shaw (2011).
__device__ __forceinline__ u4 philox(u4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const uint32_t lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
        const uint32_t lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
        c = u4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return c;
}

__device__ __forceinline__ double u01(uint32_t a, uint32_t b) {  // (0, 1], 53 bits
    const uint64_t v = ((uint64_t)a << 21) ^ (uint64_t)b;
    return ((double)(v & ((1ull << 53) - 1)) + 1.0) * (1.0 / 9007199254740992.0);
}

}  // namespace sfh_rng
