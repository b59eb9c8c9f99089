// fednl_philox.cuh -- Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) and the Feistel
// permutation built on it, shared by the FP64 and the mixed-precision translation units.  The
// CPU oracle (oracle/fednl_oracle.c, orc_philox4x32 / orc_randk_philox) computes the same stream.
#pragma once

#include <cstdint>

namespace fednl {

__device__ __forceinline__ void philox4x32(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1,
                                           uint32_t& o0)
{
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        const uint32_t hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
        const uint32_t hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
        const uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
    }
    o0 = c0;
}

__device__ __forceinline__ uint32_t philox_feistel(uint32_t x, int h, uint32_t seed, uint32_t client, uint32_t draw)
{
    const uint32_t mask = (1u << h) - 1u;
    uint32_t L = x >> h, R = x & mask;
    for (uint32_t r = 0; r < 6; ++r) {
        uint32_t o;
        philox4x32(R, r, draw, 0x52414E44u, seed, client, o);
        const uint32_t nr = L ^ (o & mask);
        L = R;
        R = nr;
    }
    return (L << h) | R;
}


__host__ __device__ inline int philox_half_bits(long long U)
{
    int b = 2;
    while ((1ll << b) < U) ++b;
    return (b + 1) / 2;
}

}  // namespace fednl
