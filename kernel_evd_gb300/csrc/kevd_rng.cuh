// Counter-based uniforms for the pivot sampler: Philox4x32-10 (Salmon, Moraes,
// Dror & Shaw, SC'11), written from the published description.
//
// counter = (slot, round, stream, 0), key = (seed lo, seed hi); stream 0 feeds
// the b pivot proposals of a round, stream 1 its b accept/reject draws.  The
// double in (0, 1] is ((w0 >> 5) * 2^26 + (w1 >> 6) + 1) * 2^-53, the same
// half-open range as the reference's cuRAND draws (ks_arpclm.cu:205, :329).
#pragma once

#include <cstdint>

namespace kevd {

__host__ __device__ inline void philox_round(uint32_t& c0, uint32_t& c1, uint32_t& c2,
                                             uint32_t& c3, uint32_t k0, uint32_t k1) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    const uint32_t n0 = hi1 ^ c1 ^ k0;
    const uint32_t n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
}

__host__ __device__ inline double philox_uniform(uint64_t seed, uint32_t round, uint32_t stream,
                                                 uint32_t slot) {
    uint32_t c0 = slot, c1 = round, c2 = stream, c3 = 0;
    uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        philox_round(c0, c1, c2, c3, k0, k1);
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    const uint64_t m = (uint64_t)(c0 >> 5) * (1ull << 26) + (uint64_t)(c1 >> 6);
    return ((double)m + 1.0) * 0x1.0p-53;
}

}  // namespace kevd
