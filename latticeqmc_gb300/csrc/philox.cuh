// Philox4x64-10 (Salmon et al., SC'11) for the on-device uniform stream.
//
// Uniform of site position p (sweep order) in sweep t of a chain keyed (seed, chain):
// word p % 4 of philox4x64_10(counter = {p / 4, t, 0, 0}, key = {seed, chain}),
// converted as (word >> 11) * 2^-53 -- the same conversion numpy's random() uses.
#pragma once
#include <stdint.h>

namespace lqmc {

__host__ __device__ __forceinline__ uint64_t mulhi64(uint64_t a, uint64_t b) {
#ifdef __CUDA_ARCH__
    return __umul64hi(a, b);
#else
    return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

__host__ __device__ __forceinline__ void philox4x64_10(uint64_t c[4], uint64_t k0, uint64_t k1) {
    const uint64_t M0 = 0xD2E7470EE14C6C93ull, M1 = 0xCA5A826395121157ull;
    const uint64_t W0 = 0x9E3779B97F4A7C15ull, W1 = 0xBB67AE8584CAA73Bull;
    for (int r = 0; r < 10; ++r) {
        if (r) { k0 += W0; k1 += W1; }
        const uint64_t hi0 = mulhi64(M0, c[0]), lo0 = M0 * c[0];
        const uint64_t hi1 = mulhi64(M1, c[2]), lo1 = M1 * c[2];
        const uint64_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
        c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
    }
}

// (word >> 11) 2^-53: a uniform on [0, 1) with 53 random bits
__host__ __device__ __forceinline__ double philox_to_unit(uint64_t w) {
    return (double)(w >> 11) * (1.0 / 9007199254740992.0);
}

// The four uniforms of positions 4 q .. 4 q + 3 of sweep t: one Philox call
__host__ __device__ __forceinline__ void philox_uniform4(uint64_t seed, uint64_t chain,
                                                         uint64_t sweep, uint64_t q, double u[4]) {
    uint64_t c[4] = {q, sweep, 0ull, 0ull};
    philox4x64_10(c, seed, chain);
    for (int w = 0; w < 4; ++w) u[w] = philox_to_unit(c[w]);
}

__host__ __device__ __forceinline__ double philox_uniform(uint64_t seed, uint64_t chain,
                                                          uint64_t sweep, uint64_t pos) {
    uint64_t c[4] = {pos >> 2, sweep, 0ull, 0ull};
    philox4x64_10(c, seed, chain);
    return philox_to_unit(c[pos & 3]);
}

}  // namespace lqmc
