// philox.cuh -- counter-based Philox4x32-10 generator (Salmon, Moraes, Dror, Shaw,
// "Parallel random numbers: as easy as 1, 2, 3", SC'11), written for this project.
// Every draw is a pure function of (key, counter), so a move's random numbers do
// not depend on which thread or in which order it runs, and a run resumes exactly
// from (seed, sweep).
#pragma once

#include <cstdint>

namespace scg {

struct U4 { uint32_t x, y, z, w; };

__host__ __device__ __forceinline__ uint32_t mulhi32(uint32_t a, uint32_t b) {
#ifdef __CUDA_ARCH__
    return __umulhi(a, b);
#else
    return (uint32_t)(((uint64_t)a * b) >> 32);
#endif
}

__host__ __device__ __forceinline__ U4 philox4x32(U4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0 = mulhi32(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
        uint32_t hi1 = mulhi32(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
        c = U4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return c;
}

// Uniform double in [0, 1) from two 32-bit words (53 random bits).
__host__ __device__ __forceinline__ double u01(uint32_t a, uint32_t b) {
    uint64_t v = ((uint64_t)a << 21) ^ (uint64_t)(b >> 11);
    return (double)(v & ((1ull << 53) - 1)) * (1.0 / 9007199254740992.0);
}

// A stream of uniforms for one (stream id, event) pair: 2 doubles per Philox block.
struct Stream {
    uint32_t k0, k1;
    U4 ctr;
    double buf[2];
    int left;
    __host__ __device__ __forceinline__ Stream(uint64_t seed, uint32_t a, uint32_t b, uint32_t c)
        : k0((uint32_t)seed), k1((uint32_t)(seed >> 32)), ctr{a, b, c, 0u}, left(0) {}
    __host__ __device__ __forceinline__ double next() {
        if (left == 0) {
            U4 r = philox4x32(ctr, k0, k1);
            ++ctr.w;
            buf[0] = u01(r.x, r.y);
            buf[1] = u01(r.z, r.w);
            left = 2;
        }
        return buf[2 - left--];
    }
};

}  // namespace scg
