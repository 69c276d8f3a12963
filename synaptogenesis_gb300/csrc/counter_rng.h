// Counter-based random numbers for generated networks: every value is a pure
// function of (seed, stream, index), so a device kernel, a host loop and a
// numpy restatement produce the same weights, delays and inputs.  The mixing
// function is the SplitMix64 finaliser (Steele, Lea, Flood: "Fast splittable
// pseudorandom number generators", OOPSLA 2014).
#pragma once
#include <cstdint>

#ifdef __CUDACC__
#define SG_HD __host__ __device__ __forceinline__
#else
#define SG_HD inline
#endif

namespace sg {

enum : uint64_t {
    RNG_CONV_WEIGHT = 1,   // index: destination * kernel + k
    RNG_FC_WEIGHT = 2,     // index: to * size + from
    RNG_FC_MASK = 3,       // index: to * size + from
    RNG_FC_DELAY = 4,      // index: to * size + from
    RNG_INPUT = 5,         // index: step * size + neuron
};

SG_HD uint64_t rng_mix(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

SG_HD uint64_t rng_bits(uint64_t seed, uint64_t stream, uint64_t index) {
    return rng_mix(seed * 0x9E3779B97F4A7C15ull + stream * 0xD1B54A32D192ED03ull + index);
}

// Uniform float in [0, 1) with 24 random bits.
SG_HD float rng_uniform(uint64_t seed, uint64_t stream, uint64_t index) {
    return (float)(rng_bits(seed, stream, index) >> 40) * (1.0f / 16777216.0f);
}

// Uniform integer in [0, n).
SG_HD uint32_t rng_below(uint64_t seed, uint64_t stream, uint64_t index, uint32_t n) {
    return (uint32_t)((rng_bits(seed, stream, index) >> 32) % n);
}

}  // namespace sg
