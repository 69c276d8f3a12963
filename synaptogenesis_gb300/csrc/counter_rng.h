// Counter-based random numbers for generated networks: every value is a pure
// function of (seed, stream, index), so a device kernel, a host loop and a
// numpy restatement produce the same weights, delays and inputs.  The mixing
// function is the SplitMix64 finaliser (Steele, Lea, Flood: "Fast splittable
// pseudorandom number generators", OOPSLA 2014).
#pragma once
#include <cmath>
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
    RNG_NOISE = 6,         // init-config noise, stream RNG_NOISE * 4 + draw;
                           // index: step << 32 | neuron
    RNG_NOISE_RATE = 7,    // per-neuron Poisson rates; index: neuron
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

// Uniform float in (0, 1): 24 random bits plus one, times the float nearest
// 1 / (2^24 + 1).
SG_HD float rng_open01(uint64_t seed, uint64_t stream, uint64_t index) {
    constexpr float kInv = (float)(1.0 / 16777217.0);
    return (float)((rng_bits(seed, stream, index) >> 40) + 1) * kInv;
}

// Natural logarithm of x in (0, 1] in float arithmetic: x = m 2^e with m in
// [sqrt(1/2), sqrt(2)), log m = 2 atanh(s), s = (m - 1) / (m + 1), from its
// series to s^9 (|s| < 0.172: the next term is below 1e-9 of the result).
// Every step is a correctly rounded float operation, so host and device
// agree bit for bit.
SG_HD float noise_log(float x) {
    uint32_t u;
#ifdef __CUDA_ARCH__
    u = __float_as_uint(x);
#else
    __builtin_memcpy(&u, &x, 4);
#endif
    int e = (int)((u >> 23) & 0xFFu) - 127;
    const uint32_t mb = (u & 0x7FFFFFu) | 0x3F800000u;
    float m;
#ifdef __CUDA_ARCH__
    m = __uint_as_float(mb);
#else
    __builtin_memcpy(&m, &mb, 4);
#endif
    if (m > 1.41421354f) {
        m = m * 0.5f;
        e += 1;
    }
    const float s = (m - 1.0f) / (m + 1.0f);
    const float z = s * s;
    float p = 0.222222224f;                 // 2/9
    p = p * z + 0.285714298f;               // 2/7
    p = p * z + 0.400000006f;               // 2/5
    p = p * z + 0.666666687f;               // 2/3
    p = p * z + 2.0f;
    return s * p + (float)e * 0.693147182f;
}

// cos(pi x) for x in [0, 2] in float arithmetic: folded onto [0, 1/4] by
// cos(pi x) = cos(pi (2 - x)) = -cos(pi (1 - x)) and cos(pi y) = sin(pi (1/2 - y)),
// then the Taylor series of cos to t^10 or of sin to t^9 (|t| <= pi/4: the
// next terms are below 3e-9).
SG_HD float noise_cospi(float x) {
    if (x > 1.0f) x = 2.0f - x;
    float sign = 1.0f;
    if (x > 0.5f) {
        x = 1.0f - x;
        sign = -1.0f;
    }
    float r;
    if (x > 0.25f) {
        const float t = (0.5f - x) * 3.14159274f;
        const float z = t * t;
        float p = 2.75573188e-06f;          // 1/9!
        p = p * z - 1.98412701e-04f;        // 1/7!
        p = p * z + 8.33333377e-03f;        // 1/5!
        p = p * z - 0.166666672f;           // 1/3!
        p = p * z + 1.0f;
        r = t * p;
    } else {
        const float t = x * 3.14159274f;
        const float z = t * t;
        float p = -2.75573188e-07f;         // 1/10!
        p = p * z + 2.48015876e-05f;        // 1/8!
        p = p * z - 1.38888892e-03f;        // 1/6!
        p = p * z + 4.16666679e-02f;        // 1/4!
        p = p * z - 0.5f;                   // 1/2!
        r = p * z + 1.0f;
    }
    return sign * r;
}

// Standard normal variate from two uniforms in (0, 1] (Box and Muller, 1958).
SG_HD float noise_normal(float u1, float u2) {
    return sqrtf(-2.0f * noise_log(u1)) * noise_cospi(2.0f * u2);
}

// Uniform integer in [0, n).
SG_HD uint32_t rng_below(uint64_t seed, uint64_t stream, uint64_t index, uint32_t n) {
    return (uint32_t)((rng_bits(seed, stream, index) >> 32) % n);
}

}  // namespace sg
