// Host build of the library's init-config noise draws (counter_rng.h), for
// tests/test_noise_cpu.py: the same float operations the device kernel runs
// (built with -ffp-contract=off), to be compared with the oracle's numpy
// restatement bit for bit.
#include <cstdint>

#include "counter_rng.h"

extern "C" void noise_batch(int kind, unsigned long long seed, unsigned long long step, int n,
                            float a, float b, const float* rates, float* out) {
    for (int i = 0; i < n; ++i) {
        const uint64_t idx = (step << 32) | (uint32_t)i;
        const float u = sg::rng_open01(seed, sg::RNG_NOISE * 4 + 0, idx);
        if (kind == 2) {
            out[i] = u < (rates ? rates[i] : a) ? b : 0.0f;
        } else if (kind == 0) {
            out[i] = (u * (b - a)) + a;
        } else {
            const float u2 = sg::rng_open01(seed, sg::RNG_NOISE * 4 + 1, idx);
            out[i] = (sg::noise_normal(u, u2) * b) + a;
        }
    }
}
