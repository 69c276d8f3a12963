// Test-only kernels: div_rn_recip (synaptogenesis_gb300/csrc/exact_div.cuh)
// against CUDA's IEEE double division, bit for bit.  Built by
// tests/test_gpu_exact_div.py with nvcc into a temporary shared library.
#include <cuda_runtime.h>

#include <cstdint>

#include "counter_rng.h"
#include "exact_div.cuh"

namespace {

struct Result {
    unsigned long long mismatches, checked, first;
};

__device__ void record(Result* r, bool bad, unsigned long long id) {
    if (bad) {
        atomicAdd(&r->mismatches, 1ull);
        atomicMin(&r->first, id);
    }
}

// (U - sw) / F for every finite float sw.
__global__ void k_constant(double U, int F, Result* r) {
    const double y = 1.0 / F;
    unsigned long long checked = 0;
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
         i < (1ull << 32); i += (unsigned long long)gridDim.x * blockDim.x) {
        const float sw = __uint_as_float((uint32_t)i);
        if (!isfinite(sw)) continue;
        const double x = U - sw;
        const double want = x / F;
        const double got = sg::div_rn_recip(x, (double)F, y);
        record(r, __double_as_longlong(want) != __double_as_longlong(got), i);
        ++checked;
    }
    atomicAdd(&r->checked, checked);
}

// Random pairs: numerator v + 0.1 * f (v, f floats with random exponents),
// denominator 1 + 0.1 * s (s a float with a random exponent and sign); and
// raw doubles over the whole exponent range.
__global__ void k_random(unsigned long long n, unsigned long long seed, Result* r) {
    unsigned long long checked = 0;
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        const uint64_t h1 = sg::rng_bits(seed, 1, i), h2 = sg::rng_bits(seed, 2, i);
        double a, b;
        if (i % 8 == 7) {
            a = __longlong_as_double((long long)h1);
            b = __longlong_as_double((long long)h2);
            if (!isfinite(a) || !isfinite(b) || b == 0.0) continue;
        } else {
            const float v = __uint_as_float(((uint32_t)h1 & 0x807FFFFFu) | ((100u + (uint32_t)(h1 >> 40) % 60u) << 23));
            const float f = __uint_as_float(((uint32_t)(h1 >> 32) & 0x807FFFFFu) | ((90u + (uint32_t)(h2 >> 50) % 80u) << 23));
            const float s = __uint_as_float(((uint32_t)h2 & 0x807FFFFFu) | ((60u + (uint32_t)(h2 >> 40) % 100u) << 23));
            a = v + 0.1 * f;
            b = 1 + (0.1 * s);
        }
        const double want = a / b;
        const double got = sg::div_rn_recip(a, b, 1.0 / b);
        record(r, __double_as_longlong(want) != __double_as_longlong(got), i);
        ++checked;
    }
    atomicAdd(&r->checked, checked);
}

// div_const_rn<F>: (U - sw) / F for every finite float sw, and raw doubles
// over the whole exponent range, against the IEEE division.
template <int F>
__global__ void k_const_int(double U, unsigned long long n_random, unsigned long long seed,
                            Result* r) {
    unsigned long long checked = 0;
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
         i < (1ull << 32) + n_random; i += (unsigned long long)gridDim.x * blockDim.x) {
        double x;
        if (i < (1ull << 32)) {
            const float sw = __uint_as_float((uint32_t)i);
            if (!isfinite(sw)) continue;
            x = U - sw;
        } else {
            x = __longlong_as_double((long long)sg::rng_bits(seed, 3, i));
            if (isnan(x)) continue;
        }
        record(r, __double_as_longlong(x / F) != __double_as_longlong(sg::div_const_rn<F>(x)), i);
        ++checked;
    }
    atomicAdd(&r->checked, checked);
}

int run(void (*launch)(Result*), unsigned long long* out) {
    Result* d = nullptr;
    if (cudaMalloc(&d, sizeof(Result)) != cudaSuccess) return -1;
    Result init{0, 0, ~0ull};
    cudaMemcpy(d, &init, sizeof(Result), cudaMemcpyHostToDevice);
    launch(d);
    Result h{};
    cudaError_t e = cudaMemcpy(&h, d, sizeof(Result), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return -2;
    out[0] = h.mismatches;
    out[1] = h.checked;
    out[2] = h.first;
    return 0;
}

double g_U;
int g_F;
unsigned long long g_n, g_seed;

}  // namespace

extern "C" int check_constant_divisor(double U, int F, unsigned long long* out) {
    g_U = U;
    g_F = F;
    return run([](Result* d) { k_constant<<<152 * 8, 256>>>(g_U, g_F, d); }, out);
}

extern "C" int check_random_pairs(unsigned long long n, unsigned long long seed,
                                  unsigned long long* out) {
    g_n = n;
    g_seed = seed;
    return run([](Result* d) { k_random<<<152 * 8, 256>>>(g_n, g_seed, d); }, out);
}

extern "C" int check_integer_divisor(double U, int F, unsigned long long n_random,
                                     unsigned long long seed, unsigned long long* out) {
    g_U = U;
    g_F = F;
    g_n = n_random;
    g_seed = seed;
    if (F == 1000) return run([](Result* d) { k_const_int<1000><<<152 * 8, 256>>>(g_U, g_n, g_seed, d); }, out);
    if (F == 20) return run([](Result* d) { k_const_int<20><<<152 * 8, 256>>>(g_U, g_n, g_seed, d); }, out);
    if (F == 3) return run([](Result* d) { k_const_int<3><<<152 * 8, 256>>>(g_U, g_n, g_seed, d); }, out);
    return -3;
}
