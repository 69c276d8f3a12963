// Test-only kernels: the integer conversions of
// synaptogenesis_gb300/csrc/exact_convert.cuh against the hardware's
// float <-> double conversions and double multiply, bit for bit.  Built by
// tests/test_gpu_exact_convert.py with nvcc into a temporary shared library.
#include <cuda_runtime.h>

#include <cstdint>

#include "counter_rng.h"
#include "exact_convert.cuh"

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

__device__ bool same(double a, double b) { return __double_as_longlong(a) == __double_as_longlong(b); }
__device__ bool same(float a, float b) { return __float_as_uint(a) == __float_as_uint(b); }

// every float bit pattern: f2d_exact(f) == (double)f
__global__ void k_f2d_all(Result* r) {
    unsigned long long checked = 0;
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
         i < (1ull << 32); i += (unsigned long long)gridDim.x * blockDim.x) {
        const float f = __uint_as_float((uint32_t)i);
        record(r, !same(sg::f2d_exact(f), (double)f), i);
        ++checked;
    }
    atomicAdd(&r->checked, checked);
}

// every float bit pattern times the constant c: mul_fd_rn(f, c) ==
// (float)((double)f * c)
__global__ void k_mul_all(double c, Result* r) {
    unsigned long long checked = 0;
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
         i < (1ull << 32); i += (unsigned long long)gridDim.x * blockDim.x) {
        const float f = __uint_as_float((uint32_t)i);
        record(r, !same(sg::mul_fd_rn(f, c), __double2float_rn(__dmul_rn((double)f, c))), i);
        ++checked;
    }
    atomicAdd(&r->checked, checked);
}

// every float bit pattern times the constant c, kept in double:
// mul_df_rn(f, c) == (double)f * c
__global__ void k_muld_all(double c, Result* r) {
    unsigned long long checked = 0;
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
         i < (1ull << 32); i += (unsigned long long)gridDim.x * blockDim.x) {
        const float f = __uint_as_float((uint32_t)i);
        record(r, !same(sg::mul_df_rn(f, c), __dmul_rn((double)f, c)), i);
        ++checked;
    }
    atomicAdd(&r->checked, checked);
}

// d2f_rn on n doubles: raw random bit patterns (every exponent), values of
// the float range whose 29 dropped bits are an exact tie, one either side of
// it, zero, all ones or random, and the exponents at the edges of the float
// range.
__global__ void k_d2f(unsigned long long n, unsigned long long seed, Result* r) {
    unsigned long long checked = 0;
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        const uint64_t h1 = sg::rng_bits(seed, 1, i), h2 = sg::rng_bits(seed, 2, i);
        uint64_t bits;
        const int kind = (int)(i % 4);
        if (kind == 0) {
            bits = h1;
        } else {
            uint64_t e;
            if (kind == 1) {
                e = 897 + h2 % 254;                          // float-normal exponents
            } else if (kind == 2) {
                const uint64_t edges[8] = {895, 896, 897, 898, 1149, 1150, 1151, 1152};
                e = edges[h2 % 8];
            } else {
                e = (h2 >> 8) % 2048;                        // any exponent
            }
            const uint32_t low_kinds[6] = {0x10000000u, 0x0FFFFFFFu, 0x10000001u, 0u, 0x1FFFFFFFu,
                                           (uint32_t)(h2 >> 32) & 0x1FFFFFFFu};
            const uint64_t low = low_kinds[(h2 >> 16) % 6];
            const uint64_t mant23 = (h1 >> 3) & 0x7FFFFFull;
            bits = (h1 & (1ull << 63)) | (e << 52) | (mant23 << 29) | low;
        }
        const double d = __longlong_as_double((long long)bits);
        record(r, !same(sg::d2f_rn(d), __double2float_rn(d)), i);
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

double g_c;
unsigned long long g_n, g_seed;

}  // namespace

extern "C" int check_f2d_all(unsigned long long* out) {
    return run([](Result* d) { k_f2d_all<<<152 * 8, 256>>>(d); }, out);
}

extern "C" int check_mul_all(double c, unsigned long long* out) {
    g_c = c;
    return run([](Result* d) { k_mul_all<<<152 * 8, 256>>>(g_c, d); }, out);
}

extern "C" int check_d2f(unsigned long long n, unsigned long long seed, unsigned long long* out) {
    g_n = n;
    g_seed = seed;
    return run([](Result* d) { k_d2f<<<152 * 8, 256>>>(g_n, g_seed, d); }, out);
}

extern "C" int check_muld_all(double c, unsigned long long* out) {
    g_c = c;
    return run([](Result* d) { k_muld_all<<<152 * 8, 256>>>(g_c, d); }, out);
}
