// Test-only kernels: the float-float evaluations of
// synaptogenesis_gb300/csrc/ff_exact.cuh against the reference's double
// expressions evaluated on the GPU's FP64 pipe, bit for bit, wherever the
// rounding test accepts.  Built by tests/test_gpu_ff_exact.py with nvcc into
// a temporary shared library.
#include <cuda_runtime.h>

#include <cstdint>

#include "ff_exact.cuh"

namespace {

struct Result {
    unsigned long long mismatches, checked, fallbacks, first;
};

__device__ void record(Result* r, bool bad, unsigned long long id) {
    if (bad) {
        atomicAdd(&r->mismatches, 1ull);
        atomicMin(&r->first, id);
    }
}

__device__ bool same(float a, float b) {
    return __float_as_uint(a) == __float_as_uint(b) || (a != a && b != b);
}

// izhikevich_attributes.cpp:486-490 in double (the spike products always added)
__device__ float ref_wd(float x, float p, float q) {
    const double c = __dsub_rn(__dadd_rn(__dmul_rn(__dsub_rn((double)x, 0.000001), 0.0001),
                                         (double)p), (double)q);
    return __double2float_rn(__dsub_rn((double)x, c));
}

// izhikevich_attributes.cpp:501-503 in double
__device__ float ref_sw(float w, bool spike, bool sub) {
    const double U = sub ? 0.2 : 0.5;
    const double F = sub ? 20.0 : 1000.0;
    const double inc = __dadd_rn(__ddiv_rn(__dsub_rn(U, (double)w), F),
                                 __dmul_rn(__dmul_rn(U, (double)__fsub_rn(1.0f, w)),
                                           spike ? 1.0 : 0.0));
    return __double2float_rn(__dadd_rn((double)w, inc));
}

__device__ uint64_t mix(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// a float in [-lim, lim] with a log-uniform magnitude over 40 octaves, or a
// special value (zero, a power of two, a neighbour of 1e-6)
__device__ float draw(uint64_t z, float lim) {
    const uint32_t sel = (uint32_t)(z >> 56);
    if (sel < 4) return 0.0f;
    if (sel < 12) return ldexpf((z & 1) ? -1.0f : 1.0f, -(int)((z >> 8) % 40));
    if (sel < 20) return __uint_as_float(__float_as_uint(0.000001f) + (int32_t)((z >> 8) % 64) - 32);
    const float u = (float)((z >> 11) & 0xFFFFFF) * (1.0f / 16777216.0f);
    const float m = lim * exp2f(-40.0f * u);
    return (z & 1) ? -m : m;
}

__global__ void k_wd_all(Result* r) {
    unsigned long long checked = 0, fallbacks = 0;
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
         i < (1ull << 32); i += (unsigned long long)gridDim.x * blockDim.x) {
        const float x = __uint_as_float((uint32_t)i);
        float out;
        ++checked;
        if (!sg::ff::weight_derivative(x, 0.0f, false, 0.0f, false, out)) { ++fallbacks; continue; }
        record(r, !same(out, ref_wd(x, 0.0f, 0.0f)), i);
    }
    atomicAdd(&r->checked, checked);
    atomicAdd(&r->fallbacks, fallbacks);
}

template <bool SUB>
__global__ void k_sw_all(bool spike, Result* r) {
    unsigned long long checked = 0, fallbacks = 0;
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
         i < (1ull << 32); i += (unsigned long long)gridDim.x * blockDim.x) {
        const float w = __uint_as_float((uint32_t)i);
        float out;
        ++checked;
        if (!sg::ff::short_term_w<SUB>(w, spike, out)) { ++fallbacks; continue; }
        record(r, !same(out, ref_sw(w, spike, SUB)), i);
    }
    atomicAdd(&r->checked, checked);
    atomicAdd(&r->fallbacks, fallbacks);
}

// random (x, p, q): x up to 0.05, p and q up to 0.01, each term present with
// probability 1/2
__global__ void k_wd_random(unsigned long long n, unsigned long long seed, Result* r) {
    unsigned long long checked = 0, fallbacks = 0;
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        const uint64_t z0 = mix(seed * 0x100000001B3ull + i), z1 = mix(z0), z2 = mix(z1);
        const float x = draw(z0, 0.05f);
        const bool hp = (z1 & 2) != 0, hq = (z2 & 2) != 0;
        const float p = hp ? draw(z1, 0.01f) : 0.0f;
        const float q = hq ? draw(z2, 0.01f) : 0.0f;
        float out;
        ++checked;
        if (!sg::ff::weight_derivative(x, p, hp, q, hq, out)) { ++fallbacks; continue; }
        record(r, !same(out, ref_wd(x, p, q)), i);
    }
    atomicAdd(&r->checked, checked);
    atomicAdd(&r->fallbacks, fallbacks);
}

int run(void (*launch)(Result*), unsigned long long* out) {
    Result* d = nullptr;
    if (cudaMalloc(&d, sizeof(Result)) != cudaSuccess) return 1;
    Result h{0, 0, 0, ~0ull};
    cudaMemcpy(d, &h, sizeof(h), cudaMemcpyHostToDevice);
    launch(d);
    cudaError_t e = cudaDeviceSynchronize();
    cudaMemcpy(&h, d, sizeof(h), cudaMemcpyDeviceToHost);
    cudaFree(d);
    out[0] = h.mismatches;
    out[1] = h.checked;
    out[2] = h.fallbacks;
    out[3] = h.first;
    return e == cudaSuccess ? 0 : 2;
}

}  // namespace

extern "C" {

int check_wd_all(unsigned long long* out) {
    return run([](Result* d) { k_wd_all<<<152 * 8, 256>>>(d); }, out);
}

int check_sw_all(int sub, int spike, unsigned long long* out) {
    static bool s;
    s = spike != 0;
    if (sub) return run([](Result* d) { k_sw_all<true><<<152 * 8, 256>>>(s, d); }, out);
    return run([](Result* d) { k_sw_all<false><<<152 * 8, 256>>>(s, d); }, out);
}

int check_wd_random(unsigned long long n, unsigned long long seed, unsigned long long* out) {
    static unsigned long long sn, ss;
    sn = n;
    ss = seed;
    return run([](Result* d) { k_wd_random<<<152 * 8, 256>>>(sn, ss, d); }, out);
}

}  // extern "C"
