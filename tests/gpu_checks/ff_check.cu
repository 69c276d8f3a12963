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

// every float bit pattern: (float)((double)p * 0.933)
__global__ void k_product_all(Result* r) {
    const float c1 = (float)0.933, c2 = (float)(0.933 - (double)c1);
    unsigned long long checked = 0, fallbacks = 0;
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
         i < (1ull << 32); i += (unsigned long long)gridDim.x * blockDim.x) {
        const float p = __uint_as_float((uint32_t)i);
        float out;
        ++checked;
        if (!sg::ff::product(p, c1, c2, out)) { ++fallbacks; continue; }
        record(r, !same(out, __double2float_rn(__dmul_rn((double)p, 0.933))), i);
    }
    atomicAdd(&r->checked, checked);
    atomicAdd(&r->fallbacks, fallbacks);
}

// every float bit pattern: (float)((double)p * c) and (float)((double)x + k)
__global__ void k_product_c_all(double c, Result* r) {
    const float c1 = (float)c, c2 = (float)(c - (double)c1);
    unsigned long long checked = 0, fallbacks = 0;
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
         i < (1ull << 32); i += (unsigned long long)gridDim.x * blockDim.x) {
        const float p = __uint_as_float((uint32_t)i);
        float out;
        ++checked;
        if (!sg::ff::product(p, c1, c2, out)) { ++fallbacks; continue; }
        record(r, !same(out, __double2float_rn(__dmul_rn((double)p, c))), i);
    }
    atomicAdd(&r->checked, checked);
    atomicAdd(&r->fallbacks, fallbacks);
}

__global__ void k_add_const_all(double k, Result* r) {
    const float k1 = (float)k, k2 = (float)(k - (double)k1);
    unsigned long long checked = 0, fallbacks = 0;
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
         i < (1ull << 32); i += (unsigned long long)gridDim.x * blockDim.x) {
        const float x = __uint_as_float((uint32_t)i);
        float out;
        ++checked;
        if (!sg::ff::add_const(x, k1, k2, out)) { ++fallbacks; continue; }
        record(r, !same(out, __double2float_rn(__dadd_rn((double)x, k))), i);
    }
    atomicAdd(&r->checked, checked);
    atomicAdd(&r->fallbacks, fallbacks);
}

// every float bit pattern: div_int<D>(a) == a / D (IEEE)
template <int D>
__global__ void k_div_all(Result* r) {
    unsigned long long checked = 0;
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
         i < (1ull << 32); i += (unsigned long long)gridDim.x * blockDim.x) {
        const float a = __uint_as_float((uint32_t)i);
        ++checked;
        record(r, !same(sg::ff::div_int<D>(a), __fdiv_rn(a, (float)D)), i);
    }
    atomicAdd(&r->checked, checked);
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

// izhikevich_attributes.cpp:155-156 and 163-168 in double
__device__ float ref_dv(float v, float rec, float cur) {
    double d = __dmul_rn(__dmul_rn(0.04, (double)v), (double)v);
    d = __dadd_rn(d, (double)__fmul_rn(5.0f, v));
    d = __dadd_rn(d, 140.0);
    d = __dsub_rn(d, (double)rec);
    d = __dadd_rn(d, (double)cur);
    return __double2float_rn(d);
}
__device__ float ref_tau(float v, float dv) {
    return __double2float_rn(__dmul_rn(__ddiv_rn((double)dv, __dadd_rn(__dsub_rn(30.0, (double)v),
                                                                         (double)dv)), 0.1));
}
__device__ float ref_voltage(float v, float drive, float sum_c) {
    return __double2float_rn(__ddiv_rn(__dadd_rn((double)v, __dmul_rn(0.1, (double)drive)),
                                       __dadd_rn(1.0, __dmul_rn(0.1, (double)sum_c))));
}

// random Izhikevich substeps (operands as in the host check)
__global__ void k_iz_random(unsigned long long n, unsigned long long seed, Result* dv, Result* vr,
                            Result* tr) {
    unsigned long long checked = 0, fb_dv = 0, fb_v = 0, fb_t = 0;
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        const uint64_t z0 = mix(seed * 0x100000001B3ull + i), z1 = mix(z0), z2 = mix(z1),
                       z3 = mix(z2);
        const uint32_t sel = (uint32_t)(z0 >> 58);
        const float v = sel < 4 ? -65.0f : sel < 6 ? -50.0f
                        : -100.0f + 130.0f * ((float)((z0 >> 11) & 0xFFFFFF) * (1.0f / 16777216.0f));
        const float rec = -30.0f + 60.0f * ((float)((z1 >> 11) & 0xFFFFFF) * (1.0f / 16777216.0f));
        const float cur = draw(z2, 100.0f);
        const float sum_c = fabsf(draw(z3, 10.0f));
        float out;
        ++checked;
        if (!sg::ff::iz_delta_v(v, rec, cur, out)) ++fb_dv;
        else record(dv, !same(out, ref_dv(v, rec, cur)), i);
        float d1, d2;
        sg::ff::iz_denominator(sum_c, d1, d2);
        if (!sg::ff::iz_voltage(v, cur, d1, d2, 1.0f / d1, out)) ++fb_v;
        else record(vr, !same(out, ref_voltage(v, cur, sum_c)), i);
        // the threshold-crossing substep: dv in [1, 1024), v past 30 by up to dv / 10
        const float dvs = ldexpf(1.0f + (v + 100.0f) / 130.0f, (int)(sum_c * 1e6f) % 10);
        const float vs = 30.0f + 0.1f * dvs * ((rec + 30.0f) / 60.0f) + 1e-3f;
        if (!sg::ff::iz_adjusted_tau(vs, dvs, out)) ++fb_t;
        else record(tr, !same(out, ref_tau(vs, dvs)), i);
    }
    atomicAdd(&tr->checked, checked);
    atomicAdd(&tr->fallbacks, fb_t);
    atomicAdd(&dv->checked, checked);
    atomicAdd(&dv->fallbacks, fb_dv);
    atomicAdd(&vr->checked, checked);
    atomicAdd(&vr->fallbacks, fb_v);
}

int run(void (*launch)(Result*), unsigned long long* out) {
    Result* d = nullptr;
    if (cudaMalloc(&d, 3 * sizeof(Result)) != cudaSuccess) return 1;
    Result h[3] = {{0, 0, 0, ~0ull}, {0, 0, 0, ~0ull}, {0, 0, 0, ~0ull}};
    cudaMemcpy(d, h, sizeof(h), cudaMemcpyHostToDevice);
    launch(d);
    cudaError_t e = cudaDeviceSynchronize();
    cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
    cudaFree(d);
    for (int k = 0; k < 3; ++k) {
        out[4 * k + 0] = h[k].mismatches;
        out[4 * k + 1] = h[k].checked;
        out[4 * k + 2] = h[k].fallbacks;
        out[4 * k + 3] = h[k].first;
    }
    return e == cudaSuccess ? 0 : 2;
}

}  // namespace

extern "C" {

int check_wd_all(unsigned long long* out) {
    return run([](Result* d) { k_wd_all<<<152 * 8, 256>>>(d); }, out);
}

int check_product_all(unsigned long long* out) {
    return run([](Result* d) { k_product_all<<<152 * 8, 256>>>(d); }, out);
}

int check_product_c_all(double c, unsigned long long* out) {
    static double cc;
    cc = c;
    return run([](Result* d) { k_product_c_all<<<152 * 8, 256>>>(cc, d); }, out);
}

int check_add_const_all(double k, unsigned long long* out) {
    static double kk;
    kk = k;
    return run([](Result* d) { k_add_const_all<<<152 * 8, 256>>>(kk, d); }, out);
}

int check_div_all(int D, unsigned long long* out) {
    if (D == 60) return run([](Result* d) { k_div_all<60><<<152 * 8, 256>>>(d); }, out);
    if (D == 700) return run([](Result* d) { k_div_all<700><<<152 * 8, 256>>>(d); }, out);
    if (D == 800) return run([](Result* d) { k_div_all<800><<<152 * 8, 256>>>(d); }, out);
    return 1;
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

int check_iz_random(unsigned long long n, unsigned long long seed, unsigned long long* out) {
    static unsigned long long sn, ss;
    sn = n;
    ss = seed;
    // three results: delta_v in out[0..3], voltage in out[4..7], tau in out[8..11]
    return run([](Result* d) { k_iz_random<<<152 * 8, 256>>>(sn, ss, d, d + 1, d + 2); }, out);
}

}  // extern "C"
