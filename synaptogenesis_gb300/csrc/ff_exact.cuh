// Exact float results of the reference's mixed float/double expressions,
// evaluated in float-float arithmetic with a rounding test.
//
// The Izhikevich STDP updater stores float results of double expressions
// (izhikevich_attributes.cpp:474-505): the weight derivative
//     wd -= (wd - 1e-6) * 1e-4 + dest_spike * src_trace - src_spike * dest_trace
// and the short-term "w"
//     sw += (U - sw) / F + U * (1 - sw) * src_spike.
// GB300 runs FP64 at 1/64 of the FP32 rate, so these are evaluated here with
// pairs of floats instead (Dekker's product and Knuth's sum, both exact; see
// Muller et al., Handbook of Floating-Point Arithmetic, ch. 4-5), giving an
// approximation R of the double result r with a proven bound |R - r| <= B
// (B = 2^-40 times a sum of magnitudes M -- the result's and the terms' whose
// roundings enter it; the float-float steps err by less than 2^-43 M in all
// and the reference's double roundings by less than 2^-50 M, so the bound
// holds with a factor of 8 to spare).  If no float rounding boundary
// (midpoint between consecutive floats) lies within B of R, then (float)r is
// the float nearest R (Ziv's rounding test).  Otherwise the function returns
// false and the caller evaluates the expression in double, exactly as the
// reference does.  Results that are zero, subnormal or near overflow, and
// operands that are not finite, also return false.
//
// The functions compile for the device and for the host (built with
// -ffp-contract=off, so the host checks run the same float operations);
// single-argument paths are also checked on the GPU over every float.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define SG_FF __host__ __device__ __forceinline__
#else
#define SG_FF inline
#endif

namespace sg {
namespace ff {

// Round-to-nearest float operations that are never contracted.
SG_FF float add(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fadd_rn(a, b);
#else
    return a + b;
#endif
}
SG_FF float sub(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fsub_rn(a, b);
#else
    return a - b;
#endif
}
SG_FF float mul(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fmul_rn(a, b);
#else
    return a * b;
#endif
}
SG_FF float fma(float a, float b, float c) {
#ifdef __CUDA_ARCH__
    return __fmaf_rn(a, b, c);
#else
    return std::fmaf(a, b, c);
#endif
}
SG_FF uint32_t bits(float f) {
#ifdef __CUDA_ARCH__
    return __float_as_uint(f);
#else
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
#endif
}
SG_FF float from_bits(uint32_t u) {
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    float f;
    std::memcpy(&f, &u, 4);
    return f;
#endif
}
SG_FF float absf(float f) { return from_bits(bits(f) & 0x7FFFFFFFu); }

// s + e = a + b exactly (Knuth's two-sum; no precondition on |a|, |b|).
SG_FF void two_sum(float a, float b, float& s, float& e) {
    s = add(a, b);
    const float bv = sub(s, a);
    const float av = sub(s, bv);
    e = add(sub(a, av), sub(b, bv));
}

// p + e = a * b exactly (no underflow at the call sites).
SG_FF void two_prod(float a, float b, float& p, float& e) {
    p = mul(a, b);
    e = fma(a, b, -p);
}

// True when every real within B of f + g rounds to f, where f = RN(f + g)
// (so |g| is at most half an ulp of f).  f must be a normal float of
// magnitude at least 2^-101; the nearest rounding boundaries are half an ulp
// away from f, a quarter of f's ulp below a power of two.  The comparison
// leaves a relative margin of 2^-20 for the rounding of |g| + B.
SG_FF bool rounds_to(float f, float g, float B) {
    const uint32_t u = bits(f) & 0x7FFFFFFFu;
    const uint32_t E = u >> 23;
    if (E < 26u || E > 253u) return false;
    const bool toward_zero = ((bits(f) ^ bits(g)) >> 31) != 0u && absf(g) != 0.0f;
    const uint32_t hE = (toward_zero && (u & 0x7FFFFFu) == 0u) ? E - 25u : E - 24u;
    const float lim = mul(from_bits(hE << 23), 0.99999904632568359375f);   // 1 - 2^-20
    return add(absf(g), B) <= lim;
}

constexpr float kBound = 9.094947017729282379e-13f;   // 2^-40

// Weight derivative of the STDP updater: (float)(x - c) with
//   c = ((x - 1e-6) * 1e-4 [+ p] [- q])
// in double, x = wd, p = dest_spike * src_trace and q = src_spike *
// dest_trace (float products, computed by the caller as the reference
// does).  p and q are added only when has_p / has_q: the reference adds a
// zero product there, which leaves the (never zero) partial sum unchanged.
SG_FF bool weight_derivative(float x, float p, bool has_p, float q, bool has_q, float& out) {
    constexpr double A = 0.000001, T = 0.0001;
    constexpr float A1 = (float)A;
    constexpr float A2 = (float)(A - (double)A1);
    constexpr float T1 = (float)T;
    constexpr float T2 = (float)(T - (double)T1);
    const float ax = absf(x), ap = has_p ? absf(p) : 0.0f, aq = has_q ? absf(q) : 0.0f;
    if (!(ax < 0x1p100f && ap < 0x1p100f && aq < 0x1p100f)) return false;   // NaN, inf, huge
    float s1, e1;
    two_sum(x, -A1, s1, e1);                 // s1 + e1 = x - A1
    const float t_lo = sub(e1, A2);          // x - A ~ s1 + t_lo
    float c_hi, c_lo;
    two_prod(s1, T1, c_hi, c_lo);            // (x - A) T ~ c_hi + c_lo
    c_lo = add(c_lo, add(mul(s1, T2), mul(t_lo, T1)));
    if (has_p) {
        float a, b;
        two_sum(c_hi, p, a, b);
        c_hi = a;
        c_lo = add(b, c_lo);
    }
    if (has_q) {
        float a, b;
        two_sum(c_hi, -q, a, b);
        c_hi = a;
        c_lo = add(b, c_lo);
    }
    float r1, r2;
    two_sum(x, -c_hi, r1, r2);
    r2 = sub(r2, c_lo);
    float f, g;
    two_sum(r1, r2, f, g);                   // R = f + g exactly
    // the bound's scale: the result, the spike terms, and (x - A) T, whose
    // rounding errors are the only ones that involve x and A
    const float M = add(add(absf(r1), add(ap, aq)), mul(add(ax, A1), T1));
    if (!rounds_to(f, g, mul(M, kBound))) return false;
    out = f;
    return true;
}

// Short-term "w" of the STP update: (float)(sw + d) with
//   d = (U - sw) / F [+ U * (float)(1 - sw)]   (the second term on a spike)
// in double; U and F are the connection opcode's constants (0.5, 1000 for
// "add"; 0.2, 20 for "sub").
template <bool SUB>
SG_FF bool short_term_w(float sw, bool spike, float& out) {
    constexpr double U = SUB ? 0.2 : 0.5;
    constexpr int F = SUB ? 20 : 1000;
    constexpr float U1 = (float)U;
    constexpr float U2 = (float)(U - (double)U1);
    constexpr float RF = (float)(1.0 / F);
    const float a = absf(sw);
    if (!(a < 0x1p100f)) return false;
    float d1, d2;
    two_sum(U1, -sw, d1, d2);
    d2 = add(d2, U2);                        // U - sw ~ d1 + d2
    const float q1 = mul(d1, RF);
    const float rho = fma(-q1, (float)F, d1);
    const float q2 = mul(add(rho, d2), RF);  // (U - sw) / F ~ q1 + q2
    float hi = q1, lo = q2, av = 0.0f;
    if (spike) {
        const float f1 = sub(1.0f, sw);
        float v1, v2;
        two_prod(U1, f1, v1, v2);
        v2 = add(v2, mul(U2, f1));           // U * f1 ~ v1 + v2
        float s, e;
        two_sum(q1, v1, s, e);
        hi = s;
        lo = add(e, add(q2, v2));
        av = absf(v1);
    }
    float r1, r2;
    two_sum(sw, hi, r1, r2);
    r2 = add(r2, lo);
    float f, g;
    two_sum(r1, r2, f, g);
    const float M = add(add(a, mul(absf(d1), RF)), av);
    if (!rounds_to(f, g, mul(M, kBound))) return false;
    out = f;
    return true;
}

}  // namespace ff
}  // namespace sg
