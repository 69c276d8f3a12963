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
    if (E - 26u > 227u) return false;                  // E outside [26, 253]
    // a power of two: the boundary below is a quarter of its ulp away (taken
    // on both sides)
    const uint32_t hE = (u & 0x7FFFFFu) == 0u ? E - 25u : E - 24u;
    const float lim = mul(from_bits(hE << 23), 0.99999904632568359375f);   // 1 - 2^-20
    return add(absf(g), B) <= lim;
}

constexpr float kBound = 9.094947017729282379e-13f;   // 2^-40
constexpr float kBound4 = 2.273736754432320595e-13f;  // 2^-42
constexpr float kBound5 = 1.136868377216160297e-13f;  // 2^-43

// a / D for a float a and a small positive integer D, correctly rounded: the
// product with the rounded reciprocal corrected by one fused multiply-add
// (Markstein's scheme).  Checked against IEEE division over every float a in
// [2^-100, 2^100] for the divisors used (20, 60, 700, 800, 1000); other
// operands (zero, tiny, huge, non-finite) take the IEEE division.
template <int D>
SG_FF float div_int(float a) {
    constexpr float y = (float)(1.0 / D);
    const float m = absf(a);
    if (!(m >= 7.888609052210118e-31f && m <= 1.2676506002282294e30f))   // 2^-100, 2^100
        return a / (float)D;
    const float q = mul(a, y);
    const float r = fma(-q, (float)D, a);
    return fma(r, y, q);
}

// (float)((double)p * c) for a double constant c ~ c1 + c2 (two floats, c2
// the rounded remainder): Dekker's product plus the remainder's, error below
// 2^-45 |p c| in all, bound 2^-40 |f|.  Operands below 2^-50 are scaled by
// 2^64 first (exact, as are both roundings of a result in the normal float
// range); results below 2^-126 return false.
SG_FF bool product(float p, float c1, float c2, float& out) {
    const bool small = absf(p) < 8.881784197001252323e-16f;             // 2^-50
    const float ps = small ? mul(p, 18446744073709551616.0f) : p;       // 2^64
    float h, l;
    two_prod(ps, c1, h, l);
    l = add(l, mul(ps, c2));
    float f, g;
    two_sum(h, l, f, g);
    if (!rounds_to(f, g, mul(absf(f), kBound))) return false;
    if (small) {
        if (absf(f) < 2.168404344971008868e-19f) return false;          // 2^-62: result below 2^-126
        f = mul(f, 5.421010862427522170e-20f);                          // 2^-64, exact for normal results
    }
    out = f;
    return true;
}

// (float)((double)x + k) for a double constant k ~ k1 + k2 (two floats, k2
// the rounded remainder): the exact sum of x and k1 plus the remainder's,
// which errs by at most 2^-24 (|e| + |k2|) <= 2^-48 (|s| + |k1|), s = RN(x +
// k1); the double addition it stands for errs by at most 2^-53 |x + k| and
// the split of k by 2^-48 |k1|: the bound 2^-43 (|s| + |k1|) covers all three
// with a factor of 10 to spare.
SG_FF bool add_const(float x, float k1, float k2, float& out) {
    float s, e;
    two_sum(x, k1, s, e);
    e = add(e, k2);
    float f, g;
    two_sum(s, e, f, g);
    if (!rounds_to(f, g, mul(add(absf(s), absf(k1)), kBound5))) return false;
    out = f;
    return true;
}

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
    // NaN, infinite and huge operands give a non-finite or huge f, which the
    // rounding test rejects
    const float ax = absf(x), ap = has_p ? absf(p) : 0.0f, aq = has_q ? absf(q) : 0.0f;
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


// Izhikevich voltage derivative of one Euler substep
// (izhikevich_attributes.cpp:155-156):
//   delta_v = (float)(0.04 * v * v + (5 * v) + 140 - recovery + current)
// with the products and sums in double and 5 * v a float product.  With
// u = 2^-24, the float-float value errs from the exact real expression by at
// most u^2 (11 |P| + 10 S), P = 0.04 v v and S the largest partial sum, and
// the reference's double roundings by less than 2^-53 (2 |P| + 5 S); the
// bound used is 2^-43 (|P| + S), a factor of 2.9 above their sum.
SG_FF bool iz_delta_v(float v, float recovery, float current, float& out) {
    constexpr double C = 0.04;
    constexpr float C1 = (float)C;
    constexpr float C2 = (float)(C - (double)C1);
    float h, l;
    two_prod(v, C1, h, l);
    l = add(l, mul(v, C2));                  // 0.04 v ~ h + l
    float h2, l2;
    two_prod(h, v, h2, l2);
    l2 = add(l2, mul(l, v));                 // 0.04 v v ~ h2 + l2
    const float v5 = mul(5.0f, v);
    float s, e;
    two_sum(h2, v5, s, e);
    l2 = add(e, l2);
    float smax = absf(s);
    two_sum(s, 140.0f, s, e);
    l2 = add(e, l2);
    smax = fmaxf(smax, absf(s));
    two_sum(s, -recovery, s, e);
    l2 = add(e, l2);
    smax = fmaxf(smax, absf(s));
    two_sum(s, current, s, e);
    l2 = add(e, l2);
    smax = fmaxf(smax, absf(s));
    float f, g;
    two_sum(s, l2, f, g);
    if (!rounds_to(f, g, mul(add(absf(h2), smax), kBound5))) return false;
    out = f;
    return true;
}

// The implicit voltage step of the substep (izhikevich_attributes.cpp:163-168):
//   voltage = (float)((v + 0.1 * drive) / den),  den = 1 + 0.1 * sum_c
// in double, where drive is the float sum the reference forms and den comes
// from iz_denominator (den ~ d1 + d2, rd = 1 / d1 to float precision).
SG_FF void iz_denominator(float sum_c, float& d1, float& d2) {
    constexpr double T = 0.1;
    constexpr float T1 = (float)T;
    constexpr float T2 = (float)(T - (double)T1);
    float b1, b2;
    two_prod(sum_c, T1, b1, b2);
    b2 = add(b2, mul(sum_c, T2));
    float e;
    two_sum(1.0f, b1, d1, e);
    d2 = add(e, b2);
}

SG_FF bool iz_voltage(float v, float drive, float d1, float d2, float rd, float& out) {
    constexpr double T = 0.1;
    constexpr float T1 = (float)T;
    constexpr float T2 = (float)(T - (double)T1);
    float a1, a2;
    two_prod(drive, T1, a1, a2);
    a2 = add(a2, mul(drive, T2));            // 0.1 drive ~ a1 + a2
    float n1, n2;
    two_sum(v, a1, n1, n2);
    n2 = add(n2, a2);                        // numerator ~ n1 + n2
    const float q1 = mul(n1, rd);
    float p1, p2;
    two_prod(q1, d1, p1, p2);                // q1 d1 exactly
    // numerator - q1 den, to float-float accuracy
    const float r = sub(add(sub(sub(n1, p1), p2), n2), mul(q1, d2));
    const float q2 = mul(r, rd);
    float f, g;
    two_sum(q1, q2, f, g);
    const float M = add(mul(add(absf(v), absf(a1)), rd), absf(f));
    if (!rounds_to(f, g, mul(M, kBound4))) return false;
    out = f;
    return true;
}

// Recovery time constant of the substep that crosses the threshold
// (izhikevich_attributes.cpp:175-179):
//   tau = (float)(delta_v / (30.0 - v + delta_v) * 0.1)
// in double; 30 - v is exact.  The quotient's float-float error is below
// 2^-44 of it plus 2^-48 of (|30 - v| + |delta_v|) / |denominator| of it.
SG_FF bool iz_adjusted_tau(float v, float delta_v, float& out) {
    constexpr double T = 0.1;
    constexpr float T1 = (float)T;
    constexpr float T2 = (float)(T - (double)T1);
    float a1, a2;
    two_sum(30.0f, -v, a1, a2);              // 30 - v exactly
    float b1, b2;
    two_sum(a1, delta_v, b1, b2);
    b2 = add(b2, a2);                        // denominator ~ b1 + b2
    const float r = 1.0f / b1;
    const float q1 = mul(delta_v, r);
    float p1, p2;
    two_prod(q1, b1, p1, p2);
    const float res = sub(sub(sub(delta_v, p1), p2), mul(q1, b2));
    const float q2 = mul(res, r);            // quotient ~ q1 + q2
    float t1, t2;
    two_prod(q1, T1, t1, t2);
    t2 = add(t2, add(mul(q1, T2), mul(q2, T1)));
    float f, g;
    two_sum(t1, t2, f, g);
    const float M = mul(absf(f), add(2.0f, mul(add(absf(a1), absf(delta_v)), absf(r))));
    if (!rounds_to(f, g, mul(M, kBound4))) return false;
    out = f;
    return true;
}

}  // namespace ff
}  // namespace sg
