// Correctly rounded double division by a divisor whose reciprocal is known.
//
// Markstein's theorem (P. Markstein, "Computation of elementary functions on
// the IBM RISC System/6000 processor", IBM J. Res. Dev. 34(1), 1990; also
// Muller et al., Handbook of Floating-Point Arithmetic, ch. 4): in binary
// floating point with round-to-nearest, if y = RN(1/b) and q is within one
// ulp of a/b, then r = a - b q is exactly representable (one fused
// multiply-add computes it) and RN(q + r y) = RN(a/b).  With q = RN(a y) the
// quotient costs one multiply and two fused multiply-adds instead of a full
// division.  Outside the range where no intermediate can underflow or
// overflow (and for zero, infinite or NaN quotients) the IEEE division is
// used instead, so the result equals a / b for every input.
#pragma once

#include <cstdint>

namespace sg {

#ifdef __CUDACC__
__device__ __forceinline__ int biased_exponent(double x) {
    return (__double2hiint(x) >> 20) & 0x7FF;
}

__device__ __forceinline__ double div_rn_recip(double a, double b, double y) {
    const double q = __dmul_rn(a, y);
    // a, b and q at least 2^-959 and below 2^961 in magnitude: r = a - b q
    // (about 2^-53 a) stays a normal number and nothing overflows
    const int ea = biased_exponent(a), eb = biased_exponent(b), eq = biased_exponent(q);
    if (ea < 64 || ea > 1983 || eb < 64 || eb > 1983 || eq < 64 || eq > 1983) {
        // a = +-0: a * y has the sign of a / b (and is NaN where a / b is)
        if ((__double2hiint(a) & 0x7FFFFFFF) == 0 && __double2loint(a) == 0) return q;
        return a / b;
    }
    const double r = __fma_rn(-q, b, a);
    return __fma_rn(r, y, q);
}

// a / F for a small positive integer constant F (2..1024), correctly
// rounded (nearest, ties to even) in integer arithmetic: the significand m
// (53 bits) shifted left by 11 is divided by F (a multiply-high for a
// constant divisor), and the quotient, with the remainder as sticky bit, is
// rounded to 53 bits.  Zero, subnormal, infinite and NaN operands and
// quotients outside the normal range use the IEEE division.
template <int F>
__device__ __forceinline__ double div_const_rn(double a) {
    static_assert(F >= 2 && F <= 1024, "divisor out of range");
    const uint64_t bits = (uint64_t)__double_as_longlong(a);
    const int e = (int)((bits >> 52) & 0x7FF);
    if (e != 0 && e != 0x7FF) {
        const uint64_t N = ((bits & 0xFFFFFFFFFFFFFull) | (1ull << 52)) << 11;   // [2^63, 2^64)
        const uint64_t Q = N / (uint64_t)F, R = N - Q * (uint64_t)F;
        int sh = 63 - __clzll((long long)Q) - 52;        // 1..11: 2^53 <= Q < 2^63
        uint64_t q = Q >> sh;
        const uint64_t rem = Q & ((1ull << sh) - 1), half = 1ull << (sh - 1);
        if (rem > half || (rem == half && (R != 0 || (q & 1)))) ++q;
        if (q >> 53) { q >>= 1; ++sh; }
        const int E = e - 11 + sh;                        // biased exponent of the quotient
        if (E >= 1 && E <= 2046)
            return __longlong_as_double((long long)((bits & (1ull << 63)) | ((uint64_t)E << 52) |
                                                    (q & 0xFFFFFFFFFFFFFull)));
    }
    return a / (double)F;
}
#endif

}  // namespace sg
