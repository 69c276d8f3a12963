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
#endif

}  // namespace sg
