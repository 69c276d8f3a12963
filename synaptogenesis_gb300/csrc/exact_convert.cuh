// Exact float <-> double conversions and a float-by-double-constant product
// in integer arithmetic.
//
// GB300 executes FP64 instructions at 1/64 of the FP32 rate, and conversions
// between float and double occupy that same pipe.  The Izhikevich update and
// the STDP updater evaluate the reference's mixed float/double expressions
// exactly, so they convert on almost every operation.  The conversions below
// produce the IEEE 754 results (round to nearest, ties to even, for double ->
// float) from the bit patterns with a handful of integer instructions; the
// rare operands outside the normal ranges (zero is handled, subnormal,
// infinite and NaN values are not) take the hardware conversion, so every
// result equals the hardware's bit for bit.
#pragma once

#include <cstdint>

namespace sg {

#ifdef __CUDACC__
// The rare operands' hardware paths, kept out of line so that the compiler
// branches around them instead of predicating their FP64 instructions into
// every lane.
static __device__ __noinline__ double f2d_hw(float f) { return (double)f; }
static __device__ __noinline__ float d2f_hw(double d) { return __double2float_rn(d); }
static __device__ __noinline__ double mul_df_hw(float f, double c) { return __dmul_rn((double)f, c); }
static __device__ __noinline__ float mul_fd_hw(float f, double c) { return __double2float_rn(__dmul_rn((double)f, c)); }

// (double)f, exact.
__device__ __forceinline__ double f2d_exact(float f) {
    const uint32_t u = __float_as_uint(f);
    const uint32_t e = (u >> 23) & 0xFFu;
    if (e - 1u < 254u) {                        // normal: rebias 127 -> 1023
        const uint32_t hi = (u & 0x80000000u) | ((e + 896u) << 20) | ((u >> 3) & 0xFFFFFu);
        return __hiloint2double((int)hi, (int)(u << 29));
    }
    if ((u << 1) == 0u) return __hiloint2double((int)(u & 0x80000000u), 0);   // +-0
    return f2d_hw(f);                           // subnormal, infinite, NaN
}

// (float)d, round to nearest even.
__device__ __forceinline__ float d2f_rn(double d) {
    const uint32_t hi = (uint32_t)__double2hiint(d), lo = (uint32_t)__double2loint(d);
    const uint32_t e = (hi >> 20) & 0x7FFu;
    if (e - 897u < 254u) {                      // float exponent e - 896 in 1..254
        uint32_t r = (hi & 0x80000000u) | ((e - 896u) << 23) | ((hi & 0xFFFFFu) << 3) | (lo >> 29);
        const uint32_t rem = lo & 0x1FFFFFFFu;  // the 29 dropped bits
        // ties to even; a carry out of the mantissa raises the exponent, up
        // to infinity, as rounding does
        if (rem > 0x10000000u || (rem == 0x10000000u && (r & 1u))) r += 1u;
        return __uint_as_float(r);
    }
    if (((hi << 1) | lo) == 0u) return __uint_as_float(hi & 0x80000000u);    // +-0
    return d2f_hw(d);                           // float subnormal, overflow, inf, NaN
}

// (double)f * c for a positive normal double c (a constant at the call
// sites): the 77-bit product of the significands rounded to nearest even.
__device__ __forceinline__ double mul_df_rn(float f, double c) {
    const uint64_t cb = (uint64_t)__double_as_longlong(c);
    const uint64_t mc = (cb & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    const int ec = (int)((cb >> 52) & 0x7FF) - 1023;
    const uint32_t u = __float_as_uint(f);
    const uint32_t e = (u >> 23) & 0xFFu;
    if (e - 1u < 254u) {
        const uint64_t mf = (u & 0x7FFFFFu) | 0x800000u;
        const uint64_t lo = mc * mf, hi = __umul64hi(mc, mf);
        const int top = (int)(hi >> 12) & 1;
        const int sh = 23 + top;
        uint64_t m = (lo >> sh) | (hi << (64 - sh));
        const uint64_t rem = lo & ((1ull << sh) - 1), half = 1ull << (sh - 1);
        int ex = (int)e - 127 + ec + top;
        m += (rem > half || (rem == half && (m & 1))) ? 1 : 0;
        if (m >> 53) { m >>= 1; ++ex; }
        if (ex >= -1022 && ex <= 1023)
            return __longlong_as_double((long long)(((uint64_t)(u & 0x80000000u) << 32) |
                                                    ((uint64_t)(ex + 1023) << 52) |
                                                    (m & 0xFFFFFFFFFFFFFull)));
    } else if ((u << 1) == 0u) {
        return __hiloint2double((int)(u & 0x80000000u), 0);      // +-0 * c = +-0
    }
    return mul_df_hw(f, c);
}

// (float)(f * c) for a positive normal double c (a constant at the call
// sites, so its significand and exponent fold at compile time): the double
// product rounded to nearest even (53 bits), then to float (24 bits) -- the
// two roundings the mixed expression performs.
__device__ __forceinline__ float mul_fd_rn(float f, double c) {
    const uint64_t cb = (uint64_t)__double_as_longlong(c);
    const uint64_t mc = (cb & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    const int ec = (int)((cb >> 52) & 0x7FF) - 1023;
    const uint32_t u = __float_as_uint(f);
    const uint32_t e = (u >> 23) & 0xFFu;
    if (e - 1u < 254u) {
        const uint64_t mf = (u & 0x7FFFFFu) | 0x800000u;         // 24 bits
        // 77-bit product in [2^75, 2^77): hi holds bits 64.., lo bits 0..63
        const uint64_t lo = mc * mf, hi = __umul64hi(mc, mf);
        const int top = (int)(hi >> 12) & 1;                      // bit 76 set?
        const int sh = 23 + top;                                  // bits below the 53 kept
        uint64_t m = (lo >> sh) | (hi << (64 - sh));              // 53 bits
        const uint64_t rem = lo & ((1ull << sh) - 1), half = 1ull << (sh - 1);
        int ex = (int)e - 127 + ec + top;
        m += (rem > half || (rem == half && (m & 1))) ? 1 : 0;
        if (m >> 53) { m >>= 1; ++ex; }
        // 53 -> 24 bits, ties to even
        uint32_t m24 = (uint32_t)(m >> 29);
        const uint32_t r2 = (uint32_t)m & 0x1FFFFFFFu;
        m24 += (r2 > 0x10000000u || (r2 == 0x10000000u && (m24 & 1u))) ? 1u : 0u;
        if (m24 >> 24) { m24 >>= 1; ++ex; }
        if (ex >= -126 && ex <= 127)
            return __uint_as_float((u & 0x80000000u) | ((uint32_t)(ex + 127) << 23) | (m24 & 0x7FFFFFu));
    } else if ((u << 1) == 0u) {
        return f;                                                 // +-0 * c = +-0
    }
    return mul_fd_hw(f, c);
}

#endif

}  // namespace sg
