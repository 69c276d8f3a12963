// Izhikevich neuron integration (src/core/state/impl/izhikevich_attributes.cpp:102-213),
// shared by the per-layer update kernel and the batched instance runner so
// both execute the same float/double expression sequence.
#pragma once

#include "exact_convert.cuh"
#include "exact_div.cuh"
#include "ff_exact.cuh"

namespace sg {

#ifdef __CUDACC__
// Up to 10 hybrid-Euler substeps that stop once v >= 30 (NaN -> 30), with the
// conductance-implicit voltage update and the recovery step whose time
// constant is adjusted on the substep that crosses threshold.
//
// Every operation is the reference's, in its types and order (the double
// literals make the voltage arithmetic double; each double operation is
// written out as the IEEE intrinsic C++ promotion implies), with four
// rewrites that leave each result bit-identical and save FP64 instructions:
//  * comparisons with 30.0 are float comparisons (30 is a float and
//    float -> double conversion is exact);
//  * the conductance sum and the implicit-update denominator do not change
//    within the step and are computed once;
//  * the division by that denominator uses its correctly rounded reciprocal
//    (div_rn_recip, exact);
//  * float <-> double conversions and the products of a float with a double
//    constant run in integer arithmetic (f2d_exact, d2f_rn, mul_df_rn), off
//    the FP64 pipe.
__device__ __forceinline__ void iz_integrate(float& voltage, float& recovery, float ampa_c,
                                             float nmda_c, float gabaa_c, float gabab_c, float mf,
                                             float base_current, float a, float b) {
    if (!(voltage < 30.0f)) return;
    const float sum_c = ampa_c + nmda_c + gabaa_c + gabab_c;
    const double den = __dadd_rn(1.0, mul_df_rn(sum_c, 0.1));   // 1 + (0.1 * sum_c)
    const double rden = 1.0 / den;
    for (int i = 0; (i < 10) && (voltage < 30.0f); ++i) {
        float current = -ampa_c * voltage;
        float q = (voltage + 80) / 60;
        float temp = q * q;
        current -= nmda_c * (temp / (1 + temp)) * voltage;
        current -= gabaa_c * (voltage + 70);
        current -= gabab_c * (voltage + 90);
        current *= 1 + mf;
        current += base_current;
        // delta_v = (0.04 * voltage * voltage) + (5 * voltage) + 140 - recovery + current
        const double vd = f2d_exact(voltage);
        double dv = __dmul_rn(mul_df_rn(voltage, 0.04), vd);
        dv = __dadd_rn(dv, f2d_exact(5 * voltage));
        dv = __dadd_rn(dv, 140.0);
        dv = __dsub_rn(dv, f2d_exact(recovery));
        dv = __dadd_rn(dv, f2d_exact(current));
        const float delta_v = d2f_rn(dv);
        // voltage = (voltage + 0.1 * (delta_v + (gabaa_c * -70) + (gabab_c * -90))) / den
        const float drive = delta_v + (gabaa_c * -70) + (gabab_c * -90);
        voltage = d2f_rn(div_rn_recip(__dadd_rn(vd, mul_df_rn(drive, 0.1)), den, rden));
        voltage = (voltage != voltage) ? 30.0f : voltage;
        float adjusted_tau = (voltage > 30.0f)
                                 ? (float)(delta_v / (30.0 - voltage + delta_v) * 0.1)
                                 : (float)0.1;
        recovery += a * adjusted_tau * ((b * voltage) - recovery);
    }
}

// The substep's three double expressions evaluated in double, one at a time:
// taken where the float-float evaluation's rounding test fails (rarely; out of
// line so that the other lanes branch around the FP64 instructions).
static __device__ __noinline__ float iz_delta_v_double(float voltage, float recovery,
                                                       float current) {
    const double vd = f2d_exact(voltage);
    double dv = __dmul_rn(mul_df_rn(voltage, 0.04), vd);
    dv = __dadd_rn(dv, f2d_exact(5 * voltage));
    dv = __dadd_rn(dv, 140.0);
    dv = __dsub_rn(dv, f2d_exact(recovery));
    dv = __dadd_rn(dv, f2d_exact(current));
    return d2f_rn(dv);
}

static __device__ __noinline__ float iz_voltage_double(float voltage, float drive, float sum_c) {
    const double den = __dadd_rn(1.0, mul_df_rn(sum_c, 0.1));
    return d2f_rn(__ddiv_rn(__dadd_rn(f2d_exact(voltage), mul_df_rn(drive, 0.1)), den));
}

static __device__ __noinline__ float iz_tau_double(float voltage, float delta_v) {
    return (float)(delta_v / (30.0 - voltage + delta_v) * 0.1);
}

// The same substeps with each double expression evaluated in float-float
// arithmetic (ff_exact.cuh) and its float result taken where the rounding
// test proves it equal to the double evaluation; elsewhere (about one
// evaluation in a hundred: results within the error bound of a rounding
// boundary, such as the first substep after a reset, where v = c is exact
// and the terms cancel) the expression is evaluated in double.  The results
// are iz_integrate's, bit for bit, at a fraction of its FP64 work.
__device__ __forceinline__ void iz_integrate_ff(float& voltage, float& recovery, float ampa_c,
                                                float nmda_c, float gabaa_c, float gabab_c,
                                                float mf, float base_current, float a, float b) {
    if (!(voltage < 30.0f)) return;
    const float sum_c = ampa_c + nmda_c + gabaa_c + gabab_c;
    float d1, d2;
    ff::iz_denominator(sum_c, d1, d2);        // 1 + 0.1 * sum_c ~ d1 + d2
    const float rd = 1.0f / d1;
    for (int i = 0; (i < 10) && (voltage < 30.0f); ++i) {
        float current = -ampa_c * voltage;
        float q = ff::div_int<60>(voltage + 80);
        float temp = q * q;
        current -= nmda_c * (temp / (1 + temp)) * voltage;
        current -= gabaa_c * (voltage + 70);
        current -= gabab_c * (voltage + 90);
        current *= 1 + mf;
        current += base_current;
        float delta_v;
        if (!ff::iz_delta_v(voltage, recovery, current, delta_v))
            delta_v = iz_delta_v_double(voltage, recovery, current);
        const float drive = delta_v + (gabaa_c * -70) + (gabab_c * -90);
        float nv;
        if (!ff::iz_voltage(voltage, drive, d1, d2, rd, nv))
            nv = iz_voltage_double(voltage, drive, sum_c);
        voltage = (nv != nv) ? 30.0f : nv;
        float adjusted_tau = (float)0.1;
        if (voltage > 30.0f && !ff::iz_adjusted_tau(voltage, delta_v, adjusted_tau))
            adjusted_tau = iz_tau_double(voltage, delta_v);
        recovery += a * adjusted_tau * ((b * voltage) - recovery);
    }
}
#endif

}  // namespace sg
