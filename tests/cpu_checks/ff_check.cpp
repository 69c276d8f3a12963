// Host checks of synaptogenesis_gb300/csrc/ff_exact.cuh: the float-float
// evaluations with their rounding test against the reference's expressions
// evaluated in double by the host compiler (built with -ffp-contract=off, so
// neither side contracts).  Wherever a fast path returns true its result must
// equal the double evaluation bit for bit; the counts of fallbacks are
// reported.  Built by tests/test_ff_exact_cpu.py into a temporary library.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <initializer_list>

#include "ff_exact.cuh"

namespace {

struct Result {
    unsigned long long mismatches, checked, fallbacks, first;
};

uint32_t fbits(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }
float ffrom(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }

// izhikevich_attributes.cpp:486-490, as the reference's C++ evaluates it
float ref_wd(float x, float p, float q) {
    double c = ((double)x - 0.000001) * 0.0001 + (double)p - (double)q;
    return (float)((double)x - c);
}

// izhikevich_attributes.cpp:501-503 (stp_ws update)
float ref_sw(float w, bool spike, bool sub) {
    const double U = sub ? 0.2 : 0.5;
    const int F = sub ? 20 : 1000;
    double inc = ((U - w) / F) + (U * (1 - w) * (double)spike);
    return (float)((double)w + inc);
}

bool same(float a, float b) { return fbits(a) == fbits(b) || (std::isnan(a) && std::isnan(b)); }

void merge(Result* r, const Result& l) {
#pragma omp critical
    {
        r->mismatches += l.mismatches;
        r->checked += l.checked;
        r->fallbacks += l.fallbacks;
        if (l.first < r->first) r->first = l.first;
    }
}

// splitmix64, for the random operand draws
uint64_t mix(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// a float in [-lim, lim] with a log-uniform magnitude, or one of a few
// special values (0, powers of two, the constants' neighbourhoods)
float draw(uint64_t z, float lim) {
    const uint32_t sel = (uint32_t)(z >> 56);
    if (sel < 4) return 0.0f;
    if (sel < 12) return std::ldexp(1.0f, -(int)((z >> 8) % 40)) * ((z & 1) ? -1.0f : 1.0f);
    if (sel < 20) return ffrom(fbits(0.000001f) + (int32_t)((z >> 8) % 64) - 32);
    const double u = (double)((z >> 11) & ((1ull << 40) - 1)) / (double)(1ull << 40);
    float m = (float)(lim * std::pow(2.0, -40.0 * u));
    return (z & 1) ? -m : m;
}

// izhikevich_attributes.cpp:155-156 and 163-168, as the reference's C++
// evaluates them
float ref_dv(float v, float rec, float cur) {
    return (float)((0.04 * v * v) + (5 * v) + 140 - rec + cur);
}
float ref_voltage(float v, float drive, float sum_c) {
    return (float)((v + 0.1 * drive) / (1 + (0.1 * sum_c)));
}
float ref_tau(float v, float dv) { return (float)(dv / (30.0 - v + dv) * 0.1); }

// Izhikevich substep operands: voltage mostly in [-100, 30] (a share exactly
// at the reset values -65 and -50), recovery in [-30, 30], current and drive
// log-uniform up to 100, conductance sums log-uniform up to 10.
void iz_operands(uint64_t z0, float& v, float& rec, float& cur, float& sum_c) {
    const uint64_t z1 = mix(z0), z2 = mix(z1), z3 = mix(z2);
    const uint32_t sel = (uint32_t)(z0 >> 58);
    v = sel < 4 ? -65.0f : sel < 6 ? -50.0f
                         : (float)(-100.0 + 130.0 * (double)((z0 >> 11) & 0xFFFFFF) / 16777216.0);
    rec = (float)(-30.0 + 60.0 * (double)((z1 >> 11) & 0xFFFFFF) / 16777216.0);
    cur = draw(z2, 100.0f);
    sum_c = std::fabs(draw(z3, 10.0f));
}

}  // namespace

extern "C" {

// n random Izhikevich substeps: delta_v and the implicit voltage update.
int check_iz_random(unsigned long long n, unsigned long long seed, Result* dv, Result* vr,
                    Result* tr) {
    for (Result* r : {dv, vr, tr}) {
        r->mismatches = r->checked = r->fallbacks = 0;
        r->first = ~0ull;
    }
#pragma omp parallel
    {
        Result a{0, 0, 0, ~0ull}, b{0, 0, 0, ~0ull}, c{0, 0, 0, ~0ull};
#pragma omp for schedule(static)
        for (long long i = 0; i < (long long)n; ++i) {
            float v, rec, cur, sum_c;
            iz_operands(mix(seed * 0x100000001B3ull + (uint64_t)i), v, rec, cur, sum_c);
            // the threshold-crossing substep: a derivative dv in [1, 1024) and
            // a voltage past 30 by up to a tenth of it (v += 0.1 dv / den)
            const float dvs = std::ldexp(1.0f + (v + 100.0f) / 130.0f, (int)((sum_c * 1e6f)) % 10);
            const float vs = 30.0f + 0.1f * dvs * ((rec + 30.0f) / 60.0f) + 1e-3f;
            float tau;
            ++c.checked;
            if (!sg::ff::iz_adjusted_tau(vs, dvs, tau)) {
                ++c.fallbacks;
            } else if (!same(tau, ref_tau(vs, dvs))) {
                ++c.mismatches;
                if ((unsigned long long)i < c.first) c.first = (unsigned long long)i;
            }
            float out;
            ++a.checked;
            if (!sg::ff::iz_delta_v(v, rec, cur, out)) {
                ++a.fallbacks;
            } else if (!same(out, ref_dv(v, rec, cur))) {
                ++a.mismatches;
                if ((unsigned long long)i < a.first) a.first = (unsigned long long)i;
            }
            float d1, d2;
            sg::ff::iz_denominator(sum_c, d1, d2);
            const float rd = 1.0f / d1;
            ++b.checked;
            if (!sg::ff::iz_voltage(v, cur, d1, d2, rd, out)) {
                ++b.fallbacks;
            } else if (!same(out, ref_voltage(v, cur, sum_c))) {
                ++b.mismatches;
                if ((unsigned long long)i < b.first) b.first = (unsigned long long)i;
            }
        }
        merge(dv, a);
        merge(vr, b);
        merge(tr, c);
    }
    return 0;
}


// Every float x with (bits - offset) % stride == 0, no spike terms.
int check_wd_strided(unsigned long long stride, unsigned long long offset, Result* r) {
    r->mismatches = r->checked = r->fallbacks = 0;
    r->first = ~0ull;
#pragma omp parallel
    {
        Result l{0, 0, 0, ~0ull};
#pragma omp for schedule(static)
        for (long long i = (long long)offset; i < (1ll << 32); i += (long long)stride) {
            const float x = ffrom((uint32_t)i);
            float out;
            ++l.checked;
            if (!sg::ff::weight_derivative(x, 0.0f, false, 0.0f, false, out)) {
                ++l.fallbacks;
                continue;
            }
            if (!same(out, ref_wd(x, 0.0f, 0.0f))) {
                ++l.mismatches;
                if ((unsigned long long)i < l.first) l.first = (unsigned long long)i;
            }
        }
        merge(r, l);
    }
    return 0;
}

// Every float p with (bits - offset) % stride == 0: (float)((double)p * 0.933).
int check_product_strided(unsigned long long stride, unsigned long long offset, Result* r) {
    r->mismatches = r->checked = r->fallbacks = 0;
    r->first = ~0ull;
    const float c1 = (float)0.933, c2 = (float)(0.933 - (double)c1);
#pragma omp parallel
    {
        Result l{0, 0, 0, ~0ull};
#pragma omp for schedule(static)
        for (long long i = (long long)offset; i < (1ll << 32); i += (long long)stride) {
            const float p = ffrom((uint32_t)i);
            float out;
            ++l.checked;
            if (!sg::ff::product(p, c1, c2, out)) {
                ++l.fallbacks;
                continue;
            }
            if (!same(out, (float)((double)p * 0.933))) {
                ++l.mismatches;
                if ((unsigned long long)i < l.first) l.first = (unsigned long long)i;
            }
        }
        merge(r, l);
    }
    return 0;
}

// Every float p with (bits - offset) % stride == 0: (float)((double)p * c).
int check_product_c_strided(double c, unsigned long long stride, unsigned long long offset,
                            Result* r) {
    r->mismatches = r->checked = r->fallbacks = 0;
    r->first = ~0ull;
    const float c1 = (float)c, c2 = (float)(c - (double)c1);
#pragma omp parallel
    {
        Result l{0, 0, 0, ~0ull};
#pragma omp for schedule(static)
        for (long long i = (long long)offset; i < (1ll << 32); i += (long long)stride) {
            const float p = ffrom((uint32_t)i);
            float out;
            ++l.checked;
            if (!sg::ff::product(p, c1, c2, out)) {
                ++l.fallbacks;
                continue;
            }
            if (!same(out, (float)((double)p * c))) {
                ++l.mismatches;
                if ((unsigned long long)i < l.first) l.first = (unsigned long long)i;
            }
        }
        merge(r, l);
    }
    return 0;
}

// Every float x with (bits - offset) % stride == 0: (float)((double)x + k).
int check_add_const_strided(double k, unsigned long long stride, unsigned long long offset,
                            Result* r) {
    r->mismatches = r->checked = r->fallbacks = 0;
    r->first = ~0ull;
    const float k1 = (float)k, k2 = (float)(k - (double)k1);
#pragma omp parallel
    {
        Result l{0, 0, 0, ~0ull};
#pragma omp for schedule(static)
        for (long long i = (long long)offset; i < (1ll << 32); i += (long long)stride) {
            const float x = ffrom((uint32_t)i);
            float out;
            ++l.checked;
            if (!sg::ff::add_const(x, k1, k2, out)) {
                ++l.fallbacks;
                continue;
            }
            if (!same(out, (float)((double)x + k))) {
                ++l.mismatches;
                if ((unsigned long long)i < l.first) l.first = (unsigned long long)i;
            }
        }
        merge(r, l);
    }
    return 0;
}

// Every float a with (bits - offset) % stride == 0: div_int<D>(a) == a / D.
int check_div_strided(int D, unsigned long long stride, unsigned long long offset, Result* r) {
    r->mismatches = r->checked = r->fallbacks = 0;
    r->first = ~0ull;
#pragma omp parallel
    {
        Result l{0, 0, 0, ~0ull};
#pragma omp for schedule(static)
        for (long long i = (long long)offset; i < (1ll << 32); i += (long long)stride) {
            const float a = ffrom((uint32_t)i);
            const float got = D == 60 ? sg::ff::div_int<60>(a)
                              : D == 700 ? sg::ff::div_int<700>(a) : sg::ff::div_int<800>(a);
            ++l.checked;
            if (!same(got, a / (float)D)) {
                ++l.mismatches;
                if ((unsigned long long)i < l.first) l.first = (unsigned long long)i;
            }
        }
        merge(r, l);
    }
    return 0;
}

// Every float w with (bits - offset) % stride == 0, with and without a spike.
int check_sw_strided(int sub, int spike, unsigned long long stride, unsigned long long offset,
                     Result* r) {
    r->mismatches = r->checked = r->fallbacks = 0;
    r->first = ~0ull;
#pragma omp parallel
    {
        Result l{0, 0, 0, ~0ull};
#pragma omp for schedule(static)
        for (long long i = (long long)offset; i < (1ll << 32); i += (long long)stride) {
            const float w = ffrom((uint32_t)i);
            float out;
            ++l.checked;
            const bool ok = sub ? sg::ff::short_term_w<true>(w, spike != 0, out)
                                : sg::ff::short_term_w<false>(w, spike != 0, out);
            if (!ok) {
                ++l.fallbacks;
                continue;
            }
            if (!same(out, ref_sw(w, spike != 0, sub != 0))) {
                ++l.mismatches;
                if ((unsigned long long)i < l.first) l.first = (unsigned long long)i;
            }
        }
        merge(r, l);
    }
    return 0;
}

// n random (x, p, q) triples with spike terms: x log-uniform up to 0.05,
// p and q log-uniform up to 0.01 (traces and their products), each term
// present with probability 1/2; plus specials.
int check_wd_random(unsigned long long n, unsigned long long seed, Result* r) {
    r->mismatches = r->checked = r->fallbacks = 0;
    r->first = ~0ull;
#pragma omp parallel
    {
        Result l{0, 0, 0, ~0ull};
#pragma omp for schedule(static)
        for (long long i = 0; i < (long long)n; ++i) {
            const uint64_t z0 = mix(seed * 0x100000001B3ull + (uint64_t)i);
            const uint64_t z1 = mix(z0), z2 = mix(z1);
            const float x = draw(z0, 0.05f);
            const bool hp = (z1 & 2) != 0, hq = (z2 & 2) != 0;
            const float p = hp ? draw(z1, 0.01f) : 0.0f;
            const float q = hq ? draw(z2, 0.01f) : 0.0f;
            float out;
            ++l.checked;
            if (!sg::ff::weight_derivative(x, p, hp, q, hq, out)) {
                ++l.fallbacks;
                continue;
            }
            if (!same(out, ref_wd(x, p, q))) {
                ++l.mismatches;
                if ((unsigned long long)i < l.first) l.first = (unsigned long long)i;
            }
        }
        merge(r, l);
    }
    return 0;
}

}  // extern "C"
