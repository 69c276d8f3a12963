// Host checks of synaptogenesis_gb300/csrc/ff_exact.cuh: the float-float
// evaluations with their rounding test against the reference's expressions
// evaluated in double by the host compiler (built with -ffp-contract=off, so
// neither side contracts).  Wherever a fast path returns true its result must
// equal the double evaluation bit for bit; the counts of fallbacks are
// reported.  Built by tests/test_ff_exact_cpu.py into a temporary library.
#include <cmath>
#include <cstdint>
#include <cstring>

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

}  // namespace

extern "C" {

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
