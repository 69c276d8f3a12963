// Izhikevich neural model: src/core/state/impl/izhikevich_attributes.cpp.
//
// Arithmetic follows the reference's mixed float/double expressions term by
// term (IZ_* and STDP constants are double literals); the library is built
// with --fmad=false so nothing is contracted.  powf(x, 2) is x * x, which is
// what the reference's optimised build computes.
#include <cmath>
#include <cstdlib>
#include <mutex>
#include <random>
#include <set>

#include "cuda_check.h"
#include "exact_convert.cuh"
#include "exact_div.cuh"
#include "ff_exact.cuh"
#include "history.cuh"
#include "iz_cols_tma.cuh"
#include "iz_neuron.cuh"
#include "models.h"
#include "state.h"
#include "weight_init.h"

namespace sg {

namespace {

struct IzParams { float a, b, c, d; };

// izhikevich_attributes.cpp:28-35
IzParams preset(const std::string& s) {
    if (s == "default") return {0.02f, 0.2f, -70.0f, 2.0f};
    if (s == "regular") return {0.02f, 0.2f, -65.0f, 8.0f};
    if (s == "bursting") return {0.02f, 0.2f, -55.0f, 4.0f};
    if (s == "chattering") return {0.02f, 0.2f, -50.0f, 2.0f};
    if (s == "fast") return {0.1f, 0.2f, -65.0f, 2.0f};
    if (s == "low_threshold") return {0.02f, 0.25f, -65.0f, 2.0f};
    if (s == "thalamo_cortical") return {0.02f, 0.25f, -65.0f, 0.05f};
    if (s == "resonator") return {0.1f, 0.26f, -65.0f, 2.0f};
    throw SgError("Unrecognized parameter string: " + s);
}

// iSTDP kernels of STDP_SUB (izhikevich_attributes.cpp:454-472).  Their
// arguments are integer times 1..31, so they are tabulated on the host with
// the host C library, evaluating the reference's expression unchanged.
float istdp_src(volatile int t) { return (float)(powf(t, 10) * 0.000001 * 2.29 * expf(-1.1 * t)); }
float istdp_dst(volatile int t) { return (float)(powf(t, 10) * 0.0000001 * 2.6 * expf(-0.94 * t)); }

}  // namespace

// iSTDP tables, indexed by the time since a spike (1..31).
struct IzLut { float src[33]; float dst[33]; };

// One synapse of the STDP + STP updaters (izhikevich_attributes.cpp:404-520).
// The reference's expressions are evaluated in its types (double literals
// make the weight-derivative and short-term-w updates double), with rewrites
// that leave every stored value bit-identical:
//  * the weight derivative and short-term w are float results of double
//    expressions, evaluated in float-float arithmetic with a rounding test
//    (ff_exact.cuh); the rare operands the test rejects take the double
//    evaluation (wd_double, sw_double), kept out of line;
//  * a spike product that is zero (no destination / source spike) adds or
//    subtracts +0.0 to a partial sum that is never zero, so it is skipped;
//  * the presynaptic trace decay product is a float-float product with the
//    same rounding test (integer arithmetic where it fails, exact_convert.cuh).
// iz_learn_load reads a synapse's variables and iz_learn_apply updates them,
// so that a thread can have several synapses' loads in flight at once.
struct LearnVals {
    float w, presyn, wd, r, sw;
};

template <bool SUB>
__device__ __forceinline__ LearnVals iz_learn_load(size_t wi, int stp_flag, const float* w,
                                                   const float* presyn, const float* wd,
                                                   const float* stp_r, const float* stp_w) {
    LearnVals v;
    v.w = w[wi];
    v.presyn = SUB ? 0.0f : presyn[wi];
    v.wd = wd[wi];
    v.r = stp_flag ? stp_r[wi] : 0.0f;
    v.sw = stp_flag ? stp_w[wi] : 0.0f;
    return v;
}

// presyn * 0.933 in double, rounded to float.
static __device__ __noinline__ float presyn_decay_exact(float p) { return mul_fd_rn(p, 0.933); }

// wd - ((wd - 1e-6) * 1e-4 [+ p] [- q]) in double, rounded to float.
static __device__ __noinline__ float wd_double(float x, float p, bool has_p, float q, bool has_q) {
    const double xd = f2d_exact(x);
    double change = __dmul_rn(__dsub_rn(xd, 0.000001), 0.0001);
    if (has_p) change = __dadd_rn(change, f2d_exact(p));
    if (has_q) change = __dsub_rn(change, f2d_exact(q));
    return d2f_rn(__dsub_rn(xd, change));
}

// sw + ((U - sw) / F + U * (1 - sw) * spike) in double, rounded to float.
template <bool SUB>
static __device__ __noinline__ float sw_double(float sw, bool spike) {
    constexpr double U = SUB ? 0.2 : 0.5;
    constexpr int F = SUB ? 20 : 1000;
    const double swd = f2d_exact(sw);
    double inc = div_const_rn<F>(__dsub_rn(U, swd));
    if (spike) inc = inc + (U * (1 - sw) * spike);
    return d2f_rn(__dadd_rn(swd, inc));
}

template <bool SUB>
__device__ __forceinline__ void iz_learn_apply(size_t wi, const LearnVals& v, int src_tss,
                                               float dest_spike, float dest_exc_trace,
                                               int dest_tss, float lr, int stp_flag,
                                               float max_weight, float* w, float* presyn,
                                               float* wd, float* stp_r, float* stp_w,
                                               const IzLut& lut) {
    constexpr double U = SUB ? 0.2 : 0.5;
    constexpr int D = SUB ? 700 : 800;
    float weight = v.w;
    if (!(weight >= 0.0001f)) return;
    const bool src_spike = src_tss == 0;
    float src_trace, dest_trace;
    if (!SUB) {
        // presyn = src_spike ? 0.004 : presyn * 0.933, stored as float
        constexpr float C1 = (float)0.933;
        constexpr float C2 = (float)(0.933 - (double)C1);
        if (src_spike) src_trace = (float)0.004;
        else if (!ff::product(v.presyn, C1, C2, src_trace)) src_trace = presyn_decay_exact(v.presyn);
        presyn[wi] = src_trace;
        dest_trace = dest_exc_trace;
    } else {
        src_trace = (dest_spike > 0.0f && src_tss > 0 && src_tss < 32) ? lut.src[src_tss] : 0.0f;
        dest_trace = (src_spike && dest_tss > 0 && dest_tss < 32) ? lut.dst[dest_tss] : 0.0f;
    }
    // wd -= (wd - 1e-6) * 1e-4 + dest_spike * src_trace - src_spike * dest_trace
    const float p = dest_spike * src_trace;
    const bool has_p = dest_spike != 0.0f;
    float weight_delta;
    if (!ff::weight_derivative(v.wd, p, has_p, dest_trace, src_spike, weight_delta))
        weight_delta = wd_double(v.wd, p, has_p, dest_trace, src_spike);
    wd[wi] = weight_delta;
    weight += lr * weight_delta;
    w[wi] = fmaxf(0.0001f, fminf(max_weight, weight));
    if (stp_flag) {
        const float r = v.r;
        const float sw = v.sw;
        // Without a source spike, R = 1 and w = U are fixed points: the
        // increments are +0.0 and the stored values would not change.
        if (src_spike || r != 1.0f || !isfinite(sw))
            stp_r[wi] = r + (ff::div_int<D>(1 - r) - (r * sw * src_spike));
        if (src_spike || !(U == (double)(float)U && sw == (float)U)) {
            // stp_w += (U - sw) / F + U * (1 - sw) * src_spike
            float nsw;
            if (!ff::short_term_w<SUB>(sw, src_spike, nsw)) nsw = sw_double<SUB>(sw, src_spike);
            stp_w[wi] = nsw;
        }
    }
}

template <bool SUB>
__device__ __forceinline__ void iz_learn_synapse(size_t wi, int src_tss, float dest_spike,
                                                 float dest_exc_trace, int dest_tss, float lr,
                                                 int stp_flag, float max_weight, float* w,
                                                 float* presyn, float* wd, float* stp_r,
                                                 float* stp_w, const IzLut& lut) {
    iz_learn_apply<SUB>(wi, iz_learn_load<SUB>(wi, stp_flag, w, presyn, wd, stp_r, stp_w), src_tss,
                        dest_spike, dest_exc_trace, dest_tss, lr, stp_flag, max_weight, w, presyn,
                        wd, stp_r, stp_w, lut);
}


// ---------------------------------------------------------------------------
// Kernels
// ---------------------------------------------------------------------------

// Trace activators (izhikevich_attributes.cpp:228-352); the time-since-spike
// bookkeeping of CALC_VAL_PREAMBLE runs in k_iz_time_since_spike.
// `serial` runs every destination in one thread: convolutional matrices share
// their per-synapse traces across destinations, which the reference updates in
// destination order.
template <int TY, int SR, bool LONG>
__global__ void __launch_bounds__(128) k_iz_activate(
    DGeom g, int serial, const uint32_t* __restrict__ src, const float* __restrict__ w,
    const float* __restrict__ stp_r, const float* __restrict__ stp_w, const int* __restrict__ delays,
    float* __restrict__ short_tr, float* __restrict__ long_tr, float gcond, float short_tau,
    float long_tau, float* short_cond, float* long_cond) {
    int d0 = blockIdx.x * blockDim.x + threadIdx.x;
    int d1 = d0 + 1;
    if (serial) { if (d0 != 0) return; d1 = g.n_dest; }
    for (int d = d0; d < d1 && d < g.n_dest; ++d) {
        float short_sum = 0.0f, long_sum = 0.0f;
        for_each_source<TY>(g, d, [&](int from, int wi) {
            float spike = extract<SR>(src[from], SR == S_BIT ? delays[wi] : 0);
            float weight = w[wi] * (stp_r[wi] * stp_w[wi]);
            float st = short_tr[wi] + (spike * weight * gcond);
            short_sum += st;
            short_tr[wi] = st * short_tau;
            if (LONG) {
                float lt = long_tr[wi] + (spike * weight * gcond);
                long_sum += lt;
                long_tr[wi] = lt * long_tau;
            }
        });
        int to = dest_of<TY>(g, d);
        short_cond[to] += short_sum;
        if (LONG) long_cond[to] += long_sum;
    }
}

// Source index of matrix row `row` (FC: the source itself; subset: its window).
template <bool SUBSET>
__device__ __forceinline__ int row_source(const DGeom& g, int row) {
    if (!SUBSET) return row;
    int fkc = g.fc1 - g.fc0;
    return (row / fkc + g.fr0) * g.from_cols + (row % fkc + g.fc0);
}

// Source of kernel position k of destination d for a non-convolutional
// convergent connection (synapse_kernel.h:384-421); -1 if it is skipped.
__device__ __forceinline__ int conv_source(const DGeom& g, int d, int k) {
    const int tr = d / g.to_cols, tc = d - (d / g.to_cols) * g.to_cols;
    const int kr = k / g.cf, kc = k - (k / g.cf) * g.cf;
    int fr = tr * g.rs + g.rsp * g.ro + kr * g.rsp;
    int fc = tc * g.cs + g.csp * g.co + kc * g.csp;
    if (g.wrap) {
        fr = wrap_coord(g, fr, g.from_rows);
        fc = wrap_coord(g, fc, g.from_cols);
    } else if (fr < 0 || fr >= g.from_rows || fc < 0 || fc >= g.from_cols) {
        return -1;
    }
    return fr * g.from_cols + fc;
}

// The same through a per-CTA table of kernel-position offsets: `koff[k]` =
// (kr * row spacing, kc * column spacing), filled by conv_offsets, and the
// destination's base coordinates from conv_base.
__device__ __forceinline__ int2 conv_base(const DGeom& g, int d) {
    const int tr = d / g.to_cols, tc = d - tr * g.to_cols;
    return make_int2(tr * g.rs + g.rsp * g.ro, tc * g.cs + g.csp * g.co);
}
__device__ __forceinline__ void conv_offsets(const DGeom& g, int K, int2* koff) {
    for (int k = threadIdx.x; k < K; k += blockDim.x) {
        const int kr = k / g.cf;
        koff[k] = make_int2(kr * g.rsp, (k - kr * g.cf) * g.csp);
    }
}
__device__ __forceinline__ int conv_source_at(const DGeom& g, int2 base, int2 off) {
    int fr = base.x + off.x, fc = base.y + off.y;
    if (g.wrap) {
        fr = wrap_coord(g, fr, g.from_rows);
        fc = wrap_coord(g, fc, g.from_cols);
    } else if (fr < 0 || fr >= g.from_rows || fc < 0 || fc >= g.from_cols) {
        return -1;
    }
    return fr * g.from_cols + fc;
}

// Trace activator for non-convolutional convergent connections.  A CTA owns
// 32 consecutive destinations; its 8 warps take the kernel positions k in
// turn (warp w: k = w, w+8, ...), one lane per destination, so every load is a
// coalesced 128-byte row of the [k][destination] layout and each warp has
// many independent loads in flight.  Pre-decay traces go to shared memory and
// lanes of warps 0 / 1 add them in k order (the reference's sequential sum),
// skipping positions outside a non-wrapping layer as the reference does.
constexpr int kConvMaxK = 128;

template <int SR, bool LONG>
__global__ void __launch_bounds__(256, 4) k_iz_activate_conv_tile(
    DGeom g, int K, const uint32_t* __restrict__ src, const float* __restrict__ w,
    const float* __restrict__ stp_r, const float* __restrict__ stp_w, const uint8_t* __restrict__ delays,
    float* __restrict__ short_tr, float* __restrict__ long_tr, float gcond, float short_tau,
    float long_tau, float* __restrict__ short_cond, float* __restrict__ long_cond) {
    __shared__ float s_st[kConvMaxK][32];
    __shared__ float s_lt[LONG ? kConvMaxK : 1][32];
    __shared__ int2 koff[kConvMaxK];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int d = blockIdx.x * 32 + lane;
    const bool ok = d < g.to_size;
    conv_offsets(g, K, koff);
    __syncthreads();
    const int2 base = conv_base(g, ok ? d : 0);
    constexpr int B = 4;                 // kernel positions whose loads are in flight together
    for (int k0 = warp; k0 < K; k0 += 8 * B) {
        uint32_t word[B];
        int dl[B];
        float wv[B], rv[B], sv[B], st0[B], lt0[B];
        bool on[B];
#pragma unroll
        for (int b = 0; b < B; ++b) {
            const int k = k0 + 8 * b;
            const int from = (ok && k < K) ? conv_source_at(g, base, koff[k]) : -1;
            on[b] = from >= 0;
            if (on[b]) {
                const size_t wi = (size_t)k * g.to_size + d;
                word[b] = __ldg(src + from);
                dl[b] = SR == S_BIT ? (int)__ldg(delays + wi) : 0;
                wv[b] = __ldg(w + wi);
                rv[b] = __ldg(stp_r + wi);
                sv[b] = __ldg(stp_w + wi);
                st0[b] = short_tr[wi];
                lt0[b] = LONG ? long_tr[wi] : 0.0f;
            }
        }
#pragma unroll
        for (int b = 0; b < B; ++b) {
            const int k = k0 + 8 * b;
            if (k >= K) break;
            float st_pre = 0.0f, lt_pre = 0.0f;
            if (on[b]) {
                const size_t wi = (size_t)k * g.to_size + d;
                const float spike = extract<SR>(word[b], dl[b]);
                const float weight = wv[b] * (rv[b] * sv[b]);
                st_pre = st0[b] + (spike * weight * gcond);
                short_tr[wi] = st_pre * short_tau;
                if (LONG) {
                    lt_pre = lt0[b] + (spike * weight * gcond);
                    long_tr[wi] = lt_pre * long_tau;
                }
            }
            s_st[k][lane] = st_pre;
            if (LONG) s_lt[k][lane] = lt_pre;
        }
    }
    __syncthreads();
    if (!ok) return;
    if (warp == 0) {
        float sum = 0.0f;
        for (int k = 0; k < K; ++k)
            if (g.wrap || conv_source_at(g, base, koff[k]) >= 0) sum += s_st[k][lane];
        short_cond[d] += sum;
    } else if (LONG && warp == 1) {
        float sum = 0.0f;
        for (int k = 0; k < K; ++k)
            if (g.wrap || conv_source_at(g, base, koff[k]) >= 0) sum += s_lt[k][lane];
        long_cond[d] += sum;
    }
}

// Updater for non-convolutional convergent connections: one thread per
// synapse (kernel position, destination), coalesced along destinations.  A
// CTA owns 32 consecutive destinations and a share of the kernel positions
// (grid.y shares of 24); its 8 warps take those positions in turn,
// kLearnBatch at a time, loading all of their variables before updating any
// (distinct synapses: no overlap).  Source coordinates come from a per-CTA
// table of kernel-position offsets.
constexpr int kLearnBatch = 4;

template <int SR, bool SUB>
__global__ void __launch_bounds__(256, 4) k_iz_learn_conv_tile(
    DGeom g, int K, const uint32_t* __restrict__ dest_out, const float* __restrict__ to_exc,
    const int* __restrict__ to_tss, const int* __restrict__ from_tss, float lr, int stp_flag,
    float max_weight, float* __restrict__ w, float* __restrict__ presyn, float* __restrict__ wd,
    float* __restrict__ stp_r, float* __restrict__ stp_w, IzLut lut) {
    __shared__ int2 koff[kConvMaxK];
    conv_offsets(g, K, koff);
    __syncthreads();
    const int d = blockIdx.x * 32 + (threadIdx.x & 31);
    if (d >= g.to_size) return;
    const float dest_exc_trace = __ldg(to_exc + d);
    const int dest_tss = __ldg(to_tss + d);
    const float dest_spike = extract<SR>(__ldg(dest_out + d), 0);
    const int2 base = conv_base(g, d);
    const int kstep = 8 * gridDim.y;
    for (int k0 = (threadIdx.x >> 5) + 8 * blockIdx.y; k0 < K; k0 += kstep * kLearnBatch) {
        LearnVals v[kLearnBatch];
        int src_tss[kLearnBatch];
        bool ok[kLearnBatch];
#pragma unroll
        for (int b = 0; b < kLearnBatch; ++b) {
            const int k = k0 + kstep * b;
            const int from = k < K ? conv_source_at(g, base, koff[k]) : -1;
            ok[b] = from >= 0;
            if (ok[b]) {
                v[b] = iz_learn_load<SUB>((size_t)k * g.to_size + d, stp_flag, w, presyn, wd,
                                          stp_r, stp_w);
                src_tss[b] = __ldg(from_tss + from);
            }
        }
#pragma unroll
        for (int b = 0; b < kLearnBatch; ++b)
            if (ok[b])
                iz_learn_apply<SUB>((size_t)(k0 + kstep * b) * g.to_size + d, v[b], src_tss[b],
                                    dest_spike, dest_exc_trace, dest_tss, lr, stp_flag, max_weight,
                                    w, presyn, wd, stp_r, stp_w, lut);
    }
}

// The largest shared-memory carveout for a kernel that runs beside the
// TMA activator (which needs it): SMs configured alike can hold both.
static void prefer_max_shared(const void* fn) {
    static std::mutex m;
    static std::set<const void*> done;
    std::lock_guard<std::mutex> lock(m);
    if (done.insert(fn).second)
        SG_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout,
                                     (int)cudaSharedmemCarveoutMaxShared));
}

// Rows (sources) and columns (destinations) of a fully connected or subset
// matrix in the device layout; false for the other connection types.
static bool matrix_shape(const Connection& c, int& nrows, int& ncols) {
    if (c.type == FULLY_CONNECTED) {
        nrows = c.from->size;
        ncols = c.to->size;
        return true;
    }
    if (c.type == SUBSET) {
        nrows = c.subset.from_size();
        ncols = c.subset.to_size();
        return true;
    }
    return false;
}

// Gap junctions (izhikevich_attributes.cpp:354-366)
template <int TY>
__global__ void k_iz_gap(DGeom g, const float* __restrict__ voltage, const float* __restrict__ w,
                         float* __restrict__ inputs) {
    int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= g.n_dest) return;
    int to = dest_of<TY>(g, d);
    float v = voltage[to];
    float sum = 0.0f;
    for_each_source<TY>(g, d, [&](int from, int wi) { sum += (voltage[from] - v) * w[wi]; });
    inputs[to] += sum;
}

// Time since the presynaptic spike, per source (CALC_VAL_PREAMBLE,
// izhikevich_attributes.cpp:257-262).  The reference updates it once per
// visit in serial order: t = spike ? 0 : min(32, t + 1).  The result depends
// only on the last visit that saw a spike and on how many visits follow it.
// Every visit with the same delay reads the same spike bit, so a source's
// last (at most 32) visits are summarised after each upload
// (k_iz_delay_summary) as, per distinct delay, the position of its last
// visit: the latest position whose delay shows a spike decides.  A source
// with more than kSummary distinct delays among those visits scans them.
//
// Summary word: bits 0-2 the number of entries (7: scan), entry i in bits
// 3 + 10 i: delay (5 bits), then position (5 bits).
constexpr int kSummary = 6;

__device__ __forceinline__ void tss_update(int f, const int* __restrict__ counts,
                                           const int* __restrict__ last,
                                           const int* __restrict__ delays,
                                           const unsigned long long* __restrict__ summary,
                                           const uint32_t* __restrict__ src, int src_type,
                                           int* __restrict__ tss) {
    int n = counts[f];
    if (n == 0) return;
    uint32_t word = src[f];
    const int m = n < 32 ? n : 32;
    const unsigned long long sm = summary[f];
    const int ne = (int)(sm & 7);
    if (ne != 7) {
        int best = -1;
        for (int i = 0; i < ne; ++i) {
            const int e = (int)(sm >> (3 + 10 * i)) & 1023;
            const int pos = e >> 5;
            if (pos > best && extract_rt(word, e & 31, src_type) > 0.0f) best = pos;
        }
        if (best >= 0) {
            tss[f] = m - 1 - best;
        } else {
            const int t = tss[f] + n;
            tss[f] = t < 32 ? t : 32;
        }
        return;
    }
    const int* L = last + (size_t)f * 32;
    for (int j = m - 1; j >= 0; --j) {
        float spike = extract_rt(word, delays[L[j]], src_type);
        if (spike > 0.0f) { tss[f] = m - 1 - j; return; }
    }
    int t = tss[f] + n;
    tss[f] = t < 32 ? t : 32;
}

__global__ void k_iz_time_since_spike(int n_src, const int* __restrict__ counts,
                                      const int* __restrict__ last, const int* __restrict__ delays,
                                      const unsigned long long* __restrict__ summary,
                                      const uint32_t* __restrict__ src, int src_type,
                                      int* __restrict__ tss) {
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= n_src) return;
    tss_update(f, counts, last, delays, summary, src, src_type, tss);
}

// The same for several connections in one launch (their sources concatenated):
// the connections of a step whose activation waits on nothing.
struct TssArgs {
    int n_src, src_type;
    const int *counts, *last, *delays;
    const unsigned long long* summary;
    const uint32_t* src;
    int* tss;
};
constexpr int kTssGroup = 8;
struct TssGroup {
    int n;
    int start[kTssGroup + 1];
    TssArgs C[kTssGroup];
};

__global__ void k_iz_time_since_spike_group(TssGroup G) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= G.start[G.n]) return;
    int c = 0;
    while (c + 1 < G.n && g >= G.start[c + 1]) ++c;
    const TssArgs& A = G.C[c];
    tss_update(g - G.start[c], A.counts, A.last, A.delays, A.summary, A.src, A.src_type, A.tss);
}
__global__ void k_iz_delay_summary(int n_src, const int* __restrict__ counts,
                                   const int* __restrict__ last, const int* __restrict__ delays,
                                   unsigned long long* __restrict__ summary) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= n_src) return;
    const int m = min(counts[f], 32);
    const int* L = last + (size_t)f * 32;
    unsigned long long sm = 0;
    unsigned seen = 0;
    int ne = 0;
    for (int j = m - 1; j >= 0 && ne <= kSummary; --j) {
        const int d = delays[L[j]];
        if (d < 0 || d > 31) { ne = kSummary + 1; break; }
        if (seen & (1u << d)) continue;
        seen |= 1u << d;
        if (ne < kSummary) sm |= (unsigned long long)(d | (j << 5)) << (3 + 10 * ne);
        ++ne;
    }
    summary[f] = ne > kSummary ? 7ull : (sm | (unsigned long long)ne);
}

// Neuron update (izhikevich_attributes.cpp:102-213).  One launch updates the
// Izhikevich layers of a step together (their neurons concatenated); each
// layer's arrays are its own.  The substeps run in float-float arithmetic
// with rounding tests (iz_integrate_ff), bit-identical to the reference's
// double evaluation; the products with double constants (decays 0.95) go
// through mul_fd_rn.
struct IzLayerArgs {
    int size, history;
    const float* inputs;
    uint32_t* spikes;
    float *ampa, *nmda, *gabaa, *gabab, *mult, *dopamine, *voltages, *recoveries, *post_traces;
    int* tss;
    const float *as, *bs, *cs, *ds;
};
constexpr int kIzGroup = 8;
struct IzUpdateGroup {
    int n;
    int start[kIzGroup + 1];           // first flattened neuron of each layer
    IzLayerArgs L[kIzGroup];
};

__global__ void __launch_bounds__(256) k_iz_update(IzUpdateGroup G) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= G.start[G.n]) return;
    int l = 0;
    while (l + 1 < G.n && g >= G.start[l + 1]) ++l;
    const IzLayerArgs& A = G.L[l];
    const int nid = g - G.start[l], size = A.size, history = A.history;
    float voltage = A.voltages[nid];
    float recovery = A.recoveries[nid];
    iz_integrate_ff(voltage, recovery, A.ampa[nid], A.nmda[nid], A.gabaa[nid], A.gabab[nid],
                    A.mult[nid], A.inputs[nid], __ldg(A.as + nid), __ldg(A.bs + nid));
    A.ampa[nid] = 0.0f;
    A.nmda[nid] = 0.0f;
    A.gabaa[nid] = 0.0f;
    A.gabab[nid] = 0.0f;
    A.mult[nid] = 0.0f;
    A.dopamine[nid] = mul_fd_rn(A.dopamine[nid], 0.95);            // dopamine *= 0.95
    const unsigned int spike = voltage >= 30.0f;                     // 30.0 is a float value
    // SHIFT_BIT_OUTPUTS (state/attributes.h:321-333)
    uint32_t* spikes = A.spikes;
    uint32_t curr = spikes[(size_t)size * (history - 1) + nid];
    for (int idx = history - 1; idx > 0; --idx) {
        uint32_t prev = spikes[(size_t)size * (idx - 1) + nid];
        spikes[(size_t)size * idx + nid] = (curr >> 1) | (prev << 31);
        curr = prev;
    }
    spikes[nid] = (curr >> 1) | (spike << 31);
    const bool prev_bit = curr >> 31;
    // post_trace = prev_bit ? 0.004 : post_trace * 0.95, stored as float
    A.post_traces[nid] = prev_bit ? (float)0.004 : mul_fd_rn(A.post_traces[nid], 0.95);
    int t = A.tss[nid] + 1;
    A.tss[nid] = prev_bit ? 0 : (t < 32 ? t : 32);
    A.voltages[nid] = spike ? __ldg(A.cs + nid) : voltage;
    A.recoveries[nid] = recovery + (spike * __ldg(A.ds + nid));
}


// STDP + STP updaters (izhikevich_attributes.cpp:404-520).  The destination
// spike goes through the connection's extractor, i.e. the SOURCE layer's
// output type (izhikevich_attributes.cpp:426).
template <int TY, int SR, bool SUB>
__global__ void __launch_bounds__(128) k_iz_learn(
    DGeom g, const uint32_t* __restrict__ dest_out, const float* __restrict__ to_exc,
    const int* __restrict__ to_tss, const int* __restrict__ from_tss, float lr, int stp_flag,
    float max_weight, float* w, float* presyn, float* wd, float* stp_r, float* stp_w, IzLut lut) {
    int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= g.n_dest) return;
    int to = dest_of<TY>(g, d);
    float dest_exc_trace = to_exc[to];
    int dest_tss = to_tss[to];
    float dest_spike = extract<SR>(dest_out[to], 0);
    for_each_source<TY>(g, d, [&](int from, int wi) {
        iz_learn_synapse<SUB>((size_t)wi, from_tss[from], dest_spike, dest_exc_trace, dest_tss, lr,
                              stp_flag, max_weight, w, presyn, wd, stp_r, stp_w, lut);
    });
}

// Updater for fully connected and subset matrices: every synapse is
// independent, so a 2-D grid covers (column tile, row block); each thread
// keeps its destination's activity in registers and walks a block of source
// rows (coalesced along the destination axis).
template <int SR, bool SUB, bool SUBSET>
__global__ void __launch_bounds__(256) k_iz_learn_2d(
    DGeom g, int nrows, int ncols, int rows_per_block, const uint32_t* __restrict__ dest_out,
    const float* __restrict__ to_exc, const int* __restrict__ to_tss,
    const int* __restrict__ from_tss, float lr, int stp_flag, float max_weight,
    float* __restrict__ w, float* __restrict__ presyn, float* __restrict__ wd,
    float* __restrict__ stp_r, float* __restrict__ stp_w, IzLut lut) {
    int col = blockIdx.x * blockDim.x + threadIdx.x;
    if (col >= ncols) return;
    int to = dest_of<SUBSET ? T_SUBSET : T_FC>(g, col);
    float dest_exc_trace = to_exc[to];
    int dest_tss = to_tss[to];
    float dest_spike = extract<SR>(dest_out[to], 0);
    int r0 = blockIdx.y * rows_per_block, r1 = min(nrows, r0 + rows_per_block);
    for (int row = r0; row < r1; ++row) {
        size_t wi = (size_t)banded_index(col, row, nrows);
        iz_learn_synapse<SUB>(wi, __ldg(from_tss + row_source<SUBSET>(g, row)), dest_spike,
                              dest_exc_trace, dest_tss, lr, stp_flag, max_weight, w, presyn, wd,
                              stp_r, stp_w, lut);
    }
}

// ---------------------------------------------------------------------------
// Model
// ---------------------------------------------------------------------------
// Neuron parameters ("params") and the settled resting voltage and recovery
// of an Izhikevich-type layer (izhikevich_attributes.cpp:587-662,
// spnet_attributes.cpp:369-425); time since spike starts at 32.
static void iz_params_and_rest(LayerState& ls) {
    const Layer& l = *ls.layer;
    float *as = ls.vars["a"]->hf(), *bs = ls.vars["b"]->hf(), *cs = ls.vars["c"]->hf(),
          *ds = ls.vars["d"]->hf();
    std::string p = l.parameter("params", "regular");
    if (p == "random positive" || p == "random negative") {
        auto rng = make_rng(l.config, 7 + l.index);
        std::uniform_real_distribution<float> u(0.0f, 1.0f);
        for (int i = 0; i < l.size; ++i) {
            if (p == "random positive") {
                as[i] = 0.02f; bs[i] = 0.2f;
                cs[i] = -65.0 + (15.0 * std::pow(u(rng), 2));
                ds[i] = 8.0 - (6.0 * std::pow(u(rng), 2));
            } else {
                as[i] = 0.02 + (0.08 * u(rng)); bs[i] = 0.25 - (0.05 * u(rng));
                cs[i] = -65.0f; ds[i] = 2.0f;
            }
        }
    } else {
        IzParams q = preset(p);
        for (int i = 0; i < l.size; ++i) { as[i] = q.a; bs[i] = q.b; cs[i] = q.c; ds[i] = q.d; }
    }
    float* v = ls.vars["voltage"]->hf();
    float* r = ls.vars["recovery"]->hf();
    int32_t* tss = ls.vars["time since spike"]->hi();
    for (int j = 0; j < l.size; ++j) {
        tss[j] = 32;
        // settle to the resting state
        float vv = cs[j], rr = bs[j] * cs[j], dv, dr, a = as[j], b = bs[j];
        do {
            dv = (0.04 * vv * vv) + (5 * vv) + 140 - rr;
            vv += dv;
            dr = a * ((b * vv) - rr);
            rr += dr;
        } while (std::fabs(dv) > 0.001 && std::fabs(dr) > 0.001);
        v[j] = vv;
        r[j] = rr;
    }
}

// Per-synapse delays (myelinated, random or from distances at 0.15 per
// step) and, per source, its last (up to 32) visits in serial order as
// device weight indices plus its visit count -- what the time-since-spike
// kernel scans (izhikevich_attributes.cpp:730-751).
static void iz_delays_and_visits(State& st, ConnState& cs) {
    Connection& c = *cs.conn;
    size_t n = c.num_weights;
    int R = c.matrix_rows, C = c.matrix_cols;
    if (!cs.delays) {
        cs.delays = st.add_array("delays", 'i', n, matrix_layout(c), R, C);
        int32_t* dl = cs.delays->hi();
        if (c.parameter("myelinated", "false") == "true") {
            for (size_t i = 0; i < n; ++i) dl[i] = c.delay;
        } else if (c.config.has("random delay")) {
            int mx = std::stoi(c.parameter("random delay", "0"));
            if (mx > 31) throw SgError("Randomized axons cannot have delays greater than 31!");
            auto rng = make_rng(c.config, 3000 + c.index);
            std::uniform_int_distribution<int> u(0, mx);
            for (size_t i = 0; i < n; ++i) dl[i] = u(rng);
        } else {
            std::vector<float> dist = cs.cached_distances;
            if (dist.empty()) {
                Indices ix = compute_indices(c);
                dist = compute_distances(c, ix,
                                         std::stof(c.from->parameter("neuron spacing", "0.1")),
                                         std::stof(c.to->parameter("neuron spacing", "0.1")),
                                         std::stof(c.parameter("x offset", "0.0")),
                                         std::stof(c.parameter("y offset", "0.0")));
            }
            compute_delays(c, dist, 0.15f, c.parameter("cap delay", "false") == "true", dl);
        }
    }
    cs.vars["delays"] = cs.delays;

    // Last (up to 32) visits of each source in serial order, device indices.
    int nsrc = c.from->size;
    cs.visit_counts = st.add_array("visit counts", 'i', nsrc);
    cs.last_visits = st.add_array("last visits", 'i', (size_t)nsrc * 32);
    cs.delay_summary = st.add_array("delay summary", 'i', 0, LAYOUT_PLAIN, 1, 1, (size_t)nsrc * 2);
    cs.delay_summary->scratch = true;
    int32_t* cnt = cs.visit_counts->hi();
    int32_t* last = cs.last_visits->hi();
    enumerate_visits(c, [&](int, int, int from, long wi, int, int) {
        long dev = (long)device_index(*cs.weights, (size_t)wi);
        last[(size_t)from * 32 + (cnt[from] % 32)] = (int)dev;
        cnt[from]++;
    });
    // unroll each ring so that entries 0..m-1 are in serial order
    std::vector<int32_t> tmp(32);
    for (int f = 0; f < nsrc; ++f) {
        int m = std::min(cnt[f], 32);
        if (cnt[f] <= 32) continue;
        int start = cnt[f] % 32;
        for (int j = 0; j < m; ++j) tmp[j] = last[(size_t)f * 32 + (start + j) % 32];
        for (int j = 0; j < m; ++j) last[(size_t)f * 32 + j] = tmp[j];
    }
}

// The delays (below 32) as bytes, element for element.
__global__ void k_iz_delay_bytes_plain(size_t n, const int* __restrict__ delays,
                                       uint8_t* __restrict__ d8) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) d8[i] = (uint8_t)delays[i];
}

class IzhikevichModel : public Model {
  public:
    const char* name() const override { return "izhikevich"; }
    OutputType output_type() const override { return OUT_BIT; }

    // After every upload (delays, weights or short-term factors may have
    // changed): which sources' last visits share one delay, and the
    // effective weights of a connection that never learns.
    void prepare_device(State&, ConnState& cs, cudaStream_t s) const override {
        if (cs.eff_weights)
            fill_iz_effective_weights(cs.weights->dev_count, cs.weights->df(),
                                      cs.var("short term R")->df(), cs.var("short term w")->df(),
                                      cs.eff_weights->df(), s);
        int nrows = 0, ncols = 0;
        if (cs.delays8 && matrix_shape(*cs.conn, nrows, ncols))
            fill_iz_delay_bytes(nrows, ncols, cs.delays->di(),
                                reinterpret_cast<uint8_t*>(cs.delays8->du()), s);
        else if (cs.delays8)
            k_iz_delay_bytes_plain<<<blocks_for((long)cs.delays->dev_count, 256), 256, 0, s>>>(
                cs.delays->dev_count, cs.delays->di(),
                reinterpret_cast<uint8_t*>(cs.delays8->du()));
        if (!cs.delay_summary) return;
        const int n = cs.conn->from->size;
        k_iz_delay_summary<<<blocks_for(n, 256), 256, 0, s>>>(
            n, cs.visit_counts->di(), cs.last_visits->di(), cs.delays->di(),
            reinterpret_cast<unsigned long long*>(cs.delay_summary->di()));
        SG_LAUNCH_CHECK();
    }

    // Constructor of IzhikevichAttributes (izhikevich_attributes.cpp:587-662)
    void build_layer(State& st, LayerState& ls) const override {
        const Layer& l = *ls.layer;
        for (const char* k : {"ampa", "nmda", "gabaa", "gabab", "mult", "dopamine", "voltage",
                              "recovery", "post trace", "a", "b", "c", "d"})
            ls.vars[k] = st.add_array(k, 'f', l.size);
        ls.vars["time since spike"] = st.add_array("time since spike", 'i', l.size);
        iz_params_and_rest(ls);
        for (Connection* c : l.inputs)
            if (c->opcode == OP_GAP && c->from != c->to)
                throw SgError("Error " + c->str() +
                              "\nGap junctions must be between neurons of the same layer.");
    }

    // process_weight_matrix (izhikevich_attributes.cpp:692-757)
    void build_matrix(State& st, ConnState& cs) const override {
        Connection& c = *cs.conn;
        size_t n = c.num_weights;
        int R = c.matrix_rows, C = c.matrix_cols;
        cs.params["conductance"] = std::stof(c.parameter("conductance", "1.0"));
        cs.params["learning rate"] = std::stof(c.parameter("learning rate", "0.1"));
        cs.params["stp"] = c.parameter("short term plasticity", "true") == "true" ? 1.0f : 0.0f;
        for (const char* k : {"short trace", "long trace", "presyn trace", "short term R",
                              "short term w", "weight derivatives"})
            cs.vars[k] = st.add_array(k, 'f', n, matrix_layout(c), R, C);
        size_t tss_n = std::max<size_t>(n, c.from->size);
        cs.vars["time since spike"] = st.add_array("time since spike", 'i', tss_n, LAYOUT_SOURCE,
                                                   1, 1, c.from->size);
        float* stp_r = cs.vars["short term R"]->hf();
        float* stp_w = cs.vars["short term w"]->hf();
        float* wd = cs.vars["weight derivatives"]->hf();
        // quirk: the ConnectionType is compared with the ADD/SUB opcodes
        // (izhikevich_attributes.cpp:723-728)
        float w0 = c.type == 0 ? 0.5f : (c.type == 1 ? 0.2f : 0.0f);
        for (size_t i = 0; i < n; ++i) { stp_r[i] = 1.0f; stp_w[i] = w0; wd[i] = 0.000001f; }
        int32_t* tss = cs.vars["time since spike"]->hi();
        for (size_t i = 0; i < tss_n; ++i) tss[i] = 32;

        iz_delays_and_visits(st, cs);
        if (c.parameter("direct", "false") != "true" && c.opcode != OP_ADD && c.opcode != OP_SUB &&
            c.opcode != OP_MULT && c.opcode != OP_REWARD && c.opcode != OP_GAP)
            throw SgError(c.str() + ": Unimplemented connection type!");
        // A fully connected or subset trace connection that never learns
        // keeps w, R and w_stp for a whole run: the TMA activator reads their
        // product, w * (R * w_stp), from one array (8 bytes less per synapse
        // and step), refilled after every upload.
        const bool trace_cols = (c.type == FULLY_CONNECTED || c.type == SUBSET) &&
                                c.parameter("direct", "false") != "true" && c.opcode != OP_GAP;
        if (trace_cols && !c.plastic) {
            cs.eff_weights = st.add_array("effective weights", 'f', n, matrix_layout(c), R, C);
            cs.eff_weights->scratch = true;
        }
        // ... and reads its delays (below 32) as bytes, as does the
        // convergent tile activator (same layout as the delays there)
        int nrows = 0, ncols = 0;
        if (trace_cols && c.from->output_type == OUT_BIT && matrix_shape(c, nrows, ncols)) {
            const size_t bytes = (size_t)((ncols + kBand - 1) / kBand) * iz_delay_bytes_pitch(nrows);
            cs.delays8 = st.add_array("delay bytes", 'u', 0, LAYOUT_PLAIN, 1, 1, (bytes + 3) / 4);
            cs.delays8->scratch = true;
        } else if (c.type == CONVERGENT && !c.convolutional && c.arbor.kernel() <= kConvMaxK &&
                   c.parameter("direct", "false") != "true" && c.opcode != OP_GAP) {
            cs.delays8 = st.add_array("delay bytes", 'u', 0, LAYOUT_PLAIN, 1, 1,
                                      (cs.delays->dev_count + 3) / 4);
            cs.delays8->scratch = true;
        }
        // trace activators write conductances, not a register, and keep no
        // weight copy: second order only through the base activator
        // (izhikevich_attributes.cpp:371-379)
        if (c.parameter("direct", "false") != "true" && c.second_order)
            throw SgError(c.str() + ": Unimplemented connection type!");
    }

    // The time-since-spike updates of trace connections (the ones activate
    // makes) whose activation waits on nothing, in launches of up to
    // kTssGroup connections.
    static bool trace_connection(const Connection& c) {
        return c.parameter("direct", "false") != "true" &&
               (c.opcode == OP_ADD || c.opcode == OP_SUB || c.opcode == OP_MULT ||
                c.opcode == OP_REWARD);
    }
    bool activate_prologue(State& st, const std::vector<ConnState*>& conns,
                           const StepCtx& ctx) const override {
        std::vector<ConnState*> todo;
        for (ConnState* cs : conns)
            if (trace_connection(*cs->conn) && cs->delay_summary) todo.push_back(cs);
        if (todo.size() < 2) return false;
        for (size_t first = 0; first < todo.size(); first += kTssGroup) {
            TssGroup G{};
            G.n = (int)std::min<size_t>(kTssGroup, todo.size() - first);
            int total = 0;
            for (int i = 0; i < G.n; ++i) {
                ConnState& cs = *todo[first + i];
                const Connection& c = *cs.conn;
                G.start[i] = total;
                G.C[i] = TssArgs{c.from->size, (int)c.from->output_type, cs.visit_counts->di(),
                                 cs.last_visits->di(), cs.delays->di(),
                                 reinterpret_cast<const unsigned long long*>(cs.delay_summary->di()),
                                 st.dev_output(c.from, word_index(c.delay, c.from->output_type)),
                                 cs.var("time since spike")->di()};
                total += c.from->size;
                cs.prologue_done = true;
            }
            G.start[G.n] = total;
            k_iz_time_since_spike_group<<<blocks_for(total, 256), 256, 0, ctx.stream>>>(G);
            SG_LAUNCH_CHECK();
            ctx.count();
        }
        return true;
    }

    void activate(State& st, ConnState& cs, const StepCtx& ctx) const override {
        Connection& c = *cs.conn;
        LayerState& to = *st.layer_state(c.to);
        if (c.parameter("direct", "false") == "true") {
            launch_base_activator(st, cs, input_register(st, cs), ctx.stream);
            ctx.count();
            return;
        }
        const int threads = 128;
        unsigned blocks = blocks_for(cs.geom.n_dest, threads);
        if (c.opcode == OP_GAP) {
            float* reg = input_register(st, cs);
            switch (c.type) {
                case 0: k_iz_gap<0><<<blocks, threads, 0, ctx.stream>>>(cs.geom, to.var("voltage")->df(), cs.weights->df(), reg); break;
                case 1: k_iz_gap<1><<<blocks, threads, 0, ctx.stream>>>(cs.geom, to.var("voltage")->df(), cs.weights->df(), reg); break;
                case 2: k_iz_gap<2><<<blocks, threads, 0, ctx.stream>>>(cs.geom, to.var("voltage")->df(), cs.weights->df(), reg); break;
                case 3: k_iz_gap<3><<<blocks, threads, 0, ctx.stream>>>(cs.geom, to.var("voltage")->df(), cs.weights->df(), reg); break;
                case 4: k_iz_gap<4><<<blocks, threads, 0, ctx.stream>>>(cs.geom, to.var("voltage")->df(), cs.weights->df(), reg); break;
                case 5: k_iz_gap<5><<<blocks, threads, 0, ctx.stream>>>(cs.geom, to.var("voltage")->df(), cs.weights->df(), reg); break;
            }
            SG_LAUNCH_CHECK();
            ctx.count();
            return;
        }
        const char *sname, *lname = nullptr;
        float stau, ltau = 0.0f;
        switch (c.opcode) {
            case OP_ADD: sname = "ampa"; stau = 0.8f; lname = "nmda"; ltau = 0.993f; break;
            case OP_SUB: sname = "gabaa"; stau = 0.833f; lname = "gabab"; ltau = 0.993f; break;
            case OP_MULT: sname = "mult"; stau = 0.95f; break;
            case OP_REWARD: sname = "dopamine"; stau = 0.95f; break;
            default: throw SgError(c.str() + ": Unimplemented connection type!");
        }
        const uint32_t* src = st.dev_output(c.from, word_index(c.delay, c.from->output_type));
        // time since spike, from the same (pre-update) source words, unless
        // activate_prologue did it with other connections of the step
        if (cs.prologue_done) {
            cs.prologue_done = false;
        } else {
            k_iz_time_since_spike<<<blocks_for(c.from->size, 256), 256, 0, ctx.stream>>>(
                c.from->size, cs.visit_counts->di(), cs.last_visits->di(), cs.delays->di(),
                reinterpret_cast<const unsigned long long*>(cs.delay_summary->di()), src,
                (int)c.from->output_type, cs.var("time since spike")->di());
            SG_LAUNCH_CHECK();
            ctx.count();
        }
        int serial = c.convolutional ? 1 : 0;
        if (serial) blocks = 1;
        float* sc = to.var(sname)->df();
        float* lc = lname ? to.var(lname)->df() : sc;
        float g = cs.params.at("conductance");
        const int K = c.arbor.kernel();
        if (c.type == CONVERGENT && !c.convolutional && K <= kConvMaxK) {
            unsigned nb = blocks_for(c.to->size, 32);
            int sr = (int)c.from->output_type;
#define SG_CONV_TILE(SRV, LV)                                                                     \
    k_iz_activate_conv_tile<SRV, LV><<<nb, 256, 0, ctx.stream>>>(                                 \
        cs.geom, K, src, cs.weights->df(), cs.var("short term R")->df(),                        \
        cs.var("short term w")->df(), reinterpret_cast<const uint8_t*>(cs.delays8->du()),        \
        cs.var("short trace")->df(),                                                            \
        cs.var("long trace")->df(), g, stau, ltau, sc, lc)
            if (lname) {
                if (sr == S_FLOAT) SG_CONV_TILE(S_FLOAT, true);
                else if (sr == S_BIT) SG_CONV_TILE(S_BIT, true);
                else SG_CONV_TILE(S_INT, true);
            } else {
                if (sr == S_FLOAT) SG_CONV_TILE(S_FLOAT, false);
                else if (sr == S_BIT) SG_CONV_TILE(S_BIT, false);
                else SG_CONV_TILE(S_INT, false);
            }
#undef SG_CONV_TILE
            SG_LAUNCH_CHECK();
            ctx.count();
            return;
        }
        int nrows = 0, ncols = 0;
        if (matrix_shape(c, nrows, ncols)) {
            if (!cs.device_plan_tried) {
                cs.device_plan_tried = true;
                const bool bit = c.from->output_type == OUT_BIT;
                cs.device_plan = make_iz_cols_plan(
                    nrows, ncols, cs.weights->df(), cs.var("short term R")->df(),
                    cs.var("short term w")->df(),
                    bit ? reinterpret_cast<const uint8_t*>(cs.delays8->du()) : nullptr,
                    cs.var("short trace")->df(), lname ? cs.var("long trace")->df() : nullptr,
                    cs.eff_weights ? cs.eff_weights->df() : nullptr);
            }
            if (cs.device_plan) {
                launch_iz_cols_tma(*static_cast<IzColsPlan*>(cs.device_plan.get()), cs.geom,
                                   (int)c.from->output_type, c.type == SUBSET, src, g, stau, ltau,
                                   sc, lc, ctx.stream);
                ctx.count();
                return;
            }
        }
#define SG_IZ_ACT(LONG)                                                                        \
    SG_DISPATCH_TYPE_SRC((int)c.type, (int)c.from->output_type,                                \
        (k_iz_activate<TY, SR, LONG><<<blocks, threads, 0, ctx.stream>>>(                      \
            cs.geom, serial, src, cs.weights->df(), cs.var("short term R")->df(),              \
            cs.var("short term w")->df(), cs.delays->di(), cs.var("short trace")->df(),        \
            cs.var("long trace")->df(), g, stau, ltau, sc, lc)))
        if (lname) { SG_IZ_ACT(true); } else { SG_IZ_ACT(false); }
#undef SG_IZ_ACT
        SG_LAUNCH_CHECK();
        ctx.count();
    }

    void update(State& st, LayerState& ls, const StepCtx& ctx) const override {
        std::vector<LayerState*> one{&ls};
        update_group(st, one, ctx);
    }

    // All of a step's Izhikevich layers in one launch (kIzGroup at a time).
    bool update_group(State&, const std::vector<LayerState*>& group,
                      const StepCtx& ctx) const override {
        for (size_t first = 0; first < group.size(); first += kIzGroup) {
            IzUpdateGroup G{};
            G.n = (int)std::min<size_t>(kIzGroup, group.size() - first);
            int total = 0;
            for (int i = 0; i < G.n; ++i) {
                LayerState& ls = *group[first + i];
                const Layer& l = *ls.layer;
                G.start[i] = total;
                G.L[i] = IzLayerArgs{l.size, l.history(), ls.input->df(), ls.output->du(),
                                     ls.var("ampa")->df(), ls.var("nmda")->df(),
                                     ls.var("gabaa")->df(), ls.var("gabab")->df(),
                                     ls.var("mult")->df(), ls.var("dopamine")->df(),
                                     ls.var("voltage")->df(), ls.var("recovery")->df(),
                                     ls.var("post trace")->df(), ls.var("time since spike")->di(),
                                     ls.var("a")->df(), ls.var("b")->df(), ls.var("c")->df(),
                                     ls.var("d")->df()};
                total += l.size;
            }
            G.start[G.n] = total;
            if (total == 0) continue;
            k_iz_update<<<blocks_for(total, 256), 256, 0, ctx.stream>>>(G);
            SG_LAUNCH_CHECK();
            ctx.count();
        }
        return true;
    }

    bool learns(const Connection& c) const override { return true; }

    // get_updaters (izhikevich_attributes.cpp:522-539)
    void learn(State& st, ConnState& cs, const StepCtx& ctx) const override {
        Connection& c = *cs.conn;
        if (c.convolutional || (c.opcode != OP_ADD && c.opcode != OP_SUB))
            throw SgError(c.str() + ": Unimplemented connection type!");
        LayerState& to = *st.layer_state(c.to);
        static IzLut lut = [] {
            IzLut t{};
            for (int i = 1; i < 32; ++i) { t.src[i] = istdp_src(i); t.dst[i] = istdp_dst(i); }
            return t;
        }();
        const int threads = 128;
        unsigned blocks = blocks_for(cs.geom.n_dest, threads);
        bool sub = c.opcode == OP_SUB;
        if (c.type == CONVERGENT && c.arbor.kernel() <= kConvMaxK) {
            const int K = c.arbor.kernel();
            dim3 grid(blocks_for(c.to->size, 32), std::max(1, (K + 23) / 24));
            int sr = (int)c.from->output_type;
#define SG_CONV_LEARN(SRV, SUBV)                                                                  \
    do {                                                                                         \
        prefer_max_shared((const void*)k_iz_learn_conv_tile<SRV, SUBV>);                        \
        k_iz_learn_conv_tile<SRV, SUBV><<<grid, 256, 0, ctx.stream>>>(                            \
            cs.geom, K, st.dev_output(c.to, 0), to.var("post trace")->df(),                     \
            to.var("time since spike")->di(), cs.var("time since spike")->di(),                 \
            cs.params.at("learning rate"), (int)cs.params.at("stp"), c.max_weight,              \
            cs.weights->df(), cs.var("presyn trace")->df(), cs.var("weight derivatives")->df(), \
            cs.var("short term R")->df(), cs.var("short term w")->df(), lut);                   \
    } while (0)
            if (sub) {
                if (sr == S_FLOAT) SG_CONV_LEARN(S_FLOAT, true);
                else if (sr == S_BIT) SG_CONV_LEARN(S_BIT, true);
                else SG_CONV_LEARN(S_INT, true);
            } else {
                if (sr == S_FLOAT) SG_CONV_LEARN(S_FLOAT, false);
                else if (sr == S_BIT) SG_CONV_LEARN(S_BIT, false);
                else SG_CONV_LEARN(S_INT, false);
            }
#undef SG_CONV_LEARN
            SG_LAUNCH_CHECK();
            ctx.count();
            return;
        }
        int nrows = 0, ncols = 0;
        if (matrix_shape(c, nrows, ncols)) {
            int rpb = 32;
            dim3 grid(blocks_for(ncols, 256), blocks_for(nrows, rpb));
            bool subset = c.type == SUBSET;
#define SG_IZ_LEARN2D(SRV, SUBV, SSV)                                                           \
    k_iz_learn_2d<SRV, SUBV, SSV><<<grid, 256, 0, ctx.stream>>>(                                \
        cs.geom, nrows, ncols, rpb, st.dev_output(c.to, 0), to.var("post trace")->df(),        \
        to.var("time since spike")->di(), cs.var("time since spike")->di(),                    \
        cs.params.at("learning rate"), (int)cs.params.at("stp"), c.max_weight,                 \
        cs.weights->df(), cs.var("presyn trace")->df(), cs.var("weight derivatives")->df(),    \
        cs.var("short term R")->df(), cs.var("short term w")->df(), lut)
#define SG_IZ_LEARN2D_SR(SRV)                                                                   \
    if (sub) { if (subset) SG_IZ_LEARN2D(SRV, true, true); else SG_IZ_LEARN2D(SRV, true, false); } \
    else { if (subset) SG_IZ_LEARN2D(SRV, false, true); else SG_IZ_LEARN2D(SRV, false, false); }
            int sr = (int)c.from->output_type;
            if (sr == S_FLOAT) { SG_IZ_LEARN2D_SR(S_FLOAT) }
            else if (sr == S_BIT) { SG_IZ_LEARN2D_SR(S_BIT) }
            else { SG_IZ_LEARN2D_SR(S_INT) }
#undef SG_IZ_LEARN2D_SR
#undef SG_IZ_LEARN2D
            SG_LAUNCH_CHECK();
            ctx.count();
            return;
        }
#define SG_IZ_LEARN(SUBV)                                                                   \
    SG_DISPATCH_TYPE_SRC((int)c.type, (int)c.from->output_type,                                \
        (k_iz_learn<TY, SR, SUBV><<<blocks, threads, 0, ctx.stream>>>(                         \
            cs.geom, st.dev_output(c.to, 0), to.var("post trace")->df(),                       \
            to.var("time since spike")->di(), cs.var("time since spike")->di(),                \
            cs.params.at("learning rate"), (int)cs.params.at("stp"), c.max_weight,             \
            cs.weights->df(), cs.var("presyn trace")->df(), cs.var("weight derivatives")->df(), \
            cs.var("short term R")->df(), cs.var("short term w")->df(), lut)))
        if (sub) { SG_IZ_LEARN(true); } else { SG_IZ_LEARN(false); }
#undef SG_IZ_LEARN
        SG_LAUNCH_CHECK();
        ctx.count();
    }
};
SG_REGISTER_MODEL(IzhikevichModel);

// ---------------------------------------------------------------------------
// spnet (spnet_attributes.cpp): Izhikevich neurons driven by the plain
// current of their synapses, sum(spike * w * conductance), with STDP on a
// presynaptic trace (+0.1, decay 0.95) and the weight derivative
// dw = 0.9 dw + post * pre - ..., weights kept in [0.0001, max weight].
// Sources' time since spike and the per-synapse delays are the Izhikevich
// model's (same visit tables and kernels).
// ---------------------------------------------------------------------------
template <int TY, int SR>
__global__ void __launch_bounds__(128) k_spnet_activate(DGeom g, const uint32_t* __restrict__ src,
                                                        const float* __restrict__ w,
                                                        const int* __restrict__ delays, float gc,
                                                        int opcode, float* __restrict__ inputs) {
    const int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= g.n_dest) return;
    float sum = 0.0f;
    if constexpr (TY == T_SPARSE) {
        // 8 synapses' loads in flight, then their terms in order
        constexpr int U = 8;
        const int n = g.nz[d];
        int i = 0, wi = d;
        for (; i + U <= n; i += U, wi += U * g.to_size) {
            int fr[U], dl[U];
            float wv[U];
            uint32_t word[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int j = wi + u * g.to_size;
                fr[u] = g.sfrom[j];
                dl[u] = delays[j];
                wv[u] = w[j];
            }
#pragma unroll
            for (int u = 0; u < U; ++u) word[u] = src[fr[u]];
#pragma unroll
            for (int u = 0; u < U; ++u) sum += extract<SR>(word[u], dl[u]) * wv[u] * gc;
        }
        for (; i < n; ++i, wi += g.to_size) sum += extract<SR>(src[g.sfrom[wi]], delays[wi]) * w[wi] * gc;
    } else {
        for_each_source<TY>(g, d, [&](int from, int wi) {
            const float spike = extract<SR>(src[from], delays[wi]);
            sum += spike * w[wi] * gc;
        });
    }
    const int to = dest_of<TY>(g, d);
    inputs[to] = aggregate(inputs[to], sum, opcode);
}

// spnet_attributes.cpp:96-166, the reference's expressions as written: the
// double constants promote, and the float stores round.
__global__ void __launch_bounds__(256) k_spnet_update(int size, int history, const float* __restrict__ in,
                                                      uint32_t* spikes, float* vs, float* rs, float* post,
                                                      int* tss, const float* __restrict__ as,
                                                      const float* __restrict__ bs,
                                                      const float* __restrict__ cs,
                                                      const float* __restrict__ ds) {
    const int nid = blockIdx.x * blockDim.x + threadIdx.x;
    if (nid >= size) return;
    float voltage = vs[nid];
    float recovery = rs[nid];
    const float current = in[nid];
    const float a = as[nid], b = bs[nid];
    for (int i = 0; (i < 10) && (voltage < 30.0); ++i) {
        const float delta_v = (0.04 * voltage * voltage) + (5 * voltage) + 140 - recovery + current;
        voltage += delta_v * 0.1;
        voltage = (voltage != voltage) ? 30.0f : voltage;
        const float adjusted_tau = (voltage > 30.0) ? delta_v / (30.0 - voltage + delta_v) * 0.1 : 0.1;
        recovery += a * adjusted_tau * ((b * voltage) - recovery);
    }
    const uint32_t spike = voltage >= 30.0;
    const uint32_t prev_bit = shift_bits(spikes, size, history, nid, spike);
    post[nid] = prev_bit ? (float)(post[nid] + 0.1) : (float)(post[nid] * 0.95);
    tss[nid] = prev_bit ? 0 : min(32, tss[nid] + 1);
    vs[nid] = spike ? cs[nid] : voltage;
    rs[nid] = recovery + (spike * ds[nid]);
}

// spnet_attributes.cpp:220-286 ("add": presynaptic trace against the
// postsynaptic trace; "sub": the inverse-STDP terms of the time since spike,
// tabulated on the host with the host's powf / expf).
template <int TY, int SR, bool SUB>
__global__ void __launch_bounds__(128) k_spnet_learn(DGeom g, const uint32_t* __restrict__ dest_out,
                                                     const float* __restrict__ post,
                                                     const int* __restrict__ to_tss,
                                                     const int* __restrict__ from_tss, float lr,
                                                     float max_weight, float* w, float* presyn,
                                                     float* dws, IzLut lut) {
    const int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= g.n_dest) return;
    const int to = dest_of<TY>(g, d);
    const float dest_exc = post[to];
    const int dtss = to_tss[to];
    const float dest_spike = extract<SR>(dest_out[to], 0);    // the source's extractor
    for_each_source<TY>(g, d, [&](int from, int wi) {
        float weight = w[wi];
        if (!(weight >= 0.0001f)) return;
        const int stss = from_tss[from];
        const bool src_spike = stss == 0;
        float src_trace, dest_trace;
        if (!SUB) {
            const float p = presyn[wi];
            src_trace = presyn[wi] = src_spike ? (float)(p + 0.1) : (float)(p * 0.95);
            dest_trace = dest_exc;
        } else {
            src_trace = (dest_spike > 0.0f && stss > 0 && stss < 32) ? lut.src[stss] : 0.0f;
            dest_trace = (src_spike && dtss > 0 && dtss < 32) ? lut.dst[dtss] : 0.0f;
        }
        const float dw = 0.9 * dws[wi] + (dest_spike * src_trace) - (src_spike * dest_trace);
        dws[wi] = dw;
        const float weight_delta = dw + 0.01;
        weight += lr * weight_delta;
        const float capped = (max_weight < weight) ? max_weight : weight;
        w[wi] = (0.0001f > capped) ? 0.0001f : capped;
    });
}

// The STDP kernel's rare double expressions, out of line (see f2d_hw).
static __device__ __noinline__ float spnet_trace_step(float p) { return (float)(p + 0.1); }
static __device__ __noinline__ float spnet_dw_full(float dw0, float f1, float f2) {
    return d2f_rn(__dadd_rn(__dadd_rn(mul_df_rn(dw0, 0.9), f2d_exact(f1)), -f2d_exact(f2)));
}

// Sparse connections: one thread per compacted synapse (blockIdx.y is the
// synapse's rank within its destination, x the destination), since each
// synapse's update is independent.  The products with 0.9 / 0.95 and the
// sums with 0.1 / 0.01 are float-float evaluations with a rounding test
// (ff_exact.cuh), falling back to the integer helpers and double sums where
// the test rejects; the full weight-derivative sum with spike terms stays
// double.  Bit-identical to k_spnet_learn.
template <int SR, bool SUB>
__global__ void __launch_bounds__(256) k_spnet_learn_sparse(DGeom g, const uint32_t* __restrict__ dest_out,
                                                            const float* __restrict__ post,
                                                            const int* __restrict__ to_tss,
                                                            const int* __restrict__ from_tss, float lr,
                                                            float max_weight, float* __restrict__ w,
                                                            float* __restrict__ presyn,
                                                            float* __restrict__ dws, IzLut lut) {
    const int d = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y;
    if (d >= g.to_size) return;
    // every load that depends on nothing but the synapse's position first
    // (the [kmax][to] arrays are allocated for the padding too), then the
    // checks, then the source's time since spike
    const int wi = i * g.to_size + d;
    const int n = g.nz[d];
    float weight = w[wi];
    const int from = g.sfrom[wi];
    const float p = SUB ? 0.0f : presyn[wi];
    const float dw0 = dws[wi];
    const uint32_t dword = dest_out[d];
    const float dest_exc = SUB ? 0.0f : post[d];
    const int dtss = SUB ? to_tss[d] : 0;
    if (i >= n || !(weight >= 0.0001f)) return;
    const int stss = from_tss[from];
    const bool src_spike = stss == 0;
    const float dest_spike = extract<SR>(dword, 0);          // the source's extractor
    float src_trace, dest_trace;
    if (!SUB) {
        float np;
        constexpr float T1 = (float)0.1, T2 = (float)(0.1 - (double)T1);
        constexpr float D1 = (float)0.95, D2 = (float)(0.95 - (double)D1);
        if (src_spike) {
            if (!ff::add_const(p, T1, T2, np)) np = spnet_trace_step(p);
        } else if (!ff::product(p, D1, D2, np)) {
            np = mul_fd_rn(p, 0.95);
        }
        src_trace = presyn[wi] = np;
        dest_trace = dest_exc;
    } else {
        src_trace = (dest_spike > 0.0f && stss > 0 && stss < 32) ? lut.src[stss] : 0.0f;
        dest_trace = (src_spike && dtss > 0 && dtss < 32) ? lut.dst[dtss] : 0.0f;
    }
    const float f1 = dest_spike * src_trace;
    const float f2 = (src_spike ? 1.0f : 0.0f) * dest_trace;
    // 0.9 dw + f1 - f2 in double: with f1, f2 zero and dw nonzero it is the
    // rounded product alone
    float dw;
    constexpr float N1 = (float)0.9, N2 = (float)(0.9 - (double)N1);
    constexpr float S1 = (float)0.01, S2 = (float)(0.01 - (double)S1);
    if (f1 == 0.0f && f2 == 0.0f && dw0 != 0.0f) {
        if (!ff::product(dw0, N1, N2, dw)) dw = mul_fd_rn(dw0, 0.9);
    } else {
        dw = spnet_dw_full(dw0, f1, f2);
    }
    dws[wi] = dw;
    float weight_delta;
    if (!ff::add_const(dw, S1, S2, weight_delta)) weight_delta = d2f_rn(__dadd_rn(f2d_exact(dw), 0.01));
    weight += lr * weight_delta;
    const float capped = (max_weight < weight) ? max_weight : weight;
    w[wi] = (0.0001f > capped) ? 0.0001f : capped;
}

class SpnetModel : public Model {
  public:
    const char* name() const override { return "spnet"; }
    OutputType output_type() const override { return OUT_BIT; }

    void prepare_device(State&, ConnState& cs, cudaStream_t s) const override {
        if (!cs.delay_summary) return;
        const int n = cs.conn->from->size;
        k_iz_delay_summary<<<blocks_for(n, 256), 256, 0, s>>>(
            n, cs.visit_counts->di(), cs.last_visits->di(), cs.delays->di(),
            reinterpret_cast<unsigned long long*>(cs.delay_summary->di()));
        SG_LAUNCH_CHECK();
    }

    void build_layer(State& st, LayerState& ls) const override {
        const Layer& l = *ls.layer;
        for (const char* k : {"voltage", "recovery", "post trace", "a", "b", "c", "d"})
            ls.vars[k] = st.add_array(k, 'f', l.size);
        ls.vars["time since spike"] = st.add_array("time since spike", 'i', l.size);
        iz_params_and_rest(ls);
    }

    // process_weight_matrix and the activator / updater checks
    // (spnet_attributes.cpp:202-214, 288-306, 440-494)
    void build_matrix(State& st, ConnState& cs) const override {
        Connection& c = *cs.conn;
        if (c.second_order) throw SgError(c.str() + ": Unimplemented connection type!");
        if (c.plastic && (c.convolutional || (c.opcode != OP_ADD && c.opcode != OP_SUB)))
            throw SgError(c.str() + ": Unimplemented connection type!");
        const size_t n = c.num_weights;
        cs.params["conductance"] = std::stof(c.parameter("conductance", "1.0"));
        cs.params["learning rate"] = std::stof(c.parameter("learning rate", "0.1"));
        for (const char* k : {"presyn trace", "weight derivative"})
            cs.vars[k] = st.add_array(k, 'f', n, matrix_layout(c), c.matrix_rows, c.matrix_cols);
        const size_t tss_n = std::max<size_t>(n, c.from->size);
        cs.vars["time since spike"] = st.add_array("time since spike", 'i', tss_n, LAYOUT_SOURCE,
                                                   1, 1, c.from->size);
        int32_t* tss = cs.vars["time since spike"]->hi();
        for (size_t i = 0; i < tss_n; ++i) tss[i] = 32;
        iz_delays_and_visits(st, cs);
    }

    void activate(State& st, ConnState& cs, const StepCtx& ctx) const override {
        const Connection& c = *cs.conn;
        const uint32_t* src = st.dev_output(c.from, word_index(c.delay, c.from->output_type));
        k_iz_time_since_spike<<<blocks_for(c.from->size, 256), 256, 0, ctx.stream>>>(
            c.from->size, cs.visit_counts->di(), cs.last_visits->di(), cs.delays->di(),
            reinterpret_cast<const unsigned long long*>(cs.delay_summary->di()), src, (int)c.from->output_type, cs.var("time since spike")->di());
        SG_LAUNCH_CHECK();
        const unsigned blocks = blocks_for(cs.geom.n_dest, 128);
        float* inputs = input_register(st, cs);
        SG_DISPATCH_TYPE_SRC((int)c.type, (int)c.from->output_type,
            (k_spnet_activate<TY, SR><<<blocks, 128, 0, ctx.stream>>>(
                cs.geom, src, cs.weights->df(), cs.delays->di(), cs.params.at("conductance"),
                (int)c.opcode, inputs)));
        SG_LAUNCH_CHECK();
        ctx.count(2);
    }

    void update(State&, LayerState& ls, const StepCtx& ctx) const override {
        const Layer& l = *ls.layer;
        k_spnet_update<<<blocks_for(l.size, 256), 256, 0, ctx.stream>>>(
            l.size, l.history(), ls.input->df(), ls.output->du(), ls.var("voltage")->df(),
            ls.var("recovery")->df(), ls.var("post trace")->df(), ls.var("time since spike")->di(),
            ls.var("a")->df(), ls.var("b")->df(), ls.var("c")->df(), ls.var("d")->df());
        SG_LAUNCH_CHECK();
        ctx.count();
    }

    bool learns(const Connection& c) const override { return true; }

    void learn(State& st, ConnState& cs, const StepCtx& ctx) const override {
        const Connection& c = *cs.conn;
        LayerState& to = *st.layer_state(c.to);
        static IzLut lut = [] {
            IzLut t{};
            for (int i = 1; i < 32; ++i) { t.src[i] = istdp_src(i); t.dst[i] = istdp_dst(i); }
            return t;
        }();
        if (c.type == SPARSE) {
            const dim3 grid(blocks_for(c.to->size, 256), std::max(1, cs.geom.kmax));
#define SG_SPNET_SPARSE(SRV, SUBV)                                                              \
    k_spnet_learn_sparse<SRV, SUBV><<<grid, 256, 0, ctx.stream>>>(                              \
        cs.geom, st.dev_output(c.to, 0), to.var("post trace")->df(),                           \
        to.var("time since spike")->di(), cs.var("time since spike")->di(),                    \
        cs.params.at("learning rate"), c.max_weight, cs.weights->df(),                         \
        cs.var("presyn trace")->df(), cs.var("weight derivative")->df(), lut)
            const bool sub = c.opcode == OP_SUB;
            switch ((int)c.from->output_type) {
                case 0: if (sub) SG_SPNET_SPARSE(0, true); else SG_SPNET_SPARSE(0, false); break;
                case 1: if (sub) SG_SPNET_SPARSE(1, true); else SG_SPNET_SPARSE(1, false); break;
                default: if (sub) SG_SPNET_SPARSE(2, true); else SG_SPNET_SPARSE(2, false); break;
            }
#undef SG_SPNET_SPARSE
            SG_LAUNCH_CHECK();
            ctx.count();
            return;
        }
        const unsigned blocks = blocks_for(cs.geom.n_dest, 128);
#define SG_SPNET_LEARN(SUBV)                                                                    \
    SG_DISPATCH_TYPE_SRC((int)c.type, (int)c.from->output_type,                                \
        (k_spnet_learn<TY, SR, SUBV><<<blocks, 128, 0, ctx.stream>>>(                          \
            cs.geom, st.dev_output(c.to, 0), to.var("post trace")->df(),                       \
            to.var("time since spike")->di(), cs.var("time since spike")->di(),                \
            cs.params.at("learning rate"), c.max_weight, cs.weights->df(),                     \
            cs.var("presyn trace")->df(), cs.var("weight derivative")->df(), lut)))
        if (c.opcode == OP_SUB) { SG_SPNET_LEARN(true); } else { SG_SPNET_LEARN(false); }
#undef SG_SPNET_LEARN
        SG_LAUNCH_CHECK();
        ctx.count();
    }
};
SG_REGISTER_MODEL(SpnetModel);

}  // namespace sg
