// Device-side synapse geometry and per-destination source iteration.
//
// One destination's sources are visited in exactly the order of the
// reference's loops (src/core/engine/kernel/synapse_kernel.h):
//   fully connected  from ascending                         :115-149
//   subset           window rows, then columns              :182-228
//   one to one       the destination itself                 :257-286
//   convergent       kernel rows/cols, wrap or skip          :384-461
//   divergent        inverse window, C truncating division   :506-581
//   sparse           the destination's compacted synapses    :303-366
// Weight indices are in the device layout.  Fully connected and subset
// matrices are stored in bands of kBand consecutive destinations,
// [destination / kBand][source][destination % kBand] (banded_index), so the
// stream of a band of destinations is contiguous in HBM and a chunk of its
// rows is one block; arborized matrices keep consecutive destinations
// contiguous:
//   fully connected  banded_index(to, from, from_size)
//   subset           banded_index(to_k, from_k, from_k_size)
//   one to one       w[i]
//   convergent       w[k * to_size + to]   (convolutional: w[k])
//   divergent        w[k * to_size + to]   (convolutional: w[k])
//   sparse           w[k * to_size + to]
// Floating-point order is the reference's serial order; the library is built
// with --fmad=false so no multiply-add is contracted.
#pragma once
#include <cstdint>

namespace sg {

struct DGeom {
    int type, conv;
    int from_rows, from_cols, from_size;
    int to_rows, to_cols, to_size;
    int rf, cf, rs, cs, rsp, csp, ro, co, wrap;
    int fr0, fr1, fc0, fc1, tr0, tc0, tk_cols, tk_size;
    int n_dest;
    // Every wrapped source coordinate lies in [-n, 2n): one conditional add or
    // subtract gives the same result as ((x % n) + n) % n.
    int wrap_fast;
    // Sparse: synapses per destination and their sources, [k][to] like the
    // weights (device pointers, set once the state is on the device).
    int kmax;
    const int* nz;
    const int* sfrom;
};

enum { T_FC = 0, T_SUBSET = 1, T_ONE = 2, T_CONV = 3, T_DIV = 4, T_SPARSE = 5 };

constexpr int kBand = 8;

#ifdef __CUDACC__
#define SG_HOST_DEVICE __host__ __device__ __forceinline__
#else
#define SG_HOST_DEVICE inline
#endif

// Device index of (destination, source) in a banded matrix with nsrc sources.
SG_HOST_DEVICE long banded_index(long dest, long src, long nsrc) {
    return (dest / kBand) * (nsrc * kBand) + src * kBand + dest % kBand;
}
enum { S_FLOAT = 0, S_BIT = 1, S_INT = 2 };

#ifdef __CUDACC__

// extractor.cpp:6-24
template <int SRC>
__device__ __forceinline__ float extract(uint32_t word, int delay) {
    if (SRC == S_FLOAT) return __uint_as_float(word);
    if (SRC == S_INT) return (float)word;
    return (float)((word << (delay & 0x1F)) >> 31);
}

__device__ __forceinline__ float extract_rt(uint32_t word, int delay, int src) {
    if (src == S_FLOAT) return __uint_as_float(word);
    if (src == S_INT) return (float)word;
    return (float)((word << (delay & 0x1F)) >> 31);
}

// aggregator.cpp:83-98 (fmaxf keeps the CPU path's std::fmax NaN handling)
__device__ __forceinline__ float aggregate(float prior, float input, int opcode) {
    switch (opcode) {
        case 0: return prior + input;                    // add
        case 1: return prior - input;                    // sub
        case 2: return prior * input;                    // mult
        case 3: return prior / input;                    // div
        case 4: return fmaxf(prior, input);              // pool
        case 8: return prior + (float)(input > 0.0f);    // add_heaviside
        case 9: return prior - (float)(input > 0.0f);    // sub_heaviside
        case 10: return prior * (float)(input > 0.0f);   // mult_heaviside
        default: return prior + input;
    }
}

__device__ __forceinline__ int wrap_idx(int x, int n) { return (x % n + n) % n; }

__device__ __forceinline__ int wrap_coord(const DGeom& g, int x, int n) {
    if (g.wrap_fast) return x < 0 ? x + n : (x >= n ? x - n : x);
    return wrap_idx(x, n);
}

// Destination index of iteration d (subset iterates its window only).
template <int TYPE>
__device__ __forceinline__ int dest_of(const DGeom& g, int d) {
    if (TYPE == T_SUBSET) return (d / g.tk_cols + g.tr0) * g.to_cols + (d % g.tk_cols + g.tc0);
    return d;
}

// Calls f(from_index, weight_index) for every source of destination
// iteration d in the reference's serial order.
template <int TYPE, class F>
__device__ __forceinline__ void for_each_source(const DGeom& g, int d, F&& f) {
    if (TYPE == T_FC) {
        int wi = (int)banded_index(d, 0, g.from_size);
        for (int from = 0; from < g.from_size; ++from, wi += kBand) f(from, wi);
    } else if (TYPE == T_SUBSET) {
        int wi = (int)banded_index(d, 0, (g.fr1 - g.fr0) * (g.fc1 - g.fc0));
        for (int fr = g.fr0; fr < g.fr1; ++fr)
            for (int fc = g.fc0; fc < g.fc1; ++fc, wi += kBand) f(fr * g.from_cols + fc, wi);
    } else if (TYPE == T_ONE) {
        f(d, d);
    } else if (TYPE == T_CONV) {
        const int tr = d / g.to_cols, tc = d % g.to_cols;
        const int s_row = tr * g.rs + g.rsp * g.ro;
        const int s_col = tc * g.cs + g.csp * g.co;
        int k = 0;
        for (int kr = 0; kr < g.rf; ++kr) {
            int fr = s_row + kr * g.rsp;
            bool row_ok = true;
            if (g.wrap) fr = wrap_coord(g, fr, g.from_rows);
            else row_ok = fr >= 0 && fr < g.from_rows;
            for (int kc = 0; kc < g.cf; ++kc, ++k) {
                int fc = s_col + kc * g.csp;
                if (g.wrap) fc = wrap_coord(g, fc, g.from_cols);
                else if (!row_ok || fc < 0 || fc >= g.from_cols) continue;
                f(fr * g.from_cols + fc, g.conv ? k : k * g.to_size + d);
            }
        }
    } else if (TYPE == T_SPARSE) {
        const int n = g.nz[d];
        int wi = d;
        for (int i = 0; i < n; ++i, wi += g.to_size) f(g.sfrom[wi], wi);
    } else {  // T_DIV
        const int tr = d / g.to_cols, tc = d % g.to_cols;
        const int sr0 = (tr + g.rsp * (-g.ro - g.rf + g.rs)) / g.rs;
        const int sc0 = (tc + g.csp * (-g.co - g.cf + g.cs)) / g.cs;
        const int sr1 = sr0 + (g.rsp * (g.rf - g.rs) / g.rs);
        const int sc1 = sc0 + (g.csp * (g.cf - g.cs) / g.cs);
        int k = 0;
        for (int sr = sr0; sr <= sr1; sr += g.rsp) {
            int fr = sr;
            bool row_ok = true;
            if (g.wrap) fr = wrap_coord(g, fr, g.from_rows);
            else row_ok = fr >= 0 && fr < g.from_rows;
            for (int sc = sc0; sc <= sc1; sc += g.csp, ++k) {
                int fc = sc;
                if (g.wrap) fc = wrap_coord(g, fc, g.from_cols);
                else if (!row_ok || fc < 0 || fc >= g.from_cols) continue;
                f(fr * g.from_cols + fc, g.conv ? k : k * g.to_size + d);
            }
        }
    }
}

#endif  // __CUDACC__

// Host-side dispatch helper: instantiates KERNEL<TYPE, SRC> for the runtime
// (type, source output type) pair.
#define SG_DISPATCH_TYPE_SRC(TYPE_RT, SRC_RT, BODY)                                   \
    switch ((TYPE_RT) * 3 + (SRC_RT)) {                                               \
        case 0: { constexpr int TY = 0, SR = 0; BODY; } break;                        \
        case 1: { constexpr int TY = 0, SR = 1; BODY; } break;                        \
        case 2: { constexpr int TY = 0, SR = 2; BODY; } break;                        \
        case 3: { constexpr int TY = 1, SR = 0; BODY; } break;                        \
        case 4: { constexpr int TY = 1, SR = 1; BODY; } break;                        \
        case 5: { constexpr int TY = 1, SR = 2; BODY; } break;                        \
        case 6: { constexpr int TY = 2, SR = 0; BODY; } break;                        \
        case 7: { constexpr int TY = 2, SR = 1; BODY; } break;                        \
        case 8: { constexpr int TY = 2, SR = 2; BODY; } break;                        \
        case 9: { constexpr int TY = 3, SR = 0; BODY; } break;                        \
        case 10: { constexpr int TY = 3, SR = 1; BODY; } break;                       \
        case 11: { constexpr int TY = 3, SR = 2; BODY; } break;                       \
        case 12: { constexpr int TY = 4, SR = 0; BODY; } break;                       \
        case 13: { constexpr int TY = 4, SR = 1; BODY; } break;                       \
        case 14: { constexpr int TY = 4, SR = 2; BODY; } break;                       \
        case 15: { constexpr int TY = 5, SR = 0; BODY; } break;                       \
        case 16: { constexpr int TY = 5, SR = 1; BODY; } break;                       \
        case 17: { constexpr int TY = 5, SR = 2; BODY; } break;                       \
    }

}  // namespace sg
