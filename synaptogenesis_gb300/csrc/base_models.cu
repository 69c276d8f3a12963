// Base activator (all connection types, every opcode) and the stateless
// neural models: relay, rate_encoding, game_of_life.
#include <algorithm>
#include <cmath>

#include "gol_step.cuh"
#include "cuda_check.h"
#include "history.cuh"
#include "models.h"
#include "state.h"

namespace sg {

// ---------------------------------------------------------------------------
// Model registry (neural_model_bank.cpp:21-83)
// ---------------------------------------------------------------------------
static std::map<std::string, const Model*>& registry() {
    static std::map<std::string, const Model*> r;
    return r;
}

const Model* find_model(const std::string& name) {
    auto it = registry().find(name);
    return it == registry().end() ? nullptr : it->second;
}

bool register_model(const Model* m) {
    if (registry().count(m->name()))
        throw SgError(std::string("Duplicate attributes neural model string: ") + m->name() + "!");
    registry()[m->name()] = m;
    return true;
}

std::vector<std::string> model_names() {
    std::vector<std::string> out;
    for (auto& kv : registry()) out.push_back(kv.first);
    return out;
}

// ---------------------------------------------------------------------------
// Base activator: one thread per destination, sources in serial order,
// sequential fp32 sum (synapse_kernel.h:887-912).
// ---------------------------------------------------------------------------
template <int TY, int SR>
__global__ void __launch_bounds__(256) k_activate_base(DGeom g, const uint32_t* __restrict__ src,
                                                       int delay, int opcode,
                                                       const float* __restrict__ w,
                                                       float* __restrict__ inputs) {
    int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= g.n_dest) return;
    float sum = 0.0f;
    for_each_source<TY>(g, d, [&](int from, int wi) {
        float val = extract<SR>(src[from], delay) * w[wi];
        sum += val;
    });
    int to = dest_of<TY>(g, d);
    inputs[to] = aggregate(inputs[to], sum, opcode);
}

void launch_base_activator(State& st, ConnState& cs, float* inputs, cudaStream_t s) {
    const Connection& c = *cs.conn;
    const uint32_t* src = st.dev_output(c.from, word_index(c.delay, c.from->output_type));
    const int threads = 128;
    unsigned blocks = blocks_for(cs.geom.n_dest, threads);
    // a second-order host reads the copy of its weights the slaves modulated
    // (synapse_data.cpp:20-23)
    const float* w = cs.so_weights ? cs.so_weights->df() : cs.weights->df();
    SG_DISPATCH_TYPE_SRC((int)c.type, (int)c.from->output_type,
        (k_activate_base<TY, SR><<<blocks, threads, 0, s>>>(cs.geom, src, c.delay, (int)c.opcode,
                                                           w, inputs)));
    SG_LAUNCH_CHECK();
}

float* input_register(State& st, const ConnState& cs) {
    const Layer* l = cs.conn->to;
    return st.layer_state(cs.conn->to)->input->df() + (size_t)cs.reg * l->size;
}

void Model::activate(State& st, ConnState& cs, const StepCtx& ctx) const {
    launch_base_activator(st, cs, input_register(st, cs), ctx.stream);
    ctx.count();
}

// ---------------------------------------------------------------------------
// Dendritic trees and second-order connections
// ---------------------------------------------------------------------------
// Second-order slave (ACTIVATE_ALL_SECOND_ORDER, synapse_kernel.h:918-975):
// every visited synapse modulates the host's weight copy with the slave's own
// opcode, so[wi] = aggregate(so[wi], extract(out[from]) * w[wi]).  Each
// weight index belongs to one destination, so threads never share an entry.
template <int TY, int SR>
__global__ void __launch_bounds__(256) k_activate_second_order(DGeom g, const uint32_t* __restrict__ src,
                                                               int delay, int opcode,
                                                               const float* __restrict__ w,
                                                               const int* __restrict__ remap,
                                                               float* __restrict__ so) {
    int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= g.n_dest) return;
    for_each_source<TY>(g, d, [&](int from, int wi) {
        const float val = extract<SR>(src[from], delay) * w[wi];
        const int si = remap ? remap[wi] : wi;
        so[si] = aggregate(so[si], val, opcode);
    });
}

// Convolutional slave: a one-to-one pass over the shared kernel, whose size
// is the source layer's (CALC_ONE_TO_ONE of the same macros).
template <int SR>
__global__ void k_activate_second_order_conv(int n, const uint32_t* __restrict__ src, int delay,
                                             int opcode, const float* __restrict__ w,
                                             float* __restrict__ so) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    so[k] = aggregate(so[k], extract<SR>(src[k], delay) * w[k], opcode);
}

void launch_second_order_slave(State& st, ConnState& cs, float* so, cudaStream_t s) {
    const Connection& c = *cs.conn;
    const uint32_t* src = st.dev_output(c.from, word_index(c.delay, c.from->output_type));
    const int sr = (int)c.from->output_type;
    if (c.convolutional) {
        const int n = c.from->size;
        unsigned blocks = blocks_for(n, 256);
        switch (sr) {
            case 0: k_activate_second_order_conv<0><<<blocks, 256, 0, s>>>(n, src, c.delay, (int)c.opcode, cs.weights->df(), so); break;
            case 1: k_activate_second_order_conv<1><<<blocks, 256, 0, s>>>(n, src, c.delay, (int)c.opcode, cs.weights->df(), so); break;
            default: k_activate_second_order_conv<2><<<blocks, 256, 0, s>>>(n, src, c.delay, (int)c.opcode, cs.weights->df(), so); break;
        }
    } else {
        const int* remap = cs.so_remap ? cs.so_remap->di() : nullptr;
        unsigned blocks = blocks_for(cs.geom.n_dest, 128);
        SG_DISPATCH_TYPE_SRC((int)c.type, sr,
            (k_activate_second_order<TY, SR><<<blocks, 128, 0, s>>>(cs.geom, src, c.delay, (int)c.opcode,
                                                                    cs.weights->df(), remap, so)));
    }
    SG_LAUNCH_CHECK();
}

// calc_internal (kernel.cpp:160-182): fold a node's register into its
// parent's with the node's opcode, then reset it to the node's init value.
__global__ void k_dendrite_fold(int n, float* __restrict__ src, float* __restrict__ dst, int opcode,
                                float trail) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    dst[i] = aggregate(dst[i], src[i], opcode);
    src[i] = trail;
}

void launch_dendrite_fold(int n, float* src, float* dst, int opcode, float trail, cudaStream_t s) {
    k_dendrite_fold<<<blocks_for(n, 256), 256, 0, s>>>(n, src, dst, opcode, trail);
    SG_LAUNCH_CHECK();
}

// relay_attributes.cpp:10-18 (the ramp is std::fmax on doubles, i.e. fmax)
__global__ void k_relay(int size, int history, const float* __restrict__ in, float* out, int ramp) {
    int nid = blockIdx.x * blockDim.x + threadIdx.x;
    if (nid >= size) return;
    float input = in[nid];
    shift_floats(out, size, history, nid, ramp ? (float)fmax(0.0, (double)input) : input);
}

// rate_encoding_attributes.cpp:122-131 (tanh of a float is tanhf)
__global__ void k_rate(int size, int history, const float* __restrict__ in, float* out) {
    int nid = blockIdx.x * blockDim.x + threadIdx.x;
    if (nid >= size) return;
    float input = in[nid];
    shift_floats(out, size, history, nid, (input > 0.0f) ? tanhf(input) : 0.0f);
}

// game_of_life_attributes.cpp:58-77: prev_live is bit 0 of word 0, i.e. the
// cell 32 steps back, while neighbours are read at delay 0 (bit 31).
__global__ void k_gol(int size, int history, const float* __restrict__ in, uint32_t* out,
                      int smin, int smax, int bmin, int bmax) {
    int nid = blockIdx.x * blockDim.x + threadIdx.x;
    if (nid >= size) return;
    int input = (int)in[nid];
    bool prev_live = out[nid] & 1u;
    bool live = prev_live ? (input >= smin && input <= smax) : (input >= bmin && input <= bmax);
    shift_bits(out, size, history, nid, live ? 1u : 0u);
}

// Fused game_of_life step for a layer whose only input is its own convergent
// connection: the base activator's sequential weighted count (prior 0, "add"),
// the life rule and the history shift in one pass.  Reads the output words of
// step t-1 from `cur` and writes step t to `next` (ping-pong), so every other
// reader of the layer still sees step t-1.  2-D blocks keep the neighbour
// words of a block in L1.
__global__ void __launch_bounds__(256) k_gol_fused(DGeom g, int delay, const uint32_t* __restrict__ cur,
                                                   uint32_t* __restrict__ next,
                                                   const float* __restrict__ w,
                                                   float* __restrict__ input_out, int smin, int smax,
                                                   int bmin, int bmax) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    int r = blockIdx.y * blockDim.y + threadIdx.y;
    if (c >= g.to_cols || r >= g.to_rows) return;
    gol_cell_step(g, delay, r, c, cur, next, w, input_out, smin, smax, bmin, bmax);
}

// Bit-sliced game_of_life step (same semantics as k_gol_fused) for a 3x3
// kernel whose weights are all 0 or 1, stride 1, spacing 1, offset -1, and
// rows of whole 32-cell segments.  With 0/1 weights the reference's fp32
// sequential sum is an exact integer count, so counting bits is exact.  For
// one 32-cell segment of one row, the step
//   * gathers bit (31 - delay) of the 32 history words into a plane word, for
//     the rows above, itself and below, plus the boundary bits of the
//     neighbouring segments (west / east shifts, wrap or zero);
//   * adds the planes selected by the weight mask with a bit-sliced counter
//     (c3 c2 c1 c0 per cell);
//   * evaluates survival / birth as plane logic against bit 0 (the state 32
//     steps back);
//   * shifts the new bit into its 32 words and stores them.
__device__ __forceinline__ uint32_t newest_bit(uint32_t w, int delay) { return (w << delay) >> 31; }

__device__ __forceinline__ void csa_add(uint32_t& c0, uint32_t& c1, uint32_t& c2, uint32_t& c3,
                                        uint32_t x) {
    uint32_t t = c0 & x; c0 ^= x; x = t;
    t = c1 & x; c1 ^= x; x = t;
    t = c2 & x; c2 ^= x; x = t;
    c3 ^= x;
}

// The bit-sliced step in shared-memory tiles.  A CTA (8 warps) owns 8 rows of
// a 1024-cell strip (32 segments).  It stages the 8 rows plus one halo row
// above and below with coalesced 128-bit loads into shared memory, padded to
// 33 words per segment so that lane j reading word i of its own segment hits
// bank (j + i) mod 32 (conflict free).  Warp w then processes row w of the
// tile with one lane per segment (plane gather, bit-sliced count, rule),
// writes its new words back into the tile, and the CTA stores the tile with
// coalesced 128-bit stores.
constexpr int kTileRows = 8;
constexpr int kSegPad = 33;

__global__ void __launch_bounds__(256) k_gol_bits_tile(int rows, int cols, int wrap, int delay,
                                                       unsigned mask9, const uint32_t* __restrict__ cur,
                                                       uint32_t* __restrict__ next,
                                                       float* __restrict__ input_out, unsigned smask,
                                                       unsigned bmask) {
    __shared__ uint32_t tile[kTileRows + 2][32 * kSegPad];
    __shared__ uint32_t cnt[4][kTileRows][32];
    const int segs = cols >> 5;
    const int sx = blockIdx.x;                 // strip
    const int r0 = blockIdx.y * kTileRows;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int strip_segs = min(32, segs - sx * 32);
    const int strip_words = strip_segs * 32;
    // stage rows r0-1 .. r0+kTileRows (wrapping or zero outside the board)
    for (int e = tid; e < (kTileRows + 2) * 256; e += 256) {
        int tr = e >> 8, q = e & 255;          // 256 uint4 per 1024-word row
        int rr = r0 - 1 + tr;
        bool valid = true;
        if (wrap) rr = rr < 0 ? rr + rows : (rr >= rows ? rr - rows : rr);
        else valid = rr >= 0 && rr < rows;
        uint4 v = make_uint4(0, 0, 0, 0);
        if (valid && rr < rows && 4 * q < strip_words)
            v = __ldg(reinterpret_cast<const uint4*>(cur + (size_t)rr * cols + sx * 1024) + q);
        int word = 4 * q, sg = word >> 5, i = word & 31;
        uint32_t* dst = &tile[tr][sg * kSegPad + i];
        dst[0] = v.x; dst[1] = v.y; dst[2] = v.z; dst[3] = v.w;
    }
    __syncthreads();
    const int r = r0 + warp;
    const bool row_ok = r < rows;
    const bool seg_ok = lane < strip_segs;
    uint32_t N[3], W[3], E[3], O = 0;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const uint32_t* t = &tile[warp + k][lane * kSegPad];
        uint32_t P = 0;
#pragma unroll
        for (int i = 0; i < 32; ++i) {
            uint32_t wv = t[i];
            P |= newest_bit(wv, delay) << i;
            if (k == 1) O |= (wv & 1u) << i;
        }
        // Boundary cells of the neighbouring segments: in the tile within the
        // strip, from the board across strips.
        uint32_t west = __shfl_up_sync(0xffffffffu, P, 1) >> 31;
        uint32_t east = __shfl_down_sync(0xffffffffu, P, 1) & 1u;
        int rr = r + k - 1;
        bool rvalid = true;
        if (wrap) rr = rr < 0 ? rr + rows : (rr >= rows ? rr - rows : rr);
        else rvalid = rr >= 0 && rr < rows;
        if (seg_ok && row_ok) {
            int seg = sx * 32 + lane;
            if (lane == 0) {
                int cl = seg * 32 - 1;
                if (!rvalid) west = 0u;
                else if (cl < 0) west = wrap ? newest_bit(__ldg(cur + (size_t)rr * cols + cols - 1), delay) : 0u;
                else west = newest_bit(__ldg(cur + (size_t)rr * cols + cl), delay);
            }
            if (lane == strip_segs - 1) {
                int ce = seg * 32 + 32;
                if (!rvalid) east = 0u;
                else if (ce >= cols) east = wrap ? newest_bit(__ldg(cur + (size_t)rr * cols), delay) : 0u;
                else east = newest_bit(__ldg(cur + (size_t)rr * cols + ce), delay);
            }
        }
        N[k] = P;
        W[k] = (P << 1) | west;
        E[k] = (P >> 1) | (east << 31);
    }
    uint32_t c0 = 0, c1 = 0, c2 = 0, c3 = 0;
#pragma unroll
    for (int kr = 0; kr < 3; ++kr) {
        if (mask9 & (1u << (kr * 3 + 0))) csa_add(c0, c1, c2, c3, W[kr]);
        if (mask9 & (1u << (kr * 3 + 1))) csa_add(c0, c1, c2, c3, N[kr]);
        if (mask9 & (1u << (kr * 3 + 2))) csa_add(c0, c1, c2, c3, E[kr]);
    }
    uint32_t S = 0, B = 0;
    for (int v = 0; v < 10; ++v) {
        if (!(((smask | bmask) >> v) & 1u)) continue;
        uint32_t e = ~((c0 ^ ((v & 1) ? ~0u : 0u)) | (c1 ^ ((v & 2) ? ~0u : 0u)) |
                       (c2 ^ ((v & 4) ? ~0u : 0u)) | (c3 ^ ((v & 8) ? ~0u : 0u)));
        if ((smask >> v) & 1u) S |= e;
        if ((bmask >> v) & 1u) B |= e;
    }
    const uint32_t L = (O & S) | (~O & B);
    // Every warp has read its three tile rows; rows are now rewritten in place.
    __syncthreads();
    // new words of this warp's row, in place in the tile (row warp + 1)
    uint32_t* own = &tile[warp + 1][lane * kSegPad];
#pragma unroll
    for (int i = 0; i < 32; ++i) own[i] = (own[i] >> 1) | (((L >> i) & 1u) << 31);
    if (input_out) {
        cnt[0][warp][lane] = c0;
        cnt[1][warp][lane] = c1;
        cnt[2][warp][lane] = c2;
        cnt[3][warp][lane] = c3;
    }
    __syncthreads();
    for (int e = tid; e < kTileRows * 256; e += 256) {
        int tr = e >> 8, q = e & 255;
        int rr = r0 + tr;
        if (rr >= rows || 4 * q >= strip_words) continue;
        int word = 4 * q, sg = word >> 5, i = word & 31;
        const uint32_t* s = &tile[tr + 1][sg * kSegPad + i];
        reinterpret_cast<uint4*>(next + (size_t)rr * cols + sx * 1024)[q] = make_uint4(s[0], s[1], s[2], s[3]);
        if (input_out) {
            float f[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                int b = i + k;
                f[k] = (float)(((cnt[0][tr][sg] >> b) & 1u) | (((cnt[1][tr][sg] >> b) & 1u) << 1) |
                               (((cnt[2][tr][sg] >> b) & 1u) << 2) | (((cnt[3][tr][sg] >> b) & 1u) << 3));
            }
            reinterpret_cast<float4*>(input_out + (size_t)rr * cols + sx * 1024)[q] =
                make_float4(f[0], f[1], f[2], f[3]);
        }
    }
}

// ---------------------------------------------------------------------------
// game_of_life on bit planes (whole-run path).
//
// A cell's state is its 32-bit output-history word (bit 31 newest).  A step
// reads the newest bit of the neighbours and the cell's own bit 0, and shifts
// the word right by one with the new state in bit 31.  Stored as bit planes --
// plane p holds bit p of 32 consecutive cells of a row in one word -- a step
// only has to produce one new plane: a ring of kPlaneRing planes where, after
// T steps, bit p of every word is plane (T + p) % kPlaneRing.  The words are
// turned into planes at the start of a run and back (with the input register
// of the last step) at its end, so nothing outside the run sees the planes.
//
// k_gol_planes_steps advances K <= kPlaneK steps per launch with no trip to
// global memory in between: a CTA keeps the newest plane of its tile of
// kPlaneTY rows x kPlaneTX words plus a halo of kPlaneK rows and one word on
// each side, and the K oldest planes it needs; wrong values enter the halo
// from its outer edge at one cell per step and never reach the tile within K
// steps (a halo word is 32 cells wide).
constexpr int kPlaneRing = 64;          // a power of two
constexpr int kPlaneK = 16;
constexpr int kPlaneTY = 64;
constexpr int kPlaneTX = 8;
constexpr int kPlaneHY = kPlaneTY + 2 * kPlaneK;
constexpr int kPlaneHX = kPlaneTX + 2;
constexpr size_t kPlaneSmem = (size_t)(2 + kPlaneK) * kPlaneHY * kPlaneHX * sizeof(uint32_t);

// Words of one row segment (32 cells) -> the 32 plane words of the segment.
__global__ void k_gol_words_to_planes(int rows, int W, const uint32_t* __restrict__ words,
                                      uint32_t* __restrict__ planes) {
    const long long seg = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (seg >= (long long)rows * W) return;
    const uint32_t w = words[seg * 32 + lane];
    const size_t plane_words = (size_t)rows * W;
    uint32_t mine = 0;
#pragma unroll
    for (int p = 0; p < 32; ++p) {
        const uint32_t b = __ballot_sync(0xFFFFFFFFu, (w >> p) & 1u);
        if (lane == p) mine = b;
    }
    planes[(size_t)lane * plane_words + seg] = mine;      // after 0 steps bit p is plane p
}

// Planes after T steps -> words; and, if T > 0, the input register of the
// last step: the weighted count of the neighbours' newest bits one step
// earlier (plane T + 30).
__global__ void k_gol_planes_to_words(int rows, int W, long long T,
                                      const uint32_t* __restrict__ planes,
                                      uint32_t* __restrict__ words, float* __restrict__ input_out,
                                      unsigned mask9) {
    const long long seg = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (seg >= (long long)rows * W) return;
    const size_t plane_words = (size_t)rows * W;
    const uint32_t pw = planes[(size_t)((T + lane) % kPlaneRing) * plane_words + seg];
    uint32_t word = 0;
#pragma unroll
    for (int p = 0; p < 32; ++p) word |= ((__shfl_sync(0xFFFFFFFFu, pw, p) >> lane) & 1u) << p;
    words[seg * 32 + lane] = word;
    if (T == 0 || !input_out) return;
    const int r = (int)(seg / W), x = (int)(seg - (long long)r * W);
    const uint32_t* prev = planes + (size_t)((T + 30) % kPlaneRing) * plane_words;
    uint32_t c0 = 0, c1 = 0, c2 = 0, c3 = 0;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        int rr = r + k - 1;
        rr = rr < 0 ? rr + rows : (rr >= rows ? rr - rows : rr);
        const int xl = x == 0 ? W - 1 : x - 1, xr = x == W - 1 ? 0 : x + 1;
        const uint32_t n = prev[(size_t)rr * W + x];
        const uint32_t wv = (n << 1) | (prev[(size_t)rr * W + xl] >> 31);
        const uint32_t ev = (n >> 1) | (prev[(size_t)rr * W + xr] << 31);
        if (mask9 & (1u << (k * 3 + 0))) csa_add(c0, c1, c2, c3, wv);
        if (mask9 & (1u << (k * 3 + 1))) csa_add(c0, c1, c2, c3, n);
        if (mask9 & (1u << (k * 3 + 2))) csa_add(c0, c1, c2, c3, ev);
    }
    const unsigned cnt = ((c0 >> lane) & 1u) | (((c1 >> lane) & 1u) << 1) |
                         (((c2 >> lane) & 1u) << 2) | (((c3 >> lane) & 1u) << 3);
    input_out[seg * 32 + lane] = (float)cnt;
}

// Neighbour count of 32 cells (bit-sliced, bits c0..c3) from the three rows'
// west / centre / east words.  MODE 1: the 8 outer neighbours; MODE 2: all 9;
// MODE 0: any subset given by mask9 (bit kr*3+kc).
__device__ __forceinline__ uint32_t maj3(uint32_t a, uint32_t b, uint32_t c) {
    return (a & b) | (c & (a ^ b));
}

template <int MODE>
__device__ __forceinline__ void plane_count(const uint32_t (&w)[3], const uint32_t (&n)[3],
                                            const uint32_t (&e)[3], unsigned mask9, uint32_t& c0,
                                            uint32_t& c1, uint32_t& c2, uint32_t& c3) {
    if (MODE == 0) {
        c0 = c1 = c2 = c3 = 0;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            if (mask9 & (1u << (k * 3 + 0))) csa_add(c0, c1, c2, c3, w[k]);
            if (mask9 & (1u << (k * 3 + 1))) csa_add(c0, c1, c2, c3, n[k]);
            if (mask9 & (1u << (k * 3 + 2))) csa_add(c0, c1, c2, c3, e[k]);
        }
        return;
    }
    // each row as a 2-bit number (ones, twos), then the three rows added
    const uint32_t ts = w[0] ^ n[0] ^ e[0], tc = maj3(w[0], n[0], e[0]);
    const uint32_t bs = w[2] ^ n[2] ^ e[2], bc = maj3(w[2], n[2], e[2]);
    uint32_t ms, mc;
    if (MODE == 2) { ms = w[1] ^ n[1] ^ e[1]; mc = maj3(w[1], n[1], e[1]); }
    else { ms = w[1] ^ e[1]; mc = w[1] & e[1]; }
    c0 = ts ^ ms ^ bs;
    const uint32_t k1 = maj3(ts, ms, bs);                 // carry into the twos
    const uint32_t x = tc ^ mc ^ bc, y = maj3(tc, mc, bc);
    c1 = x ^ k1;
    const uint32_t k2 = x & k1;                            // carry into the fours
    c2 = y ^ k2;
    c3 = y & k2;
}

__device__ __forceinline__ void cp_async_u32(uint32_t* dst, const uint32_t* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(
                     (unsigned)__cvta_generic_to_shared(dst)),
                 "l"(src)
                 : "memory");
}

// K steps (1 <= K <= kPlaneK) of a toroidal board, starting after T0 steps.
// A thread owns one word column hx of the haloed tile and kPlaneRPT rows; per
// step it loads its rows' 3 x (kPlaneRPT + 2) neighbourhood once and computes
// only rows still needed by the remaining steps.  CONWAY: survival on 2 or 3
// neighbours, birth on 3 (the rule the schema defaults to), as four logic
// operations; otherwise any survival and birth count masks.
constexpr int kPlaneThreads = 512;
constexpr int kPlaneCols = kPlaneHX;
constexpr int kPlaneGroups = kPlaneThreads / kPlaneCols;
constexpr int kPlaneRPT = (kPlaneHY + kPlaneGroups - 1) / kPlaneGroups;

template <int MODE, bool CONWAY>
__global__ void __launch_bounds__(kPlaneThreads) k_gol_planes_steps(int rows, int W, int ty,
                                                          long long T0, int K,
                                                          uint32_t* __restrict__ planes,
                                                          unsigned mask9, unsigned smask,
                                                          unsigned bmask) {
    extern __shared__ uint32_t plane_smem[];
    // cur[2][HY][HX]: newest plane, double buffered; old[K][HY][HX]: the
    // planes that are bit 0 at steps T0 .. T0+K-1
    auto cur = reinterpret_cast<uint32_t(*)[kPlaneHY][kPlaneHX]>(plane_smem);
    auto old = reinterpret_cast<uint32_t(*)[kPlaneHY][kPlaneHX]>(plane_smem + 2 * kPlaneHY * kPlaneHX);
    const size_t plane_words = (size_t)rows * W;
    // tile of ty <= kPlaneTY rows; its haloed rows 0 .. hy_n - 1
    const int r0 = blockIdx.y * ty, w0 = blockIdx.x * kPlaneTX, hy_n = ty + 2 * kPlaneK;
    const int hy0 = kPlaneK - K;             // halo rows K steps do not need
    const int t0 = (int)(T0 & (kPlaneRing - 1));           // ring index of step T0
    const uint32_t* newest = planes + (size_t)((t0 + 31) & (kPlaneRing - 1)) * plane_words;
    // every word of the K + 1 planes in flight at once (cp.async), then one wait
    for (int e = threadIdx.x; e < hy_n * kPlaneHX; e += blockDim.x) {
        const int hy = e / kPlaneHX, hx = e - hy * kPlaneHX;
        int gr = (r0 - kPlaneK + hy) % rows, gw = (w0 - 1 + hx) % W;
        if (gr < 0) gr += rows;
        if (gw < 0) gw += W;
        const size_t off = (size_t)gr * W + gw;
        cp_async_u32(&cur[0][hy][hx], newest + off);
        for (int s = 0; s < K; ++s)
            cp_async_u32(&old[s][hy][hx],
                         planes + (size_t)((t0 + s) & (kPlaneRing - 1)) * plane_words + off);
    }
    asm volatile("cp.async.commit_group;\ncp.async.wait_all;\n" ::: "memory");
    __syncthreads();
    const int hx = threadIdx.x % kPlaneCols, rg = threadIdx.x / kPlaneCols;
    const bool active = rg < kPlaneGroups;
    const int ry0 = rg * kPlaneRPT;
    // this thread's column lies in the tile (its words go to global memory)
    const bool col_out = hx >= 1 && hx <= kPlaneTX && w0 + hx - 1 < W;
    const int ty_end = min(ty, rows - r0);
    int c = 0;
    for (int s = 0; s < K; ++s) {
        // rows valid after s steps: [hy0 + s, HY - 1 - hy0 - s]; needed next:
        const int lo = hy0 + s + 1, hi = hy_n - 2 - hy0 - s;
        if (active && ry0 + kPlaneRPT - 1 >= lo && ry0 <= hi) {
            uint32_t wl[kPlaneRPT + 2], wn[kPlaneRPT + 2], we[kPlaneRPT + 2];
#pragma unroll
            for (int q = 0; q < kPlaneRPT + 2; ++q) {
                const int hy = ry0 - 1 + q;
                const bool ok = hy >= 0 && hy < hy_n;
                const uint32_t n = ok ? cur[c][hy][hx] : 0u;
                const uint32_t l = ok && hx > 0 ? cur[c][hy][hx - 1] : 0u;
                const uint32_t r = ok && hx < kPlaneHX - 1 ? cur[c][hy][hx + 1] : 0u;
                wn[q] = n;
                wl[q] = __funnelshift_l(l, n, 1);          // (n << 1) | (l >> 31)
                we[q] = __funnelshift_r(n, r, 1);          // (n >> 1) | (r << 31)
            }
            uint32_t* out = planes + (size_t)((t0 + s + 32) & (kPlaneRing - 1)) * plane_words;
#pragma unroll
            for (int q = 0; q < kPlaneRPT; ++q) {
                const int hy = ry0 + q;
                if (hy < lo || hy > hi) continue;
                const uint32_t w3[3] = {wl[q], wl[q + 1], wl[q + 2]};
                const uint32_t n3[3] = {wn[q], wn[q + 1], wn[q + 2]};
                const uint32_t e3[3] = {we[q], we[q + 1], we[q + 2]};
                uint32_t c0, c1, c2, c3;
                plane_count<MODE>(w3, n3, e3, mask9, c0, c1, c2, c3);
                const uint32_t O = old[s][hy][hx];
                uint32_t L;
                if (CONWAY) {
                    // count 3 (0011): alive; count 2 (0010): alive if it was
                    L = c1 & ~c2 & ~c3 & (c0 | O);
                } else {
                    uint32_t S = 0, B = 0;
#pragma unroll
                    for (int v = 0; v < 10; ++v) {
                        if (!(((smask | bmask) >> v) & 1u)) continue;
                        const uint32_t eq = ~((c0 ^ ((v & 1) ? ~0u : 0u)) | (c1 ^ ((v & 2) ? ~0u : 0u)) |
                                              (c2 ^ ((v & 4) ? ~0u : 0u)) | (c3 ^ ((v & 8) ? ~0u : 0u)));
                        if ((smask >> v) & 1u) S |= eq;
                        if ((bmask >> v) & 1u) B |= eq;
                    }
                    L = (O & S) | (~O & B);
                }
                cur[c ^ 1][hy][hx] = L;
                const int ty = hy - kPlaneK;
                if (col_out && (unsigned)ty < (unsigned)ty_end)
                    out[(size_t)(r0 + ty) * W + w0 + hx - 1] = L;
            }
        }
        __syncthreads();
        c ^= 1;
    }
}

// ---------------------------------------------------------------------------
// game_of_life on bit planes, full-width strips: boards whose rows are 32, 64
// or 128 words (1024, 2048 or 4096 cells) wide, counting the 8 outer cells or
// all 9 cells of the 3x3 block.
//
// A CTA advances K steps (K <= 31) of a band of ty board rows plus K halo rows
// above and below, one band per SM.  Each warp holds R consecutive band rows
// across the whole width in registers -- lane l holds words l*WPL .. l*WPL +
// WPL - 1 of a row -- so the wrap across the width is a lane rotation, and the
// words west and east of a lane's run come from shuffles.  Per row a warp
// keeps the bit-sliced horizontal sums of each cell's three-cell row (ones s3,
// twos c3) and, for the 8-cell count, of the two cells beside it (s2, c2); a
// new row is the sum of the row above's and below's (s3, c3) with its own
// (s2, c2): six three-input logic operations per word with the B3/S23 rule,
// and six more for the new row's sums.  Warps hand their top and bottom rows'
// (s3, c3) to the warps above and below through shared memory, double
// buffered, with one barrier per step.  The plane holding the cells' oldest
// bits is copied (cp.async) into a shared-memory ring kStripDepth steps ahead.
// Rows outside the tile are recomputed halo: after step s only band rows
// within K - 1 - s of the tile must be right, and a warp whose rows all lie
// outside that range stops computing.  Consecutive launches are programmatic
// dependents, so that one is scheduled while the previous one drains.
// Band rows per warp: 2 for rows of 32 or 64 words (up to 32 warps, so that
// enough warps stay busy while the band shrinks), 4 for 128-word rows (up to
// 16 warps, registers permitting).
__host__ __device__ constexpr int strip_rows(int wpl) { return wpl >= 4 ? 4 : 2; }
__host__ __device__ constexpr int strip_max_warps(int rpw) { return rpw >= 4 ? 16 : 32; }
constexpr int kStripDepth = 4;       // steps ahead the oldest-bit plane is copied

template <int WPL>
__device__ __forceinline__ void strip_ld(const uint32_t* p, uint32_t (&v)[WPL]) {
    if constexpr (WPL == 4) {
        const uint4 t = __ldcg(reinterpret_cast<const uint4*>(p));
        v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
    } else if constexpr (WPL == 2) {
        const uint2 t = __ldcg(reinterpret_cast<const uint2*>(p));
        v[0] = t.x; v[1] = t.y;
    } else {
        v[0] = __ldcg(p);
    }
}

template <int WPL>
__device__ __forceinline__ void strip_cp_async(uint32_t* dst, const uint32_t* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(
                     (unsigned)__cvta_generic_to_shared(dst)),
                 "l"(src), "n"(4 * WPL)
                 : "memory");
}

template <int WPL>
__device__ __forceinline__ void strip_lds(const uint32_t* p, uint32_t (&v)[WPL]) {
    if constexpr (WPL == 4) {
        const uint4 t = *reinterpret_cast<const uint4*>(p);
        v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
    } else if constexpr (WPL == 2) {
        const uint2 t = *reinterpret_cast<const uint2*>(p);
        v[0] = t.x; v[1] = t.y;
    } else {
        v[0] = *p;
    }
}

template <int WPL>
__device__ __forceinline__ void strip_st(uint32_t* p, const uint32_t (&v)[WPL]) {
    if constexpr (WPL == 4) __stcg(reinterpret_cast<uint4*>(p), make_uint4(v[0], v[1], v[2], v[3]));
    else if constexpr (WPL == 2) __stcg(reinterpret_cast<uint2*>(p), make_uint2(v[0], v[1]));
    else __stcg(p, v[0]);
}

// One exchange slot of a lane: N = 2 * WPL words, s3 then c3.
template <int N>
__device__ __forceinline__ void xch_put(uint32_t* p, const uint32_t (&t)[N]) {
    if constexpr (N % 4 == 0) {
#pragma unroll
        for (int k = 0; k < N; k += 4)
            reinterpret_cast<uint4*>(p)[k / 4] = make_uint4(t[k], t[k + 1], t[k + 2], t[k + 3]);
    } else {
#pragma unroll
        for (int k = 0; k < N; k += 2) reinterpret_cast<uint2*>(p)[k / 2] = make_uint2(t[k], t[k + 1]);
    }
}

template <int N>
__device__ __forceinline__ void xch_get(const uint32_t* p, uint32_t (&t)[N]) {
    if constexpr (N % 4 == 0) {
#pragma unroll
        for (int k = 0; k < N; k += 4) {
            const uint4 u = reinterpret_cast<const uint4*>(p)[k / 4];
            t[k] = u.x; t[k + 1] = u.y; t[k + 2] = u.z; t[k + 3] = u.w;
        }
    } else {
#pragma unroll
        for (int k = 0; k < N; k += 2) {
            const uint2 u = reinterpret_cast<const uint2*>(p)[k / 2];
            t[k] = u.x; t[k + 1] = u.y;
        }
    }
}

template <int WPL>
struct StripRow {
    uint32_t s3[WPL], c3[WPL], s2[WPL], c2[WPL];
};

// Horizontal sums of one row held across the warp.
template <int MODE, int WPL>
__device__ __forceinline__ void strip_sums(const uint32_t (&v)[WPL], int lane, StripRow<WPL>& r) {
    const uint32_t wi = __shfl_sync(0xFFFFFFFFu, v[WPL - 1], (lane + 31) & 31);
    const uint32_t ei = __shfl_sync(0xFFFFFFFFu, v[0], (lane + 1) & 31);
#pragma unroll
    for (int j = 0; j < WPL; ++j) {
        const uint32_t west = j == 0 ? wi : v[j > 0 ? j - 1 : 0];
        const uint32_t east = j == WPL - 1 ? ei : v[j < WPL - 1 ? j + 1 : 0];
        const uint32_t a = __funnelshift_l(west, v[j], 1);   // west neighbours: (v << 1) | (west >> 31)
        const uint32_t b = __funnelshift_r(v[j], east, 1);   // east neighbours: (v >> 1) | (east << 31)
        r.s3[j] = a ^ v[j] ^ b;
        r.c3[j] = maj3(a, v[j], b);
        if (MODE == 1) {
            r.s2[j] = a ^ b;
            r.c2[j] = a & b;
        }
    }
}

template <int MODE, bool CONWAY, int WPL, int R>
__global__ void __launch_bounds__(strip_max_warps(R) * 32) k_gol_strips_steps(
    int rows, int ty, long long T0, int K, uint32_t* __restrict__ planes, unsigned smask,
    unsigned bmask) {
    constexpr int W = 32 * WPL, XN = 2 * WPL;
    extern __shared__ uint4 strip_smem[];
    // [2][warps + 2][2][32][XN]: warp w publishes in slot w + 1; slots 0 and
    // warps + 1 stay zero (nothing above the first warp or below the last)
    uint32_t* xch = reinterpret_cast<uint32_t*>(strip_smem);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    const size_t slots = (size_t)(nw + 2) * 2 * 32 * XN;       // words of one buffer
    // launched as a programmatic dependent of the previous advance: nothing
    // global is read before it has completed; the next advance may be
    // scheduled from here on
    asm volatile("griddepcontrol.wait;\n" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
#pragma unroll
    for (int e = 0; e < 2; ++e) {
        if (e == 0 ? warp != 0 : warp != nw - 1) continue;
        const int slot = e == 0 ? 0 : nw + 1;
#pragma unroll
        for (int b = 0; b < 2; ++b)
#pragma unroll
            for (int k = 0; k < 2 * XN; ++k)
                xch[b * slots + (size_t)slot * 2 * 32 * XN + (size_t)k * 32 + lane] = 0u;
    }
    const size_t plane_words = (size_t)rows * W;
    const int r0 = blockIdx.x * ty, tile_n = min(ty, rows - r0);
    const int hb0 = warp * R;                 // first band row of this warp; band row K is board row r0
    const int t0 = (int)(T0 & (kPlaneRing - 1));
    // word offsets of the warp's rows within a plane (a plane holds fewer
    // than 2^26 words), and which of them are tile rows
    uint32_t off[R];
    unsigned tile_rows = 0;
#pragma unroll
    for (int q = 0; q < R; ++q) {
        int g = (r0 - K + hb0 + q) % rows;
        if (g < 0) g += rows;
        off[q] = (uint32_t)g * W + (uint32_t)lane * WPL;
        if (hb0 + q >= K && hb0 + q < K + tile_n) tile_rows |= 1u << q;
    }
    StripRow<WPL> cur[R];
    {
        const uint32_t* newest = planes + (size_t)((t0 + 31) & (kPlaneRing - 1)) * plane_words;
        uint32_t v[R][WPL];
#pragma unroll
        for (int q = 0; q < R; ++q) strip_ld<WPL>(newest + off[q], v[q]);
#pragma unroll
        for (int q = 0; q < R; ++q) strip_sums<MODE, WPL>(v[q], lane, cur[q]);
    }
    // the cells' oldest bits: plane T0 + s at step s
    // The cells' oldest bits, plane T0 + s at step s, come through a ring of
    // kStripDepth slots in shared memory filled by cp.async kStripDepth steps
    // ahead: a lane copies and reads only its own words, and the copies stay
    // in flight across the per-step barriers.
    uint32_t* oring = xch + 2 * slots + (size_t)lane * WPL;       // [depth][warps * R][32][WPL]
    const size_t oslot = (size_t)nw * R * 32 * WPL;
    auto fetch_oldest = [&](int s) {
        if (s < K) {
            const uint32_t* p = planes + (size_t)((t0 + s) & (kPlaneRing - 1)) * plane_words;
            uint32_t* d = oring + (size_t)(s % kStripDepth) * oslot + (size_t)hb0 * 32 * WPL;
#pragma unroll
            for (int q = 0; q < R; ++q) strip_cp_async<WPL>(d + (size_t)q * 32 * WPL, p + off[q]);
        }
        asm volatile("cp.async.commit_group;\n" ::: "memory");
    };
#pragma unroll
    for (int d = 0; d < kStripDepth; ++d) fetch_oldest(d);
    // the warp's top and bottom rows' (s3, c3) for the step that reads
    // exchange buffer b; a warp publishes after every step it computed, and
    // a warp that stopped computing holds no row a later step still needs
    auto publish = [&](int b) {
        uint32_t* xp = xch + (size_t)b * slots + (size_t)32 * 2 * XN;
        uint32_t t[XN];
#pragma unroll
        for (int j = 0; j < WPL; ++j) { t[j] = cur[0].s3[j]; t[WPL + j] = cur[0].c3[j]; }
        xch_put<XN>(xp + ((size_t)(warp * 2 + 0) * 32 + lane) * XN, t);
#pragma unroll
        for (int j = 0; j < WPL; ++j) { t[j] = cur[R - 1].s3[j]; t[WPL + j] = cur[R - 1].c3[j]; }
        xch_put<XN>(xp + ((size_t)(warp * 2 + 1) * 32 + lane) * XN, t);
    };
    publish(0);
    // the last step that still needs one of this warp's rows: after step s
    // the band rows [s + 1, 2K + ty - 2 - s] must be right
    const int s_last = min(hb0 + R - 2, 2 * K + ty - 2 - hb0);
    auto step = [&](int s) {
        const uint32_t* xb = xch + (size_t)(s & 1) * slots;
        __syncthreads();
        if (s > s_last) return;
        // this step's copies (the group committed kStripDepth groups ago)
        asm volatile("cp.async.wait_group %0;\n" ::"n"(kStripDepth - 1) : "memory");
        uint32_t Od[R][WPL];
        {
            const uint32_t* o = oring + (size_t)(s % kStripDepth) * oslot + (size_t)hb0 * 32 * WPL;
#pragma unroll
            for (int q = 0; q < R; ++q) strip_lds<WPL>(o + (size_t)q * 32 * WPL, Od[q]);
        }
        uint32_t ab[XN], be[XN];              // sums of the row above the warp's first and below its last
        xch_get<XN>(xb + ((size_t)(warp * 2 + 1) * 32 + lane) * XN, ab);
        xch_get<XN>(xb + ((size_t)((warp + 2) * 2 + 0) * 32 + lane) * XN, be);
        uint32_t* out = planes + (size_t)((t0 + s + 32) & (kPlaneRing - 1)) * plane_words;
        uint32_t prev[WPL];
#pragma unroll
        for (int q = 0; q < R; ++q) {
            uint32_t nl[WPL];
#pragma unroll
            for (int j = 0; j < WPL; ++j) {
                const uint32_t as = q == 0 ? ab[j] : cur[q > 0 ? q - 1 : 0].s3[j];
                const uint32_t ac = q == 0 ? ab[WPL + j] : cur[q > 0 ? q - 1 : 0].c3[j];
                const uint32_t bs = q == R - 1 ? be[j] : cur[q < R - 1 ? q + 1 : 0].s3[j];
                const uint32_t bc = q == R - 1 ? be[WPL + j] : cur[q < R - 1 ? q + 1 : 0].c3[j];
                const uint32_t ms = MODE == 1 ? cur[q].s2[j] : cur[q].s3[j];
                const uint32_t mc = MODE == 1 ? cur[q].c2[j] : cur[q].c3[j];
                // count = c0 + 2 (k1 + x) + 4 y
                const uint32_t c0 = as ^ ms ^ bs, k1 = maj3(as, ms, bs);
                const uint32_t x = ac ^ mc ^ bc, y = maj3(ac, mc, bc);
                if (CONWAY) {
                    // count 2 or 3: exactly one of x, k1 and no y; 3 also needs c0
                    nl[j] = (x ^ k1) & ~y & (c0 | Od[q][j]);
                } else {
                    const uint32_t c1 = x ^ k1, k2 = x & k1, c2 = y ^ k2, c3 = y & k2;
                    uint32_t S = 0, B = 0;
#pragma unroll
                    for (int v = 0; v < 10; ++v) {
                        if (!(((smask | bmask) >> v) & 1u)) continue;
                        const uint32_t eq = ~((c0 ^ ((v & 1) ? ~0u : 0u)) | (c1 ^ ((v & 2) ? ~0u : 0u)) |
                                              (c2 ^ ((v & 4) ? ~0u : 0u)) | (c3 ^ ((v & 8) ? ~0u : 0u)));
                        if ((smask >> v) & 1u) S |= eq;
                        if ((bmask >> v) & 1u) B |= eq;
                    }
                    nl[j] = (Od[q][j] & S) | (~Od[q][j] & B);
                }
            }
            // the new row q - 1 is no longer read as an old row: store it and
            // take its sums
            if (q > 0) {
                if (tile_rows & (1u << (q - 1))) strip_st<WPL>(out + off[q - 1], prev);
                strip_sums<MODE, WPL>(prev, lane, cur[q - 1]);
            }
#pragma unroll
            for (int j = 0; j < WPL; ++j) prev[j] = nl[j];
        }
        {
            if (tile_rows & (1u << (R - 1))) strip_st<WPL>(out + off[R - 1], prev);
            strip_sums<MODE, WPL>(prev, lane, cur[R - 1]);
        }
        // buffer (s + 1) & 1 was last read before this step's barrier
        publish((s + 1) & 1);
        // the slot just read takes the plane kStripDepth steps ahead
        fetch_oldest(s + kStripDepth);
    };
    for (int s = 0; s < K; ++s) step(s);
    // no copy may land in shared memory after the block ends
    asm volatile("cp.async.wait_all;\n" ::: "memory");
}

static int num_sms() {
    int dev = 0, n = 0;
    SG_CUDA(cudaGetDevice(&dev));
    SG_CUDA(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev));
    return n;
}

// Mask of counts in [lo, hi] (counts of a 3x3 kernel are 0..9).
static unsigned count_mask(int lo, int hi) {
    unsigned m = 0;
    for (int v = 0; v < 10; ++v)
        if (v >= lo && v <= hi) m |= 1u << v;
    return m;
}

class RelayModel : public Model {
  public:
    const char* name() const override { return "relay"; }
    OutputType output_type() const override { return OUT_FLOAT; }
    void build_layer(State&, LayerState& ls) const override {
        ls.params["ramp"] = ls.layer->parameter("ramp", "false") == "true" ? 1.0f : 0.0f;
    }
    void update(State&, LayerState& ls, const StepCtx& ctx) const override {
        const Layer& l = *ls.layer;
        k_relay<<<blocks_for(l.size, 256), 256, 0, ctx.stream>>>(
            l.size, l.history(), ls.input->df(), ls.output->df(), (int)ls.params.at("ramp"));
        SG_LAUNCH_CHECK();
        ctx.count();
    }
};
SG_REGISTER_MODEL(RelayModel);

class RateEncodingModel : public Model {
  public:
    const char* name() const override { return "rate_encoding"; }
    OutputType output_type() const override { return OUT_FLOAT; }
    void update(State&, LayerState& ls, const StepCtx& ctx) const override {
        const Layer& l = *ls.layer;
        k_rate<<<blocks_for(l.size, 256), 256, 0, ctx.stream>>>(l.size, l.history(), ls.input->df(),
                                                                ls.output->df());
        SG_LAUNCH_CHECK();
        ctx.count();
    }
};
SG_REGISTER_MODEL(RateEncodingModel);

class GameOfLifeModel : public Model {
  public:
    const char* name() const override { return "game_of_life"; }
    OutputType output_type() const override { return OUT_BIT; }
    // The fused step applies to a layer without dendritic nodes whose only
    // input is its own convergent "add" connection reading word 0, with no
    // init config, no environment input and a one-word history.
    static bool fusable_shape(const Layer& l) {
        if (l.inputs.size() != 1 || l.has_dendrites()) return false;
        const Connection* c = l.inputs[0];
        return c->from == &l && c->type == CONVERGENT && c->opcode == OP_ADD && c->delay < 32 &&
               l.history() == 1 && !l.config.child("init config");
    }
    void build_layer(State& st, LayerState& ls) const override {
        const Layer& l = *ls.layer;
        ls.params["smin"] = (float)std::stoi(l.parameter("survival_min", "2"));
        ls.params["smax"] = (float)std::stoi(l.parameter("survival_max", "3"));
        ls.params["bmin"] = (float)std::stoi(l.parameter("birth_min", "3"));
        ls.params["bmax"] = (float)std::stoi(l.parameter("birth_max", "3"));
        if (fusable_shape(l)) {
            Array* swap = st.add_array("output swap", 'u', l.size);
            swap->scratch = true;
            ls.internal["output swap"] = swap;
            const Connection& c = *l.inputs[0];
            if (c.delay == 0 && c.arbor.wrap && l.cols % 32 == 0) {
                Array* planes = st.add_array("planes", 'u', (size_t)kPlaneRing * (l.size / 32));
                planes->scratch = true;
                ls.internal["planes"] = planes;
            }
        }
    }
    // Steps of the full-width strip kernel per launch (at most 31: a step
    // reads the plane written 32 steps earlier, which must come from an
    // earlier launch).
    static int strip_steps_per_launch() {
        static const int k = [] {
            const char* e = std::getenv("SG_GOL_STEPS_PER_LAUNCH");
            const int v = e ? std::atoi(e) : 12;
            return v < 1 ? 1 : (v > 31 ? 31 : v);
        }();
        return k;
    }
    // exchange buffers: 2 x (warps + 2) slots of 2 rows x 32 lanes x 2 * wpl
    // words; ring of the oldest-bit planes: kStripDepth x warps x rpw rows x
    // 32 lanes x wpl words
    static size_t strip_smem_bytes(int warps, int rpw, int wpl) {
        return ((size_t)(warps + 2) * 256 + (size_t)kStripDepth * warps * rpw * 32) * wpl * 4;
    }
    static long advance_strips(int rows, int W, int mode, bool conway, long n, uint32_t* planes,
                               unsigned smask, unsigned bmask, cudaStream_t s) {
        using Kernel = void (*)(int, int, long long, int, uint32_t*, unsigned, unsigned);
        const int wpl = W / 32;
        const int rpw = strip_rows(wpl), max_warps = strip_max_warps(rpw);
        const int wi = wpl == 1 ? 0 : (wpl == 2 ? 1 : 2);
#define SG_STRIPS(M, C)                                                                  \
    {k_gol_strips_steps<M, C, 1, strip_rows(1)>, k_gol_strips_steps<M, C, 2, strip_rows(2)>, \
     k_gol_strips_steps<M, C, 4, strip_rows(4)>}
        static const Kernel kernels[2][2][3] = {{SG_STRIPS(1, false), SG_STRIPS(1, true)},
                                                {SG_STRIPS(2, false), SG_STRIPS(2, true)}};
#undef SG_STRIPS
        const Kernel kernel = kernels[mode - 1][conway ? 1 : 0][wi];
        const size_t max_smem = strip_smem_bytes(max_warps, rpw, wpl);
        static bool configured[2][2][3] = {};
        bool& cfg = configured[mode - 1][conway ? 1 : 0][wi];
        if (!cfg) {
            SG_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)max_smem));
            cfg = true;
        }
        const int sms = num_sms();
        long launches = 0;
        long long T = 0;
        while (T < n) {
            const int K = (int)std::min<long long>(strip_steps_per_launch(), n - T);
            // one band of ty rows per SM, within max_warps warps of rpw rows
            // holding the band and its 2K halo rows
            int ty = (rows + sms - 1) / sms;
            ty = std::min(ty, max_warps * rpw - 2 * K);
            const int nw = (ty + 2 * K + rpw - 1) / rpw;
            const int grid = (rows + ty - 1) / ty;
            const size_t smem = strip_smem_bytes(nw, rpw, wpl);
            // programmatic dependent launch: each launch may be scheduled
            // while the previous one drains; it waits for it to complete
            // (griddepcontrol.wait) before touching the planes
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3((unsigned)grid);
            cfg.blockDim = dim3((unsigned)(nw * 32));
            cfg.dynamicSmemBytes = smem;
            cfg.stream = s;
            cudaLaunchAttribute attr[1];
            attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
            attr[0].val.programmaticStreamSerializationAllowed = 1;
            cfg.attrs = attr;
            cfg.numAttrs = 1;
            SG_CUDA(cudaLaunchKernelEx(&cfg, kernel, rows, ty, (long long)T, K, planes, smask, bmask));
            ++launches;
            T += K;
        }
        return launches;
    }
    // Whole-run path on bit planes: a toroidal board whose only input is its
    // own 0/1-weight 3x3 connection with delay 0.
    bool can_advance_alone(State& st, const LayerState& ls) const override {
        const Layer& l = *ls.layer;
        if (!fusable_shape(l) || !ls.internal.count("planes")) return false;
        const ConnState& cs = *st.conn_state(l.inputs[0]);
        auto bm = cs.params.find("bits mask");
        return bm != cs.params.end() && bm->second >= 0.0f;
    }
    long advance_alone(State& st, LayerState& ls, long n, cudaStream_t s) const override {
        const Layer& l = *ls.layer;
        const ConnState& cs = *st.conn_state(l.inputs[0]);
        const unsigned mask9 = (unsigned)cs.params.at("bits mask");
        const unsigned smask = count_mask((int)ls.params.at("smin"), (int)ls.params.at("smax"));
        const unsigned bmask = count_mask((int)ls.params.at("bmin"), (int)ls.params.at("bmax"));
        const int W = l.cols / 32;
        uint32_t* planes = ls.internal.at("planes")->du();
        uint32_t* words = ls.output->du();
        const long long segs = (long long)l.rows * W;
        long launches = 0;
        k_gol_words_to_planes<<<blocks_for(segs * 32, 256), 256, 0, s>>>(l.rows, W, words, planes);
        SG_LAUNCH_CHECK();
        ++launches;
        // counting kernel: the 8 outer neighbours, all 9, or any other 0/1
        // mask; the B3/S23 rule as its own instance
        const int mode = (mask9 & 0x1EFu) == 0x1EFu ? ((mask9 & 0x10u) ? 2 : 1) : 0;
        const bool conway = smask == count_mask(2, 3) && bmask == count_mask(3, 3);
        if (mode != 0 && (W == 32 || W == 64 || W == 128)) {
            launches += advance_strips(l.rows, W, mode, conway, n, planes, smask, bmask, s);
            k_gol_planes_to_words<<<blocks_for(segs * 32, 256), 256, 0, s>>>(
                l.rows, W, n, planes, words, ls.input->df(), mask9);
            SG_LAUNCH_CHECK();
            return launches + 1;
        }
        using Kernel = void (*)(int, int, int, long long, int, uint32_t*, unsigned, unsigned,
                                unsigned);
        static const Kernel kernels[6] = {k_gol_planes_steps<0, false>, k_gol_planes_steps<1, false>,
                                          k_gol_planes_steps<2, false>, k_gol_planes_steps<0, true>,
                                          k_gol_planes_steps<1, true>,  k_gol_planes_steps<2, true>};
        const int which = mode + (conway ? 3 : 0);
        const Kernel kernel = kernels[which];
        static bool configured[6] = {false, false, false, false, false, false};
        if (!configured[which]) {
            SG_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)kPlaneSmem));
            configured[which] = true;
        }
        // tile height: fewest haloed rows on the busiest SM (CTAs spread
        // evenly over the SMs, all resident)
        const int gx = (W + kPlaneTX - 1) / kPlaneTX;
        const int sms = num_sms();
        int ty = kPlaneTY;
        long long best = -1;
        for (int t = kPlaneTY; t >= 16; --t) {
            const long long ctas = (long long)gx * ((l.rows + t - 1) / t);
            const long long cost = (ctas + sms - 1) / sms * (t + 2 * kPlaneK);
            if (best < 0 || cost < best) { best = cost; ty = t; }
        }
        const dim3 grid((unsigned)gx, (unsigned)((l.rows + ty - 1) / ty));
        long long T = 0;
        while (T < n) {
            const int K = (int)std::min<long long>(kPlaneK, n - T);
            kernel<<<grid, kPlaneThreads, kPlaneSmem, s>>>(l.rows, W, ty, T, K, planes, mask9,
                                                           smask, bmask);
            SG_LAUNCH_CHECK();
            ++launches;
            T += K;
        }
        k_gol_planes_to_words<<<blocks_for(segs * 32, 256), 256, 0, s>>>(
            l.rows, W, T, planes, words, ls.input->df(), mask9);
        SG_LAUNCH_CHECK();
        return launches + 1;
    }
    bool fuses_input(State&, const Connection& c, const StepCtx& ctx) const override {
        return fusable_shape(*c.to) && !ctx.is_input(*c.to);
    }
    // After every upload: can the bit-sliced kernel run this layer?  (3x3
    // convolutional kernel of 0/1 weights, stride and spacing 1, offset -1,
    // whole 32-cell row segments.)
    void prepare_device(State& st, ConnState& cs, cudaStream_t) const override {
        const Connection& c = *cs.conn;
        cs.params["bits mask"] = -1.0f;
        if (!fusable_shape(*c.to) || !c.convolutional) return;
        const Arbor& a = c.arbor;
        if (a.row_field != 3 || a.col_field != 3 || a.row_stride != 1 || a.col_stride != 1 ||
            a.row_spacing != 1 || a.col_spacing != 1 || a.row_offset != -1 || a.col_offset != -1 ||
            c.to->cols % 32 != 0)
            return;
        const float* w = cs.weights->hf();
        unsigned mask = 0;
        for (int k = 0; k < 9; ++k) {
            if (w[k] == 1.0f) mask |= 1u << k;
            else if (!(w[k] == 0.0f && !std::signbit(w[k]))) return;
        }
        cs.params["bits mask"] = (float)mask;
    }
    void update(State& st, LayerState& ls, const StepCtx& ctx) const override {
        const Layer& l = *ls.layer;
        int smin = (int)ls.params.at("smin"), smax = (int)ls.params.at("smax");
        int bmin = (int)ls.params.at("bmin"), bmax = (int)ls.params.at("bmax");
        if (fusable_shape(l) && !ctx.is_input(l)) {
            ConnState& cs = *st.conn_state(l.inputs[0]);
            Array* swap = ls.internal.at("output swap");
            auto bm = cs.params.find("bits mask");
            if (bm != cs.params.end() && bm->second >= 0.0f) {
                int strips = (l.cols / 32 + 31) / 32;
                dim3 grid(strips, blocks_for(l.rows, kTileRows));
                k_gol_bits_tile<<<grid, 256, 0, ctx.stream>>>(
                    l.rows, l.cols, cs.conn->arbor.wrap ? 1 : 0, cs.conn->delay,
                    (unsigned)bm->second, ls.output->du(), swap->du(),
                    ctx.last_step ? ls.input->df() : nullptr, count_mask(smin, smax),
                    count_mask(bmin, bmax));
                SG_LAUNCH_CHECK();
                std::swap(ls.output->dev, swap->dev);
                ctx.count();
                return;
            }
            dim3 block(32, 8);
            dim3 grid(blocks_for(l.cols, 32), blocks_for(l.rows, 8));
            k_gol_fused<<<grid, block, 0, ctx.stream>>>(
                cs.geom, cs.conn->delay, ls.output->du(), swap->du(), cs.weights->df(),
                ctx.last_step ? ls.input->df() : nullptr, smin, smax, bmin, bmax);
            SG_LAUNCH_CHECK();
            std::swap(ls.output->dev, swap->dev);
            ctx.count();
            return;
        }
        k_gol<<<blocks_for(l.size, 256), 256, 0, ctx.stream>>>(l.size, l.history(), ls.input->df(),
                                                               ls.output->du(), smin, smax, bmin, bmax);
        SG_LAUNCH_CHECK();
        ctx.count();
    }
};
SG_REGISTER_MODEL(GameOfLifeModel);

}  // namespace sg
