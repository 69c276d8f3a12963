// Differentiable leaky-integrator rate network: forward cycle and its
// hand-written adjoint (backpropagation through time with checkpoints).
//
// The reference has no differentiable model; its rate_encoding layer
// (src/core/state/impl/rate_encoding_attributes.cpp:14-34) maps input to a
// rate with no memory.  This model gives each neuron a leaky membrane:
//
//   layers l = 0..L-1 of rows x cols neurons (N), batch element b
//   I_0[t]  = x[t]                                     (input sequence)
//   I_l[t]  = sum_k W_l[i][k] * r_{l-1}[t-1][src(i,k)]  (l >= 1, convergent)
//   d_l[t]  = -v_l[t-1] + I_l[t]
//   v_l[t]  = v_l[t-1] + a_l * d_l[t],   a_l = dt / tau_l
//   r_l[t]  = sigmoid(v_l[t]),           v_l[0] = 0
//   y[t]    = R r_{L-1}[t]                             (readout, O outputs)
//   loss    = sum_{t,b,o} (y[t][b][o] - target[b][o])^2 / (T B O)
//
// Convergent connections follow the reference's arborized geometry
// (src/core/engine/kernel/synapse_kernel.h:384-421) with stride 1, spacing 1,
// offset -field/2 and no wrap: out-of-range sources are skipped; weights are
// in the CPU layout [destination][k], k = kernel row * field + kernel column.
// Synchronous update as in the reference's cycle: every layer at t reads the
// rates of t-1.
//
// Adjoint (lambda_l[t] = dloss/dv_l[t]):
//   g_{L-1}[t] = R^T gy[t],  gy[t] = grad_loss * 2 (y[t] - target) / (T B O)
//   g_l[t]     = sum over (j, k) with src(j,k) = i of W_{l+1}[j][k] a_{l+1} lambda_{l+1}[t+1][j]
//   lambda_l[t] = r (1 - r) g_l[t] + (1 - a_l) lambda_l[t+1],  lambda[T+1] = 0
//   dW_l[j][k] = a_l sum_{t,b} lambda_l[t][j] r_{l-1}[t-1][src(j,k)]
//   dR[o][i]   = sum_{t,b} gy[t][o] r_{L-1}[t][i]
//   dtau_l     = -(dt / tau_l^2) sum_{t,b,i} lambda_l[t][i] d_l[t][i]
//   dx[t]      = a_0 lambda_0[t]
// The forward pass stores v every `checkpoint` steps; the backward pass
// recomputes each segment's states from its checkpoint (bit-identical: the
// same kernel on the same inputs), then runs the adjoint back through it.
// Every sum has a fixed order, and every gradient accumulator takes one
// timestep's sum at a time, so results are deterministic and do not depend on
// the checkpoint stride.
//
// Layout on the device: the convergent weights are transposed once per call
// into the workspace as [layer][k][neuron], so that consecutive threads
// (consecutive neurons) read consecutive weights; the readout is reduced per
// 256-neuron block inside the step kernel and finished at the end.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "../../include/syngen.h"
#include "cuda_check.h"

namespace sg {
void set_last_error(const char* what);
}

namespace {
using namespace sg;

constexpr int kMaxOutputs = 16;
constexpr int kMaxField = 9;
constexpr int kTauBlocks = 64;
constexpr int kBlock = 256;

struct Dims {
    int L, rows, cols, N, field, h, K, O, B, T, k, nseg, nchunk, bg;
    float dt;
    long long S;   // L * B * N
};

// The rate network is checked against an FP64 restatement (not a bit-exact
// reference), so it uses the fast exponential and a correctly rounded
// reciprocal (relative error a few units in the last place), and explicit
// fused multiply-adds in its sums; every kernel is deterministic, so the
// backward pass recomputes the forward states bit for bit.
__device__ __forceinline__ float sigmoid(float v) { return __frcp_rn(1.0f + __expf(-v)); }

// wt[l][k][i] = w[l][i][k]
__global__ void k_rate_transpose(Dims D, const float* __restrict__ w, float* __restrict__ wt) {
    long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)(D.L - 1) * D.N * D.K) return;
    const long long per = (long long)D.N * D.K;
    const int l = (int)(idx / per);
    const int rem = (int)(idx - l * per);
    const int k = rem / D.N, i = rem - k * D.N;
    wt[idx] = w[l * per + (long long)i * D.K + k];
}

// One forward timestep: grid (tiles of 16 x 16 neurons, layers, groups of
// D.bg batch elements).  A thread keeps its neuron's field x field weights
// (and, in the last layer, its readout weights) in registers; per batch
// element the CTA stages the source rates of its tile plus the kernel's halo
// (zero outside the layer: a skipped source adds w * 0) in shared memory,
// double-buffered, with the next element's halo fetched into registers while
// the current one is summed.  Tiles of the last layer reduce their readout
// contributions (fixed tree) into ypart[b][tile][o].
constexpr int kTileSide = 16;
constexpr int kMaxBatchGroup = 8;

// Source window of a tile: element e of the (16 + 2h)^2 halo, zero outside.
// A thread copies elements threadIdx.x + q * kBlock; their plane offsets
// (-1 outside the layer) and shared-memory slots (-1 past the window) are the
// same for every batch element and are worked out once.
template <int F>
struct Halo {
    static constexpr int H = F / 2, SIDE = kTileSide + 2 * H, COUNT = SIDE * SIDE;
    static constexpr int PER = (COUNT + kBlock - 1) / kBlock;
    // row pitch = 16 (mod 32): the two tile rows a warp reads hit disjoint banks
    static constexpr int PITCH = SIDE <= 16 ? 16 : 48;
    int off[PER], slot[PER];
    __device__ Halo(const Dims& D, int ty0, int tx0) {
#pragma unroll
        for (int q = 0; q < PER; ++q) {
            const int e = threadIdx.x + q * kBlock;
            const int sy = e / SIDE, sx = e - sy * SIDE;
            const int r = ty0 - H + sy, c = tx0 - H + sx;
            slot[q] = e < COUNT ? sy * PITCH + sx : -1;
            off[q] = (r >= 0 && r < D.rows && c >= 0 && c < D.cols) ? r * D.cols + c : -1;
        }
    }
    __device__ void fetch(const float* plane, float scale, float (&reg)[PER]) const {
#pragma unroll
        for (int q = 0; q < PER; ++q)
            reg[q] = (slot[q] >= 0 && off[q] >= 0) ? scale * plane[off[q]] : 0.0f;
    }
    __device__ void stage(const float (&reg)[PER], float* dst) const {
#pragma unroll
        for (int q = 0; q < PER; ++q)
            if (slot[q] >= 0) dst[slot[q]] = reg[q];
    }
};

template <int F>
__global__ void __launch_bounds__(kBlock) k_rate_step(
    Dims D, const float* __restrict__ x_t, const float* wt, const float* wo,
    const float* __restrict__ tau, const float* __restrict__ v_prev,
    const float* __restrict__ r_prev, float* __restrict__ v_new, float* __restrict__ r_new,
    float* __restrict__ d_out, float* __restrict__ ypart) {
    using W = Halo<F>;
    __shared__ float src[2][W::SIDE][W::PITCH];
    __shared__ float red[kBlock / 32][kMaxOutputs];
    const int tiles_x = (D.cols + kTileSide - 1) / kTileSide;
    const int tile = blockIdx.x, l = blockIdx.y;
    const int ty0 = (tile / tiles_x) * kTileSide, tx0 = (tile % tiles_x) * kTileSide;
    const int tr = threadIdx.x / kTileSide, tc = threadIdx.x % kTileSide;
    const int ir = ty0 + tr, ic = tx0 + tc;
    const bool ok = ir < D.rows && ic < D.cols;
    const int i = ir * D.cols + ic;
    const bool readout = ypart && l == D.L - 1;
    const float a = D.dt / __ldg(tau + l);
    // plain loads: kept in registers across the batch loop's barriers
    float wk[F * F];
#pragma unroll
    for (int k = 0; k < F * F; ++k)
        wk[k] = (l >= 1 && ok) ? wt[((long long)(l - 1) * F * F + k) * D.N + i] : 0.0f;
    float wov[kMaxOutputs];
#pragma unroll
    for (int o = 0; o < kMaxOutputs; ++o)
        wov[o] = (readout && ok && o < D.O) ? wo[(long long)o * D.N + i] : 0.0f;
    const int b0 = blockIdx.z * D.bg, b1 = min(D.B, b0 + D.bg);
    const float* rp = l >= 1 ? r_prev + (long long)(l - 1) * D.B * D.N : nullptr;
    const W halo(D, ty0, tx0);
    float pre[W::PER];
    if (l >= 1) halo.fetch(rp + (long long)b0 * D.N, 1.0f, pre);
    for (int b = b0, buf = 0; b < b1; ++b, buf ^= 1) {
        if (l >= 1) halo.stage(pre, &src[buf][0][0]);
        const long long idx = ((long long)l * D.B + b) * D.N + i;
        const float vp = ok ? v_prev[idx] : 0.0f;
        float I = (ok && l == 0) ? __ldg(x_t + (long long)b * D.N + i) : 0.0f;
        __syncthreads();
        if (l >= 1 && b + 1 < b1) halo.fetch(rp + (long long)(b + 1) * D.N, 1.0f, pre);
        float rn = 0.0f;
        if (ok) {
            if (l >= 1) {
                // one partial sum per kernel row (independent chains), rows
                // added in order
                float part[F];
#pragma unroll
                for (int kr = 0; kr < F; ++kr) {
                    part[kr] = 0.0f;
#pragma unroll
                    for (int kc = 0; kc < F; ++kc)
                        part[kr] = __fmaf_rn(wk[kr * F + kc], src[buf][tr + kr][tc + kc], part[kr]);
                }
#pragma unroll
                for (int kr = 0; kr < F; ++kr) I += part[kr];
            }
            const float d = -vp + I;
            const float vn = vp + a * d;
            v_new[idx] = vn;
            rn = sigmoid(vn);
            r_new[idx] = rn;
            if (d_out) d_out[idx] = d;
        }
        if (readout) {
            // butterfly transpose reduction: after the exchanges with lanes
            // 16, 8, 4, 2 apart a lane holds one output's partial sum of 32
            // lanes' contributions -- output lane >> 1 -- and the exchange
            // with the neighbour completes it (16 shuffles for 16 outputs)
            const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
            float c[kMaxOutputs];
#pragma unroll
            for (int o = 0; o < kMaxOutputs; ++o) c[o] = wov[o] * rn;
#pragma unroll
            for (int half = kMaxOutputs / 2; half >= 1; half /= 2) {
                const bool up = lane & (2 * half);
#pragma unroll
                for (int j = 0; j < half; ++j) {
                    const float send = up ? c[j] : c[j + half];
                    const float keep = up ? c[j + half] : c[j];
                    c[j] = keep + __shfl_xor_sync(0xFFFFFFFFu, send, 2 * half);
                }
            }
            const float y_lane = c[0] + __shfl_xor_sync(0xFFFFFFFFu, c[0], 1);
            if ((lane & 1) == 0 && (lane >> 1) < D.O) red[warp][lane >> 1] = y_lane;
            __syncthreads();
            if (threadIdx.x < D.O) {
                float y = 0.0f;
                for (int w = 0; w < kBlock / 32; ++w) y += red[w][threadIdx.x];
                ypart[((long long)b * D.nchunk + tile) * D.O + threadIdx.x] = y;
            }
        }
    }
}

// Many timesteps of one batch element on one 16 x 16 tile in one launch.
// A layer's own state is pointwise in time and layer l at step t reads layer
// l-1 at step t-1 within +-h, so the tile of the last layer for any number
// of steps needs layer l over the tile plus (L-1-l) h on each side and
// nothing else: the CTA keeps v and r of those regions (and the stencil
// weights of layers >= 1 over them) in shared memory and advances them step
// by step with no global exchange.  Halo neurons are computed exactly as
// their owners compute them (same inputs, same operations), so each CTA's
// tile neurons equal those of any other split -- and the backward pass's
// recompute from a checkpoint reproduces the forward states bit for bit.
//   mode 0 (forward): steps 1..T from v = 0; writes the checkpoints
//     (t % k == 0, t < T) and the per-tile readout partials ypart.
//   mode 1 (recompute): nt steps from the checkpointed v at step c; writes
//     the segment's r (steps c..c+nt) and drives d, which is all the adjoint
//     kernels read.
// The input of the next step is fetched with cp.async during the current one.
struct FusedRegions {
    int L, H;
    __device__ __host__ int side(int l) const { return kTileSide + 2 * (L - 1 - l) * H; }
    __device__ __host__ int off(int l) const {      // float offset of region l
        int o = 0;
        for (int m = 0; m < l; ++m) o += side(m) * side(m);
        return o;
    }
    __device__ __host__ int total() const { return off(L); }
    __device__ __host__ int woff(int l, int K) const {   // weights of layers 1..l-1
        int o = 0;
        for (int m = 1; m < l; ++m) o += K * side(m) * side(m);
        return o;
    }
};

template <int F>
__host__ __device__ inline size_t fused_smem_floats(int L) {
    const FusedRegions R{L, F / 2};
    const int s0 = R.side(0);
    // v, r (two buffers), input (two buffers), weights, readout weights of
    // the tile, readout partials, a_l, and two per-position tables (32-bit ints)
    return (size_t)3 * R.total() + 2 * s0 * s0 + R.woff(L, F * F) +
           kMaxOutputs * kBlock + 2 * (kBlock / 32) * kMaxOutputs + L + 2 * R.total();
}

__device__ __forceinline__ void cp_async_f32_zfill(float* dst, const float* src, bool valid) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(
                     (unsigned)__cvta_generic_to_shared(dst)),
                 "l"(src), "r"(valid ? 4 : 0)
                 : "memory");
}

constexpr int kOwnBit = 1 << 30;

template <int F>
__global__ void __launch_bounds__(kBlock) k_rate_fused(
    Dims D, int mode, int c, int nt, const float* __restrict__ x, const float* __restrict__ wt,
    const float* __restrict__ wo, const float* __restrict__ tau, const float* __restrict__ v0,
    float* __restrict__ ckpt, float* __restrict__ ypart, float* __restrict__ seg_r,
    float* __restrict__ seg_d) {
    constexpr int H = F / 2, K = F * F;
    extern __shared__ float fs[];
    const FusedRegions R{D.L, H};
    const int tot = R.total(), s0 = R.side(0);
    // weights first, then v, r[2], x[2], readout weights,
    // readout partials, a_l, tables
    float* ws = fs;                                          // [k][position], layers >= 1
    float* vs = ws + R.woff(D.L, K);
    float* rs = vs + tot;
    float* xs = vs + 3 * tot;
    float* ows = xs + 2 * s0 * s0;                           // [O][256] readout weights
    float* red = ows + kMaxOutputs * kBlock;                 // [2][8][16]
    float* as = red + 2 * (kBlock / 32) * kMaxOutputs;       // dt / tau_l
    // per region position: its global index, with kOwnBit for tile neurons,
    // or -1 outside the layer; and the offset of its stencil window in the
    // previous layer's region
    int* info = reinterpret_cast<int*>(as + D.L);
    int* sbase = info + tot;
    const int tiles_x = (D.cols + kTileSide - 1) / kTileSide;
    const int tile = blockIdx.x, b = blockIdx.y;
    const int ty0 = (tile / tiles_x) * kTileSide, tx0 = (tile % tiles_x) * kTileSide;
    const int tid = threadIdx.x;
    const long long S = D.S;

    // tables, initial state, weights
    for (int l = 0, o = 0, op = 0, sp = 0, wofs = 0; l < D.L; ++l) {
        const int sd = R.side(l), q = (D.L - 1 - l) * H;
        for (int p = tid; p < sd * sd; p += kBlock) {
            const int py = p / sd, px = p - py * sd;
            const int gy = ty0 - q + py, gx = tx0 - q + px;
            const bool in = gy >= 0 && gy < D.rows && gx >= 0 && gx < D.cols;
            const int gi = in ? gy * D.cols + gx : -1;
            const bool own = py >= q && py < q + kTileSide && px >= q && px < q + kTileSide;
            info[o + p] = in ? (gi | (own ? kOwnBit : 0)) : -1;
            sbase[o + p] = l >= 1 ? op + py * sp + px : 0;
            const long long gl = ((long long)l * D.B + b) * D.N + gi;
            const float v = (in && v0) ? v0[gl] : 0.0f;
            const float r = in ? sigmoid(v) : 0.0f;
            vs[o + p] = v;
            rs[o + p] = r;
            rs[tot + o + p] = 0.0f;
            if (mode == 1 && in && own) seg_r[gl] = r;
            if (l >= 1) {
#pragma unroll
                for (int k = 0; k < K; ++k)
                    ws[wofs + k * sd * sd + p] =
                        in ? __ldg(wt + ((long long)(l - 1) * K + k) * D.N + gi) : 0.0f;
            }
            if (l == D.L - 1) {                               // the tile itself: p = tid
                for (int k = 0; k < kMaxOutputs; ++k)
                    ows[k * kBlock + p] = (in && k < D.O) ? __ldg(wo + (long long)k * D.N + gi) : 0.0f;
            }
        }
        op = o;
        sp = sd;
        o += sd * sd;
        if (l >= 1) wofs += K * sd * sd;
    }
    for (int l = tid; l < D.L; l += kBlock) as[l] = D.dt / __ldg(tau + l);
    __syncthreads();
    {
        const float* xt = x + ((long long)c * D.B + b) * D.N;
        for (int p = tid; p < s0 * s0; p += kBlock) {
            const int code = info[p];
            cp_async_f32_zfill(&xs[p], code >= 0 ? xt + (code & (kOwnBit - 1)) : xt, code >= 0);
        }
        asm volatile("cp.async.commit_group;\ncp.async.wait_all;\n" ::: "memory");
    }
    __syncthreads();

    // The last layer's region is the tile itself: thread tid owns position
    // tid, whose weights (small fields) it keeps in registers.
    constexpr bool kRegLast = F <= 5;
    float wlast[kRegLast ? K : 1];
    if (kRegLast && D.L >= 2) {
        const float* wl = ws + R.woff(D.L - 1, K) + tid;
#pragma unroll
        for (int k = 0; k < (kRegLast ? K : 1); ++k) wlast[k] = wl[k * kTileSide * kTileSide];
    }
    // Layer 1, when it is not the last: the weights of the thread's first
    // position (p = tid) in registers too, the other positions' from shared
    // memory.
    constexpr bool kRegMid = F <= 5;
    float wmid[kRegMid ? K : 1];
    if (kRegMid && D.L >= 3) {
        const int sd1 = R.side(1);
        const float* wl = ws + R.woff(1, K) + tid;
#pragma unroll
        for (int k = 0; k < (kRegMid ? K : 1); ++k) wmid[k] = wl[k * sd1 * sd1];
    }
    const int lane = tid & 31, warp = tid >> 5;
    for (int tt = 1; tt <= nt; ++tt) {
        const int t = c + tt, cur = (tt - 1) & 1;
        const float* r_old = rs + cur * tot;
        float* r_new = rs + (cur ^ 1) * tot;
        const float* x_cur = xs + cur * s0 * s0;
        if (tt < nt) {                                       // next step's input
            const float* xt = x + ((long long)t * D.B + b) * D.N;
            float* xn = xs + (cur ^ 1) * s0 * s0;
            for (int p = tid; p < s0 * s0; p += kBlock) {
                const int code = info[p];
                cp_async_f32_zfill(&xn[p], code >= 0 ? xt + (code & (kOwnBit - 1)) : xt, code >= 0);
            }
            asm volatile("cp.async.commit_group;\n" ::: "memory");
        }
        const bool store_ckpt = mode == 0 && t % D.k == 0 && t < D.T;
        float r_last = 0.0f;                                  // tile neuron of the last layer
        for (int l = 0, o = 0, wofs = 0; l < D.L; ++l) {
            const int sd = R.side(l), sd2 = sd * sd, sp = sd + 2 * H;
            const float a = as[l];
            for (int p = tid; p < sd2; p += kBlock) {
                const int code = info[o + p];
                if (code < 0) continue;
                float I;
                if (l == 0) {
                    I = x_cur[p];
                } else {
                    // one partial sum per kernel row, rows added in order
                    const float* src = r_old + sbase[o + p];
                    const float* wl = ws + wofs + p;
                    float part[F];
                    if (kRegLast && l == D.L - 1) {
#pragma unroll
                        for (int kr = 0; kr < F; ++kr) {
                            part[kr] = 0.0f;
#pragma unroll
                            for (int kc = 0; kc < F; ++kc)
                                part[kr] = __fmaf_rn(wlast[kRegLast ? kr * F + kc : 0],
                                                     src[kr * sp + kc], part[kr]);
                        }
                    } else if (kRegMid && l == 1 && p == tid) {
#pragma unroll
                        for (int kr = 0; kr < F; ++kr) {
                            part[kr] = 0.0f;
#pragma unroll
                            for (int kc = 0; kc < F; ++kc)
                                part[kr] = __fmaf_rn(wmid[kRegMid ? kr * F + kc : 0],
                                                     src[kr * sp + kc], part[kr]);
                        }
                    } else {
#pragma unroll
                        for (int kr = 0; kr < F; ++kr) {
                            part[kr] = 0.0f;
#pragma unroll
                            for (int kc = 0; kc < F; ++kc)
                                part[kr] = __fmaf_rn(wl[(kr * F + kc) * sd2], src[kr * sp + kc],
                                                     part[kr]);
                        }
                    }
                    I = 0.0f;
#pragma unroll
                    for (int kr = 0; kr < F; ++kr) I += part[kr];
                }
                const float vp = vs[o + p];
                const float d = -vp + I;
                const float vn = vp + a * d;
                const float rn = sigmoid(vn);
                vs[o + p] = vn;
                r_new[o + p] = rn;
                if (code & kOwnBit) {
                    const long long gl = ((long long)l * D.B + b) * D.N + (code & (kOwnBit - 1));
                    if (mode == 1) {
                        seg_r[tt * S + gl] = rn;
                        seg_d[(tt - 1) * S + gl] = d;
                    } else if (store_ckpt) {
                        ckpt[(long long)(t / D.k) * S + gl] = vn;
                    }
                    if (l == D.L - 1) r_last = rn;
                }
            }
            o += sd2;
            if (l >= 1) wofs += K * sd2;
        }
        if (mode == 0) {
            // readout of the tile's last-layer neurons (thread tid owns
            // position tid of the 16 x 16 region): butterfly transpose
            // reduction per warp, warps added in order
            float cv[kMaxOutputs];
#pragma unroll
            for (int q = 0; q < kMaxOutputs; ++q) cv[q] = ows[q * kBlock + tid] * r_last;
#pragma unroll
            for (int half = kMaxOutputs / 2; half >= 1; half /= 2) {
                const bool up = lane & (2 * half);
#pragma unroll
                for (int j = 0; j < half; ++j) {
                    const float send = up ? cv[j] : cv[j + half];
                    const float keep = up ? cv[j + half] : cv[j];
                    cv[j] = keep + __shfl_xor_sync(0xFFFFFFFFu, send, 2 * half);
                }
            }
            const float y_lane = cv[0] + __shfl_xor_sync(0xFFFFFFFFu, cv[0], 1);
            float* rd = red + cur * (kBlock / 32) * kMaxOutputs;
            if ((lane & 1) == 0 && (lane >> 1) < D.O) rd[warp * kMaxOutputs + (lane >> 1)] = y_lane;
        }
        asm volatile("cp.async.wait_all;\n" ::: "memory");
        __syncthreads();
        if (mode == 0 && tid < D.O) {
            const float* rd = red + cur * (kBlock / 32) * kMaxOutputs;
            float y = 0.0f;
            for (int w = 0; w < kBlock / 32; ++w) y += rd[w * kMaxOutputs + tid];
            ypart[(((long long)(t - 1) * D.B + b) * D.nchunk + tile) * D.O + tid] = y;
        }
    }
}

// r = sigmoid(v) for a whole state (checkpoint reload / initial state).
__global__ void k_rate_rates(long long S, const float* __restrict__ v, float* __restrict__ r) {
    long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx < S) r[idx] = sigmoid(v[idx]);
}

// y[t][b][o] = sum of the blocks' partial readouts (block order) and the
// squared error of each (t, b).
__global__ void k_rate_finish(Dims D, const float* __restrict__ ypart,
                              const float* __restrict__ target, float* __restrict__ y,
                              float* __restrict__ loss_tb) {
    long long tb = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (tb >= (long long)D.T * D.B) return;
    const int b = (int)(tb % D.B);
    const float* yp = ypart + tb * D.nchunk * D.O;
    float e = 0.0f;
    for (int o = 0; o < D.O; ++o) {
        float s = 0.0f;
        for (int c = 0; c < D.nchunk; ++c) s += yp[(long long)c * D.O + o];
        y[tb * D.O + o] = s;
        const float diff = s - target[(long long)b * D.O + o];
        e += diff * diff;
    }
    loss_tb[tb] = e;
}

// loss = sum over (t, b) of the squared errors / (T B O): 256 strided
// partial sums reduced in a fixed tree.
__global__ void __launch_bounds__(256) k_rate_loss(Dims D, const float* __restrict__ loss_tb,
                                                   float* __restrict__ loss) {
    __shared__ float sm[256];
    const int tid = threadIdx.x;
    float s = 0.0f;
    for (long long j = tid; j < (long long)D.T * D.B; j += 256) s += loss_tb[j];
    sm[tid] = s;
    __syncthreads();
    for (int k = 128; k > 0; k >>= 1) {
        if (tid < k) sm[tid] += sm[tid + k];
        __syncthreads();
    }
    if (tid == 0) *loss = sm[0] / (float)((long long)D.T * D.B * D.O);
}

// gy[t][b][o] = gscale * (y - target), for every step.
__global__ void k_rate_gy(Dims D, float gscale, const float* __restrict__ y,
                          const float* __restrict__ target, float* __restrict__ gy) {
    long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long long)D.T * D.B * D.O) return;
    const long long bo = e % ((long long)D.B * D.O);
    gy[e] = gscale * (y[e] - target[bo]);
}

// Adjoint of one timestep, grid like the step kernel: lambda[t] from
// lambda[t+1] (the next layer's inputs at t+1 read the rates of t).  Neuron i
// of layer l feeds destinations j = i + h - (kr, kc) of layer l+1; the thread
// keeps those field x field weights (zero where j is outside the layer) in
// registers, and per batch element the CTA stages a_{l+1} * lambda_{l+1}[t+1]
// of its tile plus halo in shared memory, double-buffered like the step.
template <int F>
__global__ void __launch_bounds__(kBlock) k_rate_lambda(
    Dims D, const float* wt, const float* wo, const float* __restrict__ tau,
    const float* __restrict__ gy_t, const float* __restrict__ r_t,
    const float* __restrict__ lam_next, float* __restrict__ lam, float* __restrict__ dx_t) {
    using W = Halo<F>;
    constexpr int H = W::H;
    __shared__ float P[2][W::SIDE][W::PITCH];
    const int tiles_x = (D.cols + kTileSide - 1) / kTileSide;
    const int tile = blockIdx.x, l = blockIdx.y;
    const int ty0 = (tile / tiles_x) * kTileSide, tx0 = (tile % tiles_x) * kTileSide;
    const int tr = threadIdx.x / kTileSide, tc = threadIdx.x % kTileSide;
    const int ir = ty0 + tr, ic = tx0 + tc;
    const bool ok = ir < D.rows && ic < D.cols;
    const int i = ir * D.cols + ic;
    const bool last = l == D.L - 1;
    const float a = D.dt / __ldg(tau + l);
    const float a1 = last ? 0.0f : D.dt / __ldg(tau + l + 1);
    float wk[F * F];
#pragma unroll
    for (int kr = 0; kr < F; ++kr)
#pragma unroll
        for (int kc = 0; kc < F; ++kc) {
            const int jr = ir + H - kr, jc = ic + H - kc;
            wk[kr * F + kc] = (!last && ok && jr >= 0 && jr < D.rows && jc >= 0 && jc < D.cols)
                                  ? wt[((long long)l * F * F + kr * F + kc) * D.N + jr * D.cols + jc]
                                  : 0.0f;
        }
    float wov[kMaxOutputs];
#pragma unroll
    for (int o = 0; o < kMaxOutputs; ++o)
        wov[o] = (last && ok && o < D.O) ? wo[(long long)o * D.N + i] : 0.0f;
    const int b0 = blockIdx.z * D.bg, b1 = min(D.B, b0 + D.bg);
    const float* ln = last ? nullptr : lam_next + (long long)(l + 1) * D.B * D.N;
    const W halo(D, ty0, tx0);
    // launched as a programmatic dependent of the previous step's adjoint:
    // the weights above are loaded while it drains; nothing it writes is
    // read before it has completed
    asm volatile("griddepcontrol.wait;\n" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
    float pre[W::PER];
    if (!last) halo.fetch(ln + (long long)b0 * D.N, a1, pre);
    for (int b = b0, buf = 0; b < b1; ++b, buf ^= 1) {
        if (!last) halo.stage(pre, &P[buf][0][0]);
        const long long idx = ((long long)l * D.B + b) * D.N + i;
        const float r = ok ? r_t[idx] : 0.0f;
        const float own = ok ? lam_next[idx] : 0.0f;
        __syncthreads();
        if (!last && b + 1 < b1) halo.fetch(ln + (long long)(b + 1) * D.N, a1, pre);
        if (ok) {
            float g = 0.0f;
            if (last) {
#pragma unroll
                for (int o = 0; o < kMaxOutputs; ++o)
                    if (o < D.O) g += wov[o] * __ldg(gy_t + (long long)b * D.O + o);
            } else {
                float part[F];
#pragma unroll
                for (int kr = 0; kr < F; ++kr) {
                    part[kr] = 0.0f;
#pragma unroll
                    for (int kc = 0; kc < F; ++kc)
                        part[kr] = __fmaf_rn(wk[kr * F + kc], P[buf][tr + 2 * H - kr][tc + 2 * H - kc],
                                             part[kr]);
                }
#pragma unroll
                for (int kr = 0; kr < F; ++kr) g += part[kr];
            }
            const float lv = r * (1.0f - r) * g + (1.0f - a) * own;
            lam[idx] = lv;
            if (l == 0 && dx_t) dx_t[(long long)b * D.N + i] = a * lv;
        }
    }
}

// The dR kernel below takes the batch in kGroups groups of thread warps,
// kUnroll elements' loads in flight at a time.
constexpr int kGroups = 8;
constexpr int kUnroll = 8;

// dW, staged: grid (tiles, layers >= 1, timesteps of the segment).  Thread
// j of a 16 x 16 tile of layer l holds its F x F sums over the batch, in
// batch order, of lambda_l[t][j] times the source rates of t-1 in its window;
// per batch element the CTA stages the window (tile plus halo, zero outside
// the layer) in shared memory, double-buffered with the next element fetched
// into registers.  The step's totals go to part[tt][l-1][j][k], and
// k_rate_dw_acc adds the steps latest first into dW: a fixed order that does
// not depend on where the segments start.
template <int F>
__global__ void __launch_bounds__(kBlock) k_rate_dw_staged(Dims D, const float* __restrict__ seg_lam,
                                                          const float* __restrict__ seg_r,
                                                          float* __restrict__ part) {
    using W = Halo<F>;
    constexpr int K = F * F;
    __shared__ float win[2][W::SIDE][W::PITCH];
    const int tiles_x = (D.cols + kTileSide - 1) / kTileSide;
    const int tile = blockIdx.x, l = 1 + blockIdx.y, tt = blockIdx.z;
    const int ty0 = (tile / tiles_x) * kTileSide, tx0 = (tile % tiles_x) * kTileSide;
    const int tr = threadIdx.x / kTileSide, tc = threadIdx.x % kTileSide;
    const int jr = ty0 + tr, jc = tx0 + tc;
    const bool ok = jr < D.rows && jc < D.cols;
    const int j = jr * D.cols + jc;
    const float* lam = seg_lam + (long long)tt * D.S + (long long)l * D.B * D.N;
    const float* rp = seg_r + (long long)tt * D.S + (long long)(l - 1) * D.B * D.N;
    const W halo(D, ty0, tx0);
    float acc[K];
#pragma unroll
    for (int k = 0; k < K; ++k) acc[k] = 0.0f;
    float pre[W::PER];
    halo.fetch(rp, 1.0f, pre);
    float lv = ok ? lam[j] : 0.0f;
    for (int b = 0, buf = 0; b < D.B; ++b, buf ^= 1) {
        halo.stage(pre, &win[buf][0][0]);
        const float lcur = lv;
        __syncthreads();
        if (b + 1 < D.B) {
            halo.fetch(rp + (long long)(b + 1) * D.N, 1.0f, pre);
            lv = ok ? lam[(long long)(b + 1) * D.N + j] : 0.0f;
        }
#pragma unroll
        for (int kr = 0; kr < F; ++kr)
#pragma unroll
            for (int kc = 0; kc < F; ++kc)
                acc[kr * F + kc] = __fmaf_rn(lcur, win[buf][tr + kr][tc + kc], acc[kr * F + kc]);
    }
    if (!ok) return;
    float* out = part + (((long long)tt * (D.L - 1) + (l - 1)) * D.N + j) * K;
#pragma unroll
    for (int k = 0; k < K; ++k) out[k] = acc[k];
}

// dW[l-1][j][k] += a_l * part[tt] for the segment's steps, latest first.
__global__ void k_rate_dw_acc(Dims D, int nt, const float* __restrict__ tau,
                              const float* __restrict__ part, float* __restrict__ dw) {
    const long long per = (long long)D.N * D.K, n = (long long)(D.L - 1) * per;
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    const float a = D.dt / __ldg(tau + 1 + (int)(e / per));
    float acc = dw[e];
    for (int tt = nt - 1; tt >= 0; --tt) acc += a * part[(long long)tt * n + e];
    dw[e] = acc;
}

// dR, the same scheme: grid (tiles of 32 neurons i, timesteps), a CTA covers
// its 32 neurons for every output with 8 groups of batch elements, the step's
// total goes to part[tt][o][i] and k_rate_dwo_acc adds the steps latest first.
__global__ void __launch_bounds__(kBlock) k_rate_dwo(Dims D, int t0, const float* __restrict__ gy,
                                                    const float* __restrict__ seg_r,
                                                    float* __restrict__ part) {
    __shared__ float gsum[kGroups][32][kMaxOutputs + 1];
    const int il = threadIdx.x & 31, g = threadIdx.x >> 5;
    const int i = blockIdx.x * 32 + il, tt = blockIdx.y;
    const bool ok = i < D.N;
    const int bpg = (D.B + kGroups - 1) / kGroups;
    const int b0 = g * bpg, b1 = min(D.B, b0 + bpg);
    const int t = t0 + tt + 1;                          // 1-based step
    const float* gt = gy + (long long)(t - 1) * D.B * D.O;
    float st[kMaxOutputs];
#pragma unroll
    for (int o = 0; o < kMaxOutputs; ++o) st[o] = 0.0f;
    if (ok) {
        const float* r = seg_r + (long long)(tt + 1) * D.S + (long long)(D.L - 1) * D.B * D.N + i;
        for (int bb = b0; bb < b1; bb += kUnroll) {
            float rv[kUnroll];
#pragma unroll
            for (int u = 0; u < kUnroll; ++u) rv[u] = bb + u < b1 ? r[(long long)(bb + u) * D.N] : 0.0f;
#pragma unroll
            for (int u = 0; u < kUnroll; ++u) {
                if (bb + u >= b1) break;
#pragma unroll
                for (int o = 0; o < kMaxOutputs; ++o)
                    if (o < D.O) st[o] = __fmaf_rn(__ldg(gt + (long long)(bb + u) * D.O + o), rv[u], st[o]);
            }
        }
    }
#pragma unroll
    for (int o = 0; o < kMaxOutputs; ++o) gsum[g][il][o] = st[o];
    __syncthreads();
    if (g == 0 && ok) {
#pragma unroll
        for (int o = 0; o < kMaxOutputs; ++o) {
            if (o >= D.O) break;
            float tot = 0.0f;
            for (int q = 0; q < kGroups; ++q) tot += gsum[q][il][o];
            part[((long long)tt * D.O + o) * D.N + i] = tot;
        }
    }
}

__global__ void k_rate_dwo_acc(Dims D, int nt, const float* __restrict__ part,
                               float* __restrict__ dwo) {
    const long long n = (long long)D.O * D.N;
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    float acc = dwo[e];
    for (int tt = nt - 1; tt >= 0; --tt) acc += part[(long long)tt * n + e];
    dwo[e] = acc;
}

// Partial sums of lambda * d per (timestep, layer): grid (kTauBlocks, L, nt),
// each block a fixed strided slice of the batch x neurons reduced in a fixed
// tree, written to part[t][l][block].
__global__ void __launch_bounds__(256) k_rate_dtau_partial(Dims D, int t0,
                                                           const float* __restrict__ seg_lam,
                                                           const float* __restrict__ seg_d,
                                                           float* __restrict__ part) {
    __shared__ float sm[256];
    const int l = blockIdx.y, tt = blockIdx.z, tid = threadIdx.x;
    const long long per = (long long)D.B * D.N;
    const long long off = (long long)tt * D.S + (long long)l * per;
    float acc = 0.0f;
    for (long long e = (long long)blockIdx.x * 256 + tid; e < per; e += (long long)gridDim.x * 256)
        acc += seg_lam[off + e] * seg_d[off + e];
    sm[tid] = acc;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (tid < s) sm[tid] += sm[tid + s];
        __syncthreads();
    }
    if (tid == 0) part[((long long)(t0 + tt) * D.L + l) * kTauBlocks + blockIdx.x] = sm[0];
}

// dtau_l = -(dt / tau_l^2) * sum over timesteps (latest first) of the step
// sums; each step sum adds its blocks' partials in block order.
__global__ void __launch_bounds__(256) k_rate_dtau_final(Dims D, const float* __restrict__ tau,
                                                         const float* __restrict__ part,
                                                         float* __restrict__ step_sums,
                                                         float* __restrict__ dtau) {
    for (int e = threadIdx.x; e < D.T * D.L; e += blockDim.x) {
        float st = 0.0f;
        for (int q = 0; q < kTauBlocks; ++q) st += part[(long long)e * kTauBlocks + q];
        step_sums[e] = st;
    }
    __syncthreads();
    const int l = threadIdx.x;
    if (l >= D.L) return;
    float s = 0.0f;
    for (int t = D.T - 1; t >= 0; --t) s += step_sums[(long long)t * D.L + l];
    const float tv = __ldg(tau + l);
    dtau[l] = s * (-D.dt / (tv * tv));
}

Dims make_dims(const SgRateShape& s) {
    if (s.layers < 1 || s.rows < 1 || s.cols < 1 || s.batch < 1 || s.steps < 1 ||
        s.checkpoint < 1)
        throw SgError("rate network: sizes must be positive");
    if (s.outputs < 1 || s.outputs > kMaxOutputs)
        throw SgError("rate network: outputs must lie in 1..16");
    if (s.field < 1 || s.field % 2 == 0 || s.field > kMaxField)
        throw SgError("rate network: field must be odd and at most 9");
    if (!(s.dt > 0.0f)) throw SgError("rate network: dt must be positive");
    if ((long long)s.layers * s.batch > 65535) throw SgError("rate network: layers x batch too large");
    if (std::min(s.checkpoint, s.steps) > 65535)
        throw SgError("rate network: at most 65535 steps between checkpoints");
    Dims D;
    D.L = s.layers;
    D.rows = s.rows;
    D.cols = s.cols;
    D.N = s.rows * s.cols;
    D.field = s.field;
    D.h = s.field / 2;
    D.K = s.field * s.field;
    D.O = s.outputs;
    D.B = s.batch;
    D.T = s.steps;
    D.k = s.checkpoint;
    D.nseg = (s.steps + s.checkpoint - 1) / s.checkpoint;
    D.nchunk = ((D.rows + kTileSide - 1) / kTileSide) * ((D.cols + kTileSide - 1) / kTileSide);
    // batch elements per CTA: the largest group that still gives four CTAs
    // per SM (152 SMs), fewer halo and weight reloads per element
    D.bg = 1;
    for (int g = kMaxBatchGroup; g > 1; g >>= 1)
        if ((long long)D.nchunk * D.L * ((D.B + g - 1) / g) >= 4 * 152) { D.bg = g; break; }
    D.dt = s.dt;
    D.S = (long long)D.L * D.B * D.N;
    return D;
}

// Workspace layout (floats): checkpoints [nseg][S], segment states v, r
// [k+1][S], drives d and adjoints lambda [k][S], the lambda carried across
// segments [S], outputs y [T][B][O] and their partial sums, squared errors
// [T][B], dloss/dy [T][B][O], tau partials, transposed weights, and the
// per-step weight and readout gradient totals of one segment.
struct Work {
    float *ckpt, *seg_v, *seg_r, *seg_d, *seg_lam, *carry, *y, *ypart, *loss_tb, *gy, *tau_part,
        *tau_steps, *wt, *dw_part, *dwo_part;
    long long floats;
};

Work carve(const Dims& D, void* base) {
    Work w{};
    float* p = static_cast<float*>(base);
    auto take = [&](long long n) {
        float* q = p;
        n = (n + 63) / 64 * 64;       // 256-byte aligned pieces
        if (p) p += n;
        w.floats += n;
        return q;
    };
    w.ckpt = take((long long)D.nseg * D.S);
    w.seg_v = take((long long)(D.k + 1) * D.S);
    w.seg_r = take((long long)(D.k + 1) * D.S);
    w.seg_d = take((long long)D.k * D.S);
    w.seg_lam = take((long long)D.k * D.S);
    w.carry = take(D.S);
    w.y = take((long long)D.T * D.B * D.O);
    w.ypart = take((long long)D.T * D.B * D.nchunk * D.O);
    w.loss_tb = take((long long)D.T * D.B);
    w.gy = take((long long)D.T * D.B * D.O);
    w.tau_part = take((long long)D.T * D.L * kTauBlocks);
    w.tau_steps = take((long long)D.T * D.L);
    w.wt = take((long long)std::max(D.L - 1, 0) * D.K * D.N);
    const long long seg = std::min(D.k, D.T);
    w.dw_part = take(seg * std::max(D.L - 1, 0) * D.N * D.K);
    w.dwo_part = take(seg * D.O * D.N);
    return w;
}

unsigned grid_of(long long n) { return (unsigned)((n + 255) / 256); }

void transpose_weights(const Dims& D, const float* w, const Work& W, cudaStream_t st) {
    if (D.L < 2) return;
    k_rate_transpose<<<grid_of((long long)(D.L - 1) * D.N * D.K), 256, 0, st>>>(D, w, W.wt);
    SG_LAUNCH_CHECK();
}

dim3 tile_grid(const Dims& D) {
    return dim3((unsigned)D.nchunk, (unsigned)D.L, (unsigned)((D.B + D.bg - 1) / D.bg));
}

#define SG_RATE_FIELD(F_RT, CALL)                                                 \
    switch (F_RT) {                                                               \
        case 1: { constexpr int F = 1; CALL; } break;                             \
        case 3: { constexpr int F = 3; CALL; } break;                             \
        case 5: { constexpr int F = 5; CALL; } break;                             \
        case 7: { constexpr int F = 7; CALL; } break;                             \
        default: { constexpr int F = 9; CALL; } break;                            \
    }

void step(const Dims& D, const float* x_t, const float* wo, const float* tau, const Work& W,
          const float* v_prev, const float* r_prev, float* v_new, float* r_new, float* d_out,
          float* ypart, cudaStream_t st) {
    SG_RATE_FIELD(D.field, (k_rate_step<F><<<tile_grid(D), kBlock, 0, st>>>(
                               D, x_t, W.wt, wo, tau, v_prev, r_prev, v_new, r_new, d_out, ypart)));
    SG_LAUNCH_CHECK();
}

// One timestep of the adjoint, launched as a programmatic dependent of the
// launch before it (the next step's adjoint, or any kernel, which then simply
// completes first): each step's weight loads overlap the previous step's tail.
void lambda_step(const Dims& D, const float* wo, const float* tau, const Work& W,
                 const float* gy_t, const float* r_t, const float* lam_next, float* lam, float* dx_t,
                 cudaStream_t st) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = tile_grid(D);
    cfg.blockDim = dim3(kBlock);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const float* wt = W.wt;
    SG_RATE_FIELD(D.field, SG_CUDA(cudaLaunchKernelEx(&cfg, k_rate_lambda<F>, D, wt, wo, tau, gy_t,
                                                      r_t, lam_next, lam, dx_t)));
}

// Shared memory of the multi-step kernel, or 0 where it does not fit (the
// per-step kernels run instead, for the forward pass and the recompute alike).
size_t fused_bytes(const Dims& D) {
    static int optin = -1;
    if (optin < 0) {
        int dev = 0;
        SG_CUDA(cudaGetDevice(&dev));
        SG_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    }
    size_t floats = 0;
    SG_RATE_FIELD(D.field, (floats = fused_smem_floats<F>(D.L)));
    const size_t bytes = floats * sizeof(float);
    return bytes <= (size_t)optin ? bytes : 0;
}

void fused(const Dims& D, int mode, int c, int nt, const float* x, const float* wo,
           const float* tau, const Work& W, const float* v0, float* ckpt, float* ypart,
           float* seg_r, float* seg_d, cudaStream_t st) {
    const size_t bytes = fused_bytes(D);
    const dim3 grid((unsigned)D.nchunk, (unsigned)D.B);
    SG_RATE_FIELD(D.field, ({
        SG_CUDA(cudaFuncSetAttribute(k_rate_fused<F>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)bytes));
        k_rate_fused<F><<<grid, kBlock, bytes, st>>>(D, mode, c, nt, x, W.wt, wo, tau, v0, ckpt,
                                                     ypart, seg_r, seg_d);
    }));
    SG_LAUNCH_CHECK();
}

void forward(const Dims& D, const float* x, const float* w, const float* wo, const float* tau,
             const float* target, float* y_out, float* loss, void* ws, cudaStream_t st) {
    Work W = carve(D, ws);
    transpose_weights(D, w, W, st);
    SG_CUDA(cudaMemsetAsync(W.ckpt, 0, D.S * sizeof(float), st));
    if (fused_bytes(D)) {
        fused(D, 0, 0, D.T, x, wo, tau, W, nullptr, W.ckpt, W.ypart, nullptr, nullptr, st);
    } else {
        float* v[2] = {W.seg_v, W.seg_v + D.S};
        float* r[2] = {W.seg_r, W.seg_r + D.S};
        SG_CUDA(cudaMemsetAsync(v[0], 0, D.S * sizeof(float), st));
        k_rate_rates<<<grid_of(D.S), 256, 0, st>>>(D.S, v[0], r[0]);
        SG_LAUNCH_CHECK();
        for (int t = 1; t <= D.T; ++t) {
            const int p = (t - 1) & 1, q = t & 1;
            step(D, x + (long long)(t - 1) * D.B * D.N, wo, tau, W, v[p], r[p], v[q], r[q], nullptr,
                 W.ypart + (long long)(t - 1) * D.B * D.nchunk * D.O, st);
            if (t % D.k == 0 && t < D.T)
                SG_CUDA(cudaMemcpyAsync(W.ckpt + (long long)(t / D.k) * D.S, v[q],
                                        D.S * sizeof(float), cudaMemcpyDeviceToDevice, st));
        }
    }
    k_rate_finish<<<grid_of((long long)D.T * D.B), 256, 0, st>>>(D, W.ypart, target, W.y,
                                                                 W.loss_tb);
    SG_LAUNCH_CHECK();
    k_rate_loss<<<1, 256, 0, st>>>(D, W.loss_tb, loss);
    SG_LAUNCH_CHECK();
    if (y_out)
        SG_CUDA(cudaMemcpyAsync(y_out, W.y, (size_t)D.T * D.B * D.O * sizeof(float),
                                cudaMemcpyDeviceToDevice, st));
}

void backward(const Dims& D, const float* x, const float* w, const float* wo, const float* tau,
              const float* target, float grad_loss, void* ws, float* dw, float* dwo,
              float* dtau, float* dx, cudaStream_t st) {
    Work W = carve(D, ws);
    transpose_weights(D, w, W, st);
    const float gscale = grad_loss * 2.0f / (float)((long long)D.T * D.B * D.O);
    k_rate_gy<<<grid_of((long long)D.T * D.B * D.O), 256, 0, st>>>(D, gscale, W.y, target, W.gy);
    SG_LAUNCH_CHECK();
    if (D.L > 1)
        SG_CUDA(cudaMemsetAsync(dw, 0, (size_t)(D.L - 1) * D.N * D.K * sizeof(float), st));
    SG_CUDA(cudaMemsetAsync(dwo, 0, (size_t)D.O * D.N * sizeof(float), st));
    SG_CUDA(cudaMemsetAsync(W.carry, 0, D.S * sizeof(float), st));
    for (int seg = D.nseg - 1; seg >= 0; --seg) {
        const int c = seg * D.k, nt = std::min(D.k, D.T - c);
        if (fused_bytes(D)) {
            fused(D, 1, c, nt, x, wo, tau, W, W.ckpt + (long long)seg * D.S, nullptr, nullptr,
                  W.seg_r, W.seg_d, st);
        } else {
            SG_CUDA(cudaMemcpyAsync(W.seg_v, W.ckpt + (long long)seg * D.S, D.S * sizeof(float),
                                    cudaMemcpyDeviceToDevice, st));
            k_rate_rates<<<grid_of(D.S), 256, 0, st>>>(D.S, W.seg_v, W.seg_r);
            SG_LAUNCH_CHECK();
            for (int tt = 1; tt <= nt; ++tt)
                step(D, x + (long long)(c + tt - 1) * D.B * D.N, wo, tau, W,
                     W.seg_v + (tt - 1) * D.S, W.seg_r + (tt - 1) * D.S, W.seg_v + tt * D.S,
                     W.seg_r + tt * D.S, W.seg_d + (tt - 1) * D.S, nullptr, st);
        }
        for (int tt = nt; tt >= 1; --tt) {
            const int t = c + tt;
            const float* lam_next = tt == nt ? W.carry : W.seg_lam + (long long)tt * D.S;
            lambda_step(D, wo, tau, W, W.gy + (long long)(t - 1) * D.B * D.O,
                        W.seg_r + (long long)tt * D.S, lam_next,
                        W.seg_lam + (long long)(tt - 1) * D.S,
                        dx ? dx + (long long)(t - 1) * D.B * D.N : nullptr, st);
        }
        SG_CUDA(cudaMemcpyAsync(W.carry, W.seg_lam, D.S * sizeof(float),
                                cudaMemcpyDeviceToDevice, st));
        if (D.L > 1) {
            const dim3 grid((unsigned)D.nchunk, (unsigned)(D.L - 1), (unsigned)nt);
            SG_RATE_FIELD(D.field, (k_rate_dw_staged<F><<<grid, kBlock, 0, st>>>(
                                       D, W.seg_lam, W.seg_r, W.dw_part)));
            SG_LAUNCH_CHECK();
            k_rate_dw_acc<<<grid_of((long long)(D.L - 1) * D.N * D.K), 256, 0, st>>>(
                D, nt, tau, W.dw_part, dw);
            SG_LAUNCH_CHECK();
        }
        k_rate_dwo<<<dim3((unsigned)((D.N + 31) / 32), (unsigned)nt), kBlock, 0, st>>>(
            D, c, W.gy, W.seg_r, W.dwo_part);
        SG_LAUNCH_CHECK();
        k_rate_dwo_acc<<<grid_of((long long)D.O * D.N), 256, 0, st>>>(D, nt, W.dwo_part, dwo);
        SG_LAUNCH_CHECK();
        k_rate_dtau_partial<<<dim3(kTauBlocks, D.L, nt), 256, 0, st>>>(D, c, W.seg_lam, W.seg_d,
                                                                       W.tau_part);
        SG_LAUNCH_CHECK();
    }
    k_rate_dtau_final<<<1, 256, 0, st>>>(D, tau, W.tau_part, W.tau_steps, dtau);
    SG_LAUNCH_CHECK();
}

}  // namespace

extern "C" {

long long sg_rate_workspace_bytes(const SgRateShape* shape) {
    if (!shape) return SG_RATE_EINVAL;
    try {
        return carve(make_dims(*shape), nullptr).floats * (long long)sizeof(float);
    } catch (const std::exception& e) {
        sg::set_last_error(e.what());
    }
    return SG_RATE_EINVAL;
}

int sg_rate_forward(const SgRateShape* shape, const float* x, const float* weights,
                    const float* readout, const float* tau, const float* target, float* y,
                    float* loss, void* workspace, void* stream) {
    if (!shape || !x || !readout || !tau || !target || !loss || !workspace) return SG_RATE_EINVAL;
    try {
        Dims D = make_dims(*shape);
        if (D.L > 1 && !weights) return SG_RATE_EINVAL;
        forward(D, x, weights, readout, tau, target, y, loss, workspace,
                static_cast<cudaStream_t>(stream));
        return 0;
    } catch (const std::exception& e) {
        sg::set_last_error(e.what());
    }
    return SG_RATE_ECUDA;
}

int sg_rate_backward(const SgRateShape* shape, const float* x, const float* weights,
                     const float* readout, const float* tau, const float* target,
                     float grad_loss, void* workspace, float* d_weights, float* d_readout,
                     float* d_tau, float* d_x, void* stream) {
    if (!shape || !x || !readout || !tau || !target || !workspace || !d_readout || !d_tau)
        return SG_RATE_EINVAL;
    try {
        Dims D = make_dims(*shape);
        if (D.L > 1 && (!weights || !d_weights)) return SG_RATE_EINVAL;
        backward(D, x, weights, readout, tau, target, grad_loss, workspace, d_weights, d_readout,
                 d_tau, d_x, static_cast<cudaStream_t>(stream));
        return 0;
    } catch (const std::exception& e) {
        sg::set_last_error(e.what());
    }
    return SG_RATE_ECUDA;
}

}  // extern "C"
