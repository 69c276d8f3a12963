// Izhikevich trace activator for fully connected and subset matrices
// (src/core/state/impl/izhikevich_attributes.cpp:228-352 over the loops of
// src/core/engine/kernel/synapse_kernel.h:111-251), fed by the Tensor Memory
// Accelerator.
//
// The matrices are banded: [destination / 8][source][destination % 8], so the
// kR source rows of a band form one contiguous block per array (1 KB for 32
// rows).  Each CTA owns a run of bands (3 or 4 for 4096 destinations: the
// bands are spread over every SM) and walks the source rows in kR-row chunks:
//   * a producer warp issues, per chunk, one 2-D tensor TMA load per array
//     (weights, short-term R and w, delays, short and long traces) whose box
//     rows are the CTA's bands' contiguous chunks, into a shared-memory ring,
//     completing on the stage's mbarrier.  A connection that never learns
//     has its weights and short-term factors fixed for a whole run: it reads
//     one array of w * (R * w) instead of the three (EFF), computed after
//     each upload with the activator's own float operations;
//   * 8 compute warps compute the chunk's synapses (every shared-memory load
//     of a thread first, then its arithmetic), write the pre-decay traces to
//     a ring of sums tiles and arrive on the stage's "consumed" mbarrier
//     (they synchronise only among themselves; warp 0 also prefetches the
//     chunks' source words);
//   * the producer refills a stage as soon as it is consumed;
//   * two sum warps, one lane per destination, add each chunk's pre-decay
//     traces in source order (the reference's sequential fp32 sum) and write
//     the decayed traces back to HBM (streaming stores, 32-byte sectors), while
//     the compute warps go on with the next chunks.  Nothing is written into
//     the stages, so they need no store to drain before a refill, and the
//     shared-memory pipe carries the loads, the sums and nothing else.
// Every mbarrier wait is bounded: if one runs out, the kernel records the
// fact in a device flag, waits (bounded) for its loads in flight and returns;
// check_iz_cols_errors reports it on the host.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_pipeline.h>

#include <algorithm>
#include <cstdlib>
#include <string>
#include <mutex>

#include "cuda_check.h"
#include "iz_cols_tma.cuh"

namespace sg {

namespace {

#ifndef SG_COLS_ROWS
#define SG_COLS_ROWS 32                  // kR * 8 floats per TMA box row: at most 256
#endif
#ifndef SG_COLS_STAGES
#define SG_COLS_STAGES 6
#endif
constexpr int kR = SG_COLS_ROWS;         // source rows per chunk
constexpr int kStages = SG_COLS_STAGES;
constexpr int kMaxBands = 4;             // bands per CTA at most (32 destinations)
constexpr int kCompute = 256;            // compute threads (8 warps)
constexpr int kSumWarps = 2;             // short-trace and long-trace sums
constexpr int kSumBufs = 3;              // chunks of sums in flight to the sum warps
constexpr int kThreads = kCompute + 32 * kSumWarps + 32;   // plus one producer warp
constexpr int kSumPitch = 40;            // sums row pitch: conflict-free writes and reads
constexpr int kWaitLimit = 1 << 20;
constexpr int kBlockFloats = kR * kBand; // one band's chunk: 32 rows x 8 destinations
// The thread that issues the TMA copies: lane 0
// of the producer warp, which takes no part in the compute warps' barriers.
constexpr int kProducer = kCompute + 32 * kSumWarps;

constexpr int kArrays = 6;               // w, R, w_stp (or w * (R * w_stp)), [delay], short, [long]

struct ColsMaps {
    CUtensorMap m[2][kArrays];           // [bands of the wider CTAs, narrower][array]
};

struct ColsParams {
    DGeom g;
    int nrows, ncols, base_bands, extra;
    const uint32_t* src;
    float gcond, short_tau, long_tau;
    float* short_cond;
    float* long_cond;
    float* short_tr;                     // the banded trace arrays (decayed traces written back)
    float* long_tr;
};

__device__ int g_cols_error = 0;
// Testing hook (sg_test_cols_skip_chunk): the producer issues no load for this
// chunk, so the consumers' bounded wait for it runs out; -1 in normal use.
__device__ int g_cols_skip_chunk = -1;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    {
        // a phase that has already completed: no suspending wait
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            " selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    for (int it = 0; it < kWaitLimit; ++it) {
        uint32_t ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            " selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(ok)
            : "r"(bar), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}

// A banded array seen as a 2-D tensor [band][source row * 8 + lane]: one box
// row is a band's whole chunk (kR * 8 contiguous floats).
__device__ __forceinline__ void tma_load2(uint32_t dst, const CUtensorMap* map, int x, int y,
                                          uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3}], [%4];"
        :
        : "r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
        : "memory");
}

template <bool SUBSET>
__device__ __forceinline__ int source_of_row(const DGeom& g, int row) {
    if (!SUBSET) return row;
    const int fkc = g.fc1 - g.fc0;
    return (row / fkc + g.fr0) * g.from_cols + (row % fkc + g.fc0);
}

template <int SR, bool LONG, bool SUBSET, bool EFF>
__global__ void __launch_bounds__(kThreads, 1)
    k_iz_cols_bulk(const __grid_constant__ ColsMaps maps, const ColsParams p) {
    constexpr int HAS_D = SR == S_BIT ? 1 : 0;
    constexpr int NW = EFF ? 1 : 3;                        // weight arrays
    constexpr int NA = NW + 1 + HAS_D + (LONG ? 1 : 0);
    constexpr int A_D = NW, A_ST = NW + HAS_D, A_LT = NW + 1 + HAS_D;
    constexpr int kTile = kMaxBands * kBlockFloats;        // floats per array per stage
    constexpr int kSumBuf = 2 * kR * kSumPitch;            // one chunk's short + long sums
    extern __shared__ unsigned char smem_raw[];
    __shared__ uint32_t s_words[kStages][kR];              // source words, one slot per stage
    __shared__ int s_abort;
    // TMA destinations: 128-byte aligned (the allocation has 128 bytes to spare)
    float* stages = reinterpret_cast<float*>(                // [S][NA][bands][kR][8]
        (reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
    float* sums = stages + (size_t)kStages * NA * kTile;   // [kSumBufs][2][kR][kSumPitch]
    uint64_t* full = reinterpret_cast<uint64_t*>(sums + kSumBufs * kSumBuf);
    uint64_t* consumed = full + kStages;
    uint64_t* sums_full = consumed + kStages;
    uint64_t* sums_empty = sums_full + kSumBufs;

    const int tid = threadIdx.x, b = blockIdx.x;
    const int nb = p.base_bands + (b < p.extra ? 1 : 0);
    const int band0 = b * p.base_bands + min(b, p.extra);
    const int ncol = nb * kBand;
    const int nchunks = (p.nrows + kR - 1) / kR;
    const CUtensorMap* mp = maps.m[b < p.extra ? 0 : 1];
    auto tile = [&](int s, int a) { return stages + ((size_t)s * NA + a) * kTile; };
    auto chunk_rows = [&](int ch) { return min(kR, p.nrows - ch * kR); };
    auto parity = [](int ch) { return (uint32_t)((ch / kStages) & 1); };
    auto sum_parity = [](int ch) { return (uint32_t)((ch / kSumBufs) & 1); };

    if (tid == 0) {
        for (int s = 0; s < kStages; ++s) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&full[s])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&consumed[s])),
                         "r"(kCompute));
        }
        for (int q = 0; q < kSumBufs; ++q) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&sums_full[q])),
                         "r"(kCompute));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&sums_empty[q])),
                         "r"(32 * kSumWarps));
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        s_abort = 0;
    }
    // Source words of a chunk, fetched by warp 0 with cp.async kStages-1
    // chunks ahead of their use (one commit group per chunk).
    auto fetch_words = [&](int ch) {
        if (ch < nchunks && tid < kR) {
            const int row = ch * kR + tid;
            if (row < p.nrows)
                __pipeline_memcpy_async(&s_words[ch % kStages][tid],
                                        p.src + source_of_row<SUBSET>(p.g, row), 4);
        }
        __pipeline_commit();
    };
    if (tid < kR) {
        for (int c = 0; c < kStages - 1; ++c) fetch_words(c);
        __pipeline_wait_prior(kStages - 2);                // chunk 0 landed
    }
    __syncthreads();

    if (tid >= kProducer) {
        // ---- producer warp: loads into free stages
        if (tid == kProducer) {
            const int skip = g_cols_skip_chunk;
            auto issue = [&](int ch) {
                if (ch == skip) return;
                const int s = ch % kStages;
                const uint32_t bar = smem_u32(&full[s]);
                // the full box is counted, rows past the end included (zero-filled)
                asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar),
                             "r"((uint32_t)(((NA - HAS_D) * 4 + HAS_D) * nb * kBlockFloats))
                             : "memory");
                for (int a = 0; a < NA; ++a)
                    tma_load2(smem_u32(tile(s, a)), &mp[a], ch * kBlockFloats, band0, bar);
            };
            int issued = min(kStages, nchunks);
            for (int c = 0; c < issued; ++c) issue(c);
            int ch = 0;
            for (; ch < nchunks; ++ch) {
                const int s = ch % kStages;
                if (!mbar_wait(smem_u32(&consumed[s]), parity(ch))) break;
                // the compute warps are done with the stage: refill it
                if (ch + kStages < nchunks) {
                    issue(ch + kStages);
                    ++issued;
                }
            }
            if (ch < nchunks) {
                // the compute warps stopped: let the loads in flight land
                // (bounded) before the shared memory goes away
                atomicExch(&g_cols_error, 1);
                for (int c = ch; c < issued; ++c) mbar_wait(smem_u32(&full[c % kStages]), parity(c));
            }
        }
    } else if (tid >= kCompute) {
        // ---- sum warps: warp kCompute/32 adds the short traces, the next the
        // long ones; one lane per destination, each chunk's rows in order
        const int kind = (tid - kCompute) / 32, c = (tid - kCompute) % 32;
        const bool owner = c < ncol && (kind == 0 || LONG);
        const float tau = kind == 0 ? p.short_tau : p.long_tau;
        // this lane's column of the banded trace array, row 0
        float* trace = (kind == 0 ? p.short_tr : p.long_tr) +
                       (size_t)(band0 + c / kBand) * p.nrows * kBand + c % kBand;
        float acc = 0.0f;
        int ch = 0;
        for (; ch < nchunks; ++ch) {
            const int q = ch % kSumBufs;
            if (!mbar_wait(smem_u32(&sums_full[q]), sum_parity(ch))) break;
            if (owner) {
                const float* col = sums + q * kSumBuf + kind * kR * kSumPitch + c;
                const int nr = chunk_rows(ch);
                float* tr = trace + (size_t)ch * kR * kBand;
                if (nr == kR) {
                    float v[kR];
#pragma unroll
                    for (int j = 0; j < kR; ++j) v[j] = col[j * kSumPitch];
#pragma unroll
                    for (int j = 0; j < kR; ++j) acc += v[j];
                    // the decayed traces go back to HBM from here (the sums
                    // hold every pre-decay trace of the chunk)
#pragma unroll
                    for (int j = 0; j < kR; ++j) __stcs(tr + j * kBand, v[j] * tau);
                } else {
                    for (int j = 0; j < nr; ++j) {
                        const float v = col[j * kSumPitch];
                        acc += v;
                        __stcs(tr + j * kBand, v * tau);
                    }
                }
            }
            asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&sums_empty[q]))
                         : "memory");
        }
        if (ch == nchunks && owner) {
            const int col = band0 * kBand + c;
            if (col < p.ncols) {
                const int to = dest_of<SUBSET ? T_SUBSET : T_FC>(p.g, col);
                if (kind == 0) p.short_cond[to] += acc;
                else p.long_cond[to] += acc;
            }
        } else if (ch < nchunks && c == 0) {
            atomicExch(&g_cols_error, 1);
        }
    } else {
        // ---- compute warps
        constexpr int kPer = kTile / kCompute;
        int eo[kPer], ej[kPer], ecol[kPer];             // offset band*kR*8 + row*8 + lane8
#pragma unroll
        for (int k = 0; k < kPer; ++k) {
            const int e = tid + k * kCompute;
            eo[k] = e < nb * kBlockFloats ? e : -1;
            ej[k] = (e % kBlockFloats) / kBand;
            ecol[k] = (e / kBlockFloats) * kBand + e % kBand;
        }
        bool aborted = false;
        for (int ch = 0; ch < nchunks; ++ch) {
            const int s = ch % kStages, q = ch % kSumBufs;
            if (!mbar_wait(smem_u32(&full[s]), parity(ch))) s_abort = 1;
            // the sums buffer is free once the sum warps have read chunk ch - kSumBufs
            if (ch >= kSumBufs &&
                !mbar_wait(smem_u32(&sums_empty[q]), sum_parity(ch - kSumBufs)))
                s_abort = 1;
            float* sb = sums + q * kSumBuf;
            const float* tw = tile(s, 0);
            const float* tr = tile(s, EFF ? 0 : 1);
            const float* tsw = tile(s, EFF ? 0 : 2);
            const float* tst = tile(s, A_ST);
            const float* tlt = tile(s, LONG ? A_LT : A_ST);
            // every load of the thread's synapses first, then the arithmetic
            // and the stores (a store into the sums would otherwise hold back
            // the next synapse's loads: the compiler cannot tell them apart)
            float term[kPer], st[kPer], lt[kPer];
#pragma unroll
            for (int k = 0; k < kPer; ++k) {
                const int o = eo[k] < 0 ? 0 : eo[k];
                const uint32_t word = s_words[s][ej[k]];
                const int delay =
                    HAS_D ? (int)reinterpret_cast<const uint8_t*>(tile(s, A_D))[o] : 0;
                const float weight = EFF ? tw[o] : tw[o] * (tr[o] * tsw[o]);
                term[k] = extract<SR>(word, delay) * weight;
                st[k] = tst[o];
                lt[k] = LONG ? tlt[o] : 0.0f;
            }
#pragma unroll
            for (int k = 0; k < kPer; ++k) {
                const int o = eo[k];
                if (o < 0) continue;
                const float add = term[k] * p.gcond;
                const float sv = st[k] + add;
                const int so = ej[k] * kSumPitch + ecol[k];
                sb[so] = sv;
                if (LONG) sb[kR * kSumPitch + so] = lt[k] + add;
            }
            asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&sums_full[q]))
                         : "memory");
            if (tid < kR) {
                fetch_words(ch + kStages - 1);
                __pipeline_wait_prior(kStages - 2);        // chunk ch+1 landed
            }
            // the stage is refilled (TMA) once every compute thread has read it
            asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&consumed[s]))
                         : "memory");
            asm volatile("bar.sync 1, %0;" ::"n"(kCompute) : "memory");
            if (s_abort) {
                aborted = true;
                break;
            }
        }
        if (aborted && tid == 0) atomicExch(&g_cols_error, 1);
    }
    __syncthreads();
}

size_t cols_smem_bytes(int na) {
    return 128 + (size_t)kStages * na * kMaxBands * kBlockFloats * 4 +
           (size_t)kSumBufs * 2 * kR * kSumPitch * 4 + (2 * kStages + 2 * kSumBufs) * sizeof(uint64_t);
}

}  // namespace

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static std::once_flag once;
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    std::call_once(once, [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault,
                                             &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
    });
    return fn;
}

struct IzColsPlan {
    ColsMaps maps;
    ColsParams base;
    int n_cta = 0, na = 0;
    bool has_delay = false, long_trace = false, eff = false;
    size_t smem = 0;
    // few source rows: one CTA per band, no pipeline (k_iz_cols_small)
    bool small = false;
    const float *w = nullptr, *stp_r = nullptr, *stp_w = nullptr;
    const uint8_t* delays = nullptr;
};

// Source rows up to which a band's pre-decay traces fit in shared memory
// (2 x rows x 8 floats) and the one-pass kernel beats the TMA pipeline.
constexpr int kSmallRows = 1536;

// One-pass activator for matrices of at most kSmallRows source rows: one CTA
// per band of 8 destinations reads the band's synapses with plain coalesced
// loads (every synapse of the band in flight across the CTA), writes the
// decayed traces back and the pre-decay traces to shared memory, then 8 (16
// for two traces) threads add each destination's terms in source order.  The
// float operations are the pipelined kernel's, in the same order.
template <int SR, bool LONG, bool SUBSET, bool EFF>
__global__ void __launch_bounds__(512) k_iz_cols_small(const ColsParams p, const float* __restrict__ w,
                                                       const float* __restrict__ stp_r,
                                                       const float* __restrict__ stp_w,
                                                       const uint8_t* __restrict__ d8, size_t pitch) {
    extern __shared__ float pre[];                         // [2][nrows * 8]
    constexpr int U = 8;                                   // synapses a thread has in flight
    const int band = blockIdx.x, n = p.nrows * kBand;
    const size_t base = (size_t)band * n;
    for (int e0 = threadIdx.x; e0 < n; e0 += U * blockDim.x) {
        uint32_t word[U];
        int delay[U];
        float weight[U], st[U], lt[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int e = min(e0 + u * (int)blockDim.x, n - 1);
            const size_t i = base + e;
            word[u] = __ldg(p.src + source_of_row<SUBSET>(p.g, e >> 3));
            delay[u] = SR == S_BIT ? (int)__ldg(d8 + (size_t)band * pitch + e) : 0;
            weight[u] = EFF ? __ldg(w + i) : __ldg(w + i) * (__ldg(stp_r + i) * __ldg(stp_w + i));
            st[u] = __ldcs(p.short_tr + i);
            lt[u] = LONG ? __ldcs(p.long_tr + i) : 0.0f;
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int e = e0 + u * (int)blockDim.x;
            if (e >= n) break;
            const size_t i = base + e;
            const float add = (extract<SR>(word[u], delay[u]) * weight[u]) * p.gcond;
            const float sv = st[u] + add;
            pre[e] = sv;
            __stcs(p.short_tr + i, sv * p.short_tau);
            if (LONG) {
                const float lv = lt[u] + add;
                pre[n + e] = lv;
                __stcs(p.long_tr + i, lv * p.long_tau);
            }
        }
    }
    __syncthreads();
    const int kind = threadIdx.x >> 3, lane = threadIdx.x & 7;
    if (threadIdx.x >= 16 || (kind == 1 && !LONG)) return;
    const float* col = pre + kind * n + lane;
    float acc = 0.0f;
    int r = 0;
    for (; r + 8 <= p.nrows; r += 8) {
        float v[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) v[j] = col[(r + j) * kBand];
#pragma unroll
        for (int j = 0; j < 8; ++j) acc += v[j];
    }
    for (; r < p.nrows; ++r) acc += col[r * kBand];
    const int c = band * kBand + lane;
    if (c < p.ncols) {
        const int to = dest_of<SUBSET ? T_SUBSET : T_FC>(p.g, c);
        if (kind == 0) p.short_cond[to] += acc;
        else p.long_cond[to] += acc;
    }
}

// w * (R * w_stp), the activator's weight of a synapse, over the whole banded
// array (padding included)
__global__ void k_iz_effective_weights(size_t n, const float* __restrict__ w,
                                       const float* __restrict__ stp_r,
                                       const float* __restrict__ stp_w, float* __restrict__ eff) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) eff[i] = w[i] * (stp_r[i] * stp_w[i]);
}

void fill_iz_effective_weights(size_t n, const float* w, const float* stp_r, const float* stp_w,
                               float* eff, cudaStream_t s) {
    k_iz_effective_weights<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, w, stp_r, stp_w, eff);
    SG_LAUNCH_CHECK();
}

size_t iz_delay_bytes_pitch(int nrows) { return ((size_t)nrows * kBand + 15) / 16 * 16; }

// d8[band][row * 8 + lane] (band pitch iz_delay_bytes_pitch) = delays[banded]
__global__ void k_iz_delays_to_bytes(int nrows, int bands, size_t pitch,
                                     const int* __restrict__ delays, uint8_t* __restrict__ d8) {
    const size_t per = (size_t)nrows * kBand;
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= per * bands) return;
    const size_t band = i / per, e = i - band * per;
    d8[band * pitch + e] = (uint8_t)delays[i];
}

void fill_iz_delay_bytes(int nrows, int ncols, const int* delays, uint8_t* d8, cudaStream_t s) {
    const int bands = (ncols + kBand - 1) / kBand;
    const size_t n = (size_t)nrows * kBand * bands;
    k_iz_delays_to_bytes<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(
        nrows, bands, iz_delay_bytes_pitch(nrows), delays, d8);
    SG_LAUNCH_CHECK();
}

std::shared_ptr<IzColsPlan> make_iz_cols_plan(int nrows, int ncols, const float* w,
                                              const float* stp_r, const float* stp_w,
                                              const uint8_t* delays, float* short_tr,
                                              float* long_tr, const float* eff, int ctas) {
    if (nrows < 1 || ncols < 1) return nullptr;
    auto encode = encode_fn();
    if (!encode) return nullptr;
    int dev = 0, sms = 0, optin = 0;
    SG_CUDA(cudaGetDevice(&dev));
    SG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    SG_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    auto plan = std::make_shared<IzColsPlan>();
    const int bands = (ncols + kBand - 1) / kBand;
    plan->n_cta = std::max(std::min(ctas > 0 ? ctas : sms, bands),
                           (bands + kMaxBands - 1) / kMaxBands);
    plan->has_delay = delays != nullptr;
    plan->long_trace = long_tr != nullptr;
    plan->eff = eff != nullptr;
    plan->w = eff ? eff : w;
    plan->stp_r = stp_r;
    plan->stp_w = stp_w;
    plan->delays = delays;
    {
        // SG_IZ_COLS_PATH=tma or small forces a path (tests run both)
        const char* e = std::getenv("SG_IZ_COLS_PATH");
        const std::string path = e ? e : "";
        plan->small = path == "small" || (path != "tma" && nrows <= kSmallRows);
        if (plan->small && nrows > kSmallRows) plan->small = false;
    }
    plan->na = (plan->eff ? 2 : 4) + (plan->has_delay ? 1 : 0) + (plan->long_trace ? 1 : 0);
    plan->smem = cols_smem_bytes(plan->na);
    if ((long long)plan->smem > optin) return nullptr;
    ColsParams& p = plan->base;
    p = ColsParams{};
    p.nrows = nrows;
    p.ncols = ncols;
    p.base_bands = bands / plan->n_cta;
    p.extra = bands % plan->n_cta;
    p.short_tr = short_tr;
    p.long_tr = long_tr;
    const void* arrays[kArrays];
    int a = 0;
    if (plan->eff) {
        arrays[a++] = eff;
    } else {
        arrays[a++] = w;
        arrays[a++] = stp_r;
        arrays[a++] = stp_w;
    }
    if (plan->has_delay) arrays[a++] = delays;
    arrays[a++] = short_tr;
    if (plan->long_trace) arrays[a++] = long_tr;
    // [band][source row * 8 + lane] as a 2-D tensor; box {kR * 8, bands}
    for (int wide = 0; wide < 2; ++wide) {
        const int nb = p.base_bands + (wide == 0 ? 1 : 0);
        if (nb < 1 || nb > kMaxBands || (wide == 0 && p.extra == 0)) continue;
        for (int i = 0; i < plan->na; ++i) {
            cuuint64_t dims[2] = {(cuuint64_t)nrows * kBand, (cuuint64_t)bands};
            cuuint64_t strides[1] = {(cuuint64_t)nrows * kBand * 4};
            cuuint32_t box[2] = {(cuuint32_t)kBlockFloats, (cuuint32_t)nb};
            cuuint32_t estr[2] = {1, 1};
            // the delays are bytes, each band's rows padded to 16 bytes
            const bool bytes = plan->has_delay && i == (plan->eff ? 1 : 3);
            if (bytes) strides[0] = (cuuint64_t)iz_delay_bytes_pitch(nrows);
            CUresult r = encode(&plan->maps.m[wide][i],
                                bytes ? CU_TENSOR_MAP_DATA_TYPE_UINT8 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2,
                                const_cast<void*>(arrays[i]), dims, strides, box, estr,
                                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
            if (r != CUDA_SUCCESS) return nullptr;
        }
    }
    return plan;
}

template <int SR, bool LONG, bool SUBSET, bool EFF>
static void launch_t(const IzColsPlan& plan, const ColsParams& p, cudaStream_t s) {
    if (plan.small) {
        const size_t bytes = (size_t)2 * p.nrows * kBand * sizeof(float);
        static size_t small_configured = 0;
        if (bytes > 48 * 1024 && small_configured < bytes) {
            SG_CUDA(cudaFuncSetAttribute(k_iz_cols_small<SR, LONG, SUBSET, EFF>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
            small_configured = bytes;
        }
        const int bands = (p.ncols + kBand - 1) / kBand;
        k_iz_cols_small<SR, LONG, SUBSET, EFF><<<bands, 512, bytes, s>>>(
            p, plan.w, plan.stp_r, plan.stp_w, plan.delays, iz_delay_bytes_pitch(p.nrows));
        SG_LAUNCH_CHECK();
        return;
    }
    static int configured = 0;
    if (configured < (int)plan.smem) {
        SG_CUDA(cudaFuncSetAttribute(k_iz_cols_bulk<SR, LONG, SUBSET, EFF>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)plan.smem));
        configured = (int)plan.smem;
    }
    k_iz_cols_bulk<SR, LONG, SUBSET, EFF><<<plan.n_cta, kThreads, plan.smem, s>>>(plan.maps, p);
    SG_LAUNCH_CHECK();
}

void launch_iz_cols_tma(const IzColsPlan& plan, const DGeom& g, int src_type, bool subset,
                        const uint32_t* src, float gcond, float short_tau, float long_tau,
                        float* short_cond, float* long_cond, cudaStream_t stream) {
    if ((src_type == S_BIT) != plan.has_delay) throw SgError("cols plan: delay array mismatch");
    ColsParams p = plan.base;
    p.g = g;
    p.src = src;
    p.gcond = gcond;
    p.short_tau = short_tau;
    p.long_tau = long_tau;
    p.short_cond = short_cond;
    p.long_cond = long_cond;
    const bool lng = plan.long_trace;
#define SG_COLS(SRV, EF)                                                     \
    if (lng) {                                                               \
        if (subset) launch_t<SRV, true, true, EF>(plan, p, stream);          \
        else launch_t<SRV, true, false, EF>(plan, p, stream);                \
    } else {                                                                 \
        if (subset) launch_t<SRV, false, true, EF>(plan, p, stream);         \
        else launch_t<SRV, false, false, EF>(plan, p, stream);               \
    }
    if (plan.eff) {
        if (src_type == S_BIT) { SG_COLS(S_BIT, true) }
        else if (src_type == S_FLOAT) { SG_COLS(S_FLOAT, true) }
        else { SG_COLS(S_INT, true) }
    } else {
        if (src_type == S_BIT) { SG_COLS(S_BIT, false) }
        else if (src_type == S_FLOAT) { SG_COLS(S_FLOAT, false) }
        else { SG_COLS(S_INT, false) }
    }
#undef SG_COLS
}

void set_iz_cols_skip_chunk(int chunk) {
    SG_CUDA(cudaMemcpyToSymbol(g_cols_skip_chunk, &chunk, sizeof(int)));
}

void check_iz_cols_errors() {
    int flag = 0;
    SG_CUDA(cudaMemcpyFromSymbol(&flag, g_cols_error, sizeof(int)));
    if (flag) {
        int zero = 0;
        SG_CUDA(cudaMemcpyToSymbol(g_cols_error, &zero, sizeof(int)));
        throw SgError("Izhikevich column activator: a TMA pipeline wait timed out");
    }
}

}  // namespace sg
