// Izhikevich trace activator for fully connected and subset matrices
// (src/core/state/impl/izhikevich_attributes.cpp:228-352 over the loops of
// src/core/engine/kernel/synapse_kernel.h:111-251), fed by the Tensor Memory
// Accelerator.
//
// The matrices are [source row][destination column] (the reference's GPU
// layout).  Each CTA owns a band of 4*k destination columns -- the columns
// are split into as many bands as there are SMs (24 or 28 columns for 4096),
// so every SM streams -- and walks every source row in 32-row chunks:
//   * one thread issues, per chunk, one 2-D TMA tile load per array (weights,
//     short-term R and w, delays, short and long traces) into an 8-stage
//     shared-memory ring, completing on the stage's mbarrier;
//   * all threads compute the synapses of the chunk, write the pre-decay
//     traces to a sums tile and the decayed traces back into the stage;
//   * one thread writes the decayed trace tiles back with TMA stores;
//   * one thread per column adds the chunk's pre-decay traces in row order,
//     keeping the reference's sequential fp32 sum.
// Every mbarrier wait is bounded: if one runs out, the kernel records the
// fact in a device flag, waits (bounded) for its loads in flight, drains its
// stores and returns; check_iz_cols_errors reports it on the host.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <mutex>

#include "cuda_check.h"
#include "iz_cols_tma.cuh"

namespace sg {

namespace {

constexpr int kR = 32;           // rows per chunk
constexpr int kStages = 8;
constexpr int kMaxWidth = 32;    // columns per CTA at most
constexpr int kThreads = 256;
constexpr int kArrays = 6;       // w, R, w_stp, [delay], short, [long]
constexpr int kWaitLimit = 1 << 20;
// The thread that issues the TMA loads and stores (and waits on its store
// groups): in a warp that adds no column sums, so neither delays the other.
constexpr int kProducer = 96;

struct ColsMaps {
    CUtensorMap m[2][kArrays];   // [wide band, narrow band][array]
};

struct ColsParams {
    DGeom g;
    int nrows, ncols, base_units, extra;
    const uint32_t* src;
    float gcond, short_tau, long_tau;
    float* short_cond;
    float* long_cond;
};

__device__ int g_cols_error = 0;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
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

__device__ __forceinline__ void tma_load(uint32_t dst, const CUtensorMap* map, int x, int y,
                                         uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3}], [%4];"
        :
        : "r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
        : "memory");
}

__device__ __forceinline__ void tma_store(const CUtensorMap* map, int x, int y, uint32_t src) {
    asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%1, %2}], [%3];"
                 :
                 : "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(src)
                 : "memory");
}

template <bool SUBSET>
__device__ __forceinline__ int source_of_row(const DGeom& g, int row) {
    if (!SUBSET) return row;
    const int fkc = g.fc1 - g.fc0;
    return (row / fkc + g.fr0) * g.from_cols + (row % fkc + g.fc0);
}

template <int SR, bool LONG, bool SUBSET>
__global__ void __launch_bounds__(kThreads, 1)
    k_iz_cols_tma(const __grid_constant__ ColsMaps maps, const ColsParams p) {
    constexpr int HAS_D = SR == S_BIT ? 1 : 0;
    constexpr int NA = 4 + HAS_D + (LONG ? 1 : 0);
    constexpr int A_ST = 3 + HAS_D, A_LT = 4 + HAS_D;
    extern __shared__ unsigned char smem_raw[];
    __shared__ uint32_t s_words[2][kR];
    __shared__ int s_abort;

    const int tid = threadIdx.x, b = blockIdx.x;
    const bool wide = b < p.extra;
    const int width = 4 * (p.base_units + (wide ? 1 : 0));
    const int col0 = 4 * (b * p.base_units + min(b, p.extra));
    const CUtensorMap* mp = maps.m[wide ? 0 : 1];
    const int tile_floats = kR * width;
    const int tile_bytes = (tile_floats * 4 + 127) / 128 * 128;
    unsigned char* base =
        reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
    float* sums = reinterpret_cast<float*>(base + (size_t)kStages * NA * tile_bytes);  // [2][2][R*w]
    uint64_t* bars = reinterpret_cast<uint64_t*>(sums + 4 * kR * kMaxWidth);
    auto tile = [&](int s, int a) {
        return reinterpret_cast<float*>(base + ((size_t)s * NA + a) * tile_bytes);
    };
    const int nchunks = (p.nrows + kR - 1) / kR;
    const uint32_t stage_tx = (uint32_t)(NA * tile_floats * 4);

    auto issue = [&](int ch) {               // producer thread only
        if (ch >= nchunks) return;
        const int s = ch % kStages;
        const uint32_t bar = smem_u32(&bars[s]);
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar),
                     "r"(stage_tx)
                     : "memory");
        for (int a = 0; a < NA; ++a) tma_load(smem_u32(tile(s, a)), &mp[a], col0, ch * kR, bar);
    };
    auto load_words = [&](int ch) {          // threads 0..R-1
        if (tid < kR) {
            const int row = ch * kR + tid;
            s_words[ch & 1][tid] =
                (ch < nchunks && row < p.nrows) ? __ldg(p.src + source_of_row<SUBSET>(p.g, row)) : 0u;
        }
    };

    if (tid == 0) {
        for (int s = 0; s < kStages; ++s)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bars[s])));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        s_abort = 0;
    }
    load_words(0);
    __syncthreads();
    if (tid == kProducer)
        for (int c = 0; c < kStages - 1; ++c) issue(c);

    // this thread's elements of a chunk tile: (row j, column c), fixed
    constexpr int kPer = kR * kMaxWidth / kThreads;
    int ej[kPer], eo[kPer];
#pragma unroll
    for (int k = 0; k < kPer; ++k) {
        const int e = tid + k * kThreads;
        ej[k] = e / width;
        eo[k] = e < tile_floats ? e : -1;      // element offset j * width + c
    }
    float short_sum = 0.0f, long_sum = 0.0f;
    const bool short_owner = tid < width;
    const bool long_owner = LONG && tid >= 128 && tid < 128 + width;
    // The column's pre-decay traces of a chunk are loaded first and then
    // added in row order: the loads overlap, only the adds are serial.
    auto consume = [&](int ch) {
        if (!short_owner && !long_owner) return;
        const int nr = min(kR, p.nrows - ch * kR);
        const float* col = sums + (ch & 1) * 2 * kR * kMaxWidth +
                           (short_owner ? tid : kR * kMaxWidth + (tid - 128));
        float acc = short_owner ? short_sum : long_sum;
        if (nr == kR) {
            float v[kR];
#pragma unroll
            for (int j = 0; j < kR; ++j) v[j] = col[j * width];
#pragma unroll
            for (int j = 0; j < kR; ++j) acc += v[j];
        } else {
            for (int j = 0; j < nr; ++j) acc += col[j * width];
        }
        if (short_owner) short_sum = acc;
        else long_sum = acc;
    };

    int ch = 0;
    for (; ch < nchunks; ++ch) {
        const int s = ch % kStages;
        if (!mbar_wait(smem_u32(&bars[s]), (uint32_t)((ch / kStages) & 1))) s_abort = 1;
        if (ch > 0) consume(ch - 1);
        float* sb = sums + (ch & 1) * 2 * kR * kMaxWidth;
        const float* tw = tile(s, 0);
        const float* tr = tile(s, 1);
        const float* tsw = tile(s, 2);
        float* tst = tile(s, A_ST);
#pragma unroll
        for (int k = 0; k < kPer; ++k) {
            const int o = eo[k];
            if (o < 0) continue;
            const uint32_t word = s_words[ch & 1][ej[k]];
            const int delay = HAS_D ? __float_as_int(tile(s, 3)[o]) : 0;
            const float spike = extract<SR>(word, delay);
            const float weight = tw[o] * (tr[o] * tsw[o]);
            const float st = tst[o] + (spike * weight * p.gcond);
            sb[o] = st;
            tst[o] = st * p.short_tau;
            if (LONG) {
                float* tlt = tile(s, A_LT);
                const float lt = tlt[o] + (spike * weight * p.gcond);
                sb[kR * kMaxWidth + o] = lt;
                tlt[o] = lt * p.long_tau;
            }
        }
        load_words(ch + 1);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (s_abort) break;
        if (tid == kProducer) {
            tma_store(&mp[A_ST], col0, ch * kR, smem_u32(tile(s, A_ST)));
            if (LONG) tma_store(&mp[A_LT], col0, ch * kR, smem_u32(tile(s, A_LT)));
            asm volatile("cp.async.bulk.commit_group;" ::: "memory");
            // the buffer about to be refilled was stored from one chunk ago
            asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory");
            issue(ch + kStages - 1);
        }
    }

    if (s_abort) {
        // loads issued for chunks ch .. ch+S-2 may still be landing: wait
        // for them (bounded) before the shared memory goes away
        if (tid == kProducer) {
            atomicExch(&g_cols_error, 1);
            for (int c = ch; c < min(nchunks, ch + kStages - 1); ++c)
                mbar_wait(smem_u32(&bars[c % kStages]), (uint32_t)((c / kStages) & 1));
            asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
        }
        __syncthreads();
        return;
    }
    if (nchunks > 0) consume(nchunks - 1);
    if (short_owner || long_owner) {
        const int c = short_owner ? tid : tid - 128;
        const int to = dest_of<SUBSET ? T_SUBSET : T_FC>(p.g, col0 + c);
        if (short_owner) p.short_cond[to] += short_sum;
        else p.long_cond[to] += long_sum;
    }
    if (tid == kProducer) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
}

size_t cols_smem_bytes(int na, int wmax) {
    const size_t tile_bytes = ((size_t)kR * wmax * 4 + 127) / 128 * 128;
    return 128 + (size_t)kStages * na * tile_bytes + (size_t)4 * kR * kMaxWidth * 4 +
           kStages * sizeof(uint64_t);
}

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

}  // namespace

struct IzColsPlan {
    ColsMaps maps;
    int nrows = 0, ncols = 0, n_cta = 0, base_units = 0, extra = 0, na = 0;
    bool has_delay = false, long_trace = false;
    size_t smem = 0;
};

std::shared_ptr<IzColsPlan> make_iz_cols_plan(int nrows, int ncols, const float* w,
                                              const float* stp_r, const float* stp_w,
                                              const int* delays, float* short_tr,
                                              float* long_tr) {
    if (nrows < 1 || ncols < 4 || ncols % 4 != 0) return nullptr;
    auto encode = encode_fn();
    if (!encode) return nullptr;
    int dev = 0, sms = 0, optin = 0;
    SG_CUDA(cudaGetDevice(&dev));
    SG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    SG_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    auto plan = std::make_shared<IzColsPlan>();
    const int q = ncols / 4;                                   // 4-column units
    plan->n_cta = std::max(std::min(sms, q), (q + kMaxWidth / 4 - 1) / (kMaxWidth / 4));
    plan->base_units = q / plan->n_cta;
    plan->extra = q % plan->n_cta;
    plan->nrows = nrows;
    plan->ncols = ncols;
    plan->has_delay = delays != nullptr;
    plan->long_trace = long_tr != nullptr;
    plan->na = 4 + (plan->has_delay ? 1 : 0) + (plan->long_trace ? 1 : 0);
    const int wmax = 4 * (plan->base_units + (plan->extra ? 1 : 0));
    plan->smem = cols_smem_bytes(plan->na, wmax);
    if (wmax > kMaxWidth || (long long)plan->smem > optin) return nullptr;
    const void* arrays[kArrays];
    int a = 0;
    arrays[a++] = w;
    arrays[a++] = stp_r;
    arrays[a++] = stp_w;
    if (plan->has_delay) arrays[a++] = delays;
    arrays[a++] = short_tr;
    if (plan->long_trace) arrays[a++] = long_tr;
    for (int band = 0; band < 2; ++band) {
        const int width = 4 * (plan->base_units + (band == 0 ? 1 : 0));
        if (width < 4 || (band == 0 && plan->extra == 0)) continue;
        for (int i = 0; i < plan->na; ++i) {
            cuuint64_t dims[2] = {(cuuint64_t)ncols, (cuuint64_t)nrows};
            cuuint64_t strides[1] = {(cuuint64_t)ncols * 4};
            cuuint32_t box[2] = {(cuuint32_t)width, (cuuint32_t)kR};
            cuuint32_t estr[2] = {1, 1};
            CUresult r = encode(&plan->maps.m[band][i], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2,
                                const_cast<void*>(arrays[i]), dims, strides, box, estr,
                                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
            if (r != CUDA_SUCCESS) return nullptr;
        }
    }
    return plan;
}

template <int SR, bool LONG, bool SUBSET>
static void launch_t(const IzColsPlan& plan, const ColsParams& p, cudaStream_t s) {
    static int configured = 0;
    if (configured < (int)plan.smem) {
        SG_CUDA(cudaFuncSetAttribute(k_iz_cols_tma<SR, LONG, SUBSET>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)plan.smem));
        configured = (int)plan.smem;
    }
    k_iz_cols_tma<SR, LONG, SUBSET><<<plan.n_cta, kThreads, plan.smem, s>>>(plan.maps, p);
    SG_LAUNCH_CHECK();
}

void launch_iz_cols_tma(const IzColsPlan& plan, const DGeom& g, int src_type, bool subset,
                        const uint32_t* src, float gcond, float short_tau, float long_tau,
                        float* short_cond, float* long_cond, cudaStream_t stream) {
    if ((src_type == S_BIT) != plan.has_delay) throw SgError("cols plan: delay array mismatch");
    ColsParams p{g, plan.nrows, plan.ncols, plan.base_units, plan.extra, src,
                 gcond, short_tau, long_tau, short_cond, long_cond};
    const bool lng = plan.long_trace;
#define SG_COLS(SRV)                                                         \
    if (lng) {                                                               \
        if (subset) launch_t<SRV, true, true>(plan, p, stream);              \
        else launch_t<SRV, true, false>(plan, p, stream);                    \
    } else {                                                                 \
        if (subset) launch_t<SRV, false, true>(plan, p, stream);             \
        else launch_t<SRV, false, false>(plan, p, stream);                   \
    }
    if (src_type == S_BIT) { SG_COLS(S_BIT) }
    else if (src_type == S_FLOAT) { SG_COLS(S_FLOAT) }
    else { SG_COLS(S_INT) }
#undef SG_COLS
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
