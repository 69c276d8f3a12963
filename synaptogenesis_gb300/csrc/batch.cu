// Batched Izhikevich instances.
//
// Hundreds of independent networks, each with the plain Izhikevich topology:
// a relay layer (FLOAT output, driven each step by value-with-probability-rate
// input) feeding an Izhikevich layer of the same shape through a wrapping
// convergent "add" connection (field x field, stride 1, offset -field/2), plus
// a recurrent fully connected "sub" connection on the Izhikevich layer with
// per-synapse delays.  Sizes, seeds and parameters differ per instance.
//
// Everything random is a counter-based function of the instance seed
// (counter_rng.h), so the same instance can be built as an ordinary network
// for the layer-by-layer path and its spike raster compared bit for bit.
//
// Per step, ONE persistent kernel advances every instance.  Its work units are
// tiles of (tile_rows x 32*tile_colblocks) destination neurons of one
// instance; CTAs take units from an atomic counter, largest first.  A unit:
//   1. stages the instance's output words of step t-1 in shared memory, and
//      the relay outputs of step t-1 (regenerated from the seed) for the
//      tile's rows plus the kernel halo;
//   2. convergent activation: per destination (one lane), the reference's
//      trace activator over k = 0..K-1 (izhikevich_attributes.cpp:228-352);
//   3. recurrent activation over the destination's non-zero synapses in
//      ascending source order.  A synapse of weight 0 keeps zero traces and
//      adds +0.0 to a non-negative sum, so skipping it is exact;
//   4. the neuron update (izhikevich_attributes.cpp:102-213) and the BIT
//      output shift, written to the other half of a ping-pong word buffer so
//      no unit reads a word another unit of the same step has written.
// Nothing in the kernel waits on another CTA: the last CTA to finish resets
// the unit counter and advances the device step counter, which the next
// launch reads.  Launches are captured in CUDA graphs.
//
// Storage.  Destinations are grouped 32 to a "group" (one image row, 32
// consecutive columns); each warp of a unit owns one group.  The recurrent
// synapses of a group are an ELL block: slot s of lane l holds the lane's
// s-th non-zero synapse {source | delay << 27, weight x short-term factors}
// in fc_in and its {short, long} traces in fc_tr, at (base + s) * 32 + l,
// padded with zero synapses to the group's largest count.  Convergent
// per-synapse data is [group][k][lane].
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <memory>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/syngen.h"
#include "counter_rng.h"
#include "cuda_check.h"
#include "iz_neuron.cuh"
#include "props.h"

namespace sg {
void set_last_error(const char* what);
}

namespace {
using namespace sg;

struct InstDev {
    int rows, cols, n, cblocks;
    int field, K;
    float a, b, c, d;
    float rate, value, gconv, gfc;
    float v0, conv_wmax, conv_factor, fc_wmax, fc_density, fc_factor;
    int fc_delays;        // delays are uniform in [0, fc_delays)
    int pad;
    unsigned long long seed;
    long long neuron_off, group_off;
};

struct Unit {
    int inst, row0, cb0, cost;
};

struct StepArgs {
    const InstDev* inst;
    const Unit* units;
    int n_units;
    int tile_rows, tile_cblocks;
    int words_cap;
    const long long* group_base;
    const int* group_slots;
    const uint2* fc_in;
    float2* fc_tr;
    const float* conv_ew;
    float2* conv_tr;
    float* v;
    float* u;
    uint32_t* words;      // [2][n_neurons]
    long long n_neurons;
    int* ctr;
    int* done;
    long long* step;
};

// Trace decays of the "add" (AMPA, NMDA) and "sub" (GABA-A, GABA-B) activators.
constexpr float kAmpaTau = 0.8f, kNmdaTau = 0.993f, kGabaaTau = 0.833f, kGababTau = 0.993f;
constexpr int kFcUnroll = 4;
constexpr int kMaxThreads = 256;

// Wrapped coordinate for x in [-n, 2n) (the field is checked against the
// layer size at creation); equal to ((x % n) + n) % n there.
__device__ __forceinline__ int wrap1(int x, int n) { return x < 0 ? x + n : (x >= n ? x - n : x); }

__device__ __forceinline__ float relay_value(const InstDev& I, long long t, int j) {
    return rng_uniform(I.seed, RNG_INPUT, (unsigned long long)t * I.n + j) < I.rate ? I.value
                                                                                    : 0.0f;
}

__global__ void __launch_bounds__(kMaxThreads) k_batch_step(StepArgs A) {
    extern __shared__ uint32_t sm[];
    __shared__ int s_unit;
    __shared__ long long s_t;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) s_t = *A.step;
    __syncthreads();
    const long long t = s_t;
    const uint32_t* words_in = A.words + (t & 1) * A.n_neurons;
    uint32_t* words_out = A.words + ((t + 1) & 1) * A.n_neurons;
    float* relay = reinterpret_cast<float*>(sm + A.words_cap);

    for (;;) {
        if (tid == 0) s_unit = atomicAdd(A.ctr, 1);
        __syncthreads();
        const int ui = s_unit;
        if (ui >= A.n_units) break;
        const Unit U = A.units[ui];
        const InstDev I = A.inst[U.inst];
        const int h = I.field / 2;
        const int tile_rows = min(A.tile_rows, I.rows - U.row0);
        const int relay_rows = tile_rows + I.field - 1;

        for (int i = tid; i < I.n; i += blockDim.x) sm[i] = words_in[I.neuron_off + i];
        for (int e = tid; e < relay_rows * I.cols; e += blockDim.x) {
            int rr = e / I.cols, cc = e - rr * I.cols;
            int fr = wrap1(U.row0 - h + rr, I.rows);
            relay[e] = t > 0 ? relay_value(I, t - 1, fr * I.cols + cc) : 0.0f;
        }
        __syncthreads();

        const int tr = warp / A.tile_cblocks, tcb = warp - tr * A.tile_cblocks;
        const int gr = U.row0 + tr, gcb = U.cb0 + tcb;
        const int col = gcb * 32 + lane;
        if (tr < tile_rows && gcb < I.cblocks && col < I.cols) {
            const long long g = I.group_off + (long long)gr * I.cblocks + gcb;

            // convergent relay -> Izhikevich, "add": AMPA (short) and NMDA (long)
            float s_sum = 0.0f, l_sum = 0.0f;
            {
                const float* ew = A.conv_ew + g * I.K * 32 + lane;
                float2* ct = A.conv_tr + g * I.K * 32 + lane;
                int k = 0;
                for (int kr = 0; kr < I.field; ++kr) {
                    const float* rrow = relay + (tr + kr) * I.cols;
                    for (int kc = 0; kc < I.field; ++kc, ++k) {
                        float spike = rrow[wrap1(col - h + kc, I.cols)];
                        float weight = __ldg(ew + k * 32);
                        float2 x = ct[k * 32];
                        float st = x.x + (spike * weight * I.gconv);
                        s_sum += st;
                        float lt = x.y + (spike * weight * I.gconv);
                        l_sum += lt;
                        ct[k * 32] = make_float2(st * kAmpaTau, lt * kNmdaTau);
                    }
                }
            }

            // recurrent fully connected, "sub": GABA-A (short) and GABA-B (long)
            float f_sum = 0.0f, fl_sum = 0.0f;
            {
                const long long base = A.group_base[g];
                const int slots = A.group_slots[g];
                const uint2* in = A.fc_in + base * 32 + lane;
                float2* trp = A.fc_tr + base * 32 + lane;
                const float gf = I.gfc;
                int s = 0;
                for (; s + kFcUnroll <= slots; s += kFcUnroll) {
                    uint2 x[kFcUnroll];
                    float2 y[kFcUnroll];
#pragma unroll
                    for (int j = 0; j < kFcUnroll; ++j) {
                        x[j] = __ldg(in + (long long)(s + j) * 32);
                        y[j] = trp[(long long)(s + j) * 32];
                    }
#pragma unroll
                    for (int j = 0; j < kFcUnroll; ++j) {
                        uint32_t word = sm[x[j].x & 0x07FFFFFFu];
                        float spike = (float)((word << (x[j].x >> 27)) >> 31);
                        float weight = __uint_as_float(x[j].y);
                        float st = y[j].x + (spike * weight * gf);
                        f_sum += st;
                        float lt = y[j].y + (spike * weight * gf);
                        fl_sum += lt;
                        trp[(long long)(s + j) * 32] = make_float2(st * kGabaaTau, lt * kGababTau);
                    }
                }
                for (; s < slots; ++s) {
                    uint2 x = __ldg(in + (long long)s * 32);
                    float2 y = trp[(long long)s * 32];
                    uint32_t word = sm[x.x & 0x07FFFFFFu];
                    float spike = (float)((word << (x.x >> 27)) >> 31);
                    float weight = __uint_as_float(x.y);
                    float st = y.x + (spike * weight * gf);
                    f_sum += st;
                    float lt = y.y + (spike * weight * gf);
                    fl_sum += lt;
                    trp[(long long)s * 32] = make_float2(st * kGabaaTau, lt * kGababTau);
                }
            }

            // neuron update; conductances were cleared by the previous update,
            // so each is 0 + this step's sum; the layer's input current is 0
            const int local = gr * I.cols + col;
            const long long nid = I.neuron_off + local;
            float voltage = A.v[nid], recovery = A.u[nid];
            iz_integrate(voltage, recovery, 0.0f + s_sum, 0.0f + l_sum, 0.0f + f_sum,
                         0.0f + fl_sum, 0.0f, 0.0f, I.a, I.b);
            unsigned int spike = voltage >= 30.0;
            words_out[nid] = (sm[local] >> 1) | (spike << 31);
            A.v[nid] = spike ? I.c : voltage;
            A.u[nid] = recovery + (spike * I.d);
        }
        __syncthreads();
    }

    if (tid == 0) {
        __threadfence();
        if (atomicAdd(A.done, 1) == (int)gridDim.x - 1) {
            *A.ctr = 0;
            *A.done = 0;
            *A.step = t + 1;
            __threadfence();
        }
    }
}

// Group of warp-global index gw: its instance, image row and column.
struct GroupPos {
    const InstDev* I;
    int gr, col;
};

__device__ __forceinline__ GroupPos group_pos(const InstDev* inst, const int* group_inst,
                                              long long gw, int lane) {
    const InstDev* I = inst + group_inst[gw];
    long long lg = gw - I->group_off;
    GroupPos p;
    p.I = I;
    p.gr = (int)(lg / I->cblocks);
    p.col = (int)(lg - (long long)p.gr * I->cblocks) * 32 + lane;
    return p;
}

// Recurrent weight of (to, from): U(0, fc_wmax) kept with probability
// fc_density, else 0.
__device__ __forceinline__ float fc_weight(const InstDev& I, unsigned long long idx) {
    if (!(rng_uniform(I.seed, RNG_FC_MASK, idx) < I.fc_density)) return 0.0f;
    return rng_uniform(I.seed, RNG_FC_WEIGHT, idx) * I.fc_wmax;
}

// Non-zero recurrent synapses per destination: the group's slot count is the
// largest of its lanes.
__global__ void k_batch_count(const InstDev* inst, const int* group_inst, long long n_groups,
                              int* group_slots, unsigned long long* total) {
    long long gw = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (gw >= n_groups) return;
    GroupPos p = group_pos(inst, group_inst, gw, lane);
    const InstDev& I = *p.I;
    int cnt = 0;
    if (p.col < I.cols) {
        unsigned long long row = (unsigned long long)(p.gr * I.cols + p.col) * I.n;
        for (int from = 0; from < I.n; ++from) cnt += fc_weight(I, row + from) != 0.0f;
    }
    int mx = __reduce_max_sync(0xFFFFFFFFu, cnt);
    unsigned long long sum = __reduce_add_sync(0xFFFFFFFFu, (unsigned)cnt);
    if (lane == 0) {
        group_slots[gw] = mx;
        atomicAdd(total, sum);
    }
}

__global__ void k_batch_fill(const InstDev* inst, const int* group_inst, long long n_groups,
                             const long long* group_base, const int* group_slots, uint2* fc_in,
                             float2* fc_tr) {
    long long gw = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (gw >= n_groups) return;
    GroupPos p = group_pos(inst, group_inst, gw, lane);
    const InstDev& I = *p.I;
    uint2* in = fc_in + group_base[gw] * 32 + lane;
    float2* tr = fc_tr + group_base[gw] * 32 + lane;
    const int slots = group_slots[gw];
    int k = 0;
    if (p.col < I.cols) {
        unsigned long long row = (unsigned long long)(p.gr * I.cols + p.col) * I.n;
        for (int from = 0; from < I.n; ++from) {
            float w = fc_weight(I, row + from);
            if (w == 0.0f) continue;
            uint32_t delay = rng_below(I.seed, RNG_FC_DELAY, row + from, (uint32_t)I.fc_delays);
            // weight x (short term R x short term w), with R = 1
            float ew = w * (1.0f * I.fc_factor);
            in[(long long)k * 32] = make_uint2((uint32_t)from | (delay << 27), __float_as_uint(ew));
            tr[(long long)k * 32] = make_float2(0.0f, 0.0f);
            ++k;
        }
    }
    for (; k < slots; ++k) {
        in[(long long)k * 32] = make_uint2(0u, 0u);
        tr[(long long)k * 32] = make_float2(0.0f, 0.0f);
    }
}

// Convergent weights U(0, conv_wmax) x (R = 1 x short term w) and zero traces;
// lanes past the row's end hold zeros.
__global__ void k_batch_conv_init(const InstDev* inst, const int* group_inst, long long n_groups,
                                  int K, float* conv_ew, float2* conv_tr) {
    long long gw = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (gw >= n_groups) return;
    GroupPos p = group_pos(inst, group_inst, gw, lane);
    const InstDev& I = *p.I;
    for (int k = 0; k < I.K; ++k) {
        float ew = 0.0f;
        if (p.col < I.cols) {
            unsigned long long to = (unsigned long long)(p.gr * I.cols + p.col);
            float w = rng_uniform(I.seed, RNG_CONV_WEIGHT, to * I.K + k) * I.conv_wmax;
            ew = w * (1.0f * I.conv_factor);
        }
        conv_ew[(gw * K + k) * 32 + lane] = ew;
        conv_tr[(gw * K + k) * 32 + lane] = make_float2(0.0f, 0.0f);
    }
}

__global__ void k_batch_neuron_init(const InstDev* inst, int n_inst, float* v, float* u) {
    int i = blockIdx.y;
    if (i >= n_inst) return;
    const InstDev& I = inst[i];
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < I.n; j += gridDim.x * blockDim.x) {
        v[I.neuron_off + j] = I.v0;
        u[I.neuron_off + j] = I.b * I.v0;
    }
}

template <class T>
T* dalloc(size_t n, std::vector<void*>& owned) {
    void* p = nullptr;
    SG_CUDA(cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)));
    owned.push_back(p);
    return static_cast<T*>(p);
}

struct TuneResult {
    int tile_rows, tile_cblocks;
    float ms;
};

class Batch {
  public:
    Batch(const SgBatchInstance* spec, int count, int tile_rows, int tile_cblocks) {
        if (!spec || count <= 0) throw SgError("batch: no instances");
        validate(spec, count);
        SG_CUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
        SG_CUDA(cudaGetDevice(&device_));
        SG_CUDA(cudaDeviceGetAttribute(&num_sms_, cudaDevAttrMultiProcessorCount, device_));
        SG_CUDA(cudaDeviceGetAttribute(&smem_optin_, cudaDevAttrMaxSharedMemoryPerBlockOptin,
                                       device_));
        layout(spec, count);
        generate();
        // counters, words and neurons start defined before the autotuner's
        // real steps (device allocations are not cleared)
        reset();
        if (tile_rows > 0 && tile_cblocks > 0) {
            set_tile(tile_rows, tile_cblocks);
        } else {
            autotune();
        }
        reset();
    }

    ~Batch() {
        if (graph_) cudaGraphExecDestroy(graph_);
        for (void* p : owned_) cudaFree(p);
        if (stream_) cudaStreamDestroy(stream_);
    }

    void step(long long n) {
        while (n >= kGraphSteps) {
            if (!graph_) capture();
            SG_CUDA(cudaGraphLaunch(graph_, stream_));
            n -= kGraphSteps;
            steps_ += kGraphSteps;
            launches_ += kGraphSteps;
        }
        for (; n > 0; --n) {
            launch();
            ++steps_;
            ++launches_;
        }
    }

    void read(int i, const std::string& key, void* out, long long count) {
        if (i < 0 || i >= (int)inst_.size()) throw SgError("batch: instance out of range");
        const InstDev& I = inst_[i];
        if (count < I.n) throw SgError("batch: output buffer smaller than the layer");
        SG_CUDA(cudaStreamSynchronize(stream_));
        const void* src;
        if (key == "voltage") src = v_ + I.neuron_off;
        else if (key == "recovery") src = u_ + I.neuron_off;
        else if (key == "output") src = words_ + (steps_ & 1) * n_neurons_ + I.neuron_off;
        else throw SgError("batch: unknown key " + key);
        SG_CUDA(cudaMemcpy(out, src, (size_t)I.n * 4, cudaMemcpyDeviceToHost));
    }

    Props* report() const {
        auto* r = new Props();
        r->set("instances", std::to_string(inst_.size()));
        r->set("neurons", std::to_string(n_neurons_));
        r->set("groups", std::to_string(n_groups_));
        r->set("slot rows", std::to_string(slot_rows_));
        r->set("fc synapses", std::to_string(fc_synapses_));
        r->set("fc slots", std::to_string(slot_rows_ * 32));
        r->set("conv synapses", std::to_string(conv_synapses_));
        r->set("device bytes", std::to_string(device_bytes_));
        r->set("step bytes", std::to_string(step_bytes()));
        r->set("tile rows", std::to_string(tile_rows_));
        r->set("tile colblocks", std::to_string(tile_cblocks_));
        r->set("units", std::to_string(units_h_.size()));
        r->set("grid", std::to_string(grid_));
        r->set("threads", std::to_string(threads_));
        r->set("shared bytes", std::to_string(smem_));
        r->set("steps", std::to_string(steps_));
        r->set("kernel launches", std::to_string(launches_));
        r->set("graph steps", std::to_string(kGraphSteps));
        for (const TuneResult& t : tuning_) {
            Props c;
            c.set("tile rows", std::to_string(t.tile_rows));
            c.set("tile colblocks", std::to_string(t.tile_cblocks));
            c.set("ms per step", std::to_string(t.ms));
            r->add_to_child_array("autotune", c);
        }
        return r;
    }

    cudaStream_t stream() const { return stream_; }

  private:
    static constexpr int kGraphSteps = 32;

    static void validate(const SgBatchInstance* s, int count) {
        for (int i = 0; i < count; ++i) {
            const SgBatchInstance& x = s[i];
            std::string who = "batch: instance " + std::to_string(i) + ": ";
            if (x.rows < 1 || x.cols < 1) throw SgError(who + "empty layer");
            if ((long long)x.rows * x.cols > (1 << 24)) throw SgError(who + "layer too large");
            if (x.conv_field < 1 || x.conv_field / 2 >= x.rows || x.conv_field / 2 >= x.cols)
                throw SgError(who + "convergent field must satisfy 1 <= field and field/2 < rows, cols");
            if (x.fc_max_delay < 0 || x.fc_max_delay > 31)
                throw SgError(who + "delays must lie in 0..31");
            if (!(x.input_rate >= 0.0f && x.input_rate <= 1.0f))
                throw SgError(who + "input rate must lie in [0, 1]");
            if (!(x.fc_density >= 0.0f && x.fc_density <= 1.0f))
                throw SgError(who + "density must lie in [0, 1]");
        }
    }

    void layout(const SgBatchInstance* spec, int count) {
        long long noff = 0, goff = 0;
        for (int i = 0; i < count; ++i) {
            const SgBatchInstance& s = spec[i];
            InstDev I{};
            I.rows = s.rows;
            I.cols = s.cols;
            I.n = s.rows * s.cols;
            I.cblocks = (s.cols + 31) / 32;
            I.field = s.conv_field;
            I.K = s.conv_field * s.conv_field;
            I.a = s.a; I.b = s.b; I.c = s.c; I.d = s.d;
            I.rate = s.input_rate;
            I.value = s.input_value;
            I.gconv = s.conv_conductance;
            I.gfc = s.fc_conductance;
            I.v0 = s.v0;
            I.conv_wmax = s.conv_wmax;
            I.conv_factor = s.conv_stp_w;
            I.fc_wmax = s.fc_wmax;
            I.fc_density = s.fc_density;
            I.fc_factor = s.fc_stp_w;
            I.fc_delays = s.fc_max_delay + 1;
            I.seed = s.seed;
            I.neuron_off = noff;
            I.group_off = goff;
            noff += I.n;
            goff += (long long)I.rows * I.cblocks;
            max_n_ = std::max(max_n_, I.n);
            max_cols_ = std::max(max_cols_, I.cols);
            max_field_ = std::max(max_field_, I.field);
            max_cblocks_ = std::max(max_cblocks_, I.cblocks);
            max_rows_ = std::max(max_rows_, I.rows);
            if (i > 0 && I.K != inst_[0].K) throw SgError("batch: every instance needs the same field");
            conv_synapses_ += (long long)I.n * I.K;
            inst_.push_back(I);
        }
        n_neurons_ = noff;
        n_groups_ = goff;
        K_ = inst_[0].K;
        group_inst_h_.resize(n_groups_);
        for (size_t i = 0; i < inst_.size(); ++i)
            for (long long g = 0; g < (long long)inst_[i].rows * inst_[i].cblocks; ++g)
                group_inst_h_[inst_[i].group_off + g] = (int)i;
    }

    void generate() {
        d_inst_ = dalloc<InstDev>(inst_.size(), owned_);
        d_group_inst_ = dalloc<int>(n_groups_, owned_);
        d_group_slots_ = dalloc<int>(n_groups_, owned_);
        d_group_base_ = dalloc<long long>(n_groups_, owned_);
        d_counters_ = dalloc<long long>(4, owned_);
        v_ = dalloc<float>(n_neurons_, owned_);
        u_ = dalloc<float>(n_neurons_, owned_);
        words_ = dalloc<uint32_t>(2 * n_neurons_, owned_);
        conv_ew_ = dalloc<float>(n_groups_ * K_ * 32, owned_);
        conv_tr_ = dalloc<float2>(n_groups_ * K_ * 32, owned_);
        // Every upload goes through stream_ (non-blocking): a plain cudaMemcpy
        // from pageable memory may return before its DMA lands and is not
        // ordered with this stream's kernels.
        SG_CUDA(cudaMemcpyAsync(d_inst_, inst_.data(), inst_.size() * sizeof(InstDev),
                                cudaMemcpyHostToDevice, stream_));
        SG_CUDA(cudaMemcpyAsync(d_group_inst_, group_inst_h_.data(), n_groups_ * sizeof(int),
                                cudaMemcpyHostToDevice, stream_));
        unsigned long long* total = reinterpret_cast<unsigned long long*>(d_counters_ + 3);
        SG_CUDA(cudaMemsetAsync(total, 0, sizeof(unsigned long long), stream_));
        unsigned blocks = blocks_for(n_groups_ * 32, 256);
        k_batch_count<<<blocks, 256, 0, stream_>>>(d_inst_, d_group_inst_, n_groups_,
                                                   d_group_slots_, total);
        SG_LAUNCH_CHECK();
        group_slots_h_.resize(n_groups_);
        SG_CUDA(cudaMemcpyAsync(group_slots_h_.data(), d_group_slots_, n_groups_ * sizeof(int),
                                cudaMemcpyDeviceToHost, stream_));
        unsigned long long nz = 0;
        SG_CUDA(cudaMemcpyAsync(&nz, total, sizeof(nz), cudaMemcpyDeviceToHost, stream_));
        SG_CUDA(cudaStreamSynchronize(stream_));
        fc_synapses_ = (long long)nz;
        std::vector<long long> base(n_groups_);
        long long acc = 0;
        for (long long g = 0; g < n_groups_; ++g) {
            base[g] = acc;
            acc += group_slots_h_[g];
        }
        slot_rows_ = acc;
        SG_CUDA(cudaMemcpyAsync(d_group_base_, base.data(), n_groups_ * sizeof(long long),
                                cudaMemcpyHostToDevice, stream_));
        fc_in_ = dalloc<uint2>(slot_rows_ * 32, owned_);
        fc_tr_ = dalloc<float2>(slot_rows_ * 32, owned_);
        k_batch_fill<<<blocks, 256, 0, stream_>>>(d_inst_, d_group_inst_, n_groups_, d_group_base_,
                                                  d_group_slots_, fc_in_, fc_tr_);
        SG_LAUNCH_CHECK();
        k_batch_conv_init<<<blocks, 256, 0, stream_>>>(d_inst_, d_group_inst_, n_groups_, K_,
                                                       conv_ew_, conv_tr_);
        SG_LAUNCH_CHECK();
        SG_CUDA(cudaStreamSynchronize(stream_));
        device_bytes_ = 0;
        device_bytes_ += inst_.size() * sizeof(InstDev) + n_groups_ * (4 + 4 + 8) + 32;
        device_bytes_ += n_neurons_ * 16;
        device_bytes_ += n_groups_ * K_ * 32 * 12;
        device_bytes_ += slot_rows_ * 32 * 16;
    }

    // Bytes one step must move: recurrent slots (read 16, write 8), convergent
    // synapses (read 12, write 8) and neurons (voltage, recovery read and
    // written, output word read and written).
    long long step_bytes() const {
        return slot_rows_ * 32 * 24 + n_groups_ * K_ * 32 * 20 + n_neurons_ * 24;
    }

    // Trace state, neurons, output words and counters back to their initial
    // values (after autotuning, which runs real steps).
    void reset() {
        SG_CUDA(cudaMemsetAsync(fc_tr_, 0, slot_rows_ * 32 * sizeof(float2), stream_));
        SG_CUDA(cudaMemsetAsync(conv_tr_, 0, n_groups_ * K_ * 32 * sizeof(float2), stream_));
        SG_CUDA(cudaMemsetAsync(words_, 0, 2 * n_neurons_ * sizeof(uint32_t), stream_));
        SG_CUDA(cudaMemsetAsync(d_counters_, 0, 3 * sizeof(long long), stream_));
        dim3 grid(std::max(1, std::min(64, (max_n_ + 255) / 256)), (unsigned)inst_.size());
        k_batch_neuron_init<<<grid, 256, 0, stream_>>>(d_inst_, (int)inst_.size(), v_, u_);
        SG_LAUNCH_CHECK();
        SG_CUDA(cudaStreamSynchronize(stream_));
        steps_ = 0;
        launches_ = 0;
    }

    void set_tile(int tile_rows, int tile_cblocks) {
        if (tile_rows < 1 || tile_cblocks < 1 || tile_rows * tile_cblocks * 32 > kMaxThreads)
            throw SgError("batch: tile must have 1..8 warps");
        tile_rows_ = tile_rows;
        tile_cblocks_ = tile_cblocks;
        threads_ = tile_rows * tile_cblocks * 32;
        words_cap_ = (max_n_ + 3) / 4 * 4;
        smem_ = (size_t)(words_cap_ + (tile_rows + max_field_ - 1) * max_cols_) * 4;
        if ((int)smem_ > smem_optin_) throw SgError("batch: instance too large for shared memory");
        SG_CUDA(cudaFuncSetAttribute(k_batch_step, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem_));
        units_h_.clear();
        for (size_t i = 0; i < inst_.size(); ++i) {
            const InstDev& I = inst_[i];
            for (int r0 = 0; r0 < I.rows; r0 += tile_rows)
                for (int c0 = 0; c0 < I.cblocks; c0 += tile_cblocks) {
                    long long cost = 0;
                    for (int r = r0; r < std::min(I.rows, r0 + tile_rows); ++r)
                        for (int c = c0; c < std::min(I.cblocks, c0 + tile_cblocks); ++c)
                            cost += group_slots_h_[I.group_off + (long long)r * I.cblocks + c] + I.K;
                    cost += I.n / 32 + 1;
                    units_h_.push_back(Unit{(int)i, r0, c0, (int)std::min<long long>(cost, 1 << 30)});
                }
        }
        std::stable_sort(units_h_.begin(), units_h_.end(),
                         [](const Unit& a, const Unit& b) { return a.cost > b.cost; });
        if (!d_units_ || units_h_.size() > units_cap_) {
            units_cap_ = std::max(units_h_.size(), (size_t)(n_groups_ + 1));
            d_units_ = dalloc<Unit>(units_cap_, owned_);
        }
        SG_CUDA(cudaMemcpyAsync(d_units_, units_h_.data(), units_h_.size() * sizeof(Unit),
                                cudaMemcpyHostToDevice, stream_));
        int per_sm = 0;
        SG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch_step, threads_,
                                                              smem_));
        if (per_sm < 1) throw SgError("batch: step kernel does not fit on an SM");
        grid_ = (int)std::min<long long>((long long)units_h_.size(), (long long)per_sm * num_sms_);
        if (graph_) {
            cudaGraphExecDestroy(graph_);
            graph_ = nullptr;
        }
    }

    StepArgs args() const {
        StepArgs a;
        a.inst = d_inst_;
        a.units = d_units_;
        a.n_units = (int)units_h_.size();
        a.tile_rows = tile_rows_;
        a.tile_cblocks = tile_cblocks_;
        a.words_cap = words_cap_;
        a.group_base = d_group_base_;
        a.group_slots = d_group_slots_;
        a.fc_in = fc_in_;
        a.fc_tr = fc_tr_;
        a.conv_ew = conv_ew_;
        a.conv_tr = conv_tr_;
        a.v = v_;
        a.u = u_;
        a.words = words_;
        a.n_neurons = n_neurons_;
        a.ctr = reinterpret_cast<int*>(d_counters_);
        a.done = reinterpret_cast<int*>(d_counters_ + 1);
        a.step = d_counters_ + 2;
        return a;
    }

    void launch() {
        k_batch_step<<<grid_, threads_, smem_, stream_>>>(args());
        SG_LAUNCH_CHECK();
    }

    void capture() {
        cudaGraph_t g;
        SG_CUDA(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
        for (int i = 0; i < kGraphSteps; ++i) k_batch_step<<<grid_, threads_, smem_, stream_>>>(args());
        SG_CUDA(cudaStreamEndCapture(stream_, &g));
        cudaError_t e = cudaGraphInstantiate(&graph_, g, 0);
        cudaGraphDestroy(g);
        SG_CUDA(e);
    }

    // Tile shapes with 4 or 8 warps, each timed over a few real steps; the
    // fastest is kept.  The state is reset afterwards.
    void autotune() {
        std::vector<std::pair<int, int>> cands;
        for (int warps : {8, 4})
            for (int tc = 1; tc <= warps; tc *= 2) {
                int tr = warps / tc;
                if (tc > max_cblocks_ && tc > 1) continue;
                if (tr > max_rows_ && tr > 1) continue;
                cands.push_back({tr, tc});
            }
        cudaEvent_t e0, e1;
        SG_CUDA(cudaEventCreate(&e0));
        SG_CUDA(cudaEventCreate(&e1));
        float best = 1e30f;
        std::pair<int, int> pick = cands.front();
        for (auto& c : cands) {
            set_tile(c.first, c.second);
            launch();
            SG_CUDA(cudaEventRecord(e0, stream_));
            const int reps = 3;
            for (int i = 0; i < reps; ++i) launch();
            SG_CUDA(cudaEventRecord(e1, stream_));
            SG_CUDA(cudaEventSynchronize(e1));
            float ms = 0.0f;
            SG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            ms /= reps;
            tuning_.push_back(TuneResult{c.first, c.second, ms});
            if (ms < best) {
                best = ms;
                pick = c;
            }
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        set_tile(pick.first, pick.second);
    }

    std::vector<InstDev> inst_;
    std::vector<int> group_inst_h_, group_slots_h_;
    std::vector<Unit> units_h_;
    std::vector<TuneResult> tuning_;
    std::vector<void*> owned_;
    long long n_neurons_ = 0, n_groups_ = 0, slot_rows_ = 0, fc_synapses_ = 0;
    long long conv_synapses_ = 0, device_bytes_ = 0, steps_ = 0, launches_ = 0;
    int max_n_ = 0, max_cols_ = 0, max_rows_ = 0, max_field_ = 0, max_cblocks_ = 0, K_ = 0;
    int tile_rows_ = 0, tile_cblocks_ = 0, threads_ = 0, grid_ = 0, words_cap_ = 0;
    size_t smem_ = 0, units_cap_ = 0;
    int device_ = 0, num_sms_ = 0, smem_optin_ = 0;
    cudaStream_t stream_ = nullptr;
    cudaGraphExec_t graph_ = nullptr;
    InstDev* d_inst_ = nullptr;
    int* d_group_inst_ = nullptr;
    int* d_group_slots_ = nullptr;
    long long* d_group_base_ = nullptr;
    long long* d_counters_ = nullptr;   // unit counter, done counter, step, synapse total
    Unit* d_units_ = nullptr;
    float *v_ = nullptr, *u_ = nullptr;
    uint32_t* words_ = nullptr;
    float* conv_ew_ = nullptr;
    float2* conv_tr_ = nullptr;
    uint2* fc_in_ = nullptr;
    float2* fc_tr_ = nullptr;
};

}  // namespace

extern "C" {

SG_BATCH sg_batch_create(const SgBatchInstance* instances, int count, int tile_rows,
                         int tile_colblocks) {
    try {
        return new Batch(instances, count, tile_rows, tile_colblocks);
    } catch (const std::exception& e) {
        sg::set_last_error(e.what());
    } catch (...) {
        sg::set_last_error("unknown error");
    }
    return nullptr;
}

int sg_batch_step(SG_BATCH b, long long steps) {
    if (!b || steps < 0) return SG_BATCH_EINVAL;
    try {
        static_cast<Batch*>(b)->step(steps);
        return 0;
    } catch (const std::exception& e) {
        sg::set_last_error(e.what());
    }
    return SG_BATCH_ECUDA;
}

int sg_batch_read(SG_BATCH b, int instance, const char* key, void* out, long long count) {
    if (!b || !key || !out) return SG_BATCH_EINVAL;
    try {
        static_cast<Batch*>(b)->read(instance, key, out, count);
        return 0;
    } catch (const std::exception& e) {
        sg::set_last_error(e.what());
    }
    return SG_BATCH_EINVAL;
}

PROPS sg_batch_report(SG_BATCH b) {
    if (!b) return nullptr;
    try {
        return static_cast<Batch*>(b)->report();
    } catch (const std::exception& e) {
        sg::set_last_error(e.what());
    }
    return nullptr;
}

void* sg_batch_stream(SG_BATCH b) { return b ? (void*)static_cast<Batch*>(b)->stream() : nullptr; }

int sg_batch_synchronize(SG_BATCH b) {
    if (!b) return SG_BATCH_EINVAL;
    return cudaStreamSynchronize(static_cast<Batch*>(b)->stream()) == cudaSuccess ? 0
                                                                                  : SG_BATCH_ECUDA;
}

void sg_batch_destroy(SG_BATCH b) {
    try {
        delete static_cast<Batch*>(b);
    } catch (...) {
    }
}

}  // extern "C"
