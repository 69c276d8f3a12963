#include "engine.h"

#include <algorithm>
#include <chrono>
#include <cstring>
#include <mutex>

#include "cuda_check.h"
#include "models.h"
#include "weight_init.h"

namespace sg {

std::atomic<bool> Engine::interrupt_flag{false};
std::atomic<bool> Engine::running{false};

cudaStream_t engine_stream() {
    static cudaStream_t s = [] {
        cudaStream_t t;
        SG_CUDA(cudaStreamCreateWithFlags(&t, cudaStreamNonBlocking));
        return t;
    }();
    return s;
}

// ---------------------------------------------------------------------------
// Input-register initialisation kernels (engine/kernel/kernel.cpp:14-158).
// Noise uses a seeded counter-based generator (the reference's is unseedable).
// ---------------------------------------------------------------------------
__global__ void k_set_value(float* p, int n, float v, int overwrite) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = overwrite ? v : p[i] + v;
}

__device__ __forceinline__ unsigned long long mix64(unsigned long long x) {
    x += 0x9E3779B97F4A7C15ULL;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
    return x ^ (x >> 31);
}

__device__ __forceinline__ float uniform01(unsigned long long seed, long step, int i, int draw) {
    unsigned long long h = mix64(seed ^ mix64((unsigned long long)step * 0x100000001B3ULL + draw) ^
                                 ((unsigned long long)i << 20));
    return ((h >> 40) + 1) * (1.0f / 16777217.0f);   // (0, 1)
}

// kind 0 uniform(a, b), 1 normal(a=mean, b=std), 2 poisson(rate a -> value b)
__global__ void k_noise(float* p, int n, int kind, float a, float b, int overwrite,
                        unsigned long long seed, long step) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float u = uniform01(seed, step, i, 0);
    float v;
    if (kind == 0) {
        v = u * (b - a) + a;
    } else if (kind == 1) {
        float u2 = uniform01(seed, step, i, 1);
        v = sqrtf(-2.0f * logf(u)) * cospif(2.0f * u2) * b + a;
    } else {
        if (overwrite) { p[i] = u < a ? b : 0.0f; return; }
        if (u < a) p[i] += b;
        return;
    }
    p[i] = overwrite ? v : p[i] + v;
}

void Engine::build_modules() {
    modules_.clear();
    layer_io_.assign(net_->layers.size(), 0);
    if (!env_) return;
    for (Props* mp : env_->config.child_array("modules")) {
        if (mp->get_bool("skip", false)) continue;
        std::string type = mp->get("type");
        if (type != "callback")
            throw SgError("Unrecognized module: " + type + "! (only \"callback\" modules are supported)");
        Module m;
        m.clear = mp->get_bool("clear", false);
        m.start_delay = mp->get_int("delay", 0);
        m.cutoff = mp->get_int("cutoff", 0);
        m.rate = mp->get_int("rate", 1);
        if (m.start_delay < 0 || m.cutoff < 0 || m.rate < 1)
            throw SgError("Error in Module : callback: invalid delay/cutoff/rate");
        for (Props* lp : mp->child_array("layers")) {
            ModLayer ml;
            ml.layer = lp->has("structure") ? net_->layer(lp->get("structure"), lp->get("layer"))
                                            : net_->find_layer(lp->get("layer"));
            ml.input = lp->get_bool("input", false);
            ml.output = lp->get_bool("output", false);
            for (auto& k : lp->array("input keys"))
                if (k != "input") throw SgError("auxiliary input key \"" + k + "\" is not supported");
            for (auto& k : lp->array("output keys"))
                if (k != "output") throw SgError("auxiliary output key \"" + k + "\" is not supported");
            if (!lp->array("input keys").empty()) ml.input = true;
            if (!lp->array("output keys").empty()) ml.output = true;
            if (!ml.input && !ml.output) throw SgError("callback module requires specified IO type!");
            if (!lp->has("function"))
                throw SgError("Unspecified callback function for layer " + ml.layer->str() + " in CallbackModule!");
            if (!lp->has("id"))
                throw SgError("Unspecified callback id for layer " + ml.layer->str() + " in CallbackModule!");
            ml.fn = Callbacks::find(Callbacks::get().io, lp->get("function"), "io");
            ml.id = lp->get_int("id", 0);
            layer_io_[ml.layer->index] |= (ml.input ? 1 : 0) | (ml.output ? 2 : 0);
            m.layers.push_back(ml);
        }
        if (!m.layers.empty()) modules_.push_back(m);
    }
}

void Engine::enqueue_step(int step, bool last, bool learning) {
    cudaStream_t s = engine_stream();
    StepCtx ctx{s, last};
    // 1. input registers
    for (auto& lp : net_->layers) {
        Layer* l = lp.get();
        LayerState* ls = state_->layer_state(l);
        float* in = ls->input->df();
        bool is_input = (layer_io_[l->index] & 1) != 0;
        if (is_input) {
            size_t k = std::find(input_layers_.begin(), input_layers_.end(), l) - input_layers_.begin();
            if (in_dirty_[k]) {
                SG_CUDA(cudaMemcpyAsync(in_staging_[k], in_pinned_[k], l->size * 4,
                                        cudaMemcpyHostToDevice, s));
                in_dirty_[k] = 0;
            }
            SG_CUDA(cudaMemcpyAsync(in, in_staging_[k], l->size * 4, cudaMemcpyDeviceToDevice, s));
        }
        Props* init = l->config.child("init config");
        if (init) {
            std::string t = init->get("type", "normal");
            int ow = is_input ? 0 : 1;
            unsigned long long seed = init->has("seed") ? std::stoull(init->get("seed"))
                                                        : (global_seed() ^ (0xA5A5ULL * (l->index + 1)));
            unsigned blocks = blocks_for(l->size, 256);
            if (t == "flat") {
                k_set_value<<<blocks, 256, 0, s>>>(in, l->size, init->get_float("value", 1.0f), ow);
            } else if (t == "uniform") {
                k_noise<<<blocks, 256, 0, s>>>(in, l->size, 0, init->get_float("min", 0.0f),
                                               init->get_float("max", 1.0f), ow, seed, step);
            } else if (t == "normal") {
                k_noise<<<blocks, 256, 0, s>>>(in, l->size, 1, init->get_float("mean", 1.0f),
                                               init->get_float("std dev", 0.1f), ow, seed, step);
            } else if (t == "poisson") {
                if (init->get_bool("random", false))
                    throw SgError("random per-neuron Poisson rates are not supported");
                k_noise<<<blocks, 256, 0, s>>>(in, l->size, 2, 0.001f * init->get_float("rate", 1.0f),
                                               init->get_float("value", 20.0f), ow, seed, step);
            } else {
                throw SgError("Error building cluster node for " + l->str() + ":\n  Unrecognized init type: " + t);
            }
            SG_LAUNCH_CHECK();
            ++launches_;
        } else if (!is_input) {
            SG_CUDA(cudaMemsetAsync(in, 0, (size_t)l->size * 4, s));
        }
    }
    // 2. synaptic input
    for (auto& lp : net_->layers) {
        const Model* m = find_model(lp->model);
        for (Connection* c : lp->inputs) {
            m->activate(*state_, *state_->conn_state(c), ctx);
            ++launches_;
        }
    }
    // 3. neuron updates
    for (auto& lp : net_->layers) {
        find_model(lp->model)->update(*state_, *state_->layer_state(lp.get()), ctx);
        ++launches_;
    }
    // 4. plasticity
    if (learning)
        for (auto& lp : net_->layers) {
            const Model* m = find_model(lp->model);
            for (Connection* c : lp->inputs)
                if (c->plastic && m->learns(*c)) {
                    m->learn(*state_, *state_->conn_state(c), ctx);
                    ++launches_;
                }
        }
}

Props* Engine::run(const Props& args) {
    bool expected = false;
    if (!running.compare_exchange_strong(expected, true))
        throw SgError("Cannot run more than one engine at once!");
    struct Guard {
        Engine* e;
        std::vector<void*> pinned;
        std::vector<void*> dev;
        ~Guard() {
            for (void* p : pinned) cudaFreeHost(p);
            for (void* p : dev) cudaFree(p);
            Engine::running = false;
            Engine::interrupt_flag = false;
        }
    } guard{this, {}, {}};

    if (args.has("devices")) {
        int n = 0;
        cudaGetDeviceCount(&n);
        int d = args.get_int("devices", 0);
        if (d != 0 && d != n) throw SgError("Failed to extract devices from Engine args!");
    }
    const bool verbose = args.get_bool("verbose", false);
    const bool learning = args.get_bool("learning flag", true);
    const bool suppress = args.get_bool("suppress output", false);
    const int env_rate = std::max(1, args.get_int("environment rate", 1));
    long iterations = args.get_int("iterations", 0);

    build_modules();
    cudaStream_t s = engine_stream();
    state_->to_device(s);

    input_layers_.clear();
    output_layers_.clear();
    for (auto& lp : net_->layers) {
        if (layer_io_[lp->index] & 1) input_layers_.push_back(lp.get());
        if (layer_io_[lp->index] & 2) output_layers_.push_back(lp.get());
    }
    in_pinned_.clear(); in_staging_.clear(); out_pinned_.clear();
    in_dirty_.assign(input_layers_.size(), 0);
    for (Layer* l : input_layers_) {
        void* h; void* d;
        SG_CUDA(cudaMallocHost(&h, (size_t)l->size * 4));
        std::memset(h, 0, (size_t)l->size * 4);
        guard.pinned.push_back(h);
        SG_CUDA(cudaMalloc(&d, (size_t)l->size * 4));
        SG_CUDA(cudaMemsetAsync(d, 0, (size_t)l->size * 4, s));
        guard.dev.push_back(d);
        in_pinned_.push_back((float*)h);
        in_staging_.push_back((float*)d);
    }
    for (Layer* l : output_layers_) {
        void* h;
        SG_CUDA(cudaMallocHost(&h, (size_t)l->size * 4));
        guard.pinned.push_back(h);
        out_pinned_.push_back((uint32_t*)h);
    }
    auto index_of = [](const std::vector<Layer*>& v, Layer* l) {
        return (size_t)(std::find(v.begin(), v.end(), l) - v.begin());
    };

    cudaEvent_t ev0, ev1;
    SG_CUDA(cudaEventCreate(&ev0));
    SG_CUDA(cudaEventCreate(&ev1));
    SG_CUDA(cudaStreamSynchronize(s));
    auto t0 = std::chrono::steady_clock::now();
    SG_CUDA(cudaEventRecord(ev0, s));
    launches_ = 0;
    long i = 0;
    for (; iterations == 0 || i < iterations; ++i) {
        // feed input (module.cpp:86-97): the callback writes the pinned
        // buffer; it must not be overwritten while a copy from it is queued.
        bool any_input_cb = false;
        for (auto& m : modules_) {
            if (m.start_delay > 0) continue;
            bool active = (m.cutoff == 0 || m.curr < m.cutoff) && m.curr % m.rate == 0;
            bool cut = m.cutoff != 0 && m.curr == m.cutoff;
            for (auto& ml : m.layers) {
                if (!ml.input) continue;
                if (!any_input_cb) { SG_CUDA(cudaStreamSynchronize(s)); any_input_cb = true; }
                size_t k = index_of(input_layers_, ml.layer);
                if (active) {
                    if (m.clear) std::memset(in_pinned_[k], 0, (size_t)ml.layer->size * 4);
                    ml.fn(ml.id, ml.layer->size, in_pinned_[k]);
                    in_dirty_[k] = 1;
                } else if (cut) {
                    std::memset(in_pinned_[k], 0, (size_t)ml.layer->size * 4);
                    in_dirty_[k] = 1;
                }
            }
        }
        bool last = iterations != 0 && i == iterations - 1;
        enqueue_step((int)i, last, learning);
        // report output (module.cpp:99-104)
        if (i % env_rate == 0 && !suppress && !output_layers_.empty()) {
            for (size_t k = 0; k < output_layers_.size(); ++k)
                SG_CUDA(cudaMemcpyAsync(out_pinned_[k], state_->dev_output(output_layers_[k], 0),
                                        (size_t)output_layers_[k]->size * 4,
                                        cudaMemcpyDeviceToHost, s));
            SG_CUDA(cudaStreamSynchronize(s));
            for (auto& m : modules_) {
                if (m.start_delay > 0 || !((m.cutoff == 0 || m.curr < m.cutoff) && m.curr % m.rate == 0))
                    continue;
                for (auto& ml : m.layers)
                    if (ml.output)
                        ml.fn(ml.id, ml.layer->size, out_pinned_[index_of(output_layers_, ml.layer)]);
            }
        }
        for (auto& m : modules_) {
            if (m.start_delay > 0) { --m.start_delay; continue; }
            if (m.cutoff == 0 || m.curr <= m.cutoff) ++m.curr;
        }
        if (interrupt_flag) { ++i; break; }
    }
    SG_CUDA(cudaEventRecord(ev1, s));
    SG_CUDA(cudaEventSynchronize(ev1));
    auto t1 = std::chrono::steady_clock::now();
    float dev_ms = 0.0f;
    SG_CUDA(cudaEventElapsedTime(&dev_ms, ev0, ev1));
    cudaEventDestroy(ev0);
    cudaEventDestroy(ev1);
    SG_CUDA(cudaGetLastError());
    state_->mark_device_newer();

    double total = std::chrono::duration<double>(t1 - t0).count();
    auto* r = new Props();
    r->set("iterations", std::to_string(i));
    r->set("total time", std::to_string((float)total));
    r->set("average time", std::to_string((float)(i ? total / i : 0.0)));
    r->set("fps", std::to_string((float)(total > 0 ? i / total : 0.0)));
    r->set("network bytes", std::to_string(state_->device_bytes()));
    r->set("state buffer bytes", "0");
    size_t eb = 0;
    for (Layer* l : input_layers_) eb += (size_t)l->size * 4;
    for (Layer* l : output_layers_) eb += (size_t)l->size * 4;
    r->set("engine buffer bytes", std::to_string(eb));
    r->set("device time", std::to_string(dev_ms / 1000.0f));
    r->set("kernel launches", std::to_string(launches_));
    r->set_child("args", args);
    r->set("interrupted", interrupt_flag ? "true" : "false");
    if (verbose)
        printf("Ran %ld iterations in %fs (device %fs)\n", i, total, dev_ms / 1000.0f);
    return r;
}

}  // namespace sg
