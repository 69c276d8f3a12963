#include "counter_rng.h"
#include "engine.h"
#include "iz_cols_tma.cuh"

#include <algorithm>
#include <cstring>

#include "cuda_check.h"
#include "models.h"
#include "weight_init.h"

namespace sg {

std::atomic<bool> Engine::interrupt_flag{false};
std::atomic<bool> Engine::running{false};

// The step's stream has the highest priority and the learning stream the
// lowest, so that CTAs of the next step's activations are scheduled ahead of
// the remaining learning CTAs as SMs free up.
cudaStream_t engine_stream() {
    static cudaStream_t s = [] {
        int least = 0, greatest = 0;
        SG_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        cudaStream_t t;
        SG_CUDA(cudaStreamCreateWithPriority(&t, cudaStreamNonBlocking, greatest));
        return t;
    }();
    return s;
}

static cudaStream_t engine_side_stream() {
    static cudaStream_t s = [] {
        int least = 0, greatest = 0;
        SG_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        cudaStream_t t;
        SG_CUDA(cudaStreamCreateWithPriority(&t, cudaStreamNonBlocking, least));
        return t;
    }();
    return s;
}

// ---------------------------------------------------------------------------
// Input-register initialisation (engine/kernel/kernel.cpp:14-158).  Noise is
// drawn from the seeded counter-based generator (counter_rng.h), keyed by
// (seed, step, neuron); the step is the layer's own counter in the state.
// ---------------------------------------------------------------------------
__global__ void k_set_value(float* p, int n, float v, int overwrite) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = overwrite ? v : p[i] + v;
}

// kind 0 uniform(a, b), 1 normal(mean a, std b), 2 Poisson (probability a, or
// rates[i] when given; value b).  Overwrite for a layer without input, add
// onto an input layer's input (kernel.cpp:42-158).  Every thread reads the
// step from ctr[0]; the last block to finish advances it (ctr[1] counts the
// finished blocks), so one launch per step keeps graphs valid.
__global__ void k_noise(float* p, int n, int kind, float a, float b, int overwrite,
                        unsigned long long seed, unsigned long long* ctr,
                        const float* __restrict__ rates) {
    const unsigned long long t = *(volatile unsigned long long*)ctr;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const unsigned long long idx = (t << 32) | (unsigned)i;
        const float u = rng_open01(seed, RNG_NOISE * 4 + 0, idx);
        if (kind == 2) {
            const float prob = rates ? rates[i] : a;
            if (overwrite) p[i] = u < prob ? b : 0.0f;
            else if (u < prob) p[i] += b;
        } else {
            float v;
            if (kind == 0) {
                v = (u * (b - a)) + a;
            } else {
                const float u2 = rng_open01(seed, RNG_NOISE * 4 + 1, idx);
                v = (noise_normal(u, u2) * b) + a;
            }
            p[i] = overwrite ? v : p[i] + v;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(ctr + 1, 1ull) == (unsigned long long)gridDim.x - 1) {
            ctr[0] = t + 1;
            ctr[1] = 0;
            __threadfence();
        }
    }
}


// ---------------------------------------------------------------------------
Engine::Engine(Network* net, Environment* env, State* state, const Props& args)
    : net_(net), env_(env), state_(state), args_(args), stream_(engine_stream()) {
    bool expected = false;
    if (!running.compare_exchange_strong(expected, true))
        throw SgError("Cannot run more than one engine at once!");
    try {
        if (args.has("devices")) {
            int d = args.get_int("devices", 0);
            if (d != 0) throw SgError("Failed to extract devices from Engine args! (one GPU: device 0)");
        }
        verbose_ = args.get_bool("verbose", false);
        learning_ = args.get_bool("learning flag", true);
        suppress_ = args.get_bool("suppress output", false);
        env_rate_ = std::max(1, args.get_int("environment rate", 1));
        profile_ = args.get_bool("profile", false);
        use_graphs_ = args.get_bool("graphs", true) && !profile_;
        // Learning overlapped with the next step's activations, for networks
        // whose learned connections are large (at least 2^20 synapses): the
        // learning kernels go to a low-priority side stream, with plain
        // launches.  Measured on the 3 x 256^2 plastic network: 237 us per
        // step, against 254 us for graphs of the same two branches
        // (instantiated to honour the node priorities copied from the
        // streams at capture) and 266 us for graphs without overlap.  One
        // stream when profiling, so that the per-group timings stay separate.
        if (learning_)
            for (auto& lp : net_->layers)
                for (Connection* c : lp->inputs)
                    if (c->plastic) {
                        std::string e = find_model(lp->model)->learning_error(*c);
                        if (!e.empty()) throw SgError(c->str() + ": " + e);
                    }
        long long learned = 0;
        if (learning_)
            for (auto& lp : net_->layers)
                for (Connection* c : lp->inputs)
                    if (c->plastic && find_model(lp->model)->learns(*c)) learned += c->num_weights;
        for (auto& sp : net_->structures) ordered_ = ordered_ || !sp->parallel();
        overlap_ = learning_ && !profile_ && !ordered_ &&
                   args.get_bool("overlap learning", learned >= (1LL << 20));
        if (overlap_) use_graphs_ = args.get_bool("graphs", false);
        if (overlap_) {
            side_ = engine_side_stream();
            SG_CUDA(cudaEventCreateWithFlags(&fork_ev_, cudaEventDisableTiming));
            SG_CUDA(cudaEventCreateWithFlags(&join_ev_, cudaEventDisableTiming));
            learn_ev_.assign(net_->connections.size(), nullptr);
            for (auto& e : learn_ev_) SG_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
            learn_pending_.assign(net_->connections.size(), 0);
        }
        graph_steps_ = std::max(2, args.get_int("graph steps", 16) / 2 * 2);
        build_modules();
        if (!modules_.empty()) use_graphs_ = false;
        // dendritic trees: activation order, and the internal registers set
        // to their init values (cluster_node.cpp:116-129; second-order nodes
        // and the root are not set)
        dend_ops_.assign(net_->layers.size(), {});
        for (auto& lp : net_->layers)
            if (lp->has_dendrites()) plan_dendrites(lp->root.get(), dend_ops_[lp->index]);
        state_->to_device(stream_);
        for (auto& lp : net_->layers) {
            if (!lp->has_dendrites()) continue;
            float* in = state_->layer_state(lp.get())->input->df();
            for (Dendrite* d : lp->dendrites()) {
                if (d == lp->root.get() || d->second_order) continue;
                k_set_value<<<blocks_for(lp->size, 256), 256, 0, stream_>>>(
                    in + (size_t)d->reg * lp->size, lp->size, d->init, 1);
                SG_LAUNCH_CHECK();
            }
            state_->mark_device_newer();
        }
        // No environment and every layer self-contained: whole runs per layer.
        alone_ = modules_.empty() && !net_->layers.empty() && !ordered_ && args.get_bool("whole runs", true);
        for (auto& lp : net_->layers)
            alone_ = alone_ && !lp->has_dendrites() &&
                     find_model(lp->model)->can_advance_alone(*state_, *state_->layer_state(lp.get()));
        for (auto& lp : net_->layers) {
            if (layer_io_[lp->index] & 1) input_layers_.push_back(lp.get());
            if (layer_io_[lp->index] & 2) output_layers_.push_back(lp.get());
        }
        in_dirty_.assign(input_layers_.size(), 0);
        for (Layer* l : input_layers_) {
            void* h;
            void* d;
            SG_CUDA(cudaMallocHost(&h, (size_t)l->size * 4));
            std::memset(h, 0, (size_t)l->size * 4);
            SG_CUDA(cudaMalloc(&d, (size_t)l->size * 4));
            SG_CUDA(cudaMemsetAsync(d, 0, (size_t)l->size * 4, stream_));
            in_pinned_.push_back((float*)h);
            in_staging_.push_back((float*)d);
        }
        for (Layer* l : output_layers_) {
            void* h;
            SG_CUDA(cudaMallocHost(&h, (size_t)l->size * 4));
            out_pinned_.push_back((uint32_t*)h);
        }
        SG_CUDA(cudaStreamSynchronize(stream_));
    } catch (...) {
        for (float* p : in_pinned_) cudaFreeHost(p);
        for (float* p : in_staging_) cudaFree(p);
        for (uint32_t* p : out_pinned_) cudaFreeHost(p);
        running = false;
        throw;
    }
}

Engine::~Engine() {
    if (side_pending_) {
        cudaEventRecord(join_ev_, side_);
        cudaStreamWaitEvent(stream_, join_ev_, 0);
    }
    cudaStreamSynchronize(stream_);
    if (fork_ev_) cudaEventDestroy(fork_ev_);
    if (join_ev_) cudaEventDestroy(join_ev_);
    for (auto& e : learn_ev_)
        if (e) cudaEventDestroy(e);
    for (float* p : in_pinned_) cudaFreeHost(p);
    for (float* p : in_staging_) cudaFree(p);
    for (uint32_t* p : out_pinned_) cudaFreeHost(p);
    for (auto& g : graphs_) cudaGraphExecDestroy(g.exec);
    for (auto& kv : prof_)
        for (auto& e : kv.second.events) { cudaEventDestroy(e.first); cudaEventDestroy(e.second); }
    running = false;
    interrupt_flag = false;
}

void Engine::plan_dendrites(Dendrite* node, std::vector<DendOp>& ops) {
    // a second-order node starts from a fresh copy of its host's weights
    if (node->second_order) ops.push_back({DendOp::SO_COPY, nullptr, node, nullptr});
    for (auto& ch : node->children) {
        if (ch.conn) {
            ops.push_back({DendOp::CONN, ch.conn, node, nullptr});
        } else {
            plan_dendrites(ch.node, ops);
            if (node->reg != ch.node->reg) ops.push_back({DendOp::FOLD, nullptr, node, ch.node});
        }
    }
    // the host goes last: it reads the weights its slaves modulated
    if (node->second_order) {
        if (!node->host)
            throw SgError("Error building cluster node for " + node->layer->str() +
                          ":\n  Missing host connection for second order node!");
        ops.push_back({DendOp::CONN, node->host, node, nullptr});
    }
}

void Engine::build_modules() {
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

template <class F>
void Engine::timed(const std::string& name, long kernels, F&& f) {
    if (!profile_) { f(); return; }
    cudaEvent_t a, b;
    SG_CUDA(cudaEventCreate(&a));
    SG_CUDA(cudaEventCreate(&b));
    SG_CUDA(cudaEventRecord(a, stream_));
    f();
    SG_CUDA(cudaEventRecord(b, stream_));
    auto& p = prof_[name];
    p.events.push_back({a, b});
    p.launches += kernels;
}

void Engine::enqueue_step(bool last) {
    StepCtx ctx{stream_, last, &layer_io_, &launches_};
    // 1. input registers
    for (auto& lp : net_->layers) {
        Layer* l = lp.get();
        const Model* m = find_model(l->model);
        LayerState* ls = state_->layer_state(l);
        m->begin_step(*state_, *ls, ctx);
        float* in = ls->input->df();
        bool is_input = (layer_io_[l->index] & 1) != 0;
        bool all_fused = !l->inputs.empty() && !l->has_dendrites();
        for (Connection* c : l->inputs) all_fused = all_fused && m->fuses_input(*state_, *c, ctx);
        if (all_fused && !is_input) continue;   // the fused update writes the register itself
        if (is_input) {
            size_t k = std::find(input_layers_.begin(), input_layers_.end(), l) - input_layers_.begin();
            if (in_dirty_[k]) {
                SG_CUDA(cudaMemcpyAsync(in_staging_[k], in_pinned_[k], (size_t)l->size * 4,
                                        cudaMemcpyHostToDevice, stream_));
                in_dirty_[k] = 0;
            }
            SG_CUDA(cudaMemcpyAsync(in, in_staging_[k], (size_t)l->size * 4, cudaMemcpyDeviceToDevice,
                                    stream_));
        }
        Props* init = l->config.child("init config");
        if (init) {
            std::string t = init->get("type", "normal");
            int ow = is_input ? 0 : 1;
            const unsigned long long seed = noise_seed(*l);
            unsigned blocks = blocks_for(l->size, 256);
            unsigned long long* ctr = nullptr;
            const float* rates = nullptr;
            if (t != "flat") {
                ctr = reinterpret_cast<unsigned long long*>(ls->internal.at("noise step")->du());
                auto r = ls->internal.find("noise rates");
                if (r != ls->internal.end()) rates = r->second->df();
            }
            timed("init", 1, [&] {
                if (t == "flat") {
                    k_set_value<<<blocks, 256, 0, stream_>>>(in, l->size, init->get_float("value", 1.0f), ow);
                } else if (t == "uniform") {
                    k_noise<<<blocks, 256, 0, stream_>>>(in, l->size, 0, init->get_float("min", 0.0f),
                                                         init->get_float("max", 1.0f), ow, seed, ctr,
                                                         nullptr);
                } else if (t == "normal") {
                    k_noise<<<blocks, 256, 0, stream_>>>(in, l->size, 1, init->get_float("mean", 1.0f),
                                                         init->get_float("std dev", 0.1f), ow, seed, ctr,
                                                         nullptr);
                } else if (t == "poisson") {
                    k_noise<<<blocks, 256, 0, stream_>>>(in, l->size, 2,
                                                         0.001f * init->get_float("rate", 1.0f),
                                                         init->get_float("value", 20.0f), ow, seed, ctr,
                                                         rates);
                } else {
                    throw SgError("Error building cluster node for " + l->str() +
                                  ":\n  Unrecognized init type: " + t);
                }
                SG_LAUNCH_CHECK();
            });
            ++launches_;
        } else if (!is_input) {
            SG_CUDA(cudaMemsetAsync(in, 0, (size_t)l->size * 4, stream_));
        }
    }
    // 2. synaptic input.  Layers whose inputs include a connection still
    // learning from the last step (side stream) go last, so that the other
    // layers' activations overlap that learning; activations into different
    // layers touch different arrays, and each layer keeps its own order.
    auto activate_conn = [&](Layer* l, const Model* m, Connection* c) {
        if (overlap_ && learn_pending_[c->index]) {    // after its learning of the last step
            SG_CUDA(cudaStreamWaitEvent(stream_, learn_ev_[c->index], 0));
            learn_pending_[c->index] = 0;
        }
        ConnState& cs = *state_->conn_state(c);
        if (c->second_order_slave) {
            float* so = state_->conn_state(c->node->host)->so_weights->df();
            timed("second_order.slave." + std::string(conn_type_name(c->type)), 1, [&] {
                launch_second_order_slave(*state_, cs, so, stream_);
            });
            ++launches_;
            return;
        }
        timed(std::string(l->model) + ".activate." + conn_type_name(c->type), 1, [&] {
            m->activate(*state_, cs, ctx);
        });
    };
    auto activate_layer = [&](Layer* l) {
        const Model* m = find_model(l->model);
        if (!l->has_dendrites()) {
            for (Connection* c : l->inputs)
                if (!m->fuses_input(*state_, *c, ctx)) activate_conn(l, m, c);
            return;
        }
        float* in = state_->layer_state(l)->input->df();
        for (const DendOp& op : dend_ops_[l->index]) {
            if (op.kind == DendOp::CONN) {
                activate_conn(l, m, op.conn);
            } else if (op.kind == DendOp::SO_COPY) {
                // SecondOrderWeightTransferInstruction (instruction.h:461-472)
                ConnState& hs = *state_->conn_state(op.node->host);
                SG_CUDA(cudaMemcpyAsync(hs.so_weights->df(), hs.weights->df(), hs.weights->dev_count * 4,
                                        cudaMemcpyDeviceToDevice, stream_));
            } else {
                timed("dendrite.fold", 1, [&] {
                    launch_dendrite_fold(l->size, in + (size_t)op.child->reg * l->size,
                                         in + (size_t)op.node->reg * l->size, (int)op.child->opcode,
                                         op.child->init, stream_);
                });
                ++launches_;
            }
        }
    };
    if (ordered_) {
        // Structures that are not all parallel: the reference's cluster
        // order (engine.cpp:226-315).  Parallel structures activate their
        // non-input layers before the input is read (parallel_cluster.cpp:
        // 27-79, 105-118), then each structure in turn: a parallel one its
        // input layers, a sequential / feedforward one every layer in its
        // order with its update right after its activations (so later layers
        // read this step's outputs); last, the parallel layers' updates.
        auto update_layer = [&](Layer* l) {
            const Model* m = find_model(l->model);
            timed(std::string(m->name()) + ".update", 1, [&] {
                m->update(*state_, *state_->layer_state(l), ctx);
            });
        };
        for (auto& sp : net_->structures)
            if (sp->parallel())
                for (Layer* l : sp->layers)
                    if (!(layer_io_[l->index] & 1)) activate_layer(l);
        for (auto& sp : net_->structures) {
            if (sp->parallel()) {
                for (Layer* l : sp->layers)
                    if (layer_io_[l->index] & 1) activate_layer(l);
            } else {
                for (Layer* l : sp->order) {
                    activate_layer(l);
                    update_layer(l);
                }
            }
        }
        for (auto& sp : net_->structures)
            if (sp->parallel())
                for (Layer* l : sp->layers) update_layer(l);
    } else {
    std::vector<Layer*> deferred;
    {
        // prologues of the connections whose activation waits on nothing,
        // grouped by the model of their destination layer
        std::vector<std::pair<const Model*, std::vector<ConnState*>>> pro;
        for (auto& lp : net_->layers) {
            const Model* m = find_model(lp->model);
            for (Connection* c : lp->inputs) {
                if (c->second_order_slave || (overlap_ && learn_pending_[c->index]) ||
                    m->fuses_input(*state_, *c, ctx))
                    continue;
                auto it = std::find_if(pro.begin(), pro.end(),
                                       [&](const auto& p) { return p.first == m; });
                if (it == pro.end()) {
                    pro.push_back({m, {}});
                    it = pro.end() - 1;
                }
                it->second.push_back(state_->conn_state(c));
            }
        }
        for (auto& p : pro)
            timed(std::string(p.first->name()) + ".prologue", 1,
                  [&] { p.first->activate_prologue(*state_, p.second, ctx); });
    }
    for (auto& lp : net_->layers) {
        bool waits = false;
        if (overlap_)
            for (Connection* c : lp->inputs) waits = waits || learn_pending_[c->index];
        if (waits) deferred.push_back(lp.get());
        else activate_layer(lp.get());
    }
    for (Layer* l : deferred) activate_layer(l);
    // learning of the last step whose connection was not activated above:
    // the destination's update must still come after it
    if (overlap_)
        for (size_t i = 0; i < learn_pending_.size(); ++i)
            if (learn_pending_[i]) {
                SG_CUDA(cudaStreamWaitEvent(stream_, learn_ev_[i], 0));
                learn_pending_[i] = 0;
            }
    // 3. neuron updates: the layers of each model together where the model
    // can (a layer's update touches only its own arrays, so the order of
    // updates does not matter)
    {
        std::vector<std::pair<const Model*, std::vector<LayerState*>>> groups;
        for (auto& lp : net_->layers) {
            const Model* m = find_model(lp->model);
            auto it = std::find_if(groups.begin(), groups.end(),
                                   [&](const auto& g) { return g.first == m; });
            if (it == groups.end()) {
                groups.push_back({m, {}});
                it = groups.end() - 1;
            }
            it->second.push_back(state_->layer_state(lp.get()));
        }
        for (auto& g : groups) {
            const std::string name = std::string(g.first->name()) + ".update";
            bool done = false;
            if (g.second.size() > 1)
                timed(name, 1, [&] { done = g.first->update_group(*state_, g.second, ctx); });
            if (!done)
                for (LayerState* ls : g.second)
                    timed(name, 1, [&] { g.first->update(*state_, *ls, ctx); });
        }
    }
    }
    // 4. plasticity (on the side stream when overlapped, after this step's
    // updates)
    if (learning_) {
        StepCtx lctx = ctx;
        bool forked = false;
        for (auto& lp : net_->layers) {
            const Model* m = find_model(lp->model);
            for (Connection* c : lp->inputs)
                if (c->plastic && m->learns(*c)) {
                    if (overlap_) {
                        if (!forked) {
                            SG_CUDA(cudaEventRecord(fork_ev_, stream_));
                            SG_CUDA(cudaStreamWaitEvent(side_, fork_ev_, 0));
                            lctx.stream = side_;
                            forked = true;
                        }
                        m->learn(*state_, *state_->conn_state(c), lctx);
                        SG_CUDA(cudaEventRecord(learn_ev_[c->index], side_));
                        learn_pending_[c->index] = 1;
                        side_pending_ = true;
                    } else {
                        timed(std::string(lp->model) + ".learn." + conn_type_name(c->type), 1, [&] {
                            m->learn(*state_, *state_->conn_state(c), ctx);
                        });
                    }
                }
        }
    }
}

void Engine::feed_input() {
    // module.cpp:86-97: callbacks write the pinned buffers; they must not be
    // overwritten while a copy from them is still queued.
    bool synced = false;
    for (auto& m : modules_) {
        if (m.start_delay > 0) continue;
        bool active = m.active();
        bool cut = m.cutoff != 0 && m.curr == m.cutoff;
        for (auto& ml : m.layers) {
            if (!ml.input || (!active && !cut)) continue;
            if (!synced) { SG_CUDA(cudaStreamSynchronize(stream_)); synced = true; }
            size_t k = std::find(input_layers_.begin(), input_layers_.end(), ml.layer) - input_layers_.begin();
            if (active) {
                if (m.clear) std::memset(in_pinned_[k], 0, (size_t)ml.layer->size * 4);
                ml.fn(ml.id, ml.layer->size, in_pinned_[k]);
            } else {
                std::memset(in_pinned_[k], 0, (size_t)ml.layer->size * 4);
            }
            in_dirty_[k] = 1;
        }
    }
}

void Engine::report_output(long i) {
    // module.cpp:99-104
    if (i % env_rate_ != 0 || suppress_ || output_layers_.empty()) return;
    for (size_t k = 0; k < output_layers_.size(); ++k)
        SG_CUDA(cudaMemcpyAsync(out_pinned_[k], state_->dev_output(output_layers_[k], 0),
                                (size_t)output_layers_[k]->size * 4, cudaMemcpyDeviceToHost, stream_));
    SG_CUDA(cudaStreamSynchronize(stream_));
    for (auto& m : modules_) {
        if (!m.active()) continue;
        for (auto& ml : m.layers)
            if (ml.output) {
                size_t k = std::find(output_layers_.begin(), output_layers_.end(), ml.layer) -
                           output_layers_.begin();
                ml.fn(ml.id, ml.layer->size, out_pinned_[k]);
            }
    }
}

void Engine::launch_step(bool last) {
    feed_input();
    enqueue_step(last);
}

long Engine::step(long n) {
    cudaEvent_t ev0, ev1;
    SG_CUDA(cudaEventCreate(&ev0));
    SG_CUDA(cudaEventCreate(&ev1));
    auto t0 = std::chrono::steady_clock::now();
    SG_CUDA(cudaEventRecord(ev0, stream_));
    long i = 0;
    if (alone_ && n > 0) {
        for (auto& lp : net_->layers) {
            const Model* m = find_model(lp->model);
            long k = 0;
            const std::string group = std::string(lp->model) + ".advance";
            timed(group, 0, [&] { k = m->advance_alone(*state_, *state_->layer_state(lp.get()), n, stream_); });
            launches_ += k;
            if (profile_) prof_[group].launches += k;
        }
        i = n;
    }
    while (n == 0 || i < n) {
        if (interrupt_flag) break;
        if (use_graphs_ && n != 0 && n - i > graph_steps_) {
            // Ping-pong outputs may sit in either buffer; a graph is only valid
            // for the buffer placement it was captured with.
            std::vector<void*> sig;
            for (auto& ls : state_->layers) sig.push_back(ls->output->dev);
            Graph* gr = nullptr;
            for (auto& cand : graphs_)
                if (cand.sig == sig) gr = &cand;
            if (!gr) {
                // Capture an even number of steps, so ping-pong buffers end
                // where they started.
                Graph ng;
                ng.sig = sig;
                long before = launches_;
                cudaGraph_t g;
                join_side();                 // nothing pending from outside the capture
                SG_CUDA(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
                for (int k = 0; k < graph_steps_; ++k) enqueue_step(false);
                join_side();                 // the side stream rejoins inside the graph
                SG_CUDA(cudaStreamEndCapture(stream_, &g));
                SG_CUDA(cudaGraphInstantiate(&ng.exec, g, cudaGraphInstantiateFlagUseNodePriority));
                SG_CUDA(cudaGraphDestroy(g));
                ng.launches = launches_ - before;
                launches_ = before;
                graphs_.push_back(ng);
                gr = &graphs_.back();
            }
            join_side();
            SG_CUDA(cudaGraphLaunch(gr->exec, stream_));
            launches_ += gr->launches;
            i += graph_steps_;
            continue;
        }
        bool last = (n != 0 && i == n - 1);
        launch_step(last);
        report_output(i);
        for (auto& m : modules_) {
            if (m.start_delay > 0) { --m.start_delay; continue; }
            if (m.cutoff == 0 || m.curr <= m.cutoff) ++m.curr;
        }
        ++i;
    }
    join_side();
    SG_CUDA(cudaEventRecord(ev1, stream_));
    SG_CUDA(cudaEventSynchronize(ev1));
    auto t1 = std::chrono::steady_clock::now();
    float ms = 0.0f;
    SG_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
    cudaEventDestroy(ev0);
    cudaEventDestroy(ev1);
    SG_CUDA(cudaGetLastError());
    state_->mark_device_newer();
    device_ms_ += ms;
    wall_s_ += std::chrono::duration<double>(t1 - t0).count();
    steps_ += i;
    return i;
}

void Engine::join_side() {
    if (!side_pending_) return;
    SG_CUDA(cudaEventRecord(join_ev_, side_));
    SG_CUDA(cudaStreamWaitEvent(stream_, join_ev_, 0));
    side_pending_ = false;
    std::fill(learn_pending_.begin(), learn_pending_.end(), 0);
}

void Engine::synchronize() {
    join_side();
    SG_CUDA(cudaStreamSynchronize(stream_));
    check_iz_cols_errors();
    check_debug_errors();
}

Props* Engine::report() {
    synchronize();
    auto* r = new Props();
    r->set("iterations", std::to_string(steps_));
    r->set("total time", std::to_string((float)wall_s_));
    r->set("average time", std::to_string((float)(steps_ ? wall_s_ / steps_ : 0.0)));
    r->set("fps", std::to_string((float)(wall_s_ > 0 ? steps_ / wall_s_ : 0.0)));
    r->set("network bytes", std::to_string(state_->device_bytes()));
    r->set("state bytes", std::to_string(state_->host_bytes()));   // moved by one upload / download
    r->set("state buffer bytes", "0");
    size_t eb = 0;
    for (Layer* l : input_layers_) eb += (size_t)l->size * 4;
    for (Layer* l : output_layers_) eb += (size_t)l->size * 4;
    r->set("engine buffer bytes", std::to_string(eb));
    r->set("device time", std::to_string(device_ms_ / 1000.0f));
    r->set("kernel launches", std::to_string(launches_));
    r->set("graphs", use_graphs_ ? "true" : "false");
    r->set_child("args", args_);
    r->set("interrupted", interrupt_flag ? "true" : "false");
    for (auto& kv : prof_) {
        double total = 0.0;
        for (auto& e : kv.second.events) {
            float ms = 0.0f;
            SG_CUDA(cudaEventElapsedTime(&ms, e.first, e.second));
            total += ms;
        }
        Props k;
        k.set("name", kv.first);
        k.set("groups", std::to_string(kv.second.events.size()));
        k.set("launches", std::to_string(kv.second.launches));
        k.set("total ms", std::to_string(total));
        k.set("mean us", std::to_string(kv.second.events.empty() ? 0.0 : 1000.0 * total / kv.second.events.size()));
        r->add_to_child_array("kernel times", k);
    }
    if (verbose_)
        printf("Ran %ld iterations in %fs (device %fs)\n", steps_, wall_s_, device_ms_ / 1000.0f);
    return r;
}

}  // namespace sg
