// The reference's smaller neural models: binary threshold, the two
// rate-encoding variants, perceptron, sine generator, Poisson generator,
// oscillator and self-organising map (src/core/state/impl/*_attributes.cpp).  Each update is one thread per
// neuron over the layer's input register and output history.
#include <cmath>

#include "counter_rng.h"
#include "cuda_check.h"
#include "history.cuh"
#include "models.h"
#include "state.h"
#include "weight_init.h"

namespace sg {

// Seed of a layer's random draws: its "seed" property, else the global seed
// mixed with the layer's position.
static unsigned long long layer_seed(const Layer& l) {
    return l.config.has("seed") ? std::stoull(l.config.get("seed"))
                                : (global_seed() ^ (0xC0FFEE1234567ULL * (unsigned long long)(l.index + 1)));
}

// The reference binds an updater's source outputs only when both layers sit
// in one feedforward structure (synapse_data.cpp:36-51); elsewhere the
// updaters that read them would dereference a null pointer.
static bool sources_bound(const Connection& c) {
    return c.from->structure == c.to->structure && c.to->structure->cluster_type == "feedforward";
}

// Update of oscillator and vp_max connections (oscillator_attributes.cpp:
// 196-206, vp_max_attributes.cpp:150-160): w += out * (post - out * w).
template <int TY, int SR>
__global__ void __launch_bounds__(128) k_learn_toward_post(DGeom g, const uint32_t* __restrict__ src,
                                                           int delay, const uint32_t* __restrict__ dest_out,
                                                           float* w) {
    const int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= g.n_dest) return;
    const int to = dest_of<TY>(g, d);
    const float to_out = extract<SR>(dest_out[to], 0);
    for_each_source<TY>(g, d, [&](int from, int wi) {
        const float from_out = extract<SR>(src[from], delay);
        const float old = w[wi];
        w[wi] = old + (from_out * (to_out - (from_out * old)));
    });
}

static void launch_learn_toward_post(State& st, ConnState& cs, const StepCtx& ctx) {
    const Connection& c = *cs.conn;
    const uint32_t* src = st.dev_output(c.from, word_index(c.delay, c.from->output_type));
    SG_DISPATCH_TYPE_SRC((int)c.type, (int)c.from->output_type,
        (k_learn_toward_post<TY, SR><<<blocks_for(cs.geom.n_dest, 128), 128, 0, ctx.stream>>>(
            cs.geom, src, c.delay, st.dev_output(c.to, 0), cs.weights->df())));
    SG_LAUNCH_CHECK();
    ctx.count();
}

// Convolutional connections learn per kernel weight
// (CALC_{CONVERGENT,DIVERGENT}_CONVOLUTIONAL_BY_WEIGHT, synapse_kernel.h:
// 610-796): the kernel weight's terms out * (post - out * w) summed over the
// destinations in row-major order (sources outside a non-wrapping layer
// skipped), then w += rate * sum / kernel size.  One thread per kernel
// weight.  A divergent destination's window starts at (t + spacing * (-offset
// - field + stride)) / stride, truncating.
template <int SR, bool DIV>
__global__ void k_learn_toward_post_conv(DGeom g, const uint32_t* __restrict__ src, int delay,
                                         const uint32_t* __restrict__ dest_out, float rate, int n_weights,
                                         float* w) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= g.rf * g.cf) return;
    const int kr = k / g.cf, kc = k % g.cf;
    const float old = w[k];
    float delta = 0.0f;
    for (int tr = 0; tr < g.to_rows; ++tr)
        for (int tc = 0; tc < g.to_cols; ++tc) {
            int fr = DIV ? (tr + g.rsp * (-g.ro - g.rf + g.rs)) / g.rs + kr * g.rsp
                         : tr * g.rs + g.rsp * g.ro + kr * g.rsp;
            int fc = DIV ? (tc + g.csp * (-g.co - g.cf + g.cs)) / g.cs + kc * g.csp
                         : tc * g.cs + g.csp * g.co + kc * g.csp;
            if (g.wrap) {
                fr = wrap_idx(fr, g.from_rows);
                fc = wrap_idx(fc, g.from_cols);
            } else if (fr < 0 || fr >= g.from_rows || fc < 0 || fc >= g.from_cols) {
                continue;
            }
            const float from_out = extract<SR>(src[fr * g.from_cols + fc], delay);
            const float to_out = extract<SR>(dest_out[tr * g.to_cols + tc], 0);
            delta += from_out * (to_out - (from_out * old));
        }
    w[k] = old + (rate * delta / n_weights);
}

static void launch_learn_toward_post_conv(State& st, ConnState& cs, const StepCtx& ctx, float rate) {
    const Connection& c = *cs.conn;
    const uint32_t* src = st.dev_output(c.from, word_index(c.delay, c.from->output_type));
    const uint32_t* dst = st.dev_output(c.to, 0);
    const int k = c.arbor.kernel(), nw = (int)c.num_weights;
    const unsigned b = blocks_for(k, 64);
    const int sel = (int)c.from->output_type * 2 + (c.type == DIVERGENT ? 1 : 0);
    switch (sel) {
        case 0: k_learn_toward_post_conv<0, false><<<b, 64, 0, ctx.stream>>>(cs.geom, src, c.delay, dst, rate, nw, cs.weights->df()); break;
        case 1: k_learn_toward_post_conv<0, true><<<b, 64, 0, ctx.stream>>>(cs.geom, src, c.delay, dst, rate, nw, cs.weights->df()); break;
        case 2: k_learn_toward_post_conv<1, false><<<b, 64, 0, ctx.stream>>>(cs.geom, src, c.delay, dst, rate, nw, cs.weights->df()); break;
        case 3: k_learn_toward_post_conv<1, true><<<b, 64, 0, ctx.stream>>>(cs.geom, src, c.delay, dst, rate, nw, cs.weights->df()); break;
        case 4: k_learn_toward_post_conv<2, false><<<b, 64, 0, ctx.stream>>>(cs.geom, src, c.delay, dst, rate, nw, cs.weights->df()); break;
        default: k_learn_toward_post_conv<2, true><<<b, 64, 0, ctx.stream>>>(cs.geom, src, c.delay, dst, rate, nw, cs.weights->df()); break;
    }
    SG_LAUNCH_CHECK();
    ctx.count();
}

static std::string toward_post_error(const Connection& c, const char* model) {
    if (!sources_bound(c))
        return std::string(model) + " learning reads source outputs that the reference binds only "
               "in feedforward structures (set \"plastic\": false or run without learning)";
    return "";
}

// ---------------------------------------------------------------------------
// binary threshold (bin_thresh_attributes.cpp:9-17): output 1 where the input
// is positive.
// ---------------------------------------------------------------------------
__global__ void k_bin_thresh(int size, int history, const float* __restrict__ in, float* out) {
    int nid = blockIdx.x * blockDim.x + threadIdx.x;
    if (nid >= size) return;
    shift_floats(out, size, history, nid, in[nid] > 0.0f ? 1.0f : 0.0f);
}

class BinaryThresholdModel : public Model {
  public:
    const char* name() const override { return "binary threshold"; }
    OutputType output_type() const override { return OUT_FLOAT; }
    void update(State&, LayerState& ls, const StepCtx& ctx) const override {
        const Layer& l = *ls.layer;
        k_bin_thresh<<<blocks_for(l.size, 256), 256, 0, ctx.stream>>>(l.size, l.history(),
                                                                      ls.input->df(), ls.output->df());
        SG_LAUNCH_CHECK();
        ctx.count();
    }
};
SG_REGISTER_MODEL(BinaryThresholdModel);

// ---------------------------------------------------------------------------
// Rate-encoding variants.  Both update like rate_encoding (tanh of positive
// input).  backprop_rate_encoding adds a per-neuron "error deltas" variable
// (backprop_rate_encoding_attributes.cpp:16-19) and builds only in
// feedforward structures (backprop_rate_encoding_attributes.h:10-12), so with
// the parallel structures supported here it reports the reference's
// compatibility error.  hebbian_rate_encoding's
// learning rule is declared as get_updater, which overrides nothing, so the
// reference's engine never applies it
// (hebbian_rate_encoding_attributes.h:10, attributes.h:44-45): its
// connections do not learn here either.
// ---------------------------------------------------------------------------
__global__ void k_rate_variant(int size, int history, const float* __restrict__ in, float* out) {
    int nid = blockIdx.x * blockDim.x + threadIdx.x;
    if (nid >= size) return;
    float input = in[nid];
    shift_floats(out, size, history, nid, (input > 0.0f) ? tanhf(input) : 0.0f);
}

class RateVariantModel : public Model {
  public:
    RateVariantModel(const char* n, bool deltas) : name_(n), deltas_(deltas) {}
    const char* name() const override { return name_; }
    OutputType output_type() const override { return OUT_FLOAT; }
    void build_layer(State& st, LayerState& ls) const override {
        if (deltas_ && ls.layer->structure->cluster_type != "feedforward")
            throw SgError("Error building attributes for " + ls.layer->str() +
                          ":\n  Cluster compatibility conflict detected!");
        if (deltas_) ls.vars["error deltas"] = st.add_array("error deltas", 'f', ls.layer->size);
    }
    void update(State&, LayerState& ls, const StepCtx& ctx) const override {
        const Layer& l = *ls.layer;
        k_rate_variant<<<blocks_for(l.size, 256), 256, 0, ctx.stream>>>(l.size, l.history(),
                                                                        ls.input->df(), ls.output->df());
        SG_LAUNCH_CHECK();
        ctx.count();
    }

  private:
    const char* name_;
    bool deltas_;
};
static const bool sg_registered_backprop =
    register_model(new RateVariantModel("backprop_rate_encoding", true));
static const bool sg_registered_hebbian =
    register_model(new RateVariantModel("hebbian_rate_encoding", false));

// ---------------------------------------------------------------------------
// perceptron (perceptron_attributes.cpp:13-47): synaptic input counts the
// weights of active sources, sum += (extract(out[from]) > 0) * w; the update
// divides the input by the layer's weights per neuron (integer division of
// the total weights of its input connections by its size).
// ---------------------------------------------------------------------------
template <int TY, int SR>
__global__ void __launch_bounds__(256) k_activate_perceptron(DGeom g, const uint32_t* __restrict__ src,
                                                             int delay, int opcode,
                                                             const float* __restrict__ w,
                                                             float* __restrict__ inputs) {
    int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= g.n_dest) return;
    float sum = 0.0f;
    for_each_source<TY>(g, d, [&](int from, int wi) {
        sum += (extract<SR>(src[from], delay) > 0.0f ? 1.0f : 0.0f) * w[wi];
    });
    int to = dest_of<TY>(g, d);
    inputs[to] = aggregate(inputs[to], sum, opcode);
}

template <int TY>
__global__ void __launch_bounds__(128) k_learn_perceptron(DGeom g, const uint32_t* __restrict__ src,
                                                          const float* __restrict__ dest_out,
                                                          const float* __restrict__ expected, float* w) {
    const int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= g.n_dest) return;
    const int to = dest_of<TY>(g, d);
    const float delta = expected[to] - dest_out[to];
    for_each_source<TY>(g, d, [&](int from, int wi) {
        w[wi] = (float)((double)w[wi] + 0.05 * delta * __uint_as_float(src[from]));
    });
}

__global__ void k_perceptron(int size, int history, int per_neuron, const float* __restrict__ in,
                             float* out) {
    int nid = blockIdx.x * blockDim.x + threadIdx.x;
    if (nid >= size) return;
    shift_floats(out, size, history, nid, in[nid] / (float)per_neuron);
}

class PerceptronModel : public Model {
  public:
    const char* name() const override { return "perceptron"; }
    OutputType output_type() const override { return OUT_FLOAT; }
    void build_layer(State& st, LayerState& ls) const override {
        ls.vars["expected"] = st.add_array("expected", 'f', ls.layer->size);
    }
    void build_matrix(State&, ConnState& cs) const override {
        const Connection& c = *cs.conn;
        if (c.second_order || c.convolutional) throw SgError(c.str() + ": Unimplemented connection type!");
    }
    // The updater reads the source outputs (bound only within a feedforward
    // structure): w += 0.05 * (expected - output) * source output
    // (perceptron_attributes.cpp:51-60).
    std::string learning_error(const Connection& c) const override {
        if (sources_bound(c)) return "";
        return "perceptron learning reads source outputs that the reference binds only in "
               "feedforward structures (set \"plastic\": false or run without learning)";
    }
    bool learns(const Connection&) const override { return true; }
    void learn(State& st, ConnState& cs, const StepCtx& ctx) const override {
        const Connection& c = *cs.conn;
        const uint32_t* src = st.dev_output(c.from, word_index(c.delay, c.from->output_type));
        const LayerState& to = *st.layer_state(c.to);
        const unsigned blocks = blocks_for(cs.geom.n_dest, 128);
        const float* out = to.output->df();
        const float* expected = to.var("expected")->df();
        switch ((int)c.type) {
            case 0: k_learn_perceptron<0><<<blocks, 128, 0, ctx.stream>>>(cs.geom, src, out, expected, cs.weights->df()); break;
            case 1: k_learn_perceptron<1><<<blocks, 128, 0, ctx.stream>>>(cs.geom, src, out, expected, cs.weights->df()); break;
            case 2: k_learn_perceptron<2><<<blocks, 128, 0, ctx.stream>>>(cs.geom, src, out, expected, cs.weights->df()); break;
            case 3: k_learn_perceptron<3><<<blocks, 128, 0, ctx.stream>>>(cs.geom, src, out, expected, cs.weights->df()); break;
            case 4: k_learn_perceptron<4><<<blocks, 128, 0, ctx.stream>>>(cs.geom, src, out, expected, cs.weights->df()); break;
            case 5: k_learn_perceptron<5><<<blocks, 128, 0, ctx.stream>>>(cs.geom, src, out, expected, cs.weights->df()); break;
        }
        SG_LAUNCH_CHECK();
        ctx.count();
    }
    void activate(State& st, ConnState& cs, const StepCtx& ctx) const override {
        const Connection& c = *cs.conn;
        const uint32_t* src = st.dev_output(c.from, word_index(c.delay, c.from->output_type));
        unsigned blocks = blocks_for(cs.geom.n_dest, 128);
        float* inputs = input_register(st, cs);
        SG_DISPATCH_TYPE_SRC((int)c.type, (int)c.from->output_type,
            (k_activate_perceptron<TY, SR><<<blocks, 128, 0, ctx.stream>>>(
                cs.geom, src, c.delay, (int)c.opcode, cs.weights->df(), inputs)));
        SG_LAUNCH_CHECK();
        ctx.count();
    }
    void update(State&, LayerState& ls, const StepCtx& ctx) const override {
        const Layer& l = *ls.layer;
        long total = 0;
        for (const Connection* c : l.inputs) total += c->num_weights;   // layer.cpp:110-115
        const int per_neuron = (int)(total / l.size);
        k_perceptron<<<blocks_for(l.size, 256), 256, 0, ctx.stream>>>(l.size, l.history(), per_neuron,
                                                                      ls.input->df(), ls.output->df());
        SG_LAUNCH_CHECK();
        ctx.count();
    }
};
SG_REGISTER_MODEL(PerceptronModel);

// ---------------------------------------------------------------------------
// Generators with per-layer state on the device: a step counter that
// persists across runs, advanced by one thread after the update.
// ---------------------------------------------------------------------------
__global__ void k_tick(int* counter) { *counter += 1; }

// sine generator (sine_generator_attributes.cpp:11-31): output = input *
// (1 + sin(frequency * iteration)) / 2 with a float frequency of
// 2 pi / 1000 * "frequency" and the iteration counting the layer's steps.
// The sine of the float argument is taken in double and rounded, as the
// reference's sin(float) expression is.
__global__ void k_sine(int size, int history, float frequency, const int* __restrict__ iteration,
                       const float* __restrict__ in, float* out) {
    int nid = blockIdx.x * blockDim.x + threadIdx.x;
    if (nid >= size) return;
    const float x = frequency * (float)*iteration;
    const float wave = (float)((1.0 + sin((double)x)) / 2.0);
    shift_floats(out, size, history, nid, in[nid] * wave);
}

class SineGeneratorModel : public Model {
  public:
    const char* name() const override { return "sine generator"; }
    OutputType output_type() const override { return OUT_FLOAT; }
    void build_layer(State& st, LayerState& ls) const override {
        const float f = std::stof(ls.layer->parameter("frequency", "10"));
        ls.params["frequency"] = (float)(2 * M_PI / 1000 * f);
        ls.internal["iteration"] = st.add_array("iteration", 'i', 1);
    }
    void update(State&, LayerState& ls, const StepCtx& ctx) const override {
        const Layer& l = *ls.layer;
        int* it = ls.internal.at("iteration")->di();
        k_sine<<<blocks_for(l.size, 256), 256, 0, ctx.stream>>>(l.size, l.history(), ls.params.at("frequency"),
                                                               it, ls.input->df(), ls.output->df());
        SG_LAUNCH_CHECK();
        k_tick<<<1, 1, 0, ctx.stream>>>(it);
        SG_LAUNCH_CHECK();
        ctx.count(2);
    }
};
SG_REGISTER_MODEL(SineGeneratorModel);

// poisson generator (poisson_generator_attributes.cpp:9-24): a neuron spikes
// when a uniform draw in [0, 1) falls below its input.  The reference draws
// from an unseeded generator; here the draw is a counter-based function of
// (seed, layer, step, neuron), reproducible under sg_set_seed or the layer's
// "seed" property.
__global__ void k_poisson_gen(int size, int history, unsigned long long seed, const int* __restrict__ tick,
                              const float* __restrict__ in, uint32_t* out) {
    int nid = blockIdx.x * blockDim.x + threadIdx.x;
    if (nid >= size) return;
    const float u = rng_uniform(seed, (uint64_t)*tick, (uint64_t)nid);
    shift_bits(out, size, history, nid, u < in[nid] ? 1u : 0u);
}

class PoissonGeneratorModel : public Model {
  public:
    const char* name() const override { return "poisson generator"; }
    OutputType output_type() const override { return OUT_BIT; }
    void build_layer(State& st, LayerState& ls) const override {
        ls.internal["tick"] = st.add_array("tick", 'i', 1);
    }
    void update(State& st, LayerState& ls, const StepCtx& ctx) const override {
        const Layer& l = *ls.layer;
        int* tick = ls.internal.at("tick")->di();
        const unsigned long long seed = layer_seed(l);
        k_poisson_gen<<<blocks_for(l.size, 256), 256, 0, ctx.stream>>>(l.size, l.history(), seed, tick,
                                                                       ls.input->df(), ls.output->du());
        SG_LAUNCH_CHECK();
        k_tick<<<1, 1, 0, ctx.stream>>>(tick);
        SG_LAUNCH_CHECK();
        ctx.count(2);
    }
};
SG_REGISTER_MODEL(PoissonGeneratorModel);

// ---------------------------------------------------------------------------
// oscillator (oscillator_attributes.cpp): a leaky state relaxing towards
// "tonic", output max(0, tanh(state)), and a "bold" signal -- cleared every
// step (its init key), then the absolute synaptic inputs and the leak added.
// Its updaters read source outputs the reference binds only in feedforward
// structures (learning elsewhere is refused), and its second-order kernels
// write the weight copy of the slave's own matrix, which only hosts have
// (refused).
// ---------------------------------------------------------------------------
template <int TY, int SR>
__global__ void __launch_bounds__(128) k_activate_oscillator(DGeom g, const uint32_t* __restrict__ src,
                                                             int delay, int opcode,
                                                             const float* __restrict__ w,
                                                             float* __restrict__ inputs,
                                                             float* __restrict__ bold) {
    const int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= g.n_dest) return;
    float sum = 0.0f, abs_sum = 0.0f;
    for_each_source<TY>(g, d, [&](int from, int wi) {
        const float val = extract<SR>(src[from], delay) * w[wi];
        sum += val;
        abs_sum += fabsf(val);
    });
    const int to = dest_of<TY>(g, d);
    inputs[to] = aggregate(inputs[to], sum, opcode);
    bold[to] += abs_sum;
}

__global__ void k_oscillator(int size, int history, float tonic, float tau, float decay,
                             const float* __restrict__ in, float* state, float* bold, float* out) {
    const int nid = blockIdx.x * blockDim.x + threadIdx.x;
    if (nid >= size) return;
    float st = state[nid];
    const float recur = st + (decay * (tonic - st));
    state[nid] = st = (tau * in[nid]) + recur;
    bold[nid] += recur;
    const float t = tanhf(st);
    shift_floats(out, size, history, nid, (0.0f > t) ? 0.0f : t);
}

class OscillatorModel : public Model {
  public:
    const char* name() const override { return "oscillator"; }
    OutputType output_type() const override { return OUT_FLOAT; }
    void build_layer(State& st, LayerState& ls) const override {
        const Layer& l = *ls.layer;
        ls.params["tonic"] = std::stof(l.parameter("tonic", "0.0"));
        ls.params["tau"] = std::stof(l.parameter("tau", "0.1"));
        ls.params["decay"] = std::stof(l.parameter("decay", "0.1"));
        ls.vars["state"] = st.add_array("state", 'f', l.size);
        ls.vars["bold"] = st.add_array("bold", 'f', l.size);
    }
    void build_matrix(State&, ConnState& cs) const override {
        if (cs.conn->second_order) throw SgError(cs.conn->str() + ": Unimplemented connection type!");
    }
    std::string learning_error(const Connection& c) const override {
        return toward_post_error(c, "oscillator");
    }
    bool learns(const Connection&) const override { return true; }
    void learn(State& st, ConnState& cs, const StepCtx& ctx) const override {
        if (cs.conn->convolutional) launch_learn_toward_post_conv(st, cs, ctx, 1.0f);
        else launch_learn_toward_post(st, cs, ctx);
    }
    void begin_step(State&, LayerState& ls, const StepCtx& ctx) const override {
        SG_CUDA(cudaMemsetAsync(ls.var("bold")->df(), 0, (size_t)ls.layer->size * 4, ctx.stream));
    }
    void activate(State& st, ConnState& cs, const StepCtx& ctx) const override {
        const Connection& c = *cs.conn;
        const uint32_t* src = st.dev_output(c.from, word_index(c.delay, c.from->output_type));
        float* bold = st.layer_state(c.to)->var("bold")->df();
        SG_DISPATCH_TYPE_SRC((int)c.type, (int)c.from->output_type,
            (k_activate_oscillator<TY, SR><<<blocks_for(cs.geom.n_dest, 128), 128, 0, ctx.stream>>>(
                cs.geom, src, c.delay, (int)c.opcode, cs.weights->df(), input_register(st, cs), bold)));
        SG_LAUNCH_CHECK();
        ctx.count();
    }
    void update(State&, LayerState& ls, const StepCtx& ctx) const override {
        const Layer& l = *ls.layer;
        k_oscillator<<<blocks_for(l.size, 256), 256, 0, ctx.stream>>>(
            l.size, l.history(), ls.params.at("tonic"), ls.params.at("tau"), ls.params.at("decay"),
            ls.input->df(), ls.var("state")->df(), ls.var("bold")->df(), ls.output->df());
        SG_LAUNCH_CHECK();
        ctx.count();
    }
};
SG_REGISTER_MODEL(OscillatorModel);

// ---------------------------------------------------------------------------
// som (som_attributes.cpp): synaptic input is the squared distance between
// the sources' outputs and the weights (added, whatever the opcode), with
// the outputs cached per synapse; "modulate" connections set the neuron's
// plasticity instead.  The update finds the winner (first neuron of least
// input) and outputs exp(-rbf scale * input^2); learning pulls the winner's
// weights (and, slower, those within the Manhattan neighbourhood) towards
// the cached outputs.  A convolutional connection's cache entry would be
// written by every destination in turn: refused here.
// ---------------------------------------------------------------------------
template <int TY, int SR, bool MOD>
__global__ void __launch_bounds__(128) k_activate_som(DGeom g, const uint32_t* __restrict__ src,
                                                      int delay, const float* __restrict__ w,
                                                      float* __restrict__ cache,
                                                      float* __restrict__ inputs,
                                                      float* __restrict__ plasticity) {
    const int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= g.n_dest) return;
    float acc = 0.0f;
    for_each_source<TY>(g, d, [&](int from, int wi) {
        const float out = extract<SR>(src[from], delay);
        if (MOD) {
            acc += w[wi] * out;
        } else {
            const float val = out - w[wi];
            cache[wi] = out;
            acc += val * val;
        }
    });
    const int to = dest_of<TY>(g, d);
    if (MOD) plasticity[to] = acc;
    else inputs[to] += acc;
}

// The serial scan's winner (som_attributes.cpp:18-27): starting from neuron
// 0, each strictly smaller input takes over, so the winner is the first
// neuron of least (non-NaN) input, or 0 when input 0 is NaN.  One block: a
// strided scan per thread, then a tree that keeps the lower index on ties.
__global__ void __launch_bounds__(1024) k_som_winner(int size, const float* __restrict__ in, int* winner) {
    __shared__ float sv[1024];
    __shared__ int si[1024];
    float best = 0.0f;
    int bi = -1;
    for (int i = threadIdx.x; i < size; i += blockDim.x) {
        const float v = in[i];
        if (v == v && (bi < 0 || v < best)) { best = v; bi = i; }
    }
    sv[threadIdx.x] = best;
    si[threadIdx.x] = bi;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if (threadIdx.x < h) {
            const float ov = sv[threadIdx.x + h], mv = sv[threadIdx.x];
            const int oi = si[threadIdx.x + h], mi = si[threadIdx.x];
            if (oi >= 0 && (mi < 0 || ov < mv || (ov == mv && oi < mi))) {
                sv[threadIdx.x] = ov;
                si[threadIdx.x] = oi;
            }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) *winner = (si[0] < 0 || in[0] != in[0]) ? 0 : si[0];
}

__global__ void k_som(int size, int history, float rbf_scale, const float* __restrict__ in, float* out) {
    const int nid = blockIdx.x * blockDim.x + threadIdx.x;
    if (nid >= size) return;
    const float input = in[nid];
    shift_floats(out, size, history, nid, expf(-rbf_scale * (input * input)));
}

template <int TY>
__global__ void __launch_bounds__(128) k_learn_som(DGeom g, const int* __restrict__ winner,
                                                   const float* __restrict__ plasticity,
                                                   const float* __restrict__ cache, float lr, float nlr,
                                                   int nbhd, float* w) {
    const int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= g.n_dest) return;
    const int to = dest_of<TY>(g, d);
    const int win = *winner;
    const int row_dist = abs(win / g.to_cols - to / g.to_cols);
    const int col_dist = abs(win % g.to_cols - to % g.to_cols);
    const bool is_win = to == win;
    if (!is_win && row_dist + col_dist > nbhd) return;
    const float rate = is_win ? lr : nlr;
    const float p = plasticity[to];
    for_each_source<TY>(g, d, [&](int, int wi) { w[wi] += p * rate * (cache[wi] - w[wi]); });
}

class SomModel : public Model {
  public:
    const char* name() const override { return "som"; }
    OutputType output_type() const override { return OUT_FLOAT; }
    void build_layer(State& st, LayerState& ls) const override {
        ls.params["rbf scale"] = std::stof(ls.layer->parameter("rbf scale", "1"));
        ls.vars["plasticity"] = st.add_array("plasticity", 'f', ls.layer->size);
        ls.internal["winner"] = st.add_array("winner", 'i', 1);
    }
    void build_matrix(State& st, ConnState& cs) const override {
        const Connection& c = *cs.conn;
        if (c.second_order || c.convolutional) throw SgError(c.str() + ": Unimplemented connection type!");
        cs.params["learning rate"] = std::stof(c.parameter("learning rate", "0.01"));
        cs.params["neighbor learning rate"] = std::stof(c.parameter("neighbor learning rate", "0.001"));
        cs.params["neighborhood size"] = (float)std::stoi(c.parameter("neighborhood size", "2"));
        cs.vars["output cache"] = st.add_array("output cache", 'f', c.num_weights, matrix_layout(c),
                                               c.matrix_rows, c.matrix_cols);
    }
    void activate(State& st, ConnState& cs, const StepCtx& ctx) const override {
        const Connection& c = *cs.conn;
        const uint32_t* src = st.dev_output(c.from, word_index(c.delay, c.from->output_type));
        float* plast = st.layer_state(c.to)->var("plasticity")->df();
        const unsigned blocks = blocks_for(cs.geom.n_dest, 128);
        if (c.opcode == OP_MODULATE) {
            SG_DISPATCH_TYPE_SRC((int)c.type, (int)c.from->output_type,
                (k_activate_som<TY, SR, true><<<blocks, 128, 0, ctx.stream>>>(
                    cs.geom, src, c.delay, cs.weights->df(), cs.var("output cache")->df(),
                    input_register(st, cs), plast)));
        } else {
            SG_DISPATCH_TYPE_SRC((int)c.type, (int)c.from->output_type,
                (k_activate_som<TY, SR, false><<<blocks, 128, 0, ctx.stream>>>(
                    cs.geom, src, c.delay, cs.weights->df(), cs.var("output cache")->df(),
                    input_register(st, cs), plast)));
        }
        SG_LAUNCH_CHECK();
        ctx.count();
    }
    void update(State&, LayerState& ls, const StepCtx& ctx) const override {
        const Layer& l = *ls.layer;
        k_som_winner<<<1, 1024, 0, ctx.stream>>>(l.size, ls.input->df(), ls.internal.at("winner")->di());
        SG_LAUNCH_CHECK();
        k_som<<<blocks_for(l.size, 256), 256, 0, ctx.stream>>>(l.size, l.history(), ls.params.at("rbf scale"),
                                                              ls.input->df(), ls.output->df());
        SG_LAUNCH_CHECK();
        ctx.count(2);
    }
    bool learns(const Connection&) const override { return true; }
    void learn(State& st, ConnState& cs, const StepCtx& ctx) const override {
        const Connection& c = *cs.conn;
        LayerState& to = *st.layer_state(c.to);
        const unsigned blocks = blocks_for(cs.geom.n_dest, 128);
        const int* win = to.internal.at("winner")->di();
        const float* plast = to.var("plasticity")->df();
        const float* cache = cs.var("output cache")->df();
        const float lr = cs.params.at("learning rate"), nlr = cs.params.at("neighbor learning rate");
        const int nb = (int)cs.params.at("neighborhood size");
        switch ((int)c.type) {
            case 0: k_learn_som<0><<<blocks, 128, 0, ctx.stream>>>(cs.geom, win, plast, cache, lr, nlr, nb, cs.weights->df()); break;
            case 1: k_learn_som<1><<<blocks, 128, 0, ctx.stream>>>(cs.geom, win, plast, cache, lr, nlr, nb, cs.weights->df()); break;
            case 2: k_learn_som<2><<<blocks, 128, 0, ctx.stream>>>(cs.geom, win, plast, cache, lr, nlr, nb, cs.weights->df()); break;
            case 3: k_learn_som<3><<<blocks, 128, 0, ctx.stream>>>(cs.geom, win, plast, cache, lr, nlr, nb, cs.weights->df()); break;
            case 4: k_learn_som<4><<<blocks, 128, 0, ctx.stream>>>(cs.geom, win, plast, cache, lr, nlr, nb, cs.weights->df()); break;
            case 5: k_learn_som<5><<<blocks, 128, 0, ctx.stream>>>(cs.geom, win, plast, cache, lr, nlr, nb, cs.weights->df()); break;
        }
        SG_LAUNCH_CHECK();
        ctx.count();
    }
};
SG_REGISTER_MODEL(SomModel);

// ---------------------------------------------------------------------------
// vp_max (vp_max_attributes.cpp): synaptic input is the largest weighted
// source value (at least 0), aggregated with the opcode; the output is the
// input.  Learning and second order as for the oscillator.
// ---------------------------------------------------------------------------
template <int TY, int SR>
__global__ void __launch_bounds__(128) k_activate_vp_max(DGeom g, const uint32_t* __restrict__ src,
                                                         int delay, int opcode,
                                                         const float* __restrict__ w,
                                                         float* __restrict__ inputs) {
    const int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= g.n_dest) return;
    float max_val = 0.0f;
    for_each_source<TY>(g, d, [&](int from, int wi) {
        const float val = extract<SR>(src[from], delay) * w[wi];
        if (val > max_val) max_val = val;
    });
    const int to = dest_of<TY>(g, d);
    inputs[to] = aggregate(inputs[to], max_val, opcode);
}

__global__ void k_identity(int size, int history, const float* __restrict__ in, float* out) {
    const int nid = blockIdx.x * blockDim.x + threadIdx.x;
    if (nid >= size) return;
    shift_floats(out, size, history, nid, in[nid]);
}

class VpMaxModel : public Model {
  public:
    const char* name() const override { return "vp_max"; }
    OutputType output_type() const override { return OUT_FLOAT; }
    void build_matrix(State&, ConnState& cs) const override {
        if (cs.conn->second_order) throw SgError(cs.conn->str() + ": Unimplemented connection type!");
    }
    std::string learning_error(const Connection& c) const override {
        return toward_post_error(c, "vp_max");
    }
    bool learns(const Connection&) const override { return true; }
    void learn(State& st, ConnState& cs, const StepCtx& ctx) const override {
        if (cs.conn->convolutional) launch_learn_toward_post_conv(st, cs, ctx, 1.0f);
        else launch_learn_toward_post(st, cs, ctx);
    }
    void activate(State& st, ConnState& cs, const StepCtx& ctx) const override {
        const Connection& c = *cs.conn;
        const uint32_t* src = st.dev_output(c.from, word_index(c.delay, c.from->output_type));
        SG_DISPATCH_TYPE_SRC((int)c.type, (int)c.from->output_type,
            (k_activate_vp_max<TY, SR><<<blocks_for(cs.geom.n_dest, 128), 128, 0, ctx.stream>>>(
                cs.geom, src, c.delay, (int)c.opcode, cs.weights->df(), input_register(st, cs))));
        SG_LAUNCH_CHECK();
        ctx.count();
    }
    void update(State&, LayerState& ls, const StepCtx& ctx) const override {
        const Layer& l = *ls.layer;
        k_identity<<<blocks_for(l.size, 256), 256, 0, ctx.stream>>>(l.size, l.history(), ls.input->df(),
                                                                    ls.output->df());
        SG_LAUNCH_CHECK();
        ctx.count();
    }
};
SG_REGISTER_MODEL(VpMaxModel);

// sample (sample_attributes.cpp): the reference's template model, built only
// in feedforward structures.  Base synaptic input, output = 0 * input (its
// layer variable stays 0), and two per-synapse variables: var1 = weight * the
// source layer's "value" where "second weights" is set, var2 = 0 for
// "modulate" and 1 for "sub" connections.  Its updater for a
// non-convolutional connection is its activator (get_updaters returns
// activate_sample_map, sample_attributes.cpp:229-247): learning activates the
// connection once more into the input register and leaves the weights.  A
// convolutional one learns per kernel weight at the rate of the connection's
// "connection variable".
__global__ void k_scale(int size, int history, float scale, const float* __restrict__ in, float* out) {
    const int nid = blockIdx.x * blockDim.x + threadIdx.x;
    if (nid >= size) return;
    shift_floats(out, size, history, nid, scale * in[nid]);
}

class SampleModel : public Model {
  public:
    const char* name() const override { return "sample"; }
    OutputType output_type() const override { return OUT_FLOAT; }
    void build_layer(State& st, LayerState& ls) const override {
        if (ls.layer->structure->cluster_type != "feedforward")
            throw SgError("Error building attributes for " + ls.layer->str() +
                          ":\n  Cluster compatibility conflict detected!");
        ls.vars["neuron_var"] = st.add_array("neuron_var", 'f', ls.layer->size);
    }
    void build_matrix(State& st, ConnState& cs) const override {
        const Connection& c = *cs.conn;
        if (c.second_order) throw SgError(c.str() + ": Unimplemented connection type!");
        cs.params["connection variable"] = std::stof(c.parameter("connection variable", "1.0"));
        const size_t n = c.num_weights;
        Array* v1 = cs.vars["var1"] = st.add_array("var1", 'f', n, matrix_layout(c), c.matrix_rows, c.matrix_cols);
        Array* v2 = cs.vars["var2"] = st.add_array("var2", 'f', n, matrix_layout(c), c.matrix_rows, c.matrix_cols);
        if (c.parameter("second weights", "false") == "true") {
            const float val = std::stof(c.from->parameter("value", "1.0"));
            if (val < 0)
                throw SgError("Error initializing weight matrix for " + c.str() + " \n  Val cannot be negative!");
            for (size_t i = 0; i < n; ++i) v1->hf()[i] = cs.weights->hf()[i] * val;
        }
        if (c.opcode == OP_SUB)
            for (size_t i = 0; i < n; ++i) v2->hf()[i] = 1.0f;
    }
    std::string learning_error(const Connection& c) const override { return toward_post_error(c, "sample"); }
    bool learns(const Connection&) const override { return true; }
    void learn(State& st, ConnState& cs, const StepCtx& ctx) const override {
        if (cs.conn->convolutional) {       // update_sample_{convergent,divergent}_convolutional
            launch_learn_toward_post_conv(st, cs, ctx, cs.params.at("connection variable"));
            return;
        }
        launch_base_activator(st, cs, input_register(st, cs), ctx.stream);
        ctx.count();
    }
    void update(State&, LayerState& ls, const StepCtx& ctx) const override {
        const Layer& l = *ls.layer;
        k_scale<<<blocks_for(l.size, 256), 256, 0, ctx.stream>>>(l.size, l.history(), 0.0f, ls.input->df(),
                                                                 ls.output->df());
        SG_LAUNCH_CHECK();
        ctx.count();
    }
};
SG_REGISTER_MODEL(SampleModel);

}  // namespace sg
