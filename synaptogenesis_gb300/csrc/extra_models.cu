// The reference's smaller neural models: binary threshold, the two
// rate-encoding variants, perceptron, sine generator and Poisson generator
// (src/core/state/impl/*_attributes.cpp).  Each update is one thread per
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
    // The reference's updater reads the source outputs, which it binds only
    // within feedforward structures (synapse_data.cpp:36-51); in the parallel
    // structures supported here its source pointer is null.
    std::string learning_error(const Connection&) const override {
        return "perceptron learning reads source outputs that the reference binds only in "
               "feedforward structures (set \"plastic\": false or run without learning)";
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

}  // namespace sg
