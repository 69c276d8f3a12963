// The neural virtual machine models: nvm, nvm_heaviside, nvm_compare
// (src/core/state/impl/nvm_attributes.cpp, nvm_heaviside_attributes.cpp,
// nvm_compare_attributes.cpp).
//
// Each layer keeps three gates on the device -- activity, learning, noise --
// which start at 1, 0, 0 and which gate connections ("decay", "gate",
// "learning", "noise" on a subset window) overwrite as they activate.  Later
// activations of the same step see the new values, earlier ones last step's,
// exactly as the stream orders the launches.  "gated" and plastic
// activations run only while the gates are open (above 0.5) and, except for
// nvm_compare, for destinations whose context exceeds 0.5; plastic ones also
// learn inside the activation (weights move toward the state, or for
// nvm_compare are set from the true state).
#include "counter_rng.h"
#include "cuda_check.h"
#include "history.cuh"
#include "models.h"
#include "state.h"
#include "weight_init.h"

namespace sg {

enum { NVM_PLAIN = 0, NVM_GATED = 1, NVM_PLASTIC = 2, NVM_COMPARE = 3 };
enum { GATE_DECAY = 0, GATE_ACTIVITY = 1, GATE_LEARNING = 2, GATE_NOISE = 3 };

// Gate connection: every destination of the subset window reduces the same
// source window (min from 1 for "decay", max from 0 otherwise), so one
// thread computes the value the last destination writes.
template <int SR>
__global__ void k_nvm_gate(DGeom g, const uint32_t* __restrict__ src, int delay, int kind,
                           float* gates) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const bool decay = kind == GATE_DECAY;
    float gv = decay ? 1.0f : 0.0f;
    for (int fr = g.fr0; fr < g.fr1; ++fr)
        for (int fc = g.fc0; fc < g.fc1; ++fc) {
            const float v = extract<SR>(src[fr * g.from_cols + fc], delay);
            gv = decay ? ((gv < v) ? gv : v) : ((gv > v) ? gv : v);
        }
    if (kind == GATE_DECAY) gates[0] = 1.0f - gv;
    else if (kind == GATE_ACTIVITY) gates[0] = gv;
    else if (kind == GATE_LEARNING) gates[1] = gv;
    else gates[2] = gv;
}

template <int TY, int SR, int KIND>
__global__ void __launch_bounds__(128) k_nvm_activate(DGeom g, const uint32_t* __restrict__ src, int delay,
                                                      int opcode, float* w, float* inputs,
                                                      const float* __restrict__ gates,
                                                      const float* __restrict__ state,
                                                      const float* __restrict__ context,
                                                      const float* __restrict__ true_state,
                                                      float norm, int per_neuron, float tolerance) {
    const int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= g.n_dest) return;
    const float ag = gates[0], lg = gates[1];
    if (KIND == NVM_GATED && ag < 0.5f) return;
    if ((KIND == NVM_PLASTIC || KIND == NVM_COMPARE) && ag < 0.5f && lg < 0.5f) return;
    const int to = dest_of<TY>(g, d);
    if ((KIND == NVM_GATED || KIND == NVM_PLASTIC) && !(context[to] > 0.5f)) return;
    float sum = 0.0f;
    for_each_source<TY>(g, d, [&](int from, int wi) { sum += extract<SR>(src[from], delay) * w[wi]; });
    if (KIND == NVM_PLAIN || KIND == NVM_GATED) {
        inputs[to] = aggregate(inputs[to], sum, opcode);
    } else if (KIND == NVM_PLASTIC) {
        if (ag > 0.5f) inputs[to] = aggregate(inputs[to], sum, opcode);
        if (lg > 0.5f) {
            const float temp = state[to] - sum;
            const float nrm = norm * per_neuron;
            for_each_source<TY>(g, d, [&](int from, int wi) {
                w[wi] += extract<SR>(src[from], delay) * temp / nrm;
            });
        }
    } else {
        if (ag > 0.5f) {
            sum -= true_state[to] * ((tolerance * per_neuron) - 1);
            inputs[to] = ag * aggregate(inputs[to], sum, opcode);
        }
        if (lg > 0.5f) {
            const float temp = inputs[to] = true_state[to];
            for_each_source<TY>(g, d, [&](int from, int wi) {
                w[wi] = extract<SR>(src[from], delay) * temp / norm;
            });
        }
    }
}

// "context" connections: the one-to-one loop, into the context variable.
template <int SR>
__global__ void k_nvm_context(int n, const uint32_t* __restrict__ src, int delay, int opcode,
                              const float* __restrict__ w, const float* __restrict__ gates,
                              float* context) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || gates[0] < 0.5f) return;
    float sum = 0.0f;
    sum += extract<SR>(src[i], delay) * w[i];
    context[i] = aggregate(context[i], sum, opcode);
}

// nvm: state = input (+ gain * +-1 noise while the noise gate is set),
// output tanh(state); nvm_heaviside: state = gain * sign, output the step.
// Both reset the context to 1.
template <bool HEAVISIDE>
__global__ void k_nvm_update(int size, int history, const float* __restrict__ in, float* state,
                             float* context, float* out, const float* __restrict__ gates, float gain,
                             float noise_offset, unsigned long long seed, const int* __restrict__ tick) {
    const int nid = blockIdx.x * blockDim.x + threadIdx.x;
    if (nid >= size) return;
    const float noise = gates[2];
    const float r = noise != 0.0f ? rng_uniform(seed, (uint64_t)*tick, (uint64_t)nid) : 0.0f;
    if (!HEAVISIDE) {
        const float n = gain * (float)((r >= noise_offset) - (r < noise_offset));
        const float input = state[nid] = (float)((double)in[nid] + (noise != 0.0f ? (double)n : 0.0));
        context[nid] = 1.0f;
        shift_floats(out, size, history, nid, tanhf(input));
    } else {
        const float input = (float)((double)in[nid] + (noise != 0.0f ? (double)(r - noise_offset) : 0.0));
        state[nid] = gain * (float)((input > 0) - (input <= 0));
        context[nid] = 1.0f;
        shift_floats(out, size, history, nid, (float)(input > 0.0));
    }
}

__global__ void k_nvm_tick(int* counter) { *counter += 1; }

class NvmModel : public Model {
  public:
    NvmModel(const char* n, bool heaviside, bool compare) : name_(n), heaviside_(heaviside), compare_(compare) {}
    const char* name() const override { return name_; }
    OutputType output_type() const override { return OUT_FLOAT; }

    // NVMAttributes / NVMCompareAttributes constructors
    void build_layer(State& st, LayerState& ls) const override {
        const Layer& l = *ls.layer;
        const float off = (float)(1. - std::stof(l.parameter("noise offset", "0.5")));
        if (off > 1. || off < 0.) throw SgError("Noise offset must be in [0,1]!");
        ls.params["noise offset"] = off;
        ls.params["gain"] = std::stof(l.parameter("gain", "1."));
        ls.vars["state"] = st.add_array("state", 'f', l.size);
        ls.vars["context"] = st.add_array("context", 'f', l.size);
        float* ctx = ls.vars["context"]->hf();
        for (int i = 0; i < l.size; ++i) ctx[i] = 1.0f;
        if (compare_) {
            ls.vars["true_state"] = st.add_array("true_state", 'f', l.size);
            ls.params["tolerance"] = (float)(1. - std::stof(l.parameter("tolerance", "1.0")));
        }
        Array* gates = st.add_array("gates", 'f', 3);
        gates->hf()[0] = 1.0f;
        ls.internal["gates"] = gates;
        ls.internal["tick"] = st.add_array("tick", 'i', 1);
    }

    // Which activator a connection gets (nvm_attributes.cpp:163-187,
    // nvm_compare_attributes.cpp:60-69).
    int kind(const Connection& c) const {
        if (compare_ && c.plastic) return 10 + NVM_COMPARE;
        auto flag = [&](const char* k) { return c.parameter(k, "false") == "true"; };
        if (flag("decay")) return GATE_DECAY;
        if (flag("gate")) return GATE_ACTIVITY;
        if (flag("learning")) return GATE_LEARNING;
        if (flag("noise")) return GATE_NOISE;
        if (flag("context")) return 5;
        if (c.plastic) return 10 + NVM_PLASTIC;
        if (flag("gated")) return 10 + NVM_GATED;
        return 10 + NVM_PLAIN;
    }

    void build_matrix(State&, ConnState& cs) const override {
        const Connection& c = *cs.conn;
        if (c.second_order) throw SgError(c.str() + ": Unimplemented connection type!");
        cs.params["norm"] = std::stof(c.parameter("norm", "1.0"));
        const int k = kind(c);
        // learning inside the activation would update a shared kernel weight
        // from every destination at once; the context loop reads the source
        // layer's size of weights and context entries
        if ((k == 10 + NVM_PLASTIC || k == 10 + NVM_COMPARE) && c.convolutional)
            throw SgError(c.str() + ": plastic convolutional NVM connections are not supported");
        if (k == 5 && c.type != ONE_TO_ONE)
            throw SgError(c.str() + ": NVM context connections must be one to one");
    }

    void activate(State& st, ConnState& cs, const StepCtx& ctx) const override {
        const Connection& c = *cs.conn;
        LayerState& ls = *st.layer_state(c.to);
        const uint32_t* src = st.dev_output(c.from, word_index(c.delay, c.from->output_type));
        float* gates = ls.internal.at("gates")->df();
        const int sr = (int)c.from->output_type;
        const int k = kind(c);
        if (k <= GATE_NOISE) {
            if (c.dense_type != SUBSET) return;    // an empty subset window writes nothing
            switch (sr) {
                case 0: k_nvm_gate<0><<<1, 32, 0, ctx.stream>>>(cs.geom, src, c.delay, k, gates); break;
                case 1: k_nvm_gate<1><<<1, 32, 0, ctx.stream>>>(cs.geom, src, c.delay, k, gates); break;
                default: k_nvm_gate<2><<<1, 32, 0, ctx.stream>>>(cs.geom, src, c.delay, k, gates); break;
            }
            SG_LAUNCH_CHECK();
            ctx.count();
            return;
        }
        if (k == 5) {
            const int n = c.from->size;
            float* context = ls.var("context")->df();
            switch (sr) {
                case 0: k_nvm_context<0><<<blocks_for(n, 256), 256, 0, ctx.stream>>>(n, src, c.delay, (int)c.opcode, cs.weights->df(), gates, context); break;
                case 1: k_nvm_context<1><<<blocks_for(n, 256), 256, 0, ctx.stream>>>(n, src, c.delay, (int)c.opcode, cs.weights->df(), gates, context); break;
                default: k_nvm_context<2><<<blocks_for(n, 256), 256, 0, ctx.stream>>>(n, src, c.delay, (int)c.opcode, cs.weights->df(), gates, context); break;
            }
            SG_LAUNCH_CHECK();
            ctx.count();
            return;
        }
        const float* state = ls.var("state")->df();
        const float* context = ls.var("context")->df();
        const float* truth = compare_ ? ls.var("true_state")->df() : nullptr;
        const float tol = compare_ ? ls.params.at("tolerance") : 0.0f;
        const int per_neuron = (int)(c.num_weights / c.to->size);
        const unsigned blocks = blocks_for(cs.geom.n_dest, 128);
        float* reg = input_register(st, cs);
#define SG_NVM_ACT(KV)                                                                           \
    SG_DISPATCH_TYPE_SRC((int)c.type, sr,                                                        \
        (k_nvm_activate<TY, SR, KV><<<blocks, 128, 0, ctx.stream>>>(                             \
            cs.geom, src, c.delay, (int)c.opcode, cs.weights->df(), reg, gates, state, context,  \
            truth, cs.params.at("norm"), per_neuron, tol)))
        switch (k - 10) {
            case NVM_PLAIN: SG_NVM_ACT(NVM_PLAIN); break;
            case NVM_GATED: SG_NVM_ACT(NVM_GATED); break;
            case NVM_PLASTIC: SG_NVM_ACT(NVM_PLASTIC); break;
            default: SG_NVM_ACT(NVM_COMPARE); break;
        }
#undef SG_NVM_ACT
        SG_LAUNCH_CHECK();
        ctx.count();
    }

    void update(State&, LayerState& ls, const StepCtx& ctx) const override {
        const Layer& l = *ls.layer;
        const unsigned long long seed =
            l.config.has("seed") ? std::stoull(l.config.get("seed"))
                                 : (global_seed() ^ (0xC0FFEE1234567ULL * (unsigned long long)(l.index + 1)));
        int* tick = ls.internal.at("tick")->di();
        const unsigned blocks = blocks_for(l.size, 256);
        if (heaviside_)
            k_nvm_update<true><<<blocks, 256, 0, ctx.stream>>>(
                l.size, l.history(), ls.input->df(), ls.var("state")->df(), ls.var("context")->df(),
                ls.output->df(), ls.internal.at("gates")->df(), ls.params.at("gain"),
                ls.params.at("noise offset"), seed, tick);
        else
            k_nvm_update<false><<<blocks, 256, 0, ctx.stream>>>(
                l.size, l.history(), ls.input->df(), ls.var("state")->df(), ls.var("context")->df(),
                ls.output->df(), ls.internal.at("gates")->df(), ls.params.at("gain"),
                ls.params.at("noise offset"), seed, tick);
        SG_LAUNCH_CHECK();
        k_nvm_tick<<<1, 1, 0, ctx.stream>>>(tick);
        SG_LAUNCH_CHECK();
        ctx.count(2);
    }

  private:
    const char* name_;
    bool heaviside_, compare_;
};
static const bool sg_registered_nvm = register_model(new NvmModel("nvm", false, false));
static const bool sg_registered_nvm_heaviside = register_model(new NvmModel("nvm_heaviside", true, false));
static const bool sg_registered_nvm_compare = register_model(new NvmModel("nvm_compare", true, true));

}  // namespace sg
