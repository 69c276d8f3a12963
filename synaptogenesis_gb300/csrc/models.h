// Neural-model plugin API.
//
// The GB300 counterpart of the reference's Attributes plugin base
// (src/core/state/attributes.h:24-129) and its registry
// (src/core/state/neural_model_bank.cpp:21-83): a model registers under its
// JSON name with its output type, declares its per-neuron and per-synapse
// variables, initialises them on the host (the constructor and
// process_weight_matrix of the reference), and launches its CUDA kernels for
// synaptic input (get_activators), the neuron update (get_kernel) and
// plasticity (get_updaters).
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "network.h"

namespace sg {

class State;
struct LayerState;
struct ConnState;

// Per-step launch context handed to model kernels.
struct StepCtx {
    cudaStream_t stream;
    bool last_step;                        // input registers stay observable after it
    const std::vector<int>* layer_io;      // per layer: bit 0 input module, bit 1 output
    long* launches;                        // kernel launch counter
    bool is_input(const Layer& l) const { return layer_io && ((*layer_io)[l.index] & 1); }
    void count(long n = 1) const { if (launches) *launches += n; }
};

class Model {
  public:
    virtual ~Model() = default;
    virtual const char* name() const = 0;
    virtual OutputType output_type() const = 0;

    // Allocate model variables (State::add_array) and set host initial values.
    virtual void build_layer(State& st, LayerState& ls) const {}
    // Allocate and initialise per-synapse variables after the weights.
    virtual void build_matrix(State& st, ConnState& cs) const {}
    // Called once the state is on the device (device-only tables).
    virtual void prepare_device(State& st, ConnState& cs, cudaStream_t s) const {}

    // Synaptic input of one incoming connection (default: base activator).
    virtual void activate(State& st, ConnState& cs, const StepCtx& ctx) const;
    // True when the model's update computes this connection's input itself
    // (fused kernel); the engine then skips activate() for it.
    virtual bool fuses_input(State& st, const Connection& c, const StepCtx& ctx) const {
        return false;
    }
    // Before a step's synaptic input: work of several of the step's
    // connections into this model's layers that activate() would otherwise
    // launch one connection at a time.  A model that takes a connection's
    // share sets its ConnState::prologue_done (activate() clears it).
    virtual bool activate_prologue(State& st, const std::vector<ConnState*>& conns,
                                   const StepCtx& ctx) const {
        return false;
    }
    // Start of a step, before any synaptic input: per-layer buffers the
    // reference re-initialises every step (get_init_keys, cluster_node.cpp:46-50).
    virtual void begin_step(State& st, LayerState& ls, const StepCtx& ctx) const {}
    // Neuron update of one layer.
    virtual void update(State& st, LayerState& ls, const StepCtx& ctx) const = 0;
    // Update several layers of this model at once (their updates touch only
    // their own arrays); false: the engine updates them one by one.
    virtual bool update_group(State& st, const std::vector<LayerState*>& group,
                              const StepCtx& ctx) const {
        return false;
    }
    // Whether a plastic connection into this model has an updater.
    virtual bool learns(const Connection& c) const { return false; }
    // Non-empty when a run with learning cannot update this plastic
    // connection; the engine refuses to start with that message.
    virtual std::string learning_error(const Connection& c) const { return ""; }
    // Whole-run path: can this layer advance n steps on its own -- nothing
    // else reads or writes it between steps (the engine has checked that no
    // environment module touches it)?  If so, advance_alone runs the n steps
    // and leaves the state exactly as n calls of the per-step path would;
    // it returns the number of kernels launched.
    virtual bool can_advance_alone(State& st, const LayerState& ls) const { return false; }
    virtual long advance_alone(State& st, LayerState& ls, long n, cudaStream_t s) const {
        return 0;
    }
    virtual void learn(State& st, ConnState& cs, const StepCtx& ctx) const {}
};

const Model* find_model(const std::string& name);
bool register_model(const Model* m);
std::vector<std::string> model_names();

// Failed checks of the debug model's kernels since the last call, as an error
// (debug_model.cu).
void check_debug_errors();

// Register in the model's translation unit: SG_REGISTER_MODEL(MyModel);
#define SG_REGISTER_MODEL(CLS) \
    static const bool sg_registered_##CLS = ::sg::register_model(new CLS())

// Base activator launch (ACTIVATE_ALL(activate_base), kernel.cpp:217):
// inputs[to] = aggregate(inputs[to], sum_k extract(out[from], delay) * w).
void launch_base_activator(State& st, ConnState& cs, float* inputs, cudaStream_t s);
// Input register of the dendritic node a connection feeds.
float* input_register(State& st, const ConnState& cs);
// Second-order slave: modulates the host's per-step weight copy `so`.
void launch_second_order_slave(State& st, ConnState& cs, float* so, cudaStream_t s);
// Internal dendritic node: dst = aggregate(dst, src); src = trail.
void launch_dendrite_fold(int n, float* src, float* dst, int opcode, float trail, cudaStream_t s);

}  // namespace sg
