// Engine: runs the per-timestep cycle of a State on one GPU.
//
// Step order follows the reference's single-threaded loop for "parallel"
// structures (src/core/engine/engine.cpp:226-315,
// src/core/engine/cluster/parallel_cluster.cpp:107-131):
//   1. input registers: environment input copied in, init configs applied,
//      other layers cleared (engine/instruction.cpp:3-30);
//   2. every connection's synaptic input, reading outputs of step t-1, in
//      network order and, per layer, in connection order;
//   3. every layer's neuron update (output history shift);
//   4. plasticity of plastic connections (if the learning flag is set);
//   5. output of the new step to the environment.
// All kernels go to one CUDA stream.  Host callbacks (the "callback" module,
// src/core/io/impl/callback_module.cpp:29-51) fill pinned input buffers and read
// pinned output buffers between steps.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <string>
#include <vector>

#include "callbacks.h"
#include "network.h"
#include "props.h"
#include "state.h"

namespace sg {

class Environment {
  public:
    explicit Environment(const Props& p) : config(p) {}
    Props config;
};

cudaStream_t engine_stream();

class Engine {
  public:
    Engine(Network* net, Environment* env, State* state) : net_(net), env_(env), state_(state) {}
    Props* run(const Props& args);

    static std::atomic<bool> interrupt_flag;
    static std::atomic<bool> running;

  private:
    struct ModLayer {
        Layer* layer;
        bool input = false, output = false;
        IoCallback fn = nullptr;
        int id = 0;
    };
    struct Module {
        std::vector<ModLayer> layers;
        bool clear = false;
        int start_delay = 0, cutoff = 0, rate = 1, curr = 0;
    };

    void build_modules();
    void enqueue_step(int step, bool last, bool learning);

    Network* net_;
    Environment* env_;
    State* state_;
    std::vector<Module> modules_;
    std::vector<Layer*> input_layers_, output_layers_;
    std::vector<float*> in_pinned_;      // per input layer (host)
    std::vector<float*> in_staging_;     // per input layer (device)
    std::vector<char> in_dirty_;
    std::vector<uint32_t*> out_pinned_;  // per output layer (host)
    std::vector<int> layer_io_;          // per layer: bit0 input, bit1 output
    long launches_ = 0;
};

}  // namespace sg
