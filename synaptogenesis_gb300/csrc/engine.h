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
// pinned output buffers between steps.  Without host callbacks, pairs of steps
// are captured once into a CUDA graph and replayed.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <chrono>
#include <map>
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
    Engine(Network* net, Environment* env, State* state, const Props& args);
    ~Engine();

    // Runs n steps (n == 0: until interrupted).  Returns steps run.
    long step(long n);
    void synchronize();
    Props* report();
    cudaStream_t stream() const { return stream_; }

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
        bool active() const {
            return start_delay <= 0 && (cutoff == 0 || curr < cutoff) && curr % rate == 0;
        }
    };
    struct Prof {
        std::vector<std::pair<cudaEvent_t, cudaEvent_t>> events;
        long launches = 0;
    };

    // One step of a layer's synaptic input, in the order of the dendritic
    // tree's post-order walk (cluster_node.cpp:115-207).
    struct DendOp {
        enum Kind { CONN, SO_COPY, FOLD } kind;
        Connection* conn = nullptr;      // CONN
        Dendrite* node = nullptr;        // CONN: node fed; SO_COPY: second-order node; FOLD: parent
        Dendrite* child = nullptr;       // FOLD: internal child folded into node
    };
    void plan_dendrites(Dendrite* node, std::vector<DendOp>& ops);

    void build_modules();
    void feed_input();
    void report_output(long i);
    void enqueue_step(bool last);
    void launch_step(bool last);
    template <class F>
    void timed(const std::string& name, long kernels, F&& f);

    Network* net_;
    Environment* env_;
    State* state_;
    Props args_;
    cudaStream_t stream_;
    // Learning runs on a second stream, overlapping the next step's input and
    // activations: learn(c) at step t reads the destination's state of t and
    // writes c's arrays, and the only later work touching either before the
    // next learning is activate(c) at t+1 (the destination's update comes
    // after it), so learn_ev_[c] orders the two.  Joined back before a graph
    // capture ends, a run returns and the state is read.
    cudaStream_t side_ = nullptr;
    bool overlap_ = false, side_pending_ = false;
    cudaEvent_t fork_ev_ = nullptr, join_ev_ = nullptr;
    std::vector<cudaEvent_t> learn_ev_;
    std::vector<char> learn_pending_;
    void join_side();
    bool learning_ = true, suppress_ = false, verbose_ = false, use_graphs_ = true;
    bool profile_ = false;
    int env_rate_ = 1;
    std::vector<Module> modules_;
    std::vector<std::vector<DendOp>> dend_ops_;   // per layer, for layers with dendritic trees
    std::vector<int> layer_io_;          // per layer: bit0 input, bit1 output
    std::vector<Layer*> input_layers_, output_layers_;
    std::vector<float*> in_pinned_, in_staging_;
    std::vector<char> in_dirty_;
    std::vector<uint32_t*> out_pinned_;
    struct Graph {
        std::vector<void*> sig;          // output buffers the graph was captured with
        cudaGraphExec_t exec = nullptr;
        long launches = 0;
    };
    std::vector<Graph> graphs_;          // one per ping-pong placement
    int graph_steps_ = 16;               // steps per captured graph (even)
    bool alone_ = false;                 // every layer advances whole runs on its own
    bool ordered_ = false;               // a sequential or feedforward structure sets the step order
    long launches_ = 0, steps_ = 0;
    double wall_s_ = 0.0;
    float device_ms_ = 0.0f;
    std::map<std::string, Prof> prof_;
};

}  // namespace sg
