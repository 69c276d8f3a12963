// Simulation state: every neuron and synapse array of a network.
//
// Each array has a host mirror in the reference's host layout (what the C-ABI
// getters hand out, src/core/state/state.cpp:706-764) and a device copy in the
// GPU layout (per-synapse arrays transposed so consecutive destinations are
// contiguous, src/core/state/weight_matrix.cpp:192-228).  Device copies live in
// one arena allocation.  Like the reference (state.cpp:259-323), handing out
// host pointers moves the state to the host, and the next run moves it back.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "network.h"
#include "synapse.cuh"

namespace sg {

enum ArrayLayout {
    LAYOUT_PLAIN = 0,        // same layout on host and device
    LAYOUT_MATRIX = 1,       // host [rows][cols] <-> device [cols][rows]
    LAYOUT_SOURCE = 2,       // host array of num_weights, device keeps the first from_size
    LAYOUT_BANDED = 3,       // host [rows][cols] <-> device banded_index(row, col, cols)
};

struct Array {
    std::string name;
    char dtype = 'f';        // 'f' float, 'i' int32, 'u' output word
    size_t count = 0;        // host elements
    size_t dev_count = 0;    // device elements
    ArrayLayout layout = LAYOUT_PLAIN;
    int rows = 1, cols = 1;
    std::vector<uint32_t> host;
    void* dev = nullptr;
    size_t dev_offset = 0;
    bool scratch = false;    // device-only working buffer: never uploaded or downloaded

    float* hf() { return reinterpret_cast<float*>(host.data()); }
    int32_t* hi() { return reinterpret_cast<int32_t*>(host.data()); }
    uint32_t* hu() { return host.data(); }
    float* df() const { return static_cast<float*>(dev); }
    int32_t* di() const { return static_cast<int32_t*>(dev); }
    uint32_t* du() const { return static_cast<uint32_t*>(dev); }
};

// Device layout of a connection's per-synapse matrices: banded for fully
// connected and subset connections, transposed otherwise.
ArrayLayout matrix_layout(const Connection& c);

// Device element of host element `i` of a per-synapse array.
size_t device_index(const Array& a, size_t i);

struct LayerState {
    Layer* layer = nullptr;
    Array* input = nullptr;
    Array* output = nullptr;
    std::map<std::string, Array*> vars;
    std::map<std::string, Array*> internal;   // model buffers not exposed by the getters
    std::map<std::string, float> params;      // model scalars (e.g. game_of_life rules)
    Array* var(const std::string& k) const;
};

struct ConnState {
    Connection* conn = nullptr;
    Array* weights = nullptr;
    Array* delays = nullptr;               // per-synapse delays (models that use them)
    std::map<std::string, Array*> vars;
    std::map<std::string, float> params;
    DGeom geom{};
    // Per-source table of the last (up to 32) visits in serial order, device
    // weight indices, plus the visit count per source (time-since-spike rule).
    Array* last_visits = nullptr;
    Array* visit_counts = nullptr;
    // Per source: a summary of the delays its last visits read (device only,
    // recomputed after every upload; see k_iz_delay_summary).
    Array* delay_summary = nullptr;
    // Distances computed for a distance callback, reused by distance-based
    // delays like the reference's cached distances (weight_matrix.cpp:1372-1374).
    std::vector<float> cached_distances;
    // Launch plan a model keeps for this connection's device arrays (built at
    // the first step, once the arena exists).
    std::shared_ptr<void> device_plan;
    bool device_plan_tried = false;
    // Input register of the dendritic node the connection feeds.
    int reg = 0;
    // This step's per-connection prologue ran with other connections'
    // (Model::activate_prologue); the connection's activation clears it.
    bool prologue_done = false;
    // Fully connected or subset trace connection that never learns: the
    // activator's per-synapse weight w * (R * w_stp), constant during a run
    // and refilled after every upload (device only, same layout as the
    // weights).
    Array* eff_weights = nullptr;
    // Fully connected or subset trace connection from a BIT layer: its
    // delays as bytes for the TMA activator, [band][row * 8 + lane] with each
    // band's rows padded to 16 bytes (device only, refilled after every
    // upload).
    Array* delays8 = nullptr;
    // Second-order host: the per-step copy of its weights that the slaves
    // modulate and the host's activation reads (device only, same layout as
    // the weights; weight_matrix.cpp:79-80).
    Array* so_weights = nullptr;
    // Second-order slave whose device layout differs from the host's (subset
    // windows of another shape): host device index of each slave device index.
    Array* so_remap = nullptr;
    // Sparse connection: synapses per destination ([to_size]) and each
    // synapse's source (same layout as the weights).
    Array* sparse_nonzero = nullptr;
    Array* sparse_from = nullptr;
    Array* var(const std::string& k) const;
};

class State {
  public:
    explicit State(Network* net);
    ~State();

    Network* network;
    std::vector<std::unique_ptr<LayerState>> layers;      // network order
    std::vector<std::unique_ptr<ConnState>> conns;        // connection order

    LayerState* layer_state(Layer* l) { return layers[l->index].get(); }
    ConnState* conn_state(Connection* c) { return conns[c->index].get(); }

    // Allocation helpers used by models while the state is being built.
    Array* add_array(const std::string& name, char dtype, size_t count,
                     ArrayLayout layout = LAYOUT_PLAIN, int rows = 1, int cols = 1,
                     size_t dev_count = 0);
    void remove_array(Array* a);

    // Host <-> device movement.
    void to_device(cudaStream_t stream);     // uploads if the host copy is newer
    void to_host(cudaStream_t stream);       // downloads if the device copy is newer
    bool on_host() const { return on_host_; }
    void mark_device_newer() { on_host_ = false; }

    // Output word `word` of a layer on the device.
    uint32_t* dev_output(Layer* l, int word = 0) {
        auto* ls = layer_state(l);
        return ls->output->du() + (size_t)word * l->size;
    }
    size_t device_bytes() const { return arena_bytes_; }
    size_t host_bytes() const;

    // Save / load in the reference's record format (state.cpp:365-447).
    void save(const std::string& path);
    void load(const std::string& path);

  private:
    void build();
    void allocate_device();
    std::vector<std::unique_ptr<Array>> arrays_;
    void* arena_ = nullptr;
    size_t arena_bytes_ = 0;
    // device buffer for the layout conversions of uploads and downloads
    uint32_t* stage_ = nullptr;
    // host arrays registered with CUDA (page-locked in place) for the copies
    std::vector<void*> registered_;
    bool on_host_ = true;
};

// Layout conversions on the device (csrc/layout.cu): host [rows][cols] to and
// from the banded device layout, and a [rows][cols] -> [cols][rows] transpose.
void launch_to_bands(const uint32_t* in, uint32_t* out, int rows, int cols, size_t dev_count,
                     cudaStream_t s);
void launch_from_bands(const uint32_t* in, uint32_t* out, int rows, int cols, size_t dev_count,
                       cudaStream_t s);
void launch_transpose(const uint32_t* in, uint32_t* out, int rows, int cols, cudaStream_t s);

DGeom make_geom(const Connection& c);

// Seed of a layer's init-config noise: its "seed", else derived from the
// global seed and the layer's index.
uint64_t noise_seed(const Layer& l);

// Serial-order enumeration of a connection's visits, host layout weight
// indices: f(row, to_index, from_index, weight_index, pre_wrap_row, pre_wrap_col).
// Shared by the index/distance/delay initialisers and the visit tables.
template <class F>
void enumerate_visits(const Connection& c, F&& f);

}  // namespace sg

#include "visits.inl"
