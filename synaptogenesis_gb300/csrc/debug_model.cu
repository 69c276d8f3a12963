// The debug model (src/core/state/impl/debug_attributes.cpp:18-151): a
// checker.  Its layers' outputs are FLOAT and never written; its neuron
// variable "neuron_var" and its weight matrices' marker hold a dummy value
// (1.0); its neuron update, activators and updaters only check invariants:
// the dummy values, and that every destination, source and weight index the
// connection visits lies inside its layer or matrix.  The reference checks
// with device asserts; here a failed check increments a device error count
// (with the first failure's kind and index), and the host turns a nonzero
// count into an error when the run is synchronised (check_debug_errors).
#include <string>

#include "cuda_check.h"
#include "models.h"
#include "state.h"
#include "synapse.cuh"

namespace sg {

namespace {

// [0] failures, [1] first failure's kind, [2] its index
__device__ int g_debug_errors[3];

enum { DBG_NEURON_VAR = 1, DBG_TO = 2, DBG_FROM = 3, DBG_WEIGHT = 4, DBG_MARK = 5 };

__device__ __forceinline__ void debug_fail(int kind, long index) {
    if (atomicAdd(&g_debug_errors[0], 1) == 0) {
        g_debug_errors[1] = kind;
        g_debug_errors[2] = (int)index;
    }
}

constexpr float kDummy = 1.0f;

// attribute kernel: nid < size and neuron_var[nid] == DUMMY_VAL
__global__ void k_debug_neurons(int size, const float* __restrict__ neuron_var) {
    const int nid = blockIdx.x * blockDim.x + threadIdx.x;
    if (nid >= size) return;
    if (!(neuron_var[nid] == kDummy)) debug_fail(DBG_NEURON_VAR, nid);
}

// activators and updaters (CHECK_ATT / CHECK_TO / CHECK_FROM / CHECK_WEIGHT):
// every visit's indices within bounds -- weight indices within the device
// matrix (its layout pads fully connected and subset matrices to whole bands
// of destinations); the weights are read, nothing written
template <int TY>
__global__ void k_debug_synapses(DGeom g, long num_weights, float mark,
                                 const float* __restrict__ w) {
    const int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= g.n_dest) return;
    if (d == 0 && !(mark == kDummy)) debug_fail(DBG_MARK, 0);
    const int to = dest_of<TY>(g, d);
    if (to < 0 || to >= g.to_size) debug_fail(DBG_TO, to);
    float sink = 0.0f;
    for_each_source<TY>(g, d, [&](int from, int wi) {
        if (from < 0 || from >= g.from_size) debug_fail(DBG_FROM, from);
        if (wi < 0 || wi >= num_weights) debug_fail(DBG_WEIGHT, wi);
        else sink += __ldg(w + wi);
    });
    if (sink != sink) debug_fail(0, d);   // keeps the weight reads; never true for finite data
}

const char* kind_name(int k) {
    switch (k) {
        case DBG_NEURON_VAR: return "neuron_var differs from the dummy value";
        case DBG_TO: return "destination index outside the layer";
        case DBG_FROM: return "source index outside the layer";
        case DBG_WEIGHT: return "weight index outside the matrix";
        case DBG_MARK: return "weight matrix marker differs from the dummy value";
        default: return "weight is not a number";
    }
}

}  // namespace

void check_debug_errors() {
    int h[3] = {0, 0, 0};
    SG_CUDA(cudaMemcpyFromSymbol(h, g_debug_errors, sizeof(h)));
    if (h[0]) {
        int zero[3] = {0, 0, 0};
        SG_CUDA(cudaMemcpyToSymbol(g_debug_errors, zero, sizeof(zero)));
        throw SgError("debug model: " + std::to_string(h[0]) + " failed checks; first: " +
                      kind_name(h[1]) + " (index " + std::to_string(h[2]) + ")");
    }
}

class DebugModel : public Model {
  public:
    const char* name() const override { return "debug"; }
    OutputType output_type() const override { return OUT_FLOAT; }

    void build_layer(State& st, LayerState& ls) const override {
        Array* a = st.add_array("neuron_var", 'f', ls.layer->size);
        for (int i = 0; i < ls.layer->size; ++i) a->hf()[i] = kDummy;
        ls.vars["neuron_var"] = a;
    }
    // process_weight_matrix: the matrix's marker x = DUMMY_VAL
    void build_matrix(State&, ConnState& cs) const override {
        if (cs.conn->second_order)
            throw SgError(cs.conn->str() + ": second-order connections into debug layers are not "
                          "supported");
        cs.params["x"] = kDummy;
    }
    void activate(State&, ConnState& cs, const StepCtx& ctx) const override {
        check(cs, ctx);
    }
    void update(State&, LayerState& ls, const StepCtx& ctx) const override {
        k_debug_neurons<<<blocks_for(ls.layer->size, 256), 256, 0, ctx.stream>>>(
            ls.layer->size, ls.var("neuron_var")->df());
        SG_LAUNCH_CHECK();
        ctx.count();
    }
    bool learns(const Connection& c) const override { return true; }
    void learn(State&, ConnState& cs, const StepCtx& ctx) const override { check(cs, ctx); }

  private:
    static void check(ConnState& cs, const StepCtx& ctx) {
        const Connection& c = *cs.conn;
        const unsigned blocks = blocks_for(cs.geom.n_dest, 128);
        const float mark = cs.params.at("x");
        SG_DISPATCH_TYPE_SRC((int)c.type, 0,
            (k_debug_synapses<TY><<<blocks, 128, 0, ctx.stream>>>(
                cs.geom, (long)cs.weights->dev_count, mark, cs.weights->df())));
        SG_LAUNCH_CHECK();
        ctx.count();
    }
};
SG_REGISTER_MODEL(DebugModel);

}  // namespace sg
