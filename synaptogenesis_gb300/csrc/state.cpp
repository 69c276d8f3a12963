#include "counter_rng.h"
#include "state.h"
#include "iz_cols_tma.cuh"

#include <algorithm>
#include <cstring>
#include <fstream>
#include <functional>

#include "cuda_check.h"
#include "models.h"
#include "weight_init.h"

namespace sg {

Array* LayerState::var(const std::string& k) const {
    if (k == "input") return input;
    if (k == "output") return output;
    auto it = vars.find(k);
    if (it == vars.end())
        throw SgError("Failed to retrieve neuron data \"" + k + "\" in Attributes!");
    return it->second;
}

Array* ConnState::var(const std::string& k) const {
    if (k == "weights") return weights;
    if (k == "delays" && delays) return delays;
    auto it = vars.find(k);
    if (it == vars.end())
        throw SgError("Failed to retrieve data \"" + k + "\" in WeightMatrix for connection:" +
                      conn->str());
    return it->second;
}

DGeom make_geom(const Connection& c) {
    DGeom g{};
    g.type = (int)c.type;
    g.conv = c.convolutional ? 1 : 0;
    g.from_rows = c.from->rows; g.from_cols = c.from->cols; g.from_size = c.from->size;
    g.to_rows = c.to->rows; g.to_cols = c.to->cols; g.to_size = c.to->size;
    const Arbor& a = c.arbor;
    g.rf = a.row_field; g.cf = a.col_field; g.rs = a.row_stride; g.cs = a.col_stride;
    g.rsp = a.row_spacing; g.csp = a.col_spacing; g.ro = a.row_offset; g.co = a.col_offset;
    g.wrap = a.wrap ? 1 : 0;
    const SubsetCfg& s = c.subset;
    g.fr0 = s.fr0; g.fr1 = s.fr1; g.fc0 = s.fc0; g.fc1 = s.fc1; g.tr0 = s.tr0; g.tc0 = s.tc0;
    g.tk_cols = s.tc1 - s.tc0;
    g.tk_size = s.to_size();
    g.n_dest = c.dest_count();
    g.kmax = c.sparse_table ? c.sparse_table->kmax : 0;
    // Range of source coordinates before wrapping, per axis.
    g.wrap_fast = 0;
    if (c.type == CONVERGENT || c.type == DIVERGENT) {
        auto range = [&](int to_n, int stride, int spacing, int offset, int field, int from_n) {
            long lo = 1L << 40, hi = -(1L << 40);
            for (int t = 0; t < to_n; ++t) {
                long a, b;
                if (c.type == CONVERGENT) {
                    a = (long)t * stride + (long)spacing * offset;
                    b = a + (long)(field - 1) * spacing;
                } else {
                    a = (t + spacing * (-offset - field + stride)) / stride;
                    b = a + (spacing * (field - stride) / stride);
                }
                lo = std::min(lo, a);
                hi = std::max(hi, b);
            }
            return lo >= -(long)from_n && hi < 2L * from_n;
        };
        g.wrap_fast = range(c.to->rows, a.row_stride, a.row_spacing, a.row_offset, a.row_field,
                            c.from->rows) &&
                      range(c.to->cols, a.col_stride, a.col_spacing, a.col_offset, a.col_field,
                            c.from->cols);
    }
    return g;
}

State::State(Network* net) : network(net) { build(); }

State::~State() {
    for (void* p : registered_) cudaHostUnregister(p);
    if (stage_) cudaFree(stage_);
    if (arena_) cudaFree(arena_);
}

void State::remove_array(Array* a) {
    if (arena_) throw SgError("state arrays cannot be removed after device allocation");
    arrays_.erase(std::remove_if(arrays_.begin(), arrays_.end(),
                                 [a](const std::unique_ptr<Array>& p) { return p.get() == a; }),
                  arrays_.end());
}

Array* State::add_array(const std::string& name, char dtype, size_t count, ArrayLayout layout,
                        int rows, int cols, size_t dev_count) {
    if (arena_) throw SgError("state arrays cannot be added after device allocation");
    auto a = std::make_unique<Array>();
    a->name = name;
    a->dtype = dtype;
    a->count = count;
    if (!dev_count && layout == LAYOUT_BANDED)     // whole bands of destinations
        dev_count = (size_t)((rows + kBand - 1) / kBand) * kBand * (size_t)cols;
    a->dev_count = dev_count ? dev_count : count;
    a->layout = layout;
    a->rows = rows;
    a->cols = cols;
    a->host.assign(count, 0u);
    arrays_.push_back(std::move(a));
    return arrays_.back().get();
}

uint64_t noise_seed(const Layer& l) {
    Props* init = l.config.child("init config");
    return (init && init->has("seed")) ? std::stoull(init->get("seed"))
                                       : (global_seed() ^ (0xA5A5ULL * (uint64_t)(l.index + 1)));
}

void State::build() {
    // a sparse connection is compacted anew from this state's weights
    for (auto& cp : network->connections) {
        Connection* c = cp.get();
        if (!c->sparse) continue;
        c->type = c->dense_type;
        c->num_weights = c->dense_num_weights;
        c->matrix_rows = c->dense_rows;
        c->matrix_cols = c->dense_cols;
        c->sparse_table.reset();
    }
    for (auto& lp : network->layers) {
        Layer* l = lp.get();
        auto ls = std::make_unique<LayerState>();
        ls->layer = l;
        // one register per dendritic node with its own register
        // (attributes.cpp:21-26); get_neuron_data("input") returns them all
        ls->input = add_array("input", 'f', (size_t)l->registers * l->size);
        ls->output = add_array("output", 'u', (size_t)l->history() * l->size);
        // init-config noise: the layer's step counter and dispatch ticket
        // (two 64-bit words, kept with the state so that a later run continues
        // the draws) and the per-neuron Poisson rates of "random": rates
        // uniform in [0, rate) like the reference's fRand
        // (instruction.h:255-268), drawn from the layer's noise seed
        if (Props* init = l->config.child("init config")) {
            const std::string t = init->get("type", "normal");
            if (t != "flat") ls->internal["noise step"] = add_array("noise step", 'i', 4);
            if (t == "poisson" && init->get_bool("random", false)) {
                Array* rates = add_array("noise rates", 'f', l->size);
                const float rate = 0.001f * init->get_float("rate", 1.0f);
                const uint64_t seed = noise_seed(*l);
                for (int i = 0; i < l->size; ++i)
                    rates->hf()[i] = rng_uniform(seed, RNG_NOISE_RATE, (uint64_t)i) * rate;
                ls->internal["noise rates"] = rates;
            }
        }
        find_model(l->model)->build_layer(*this, *ls);
        layers.push_back(std::move(ls));
    }
    for (auto& cp : network->connections) {
        Connection* c = cp.get();
        auto cs = std::make_unique<ConnState>();
        cs->conn = c;
        cs->geom = make_geom(*c);
        cs->weights = add_array("weights", 'f', c->num_weights, matrix_layout(*c), c->matrix_rows,
                                c->matrix_cols);
        cs->reg = c->node ? c->node->reg : 0;
        if (c->second_order_host) {
            cs->so_weights = add_array("second order weights", 'f', c->num_weights, matrix_layout(*c),
                                       c->matrix_rows, c->matrix_cols);
            cs->so_weights->scratch = true;
        }
        conns.push_back(std::move(cs));
    }
    // Slaves share the host's flat weight index; where their device layouts
    // differ, a table maps the slave's device positions to the host's.
    for (auto& cp : network->connections) {
        Connection* c = cp.get();
        if (!c->second_order_slave || c->convolutional) continue;
        const Array& hw = *conns[c->node->host->index]->weights;
        const Array& sw = *conns[c->index]->weights;
        if (hw.layout == sw.layout && hw.rows == sw.rows && hw.cols == sw.cols) continue;
        Array* remap = add_array("second order remap", 'i', sw.dev_count);
        for (size_t i = 0; i < (size_t)c->num_weights; ++i)
            remap->hi()[device_index(sw, i)] = (int32_t)device_index(hw, i);
        conns[c->index]->so_remap = remap;
    }
    // Weight initialisation and model processing follow the reference's order:
    // all matrices of a layer are created with the layer's attributes
    // (attributes.cpp:31-36), then processed (state.cpp:98-106).
    for (auto& lp : network->layers) {
        for (Connection* c : lp->inputs) {
            init_weights(*this, *conns[c->index]);
            if (c->sparse) sparsify(*this, *conns[c->index]);
        }
        for (Connection* c : lp->inputs)
            find_model(lp->model)->build_matrix(*this, *conns[c->index]);
    }
}

size_t State::host_bytes() const {
    size_t n = 0;
    for (auto& a : arrays_)
        if (!a->scratch) n += std::min(a->count, a->dev_count) * 4;
    return n;
}

void State::allocate_device() {
    size_t off = 0;
    for (auto& a : arrays_) {
        a->dev_offset = off;
        off += (a->dev_count * 4 + 255) / 256 * 256;
    }
    arena_bytes_ = std::max<size_t>(off, 256);
    SG_CUDA(cudaMalloc(&arena_, arena_bytes_));
    SG_CUDA(cudaMemset(arena_, 0, arena_bytes_));
    // staging for the arrays whose device layout differs from the host's
    size_t stage = 0;
    for (auto& a : arrays_) {
        if (a->scratch || a->dev_count == 0) continue;
        if (a->layout == LAYOUT_BANDED) stage = std::max(stage, a->count);
        else if (a->layout == LAYOUT_MATRIX && a->rows > 1 && a->cols > 1)
            stage = std::max(stage, a->count);
    }
    if (stage) SG_CUDA(cudaMalloc(&stage_, stage * sizeof(uint32_t)));
    // page-lock the host mirrors in place, so that the copies are direct DMA;
    // where the system refuses, copies go through the driver's staging
    for (auto& a : arrays_) {
        if (a->scratch || a->host.empty()) continue;
        if (cudaHostRegister(a->host.data(), a->host.size() * sizeof(uint32_t),
                             cudaHostRegisterDefault) == cudaSuccess)
            registered_.push_back(a->host.data());
        else
            cudaGetLastError();
    }
    // the engine's streams are non-blocking: nothing orders them after this
    // legacy-stream memset, so it completes before any upload or kernel
    SG_CUDA(cudaDeviceSynchronize());
    for (auto& a : arrays_) a->dev = static_cast<char*>(arena_) + a->dev_offset;
    for (auto& cs : conns)
        if (cs->sparse_nonzero) {
            cs->geom.nz = cs->sparse_nonzero->di();
            cs->geom.sfrom = cs->sparse_from->di();
        }
}

static bool needs_transpose(const Array& a) {
    return a.layout == LAYOUT_MATRIX && a.rows > 1 && a.cols > 1;
}

ArrayLayout matrix_layout(const Connection& c) {
    return (c.type == FULLY_CONNECTED || c.type == SUBSET) ? LAYOUT_BANDED : LAYOUT_MATRIX;
}

size_t device_index(const Array& a, size_t i) {
    if (a.layout == LAYOUT_BANDED) return (size_t)banded_index(i / a.cols, i % a.cols, a.cols);
    if (needs_transpose(a)) return (i % a.cols) * a.rows + i / a.cols;
    return i;
}

void State::to_device(cudaStream_t stream) {
    if (!arena_) allocate_device();
    if (!on_host_) return;
    // Everything on the engine's stream (a pageable cudaMemcpy may return
    // before its DMA lands and would not be ordered with that stream's
    // kernels).  Arrays with another device layout go through the staging
    // buffer and a conversion kernel; the stream orders each conversion
    // before the next copy into the buffer.
    for (auto& a : arrays_) {
        if (a->dev_count == 0 || a->scratch) continue;
        const uint32_t* src = a->host.data();
        if (a->layout == LAYOUT_BANDED) {
            SG_CUDA(cudaMemcpyAsync(stage_, src, a->count * 4, cudaMemcpyHostToDevice, stream));
            launch_to_bands(stage_, a->du(), a->rows, a->cols, a->dev_count, stream);
        } else if (needs_transpose(*a)) {
            SG_CUDA(cudaMemcpyAsync(stage_, src, a->count * 4, cudaMemcpyHostToDevice, stream));
            launch_transpose(stage_, a->du(), a->rows, a->cols, stream);
        } else {
            const size_t n = std::min(a->dev_count, a->count);
            SG_CUDA(cudaMemcpyAsync(a->dev, src, n * 4, cudaMemcpyHostToDevice, stream));
        }
    }
    for (auto& cp : network->connections)
        find_model(cp->to->model)->prepare_device(*this, *conns[cp->index], stream);
    SG_CUDA(cudaStreamSynchronize(stream));
    on_host_ = false;
}

void State::to_host(cudaStream_t stream) {
    if (on_host_) return;
    SG_CUDA(cudaStreamSynchronize(stream));
    check_iz_cols_errors();
    check_debug_errors();
    for (auto& a : arrays_) {
        if (a->dev_count == 0 || a->scratch) continue;
        const size_t n = std::min(a->dev_count, a->count);
        if (a->layout == LAYOUT_BANDED) {
            launch_from_bands(a->du(), stage_, a->rows, a->cols, a->dev_count, stream);
            SG_CUDA(cudaMemcpyAsync(a->host.data(), stage_, a->count * 4, cudaMemcpyDeviceToHost,
                                    stream));
        } else if (needs_transpose(*a)) {
            // device [cols][rows] -> host [rows][cols]
            launch_transpose(a->du(), stage_, a->cols, a->rows, stream);
            SG_CUDA(cudaMemcpyAsync(a->host.data(), stage_, a->count * 4, cudaMemcpyDeviceToHost,
                                    stream));
        } else {
            SG_CUDA(cudaMemcpyAsync(a->host.data(), a->dev, n * 4, cudaMemcpyDeviceToHost, stream));
        }
    }
    SG_CUDA(cudaStreamSynchronize(stream));
    on_host_ = true;
}

// ---------------------------------------------------------------------------
// Save / load: a sequence of records [hash, type-hash, bytes][bytes of data],
// keyed like the reference (PointerKey, util/resources/pointer.h:9-30): the
// owner hash is std::hash of "structure/layer" or of the connection's str(),
// the type hash is std::hash of the variable name.
// ---------------------------------------------------------------------------
namespace {
struct Rec {
    size_t hash, type, bytes;
    Array* arr;
};
}  // namespace

static std::vector<Rec> records(State& st) {
    std::hash<std::string> h;
    std::vector<Rec> out;
    for (auto& ls : st.layers) {
        size_t owner = h(ls->layer->structure->name + "/" + ls->layer->name);
        out.push_back({owner, h("input"), ls->input->count * 4, ls->input});
        out.push_back({owner, h("output"), ls->output->count * 4, ls->output});
        for (auto& kv : ls->vars) out.push_back({owner, h(kv.first), kv.second->count * 4, kv.second});
    }
    for (auto& cs : st.conns) {
        size_t owner = h(cs->conn->str());
        out.push_back({owner, h("weights"), cs->weights->count * 4, cs->weights});
        if (cs->delays) out.push_back({owner, h("delays"), cs->delays->count * 4, cs->delays});
        for (auto& kv : cs->vars) out.push_back({owner, h(kv.first), kv.second->count * 4, kv.second});
    }
    std::sort(out.begin(), out.end(), [](const Rec& a, const Rec& b) {
        return a.hash == b.hash ? a.type < b.type : a.hash < b.hash;
    });
    return out;
}

void State::save(const std::string& path) {
    to_host(0);
    std::ofstream f(path, std::ios::binary);
    if (!f) throw SgError("Error writing state to file!");
    for (auto& r : records(*this)) {
        if (r.bytes == 0) continue;
        size_t key[3] = {r.hash, r.type, r.bytes};
        f.write(reinterpret_cast<const char*>(key), sizeof(key));
        f.write(reinterpret_cast<const char*>(r.arr->host.data()), r.bytes);
        if (!f) throw SgError("Error writing state to file!");
    }
}

void State::load(const std::string& path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw SgError("Could not open file: " + path);
    to_host(0);
    auto recs = records(*this);
    for (;;) {
        size_t key[3];
        if (!f.read(reinterpret_cast<char*>(key), sizeof(key))) break;
        // records are matched on (owner, variable) like the reference's
        // PointerKey; ones this state does not hold (a transposed weight
        // copy, distances, sparse index arrays) are skipped, as the
        // reference skips unknown ones
        const Rec* target = nullptr;
        for (auto& r : recs)
            if (r.hash == key[0] && r.type == key[1]) target = &r;
        if (!target) {
            f.ignore(key[2]);
            continue;
        }
        // the reference resizes such an array (sparse matrices); every array
        // here has the size its network fixes
        if (target->bytes != key[2])
            throw SgError("State record '" + target->arr->name + "' holds " +
                          std::to_string(key[2]) + " bytes; the network's array has " +
                          std::to_string(target->bytes));
        if (!f.read(reinterpret_cast<char*>(target->arr->host.data()), key[2]))
            throw SgError("Error reading data from file!");
    }
    on_host_ = true;
}

}  // namespace sg
