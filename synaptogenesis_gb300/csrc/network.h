// Network / Structure / Layer / Connection built from the reference's JSON
// schema.  Field meanings, defaults and quirks follow
//   src/core/network/network.cpp:5-217      (structure resolution)
//   src/core/network/layer_config.cpp:11-33 (layer fields)
//   src/core/network/connection_config.cpp:8-45, 112-134, 207-257
//   src/core/network/connection.cpp:7-61, 224-248 (weight counts, matrix shape)
#pragma once
#include <memory>
#include <string>
#include <vector>

#include "props.h"

namespace sg {

enum OutputType { OUT_FLOAT = 0, OUT_BIT = 1, OUT_INT = 2 };
// SPARSE is internal (util/constants.h:71-78): a "sparse" connection takes it
// when its state is built and its zero weights are compacted away.
enum ConnType { FULLY_CONNECTED = 0, SUBSET = 1, ONE_TO_ONE = 2, CONVERGENT = 3, DIVERGENT = 4,
                SPARSE = 5 };
enum Opcode {
    OP_ADD = 0, OP_SUB, OP_MULT, OP_DIV, OP_POOL, OP_REWARD, OP_MODULATE, OP_GAP,
    OP_ADD_HEAVISIDE, OP_SUB_HEAVISIDE, OP_MULT_HEAVISIDE
};

ConnType parse_conn_type(const std::string& s);
Opcode parse_opcode(const std::string& s);
const char* conn_type_name(ConnType t);
const char* opcode_name(Opcode o);

// Words of output history needed to serve a delay (util/constants.h:24-37).
inline int word_index(int delay, OutputType t) { return t == OUT_BIT ? delay / 32 : delay; }

struct Arbor {
    int row_field = 0, col_field = 0, row_stride = 0, col_stride = 0;
    int row_spacing = 0, col_spacing = 0, row_offset = 0, col_offset = 0;
    bool wrap = false;
    int kernel() const { return row_field * col_field; }
};

struct SubsetCfg {
    int fr0 = 0, fr1 = 0, fc0 = 0, fc1 = 0, tr0 = 0, tr1 = 0, tc0 = 0, tc1 = 0;
    int from_size() const { return (fr1 - fr0) * (fc1 - fc0); }
    int to_size() const { return (tr1 - tr0) * (tc1 - tc0); }
};

struct Structure;
struct Connection;
struct Layer;

// Compacted synapse table of a sparse connection (weight_matrix.cpp:510-651,
// 253-338): destination to keeps its nonzero[to] synapses first in row
// to of a [to_size][kmax] matrix, in the dense matrix's order; -1 pads.
struct SparseTable {
    int kmax = 0;
    std::vector<int> nonzero;             // [to_size]
    std::vector<int> from;                // [to_size * kmax] source index, wrapped
    // Indices before wrapping (what distances are measured from), -1 pads.
    std::vector<int> from_row, from_col, to_row, to_col;
};

// A node of a layer's dendritic tree (network/dendritic_node.cpp:5-146).
// The root owns input register 0; every internal node gets its own register,
// one past the highest register of the tree when it is created (so registers
// follow the pre-order of the layer's "dendrites" config); connections
// aggregate into the register of the node they name.  Children keep creation
// order: the internal nodes of the layer config first, then the connections
// in the order they are created.  A second-order node holds no internal
// children; its first connection is the host, whose weights the other
// connections (slaves) modulate every step, and the host is not a child.
struct Dendrite {
    std::string name;
    Layer* layer = nullptr;
    Dendrite* parent = nullptr;
    int reg = 0;
    Opcode opcode = OP_ADD;        // aggregation into the parent's register
    bool second_order = false;
    float init = 0.0f;             // register value after each aggregation
    struct Child {
        Dendrite* node;            // internal child, or
        Connection* conn;          // leaf connection
    };
    std::vector<Child> children;
    Connection* host = nullptr;    // second-order host connection
    std::vector<std::unique_ptr<Dendrite>> owned;

    int max_register() const;
    std::string str() const;
};

struct Layer {
    Props config;
    std::string name;
    Structure* structure = nullptr;
    std::string model;
    int rows = 0, cols = 0, size = 0;
    bool plastic = false;
    OutputType output_type = OUT_FLOAT;
    std::vector<Connection*> inputs;    // in JSON order
    std::vector<Connection*> outputs;
    int index = 0;                      // position in network order
    std::unique_ptr<Dendrite> root;     // dendritic tree (register 0)
    int registers = 1;                  // input registers: max register + 1

    // Nodes in breadth-first order, root first (layer.cpp:62-77).
    std::vector<Dendrite*> dendrites() const;
    Dendrite* dendrite(const std::string& name) const;      // nullptr if absent
    bool has_dendrites() const { return registers > 1; }   // internal nodes

    int max_delay() const;
    int history() const { return 1 + word_index(max_delay(), output_type); }
    std::string parameter(const std::string& k, const std::string& def) const {
        return config.get(k, def);
    }
    std::string str() const;
};

struct Connection {
    Props config;
    std::string name;
    Layer* from = nullptr;
    Layer* to = nullptr;
    bool plastic = true;
    bool recurrent = false;             // ignored when ordering a structure's layers
    int delay = 0;
    float max_weight = 1.0f;
    ConnType type = FULLY_CONNECTED;
    Opcode opcode = OP_ADD;
    bool convolutional = false;
    Arbor arbor;
    SubsetCfg subset;
    bool sparse = false;                // "sparse": compacted at state build
    bool randomized = false;            // "randomized projection" (also sparse)
    // Set while a state is built from this network, like the reference's
    // Connection::sparsify (connection.cpp:219-222): type SPARSE, num_weights
    // and matrix_cols of the compacted matrix, and its table.  The dense
    // description is kept so that another state can be built.
    std::shared_ptr<SparseTable> sparse_table;
    ConnType dense_type = FULLY_CONNECTED;
    long dense_num_weights = 0;
    int dense_rows = 0, dense_cols = 0;
    Dendrite* node = nullptr;           // dendritic node it feeds
    bool second_order = false;          // on a second-order node
    bool second_order_host = false;     // that node's first connection
    bool second_order_slave = false;
    long num_weights = 0;
    int matrix_rows = 0, matrix_cols = 0;
    int index = 0;

    // Destinations the per-destination loop visits (subset: its window).
    int dest_count() const { return type == SUBSET ? subset.to_size() : to->size; }
    std::string parameter(const std::string& k, const std::string& def) const {
        return config.get(k, def);
    }
    std::string str() const;
};

struct Structure {
    std::string name;
    std::string cluster_type;          // "parallel", "sequential" or "feedforward"
    std::vector<Layer*> layers;
    // Sequential / feedforward: the layers in the order they step, each after
    // the layers that feed it (sequential_cluster.cpp:10-67).
    std::vector<Layer*> order;
    bool parallel() const { return cluster_type == "parallel"; }
};

class Network {
  public:
    explicit Network(const Props& config);
    const Props& config() const { return config_; }

    Structure* structure(const std::string& name) const;
    Layer* layer(const std::string& structure, const std::string& name) const;
    Layer* find_layer(const std::string& name) const;          // unique across structures
    Connection* connection(const std::string& name) const;     // last match wins

    std::vector<std::unique_ptr<Structure>> structures;
    std::vector<std::unique_ptr<Layer>> layers;                 // network order
    std::vector<std::unique_ptr<Connection>> connections;       // JSON order

    long total_weights() const;
    int max_layer_size() const;

  private:
    void add_connection(const Props& p);
    void order_structure(Structure& st);
    Props config_;
};

}  // namespace sg
