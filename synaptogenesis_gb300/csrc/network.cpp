#include "network.h"

#include <algorithm>
#include <deque>
#include <functional>
#include <map>

#include "models.h"

namespace sg {

static const std::vector<std::pair<std::string, ConnType>> kConnTypes = {
    {"fully connected", FULLY_CONNECTED}, {"subset", SUBSET}, {"one to one", ONE_TO_ONE},
    {"convergent", CONVERGENT}, {"divergent", DIVERGENT}};
static const std::vector<std::pair<std::string, Opcode>> kOpcodes = {
    {"add", OP_ADD}, {"sub", OP_SUB}, {"mult", OP_MULT}, {"div", OP_DIV}, {"pool", OP_POOL},
    {"reward", OP_REWARD}, {"modulate", OP_MODULATE}, {"gap", OP_GAP},
    {"add_heaviside", OP_ADD_HEAVISIDE}, {"sub_heaviside", OP_SUB_HEAVISIDE},
    {"mult_heaviside", OP_MULT_HEAVISIDE}};

ConnType parse_conn_type(const std::string& s) {
    for (auto& p : kConnTypes) if (p.first == s) return p.second;
    throw SgError("Unrecognized ConnectionType: " + s);
}
Opcode parse_opcode(const std::string& s) {
    for (auto& p : kOpcodes) if (p.first == s) return p.second;
    throw SgError("Unrecognized Opcode: " + s);
}
const char* conn_type_name(ConnType t) {
    for (auto& p : kConnTypes) if (p.second == t) return p.first.c_str();
    return t == SPARSE ? "sparse" : "?";
}
const char* opcode_name(Opcode o) {
    for (auto& p : kOpcodes) if (p.second == o) return p.first.c_str();
    return "?";
}

int Layer::max_delay() const {
    int m = 0;
    for (auto* c : outputs) m = std::max(m, c->delay);
    return m;
}

std::string Layer::str() const {
    return "[Layer: " + name + " (" + structure->name + ")]";
}

int Dendrite::max_register() const {
    int m = reg;
    for (auto& ch : children)
        if (ch.node) m = std::max(m, ch.node->max_register());
    return m;
}

std::string Dendrite::str() const { return "[Dendrite: " + name + " (" + layer->name + ")]"; }

std::vector<Dendrite*> Layer::dendrites() const {
    std::vector<Dendrite*> out{root.get()};
    for (size_t i = 0; i < out.size(); ++i)
        for (auto& ch : out[i]->children)
            if (ch.node) out.push_back(ch.node);
    return out;
}

Dendrite* Layer::dendrite(const std::string& n) const {
    for (Dendrite* d : dendrites())
        if (d->name == n) return d;
    return nullptr;
}

// Layer::add_dendrites and DendriticNode::add_child (layer.cpp:135-153,
// dendritic_node.cpp:80-104): depth first, so registers follow the pre-order
// of the config.
static void add_dendrites(Layer* l, Dendrite* parent, const std::vector<Props*>& configs) {
    for (Props* d : configs) {
        if (!d->has("name")) throw SgError("Attempted to dendrite without name to layer!");
        const std::string name = d->get("name");
        if (parent->second_order)
            throw SgError("Error in dendritic node " + name + " of " + l->str() +
                          "\n  Second order dendritic nodes cannot have internal children!");
        if (l->dendrite(name))
            throw SgError("Error in dendritic node of " + l->str() +
                          "\n  Duplicate dendritic node name: " + name + "!");
        auto node = std::make_unique<Dendrite>();
        node->name = name;
        node->layer = l;
        node->parent = parent;
        node->reg = l->root->max_register() + 1;
        node->opcode = parse_opcode(d->get("opcode", "add"));
        node->second_order = d->get_bool("second order", false);
        node->init = d->get_float("init", 0.0f);
        Dendrite* raw = node.get();
        parent->children.push_back({raw, nullptr});
        parent->owned.push_back(std::move(node));
        add_dendrites(l, raw, d->child_array("children"));
    }
}

// Same text as the reference's Connection::str() (connection.cpp:251-259); it
// also keys saved state records.
std::string Connection::str() const {
    return "[Connection: " + from->name + " (" + from->structure->name + ") -> " + to->name +
           " (" + to->structure->name + ") {Node: " + (node ? node->name : std::string("root")) +
           "} name=" + name + "]";
}

// ArborizedConfig (connection_config.cpp:8-45), including the "column offset"
// quirk: the column offset is first read from "row offset".
static Arbor parse_arbor(const Props& a) {
    Arbor r;
    r.row_field = a.get_int("row field size", 0);
    r.col_field = a.get_int("column field size", 0);
    r.row_stride = a.get_int("row stride", 1);
    r.col_stride = a.get_int("column stride", 1);
    r.row_spacing = a.get_int("row spacing", 1);
    r.col_spacing = a.get_int("column spacing", 1);
    r.row_offset = a.get_int("row offset", 0);
    r.col_offset = a.get_int("row offset", 0);
    r.wrap = a.get_bool("wrap", false);
    if (a.has("field size")) r.row_field = r.col_field = a.get_int("field size", 0);
    if (a.has("stride")) r.row_stride = r.col_stride = a.get_int("stride", 0);
    if (a.has("spacing")) r.row_spacing = r.col_spacing = a.get_int("spacing", 0);
    if (a.has("offset")) r.row_offset = r.col_offset = a.get_int("offset", 0);
    if (r.row_field <= 0 || r.col_field <= 0)
        throw SgError("Unspecified field size for arborized config!");
    if (r.row_stride < 0 || r.col_stride < 0)
        throw SgError("Cannot have negative stride in arborized config!");
    if (r.row_spacing < 1 || r.col_spacing < 1)
        throw SgError("Cannot have zero or negative spacing in arborized config!");
    if (!a.has("row offset") && !a.has("offset")) r.row_offset = -r.row_field / 2;
    if (!a.has("column offset") && !a.has("offset")) r.col_offset = -r.col_field / 2;
    return r;
}

static SubsetCfg parse_subset(const Props& s) {
    SubsetCfg r;
    r.fr0 = s.get_int("from row start", 0);
    r.fr1 = s.get_int("from row end", 0);
    r.tr0 = s.get_int("to row start", 0);
    r.tr1 = s.get_int("to row end", 0);
    r.fc0 = s.get_int("from column start", 0);
    r.fc1 = s.get_int("from column end", 0);
    r.tc0 = s.get_int("to column start", 0);
    r.tc1 = s.get_int("to column end", 0);
    if (r.fr1 - r.fr0 <= 0 || r.tr1 - r.tr0 <= 0 || r.fc1 - r.fc0 <= 0 || r.tc1 - r.tc0 <= 0)
        throw SgError("Invalid subset dimensions!");
    return r;
}

Network::Network(const Props& config) : config_(config) {
    for (Props* sp : config.child_array("structures")) {
        if (!sp->has("name")) throw SgError("Unspecified name for structure!");
        for (auto& s : structures)
            if (s->name == sp->get("name")) throw SgError("Repeated structure name: " + s->name);
        auto st = std::make_unique<Structure>();
        st->name = sp->get("name");
        st->cluster_type = sp->get("type", "parallel");
        if (st->cluster_type != "parallel" && st->cluster_type != "sequential" &&
            st->cluster_type != "feedforward")
            throw SgError("Unrecognized ClusterType: " + st->cluster_type);
        for (Props* lp : sp->child_array("layers")) {
            auto l = std::make_unique<Layer>();
            l->config = *lp;
            if (!lp->has("name")) throw SgError("Attempted to construct LayerConfig without name!");
            if (!lp->has("neural model"))
                throw SgError("Attempted to construct LayerConfig without neural model!");
            if (lp->has("image")) throw SgError("image-sized layers are not supported");
            l->name = lp->get("name");
            l->model = lp->get("neural model");
            l->rows = lp->get_int("rows", 0);
            l->cols = lp->get_int("columns", 0);
            if (l->rows <= 0 || l->cols <= 0)
                throw SgError("Invalid dimensions for layer " + l->name);
            l->size = l->rows * l->cols;
            l->plastic = lp->get_bool("plastic", false);
            if (lp->get_bool("ghost", false)) throw SgError("ghost layers are not supported");
            const Model* m = find_model(l->model);
            if (!m) throw SgError("Unrecognized neural model \"" + l->model + "\"");
            l->output_type = m->output_type();
            l->structure = st.get();
            l->root = std::make_unique<Dendrite>();
            l->root->name = "root";
            l->root->layer = l.get();
            add_dendrites(l.get(), l->root.get(), lp->child_array("dendrites"));
            l->registers = l->root->max_register() + 1;
            for (auto* other : st->layers)
                if (other->name == l->name) throw SgError("Repeated layer name : \"" + l->name + "\"");
            l->index = (int)layers.size();
            st->layers.push_back(l.get());
            layers.push_back(std::move(l));
        }
        structures.push_back(std::move(st));
    }
    for (Props* cp : config.child_array("connections")) add_connection(*cp);
    for (auto& st : structures)
        if (!st->parallel()) order_structure(*st);
}

// SequentialCluster (sequential_cluster.cpp:10-67): a breadth-first walk
// backwards from the structure's outputs; a layer is placed once every layer
// it feeds (within the structure, not over recurrent connections) is placed,
// and goes in front of them.  The reference loops forever on a cycle; here
// a pass that places nothing ends the walk with its error.  Feedforward
// structures must also have no cycle reachable from their inputs
// (feedforward_cluster.cpp:8-36).
void Network::order_structure(Structure& st) {
    auto inner = [&](const Connection* c) { return c->from->structure == &st && c->to->structure == &st; };
    std::deque<Layer*> queue;
    for (Layer* l : st.layers) {
        bool output = true;
        for (Connection* c : l->outputs)
            if (c->to->structure == &st && !c->recurrent) output = false;
        if (output || l->outputs.empty()) queue.push_back(l);
    }
    std::vector<Layer*> placed;
    auto is_placed = [&](const Layer* l) { return std::find(placed.begin(), placed.end(), l) != placed.end(); };
    size_t stalled = 0;
    while (!queue.empty()) {
        Layer* cur = queue.front();
        queue.pop_front();
        if (is_placed(cur)) { stalled = 0; continue; }
        bool wait = false;
        for (Connection* c : cur->outputs)
            if (c->to != cur && inner(c) && !c->recurrent && !is_placed(c->to)) wait = true;
        if (wait) {
            queue.push_back(cur);
            if (++stalled > queue.size()) break;       // a full pass placed nothing: a cycle
            continue;
        }
        stalled = 0;
        placed.push_back(cur);
        for (Connection* c : cur->inputs)
            if (c->from != cur && inner(c) && !c->recurrent && !is_placed(c->from)) queue.push_back(c->from);
    }
    if (placed.size() < st.layers.size()) throw SgError("Sequential cluster failed to process all layers!");
    st.order.assign(placed.rbegin(), placed.rend());
    if (st.cluster_type == "feedforward") {
        std::vector<Layer*> path;
        std::function<bool(Layer*)> acyclic = [&](Layer* l) {
            if (std::find(path.begin(), path.end(), l) != path.end()) return false;
            path.push_back(l);
            for (Connection* c : l->outputs)
                if (c->to->structure == &st && !acyclic(c->to)) return false;
            path.pop_back();
            return true;
        };
        for (Layer* l : st.layers) {
            bool input = true;
            for (Connection* c : l->inputs)
                if (c->from->structure == &st && !c->recurrent) input = false;
            if (input && !acyclic(l)) throw SgError("Feedforward engine requires a structure with no cycles!");
        }
    }
}

Structure* Network::structure(const std::string& name) const {
    Structure* found = nullptr;
    for (auto& s : structures) if (s->name == name) found = s.get();
    return found;
}

Layer* Network::layer(const std::string& sname, const std::string& name) const {
    Structure* s = structure(sname);
    if (!s) throw SgError("Could not find structure: " + sname);
    for (auto* l : s->layers) if (l->name == name) return l;
    throw SgError("Could not find layer \"" + name + "\"");
}

Layer* Network::find_layer(const std::string& name) const {
    Layer* found = nullptr;
    for (auto& l : layers)
        if (l->name == name) {
            if (found) throw SgError("Ambiguous layer name: " + name);
            found = l.get();
        }
    if (!found) throw SgError("Could not find layer: " + name);
    return found;
}

Connection* Network::connection(const std::string& name) const {
    Connection* found = nullptr;
    for (auto& c : connections) if (c->name == name) found = c.get();
    if (!found) throw SgError("Could not find connection: " + name);
    return found;
}

long Network::total_weights() const {
    long n = 0;
    for (auto& c : connections) n += c->num_weights;
    return n;
}

int Network::max_layer_size() const {
    int m = 0;
    for (auto& l : layers) m = std::max(m, l->size);
    return m;
}

void Network::add_connection(const Props& p) {
    if (!p.has("from layer")) throw SgError("Attempted to construct ConnectionConfig without source layer!");
    if (!p.has("to layer")) throw SgError("Attempted to construct ConnectionConfig without destination layer!");
    auto c = std::make_unique<Connection>();
    c->config = p;
    c->name = p.get("name", "");
    std::string fl = p.get("from layer"), tl = p.get("to layer");
    if (structures.size() == 1) {
        c->from = layer(structures[0]->name, fl);
        c->to = layer(structures[0]->name, tl);
    } else {
        c->from = p.has("from structure") ? layer(p.get("from structure"), fl) : find_layer(fl);
        c->to = p.has("to structure") ? layer(p.get("to structure"), tl) : find_layer(tl);
    }
    const std::string dn = p.get("dendrite", "root");
    c->node = c->to->dendrite(dn);
    if (!c->node) throw SgError("Error in " + c->to->str() + ":\n  Cannot find Dendritic Node " + dn + "!");
    c->second_order = c->node->second_order;
    c->second_order_host = c->second_order && !c->node->host;
    c->second_order_slave = c->second_order && !c->second_order_host;
    c->plastic = p.get_bool("plastic", true);
    c->recurrent = p.get_bool("recurrent", false);
    c->delay = p.get_int("delay", 0);
    c->max_weight = p.get_float("max weight", 1.0f);
    c->type = parse_conn_type(p.get("type", "fully connected"));
    c->opcode = parse_opcode(p.get("opcode", "add"));
    c->convolutional = p.get_bool("convolutional", false);
    if (c->delay < 0) throw SgError("Attempted to construct ConnectionConfig with negative delay!");
    c->sparse = p.get_bool("sparse", false) || p.get_bool("randomized projection", false);
    if (c->sparse && c->second_order)
        throw SgError("Error in " + c->str() + ":\n  Sparse second order connections are not supported!");
    c->randomized = p.get_bool("randomized projection", false);
    if (c->convolutional && c->type != CONVERGENT && c->type != DIVERGENT)
        throw SgError("Only convergent/divergent connections can be convolutional!");
    Layer *from = c->from, *to = c->to;
    switch (c->type) {
        case FULLY_CONNECTED:
            c->num_weights = (long)from->size * to->size;
            c->matrix_rows = to->size;
            c->matrix_cols = from->size;
            break;
        case SUBSET: {
            Props* s = p.child("subset config");
            if (!s) throw SgError("Attempted to create SUBSET connection without specifying subset configuration!");
            c->subset = parse_subset(*s);
            auto& sc = c->subset;
            if (!(sc.fr1 <= from->rows && sc.fc1 <= from->cols && sc.tr1 <= to->rows && sc.tc1 <= to->cols))
                throw SgError(c->str() + ": Invalid connection config!");
            c->num_weights = (long)sc.from_size() * sc.to_size();
            c->matrix_rows = sc.to_size();
            c->matrix_cols = sc.from_size();
            break;
        }
        case ONE_TO_ONE:
            if (from->rows != to->rows || from->cols != to->cols)
                throw SgError(c->str() + ": Cannot connect differently sized layers one-to-one!");
            c->num_weights = to->size;
            c->matrix_rows = to->size;
            c->matrix_cols = 1;
            break;
        case CONVERGENT:
        case DIVERGENT: {
            Props* a = p.child("arborized config");
            if (!a) throw SgError("Attempted to create arborized connection without specifying arborized configuration!");
            c->arbor = parse_arbor(*a);
            if (c->type == DIVERGENT && (c->arbor.row_stride == 0 || c->arbor.col_stride == 0))
                throw SgError(c->str() + ": Divergent connections cannot have zero stride!");
            c->num_weights = c->convolutional ? c->arbor.kernel() : (long)to->size * c->arbor.kernel();
            c->matrix_rows = c->convolutional ? 1 : to->size;
            c->matrix_cols = c->arbor.kernel();
            break;
        }
    }
    if (c->num_weights >= (1L << 31)) throw SgError(c->str() + ": more than 2^31 weights");
    // WeightMatrix::randomize_projection (weight_matrix.cpp:355-507)
    if (c->randomized) {
        if (c->convolutional)
            throw SgError("Error intializing weight matrix for " + c->str() +
                          "\n   Cannot randomize projection on convolutional weight matrix!");
        if (c->type == FULLY_CONNECTED)
            throw SgError("Error intializing weight matrix for " + c->str() +
                          "\n   Cannot randomize projection on fully connectedweight matrix!");
        if (c->type == SUBSET)
            throw SgError("Error intializing weight matrix for " + c->str() +
                          "\n   Cannot randomize projection on subset weight matrix!");
    }
    c->dense_type = c->type;
    c->dense_num_weights = c->num_weights;
    c->dense_rows = c->matrix_rows;
    c->dense_cols = c->matrix_cols;
    // second-order rules (connection.cpp:149-191)
    if (c->second_order && c->plastic)
        throw SgError("Error in " + c->str() + ":\n  Plastic second order connections are not supported!");
    if (c->second_order_slave) {
        const Connection* host = c->node->host;
        if (c->type != host->type || c->convolutional != host->convolutional ||
            c->num_weights != host->num_weights)
            throw SgError("Error in " + c->str() + ":\n  Second order connection does not match host connection!");
        // a convolutional slave runs like a one-to-one connection over the
        // host's kernel, so its field is the whole source layer
        const Arbor& a = c->arbor;
        if (c->convolutional && (a.kernel() != from->size || a.row_spacing != 1 ||
                                 a.col_spacing != 1 || a.row_stride != 0 || a.col_stride != 0))
            throw SgError("Error in " + c->str() +
                          ":\n  Second order convolutional connections must have fields that are the "
                          "size of the input layer, and must have 0 stride and 1 spacing!");
    }
    c->index = (int)connections.size();
    from->outputs.push_back(c.get());
    to->inputs.push_back(c.get());
    // DendriticNode::add_child(Connection*) (dendritic_node.cpp:106-140)
    if (c->second_order_host) c->node->host = c.get();
    else c->node->children.push_back({nullptr, c.get()});
    connections.push_back(std::move(c));
}

}  // namespace sg
