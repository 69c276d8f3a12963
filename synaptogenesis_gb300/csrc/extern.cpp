// C-ABI of the library: the symbol set of the reference's src/core/extern.h
// (bound by lib/syngen.py:90-175) with the same argument meaning and error
// behaviour (every entry point catches and returns nullptr / false / an empty
// ARRAY, src/core/extern.cpp:151-279), plus sg_* extensions declared in
// include/syngen.h.
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>

#include "../../include/syngen.h"
#include "callbacks.h"
#include "cuda_check.h"
#include "engine.h"
#include "iz_cols_tma.cuh"
#include "models.h"
#include "weight_init.h"

using namespace sg;

namespace {

thread_local std::string g_last_error;
bool g_warnings = true, g_debug = false, g_suppress = false;

void set_error(const char* what) { g_last_error = what ? what : "unknown error"; }

ARRAY null_array() { return ARRAY{0, VOID_POINTER, nullptr, false}; }

ARRAY string_array(const std::vector<std::string>& v) {
    if (v.empty()) return null_array();
    char** pp = (char**)malloc(v.size() * sizeof(char*));
    for (size_t i = 0; i < v.size(); ++i) {
        pp[i] = (char*)malloc(v[i].size() + 1);
        std::memcpy(pp[i], v[i].c_str(), v[i].size() + 1);
    }
    return ARRAY{(int)v.size(), STRING_POINTER, pp, true};
}

ARRAY array_of(Array* a) {
    POINTER_TYPE t = a->dtype == 'i' ? INT_POINTER : FLOAT_POINTER;
    return ARRAY{(int)a->count, t, a->host.data(), false};
}

struct NetHandle {
    Network* net;
    Props props;
};

struct StateHandle {
    Network* net;
    State* state;
};

}  // namespace

namespace sg {
// Error text for sg_last_error from entry points defined in other files.
void set_last_error(const char* what) { set_error(what); }
}  // namespace sg

#define SG_TRY(fail)                          \
    try {
#define SG_CATCH(fail)                        \
    } catch (const std::exception& e) {       \
        set_error(e.what());                  \
        return fail;                          \
    } catch (...) {                           \
        set_error("unknown error");           \
        return fail;                          \
    }

extern "C" {

void free_array(ARRAY arr) {
    if (arr.owner) free(arr.data);
}

void free_array_deep(ARRAY arr) {
    if (arr.owner) {
        for (int i = 0; i < arr.size; ++i) free(((void**)arr.data)[i]);
        free(arr.data);
    }
}

PROPS create_properties() { return new Props(); }

void add_property(PROPS p, char* key, char* val) { ((Props*)p)->set(key, val); }
void add_child(PROPS p, char* key, PROPS child) { ((Props*)p)->set_child(key, *(Props*)child); }
void add_to_array(PROPS p, char* key, char* val) { ((Props*)p)->add_to_array(key, val); }
void add_to_child_array(PROPS p, char* key, PROPS child) {
    ((Props*)p)->add_to_child_array(key, *(Props*)child);
}

ARRAY get_keys(PROPS p) { return string_array(((Props*)p)->keys()); }
ARRAY get_child_keys(PROPS p) { return string_array(((Props*)p)->child_keys()); }
ARRAY get_array_keys(PROPS p) { return string_array(((Props*)p)->array_keys()); }
ARRAY get_child_array_keys(PROPS p) { return string_array(((Props*)p)->child_array_keys()); }

const char* get_property(PROPS p, char* key) { return ((Props*)p)->get_c_str(key); }
PROPS get_child(PROPS p, char* key) { return ((Props*)p)->child(key); }
ARRAY get_array(PROPS p, char* key) { return string_array(((Props*)p)->array(key)); }
ARRAY get_child_array(PROPS p, char* key) {
    auto v = ((Props*)p)->child_array(key);
    if (v.empty()) return null_array();
    void** pp = (void**)malloc(v.size() * sizeof(void*));
    for (size_t i = 0; i < v.size(); ++i) pp[i] = v[i];
    return ARRAY{(int)v.size(), PROPS_POINTER, pp, true};
}

ENVIRONMENT create_environment(PROPS p) {
    SG_TRY(nullptr)
    return new Environment(*(Props*)p);
    SG_CATCH(nullptr)
}

static std::string read_file(const char* path) {
    std::ifstream f(path);
    if (!f) throw SgError(std::string("Could not open file: ") + path);
    std::stringstream ss;
    ss << f.rdbuf();
    return ss.str();
}

ENVIRONMENT load_env(char* filename) {
    SG_TRY(nullptr)
    return new Environment(parse_json(read_file(filename)));
    SG_CATCH(nullptr)
}

bool save_env(ENVIRONMENT env, char* filename) {
    SG_TRY(false)
    std::ofstream f(filename);
    f << write_json(((Environment*)env)->config) << std::endl;
    return (bool)f;
    SG_CATCH(false)
}

NETWORK create_network(PROPS p) {
    SG_TRY(nullptr)
    return new NetHandle{new Network(*(Props*)p), *(Props*)p};
    SG_CATCH(nullptr)
}

NETWORK load_net(char* filename) {
    SG_TRY(nullptr)
    Props p = parse_json(read_file(filename));
    return new NetHandle{new Network(p), p};
    SG_CATCH(nullptr)
}

bool save_net(NETWORK net, char* filename) {
    SG_TRY(false)
    std::ofstream f(filename);
    f << write_json(((NetHandle*)net)->props) << std::endl;
    return (bool)f;
    SG_CATCH(false)
}

STATE build_state(NETWORK net) {
    if (!net) return nullptr;
    SG_TRY(nullptr)
    Network* n = ((NetHandle*)net)->net;
    return new StateHandle{n, new State(n)};
    SG_CATCH(nullptr)
}

STATE build_load_state(NETWORK net, char* filename) {
    if (!net) return nullptr;
    SG_TRY(nullptr)
    Network* n = ((NetHandle*)net)->net;
    auto* h = new StateHandle{n, new State(n)};
    h->state->load(filename);
    return h;
    SG_CATCH(nullptr)
}

bool load_state(STATE st, char* filename) {
    SG_TRY(false)
    ((StateHandle*)st)->state->load(filename);
    return true;
    SG_CATCH(false)
}

bool save_state(STATE st, char* filename) {
    SG_TRY(false)
    ((StateHandle*)st)->state->save(filename);
    return true;
    SG_CATCH(false)
}

ARRAY get_neuron_data(STATE st, char* structure, char* layer, char* key) {
    SG_TRY(null_array())
    auto* h = (StateHandle*)st;
    Layer* l = h->net->layer(structure, layer);
    if (!h->state->on_host()) h->state->to_host(engine_stream());
    return array_of(h->state->layer_state(l)->var(key));
    SG_CATCH(null_array())
}

ARRAY get_layer_data(STATE, char*, char*, char*) { return null_array(); }
ARRAY get_connection_data(STATE, char*, char*) { return null_array(); }

ARRAY get_weight_matrix(STATE st, char* conn, char* key) {
    SG_TRY(null_array())
    auto* h = (StateHandle*)st;
    Connection* c = h->net->connection(conn);
    if (!h->state->on_host()) h->state->to_host(engine_stream());
    return array_of(h->state->conn_state(c)->var(key ? key : "weights"));
    SG_CATCH(null_array())
}

PROPS run(NETWORK net, ENVIRONMENT env, STATE st, PROPS args) {
    if (!net || !st) return nullptr;
    SG_TRY(nullptr)
    Props empty;
    const Props& a = args ? *(Props*)args : empty;
    Engine e(((NetHandle*)net)->net, (Environment*)env, ((StateHandle*)st)->state, a);
    e.step(a.get_int("iterations", 0));
    return e.report();
    SG_CATCH(nullptr)
}

void destroy(void* obj) { delete (Props*)obj; }
void destroy_network(NETWORK net) {
    if (!net) return;
    delete ((NetHandle*)net)->net;
    delete (NetHandle*)net;
}
void destroy_environment(ENVIRONMENT env) { delete (Environment*)env; }
void destroy_state(STATE st) {
    if (!st) return;
    delete ((StateHandle*)st)->state;
    delete (StateHandle*)st;
}
void destroy_properties(PROPS p) { delete (Props*)p; }

int get_num_gpus() {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) { cudaGetLastError(); n = 0; }
    return n;
}
int get_cpu() { return get_num_gpus(); }
ARRAY get_gpus() {
    int n = get_num_gpus();
    int* p = (int*)malloc(sizeof(int) * (n ? n : 1));
    for (int i = 0; i < n; ++i) p[i] = i;
    return ARRAY{n, INT_POINTER, p, true};
}
ARRAY get_all_devices() {
    int n = get_num_gpus();
    int* p = (int*)malloc(sizeof(int) * (n + 1));
    for (int i = 0; i <= n; ++i) p[i] = i;
    return ARRAY{n + 1, INT_POINTER, p, true};
}

void set_suppress_output(bool v) { g_suppress = v; }
void set_warnings(bool v) { g_warnings = v; }
void set_debug(bool v) { g_debug = v; }
void interrupt_engine() { if (Engine::running) Engine::interrupt_flag = true; }

void add_io_callback(char* name, long long addr) {
    Callbacks::get().io[name] = (IoCallback)addr;
}
void add_weight_callback(char* name, long long addr) {
    Callbacks::get().weight[name] = (WeightCallback)addr;
}
void add_indices_weight_callback(char* name, long long addr) {
    Callbacks::get().indices[name] = (IndicesCallback)addr;
}
void add_distance_weight_callback(char* name, long long addr) {
    Callbacks::get().distance[name] = (DistanceCallback)addr;
}
void add_delay_weight_callback(char* name, long long addr) {
    Callbacks::get().delay[name] = (DelayCallback)addr;
}

void initialize_mpi() {}
int get_mpi_rank() { return 0; }
int get_mpi_size() { return 1; }
void finalize_mpi() {}

// ---------------------------------------------------------------------------
// Extensions
// ---------------------------------------------------------------------------
const char* sg_last_error(void) { return g_last_error.c_str(); }

SG_ENGINE sg_engine_create(NETWORK net, ENVIRONMENT env, STATE st, PROPS args) {
    if (!net || !st) return nullptr;
    SG_TRY(nullptr)
    Props empty;
    return new Engine(((NetHandle*)net)->net, (Environment*)env, ((StateHandle*)st)->state,
                      args ? *(Props*)args : empty);
    SG_CATCH(nullptr)
}

long long sg_engine_step(SG_ENGINE eng, long long steps) {
    if (!eng || steps <= 0) return -1;
    SG_TRY(-1)
    return ((Engine*)eng)->step((long)steps);
    SG_CATCH(-1)
}

void* sg_engine_stream(SG_ENGINE eng) {
    return eng ? (void*)((Engine*)eng)->stream() : nullptr;
}

PROPS sg_engine_report(SG_ENGINE eng) {
    if (!eng) return nullptr;
    SG_TRY(nullptr)
    return ((Engine*)eng)->report();
    SG_CATCH(nullptr)
}

void sg_engine_destroy(SG_ENGINE eng) {
    try {
        delete (Engine*)eng;
    } catch (...) {
    }
}

void sg_set_seed(unsigned long long seed) { set_global_seed(seed); }

int sg_version(void) { return SG_ABI_VERSION; }

bool sg_test_cols_skip_chunk(int chunk) {
    SG_TRY(false)
    set_iz_cols_skip_chunk(chunk);
    return true;
    SG_CATCH(false)
}

}  // extern "C"
