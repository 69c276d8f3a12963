/*
 * syngen.h -- C-ABI of the GB300 synaptogenesis simulation-cycle library
 * (libsyngen.so built from synaptogenesis_gb300/csrc).
 *
 * The first block is a drop-in for the reference's src/core/extern.h: same
 * symbol names, argument meaning, ownership and error behaviour, so the
 * reference front-end (lib/syngen.py) binds it unchanged.  Line numbers cite
 * src/core/extern.h (declarations) and src/core/extern.cpp (behaviour).
 *
 * Errors: entry points never throw; on failure they return nullptr, false or
 * an empty ARRAY{0, VOID_POINTER, NULL, false} (extern.cpp:151-279).  The
 * message of the last failure on the calling thread is sg_last_error().
 *
 * Ownership: data getters return non-owning pointers into the live host copy
 * of the state (they first move the state to the host; the next run moves it
 * back, extern.cpp:214-258, state.cpp:706-764).  STRING / PROPS arrays are
 * owned and are released with free_array / free_array_deep.
 */
#ifndef SYNGEN_GB300_H
#define SYNGEN_GB300_H

#ifdef __cplusplus
#include <cstddef>
extern "C" {
#else
#include <stdbool.h>
#include <stddef.h>
#endif

#define SG_ABI_VERSION 1

/* extern.h:6-12 */
typedef enum {
    FLOAT_POINTER = 1,
    INT_POINTER = 2,
    STRING_POINTER = 3,
    PROPS_POINTER = 4,
    VOID_POINTER = 5
} POINTER_TYPE;

/* extern.h:14-19 */
typedef struct ARRAY {
    int size;
    POINTER_TYPE type;
    void* data;
    bool owner;
} ARRAY;

/* extern.h:25-28 */
typedef void* NETWORK;
typedef void* ENVIRONMENT;
typedef void* STATE;
typedef void* PROPS;

/* extern.h:23-24 */
void free_array(ARRAY arr);
void free_array_deep(ARRAY arr);

/* Properties, extern.h:30-45 */
PROPS create_properties(void);
void add_property(PROPS properties, char* key, char* val);
void add_child(PROPS properties, char* key, PROPS child);
void add_to_array(PROPS properties, char* key, char* val);
void add_to_child_array(PROPS properties, char* key, PROPS props);
ARRAY get_keys(PROPS properties);
ARRAY get_child_keys(PROPS properties);
ARRAY get_array_keys(PROPS properties);
ARRAY get_child_array_keys(PROPS properties);
const char* get_property(PROPS properties, char* key);
PROPS get_child(PROPS properties, char* key);
ARRAY get_array(PROPS properties, char* key);
ARRAY get_child_array(PROPS properties, char* key);

/* Environment / network objects, extern.h:47-53 */
ENVIRONMENT create_environment(PROPS properties);
ENVIRONMENT load_env(char* filename);
bool save_env(ENVIRONMENT env, char* filename);
NETWORK create_network(PROPS properties);
NETWORK load_net(char* filename);
bool save_net(NETWORK network, char* filename);

/* State, extern.h:55-58 */
STATE build_state(NETWORK net);
STATE build_load_state(NETWORK net, char* filename);
bool load_state(STATE state, char* filename);
bool save_state(STATE state, char* filename);

/* Data access, extern.h:60-65 (host layout views) */
ARRAY get_neuron_data(STATE state, char* structure_name, char* layer_name, char* key);
ARRAY get_layer_data(STATE state, char* structure_name, char* layer_name, char* key);
ARRAY get_connection_data(STATE state, char* conn_name, char* key);
ARRAY get_weight_matrix(STATE state, char* conn_name, char* key);

/* One run of the simulation cycle, extern.h:67; returns the report */
PROPS run(NETWORK net, ENVIRONMENT env, STATE state, PROPS args);

/* Teardown, extern.h:69-73 */
void destroy(void* obj);
void destroy_network(NETWORK net);
void destroy_environment(ENVIRONMENT env);
void destroy_state(STATE state);
void destroy_properties(PROPS props);

/* Devices, extern.h:75-78 (the host id is the number of GPUs) */
int get_num_gpus(void);
int get_cpu(void);
ARRAY get_gpus(void);
ARRAY get_all_devices(void);

/* Logging and control, extern.h:80-84 */
void set_suppress_output(bool val);
void set_warnings(bool val);
void set_debug(bool val);
void interrupt_engine(void);

/* Named host callbacks, extern.h:86-90 */
void add_io_callback(char* name, long long addr);
void add_weight_callback(char* name, long long addr);
void add_indices_weight_callback(char* name, long long addr);
void add_distance_weight_callback(char* name, long long addr);
void add_delay_weight_callback(char* name, long long addr);

/* MPI, extern.h:92-95: single-process no-ops (rank 0 of 1) */
void initialize_mpi(void);
int get_mpi_rank(void);
int get_mpi_size(void);
void finalize_mpi(void);

/* ---------------- Extensions (no counterpart in extern.h) ---------------- */

/* Message of the last failed call on this thread ("" if none). */
const char* sg_last_error(void);

/* Persistent engine: run() split into create / step / report / destroy, so a
 * caller can advance the same state repeatedly without rebuilding.  Behaves
 * like run() (src/core/engine/engine.cpp:462-596): same args, same step order,
 * same callbacks.  Without host callbacks, steps replay a captured CUDA graph.
 * At most one engine exists at a time (engine.cpp:466-471). */
typedef void* SG_ENGINE;
SG_ENGINE sg_engine_create(NETWORK net, ENVIRONMENT env, STATE state, PROPS args);
/* Runs `steps` (> 0) timesteps; returns the number run, or -1 on error. */
long long sg_engine_step(SG_ENGINE engine, long long steps);
/* The CUDA stream (cudaStream_t) every kernel of the engine is launched on. */
void* sg_engine_stream(SG_ENGINE engine);
/* Report of all steps so far (same keys as run()'s report), owned by caller. */
PROPS sg_engine_report(SG_ENGINE engine);
void sg_engine_destroy(SG_ENGINE engine);
/* Seed of the random weight / parameter / noise initialisers. */
void sg_set_seed(unsigned long long seed);
/* ABI version of this header. */
int sg_version(void);

/* Testing hook, no counterpart in the reference: from now on the TMA
 * activator of fully connected / subset Izhikevich connections issues no
 * loads for chunk `chunk` of its source rows (-1: back to normal), so that its
 * consumers' bounded wait runs out and the run reports the timeout as an
 * error.  The state of a network run meanwhile is not meaningful.  Returns
 * false on a CUDA error. */
bool sg_test_cols_skip_chunk(int chunk);

/* Allocation-free game_of_life stepping.  No counterpart in the reference.
 *
 * For callers that cannot call cudaMalloc: a host program whose device memory
 * belongs to another allocator, or a loop that must not allocate between steps.
 * Advances `steps` timesteps of a toroidal game_of_life board held in the
 * caller's device buffers, with the semantics of a game_of_life layer whose only
 * input is its own convergent, convolutional, wrapping "add" connection
 * (field x field weights, stride 1, spacing 1, offset -field/2, delay 0):
 *   words      device, rows*cols output-history words, updated in place
 *   input_out  device, rows*cols floats receiving the last step's input
 *              register (the weighted neighbour count), or NULL
 *   weights    device, field*field floats (row-major kernel)
 *   stream     cudaStream_t to launch on (NULL: the default stream)
 * Allocates nothing: its only working memory is a static device array of
 * SG_GOL_NOALLOC_MAX_CELLS words that every GPU loading the library holds until
 * exit.  Boards larger than that are rejected (SG_NOALLOC_ETOOBIG).  The first
 * call on a device (and the first after a cudaDeviceReset gave the device a new
 * context) looks up that array's device address; make that first call before
 * any stream capture.  All calls share the array, so calls that overlap on the
 * GPU race.  Returns 0, or a negative SG_NOALLOC_* code; a launch that fails
 * returns SG_NOALLOC_ECUDA without touching errors the caller's earlier work
 * left pending.  The work is asynchronous on `stream`. */
#define SG_GOL_NOALLOC_MAX_CELLS (1 << 20)
#define SG_NOALLOC_EINVAL (-1)
#define SG_NOALLOC_ETOOBIG (-2)
#define SG_NOALLOC_ECUDA (-3)
int sg_gol_steps_noalloc(unsigned int* words, float* input_out, int rows, int cols,
                         const float* weights, int field, int steps, int survival_min,
                         int survival_max, int birth_min, int birth_max, void* stream);

/* Batched Izhikevich instances.  No counterpart in the reference, which runs
 * one network per engine (src/core/engine/engine.cpp:466-471); a batch
 * replaces running that engine once per instance.
 *
 * Every instance is the plain Izhikevich topology: a relay layer of rows x cols
 * (FLOAT output) whose input each step is `input_value` with probability
 * `input_rate`, a convergent wrapping "add" connection (conv_field^2 kernel,
 * stride 1, offset -field/2) into an Izhikevich layer of the same shape, and
 * a recurrent fully connected "sub" connection on that layer.  Weights, delays
 * and inputs are counter-based functions of `seed` (convergent weights
 * U(0, conv_wmax); recurrent weights U(0, fc_wmax) kept with probability
 * fc_density, delays U{0..fc_max_delay}); the effective weight of a synapse is
 * weight x (short term R = 1) x (short term w = *_stp_w), as in the
 * reference's activator.  Initial voltage v0 and recovery b * v0.  The same
 * instance built as an ordinary network gives the same spike raster, bit for
 * bit.  All instances need the same conv_field. */
typedef struct SgBatchInstance {
    int rows, cols;
    float a, b, c, d;
    float v0;
    unsigned long long seed;
    float input_rate, input_value;
    int conv_field;
    float conv_wmax, conv_stp_w, conv_conductance;
    float fc_wmax, fc_density, fc_stp_w, fc_conductance;
    int fc_max_delay;
} SgBatchInstance;

#define SG_BATCH_EINVAL (-1)
#define SG_BATCH_ECUDA (-3)
typedef void* SG_BATCH;

/* Builds the batch on the current device.  tile_rows x tile_colblocks (rows x
 * blocks of 32 columns, at most 8 warps) is the work unit of the step kernel;
 * 0, 0 runs the autotuner, which times each candidate over real steps and
 * then resets the state.  NULL on error (sg_last_error). */
SG_BATCH sg_batch_create(const SgBatchInstance* instances, int count, int tile_rows,
                         int tile_colblocks);
/* Advances every instance by `steps` timesteps, one kernel launch per step
 * (captured in CUDA graphs of 32 steps).  Asynchronous on sg_batch_stream. */
int sg_batch_step(SG_BATCH batch, long long steps);
/* Copies an instance's "voltage", "recovery" (float) or "output" (newest
 * output-history word, uint32) to host memory of at least rows*cols values. */
int sg_batch_read(SG_BATCH batch, int instance, const char* key, void* out, long long count);
/* Sizes, chosen tile, autotuner timings and launch counts; owned by the
 * caller (destroy_properties). */
PROPS sg_batch_report(SG_BATCH batch);
void* sg_batch_stream(SG_BATCH batch);
int sg_batch_synchronize(SG_BATCH batch);
void sg_batch_destroy(SG_BATCH batch);

/* Differentiable leaky-integrator rate network.  No counterpart in the
 * reference, whose rate_encoding layer has no memory
 * (src/core/state/impl/rate_encoding_attributes.cpp:14-34).
 *
 * `layers` layers of rows x cols neurons; layer 0 is driven by the input
 * sequence x, layer l >= 1 by a convergent connection from layer l-1
 * (field x field with field odd and at most 9, stride 1, offset -field/2, no
 * wrap: out-of-range sources are skipped); outputs at most 16; every layer integrates v += (dt / tau_l) (-v + I), rate
 * sigmoid(v), v = 0 at the start; every layer reads the previous step's rates.
 * A readout R (outputs x N) of the last layer's rates gives y[t]; the loss is
 * the mean over (t, b, o) of (y[t][b][o] - target[b][o])^2.
 * Device arrays, float32:
 *   x        [steps][batch][rows*cols]
 *   weights  [layers-1][rows*cols][field*field]  (destination-major, k row-major)
 *   readout  [outputs][rows*cols]
 *   tau      [layers]
 *   target   [batch][outputs]
 *   y        [steps][batch][outputs] (optional output)
 *   loss     one float
 * The workspace (sg_rate_workspace_bytes, device memory owned by the caller)
 * keeps the forward pass's checkpoints (v every `checkpoint` steps) for the
 * backward pass, which recomputes each segment from its checkpoint and runs
 * the hand-written adjoint back through it.  d_weights, d_readout, d_tau (and
 * d_x, or NULL) receive grad_loss * dloss/d(parameter).  Work is asynchronous
 * on `stream` (a cudaStream_t; NULL = default stream).  Returns 0 or a
 * negative SG_RATE_* code (sg_last_error). */
typedef struct SgRateShape {
    int layers, rows, cols, field, outputs, batch, steps, checkpoint;
    float dt;
} SgRateShape;

#define SG_RATE_EINVAL (-1)
#define SG_RATE_ECUDA (-3)
long long sg_rate_workspace_bytes(const SgRateShape* shape);
int sg_rate_forward(const SgRateShape* shape, const float* x, const float* weights,
                    const float* readout, const float* tau, const float* target, float* y,
                    float* loss, void* workspace, void* stream);
int sg_rate_backward(const SgRateShape* shape, const float* x, const float* weights,
                     const float* readout, const float* tau, const float* target,
                     float grad_loss, void* workspace, float* d_weights, float* d_readout,
                     float* d_tau, float* d_x, void* stream);

#ifdef __cplusplus
}
#endif
#endif
