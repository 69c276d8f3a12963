// Game-of-life steps that allocate no device memory.
//
// Some callers cannot call cudaMalloc: a host program whose device memory is
// owned by another allocator (a framework's caching allocator, or a controller
// with a fixed device-memory budget), or a loop that must not allocate between
// steps to keep its latency bounded.  This entry point advances a game_of_life
// board that lives in the caller's own buffers.  The only extra memory is
// g_gol_scratch below: a file-scope device array that holds the other half of
// the ping-pong pair.  Every GPU that loads this library keeps the array until
// the process exits.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "../../include/syngen.h"
#include "gol_step.cuh"

namespace {

// Scratch for the alternate output-history buffer, SG_GOL_NOALLOC_MAX_CELLS
// 32-bit words (4 MiB).  Each step writes every cell of the board into the
// buffer it does not read, so nothing needs clearing between calls; calls that
// overlap on the GPU share this array and race.
__device__ __align__(256) uint32_t g_gol_scratch[SG_GOL_NOALLOC_MAX_CELLS];

// One game_of_life step on a toroidal board (the engine's fused step with
// delay 0).
__global__ void __launch_bounds__(256) k_gol_step_noalloc(
    sg::DGeom g, const uint32_t* __restrict__ cur, uint32_t* __restrict__ next,
    const float* __restrict__ w, float* __restrict__ input_out, int smin, int smax, int bmin,
    int bmax) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    int r = blockIdx.y * blockDim.y + threadIdx.y;
    if (c >= g.to_cols || r >= g.to_rows) return;
    sg::gol_cell_step(g, 0, r, c, cur, next, w, input_out, smin, smax, bmin, bmax);
}

// The current context's identity, through the driver entry points the
// runtime hands out (no link to the driver library): a cudaDeviceReset
// replaces the device's context, and with it the array's address.
typedef int (*CtxGetCurrentFn)(void**);
typedef int (*CtxGetIdFn)(void*, unsigned long long*);

bool current_context_id(unsigned long long* id) {
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess && q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<CtxGetCurrentFn>(f);
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess && q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<CtxGetIdFn>(f);
    });
    void* ctx = nullptr;
    if (!get_current || !get_id || get_current(&ctx) != 0 || !ctx) return false;
    return get_id(ctx, id) == 0;
}

std::mutex g_setup_mutex;
struct ScratchAddr {
    unsigned long long ctx = 0;
    uint32_t* addr = nullptr;
};
ScratchAddr g_scratch_addr[256];   // per device ordinal

// Device address of the scratch array on the current device (host code cannot
// use the symbol's name as a device address).  Looked up once per device
// context: again after a cudaDeviceReset gave the device a new context.
uint32_t* scratch_on_current_device() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 256) return nullptr;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    ScratchAddr& a = g_scratch_addr[dev];
    unsigned long long ctx = 0;
    // no current context (none made yet, or reset) also means a new lookup
    const bool known = current_context_id(&ctx);
    if (!a.addr || !known || a.ctx != ctx) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_gol_scratch) != cudaSuccess) return nullptr;
        a.addr = static_cast<uint32_t*>(p);
        // the lookup made the device's context current
        a.ctx = current_context_id(&ctx) ? ctx : 0;
    }
    return a.addr;
}

}  // namespace

extern "C" int sg_gol_steps_noalloc(unsigned int* words, float* input_out, int rows, int cols,
                                    const float* weights, int field, int steps, int survival_min,
                                    int survival_max, int birth_min, int birth_max, void* stream) {
    if (!words || !weights || rows <= 0 || cols <= 0 || steps < 0 || field < 1 ||
        field > rows || field > cols)
        return SG_NOALLOC_EINVAL;
    if ((long long)rows * (long long)cols > (long long)SG_GOL_NOALLOC_MAX_CELLS)
        return SG_NOALLOC_ETOOBIG;
    uint32_t* scratch = scratch_on_current_device();
    if (!scratch) return SG_NOALLOC_ECUDA;
    if (steps == 0) return 0;

    sg::DGeom g{};
    g.type = sg::T_CONV;
    g.conv = 1;
    g.from_rows = g.to_rows = rows;
    g.from_cols = g.to_cols = cols;
    g.from_size = g.to_size = rows * cols;
    g.rf = g.cf = field;
    g.rs = g.cs = 1;
    g.rsp = g.csp = 1;
    g.ro = g.co = -field / 2;
    g.wrap = 1;
    g.wrap_fast = 1;   // field <= rows, cols keeps every coordinate in [-n, 2n)
    g.n_dest = rows * cols;

    cudaStream_t s = static_cast<cudaStream_t>(stream);
    dim3 block(32, 8);
    dim3 grid((cols + 31) / 32, (rows + 7) / 8);
    uint32_t* bufs[2] = {reinterpret_cast<uint32_t*>(words), scratch};
    // each launch's own status (an error the caller's earlier work left
    // pending is neither read nor cleared here)
    for (int t = 0; t < steps; ++t) {
        const uint32_t* cur = bufs[t & 1];
        uint32_t* next = bufs[(t + 1) & 1];
        float* in_out = t == steps - 1 ? input_out : nullptr;
        void* args[] = {&g, &cur, &next, const_cast<float**>(&weights), &in_out, &survival_min,
                        &survival_max, &birth_min, &birth_max};
        if (cudaLaunchKernel((const void*)k_gol_step_noalloc, grid, block, args, 0, s) !=
            cudaSuccess)
            return SG_NOALLOC_ECUDA;
    }
    if (steps & 1)
        if (cudaMemcpyAsync(words, scratch, (size_t)rows * cols * 4, cudaMemcpyDeviceToDevice, s) !=
            cudaSuccess)
            return SG_NOALLOC_ECUDA;
    return 0;
}
