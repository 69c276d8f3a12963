// One game_of_life cell step on the word layout, shared by the engine's fused
// kernel and the allocation-free entry point (game_of_life_attributes.cpp:14-45
// with the base activator's input, synapse_kernel.h:887-912).
#pragma once

#include "synapse.cuh"

namespace sg {

#ifdef __CUDACC__
// Cell (r, c) of a layer whose only input is its own convergent connection:
// the sequential weighted count of the neighbours' bits at `delay` (prior 0,
// "add"), the survival / birth rule on the cell's bit 0, and the history shift.
// Reads step t-1 from `cur`, writes step t to `next`.
__device__ __forceinline__ void gol_cell_step(const DGeom& g, int delay, int r, int c,
                                              const uint32_t* __restrict__ cur,
                                              uint32_t* __restrict__ next,
                                              const float* __restrict__ w,
                                              float* __restrict__ input_out, int smin, int smax,
                                              int bmin, int bmax) {
    const int d = r * g.to_cols + c;
    float sum = 0.0f;
    for_each_source<T_CONV>(g, d, [&](int from, int wi) {
        float val = extract<S_BIT>(__ldg(cur + from), delay) * __ldg(w + wi);
        sum += val;
    });
    const float input = 0.0f + sum;
    if (input_out) input_out[d] = input;
    const int n = (int)input;
    const uint32_t word = cur[d];
    const bool live = (word & 1u) ? (n >= smin && n <= smax) : (n >= bmin && n <= bmax);
    next[d] = (word >> 1) | ((live ? 1u : 0u) << 31);
}
#endif

}  // namespace sg
