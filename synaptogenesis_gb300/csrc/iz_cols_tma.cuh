// Izhikevich trace activator for fully connected and subset matrices, fed by
// the Tensor Memory Accelerator's bulk copies (see iz_cols_tma.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <memory>

#include "synapse.cuh"

namespace sg {

// Column split of one connection's banded matrices.
struct IzColsPlan;

// nrows sources x ncols destinations, every array banded
// (banded_index(destination, source, nrows)); delays may be null (FLOAT / INT
// sources), long_tr null for single-trace opcodes.  bands_per_cta_max limits
// each CTA to that many bands of kBand destinations; ctas = 0 spreads the
// bands over every SM.  Returns null if the kernel cannot run this shape
// (the caller then uses the per-destination activator).
std::shared_ptr<IzColsPlan> make_iz_cols_plan(int nrows, int ncols, const float* w,
                                              const float* stp_r, const float* stp_w,
                                              const int* delays, float* short_tr,
                                              float* long_tr, int ctas = 0);

void launch_iz_cols_tma(const IzColsPlan& plan, const DGeom& g, int src_type, bool subset,
                        const uint32_t* src, float gcond, float short_tau, float long_tau,
                        float* short_cond, float* long_cond, cudaStream_t stream);

// Throws if a pipeline wait of the kernel ran out (reads a device flag; call
// after the stream has synchronised).
void check_iz_cols_errors();
// Testing hook: the producer skips the loads of chunk `chunk` of every launch
// (-1: none), so that a bounded wait runs out and the error path is taken.
void set_iz_cols_skip_chunk(int chunk);

}  // namespace sg
