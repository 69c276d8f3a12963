// Izhikevich trace activator for fully connected and subset matrices, fed by
// the Tensor Memory Accelerator (see iz_cols_tma.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <memory>

#include "synapse.cuh"

namespace sg {

// Tensor maps and the column split of one connection's matrices, built once
// for the arrays' device addresses.
struct IzColsPlan;

// nrows x ncols device matrices ([source row][destination column], ncols a
// multiple of 4); delays may be null (FLOAT / INT sources), long_tr null for
// single-trace opcodes.  Returns null when the split or the tensor maps are
// not possible (the caller then uses the cp.async kernel).
std::shared_ptr<IzColsPlan> make_iz_cols_plan(int nrows, int ncols, const float* w,
                                              const float* stp_r, const float* stp_w,
                                              const int* delays, float* short_tr,
                                              float* long_tr);

void launch_iz_cols_tma(const IzColsPlan& plan, const DGeom& g, int src_type, bool subset,
                        const uint32_t* src, float gcond, float short_tau, float long_tau,
                        float* short_cond, float* long_cond, cudaStream_t stream);

// Throws if a pipeline wait of the kernel ran out (reads a device flag; call
// after the stream has synchronised).
void check_iz_cols_errors();

}  // namespace sg
