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
// (banded_index(destination, source, nrows)); delays (bytes, filled by
// fill_iz_delay_bytes) may be null (FLOAT / INT sources), long_tr null for
// single-trace opcodes.  eff, if not null, holds
// w * (R * w_stp) for a connection whose weights and short-term factors do
// not change during a run (fill_iz_effective_weights after each upload); the
// kernel then reads it instead of w, stp_r and stp_w.  ctas = 0 spreads the
// bands over every SM.  Returns null if the kernel cannot run this shape (the
// caller then uses the per-destination activator).
std::shared_ptr<IzColsPlan> make_iz_cols_plan(int nrows, int ncols, const float* w,
                                              const float* stp_r, const float* stp_w,
                                              const uint8_t* delays, float* short_tr,
                                              float* long_tr, const float* eff = nullptr,
                                              int ctas = 0);

// The delays of a banded int array as bytes, [band][row * 8 + lane], each
// band's rows padded to a multiple of 16 bytes (iz_delay_bytes_pitch): the
// activator's TMA reads 1 byte per synapse instead of 4 (delays are below 32).
size_t iz_delay_bytes_pitch(int nrows);
void fill_iz_delay_bytes(int nrows, int ncols, const int* delays, uint8_t* d8, cudaStream_t s);

// eff[i] = w[i] * (stp_r[i] * stp_w[i]) for i < n (the activator's weight).
void fill_iz_effective_weights(size_t n, const float* w, const float* stp_r, const float* stp_w,
                               float* eff, cudaStream_t s);

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
