// Weight-matrix initialisation on the host (host layout), following
// src/core/state/weight_matrix.cpp:676-1034 and the delay/distance helpers
// at :1197-1435.  Random initialisers draw from a seeded generator (the
// reference's generator is unseedable); every other initialiser, the masks and
// the callbacks behave as in the reference.
#pragma once
#include <cstdint>
#include <random>
#include <vector>

#include "state.h"

namespace sg {

// Library-wide seed for random initialisers ("seed" in a weight config or
// layer overrides it for that object).
void set_global_seed(uint64_t seed);
uint64_t global_seed();
std::mt19937_64 make_rng(const Props& cfg, uint64_t salt);

void init_weights(State& st, ConnState& cs);
// Compacts a "sparse" connection's initialised weights (and any callback
// delays / distances): the connection becomes SPARSE.
void sparsify(State& st, ConnState& cs);

// Pre-wrap source / destination coordinates per weight (host layout), as the
// reference's index kernels leave them (weight_matrix.cpp:1039-1195).
struct Indices {
    std::vector<int> from_row, from_col, from_index, to_row, to_col, to_index, used;
};
Indices compute_indices(const Connection& c);
std::vector<float> compute_distances(const Connection& c, const Indices& ix, float from_spacing,
                                     float to_spacing, float x_offset, float y_offset);
// delay = base + distance / velocity, capped at 31 (errors above 31 unless capped).
void compute_delays(const Connection& c, const std::vector<float>& dist, float velocity,
                    bool cap, int32_t* delays);

}  // namespace sg
