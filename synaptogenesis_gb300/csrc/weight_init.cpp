#include "weight_init.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <sstream>

#include "callbacks.h"
#include "counter_rng.h"

namespace sg {

static uint64_t g_seed = 0x5eed5eedULL;

void set_global_seed(uint64_t seed) { g_seed = seed; }
uint64_t global_seed() { return g_seed; }

std::mt19937_64 make_rng(const Props& cfg, uint64_t salt) {
    uint64_t seed = cfg.has("seed") ? std::stoull(cfg.get("seed")) : g_seed;
    return std::mt19937_64(seed ^ (salt * 0x9E3779B97F4A7C15ULL));
}

Indices compute_indices(const Connection& c) {
    Indices ix;
    size_t n = c.num_weights;
    if (c.type == SPARSE) {      // the compacted indices, as before wrapping
        const SparseTable& t = *c.sparse_table;
        const int fcols = c.from->cols, tcols = c.to->cols;
        ix.from_row = t.from_row; ix.from_col = t.from_col;
        ix.to_row = t.to_row; ix.to_col = t.to_col;
        ix.from_index.assign(n, -1); ix.to_index.assign(n, -1); ix.used.assign(n, 0);
        for (size_t i = 0; i < n; ++i) {
            if (t.to_row[i] < 0) continue;
            ix.from_index[i] = t.from_row[i] * fcols + t.from_col[i];
            ix.to_index[i] = t.to_row[i] * tcols + t.to_col[i];
            ix.used[i] = 1;
        }
        return ix;
    }
    ix.from_row.assign(n, -1); ix.from_col.assign(n, -1); ix.from_index.assign(n, -1);
    ix.to_row.assign(n, -1); ix.to_col.assign(n, -1); ix.to_index.assign(n, -1);
    ix.used.assign(n, 0);
    const bool arbor = c.type == CONVERGENT || c.type == DIVERGENT;
    const int fcols = c.from->cols, tcols = c.to->cols;
    enumerate_visits(c, [&](int, int to, int from, long wi, int pr, int pc) {
        int r = arbor ? pr : from / fcols;
        int cc = arbor ? pc : from % fcols;
        ix.from_row[wi] = r;
        ix.from_col[wi] = cc;
        ix.from_index[wi] = r * fcols + cc;
        ix.to_row[wi] = to / tcols;
        ix.to_col[wi] = to % tcols;
        ix.to_index[wi] = to;
        ix.used[wi] = 1;
    });
    return ix;
}

std::vector<float> compute_distances(const Connection& c, const Indices& ix, float from_spacing,
                                     float to_spacing, float x_offset, float y_offset) {
    std::vector<float> d(c.num_weights, 0.0f);
    for (size_t i = 0; i < d.size(); ++i) {
        float f_y = ix.from_row[i] * from_spacing;
        float f_x = ix.from_col[i] * from_spacing;
        float t_y = ix.to_row[i] * to_spacing + y_offset;
        float t_x = ix.to_col[i] * to_spacing + x_offset;
        d[i] = std::pow(std::pow(t_x - f_x, 2) + std::pow(t_y - f_y, 2), 0.5);
    }
    return d;
}

void compute_delays(const Connection& c, const std::vector<float>& dist, float velocity,
                    bool cap, int32_t* delays) {
    for (size_t i = 0; i < dist.size(); ++i) {
        int delay = c.delay + (dist[i] / velocity);
        if (delay > 31 && !cap)
            throw SgError(c.str() + ": BIT delays cannot be greater than 31!");
        delays[i] = delay < 31 ? delay : 31;
    }
}

// ---------------------------------------------------------------------------
// Initialisers (weight_matrix.cpp:676-851)
// ---------------------------------------------------------------------------
static void set_fraction(float* w, size_t n, float val, float fraction, std::mt19937_64& rng) {
    if (fraction == 1.0f) {
        for (size_t i = 0; i < n; ++i) w[i] = val;
    } else {
        std::uniform_real_distribution<float> d(0.0f, 1.0f);
        for (size_t i = 0; i < n; ++i)
            if (d(rng) < fraction) w[i] = val;
    }
}

static void circular_mask(const Connection& c, const Props& cfg, float* w) {
    if (c.type != CONVERGENT)
        throw SgError(c.str() + ": CircularMaskConfig can only be used on convergent arborized connections!");
    int rf = c.arbor.row_field, cf = c.arbor.col_field, K = c.arbor.kernel();
    float row_radius = cfg.get_float("row radius", 0), col_radius = cfg.get_float("column radius", 0);
    float row_d = cfg.get_float("row diameter", 0), col_d = cfg.get_float("column diameter", 0);
    float radius = cfg.get_float("radius", 0), diameter = cfg.get_float("diameter", 0);
    bool invert = cfg.get_bool("invert", false);
    float value = cfg.get_float("value", 0.0f);
    if (row_radius <= 0)
        row_radius = row_d > 0 ? row_d / 2 : radius > 0 ? radius : diameter > 0 ? diameter / 2 : float(rf) / 2;
    if (col_radius <= 0)
        col_radius = col_d > 0 ? col_d / 2 : radius > 0 ? radius : diameter > 0 ? diameter / 2 : float(cf) / 2;
    if (row_radius <= 0 || col_radius <= 0)
        throw SgError(c.str() + ": Circular mask weight config radii must be positive!");
    float row_center = float(rf) / 2, col_center = float(cf) / 2;
    float row_sq = row_radius * row_radius, col_sq = col_radius * col_radius;
    float sq_mult = row_sq * col_sq;
    long reps = c.convolutional ? 1 : c.to->size;
    for (long idx = 0; idx < reps; ++idx)
        for (int kr = 0; kr < rf; ++kr)
            for (int kc = 0; kc < cf; ++kc) {
                float a = (float)(kr + 0.5 - row_center);
                float b = (float)(kc + 0.5 - col_center);
                float term = (a * a * col_sq) + (b * b * row_sq);
                if (invert == (term <= sq_mult)) w[idx * K + kr * cf + kc] = value;
            }
}

static void clear_diagonal(const Connection& c, float* w) {
    switch (c.type) {
        case FULLY_CONNECTED: {
            if (c.from->size != c.to->size)
                throw SgError("Attempted to clear diagonal of non-square weight matrix!");
            for (long i = 0; i < c.from->size; ++i) w[i * c.from->size + i] = 0.0f;
            break;
        }
        case SUBSET: {
            int fs = c.subset.from_size();
            if (fs != c.subset.to_size())
                throw SgError("Attempted to clear diagonal of non-square weight matrix!");
            for (long i = 0; i < fs; ++i) w[i * fs + i] = 0.0f;
            break;
        }
        case CONVERGENT: {
            Props p;
            p.set("radius", "0.5");
            p.set("invert", "true");
            circular_mask(c, p, w);
            break;
        }
        default: break;
    }
}

void init_weights(State& st, ConnState& cs) {
    Connection& c = *cs.conn;
    Props empty;
    const Props& cfg = c.config.child("weight config") ? *c.config.child("weight config") : empty;
    size_t n = c.num_weights;
    float* w = cs.weights->hf();
    auto rng = make_rng(cfg, 1000 + c.index);

    if (cfg.has("fraction")) {
        float f = cfg.get_float("fraction", 1.0f);
        if (f < 0 || f > 1.0f) throw SgError(c.str() + ": Weight config fraction must be between 0 and 1!");
    }
    float fraction = cfg.get_float("fraction", 1.0f);
    std::string type = cfg.get("type", "flat");
    if (type == "flat") {
        set_fraction(w, n, cfg.get_float("weight", 1.0f), fraction, rng);
    } else if (type == "random") {
        float mx = cfg.get_float("max weight", c.max_weight), mn = cfg.get_float("min weight", 0.0f);
        std::uniform_real_distribution<float> d(mn, mx);
        std::uniform_real_distribution<float> fd(0.0f, 1.0f);
        for (size_t i = 0; i < n; ++i)
            if (fraction == 1.0f || fd(rng) < fraction) w[i] = d(rng);
    } else if (type == "gaussian" || type == "log normal") {
        float mean = cfg.get_float("mean", 1.0f), sd = cfg.get_float("std dev", 0.3f);
        if (sd < 0) throw SgError(c.str() + ": weight config std_dev must be positive!");
        if (sd == 0.0f) {
            set_fraction(w, n, mean, fraction, rng);
        } else {
            std::normal_distribution<double> nd(mean, sd);
            std::lognormal_distribution<double> ld(mean, sd);
            std::uniform_real_distribution<double> fd(0.0, 1.0);
            bool logn = type == "log normal";
            for (size_t i = 0; i < n; ++i) {
                if (fraction != 1.0f && !(fd(rng) < fraction)) { w[i] = 0.0f; continue; }
                double v = logn ? ld(rng) : nd(rng);
                w[i] = (float)std::min((double)c.max_weight, std::max(0.0, v));
            }
        }
    } else if (type == "power law") {
        float ex = std::fabs(cfg.get_float("exponent", 1.5f));
        float mx = cfg.get_float("max weight", c.max_weight), mn = cfg.get_float("min weight", 0.0f);
        if (c.max_weight < 0) throw SgError(c.str() + ": Power law config max must be positive!");
        std::uniform_real_distribution<float> d(0.0f, 1.0f);
        float ca = std::pow(mx, 1.0 - ex);
        float cb = std::pow(std::max(mn, 0.00001f), 1.0 - ex);
        float coeff = ca - cb, pexp = 1.0 / (1.0 - ex);
        for (size_t i = 0; i < n; ++i) {
            if (fraction != 1.0f && !(d(rng) < fraction)) { w[i] = 0.0f; continue; }
            w[i] = std::pow(coeff * d(rng) + cb, pexp);
        }
    } else if (type == "specified") {
        std::string s = cfg.get("weight string", "");
        if (s.empty()) throw SgError(c.str() + ": Missing weight string for specified weight config!");
        std::stringstream ss(s);
        float v = 0.0f;
        for (long i = 0; i < (long)n; ++i) {
            if (!(ss >> v)) throw SgError(c.str() + ": Insufficient number of weights specified!");
            w[i] = v;
        }
    } else {
        throw SgError(c.str() + ": Unrecognized weight config type: " + type);
    }

    auto& cb = Callbacks::get();
    int id = cfg.get_int("id", 0);
    if (cfg.has("callback"))
        Callbacks::find(cb.weight, cfg.get("callback"), "weight")(id, (int)n, w);
    if (cfg.has("indices callback")) {
        Indices ix = compute_indices(c);
        Callbacks::find(cb.indices, cfg.get("indices callback"), "indices")(
            id, (int)n, w, ix.from_index.data(), ix.to_index.data(), ix.used.data());
    }
    if (cfg.has("distance callback")) {
        float fs = cfg.has("from spacing") ? cfg.get_float("from spacing", 1.0f)
                                           : c.from->config.get_float("neuron spacing", 1.0f);
        float ts = cfg.has("to spacing") ? cfg.get_float("to spacing", 1.0f)
                                         : c.to->config.get_float("neuron spacing", 1.0f);
        Indices ix = compute_indices(c);
        std::vector<float> dist = compute_distances(c, ix, fs, ts, cfg.get_float("x offset", 0.0f),
                                                    cfg.get_float("y offset", 0.0f));
        Callbacks::find(cb.distance, cfg.get("distance callback"), "distance")(id, (int)n, w, dist.data());
        cs.params["__has_distances"] = 1.0f;
        cs.cached_distances = std::move(dist);
    }
    if (cfg.has("delay callback")) {
        if (!cs.delays) {
            cs.delays = st.add_array("delays", 'i', n, matrix_layout(c), c.matrix_rows, c.matrix_cols);
            for (size_t i = 0; i < n; ++i) cs.delays->hi()[i] = c.delay;
        }
        Callbacks::find(cb.delay, cfg.get("delay callback"), "delay")(id, (int)n, w, cs.delays->hi());
    }
    if (Props* m = cfg.child("circular mask")) circular_mask(c, *m, w);
    for (Props* m : cfg.child_array("circular mask")) circular_mask(c, *m, w);
    if (!cfg.get_bool("diagonal", true)) clear_diagonal(c, w);
}

// Seed of a randomized projection's draws: the weight config's "seed", else
// derived from the global seed and the connection's index (the reference's
// generator is unseeded).
static uint64_t randomized_seed(const Connection& c) {
    const Props* wc = c.config.child("weight config");
    return (wc && wc->has("seed")) ? std::stoull(wc->get("seed"))
                                   : (g_seed ^ (0xA11CE5ULL * (uint64_t)(c.index + 1)));
}

// Randomized divergent projection (weight_matrix.cpp:443-504): the inverted,
// convergent connection (destination and source layers swapped, the same
// arborized config; Connection::invert, connection.cpp:108-124) is built and
// randomized as a convergent one -- each source's field shifted so that its
// first position lands on a random destination (seeded draws), indexed with
// the destination layer's row count as the row pitch -- and its indices are
// adjusted (wrapped, or positions outside the layer dropped); then every kept
// (source, destination) pair is flipped into the divergent matrix, in the
// inverse's order, at the destination's next free position.  Where a
// destination would receive more sources than the kernel has positions the
// reference writes past that destination's row; that is refused here, as is
// a pitch-quirk index outside the destination layer.  (The reference also
// drops the inverse's zero weights, drawn from the same weight config and
// unseeded; here every kept pair of the inverse is flipped.)
static Indices randomized_divergent(const Connection& c, uint64_t seed) {
    const Layer& S = *c.from;
    const Layer& D = *c.to;
    const Arbor& a = c.arbor;
    const int K = a.kernel();
    const size_t n = (size_t)D.size * K;
    Indices ix;
    ix.from_row.assign(n, -1); ix.from_col.assign(n, -1); ix.from_index.assign(n, -1);
    ix.to_row.assign(n, -1); ix.to_col.assign(n, -1); ix.to_index.assign(n, -1);
    ix.used.assign(n, 0);
    std::vector<int> count(D.size, 0);
    for (int s = 0; s < S.size; ++s) {
        const int sr = s / S.cols, sc = s % S.cols;
        // the inverse's window of s in D starts at s * stride + spacing * offset
        const int r0 = sr * a.row_stride + a.row_spacing * a.row_offset;
        const int c0 = sc * a.col_stride + a.col_spacing * a.col_offset;
        const int nr = (int)rng_below(seed, 2 * (uint64_t)s, 0, (uint32_t)D.rows);
        const int nc = (int)rng_below(seed, 2 * (uint64_t)s + 1, 0, (uint32_t)D.cols);
        for (int kr = 0; kr < a.row_field; ++kr)
            for (int kc = 0; kc < a.col_field; ++kc) {
                int r = r0 + kr * a.row_spacing + (nr - r0);
                int q = c0 + kc * a.col_spacing + (nc - c0);
                int idx = r * D.rows + q;
                if (a.wrap) {
                    r = (r % D.rows + D.rows) % D.rows;
                    q = (q % D.cols + D.cols) % D.cols;
                    idx = r * D.cols + q;
                } else if (r < 0 || r >= D.rows || q < 0 || q >= D.cols) {
                    continue;
                }
                if (idx < 0 || idx >= D.size)
                    throw SgError(c.str() + ": randomized projection indexes outside the "
                                  "destination layer (the row pitch is its row count; use a "
                                  "square layer)");
                const int slot = count[idx]++;
                if (slot >= K)
                    throw SgError(c.str() + ": randomized divergent projection gives destination " +
                                  std::to_string(idx) + " more than " + std::to_string(K) +
                                  " sources");
                const size_t j = (size_t)idx * K + slot;
                ix.from_row[j] = sr; ix.from_col[j] = sc; ix.from_index[j] = s;
                ix.to_row[j] = r; ix.to_col[j] = q; ix.to_index[j] = idx;
                ix.used[j] = 1;
            }
    }
    return ix;
}

// ---------------------------------------------------------------------------
// WeightMatrix::sparsify and adjust_sparse_indices (weight_matrix.cpp:510-651,
// 253-338), run when the dense weights (and any callback delays or
// distances) are in place, before the model processes the matrix.
// ---------------------------------------------------------------------------
void sparsify(State& st, ConnState& cs) {
    Connection& c = *cs.conn;
    if (c.convolutional)
        throw SgError("Error intializing weight matrix for " + c.str() +
                      "\n   Cannot sparsify convolutional weight matrix!");
    const int rows = c.matrix_rows, cols = c.matrix_cols, to_size = c.to->size;
    const float* w = cs.weights->hf();
    Indices ix = compute_indices(c);
    const int frows = c.from->rows, fcols = c.from->cols;
    if (c.randomized && c.type == DIVERGENT) {
        ix = randomized_divergent(c, randomized_seed(c));
    } else if (c.randomized) {
        // randomize_projection (weight_matrix.cpp:377-437), with seeded draws
        // (the reference's generator is unseeded): one to one takes a random
        // source per destination; convergent shifts each destination's field
        // so that its first position lands on a random source, and -- as the
        // reference -- indexes the shifted sources with the source layer's
        // row count as the row pitch.
        const uint64_t seed = randomized_seed(c);
        for (int d = 0; d < to_size; ++d) {
            const int nr = (int)rng_below(seed, 2 * (uint64_t)d, 0, (uint32_t)frows);
            const int nc = (int)rng_below(seed, 2 * (uint64_t)d + 1, 0, (uint32_t)fcols);
            if (c.type == ONE_TO_ONE) {
                ix.from_row[d] = nr;
                ix.from_col[d] = nc;
                ix.from_index[d] = nr * fcols + nc;
            } else {
                const size_t corner = (size_t)d * cols;
                const int dr = nr - ix.from_row[corner], dc = nc - ix.from_col[corner];
                for (int k = 0; k < cols; ++k) {
                    const int r = ix.from_row[corner + k] += dr;
                    const int q = ix.from_col[corner + k] += dc;
                    ix.from_index[corner + k] = r * frows + q;
                }
            }
        }
    }
    std::vector<int> used(ix.used);
    int kmax = 0;
    for (int r = 0; r < rows; ++r) {
        int nz = 0;
        for (int k = 0; k < cols; ++k) {
            size_t i = (size_t)r * cols + k;
            if (w[i] == 0.0f) used[i] = 0;
            nz += used[i];
        }
        kmax = std::max(kmax, nz);
    }
    if (kmax == 0) {
        // an all-zero matrix keeps one synapse per row (its first weight
        // position); rows whose first position is no synapse stay empty
        // instead of reading outside the source layer
        kmax = 1;
        for (int r = 0; r < rows; ++r) used[(size_t)r * cols] = ix.used[(size_t)r * cols];
    }
    const size_t n = (size_t)kmax * to_size;
    auto t = std::make_shared<SparseTable>();
    t->kmax = kmax;
    t->nonzero.assign(to_size, 0);
    t->from.assign(n, -1);
    t->from_row.assign(n, -1); t->from_col.assign(n, -1);
    t->to_row.assign(n, -1); t->to_col.assign(n, -1);
    std::vector<float> nw(n, 0.0f);
    std::vector<size_t> old_of(n, (size_t)-1);
    for (int r = 0; r < rows; ++r) {
        int k = 0;
        for (int col = 0; col < cols; ++col) {
            size_t i = (size_t)r * cols + col;
            if (!used[i]) continue;
            size_t j = (size_t)r * kmax + k++;
            nw[j] = w[i];
            old_of[j] = i;
            t->from_row[j] = ix.from_row[i]; t->from_col[j] = ix.from_col[i];
            t->to_row[j] = ix.to_row[i]; t->to_col[j] = ix.to_col[i];
        }
        t->nonzero[r] = k;
    }
    // Source indices for the kernels (adjust_sparse_indices,
    // weight_matrix.cpp:253-338): a wrapping arbor wraps its coordinates and
    // recomputes the index; otherwise a synapse outside the source layer
    // (only a randomized projection has them) is dropped and the row's later
    // sources move up -- the sources only: the weights and delays stay where
    // they are, as in the reference.
    const bool wrap = (c.dense_type == CONVERGENT || c.dense_type == DIVERGENT) && c.arbor.wrap;
    const int fr = frows, fc = fcols;
    for (int r = 0; r < to_size; ++r) {
        int kept = 0;
        for (int k = 0; k < t->nonzero[r]; ++k) {
            const size_t j = (size_t)r * kmax + k;
            int a = t->from_row[j], b = t->from_col[j];
            int idx = (int)ix.from_index[old_of[j]];
            if (wrap) {
                a = (a % fr + fr) % fr;
                b = (b % fc + fc) % fc;
                idx = a * fc + b;
            } else if (a < 0 || a >= fr || b < 0 || b >= fc) {
                continue;
            }
            // the row-pitch quirk of randomized convergent projections can
            // index past a non-square source layer; the reference then reads
            // outside its output array
            if (idx < 0 || idx >= c.from->size)
                throw SgError(c.str() + ": randomized projection indexes outside the source layer "
                              "(the row pitch is its row count; use a square source layer)");
            t->from[(size_t)r * kmax + kept++] = idx;
        }
        for (int k = kept; k < t->nonzero[r]; ++k) t->from[(size_t)r * kmax + k] = -1;
        t->nonzero[r] = kept;
    }
    // compact the callback-set per-synapse arrays the same way
    auto compact = [&](const uint32_t* src, uint32_t fill) {
        std::vector<uint32_t> out(n, fill);
        for (size_t j = 0; j < n; ++j) if (old_of[j] != (size_t)-1) out[j] = src[old_of[j]];
        return out;
    };
    if (!cs.cached_distances.empty()) {
        std::vector<float> d(n, 0.0f);
        for (size_t j = 0; j < n; ++j) if (old_of[j] != (size_t)-1) d[j] = cs.cached_distances[old_of[j]];
        cs.cached_distances = std::move(d);
    }
    std::vector<uint32_t> delays;
    if (cs.delays) delays = compact(cs.delays->hu(), 0u);
    // Connection::sparsify: the compacted shape (connection.cpp:219-222)
    c.type = SPARSE;
    c.num_weights = (long)n;
    c.matrix_rows = to_size;
    c.matrix_cols = kmax;
    c.sparse_table = t;
    st.remove_array(cs.weights);
    cs.weights = st.add_array("weights", 'f', n, matrix_layout(c), c.matrix_rows, c.matrix_cols);
    std::memcpy(cs.weights->hf(), nw.data(), n * 4);
    if (cs.delays) {
        st.remove_array(cs.delays);
        cs.delays = st.add_array("delays", 'i', n, matrix_layout(c), c.matrix_rows, c.matrix_cols);
        std::memcpy(cs.delays->hu(), delays.data(), n * 4);
    }
    cs.sparse_nonzero = st.add_array("nonzero counts", 'i', to_size);
    std::memcpy(cs.sparse_nonzero->hi(), t->nonzero.data(), (size_t)to_size * 4);
    cs.sparse_from = st.add_array("from indices", 'i', n, matrix_layout(c), c.matrix_rows, c.matrix_cols);
    std::memcpy(cs.sparse_from->hi(), t->from.data(), n * 4);
    cs.geom = make_geom(c);
}

}  // namespace sg
