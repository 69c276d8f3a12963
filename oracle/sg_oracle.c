/*
 * sg_oracle.c -- CPU restatement of the synaptogenesis per-timestep cycle.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker used by tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg.  The product
 * (synaptogenesis_gb300/) never links, loads or calls it.
 *
 * Each function restates the serial (OpenMP, one thread) loop of the
 * reference with the same operation order and the same float/double
 * promotions, so that results are bit-identical to the reference's CPU path
 * when built with -ffp-contract=off.  Citations are file:line in the
 * reference checkout.
 *
 * Layouts are the reference's host ("CPU") layouts:
 *   fully connected  w[to * from_size + from]         synapse_kernel.h:143
 *   subset           w[to_k * from_k_size + from_k]   synapse_kernel.h:218-220
 *   one to one       w[i]                             synapse_kernel.h:265
 *   convergent       w[to * K + k] or w[k] (conv.)    synapse_kernel.h:440-443
 *   divergent        w[to * (n_w / to_size) + k] / w[k]  synapse_kernel.h:567-570
 */
#include <math.h>
#include <stdlib.h>
#include <stdint.h>
#include <string.h>

enum { FULLY_CONNECTED = 0, SUBSET = 1, ONE_TO_ONE = 2, CONVERGENT = 3, DIVERGENT = 4 };
enum { OUT_FLOAT = 0, OUT_BIT = 1, OUT_INT = 2 };
enum { OP_ADD, OP_SUB, OP_MULT, OP_DIV, OP_POOL, OP_REWARD, OP_MODULATE, OP_GAP,
       OP_ADD_HEAVISIDE, OP_SUB_HEAVISIDE, OP_MULT_HEAVISIDE };

/* Connection geometry, as derived by ConnectionConfig / ArborizedConfig /
 * SubsetConfig (network/connection_config.cpp:8-45, 112-134). */
typedef struct {
    int type, opcode, convolutional, num_weights;
    int from_rows, from_cols, to_rows, to_cols;
    int row_field, col_field, row_stride, col_stride;
    int row_spacing, col_spacing, row_offset, col_offset, wrap;
    int fr0, fr1, fc0, fc1, tr0, tr1, tc0, tc1;
} sg_conn;

static int wrap_index(int x, int n) { return (x % n + n) % n; }

/* Enumerates every (destination, source, weight) visit of a connection in the
 * reference's serial loop order.  Rows are destinations in loop order; for row
 * r, visits ptr[r] .. ptr[r+1]-1.  pre_row/pre_col receive the pre-wrap source
 * coordinates (used by the index kernels, weight_matrix.cpp:1049-1083).
 * Returns the number of visits; pass NULL arrays to count only.
 *   FC          synapse_kernel.h:115-149
 *   subset      synapse_kernel.h:182-228
 *   one to one  synapse_kernel.h:257-286
 *   convergent  synapse_kernel.h:384-461 (out-of-range sources skipped, k advances)
 *   divergent   synapse_kernel.h:506-581 (C truncating division) */
long sg_visits(const sg_conn *c, int *rows_out, int *dst, long *ptr,
               int *from_idx, int *w_idx, int *pre_row, int *pre_col) {
    long n = 0;
    int r = 0;
    const int from_size = c->from_rows * c->from_cols;
    const int to_size = c->to_rows * c->to_cols;
#define VISIT(F, W, PR, PC) do { if (from_idx) { from_idx[n] = (F); w_idx[n] = (W); \
        if (pre_row) { pre_row[n] = (PR); pre_col[n] = (PC); } } ++n; } while (0)
#define ROW_OPEN(T) do { if (dst) { dst[r] = (T); ptr[r] = n; } } while (0)
    switch (c->type) {
    case FULLY_CONNECTED:
        for (int to = 0; to < to_size; ++to, ++r) {
            ROW_OPEN(to);
            int wi = to * from_size;
            for (int fr = 0; fr < c->from_rows; ++fr)
                for (int fc = 0; fc < c->from_cols; ++fc, ++wi)
                    VISIT(fr * c->from_cols + fc, wi, fr, fc);
        }
        break;
    case SUBSET: {
        int kcols = c->tc1 - c->tc0, krows = c->tr1 - c->tr0;
        int from_k_size = (c->fr1 - c->fr0) * (c->fc1 - c->fc0);
        for (int i = 0; i < krows; ++i)
            for (int j = 0; j < kcols; ++j, ++r) {
                int to_k = i * kcols + j;
                ROW_OPEN((i + c->tr0) * c->to_cols + (j + c->tc0));
                int fk = 0;
                for (int fr = c->fr0; fr < c->fr1; ++fr)
                    for (int fc = c->fc0; fc < c->fc1; ++fc, ++fk)
                        VISIT(fr * c->from_cols + fc, to_k * from_k_size + fk, fr, fc);
            }
        break;
    }
    case ONE_TO_ONE:
        for (int i = 0; i < from_size; ++i, ++r) {
            ROW_OPEN(i);
            VISIT(i, i, i / c->from_cols, i % c->from_cols);
        }
        break;
    case CONVERGENT: {
        int K = c->row_field * c->col_field;
        for (int tr = 0; tr < c->to_rows; ++tr)
            for (int tc = 0; tc < c->to_cols; ++tc, ++r) {
                int to = tr * c->to_cols + tc;
                ROW_OPEN(to);
                int woff = c->convolutional ? 0 : to * K;
                int s_row = tr * c->row_stride + c->row_spacing * c->row_offset;
                int s_col = tc * c->col_stride + c->col_spacing * c->col_offset;
                int k = 0;
                for (int kr = 0; kr < c->row_field; ++kr)
                    for (int kc = 0; kc < c->col_field; ++kc, ++k) {
                        int fr = s_row + kr * c->row_spacing, fc = s_col + kc * c->col_spacing;
                        int pr = fr, pc = fc;
                        if (c->wrap) { fr = wrap_index(fr, c->from_rows); fc = wrap_index(fc, c->from_cols); }
                        else if (fr < 0 || fr >= c->from_rows || fc < 0 || fc >= c->from_cols) continue;
                        VISIT(fr * c->from_cols + fc, woff + k, pr, pc);
                    }
            }
        break;
    }
    case DIVERGENT: {
        int per = c->num_weights / to_size;
        for (int tr = 0; tr < c->to_rows; ++tr)
            for (int tc = 0; tc < c->to_cols; ++tc, ++r) {
                int to = tr * c->to_cols + tc;
                ROW_OPEN(to);
                int woff = c->convolutional ? 0 : to * per;
                int sr0 = (tr + c->row_spacing * (-c->row_offset - c->row_field + c->row_stride)) / c->row_stride;
                int sc0 = (tc + c->col_spacing * (-c->col_offset - c->col_field + c->col_stride)) / c->col_stride;
                int sr1 = sr0 + (c->row_spacing * (c->row_field - c->row_stride) / c->row_stride);
                int sc1 = sc0 + (c->col_spacing * (c->col_field - c->col_stride) / c->col_stride);
                int k = 0;
                for (int sr = sr0; sr <= sr1; sr += c->row_spacing)
                    for (int sc = sc0; sc <= sc1; sc += c->col_spacing, ++k) {
                        int fr = sr, fc = sc;
                        if (c->wrap) { fr = wrap_index(fr, c->from_rows); fc = wrap_index(fc, c->from_cols); }
                        else if (fr < 0 || fr >= c->from_rows || fc < 0 || fc >= c->from_cols) continue;
                        VISIT(fr * c->from_cols + fc, woff + k, sr, sc);
                    }
            }
        break;
    }
    }
    if (dst) ptr[r] = n;
    if (rows_out) *rows_out = r;
#undef VISIT
#undef ROW_OPEN
    return n;
}

/* extractor.cpp:6-14 -- bit: (w << (delay & 31)) >> 31 on the chosen word. */
static float extract(uint32_t word, int delay, int src_type) {
    union { uint32_t i; float f; } u;
    u.i = word;
    switch (src_type) {
    case OUT_FLOAT: return u.f;
    case OUT_INT: return (float)u.i;
    default: return (float)((word << (delay & 0x1F)) >> 31);
    }
}

/* aggregator.cpp:66-81 (serial build: MAX is std::fmax, util/parallel.h:66-67) */
static float aggregate(float prior, float input, int opcode) {
    switch (opcode) {
    case OP_ADD: return prior + input;
    case OP_SUB: return prior - input;
    case OP_MULT: return prior * input;
    case OP_DIV: return prior / input;
    case OP_POOL: return fmaxf(prior, input);
    case OP_ADD_HEAVISIDE: return prior + (input > 0);
    case OP_SUB_HEAVISIDE: return prior - (input > 0);
    case OP_MULT_HEAVISIDE: return prior * (input > 0);
    default: return prior + input;
    }
}

/* Base activator ACTIVATE_ALL(activate_base): synapse_kernel.h:887-912,
 * kernel.cpp:217.  sum starts at 0.0 and accumulates sequentially per
 * destination; the source word is the connection's word index slice. */
void sg_act_base(int rows, const int *dst, const long *ptr, const int *from_idx,
                 const int *w_idx, const uint32_t *src_words, int src_type, int delay,
                 int opcode, const float *weights, float *inputs) {
    for (int r = 0; r < rows; ++r) {
        float sum = 0.0;
        for (long v = ptr[r]; v < ptr[r + 1]; ++v) {
            float val = extract(src_words[from_idx[v]], delay, src_type) * weights[w_idx[v]];
            sum += val;
        }
        inputs[dst[r]] = aggregate(inputs[dst[r]], sum, opcode);
    }
}

/* Second-order slave (ACTIVATE_ALL_SECOND_ORDER, synapse_kernel.h:918-975):
 * each visited synapse modulates the host's weight copy with the slave's own
 * opcode; the host later activates with that copy. */
void sg_act_second_order(int rows, const int *dst, const long *ptr, const int *from_idx,
                         const int *w_idx, const uint32_t *src_words, int src_type, int delay,
                         int opcode, const float *weights, float *so) {
    (void)dst;
    for (int r = 0; r < rows; ++r)
        for (long v = ptr[r]; v < ptr[r + 1]; ++v) {
            float val = extract(src_words[from_idx[v]], delay, src_type) * weights[w_idx[v]];
            so[w_idx[v]] = aggregate(so[w_idx[v]], val, opcode);
        }
}

/* Convolutional slave: the one-to-one loop (synapse_kernel.h:255-275) over
 * the shared kernel, whose size is the source layer's. */
void sg_act_second_order_conv(int n, const uint32_t *src_words, int src_type, int delay,
                              int opcode, const float *weights, float *so) {
    for (int k = 0; k < n; ++k)
        so[k] = aggregate(so[k], extract(src_words[k], delay, src_type) * weights[k], opcode);
}

/* calc_internal_SERIAL (kernel.cpp:161-170): fold an internal dendritic
 * node's register into its parent's, then reset it to its init value. */
void sg_calc_internal(int size, float *src, float *dst, int opcode, float trail) {
    for (int i = 0; i < size; ++i) {
        dst[i] = aggregate(dst[i], src[i], opcode);
        src[i] = trail;
    }
}

/* Izhikevich trace activators: izhikevich_attributes.cpp:228-352.
 * long_tau < 0 selects the single-trace variants (mult, reward).
 * from_tss is updated per visit in serial order (F7). */
void sg_act_iz(int rows, const int *dst, const long *ptr, const int *from_idx,
               const int *w_idx, const uint32_t *src_words, int src_type,
               const float *weights, const float *stp_rs, const float *stp_ws,
               const int *delays, int *from_tss, float *short_traces, float *long_traces,
               float baseline_conductance, float short_tau, float long_tau,
               float *short_cond, float *long_cond) {
    for (int r = 0; r < rows; ++r) {
        float short_sum = 0.0;
        float long_sum = 0.0;
        for (long v = ptr[r]; v < ptr[r + 1]; ++v) {
            int f = from_idx[v], w = w_idx[v];
            float spike = extract(src_words[f], delays[w], src_type);
            from_tss[f] = (spike > 0.0) ? 0 : (int)fmin(32, from_tss[f] + 1);
            float weight = weights[w] * (stp_rs[w] * stp_ws[w]);
            float short_trace = short_traces[w] + (spike * weight * baseline_conductance);
            short_sum += short_trace;
            short_traces[w] = short_trace * short_tau;
            if (long_tau >= 0) {
                float long_trace = long_traces[w] + (spike * weight * baseline_conductance);
                long_sum += long_trace;
                long_traces[w] = long_trace * long_tau;
            }
        }
        short_cond[dst[r]] += short_sum;
        if (long_tau >= 0) long_cond[dst[r]] += long_sum;
    }
}

/* Gap junction activator: izhikevich_attributes.cpp:354-366 */
void sg_act_gap(int rows, const int *dst, const long *ptr, const int *from_idx,
                const int *w_idx, const float *voltage, const float *weights, float *inputs) {
    for (int r = 0; r < rows; ++r) {
        float v = voltage[dst[r]];
        float sum = 0.0;
        for (long e = ptr[r]; e < ptr[r + 1]; ++e)
            sum += (voltage[from_idx[e]] - v) * weights[w_idx[e]];
        inputs[dst[r]] += sum;
    }
}

/* iSTDP terms of STDP_SUB (izhikevich_attributes.cpp:454-472), evaluated with
 * the C library's powf/expf exactly as the reference's expression does. */
float sg_istdp_src(int t) {
    return (float)(powf(t, 10) * 0.000001 * 2.29 * expf(-1.1 * t));
}
float sg_istdp_dst(int t) {
    return (float)(powf(t, 10) * 0.0000001 * 2.6 * expf(-0.94 * t));
}

/* Izhikevich updaters update_iz_add / update_iz_sub:
 * izhikevich_attributes.cpp:404-520.  dest_words is word 0 of the destination
 * output (the new step's spike in bit 31).  The destination spike goes through
 * the connection's extractor, which follows the SOURCE layer's output type
 * (izhikevich_attributes.cpp:426, synapse_data.cpp:212): for a FLOAT source
 * the destination's spike word is read as a float. */
void sg_upd_iz(int rows, const int *dst, const long *ptr, const int *from_idx,
               const int *w_idx, int src_type, int is_sub, float learning_rate, int stp_flag,
               float max_weight, const float *to_exc_traces, const int *to_tss,
               const uint32_t *dest_words, const int *from_tss, float *weights,
               float *presyn_traces, float *weight_derivatives, float *stp_rs, float *stp_ws) {
    const double U = is_sub ? 0.2 : 0.5;
    const int F = is_sub ? 20 : 1000;
    const int D = is_sub ? 700 : 800;
    for (int r = 0; r < rows; ++r) {
        int to = dst[r];
        float dest_exc_trace = to_exc_traces[to];
        int dest_time_since_spike = to_tss[to];
        float dest_spike = extract(dest_words[to], 0, src_type);
        for (long e = ptr[r]; e < ptr[r + 1]; ++e) {
            int f = from_idx[e], w = w_idx[e];
            float weight = weights[w];
            if (weight >= 0.0001f) {
                int src_time_since_spike = from_tss[f];
                int src_spike = src_time_since_spike == 0;
                float src_trace, dest_trace;
                if (!is_sub) {
                    src_trace = (presyn_traces[w] = (src_spike) ? 0.004 : presyn_traces[w] * 0.933);
                    dest_trace = dest_exc_trace;
                } else {
                    src_trace = (dest_spike > 0.0 && src_time_since_spike > 0 && src_time_since_spike < 32)
                        ? sg_istdp_src(src_time_since_spike) : 0.0f;
                    dest_trace = (src_spike && dest_time_since_spike > 0 && dest_time_since_spike < 32)
                        ? sg_istdp_dst(dest_time_since_spike) : 0.0f;
                }
                float weight_delta = weight_derivatives[w];
                weight_delta = weight_derivatives[w] -=
                    (weight_delta - 0.000001) * 0.0001 + (dest_spike * src_trace)
                    - (src_spike * dest_trace);
                weight += learning_rate * weight_delta;
                weights[w] = fmaxf(0.0001f, fminf(max_weight, weight));
                if (stp_flag) {
                    float rr = stp_rs[w];
                    float ww = stp_ws[w];
                    stp_rs[w] += ((1 - rr) / D) - (rr * ww * src_spike);
                    stp_ws[w] += ((U - ww) / F) + (U * (1 - ww) * src_spike);
                }
            }
        }
    }
}

/* SHIFT_BIT_OUTPUTS (state/attributes.h:321-333); returns prev_bit. */
static int shift_bit(uint32_t *out, int size, int history, int nid, uint32_t new_bit) {
    uint32_t curr = out[(long)size * (history - 1) + nid];
    for (int idx = history - 1; idx > 0; --idx) {
        uint32_t prev = out[(long)size * (idx - 1) + nid];
        out[(long)size * idx + nid] = (curr >> 1) | (prev << 31);
        curr = prev;
    }
    out[nid] = (curr >> 1) | (new_bit << 31);
    return (int)(curr >> 31);
}

/* SHIFT_FLOAT_OUTPUTS (state/attributes.h:316-319) */
static void shift_float(float *out, int size, int history, int nid, float v) {
    for (int idx = history - 1; idx > 0; --idx)
        out[(long)size * idx + nid] = out[(long)size * (idx - 1) + nid];
    out[nid] = v;
}

/* Izhikevich neuron update: izhikevich_attributes.cpp:102-213 (powf(x,2) is
 * x*x in the reference's optimised build; IZ_* constants are doubles). */
void sg_iz_neurons(int size, int history, const float *inputs, uint32_t *spikes,
                   float *ampa, float *nmda, float *gabaa, float *gabab, float *mult,
                   float *dopamine, float *voltages, float *recoveries, float *post_traces,
                   int *tss, const float *as, const float *bs, const float *cs, const float *ds) {
    for (int nid = 0; nid < size; ++nid) {
        float ampa_conductance = ampa[nid];
        float nmda_conductance = nmda[nid];
        float gabaa_conductance = gabaa[nid];
        float gabab_conductance = gabab[nid];
        float multiplicative_factor = mult[nid];
        float voltage = voltages[nid];
        float recovery = recoveries[nid];
        float base_current = inputs[nid];
        float a = as[nid];
        float b = bs[nid];
        for (int i = 0; (i < 10) && (voltage < 30.0); ++i) {
            float current = -ampa_conductance * voltage;
            float q = (voltage + 80) / 60;
            float temp = q * q;
            current -= nmda_conductance * (temp / (1 + temp)) * voltage;
            current -= gabaa_conductance * (voltage + 70);
            current -= gabab_conductance * (voltage + 90);
            current *= 1 + multiplicative_factor;
            current += base_current;
            float delta_v = (0.04 * voltage * voltage) + (5 * voltage) + 140 - recovery + current;
            float sum_conductances = ampa_conductance + nmda_conductance
                + gabaa_conductance + gabab_conductance;
            voltage = (voltage + 0.1 * (delta_v + (gabaa_conductance * -70)
                                        + (gabab_conductance * -90)))
                      / (1 + (0.1 * sum_conductances));
            voltage = (voltage != voltage) ? 30.0 : voltage;
            float adjusted_tau = (voltage > 30.0)
                ? delta_v / (30.0 - voltage + delta_v) * 0.1
                : 0.1;
            recovery += a * adjusted_tau * ((b * voltage) - recovery);
        }
        ampa[nid] = 0.0;
        nmda[nid] = 0.0;
        gabaa[nid] = 0.0;
        gabab[nid] = 0.0;
        mult[nid] = 0.0;
        dopamine[nid] *= 0.95;
        unsigned int spike = voltage >= 30.0;
        int prev_bit = shift_bit(spikes, size, history, nid, spike);
        post_traces[nid] = (prev_bit) ? 0.004 : (post_traces[nid] * 0.95);
        tss[nid] = (prev_bit) ? 0 : (int)fmin(32, tss[nid] + 1);
        voltages[nid] = (spike) ? cs[nid] : voltage;
        recoveries[nid] = recovery + (spike * ds[nid]);
    }
}

/* Resting-state settle loop of the Izhikevich constructor:
 * izhikevich_attributes.cpp:628-649 */
/* spnet neuron update (spnet_attributes.cpp:96-166): the Izhikevich Euler
 * loop without conductances; the post trace steps by 0.1 or decays by 0.95. */
void sg_spnet_neurons(int size, int history, const float *inputs, uint32_t *spikes,
                      float *voltages, float *recoveries, float *post_traces, int *tss,
                      const float *as, const float *bs, const float *cs, const float *ds) {
    for (int nid = 0; nid < size; ++nid) {
        float voltage = voltages[nid];
        float recovery = recoveries[nid];
        float current = inputs[nid];
        float a = as[nid];
        float b = bs[nid];
        for (int i = 0; (i < 10) && (voltage < 30.0); ++i) {
            float delta_v = (0.04 * voltage * voltage) + (5 * voltage) + 140 - recovery + current;
            voltage += delta_v * 0.1;
            voltage = (voltage != voltage) ? 30.0 : voltage;
            float adjusted_tau = (voltage > 30.0) ? delta_v / (30.0 - voltage + delta_v) * 0.1 : 0.1;
            recovery += a * adjusted_tau * ((b * voltage) - recovery);
        }
        unsigned int spike = voltage >= 30.0;
        int prev_bit = shift_bit(spikes, size, history, nid, spike);
        post_traces[nid] = (prev_bit) ? (post_traces[nid] + 0.1) : (post_traces[nid] * 0.95);
        tss[nid] = (prev_bit) ? 0 : (tss[nid] + 1 < 32 ? tss[nid] + 1 : 32);
        voltages[nid] = (spike) ? cs[nid] : voltage;
        recoveries[nid] = recovery + (spike * ds[nid]);
    }
}

/* spnet activator (spnet_attributes.cpp:172-214): per-synapse delays, the
 * source's time since spike updated per visit, any aggregation opcode. */
void sg_act_spnet(int rows, const int *dst, const long *ptr, const int *from_idx,
                  const int *w_idx, const uint32_t *src_words, int src_type,
                  const float *weights, const int *delays, int *from_tss,
                  float baseline_conductance, int opcode, float *inputs) {
    for (int r = 0; r < rows; ++r) {
        float sum = 0.0;
        for (long v = ptr[r]; v < ptr[r + 1]; ++v) {
            int f = from_idx[v], w = w_idx[v];
            float spike = extract(src_words[f], delays[w], src_type);
            from_tss[f] = (spike > 0.0) ? 0 : (from_tss[f] + 1 < 32 ? from_tss[f] + 1 : 32);
            float weight = weights[w];
            sum += spike * weight * baseline_conductance;
        }
        inputs[dst[r]] = aggregate(inputs[dst[r]], sum, opcode);
    }
}

/* spnet updater (spnet_attributes.cpp:220-306) */
void sg_upd_spnet(int rows, const int *dst, const long *ptr, const int *from_idx,
                  const int *w_idx, int src_type, int is_sub, float learning_rate,
                  float max_weight, const float *to_exc_traces, const int *to_tss,
                  const uint32_t *dest_words, const int *from_tss, float *weights,
                  float *presyn_traces, float *dws) {
    for (int r = 0; r < rows; ++r) {
        int to = dst[r];
        float dest_exc_trace = to_exc_traces[to];
        int dest_time_since_spike = to_tss[to];
        float dest_spike = extract(dest_words[to], 0, src_type);
        for (long e = ptr[r]; e < ptr[r + 1]; ++e) {
            int f = from_idx[e], w = w_idx[e];
            float weight = weights[w];
            if (weight >= 0.0001f) {
                int src_time_since_spike = from_tss[f];
                int src_spike = src_time_since_spike == 0;
                float src_trace = (!is_sub)
                    ? (presyn_traces[w] = (src_spike) ? (presyn_traces[w] + 0.1)
                                                      : presyn_traces[w] * 0.95)
                    : ((dest_spike > 0.0 && src_time_since_spike > 0 && src_time_since_spike < 32)
                           ? sg_istdp_src(src_time_since_spike) : 0.0f);
                float dest_trace = (!is_sub)
                    ? dest_exc_trace
                    : ((src_spike && dest_time_since_spike > 0 && dest_time_since_spike < 32)
                           ? sg_istdp_dst(dest_time_since_spike) : 0.0f);
                float dw = dws[w] = 0.9 * dws[w] + (dest_spike * src_trace) - (src_spike * dest_trace);
                float weight_delta = dw + 0.01;
                weight += learning_rate * weight_delta;
                float capped = (max_weight < weight) ? max_weight : weight;
                weights[w] = (0.0001f > capped) ? 0.0001f : capped;
            }
        }
    }
}

void sg_iz_init(int size, const float *as, const float *bs, const float *cs,
                float *v_out, float *r_out) {
    for (int j = 0; j < size; ++j) {
        float v = cs[j];
        float r = bs[j] * cs[j];
        float delta_v, delta_r;
        float a = as[j], b = bs[j];
        do {
            delta_v = (0.04 * v * v) + (5 * v) + 140 - r;
            v += delta_v;
            delta_r = a * ((b * v) - r);
            r += delta_r;
        } while (fabsf(delta_v) > 0.001 && fabsf(delta_r) > 0.001);
        v_out[j] = v;
        r_out[j] = r;
    }
}

/* Relay: relay_attributes.cpp:10-18 (MAX is std::fmax on doubles) */
void sg_relay(int size, int history, const float *inputs, float *outputs, int ramp) {
    for (int nid = 0; nid < size; ++nid) {
        float input = inputs[nid];
        shift_float(outputs, size, history, nid, ramp ? (float)fmax(0.0, input) : input);
    }
}

/* Rate encoding: rate_encoding_attributes.cpp:122-131.  In C++ tanh(float)
 * resolves to the float overload, i.e. tanhf. */
/* binary threshold (bin_thresh_attributes.cpp:9-17) */
void sg_bin_thresh(int size, int history, const float *inputs, float *outputs) {
    for (int nid = 0; nid < size; ++nid)
        shift_float(outputs, size, history, nid, inputs[nid] > 0);
}

/* perceptron update (perceptron_attributes.cpp:13-21): the input over the
 * layer's weights per neuron (an int) */
void sg_perceptron(int size, int history, int per_neuron, const float *inputs, float *outputs) {
    for (int nid = 0; nid < size; ++nid)
        shift_float(outputs, size, history, nid, inputs[nid] / per_neuron);
}

/* perceptron activator (perceptron_attributes.cpp:27-33) */
void sg_act_perceptron(int rows, const int *dst, const long *ptr, const int *from_idx,
                       const int *w_idx, const uint32_t *src_words, int src_type, int delay,
                       int opcode, const float *weights, float *inputs) {
    for (int r = 0; r < rows; ++r) {
        float sum = 0.0;
        for (long v = ptr[r]; v < ptr[r + 1]; ++v)
            sum += (extract(src_words[from_idx[v]], delay, src_type) > 0) * weights[w_idx[v]];
        inputs[dst[r]] = aggregate(inputs[dst[r]], sum, opcode);
    }
}

/* sine generator (sine_generator_attributes.cpp:11-23): wave from the float
 * product frequency * iteration; use_sinf selects the float sine overload,
 * otherwise the sine is taken in double and the wave rounded to float. */
void sg_sine(int size, int history, float frequency, int iteration, int use_sinf,
             const float *inputs, float *outputs) {
    float x = frequency * iteration;
    float wave = use_sinf ? (1 + sinf(x)) / 2 : (float)((1 + sin(x)) / 2);
    for (int nid = 0; nid < size; ++nid)
        shift_float(outputs, size, history, nid, inputs[nid] * wave);
}

/* poisson generator (poisson_generator_attributes.cpp:9-24) with the draws
 * given */
void sg_poisson_gen(int size, int history, const float *draws, const float *inputs,
                    uint32_t *spikes) {
    for (int nid = 0; nid < size; ++nid)
        shift_bit(spikes, size, history, nid, draws[nid] < inputs[nid]);
}

/* oscillator activator (oscillator_attributes.cpp:60-92) */
void sg_act_oscillator(int rows, const int *dst, const long *ptr, const int *from_idx,
                       const int *w_idx, const uint32_t *src_words, int src_type, int delay,
                       int opcode, const float *weights, float *inputs, float *bold) {
    for (int r = 0; r < rows; ++r) {
        float sum = 0.0, abs_sum = 0.0;
        for (long v = ptr[r]; v < ptr[r + 1]; ++v) {
            float val = extract(src_words[from_idx[v]], delay, src_type) * weights[w_idx[v]];
            sum += val;
            abs_sum += fabsf(val);
        }
        inputs[dst[r]] = aggregate(inputs[dst[r]], sum, opcode);
        bold[dst[r]] += abs_sum;
    }
}

/* oscillator update (oscillator_attributes.cpp:38-55) */
void sg_oscillator(int size, int history, float tonic, float tau, float decay,
                   const float *inputs, float *state, float *bold, float *outputs) {
    for (int nid = 0; nid < size; ++nid) {
        float st = state[nid];
        float recur = st + (decay * (tonic - st));
        state[nid] = st = (tau * inputs[nid]) + recur;
        bold[nid] += recur;
        float t = tanhf(st);
        shift_float(outputs, size, history, nid, (0.0f > t) ? 0.0f : t);
    }
}

/* som activators (som_attributes.cpp:35-56): squared distance added to the
 * input (outputs cached per synapse), or for "modulate" the plasticity */
void sg_act_som(int rows, const int *dst, const long *ptr, const int *from_idx,
                const int *w_idx, const uint32_t *src_words, int src_type, int delay,
                int modulate, const float *weights, float *cache, float *inputs,
                float *plasticity) {
    for (int r = 0; r < rows; ++r) {
        float acc = 0.0;
        for (long v = ptr[r]; v < ptr[r + 1]; ++v) {
            int w = w_idx[v];
            float out = extract(src_words[from_idx[v]], delay, src_type);
            if (modulate) {
                acc += weights[w] * out;
            } else {
                float val = out - weights[w];
                cache[w] = out;
                acc += val * val;
            }
        }
        if (modulate) plasticity[dst[r]] = acc;
        else inputs[dst[r]] += acc;
    }
}

/* som update (som_attributes.cpp:13-31): winner, then exp(-rbf * x^2) */
void sg_som(int size, int history, float rbf_scale, const float *inputs, float *outputs,
            int *winner) {
    float min = inputs[0];
    int min_node = 0;
    for (int i = 0; i < size; ++i)
        if (inputs[i] < min) { min = inputs[i]; min_node = i; }
    *winner = min_node;
    for (int nid = 0; nid < size; ++nid) {
        float input = inputs[nid];
        shift_float(outputs, size, history, nid, expf(-rbf_scale * (input * input)));
    }
}

/* som updater (som_attributes.cpp:58-79) */
void sg_upd_som(int rows, const int *dst, const long *ptr, const int *w_idx, int to_cols,
                int winner, const float *plasticity, const float *cache, float lr, float nlr,
                int nbhd, float *weights) {
    int wr = winner / to_cols, wc = winner % to_cols;
    for (int r = 0; r < rows; ++r) {
        int to = dst[r];
        int rd = abs(wr - (to / to_cols)), cd = abs(wc - (to % to_cols));
        for (long v = ptr[r]; v < ptr[r + 1]; ++v) {
            int w = w_idx[v];
            if (to == winner)
                weights[w] += plasticity[to] * lr * (cache[w] - weights[w]);
            else if (rd + cd <= nbhd)
                weights[w] += plasticity[to] * nlr * (cache[w] - weights[w]);
        }
    }
}

/* NVM gate connection (nvm_attributes.cpp:61-95): the subset window's
 * sources reduced by min from 1 (decay) or max from 0; returns the value */
float sg_nvm_gate(const sg_conn *c, const uint32_t *src_words, int src_type, int delay,
                  int decay) {
    float gv = decay ? 1.0f : 0.0f;
    for (int fr = c->fr0; fr < c->fr1; ++fr)
        for (int fc = c->fc0; fc < c->fc1; ++fc) {
            float v = extract(src_words[fr * c->from_cols + fc], delay, src_type);
            gv = decay ? ((gv < v) ? gv : v) : ((gv > v) ? gv : v);
        }
    return gv;
}

/* NVM activators (nvm_attributes.cpp:97-160, nvm_compare_attributes.cpp:
 * 26-58): kind 0 plain, 1 gated, 2 plastic, 3 compare-plastic */
void sg_act_nvm(int kind, int rows, const int *dst, const long *ptr, const int *from_idx,
                const int *w_idx, const uint32_t *src_words, int src_type, int delay,
                int opcode, float *weights, float *inputs, float ag, float lg,
                const float *state, const float *context, const float *true_state,
                float norm_param, int per_neuron, float tolerance) {
    if (kind == 1 && ag < 0.5f) return;
    if ((kind == 2 || kind == 3) && ag < 0.5f && lg < 0.5f) return;
    float norm = (kind == 2) ? norm_param * per_neuron : norm_param;
    for (int r = 0; r < rows; ++r) {
        int to = dst[r];
        if ((kind == 1 || kind == 2) && !(context[to] > 0.5f)) continue;
        float sum = 0.0;
        for (long v = ptr[r]; v < ptr[r + 1]; ++v)
            sum += extract(src_words[from_idx[v]], delay, src_type) * weights[w_idx[v]];
        if (kind <= 1) {
            inputs[to] = aggregate(inputs[to], sum, opcode);
        } else if (kind == 2) {
            if (ag > 0.5f) inputs[to] = aggregate(inputs[to], sum, opcode);
            if (lg > 0.5f) {
                float temp = state[to] - sum;
                for (long v = ptr[r]; v < ptr[r + 1]; ++v)
                    weights[w_idx[v]] += extract(src_words[from_idx[v]], delay, src_type) * temp / norm;
            }
        } else {
            if (ag > 0.5f) {
                sum -= true_state[to] * ((tolerance * per_neuron) - 1);
                inputs[to] = ag * aggregate(inputs[to], sum, opcode);
            }
            if (lg > 0.5f) {
                float temp = inputs[to] = true_state[to];
                for (long v = ptr[r]; v < ptr[r + 1]; ++v)
                    weights[w_idx[v]] = extract(src_words[from_idx[v]], delay, src_type) * temp / norm;
            }
        }
    }
}

/* NVM context connection (nvm_attributes.cpp:150-160): the one-to-one loop */
void sg_act_nvm_context(int n, const uint32_t *src_words, int src_type, int delay, int opcode,
                        const float *weights, float ag, float *context) {
    if (ag < 0.5f) return;
    for (int i = 0; i < n; ++i) {
        float sum = 0.0;
        sum += extract(src_words[i], delay, src_type) * weights[i];
        context[i] = aggregate(context[i], sum, opcode);
    }
}

/* nvm / nvm_heaviside updates with the noise gate closed
 * (nvm_attributes.cpp:38-52, nvm_heaviside_attributes.cpp:11-25) */
void sg_nvm_update(int heaviside, int size, int history, const float *inputs, float *state,
                   float *context, float *outputs, float gain) {
    for (int nid = 0; nid < size; ++nid) {
        float input = inputs[nid] + 0.;
        if (!heaviside) {
            state[nid] = input;
            context[nid] = 1.;
            shift_float(outputs, size, history, nid, tanhf(input));
        } else {
            state[nid] = gain * ((input > 0) - (input <= 0));
            context[nid] = 1.;
            shift_float(outputs, size, history, nid, (float)(input > 0.));
        }
    }
}

/* vp_max activator (vp_max_attributes.cpp:46-70) */
void sg_act_vp_max(int rows, const int *dst, const long *ptr, const int *from_idx,
                   const int *w_idx, const uint32_t *src_words, int src_type, int delay,
                   int opcode, const float *weights, float *inputs) {
    for (int r = 0; r < rows; ++r) {
        float max_val = 0.0;
        for (long v = ptr[r]; v < ptr[r + 1]; ++v) {
            float val = extract(src_words[from_idx[v]], delay, src_type) * weights[w_idx[v]];
            if (val > max_val) max_val = val;
        }
        inputs[dst[r]] = aggregate(inputs[dst[r]], max_val, opcode);
    }
}

/* output = scale * input (sample_attributes.cpp:52-58) */
void sg_scale(int size, int history, float scale, const float *inputs, float *outputs) {
    for (int nid = 0; nid < size; ++nid)
        shift_float(outputs, size, history, nid, scale * inputs[nid]);
}

/* perceptron updater (perceptron_attributes.cpp:51-60): source outputs read
 * as floats */
void sg_upd_perceptron(int rows, const int *dst, const long *ptr, const int *from_idx,
                       const int *w_idx, const uint32_t *src_words, const float *dest_out,
                       const float *expected, float *weights) {
    for (int r = 0; r < rows; ++r) {
        int to = dst[r];
        float delta = expected[to] - dest_out[to];
        for (long v = ptr[r]; v < ptr[r + 1]; ++v) {
            union { uint32_t i; float f; } u;
            u.i = src_words[from_idx[v]];
            weights[w_idx[v]] += 0.05 * delta * u.f;
        }
    }
}

/* oscillator / vp_max / sample updaters (oscillator_attributes.cpp:196-206,
 * vp_max_attributes.cpp:150-160, sample_attributes.cpp:201-212) */
void sg_upd_toward_post(int rows, const int *dst, const long *ptr, const int *from_idx,
                        const int *w_idx, const uint32_t *src_words, int src_type, int delay,
                        const uint32_t *dest_words, float rate, float *weights) {
    for (int r = 0; r < rows; ++r) {
        int to = dst[r];
        float to_out = extract(dest_words[to], 0, src_type);
        for (long v = ptr[r]; v < ptr[r + 1]; ++v) {
            float from_out = extract(src_words[from_idx[v]], delay, src_type);
            float old = weights[w_idx[v]];
            weights[w_idx[v]] = old + (rate * from_out * (to_out - (from_out * old)));
        }
    }
}

/* Convolutional learning per kernel weight
 * (CALC_{CONVERGENT,DIVERGENT}_CONVOLUTIONAL_BY_WEIGHT, synapse_kernel.h:610-796) */
void sg_upd_toward_post_conv(const sg_conn *c, const uint32_t *src_words, int src_type,
                             int delay, const uint32_t *dest_words, float rate,
                             float *weights) {
    for (int kr = 0; kr < c->row_field; ++kr)
        for (int kc = 0; kc < c->col_field; ++kc) {
            int k = kr * c->col_field + kc;
            float old = weights[k];
            float delta = 0.0;
            for (int tr = 0; tr < c->to_rows; ++tr)
                for (int tc = 0; tc < c->to_cols; ++tc) {
                    int fr, fc;
                    if (c->type == DIVERGENT) {   /* synapse_kernel.h:710-746 */
                        fr = (tr + c->row_spacing * (-c->row_offset - c->row_field + c->row_stride))
                                 / c->row_stride + kr * c->row_spacing;
                        fc = (tc + c->col_spacing * (-c->col_offset - c->col_field + c->col_stride))
                                 / c->col_stride + kc * c->col_spacing;
                    } else {
                        fr = tr * c->row_stride + (c->row_spacing * c->row_offset) + kr * c->row_spacing;
                        fc = tc * c->col_stride + (c->col_spacing * c->col_offset) + kc * c->col_spacing;
                    }
                    if (c->wrap) {
                        fr = wrap_index(fr, c->from_rows);
                        fc = wrap_index(fc, c->from_cols);
                    } else if (fr < 0 || fr >= c->from_rows || fc < 0 || fc >= c->from_cols) {
                        continue;
                    }
                    float from_out = extract(src_words[fr * c->from_cols + fc], delay, src_type);
                    float to_out = extract(dest_words[tr * c->to_cols + tc], 0, src_type);
                    delta += from_out * (to_out - (from_out * old));
                }
            weights[k] = old + (rate * delta / c->num_weights);
        }
}

void sg_rate(int size, int history, const float *inputs, float *outputs) {
    for (int nid = 0; nid < size; ++nid) {
        float input = inputs[nid];
        shift_float(outputs, size, history, nid, (input > 0.0) ? tanhf(input) : 0.0f);
    }
}

/* Game of life: game_of_life_attributes.cpp:58-77 (prev_live = bit 0, F3) */
void sg_gol(int size, int history, const float *inputs, uint32_t *lives,
            int smin, int smax, int bmin, int bmax) {
    for (int nid = 0; nid < size; ++nid) {
        int input = (int)inputs[nid];
        int prev_live = lives[nid] & 1;
        int live = prev_live ? (input >= smin && input <= smax)
                             : (input >= bmin && input <= bmax);
        shift_bit(lives, size, history, nid, (uint32_t)live);
    }
}

/* Default Izhikevich delays: distances from (pre-wrap) indices
 * (weight_matrix.cpp:1199-1217) then delay = base + dist / velocity capped at
 * 31 (weight_matrix.cpp:1321-1335).  Returns -1 if a delay exceeds 31 without
 * cap (the reference asserts). */
int sg_distance_delays(long n, const int *from_r, const int *from_c, const int *to_r,
                       const int *to_c, float from_spacing, float to_spacing,
                       float x_offset, float y_offset, float velocity, int cap,
                       int base_delay, float *distances, int *delays) {
    for (long i = 0; i < n; ++i) {
        float f_y = from_r[i] * from_spacing;
        float f_x = from_c[i] * from_spacing;
        float t_y = to_r[i] * to_spacing + y_offset;
        float t_x = to_c[i] * to_spacing + x_offset;
        distances[i] = pow(pow(t_x - f_x, 2) + pow(t_y - f_y, 2), 0.5);
        int delay = base_delay + (distances[i] / velocity);
        if (delay > 31 && !cap) return -1;
        delays[i] = (int)fmin(31, delay);
    }
    return 0;
}
