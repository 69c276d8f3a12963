// Host-side serial enumeration of a connection's synapse visits (host layout
// weight indices), in the reference's loop order:
//   src/core/engine/kernel/synapse_kernel.h:115-149 (FC), :182-228 (subset),
//   :257-286 (one to one), :384-461 (convergent), :506-581 (divergent),
//   :303-366 (sparse: each destination's compacted synapses).
#pragma once

namespace sg {

template <class F>
void enumerate_visits(const Connection& c, F&& f) {
    const Layer& fl = *c.from;
    const Layer& tl = *c.to;
    auto wrap = [](int x, int n) { return (x % n + n) % n; };
    switch (c.type) {
        case FULLY_CONNECTED: {
            for (int to = 0; to < tl.size; ++to) {
                long wi = (long)to * fl.size;
                for (int from = 0; from < fl.size; ++from, ++wi)
                    f(to, to, from, wi, from / fl.cols, from % fl.cols);
            }
            break;
        }
        case SUBSET: {
            const auto& s = c.subset;
            int kcols = s.tc1 - s.tc0, krows = s.tr1 - s.tr0, fks = s.from_size();
            int row = 0;
            for (int i = 0; i < krows; ++i)
                for (int j = 0; j < kcols; ++j, ++row) {
                    int to = (i + s.tr0) * tl.cols + (j + s.tc0);
                    int tk = i * kcols + j;
                    int fk = 0;
                    for (int fr = s.fr0; fr < s.fr1; ++fr)
                        for (int fc = s.fc0; fc < s.fc1; ++fc, ++fk)
                            f(row, to, fr * fl.cols + fc, (long)tk * fks + fk, fr, fc);
                }
            break;
        }
        case ONE_TO_ONE:
            for (int i = 0; i < fl.size; ++i) f(i, i, i, (long)i, i / fl.cols, i % fl.cols);
            break;
        case CONVERGENT: {
            const auto& a = c.arbor;
            int K = a.kernel();
            for (int tr = 0; tr < tl.rows; ++tr)
                for (int tc = 0; tc < tl.cols; ++tc) {
                    int to = tr * tl.cols + tc;
                    long woff = c.convolutional ? 0 : (long)to * K;
                    int s_row = tr * a.row_stride + a.row_spacing * a.row_offset;
                    int s_col = tc * a.col_stride + a.col_spacing * a.col_offset;
                    int k = 0;
                    for (int kr = 0; kr < a.row_field; ++kr)
                        for (int kc = 0; kc < a.col_field; ++kc, ++k) {
                            int fr = s_row + kr * a.row_spacing, fc = s_col + kc * a.col_spacing;
                            int pr = fr, pc = fc;
                            if (a.wrap) { fr = wrap(fr, fl.rows); fc = wrap(fc, fl.cols); }
                            else if (fr < 0 || fr >= fl.rows || fc < 0 || fc >= fl.cols) continue;
                            f(to, to, fr * fl.cols + fc, woff + k, pr, pc);
                        }
                }
            break;
        }
        case DIVERGENT: {
            const auto& a = c.arbor;
            long per = c.num_weights / tl.size;
            for (int tr = 0; tr < tl.rows; ++tr)
                for (int tc = 0; tc < tl.cols; ++tc) {
                    int to = tr * tl.cols + tc;
                    long woff = c.convolutional ? 0 : (long)to * per;
                    int sr0 = (tr + a.row_spacing * (-a.row_offset - a.row_field + a.row_stride)) / a.row_stride;
                    int sc0 = (tc + a.col_spacing * (-a.col_offset - a.col_field + a.col_stride)) / a.col_stride;
                    int sr1 = sr0 + (a.row_spacing * (a.row_field - a.row_stride) / a.row_stride);
                    int sc1 = sc0 + (a.col_spacing * (a.col_field - a.col_stride) / a.col_stride);
                    int k = 0;
                    for (int sr = sr0; sr <= sr1; sr += a.row_spacing)
                        for (int sc = sc0; sc <= sc1; sc += a.col_spacing, ++k) {
                            int fr = sr, fc = sc;
                            if (a.wrap) { fr = wrap(fr, fl.rows); fc = wrap(fc, fl.cols); }
                            else if (fr < 0 || fr >= fl.rows || fc < 0 || fc >= fl.cols) continue;
                            f(to, to, fr * fl.cols + fc, woff + k, sr, sc);
                        }
                }
            break;
        }
        case SPARSE: {
            const SparseTable& t = *c.sparse_table;
            for (int to = 0; to < tl.size; ++to) {
                long wi = (long)to * t.kmax;
                for (int i = 0; i < t.nonzero[to]; ++i, ++wi)
                    f(to, to, t.from[wi], wi, t.from_row[wi], t.from_col[wi]);
            }
            break;
        }
    }
}

}  // namespace sg
