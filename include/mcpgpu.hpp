// C++ host mirror of MCPNet's helper-level compute calls on top of the mcpgpu
// C ABI (mcpgpu.h).  Header-only; link against libmcpgpu.so.
//
// The function names, argument meaning and output shapes follow the
// reference's helpers in apps/pipeline/mcpnet_helper.hpp so that a call site
// switches by changing the namespace:
//
//   compute_mi(input, bins, dmi)          mcpnet_helper.hpp:56-99   (B-spline MI)
//   compute_maxmin1/2/3(g2g, dmaxmin)     mcpnet_helper.hpp:189-196, 248-268, 336-355
//   compute_ratio(mi, dmaxmin, dmcp)      mcpnet_helper.hpp:172-184
//   compute_mcp2/3/4(g2g, dmcp)           mcpnet_helper.hpp:199-206, 271-278, 358-365
//   dpi_filter(input, tol, out)           apps/filter/dpi.cpp:236-287
//   set_diagonal(m, value)                apps/pipeline/mcpnet.cpp:299-308
//   compute_ap_mi(input, dmi, add_noise)  mcpnet_helper.hpp:101-164   (adaptive-partitioning MI)
//   compute_maxmins(g2g, m1, m2, m3)      mcpnet_helper.hpp:437-460
//   compute_combo(mi, m1, m2, m3, c, out) mcpnet_helper.hpp:507-573
//   compute_aupr_auroc(truth, values)     mcpnet_helper.hpp:1050-1071 (AUPR returned, AUROC too)
//   select_combo(...)                     the coefficient loop of apps/pipeline/mcpnet.cpp:575-616
//   compute_stouffer(in, out)             mcpnet_helper.hpp:575-586 (row statistics: see mcpgpu.h)
//   select_combo_stouffer(...)            the Stouffer half of that loop, mcpnet.cpp:622-661
//
// Matrices are float, row-major with a leading dimension (the layout of
// splash::ds::aligned_matrix<float> with its padded column_bytes()).  Errors
// throw mcpgpu::Error carrying the library status and message; there is no
// CPU fallback.
#pragma once

#include <cstdint>
#include <initializer_list>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "mcpgpu.h"

namespace mcpgpu {

class Error : public std::runtime_error {
  public:
    Error(int status, const std::string& msg) : std::runtime_error(msg), status_(status) {}
    int status() const { return status_; }

  private:
    int status_;
};

// Owning host matrix (row-major, leading dimension >= columns).
template <typename T>
class Matrix {
  public:
    Matrix() = default;
    Matrix(int64_t rows, int64_t cols, int64_t ld = -1)
        : rows_(rows), cols_(cols), ld_(ld < 0 ? cols : ld), data_((size_t)(rows * (ld < 0 ? cols : ld))) {}
    int64_t rows() const { return rows_; }
    int64_t columns() const { return cols_; }
    int64_t ld() const { return ld_; }
    T* data(int64_t r = 0) { return data_.data() + r * ld_; }
    const T* data(int64_t r = 0) const { return data_.data() + r * ld_; }
    T& at(int64_t r, int64_t c) { return data_[(size_t)(r * ld_ + c)]; }
    const T& at(int64_t r, int64_t c) const { return data_[(size_t)(r * ld_ + c)]; }
    void resize(int64_t rows, int64_t cols) {
        rows_ = rows;
        cols_ = cols;
        ld_ = cols;
        data_.assign((size_t)(rows * cols), T());
    }

  private:
    int64_t rows_ = 0, cols_ = 0, ld_ = 0;
    std::vector<T> data_;
};

// One device, one CUDA stream; not thread-safe (as the C handle).
class Context {
  public:
    explicit Context(int device = 0) {
        int rc = mcpg_create(&h_, device);
        if (rc) throw Error(rc, std::string("mcpg_create failed: ") + mcpg_status_string(rc));
    }
    ~Context() { mcpg_destroy(h_); }
    Context(const Context&) = delete;
    Context& operator=(const Context&) = delete;
    mcpg_handle* handle() const { return h_; }
    void check(int rc, const char* what) const {
        if (rc) throw Error(rc, std::string(what) + ": " + mcpg_last_error(h_));
    }

  private:
    mcpg_handle* h_ = nullptr;
};

enum class MIPrecision : int {
    FP32 = MCPG_MI_FP32,
    BF16 = MCPG_MI_BF16,
    BF16X3 = MCPG_MI_BF16X3,
    FP16 = MCPG_MI_FP16,
    FP16X3 = MCPG_MI_FP16X3,
    BF16F8 = MCPG_MI_BF16F8,
};

// compute_mi: scale -> B-spline weights (order 3, as the reference hard-codes)
// -> all-pairs MI in bits.  dmi is resized to n x n.
inline void compute_mi(Context& ctx, const Matrix<float>& input, int bins, Matrix<float>& dmi,
                       MIPrecision prec = MIPrecision::BF16X3, int order = 3, std::vector<double>* H = nullptr) {
    const int64_t n = input.rows(), m = input.columns();
    dmi.resize(n, n);
    if (H) H->assign((size_t)n, 0.0);
    ctx.check(mcpg_bspline_mi(ctx.handle(), input.data(), n, m, input.ld(), bins, order, (int)prec, dmi.data(),
                              dmi.ld(), H ? H->data() : nullptr),
              "compute_mi");
}

inline void set_diagonal(Matrix<float>& mi, float value) {
    if (value < 0.0f) return;
    const int64_t mc = mi.rows() < mi.columns() ? mi.rows() : mi.columns();
    for (int64_t i = 0; i < mc; ++i) mi.at(i, i) = value;
}

// InnerProduct(a, b) with mcp2_maxmin_kernel: out[i][j] = max_k min(a[i][k], b[j][k]).
inline void maxmin(Context& ctx, const Matrix<float>& a, const Matrix<float>& b, Matrix<float>& out) {
    if (a.columns() != b.columns()) throw Error(MCPG_ERR_ARG, "maxmin: operand column counts differ");
    out.resize(a.rows(), b.rows());
    ctx.check(mcpg_maxmin(ctx.handle(), a.data(), a.ld(), b.data(), b.ld(), a.rows(), b.rows(), a.columns(),
                          out.data(), out.ld()),
              "maxmin");
}

inline void compute_maxmin1(Context& ctx, const Matrix<float>& g2g, Matrix<float>& dmaxmin) {
    maxmin(ctx, g2g, g2g, dmaxmin);
}
inline void compute_maxmin2(Context& ctx, const Matrix<float>& g2g, Matrix<float>& dmaxmin) {
    dmaxmin.resize(g2g.rows(), g2g.columns());
    ctx.check(mcpg_mcp(ctx.handle(), g2g.data(), g2g.rows(), g2g.ld(), 3, 0, dmaxmin.data(), dmaxmin.ld(), nullptr, 0),
              "compute_maxmin2");
}
inline void compute_maxmin3(Context& ctx, const Matrix<float>& g2g, Matrix<float>& dmaxmin) {
    dmaxmin.resize(g2g.rows(), g2g.columns());
    ctx.check(mcpg_mcp(ctx.handle(), g2g.data(), g2g.rows(), g2g.ld(), 4, 0, dmaxmin.data(), dmaxmin.ld(), nullptr, 0),
              "compute_maxmin3");
}

inline void compute_ratio(Context& ctx, const Matrix<float>& mi, const Matrix<float>& dmaxmin, Matrix<float>& dmcp) {
    dmcp.resize(dmaxmin.rows(), dmaxmin.columns());
    ctx.check(mcpg_ratio(ctx.handle(), mi.data(), mi.ld(), dmaxmin.data(), dmaxmin.ld(), dmaxmin.rows(),
                         dmaxmin.columns(), dmcp.data(), dmcp.ld()),
              "compute_ratio");
}

// compute_mcp{2,3,4}: ratio(mi, maxmin of path length L); the max-min matrix
// is returned through `maxmin_out` when given.  symmetrize reproduces the mcp
// app's max(M, M^T) step for MCP3.
inline void compute_mcp(Context& ctx, const Matrix<float>& g2g, int path_len, Matrix<float>& dmcp,
                        Matrix<float>* maxmin_out = nullptr, bool symmetrize = false) {
    const int64_t n = g2g.rows();
    dmcp.resize(n, n);
    if (maxmin_out) maxmin_out->resize(n, n);
    ctx.check(mcpg_mcp(ctx.handle(), g2g.data(), n, g2g.ld(), path_len, symmetrize ? 1 : 0,
                       maxmin_out ? maxmin_out->data() : nullptr, maxmin_out ? maxmin_out->ld() : n, dmcp.data(),
                       dmcp.ld()),
              "compute_mcp");
}
inline void compute_mcp2(Context& ctx, const Matrix<float>& g2g, Matrix<float>& dmcp) { compute_mcp(ctx, g2g, 2, dmcp); }
inline void compute_mcp3(Context& ctx, const Matrix<float>& g2g, Matrix<float>& dmcp) { compute_mcp(ctx, g2g, 3, dmcp); }
inline void compute_mcp4(Context& ctx, const Matrix<float>& g2g, Matrix<float>& dmcp) { compute_mcp(ctx, g2g, 4, dmcp); }

// The dpi app's filter: returns the reference's "Mask removing N elements" count.
inline int64_t dpi_filter(Context& ctx, const Matrix<float>& input, float tolerance, Matrix<float>& output,
                          std::vector<uint8_t>* mask = nullptr) {
    const int64_t n = input.rows();
    output.resize(n, n);
    if (mask) mask->assign((size_t)(n * n), 0);
    int64_t removed = 0;
    ctx.check(mcpg_dpi(ctx.handle(), input.data(), n, input.ld(), tolerance, output.data(), output.ld(),
                       mask ? mask->data() : nullptr, &removed),
              "dpi_filter");
    return removed;
}

// Maximum-capacity closure by repeated squaring; returns the number of products.
inline int max_capacity_closure(Context& ctx, const Matrix<float>& a, Matrix<float>& out, int max_iter = 64) {
    const int64_t n = a.rows();
    out.resize(n, n);
    int it = 0;
    ctx.check(mcpg_closure(ctx.handle(), a.data(), n, a.ld(), max_iter, out.data(), out.ld(), &it),
              "max_capacity_closure");
    return it;
}

// compute_ap_mi: optional U[0, 1e-5) noise (the reference adds it: add_noise = true),
// descending ranks, adaptive-partitioning MI in bits.  dmi is resized to n x n.
inline void compute_ap_mi(Context& ctx, const Matrix<float>& input, Matrix<float>& dmi, bool add_noise = false,
                          uint64_t seed = 1) {
    const int64_t n = input.rows(), m = input.columns();
    dmi.resize(n, n);
    ctx.check(mcpg_ap_mi(ctx.handle(), input.data(), n, m, input.ld(), add_noise ? 1e-5f : 0.0f, seed, dmi.data(),
                         dmi.ld()),
              "compute_ap_mi");
}

// compute_maxmins: M1 = A (x) A, M2 = A (x) M1, M3 = M1 (x) M1.
inline void compute_maxmins(Context& ctx, const Matrix<float>& g2g, Matrix<float>& m1, Matrix<float>& m2,
                            Matrix<float>& m3) {
    const int64_t n = g2g.rows();
    m1.resize(n, n);
    m2.resize(n, n);
    m3.resize(n, n);
    ctx.check(mcpg_maxmins(ctx.handle(), g2g.data(), n, g2g.ld(), m1.data(), m1.ld(), m2.data(), m2.ld(), m3.data(),
                           m3.ld(), nullptr, 0, nullptr, 0, nullptr, 0),
              "compute_maxmins");
}

// compute_combo: out = mi / (c0 mi + c1 m1 + c2 m2 + c3 m3) (coefficients as doubles).
inline void compute_combo(Context& ctx, const Matrix<float>& mi, const Matrix<float>& m1, const Matrix<float>& m2,
                          const Matrix<float>& m3, const double coeffs[4], Matrix<float>& out) {
    out.resize(mi.rows(), mi.columns());
    ctx.check(mcpg_combo(ctx.handle(), mi.data(), mi.ld(), m1.data(), m1.ld(), m2.data(), m2.ld(), m3.data(), m3.ld(),
                         mi.rows(), mi.columns(), coeffs, out.data(), out.ld()),
              "compute_combo");
}

// Truth labels for evaluation: 1 = positive, 0 = negative, anything else unknown.
enum class TruthRegion : int { LowerTriangle = MCPG_TRUTH_LOWER, All = MCPG_TRUTH_ALL, TFRows = MCPG_TRUTH_TF };

struct Curves {
    double aupr = 0.0, auroc = 0.0;
    int64_t n_pos = 0, n_neg = 0;
};

// compute_aupr_auroc over the labelled entries of `values` (same shape as labels).
inline Curves compute_aupr_auroc(Context& ctx, const Matrix<int8_t>& labels, const Matrix<float>& values,
                                 TruthRegion region = TruthRegion::LowerTriangle,
                                 const std::vector<int32_t>* row_gene = nullptr,
                                 const std::vector<uint8_t>* col_tf = nullptr) {
    if (labels.rows() != values.rows() || labels.columns() != values.columns())
        throw Error(MCPG_ERR_ARG, "compute_aupr_auroc: labels and values differ in shape");
    Curves c;
    ctx.check(mcpg_eval_truth(ctx.handle(), values.data(), values.rows(), values.columns(), values.ld(), labels.data(),
                              labels.ld(), (int)region, row_gene ? row_gene->data() : nullptr,
                              col_tf ? col_tf->data() : nullptr, &c.aupr, &c.auroc, &c.n_pos, &c.n_neg),
              "compute_aupr_auroc");
    return c;
}

// The ensemble coefficient search: AUPR / AUROC of every coefficient row
// (n x 4, row-major) and the reference's choice of row.
inline int64_t select_combo(Context& ctx, const Matrix<float>& mi, const Matrix<float>& m1, const Matrix<float>& m2,
                            const Matrix<float>& m3, const Matrix<int8_t>& labels, const std::vector<double>& coeffs,
                            std::vector<double>* aupr = nullptr, std::vector<double>* auroc = nullptr,
                            TruthRegion region = TruthRegion::LowerTriangle,
                            const std::vector<int32_t>* row_gene = nullptr,
                            const std::vector<uint8_t>* col_tf = nullptr) {
    const int64_t nc = (int64_t)(coeffs.size() / 4);
    std::vector<double> a((size_t)nc), b((size_t)nc);
    int64_t best = 0;
    ctx.check(mcpg_combo_eval(ctx.handle(), mi.data(), mi.ld(), m1.data(), m1.ld(), m2.data(), m2.ld(), m3.data(),
                              m3.ld(), mi.rows(), mi.columns(), labels.data(), labels.ld(), (int)region,
                              row_gene ? row_gene->data() : nullptr, col_tf ? col_tf->data() : nullptr, coeffs.data(),
                              nc, a.data(), b.data(), &best),
              "select_combo");
    if (aupr) *aupr = a;
    if (auroc) *auroc = b;
    return best;
}

// compute_stouffer (or CLR with clr = true): row statistics then the per-entry transform.
inline void compute_stouffer(Context& ctx, const Matrix<float>& in, Matrix<float>& out, bool clr = false,
                             int stats_mode = MCPG_ROWSTATS_EXCLUDE_DIAGONAL) {
    const int64_t n = in.rows();
    out.resize(n, n);
    ctx.check(mcpg_transform(ctx.handle(), in.data(), n, in.ld(), clr ? MCPG_TRANSFORM_CLR : MCPG_TRANSFORM_STOUFFER,
                             stats_mode, out.data(), out.ld()),
              "compute_stouffer");
}

// The Stouffer half of the coefficient search: per row the AUPR / AUROC of the
// Stouffer-transformed combo matrix, and the reference's choice of row.
inline int64_t select_combo_stouffer(Context& ctx, const Matrix<float>& mi, const Matrix<float>& m1,
                                     const Matrix<float>& m2, const Matrix<float>& m3, const Matrix<int8_t>& labels,
                                     const std::vector<double>& coeffs, std::vector<double>* aupr = nullptr,
                                     std::vector<double>* auroc = nullptr,
                                     TruthRegion region = TruthRegion::LowerTriangle,
                                     int stats_mode = MCPG_ROWSTATS_EXCLUDE_DIAGONAL) {
    const int64_t nc = (int64_t)(coeffs.size() / 4);
    std::vector<double> a((size_t)nc), b((size_t)nc);
    int64_t best = 0;
    ctx.check(mcpg_combo_stouffer_eval(ctx.handle(), mi.data(), mi.ld(), m1.data(), m1.ld(), m2.data(), m2.ld(),
                                       m3.data(), m3.ld(), mi.rows(), labels.data(), labels.ld(), (int)region,
                                       nullptr, nullptr, coeffs.data(), nc, stats_mode, a.data(), b.data(), &best),
              "select_combo_stouffer");
    if (aupr) *aupr = a;
    if (auroc) *auroc = b;
    return best;
}

// ---- semi-supervised split evaluation (the eval_mcpnet app) ----
// The app's training sizes (size_t)(f * entries), f = 0.005 .. 0.1 (to 0.5 with TFs).
inline std::vector<int64_t> train_counts(int64_t entries, bool tf) {
    std::vector<double> fr = {0.005, 0.01, 0.02, 0.05, 0.1};
    if (tf) fr.insert(fr.end(), {0.2, 0.3, 0.4, 0.5});
    std::vector<int64_t> out;
    for (double f : fr) out.push_back((int64_t)(size_t)(f * (double)entries));
    return out;
}

// shuffle_truth (apps/pipeline/eval_mcpnet.cpp:214-224): iteration `seed`'s shuffled order of
// `entries` labelled entries as mask positions (host only; seed 0 keeps the order).
inline std::vector<uint32_t> shuffle_positions(int64_t entries, uint64_t seed) {
    std::vector<uint32_t> out((size_t)(entries > 0 ? entries : 0));
    const int rc = mcpg_shuffle_positions(out.data(), entries, seed);
    if (rc != MCPG_OK) throw Error(rc, "shuffle_positions: bad entry count");
    return out;
}

struct SplitAupr {
    double full = 0.0;
    std::vector<double> train, test;  // iterations x parts, row-major
};

// eval_aupr_mcp: the AUPR of all labelled entries and of the shuffled train / test splits.
inline SplitAupr split_aupr(Context& ctx, const Matrix<int8_t>& labels, const Matrix<float>& values, int64_t iterations,
                            const std::vector<int64_t>& counts, TruthRegion region,
                            const std::vector<int32_t>* row_gene = nullptr,
                            const std::vector<uint8_t>* col_tf = nullptr) {
    SplitAupr r;
    const int64_t parts = (int64_t)counts.size();
    r.train.assign((size_t)(iterations * parts), 0.0);
    r.test.assign((size_t)(iterations * parts), 0.0);
    ctx.check(mcpg_split_aupr(ctx.handle(), values.data(), values.rows(), values.columns(), values.ld(), labels.data(),
                              labels.ld(), (int)region, row_gene ? row_gene->data() : nullptr,
                              col_tf ? col_tf->data() : nullptr, iterations, counts.data(), parts, &r.full,
                              r.train.data(), r.test.data()),
              "split_aupr");
    return r;
}

// eval_combos over the splits: results iterations x parts x 6 (train, test, Stouffer train,
// Stouffer test, full, Stouffer full); stouffer: MCPG_STOUFFER_NONE, a MCPG_ROWSTATS_* mode or
// MCPG_STOUFFER_TF.
inline std::vector<double> split_combo_eval(Context& ctx, const Matrix<float>& mi, const Matrix<float>& m1,
                                            const Matrix<float>& m2, const Matrix<float>& m3,
                                            const Matrix<int8_t>& labels, const std::vector<double>& coeffs,
                                            int stouffer, int64_t iterations, const std::vector<int64_t>& counts,
                                            TruthRegion region, const std::vector<int32_t>* row_gene = nullptr,
                                            const std::vector<uint8_t>* col_tf = nullptr,
                                            std::vector<int64_t>* best = nullptr) {
    const int64_t parts = (int64_t)counts.size();
    std::vector<double> res((size_t)(iterations * parts * 6), 0.0);
    std::vector<int64_t> b((size_t)(iterations * parts * 2), 0);
    ctx.check(mcpg_split_combo_eval(ctx.handle(), mi.data(), mi.ld(), m1.data(), m1.ld(), m2.data(), m2.ld(),
                                    m3.data(), m3.ld(), mi.rows(), mi.columns(), labels.data(), labels.ld(),
                                    (int)region, row_gene ? row_gene->data() : nullptr,
                                    col_tf ? col_tf->data() : nullptr, coeffs.data(), (int64_t)(coeffs.size() / 4),
                                    stouffer, iterations, counts.data(), parts, res.data(), b.data()),
              "split_combo_eval");
    if (best) *best = b;
    return res;
}

// ---- TF-restricted forms (--tf-input) ----
// tfs: one value per gene, +inf for a transcription factor, -inf otherwise
// (load_tfs, mcpnet_helper.hpp:1074-1123).  Outputs have one row per TF, in
// gene order.

// compute_mcp{2,3,4}_tfs (path_len 2..4, tf_gene_transition 0..path_len-1).
inline void compute_mcp_tfs(Context& ctx, const Matrix<float>& g2g, const std::vector<float>& tfs, int path_len,
                            int tf_gene_transition, Matrix<float>& dmcp, Matrix<float>* maxmin_out = nullptr) {
    const int64_t n = g2g.rows();
    int64_t t = 0;
    for (float v : tfs) t += v > 0.0f;
    dmcp.resize(t, n);
    if (maxmin_out) maxmin_out->resize(t, n);
    ctx.check(mcpg_mcp_tf(ctx.handle(), g2g.data(), n, g2g.ld(), tfs.data(), path_len, tf_gene_transition,
                          maxmin_out ? maxmin_out->data() : nullptr, maxmin_out ? maxmin_out->ld() : n, dmcp.data(),
                          dmcp.ld()),
              "compute_mcp_tfs");
}

// dpi_tf_kernel + mask over the n x n matrix; returns the removed count.
inline int64_t dpi_filter_tfs(Context& ctx, const Matrix<float>& input, float tolerance, const std::vector<float>& tfs,
                              Matrix<float>& output) {
    const int64_t n = input.rows();
    output.resize(n, n);
    int64_t removed = 0;
    ctx.check(mcpg_dpi_tf(ctx.handle(), input.data(), n, input.ld(), tolerance, tfs.data(), output.data(),
                          output.ld(), nullptr, &removed),
              "dpi_filter_tfs");
    return removed;
}

// compute_maxmins_tfs; tf_rows (the mi operand of the TF ensemble) gets the TF rows of g2g.
inline void compute_maxmins_tfs(Context& ctx, const Matrix<float>& g2g, const std::vector<float>& tfs,
                                Matrix<float>& tf_rows, Matrix<float>& m1, Matrix<float>& m2, Matrix<float>& m3) {
    const int64_t n = g2g.rows();
    int64_t t = 0;
    for (float v : tfs) t += v > 0.0f;
    for (Matrix<float>* m : {&tf_rows, &m1, &m2, &m3}) m->resize(t, n);
    ctx.check(mcpg_maxmins_tf(ctx.handle(), g2g.data(), n, g2g.ld(), tfs.data(), tf_rows.data(), tf_rows.ld(),
                              m1.data(), m1.ld(), m2.data(), m2.ld(), m3.data(), m3.ld()),
              "compute_maxmins_tfs");
}

// compute_stouffer_tf of a TFs x genes matrix (clr = true: the transform app's
// zscored_clr_kernel instead).
inline void compute_stouffer_tf(Context& ctx, const Matrix<float>& in, Matrix<float>& out, bool clr = false) {
    out.resize(in.rows(), in.columns());
    ctx.check(mcpg_transform_tf(ctx.handle(), in.data(), in.rows(), in.columns(), in.ld(),
                                clr ? MCPG_TRANSFORM_CLR : MCPG_TRANSFORM_STOUFFER, out.data(), out.ld()),
              "compute_stouffer_tf");
}

// The Stouffer half of the TF coefficient search.
inline int64_t select_combo_stouffer_tf(Context& ctx, const Matrix<float>& mi, const Matrix<float>& m1,
                                        const Matrix<float>& m2, const Matrix<float>& m3, const Matrix<int8_t>& labels,
                                        const std::vector<double>& coeffs, std::vector<double>* aupr,
                                        std::vector<double>* auroc, TruthRegion region,
                                        const std::vector<int32_t>* row_gene = nullptr,
                                        const std::vector<uint8_t>* col_tf = nullptr) {
    const int64_t nc = (int64_t)(coeffs.size() / 4);
    std::vector<double> a((size_t)nc), b((size_t)nc);
    int64_t best = 0;
    ctx.check(mcpg_combo_stouffer_tf_eval(ctx.handle(), mi.data(), mi.ld(), m1.data(), m1.ld(), m2.data(), m2.ld(),
                                          m3.data(), m3.ld(), mi.rows(), mi.columns(), labels.data(), labels.ld(),
                                          (int)region, row_gene ? row_gene->data() : nullptr,
                                          col_tf ? col_tf->data() : nullptr, coeffs.data(), nc, a.data(), b.data(),
                                          &best),
              "select_combo_stouffer_tf");
    if (aupr) *aupr = a;
    if (auroc) *auroc = b;
    return best;
}

}  // namespace mcpgpu
