// C ABI: the ensemble combination (compute_combo, mcpnet_helper.hpp:507-573),
// Stouffer / CLR transforms, the AUPR / AUROC evaluator (compute_aupr_auroc,
// mcpnet_helper.hpp:1050-1071), the coefficient searches of apps/pipeline/mcpnet.cpp
// and the semi-supervised split evaluation of apps/pipeline/eval_mcpnet.cpp.
#include "api_internal.h"

namespace {

using namespace mcpg_api;

// ---- gold-standard evaluation (AUPR / AUROC) ----
struct EvalWs {
    int* flag;         // NaN seen
    unsigned* ticket;  // curve reduction
    double* out;       // curve sums [2]
    double* part;      // curve partials
};

int ev_ws(mcpg_handle* h, EvalWs& w) {
    void* p;
    int rc = scratch(h, S_EV_RED, 64 + (size_t)mcpg::curve_part_elems() * sizeof(double), &p);
    if (rc) return rc;
    char* b = (char*)p;
    w.flag = (int*)b;
    w.ticket = (unsigned*)(b + 8);
    w.out = (double*)(b + 16);
    w.part = (double*)(b + 64);
    CK(h, cudaMemsetAsync(w.flag, 0, sizeof(int), h->stream), "memset");
    return MCPG_OK;
}

int ev_nan_check(mcpg_handle* h, const EvalWs& w) {
    int f = 0;
    CK(h, cudaMemcpyAsync(&f, w.flag, sizeof(int), cudaMemcpyDeviceToHost, h->stream), "device-to-host copy");
    CK(h, cudaStreamSynchronize(h->stream), "stream synchronize");
    if (f) return fail(h, MCPG_ERR_ARG, "evaluation: NaN score among the labelled entries");
    return MCPG_OK;
}

int ev_sort(mcpg_handle* h, uint32_t* keys, int64_t n) {
    if (n <= 1) return MCPG_OK;
    const int64_t nb = mcpg::radix_blocks(n);
    void *alt, *bh, *bo, *tmp;
    int rc;
    if ((rc = scratch(h, S_EV_ALT, (size_t)n * 4, &alt))) return rc;
    if ((rc = scratch(h, S_EV_BH, (size_t)(256 * nb) * 4, &bh))) return rc;
    if ((rc = scratch(h, S_EV_BHOFF, (size_t)(256 * nb + 1) * 8, &bo))) return rc;
    if ((rc = scratch(h, S_EV_TMP, (size_t)mcpg::scan_tmp_elems(256 * nb) * 8, &tmp))) return rc;
    PROF(h, "radix_sort");
    CK(h, mcpg::launch_radix_sort(keys, (uint32_t*)alt, n, (uint32_t*)bh, (uint64_t*)bo, (uint64_t*)tmp, h->stream,
                                  &h->launches),
       "radix sort");
    return MCPG_OK;
}

// Places the Y scores (through `count(lt, eq, dir)`) into the sorted X and returns
// the two curve sums of launch_curve in res.
template <class Count>
int ev_curve(mcpg_handle* h, const uint32_t* X, int64_t nX, int64_t nY, const EvalWs& w, Count count, double res[2]) {
    if (nX >= ((int64_t)1 << 31)) return fail(h, MCPG_ERR_UNSUPPORTED, "evaluation: more than 2^31 - 1 sorted scores");
    void *hist, *tmp;
    int rc;
    if ((rc = scratch(h, S_EV_HIST, (size_t)(4 * nX + 3) * 8 + (size_t)mcpg::rank_dir_elems() * 4, &hist))) return rc;
    if ((rc = scratch(h, S_EV_TMP, (size_t)mcpg::scan_tmp_elems(nX) * 8, &tmp))) return rc;
    uint64_t* lt = (uint64_t*)hist;
    uint64_t* eq = lt + nX + 1;
    uint64_t* work = eq + nX + 1;
    uint32_t* dir = (uint32_t*)(work + 2 * nX + 1);
    {
        PROF(h, "rank_count");
        CK(h, count(lt, eq, dir), "rank count");
    }
    {
        PROF(h, "curve");
        CK(h, mcpg::launch_curve(X, nX, nY, lt, eq, work, (uint64_t*)tmp, w.part, w.ticket, w.out, h->stream,
                                 &h->launches),
           "curve");
    }
    CK(h, cudaMemcpyAsync(res, w.out, 2 * sizeof(double), cudaMemcpyDeviceToHost, h->stream), "device-to-host copy");
    CK(h, cudaStreamSynchronize(h->stream), "stream synchronize");
    return MCPG_OK;
}

// AUPR / AUROC from P positive keys kp (any order; sorted here in place), N
// negatives ranked by neg_rank(X, nX, lt, eq, dir), and -- only for the AUROC
// branch n_pos >= n_neg > 0 -- compact negative keys from neg_keys(&kn).
template <class NegRank, class NegKeys>
int ev_aupr_auroc(mcpg_handle* h, const EvalWs& w, uint32_t* kp, int64_t P, int64_t N, NegRank neg_rank,
                  NegKeys neg_keys, double* aupr, double* auroc) {
    double res[2] = {0.0, 0.0};
    int rc;
    if (P > 0) {
        if ((rc = ev_sort(h, kp, P))) return rc;
        if ((rc = ev_curve(h, kp, P, N, w,
                           [&](uint64_t* lt, uint64_t* eq, uint32_t* dir) {
                               return neg_rank((const uint32_t*)kp, P, lt, eq, dir);
                           },
                           res)))
            return rc;
    }
    const double pr = P == 0 ? 0.0 : res[0];
    double roc;
    if (P < N) {
        roc = P == 0 ? 1.0 : 1.0 - res[1];
    } else if (N == 0) {
        roc = 0.0;
    } else {
        uint32_t* kn = nullptr;
        if ((rc = neg_keys(&kn))) return rc;
        if ((rc = ev_sort(h, kn, N))) return rc;
        double r2[2];
        if ((rc = ev_curve(h, kn, N, P, w,
                           [&](uint64_t* lt, uint64_t* eq, uint32_t* dir) {
                               return mcpg::launch_rank_count_keys(kn, N, kp, P, lt, eq, dir, h->stream,
                                                                   &h->launches);
                           },
                           r2)))
            return rc;
        roc = r2[1];
    }
    if ((rc = ev_nan_check(h, w))) return rc;
    if (aupr) *aupr = pr;
    if (auroc) *auroc = roc;
    return MCPG_OK;
}

int aupr_auroc_dev(mcpg_handle* h, const float* pos, int64_t P, const float* neg, int64_t N, double* aupr,
                   double* auroc) {
    if (P < 0 || N < 0) return fail(h, MCPG_ERR_ARG, "aupr_auroc: negative count");
    if ((P > 0 && !pos) || (N > 0 && !neg)) return fail(h, MCPG_ERR_ARG, "aupr_auroc: null score vector");
    EvalWs w;
    int rc;
    if ((rc = ev_ws(h, w))) return rc;
    void *kp, *kn;
    if ((rc = scratch(h, S_EV_KP, (size_t)P * 4, &kp))) return rc;
    if ((rc = scratch(h, S_EV_KN, (size_t)N * 4, &kn))) return rc;
    {
        PROF(h, "keys");
        CK(h, mcpg::launch_keys_from_floats(pos, P, (uint32_t*)kp, w.flag, h->stream, &h->launches), "keys");
        if (P > 0) CK(h, mcpg::launch_keys_from_floats(neg, N, (uint32_t*)kn, w.flag, h->stream, &h->launches), "keys");
    }
    uint32_t* knk = (uint32_t*)kn;
    return ev_aupr_auroc(
        h, w, (uint32_t*)kp, P, N,
        [&](const uint32_t* X, int64_t nX, uint64_t* lt, uint64_t* eq, uint32_t* dir) {
            return mcpg::launch_rank_count_keys(X, nX, knk, N, lt, eq, dir, h->stream, &h->launches);
        },
        [&](uint32_t** out) {
            if (P == 0) {  // keys not made above
                PROF(h, "keys");
                CK(h, mcpg::launch_keys_from_floats(neg, N, knk, w.flag, h->stream, &h->launches), "keys");
            }
            *out = knk;
            return MCPG_OK;
        },
        aupr, auroc);
}

int truth_region(mcpg_handle* h, const char* who, const int8_t* labels, int64_t rows, int64_t cols, int64_t ldl,
                 int region, const int32_t* row_gene, const uint8_t* col_tf, mcpg::TruthRegion* r) {
    if (rows < 0 || cols < 0) return fail(h, MCPG_ERR_ARG, "%s: negative size", who);
    if (rows > 0 && cols > 0 && !labels) return fail(h, MCPG_ERR_ARG, "%s: null labels", who);
    if (ldl < cols) return fail(h, MCPG_ERR_ARG, "%s: label leading dimension too small", who);
    if (region != MCPG_TRUTH_LOWER && region != MCPG_TRUTH_ALL && region != MCPG_TRUTH_TF)
        return fail(h, MCPG_ERR_ARG, "%s: unknown truth region %d", who, region);
    if (region == MCPG_TRUTH_TF && rows > 0 && cols > 0 && (!row_gene || !col_tf))
        return fail(h, MCPG_ERR_ARG, "%s: MCPG_TRUTH_TF needs row_gene and col_tf", who);
    r->labels = labels;
    r->ldl = ldl;
    r->rows = rows;
    r->cols = cols;
    r->mode = region;
    r->row_gene = row_gene;
    r->col_tf = col_tf;
    return MCPG_OK;
}

// Per-item counts and their scans; P / N on the host.
int truth_offsets(mcpg_handle* h, const mcpg::TruthRegion& r, uint64_t** offp, uint64_t** offn, int64_t* P,
                  int64_t* N) {
    const int64_t items = mcpg::truth_items(r);
    void *cnt, *off, *tmp;
    int rc;
    if ((rc = scratch(h, S_EV_CNT, (size_t)(2 * items) * 4, &cnt))) return rc;
    if ((rc = scratch(h, S_EV_OFF, (size_t)(2 * (items + 1)) * 8, &off))) return rc;
    if ((rc = scratch(h, S_EV_TMP, (size_t)mcpg::scan_tmp_elems(items) * 8, &tmp))) return rc;
    uint32_t* cp = (uint32_t*)cnt;
    uint32_t* cn = cp + items;
    *offp = (uint64_t*)off;
    *offn = *offp + items + 1;
    {
        PROF(h, "truth_count");
        CK(h, mcpg::launch_truth_count(r, cp, cn, h->stream, &h->launches), "truth count");
        CK(h, mcpg::launch_scan_u32(cp, items, *offp, (uint64_t*)tmp, h->stream, &h->launches), "scan");
        CK(h, mcpg::launch_scan_u32(cn, items, *offn, (uint64_t*)tmp, h->stream, &h->launches), "scan");
    }
    uint64_t tot[2];
    CK(h, cudaMemcpyAsync(&tot[0], *offp + items, 8, cudaMemcpyDeviceToHost, h->stream), "device-to-host copy");
    CK(h, cudaMemcpyAsync(&tot[1], *offn + items, 8, cudaMemcpyDeviceToHost, h->stream), "device-to-host copy");
    CK(h, cudaStreamSynchronize(h->stream), "stream synchronize");
    *P = (int64_t)tot[0];
    *N = (int64_t)tot[1];
    return MCPG_OK;
}

int gather_one(mcpg_handle* h, const mcpg::TruthRegion& r, int lab, const uint64_t* off, const float* v, int64_t ldv,
               float* dst, int* flag) {
    mcpg::GatherSrc g{};
    g.n = 1;
    g.src[0] = v;
    g.lds[0] = ldv;
    g.dst[0] = dst;
    PROF(h, "truth_gather");
    CK(h, mcpg::launch_truth_gather(r, lab, off, g, flag, h->stream, &h->launches), "truth gather");
    return MCPG_OK;
}

int eval_truth_dev(mcpg_handle* h, const float* values, int64_t ldv, const mcpg::TruthRegion& r, double* aupr,
                   double* auroc, int64_t* n_pos, int64_t* n_neg) {
    if (r.rows > 0 && r.cols > 0 && (!values || ldv < r.cols))
        return fail(h, MCPG_ERR_ARG, "eval_truth: null values or leading dimension too small");
    EvalWs w;
    int rc;
    if ((rc = ev_ws(h, w))) return rc;
    uint64_t *offp = nullptr, *offn = nullptr;
    int64_t P = 0, N = 0;
    if ((rc = truth_offsets(h, r, &offp, &offn, &P, &N))) return rc;
    if (n_pos) *n_pos = P;
    if (n_neg) *n_neg = N;
    void* kp;
    if ((rc = scratch(h, S_EV_KP, (size_t)P * 4, &kp))) return rc;
    if (P > 0) {
        if ((rc = gather_one(h, r, 1, offp, values, ldv, (float*)kp, w.flag))) return rc;
        PROF(h, "keys");
        CK(h, mcpg::launch_keys_from_floats((const float*)kp, P, (uint32_t*)kp, w.flag, h->stream, &h->launches),
           "keys");
    }
    return ev_aupr_auroc(
        h, w, (uint32_t*)kp, P, N,
        [&](const uint32_t* X, int64_t nX, uint64_t* lt, uint64_t* eq, uint32_t* dir) {
            return mcpg::launch_rank_count_matrix(X, nX, r, values, ldv, 0, lt, eq, dir, w.flag, h->stream,
                                                  &h->launches);
        },
        [&](uint32_t** out) {
            void* kn;
            int rc2 = scratch(h, S_EV_KN, (size_t)N * 4, &kn);
            if (rc2) return rc2;
            if ((rc2 = gather_one(h, r, 0, offn, values, ldv, (float*)kn, w.flag))) return rc2;
            PROF(h, "keys");
            CK(h, mcpg::launch_keys_from_floats((const float*)kn, N, (uint32_t*)kn, w.flag, h->stream, &h->launches),
               "keys");
            *out = (uint32_t*)kn;
            return MCPG_OK;
        },
        aupr, auroc);
}

int select_truth_dev(mcpg_handle* h, const float* values, int64_t ldv, const mcpg::TruthRegion& r, float* pos,
                     int64_t pos_cap, float* neg, int64_t neg_cap, int64_t* n_pos, int64_t* n_neg) {
    if (r.rows > 0 && r.cols > 0 && (!values || ldv < r.cols))
        return fail(h, MCPG_ERR_ARG, "select_truth: null values or leading dimension too small");
    if (pos_cap < 0 || neg_cap < 0) return fail(h, MCPG_ERR_ARG, "select_truth: negative capacity");
    EvalWs w;
    int rc;
    if ((rc = ev_ws(h, w))) return rc;
    uint64_t *offp = nullptr, *offn = nullptr;
    int64_t P = 0, N = 0;
    if ((rc = truth_offsets(h, r, &offp, &offn, &P, &N))) return rc;
    if (n_pos) *n_pos = P;
    if (n_neg) *n_neg = N;
    if ((pos && P > pos_cap) || (neg && N > neg_cap))
        return fail(h, MCPG_ERR_ARG, "select_truth: capacity too small (need %lld positives, %lld negatives)",
                    (long long)P, (long long)N);
    if (pos && P > 0 && (rc = gather_one(h, r, 1, offp, values, ldv, pos, w.flag))) return rc;
    if (neg && N > 0 && (rc = gather_one(h, r, 0, offn, values, ldv, neg, w.flag))) return rc;
    return finish(h);
}

int combo_eval_dev(mcpg_handle* h, const float* const mats[4], const int64_t lds[4], const mcpg::TruthRegion& r,
                   const double* coeffs, int64_t nc, double* aupr, double* auroc, int64_t* best) {
    if (nc < 0 || (nc > 0 && !coeffs)) return fail(h, MCPG_ERR_ARG, "combo_eval: bad coefficient table");
    if (r.rows > 0 && r.cols > 0) {
        if (!mats[0] || lds[0] < r.cols) return fail(h, MCPG_ERR_ARG, "combo_eval: null mi or leading dimension");
        for (int k = 1; k < 4; ++k) {
            if (mats[k] && lds[k] < r.cols) return fail(h, MCPG_ERR_ARG, "combo_eval: leading dimension too small");
            for (int64_t c = 0; c < nc; ++c)
                if (!mats[k] && coeffs[4 * c + k] != 0.0)
                    return fail(h, MCPG_ERR_ARG, "combo_eval: coefficient row %lld uses a null matrix", (long long)c);
        }
    }
    EvalWs w;
    int rc;
    if ((rc = ev_ws(h, w))) return rc;
    uint64_t *offp = nullptr, *offn = nullptr;
    int64_t P = 0, N = 0;
    if ((rc = truth_offsets(h, r, &offp, &offn, &P, &N))) return rc;
    void *gp, *gn, *kp;
    if ((rc = scratch(h, S_EV_GP, (size_t)(4 * P) * 4, &gp))) return rc;
    if ((rc = scratch(h, S_EV_GN, (size_t)(4 * N) * 4, &gn))) return rc;
    if ((rc = scratch(h, S_EV_KP, (size_t)P * 4, &kp))) return rc;
    const float* gpk[4];
    const float* gnk[4];
    for (int lab = 0; lab < 2; ++lab) {
        mcpg::GatherSrc g{};
        float* base = (float*)(lab ? gp : gn);
        const int64_t cnt = lab ? P : N;
        for (int k = 0; k < 4; ++k) {
            (lab ? gpk : gnk)[k] = base + k * cnt;
            if (!mats[k]) continue;
            g.src[g.n] = mats[k];
            g.lds[g.n] = lds[k];
            g.dst[g.n] = base + k * cnt;
            ++g.n;
        }
        if (cnt == 0) continue;
        PROF(h, "truth_gather");
        CK(h, mcpg::launch_truth_gather(r, lab, lab ? offp : offn, g, w.flag, h->stream, &h->launches),
           "truth gather");
    }
    double max_aupr = 0.0;
    int64_t co = 0;
    for (int64_t c = 0; c < nc; ++c) {
        const double* cs = coeffs + 4 * c;
        if (cs[0] == 1.0 && cs[1] == 0.0 && cs[2] == 0.0 && cs[3] == 0.0) {  // mcpnet.cpp:589
            if (aupr) aupr[c] = NAN;
            if (auroc) auroc[c] = NAN;
            continue;
        }
        mcpg::ComboSrc sp{}, sn{};
        for (int k = 0; k < 4; ++k) {
            sp.g[k] = gpk[k];
            sn.g[k] = gnk[k];
            sp.cs[k] = sn.cs[k] = cs[k];
        }
        sp.kc = sn.kc = mcpg::make_combo_coef(cs);
        sp.n = P;
        sn.n = N;
        {
            PROF(h, "keys");
            CK(h, mcpg::launch_combo_keys(sp, (uint32_t*)kp, w.flag, h->stream, &h->launches), "combo keys");
        }
        double a = 0.0, b = 0.0;
        rc = ev_aupr_auroc(
            h, w, (uint32_t*)kp, P, N,
            [&](const uint32_t* X, int64_t nX, uint64_t* lt, uint64_t* eq, uint32_t* dir) {
                return mcpg::launch_rank_count_combo(X, nX, sn, lt, eq, dir, w.flag, h->stream, &h->launches);
            },
            [&](uint32_t** out) {
                void* kn;
                int rc2 = scratch(h, S_EV_KN, (size_t)N * 4, &kn);
                if (rc2) return rc2;
                PROF(h, "keys");
                CK(h, mcpg::launch_combo_keys(sn, (uint32_t*)kn, w.flag, h->stream, &h->launches), "combo keys");
                *out = (uint32_t*)kn;
                return MCPG_OK;
            },
            &a, &b);
        if (rc) return rc;
        if (aupr) aupr[c] = a;
        if (auroc) auroc[c] = b;
        if (a > max_aupr) {  // mcpnet.cpp:602-606
            max_aupr = a;
            co = c;
        }
    }
    if (best) *best = co;
    return MCPG_OK;
}

// ---- Stouffer / CLR ----
int transform_dev(mcpg_handle* h, const float* A, int64_t n, int64_t lda, int transform, int stats_mode, float* out,
                  int64_t ldo) {
    if (n < 0) return fail(h, MCPG_ERR_ARG, "transform: negative size");
    if (n == 0) return MCPG_OK;
    if (!A || !out || lda < n || ldo < n) return fail(h, MCPG_ERR_ARG, "transform: null pointer or leading dimension");
    if (transform != MCPG_TRANSFORM_STOUFFER && transform != MCPG_TRANSFORM_CLR)
        return fail(h, MCPG_ERR_ARG, "transform: unknown transform %d", transform);
    if (stats_mode != MCPG_ROWSTATS_ALL && stats_mode != MCPG_ROWSTATS_EXCLUDE_DIAGONAL)
        return fail(h, MCPG_ERR_ARG, "transform: unknown statistics mode %d", stats_mode);
    void* st;
    int rc = scratch(h, S_ST_STATS, (size_t)(2 * n) * sizeof(float), &st);
    if (rc) return rc;
    float* mean = (float*)st;
    float* sd = mean + n;
    {
        PROF(h, "row_stats");
        CK(h, mcpg::launch_row_stats(A, n, n, lda, stats_mode == MCPG_ROWSTATS_EXCLUDE_DIAGONAL, 1, mean, sd, h->stream,
                                     &h->launches),
           "row stats");
    }
    {
        PROF(h, "transform");
        CK(h, mcpg::launch_transform(A, n, lda, mean, sd, transform == MCPG_TRANSFORM_CLR, out, ldo, h->stream,
                                     &h->launches),
           "transform");
    }
    return MCPG_OK;
}

// compute_stouffer_tf (mcpnet_helper.hpp:589-634) of a rows x cols (TFs x genes)
// matrix: population z-scores of every row and every column, combined by
// zscored_stouffer_kernel (stouffer.hpp:84-100).
int tf_stats_dev(mcpg_handle* h, const float* A, int64_t rows, int64_t cols, int64_t lda, float* rmean, float* rsd,
                 float* cmean, float* csd) {
    {
        PROF(h, "row_stats");
        CK(h, mcpg::launch_row_stats(A, rows, cols, lda, 0, 0, rmean, rsd, h->stream, &h->launches), "row stats");
    }
    {
        PROF(h, "col_stats");
        CK(h, mcpg::launch_col_stats(A, rows, cols, lda, cmean, csd, h->stream, &h->launches), "column stats");
    }
    return MCPG_OK;
}

int stouffer_tf_dev(mcpg_handle* h, const float* A, int64_t rows, int64_t cols, int64_t lda, float* out, int64_t ldo,
                    int clr = 0) {
    if (rows < 0 || cols < 0) return fail(h, MCPG_ERR_ARG, "stouffer_tf: negative size");
    if (rows == 0 || cols == 0) return MCPG_OK;
    if (!A || !out || lda < cols || ldo < cols)
        return fail(h, MCPG_ERR_ARG, "stouffer_tf: null pointer or leading dimension");
    void* st;
    int rc = scratch(h, S_ST_STATS, (size_t)(2 * rows + 2 * cols) * sizeof(float), &st);
    if (rc) return rc;
    float* rmean = (float*)st;
    float* rsd = rmean + rows;
    float* cmean = rsd + rows;
    float* csd = cmean + cols;
    if ((rc = tf_stats_dev(h, A, rows, cols, lda, rmean, rsd, cmean, csd))) return rc;
    {
        PROF(h, "transform");
        CK(h, mcpg::launch_stouffer_tf(A, rows, cols, lda, rmean, rsd, cmean, csd, clr, out, ldo, h->stream,
                                       &h->launches),
           "TF transform");
    }
    return MCPG_OK;
}

// Stouffer form of the coefficient search: stats_mode MCPG_ROWSTATS_* (square
// matrices, mcpg_transform_dev) or ST_TF (compute_stouffer_tf, any shape).
constexpr int ST_TF = -1;

int combo_stouffer_eval_dev(mcpg_handle* h, const float* const mats[4], const int64_t lds[4],
                            const mcpg::TruthRegion& r, const double* coeffs, int64_t nc, int stats_mode,
                            double* aupr, double* auroc, int64_t* best) {
    const int64_t rows = r.rows, cols = r.cols;
    if (stats_mode != ST_TF && rows != cols)
        return fail(h, MCPG_ERR_ARG, "combo_stouffer_eval: the matrices must be square");
    if (nc < 0 || (nc > 0 && !coeffs)) return fail(h, MCPG_ERR_ARG, "combo_stouffer_eval: bad coefficient table");
    const bool live = rows > 0 && cols > 0;
    if (live) {
        if (!mats[0] || lds[0] < cols)
            return fail(h, MCPG_ERR_ARG, "combo_stouffer_eval: null mi or leading dimension");
        for (int k = 1; k < 4; ++k) {
            if (mats[k] && lds[k] < cols)
                return fail(h, MCPG_ERR_ARG, "combo_stouffer_eval: leading dimension too small");
            for (int64_t c = 0; c < nc; ++c)
                if (!mats[k] && coeffs[4 * c + k] != 0.0)
                    return fail(h, MCPG_ERR_ARG, "combo_stouffer_eval: coefficient row %lld uses a null matrix",
                                (long long)c);
        }
    }
    float *cm = nullptr, *tm = nullptr;
    int64_t ldc = 0;
    int rc;
    if ((rc = stage_out_alloc(h, S_ST_A, rows, cols, &cm, &ldc))) return rc;
    if ((rc = stage_out_alloc(h, S_ST_B, rows, cols, &tm, &ldc))) return rc;
    double max_aupr = 0.0;
    int64_t co = 0;
    for (int64_t c = 0; c < nc; ++c) {
        const double* cs = coeffs + 4 * c;
        if (cs[0] == 1.0 && cs[1] == 0.0 && cs[2] == 0.0 && cs[3] == 0.0) {  // mcpnet.cpp:589
            if (aupr) aupr[c] = NAN;
            if (auroc) auroc[c] = NAN;
            continue;
        }
        double a = 0.0, b = 0.0;
        if (live) {
            {
                PROF(h, "combo");
                CK(h, mcpg::launch_combo(mats[0], lds[0], mats[1], lds[1], mats[2], lds[2], mats[3], lds[3], rows,
                                         cols, cs, cm, ldc, h->stream, &h->launches),
                   "combo kernel");
            }
            rc = stats_mode == ST_TF ? stouffer_tf_dev(h, cm, rows, cols, ldc, tm, ldc)
                                     : transform_dev(h, cm, rows, ldc, MCPG_TRANSFORM_STOUFFER, stats_mode, tm, ldc);
            if (rc) return rc;
            if ((rc = eval_truth_dev(h, tm, ldc, r, &a, &b, nullptr, nullptr))) return rc;
        }
        if (aupr) aupr[c] = a;
        if (auroc) auroc[c] = b;
        if (a > max_aupr) {  // mcpnet.cpp:644-648
            max_aupr = a;
            co = c;
        }
    }
    if (best) *best = co;
    return MCPG_OK;
}

// ---------------- semi-supervised split evaluation (eval_mcpnet) ----------------
// The labelled entries of a region in the reference's mask order -- row-major,
// as select_lower_triangle, the sorted mask of select_from_list
// (mcpnet_helper.hpp:818-826) and select_tfs_from_mat produce it -- with their
// scores from up to four sources (vals[k], null where src[k] is null) and labels.
struct SplitEntries {
    const float* vals[4] = {};
    const int8_t* lab = nullptr;
    const uint64_t* off = nullptr;  // scanned per-item entry counts (for later gathers)
    int64_t E = 0;
};

int split_entries(mcpg_handle* h, const mcpg::TruthRegion& r, const float* const src[4], const int64_t lds[4],
                  SplitEntries& se, int* flag) {
    const int64_t items = mcpg::truth_items(r);
    void *cnt, *off, *tmp;
    int rc;
    if ((rc = scratch(h, S_EV_CNT, (size_t)(2 * items + 1) * 4, &cnt))) return rc;
    if ((rc = scratch(h, S_EV_OFF, (size_t)(items + 1) * 8, &off))) return rc;
    if ((rc = scratch(h, S_EV_TMP, (size_t)mcpg::scan_tmp_elems(items) * 8, &tmp))) return rc;
    uint32_t* cp = (uint32_t*)cnt;
    uint32_t* cn = cp + items;
    uint64_t tot = 0;
    if (items > 0) {
        PROF(h, "truth_count");
        CK(h, mcpg::launch_truth_count(r, cp, cn, h->stream, &h->launches), "truth count");
        CK(h, mcpg::launch_add_u32(cp, cn, items, cp, h->stream, &h->launches), "add");
        CK(h, mcpg::launch_scan_u32(cp, items, (uint64_t*)off, (uint64_t*)tmp, h->stream, &h->launches), "scan");
        CK(h, cudaMemcpyAsync(&tot, (uint64_t*)off + items, 8, cudaMemcpyDeviceToHost, h->stream),
           "device-to-host copy");
        CK(h, cudaStreamSynchronize(h->stream), "stream synchronize");
    }
    const int64_t E = (int64_t)tot;
    if (E >= ((int64_t)1 << 32)) return fail(h, MCPG_ERR_UNSUPPORTED, "split evaluation: 2^32 or more labelled entries");
    int nsrc = 0;
    for (int k = 0; k < 4; ++k) nsrc += src[k] != nullptr;
    void *val, *lab;
    if ((rc = scratch(h, S_SP_VAL, (size_t)(nsrc > 0 ? nsrc : 1) * (size_t)(E > 0 ? E : 1) * 4, &val))) return rc;
    if ((rc = scratch(h, S_SP_LAB, (size_t)(E > 0 ? E : 1), &lab))) return rc;
    mcpg::GatherSrc g{};
    for (int k = 0; k < 4; ++k) {
        se.vals[k] = nullptr;
        if (!src[k]) continue;
        float* d = (float*)val + (size_t)g.n * (size_t)E;
        se.vals[k] = d;
        g.src[g.n] = src[k];
        g.lds[g.n] = lds[k];
        g.dst[g.n] = d;
        ++g.n;
    }
    g.lab_dst = (int8_t*)lab;
    se.lab = (const int8_t*)lab;
    se.off = (const uint64_t*)off;
    se.E = E;
    if (E > 0) {
        PROF(h, "truth_gather");
        CK(h, mcpg::launch_truth_gather(r, -1, (const uint64_t*)off, g, flag, h->stream, &h->launches),
           "truth gather");
    }
    return MCPG_OK;
}

// std::shuffle over E >= 65,536 positions with a 32-bit std::mt19937 swaps a[i]
// with a[j], j uniform in [0, i], for i = 1 .. E-1 (up to 65,535 positions the
// library draws two positions per generator call, and std::shuffle itself runs).
// Every j depends only on the generator, so here the draws run D steps ahead of
// the swaps and prefetch their targets' cache lines, hiding the random-access
// latency that bounds the plain loop over a multi-GB array; the swaps keep their
// order.  The draw is the multiply-shift reduction with rejection of Lemire,
// "Fast Random Integer Generation in an Interval" (ACM TOMACS 29(1), 2019), the
// method libstdc++'s uniform_int_distribution applies to a 32-bit generator.  The
// result is checked against std::shuffle once per process; if they differ (another
// standard library), std::shuffle runs instead.
constexpr int64_t SHUFFLE_PAIRED_MAX = 65535;

inline uint32_t draw_below(std::mt19937& g, uint32_t range) {  // uniform in [0, range)
    uint64_t prod = (uint64_t)(uint32_t)g() * range;
    uint32_t low = (uint32_t)prod;
    if (low < range) {
        const uint32_t threshold = (uint32_t)(0u - range) % range;
        while (low < threshold) {
            prod = (uint64_t)(uint32_t)g() * range;
            low = (uint32_t)prod;
        }
    }
    return (uint32_t)(prod >> 32);
}

void shuffle_prefetched(uint32_t* a, int64_t E, std::mt19937& g) {
    constexpr int D = 32;  // steps of look-ahead (a power of two)
    uint32_t ring[D];
    const int64_t first = E - 1 < D ? E - 1 : D;
    for (int64_t k = 1; k <= first; ++k) {  // the targets of steps 1 .. D
        ring[(k - 1) & (D - 1)] = draw_below(g, (uint32_t)(k + 1));
        __builtin_prefetch(a + ring[(k - 1) & (D - 1)], 1);
    }
    for (int64_t i = 1; i < E; ++i) {
        const int slot = (int)((i - 1) & (D - 1));
        const uint32_t j = ring[slot];
        if (i + D < E) {  // the target of step i + D, drawn after those of steps < i + D
            ring[slot] = draw_below(g, (uint32_t)(i + D + 1));
            __builtin_prefetch(a + ring[slot], 1);
        }
        const uint32_t t = a[i];
        a[i] = a[j];
        a[j] = t;
    }
}

bool prefetched_shuffle_matches() {
    static const bool ok = [] {
        for (uint32_t seed : {1u, 7u, 2026u}) {
            const int64_t E = SHUFFLE_PAIRED_MAX + 1 + 4097;
            std::vector<uint32_t> x((size_t)E), y;
            std::iota(x.begin(), x.end(), 0u);
            y = x;
            std::mt19937 g1(seed), g2(seed);
            std::shuffle(x.begin(), x.end(), g1);
            shuffle_prefetched(y.data(), E, g2);
            if (x != y || g1() != g2()) return false;  // same order and the same generator state after
        }
        return true;
    }();
    return ok;
}

// shuffle_truth (apps/pipeline/eval_mcpnet.cpp:214-224): std::shuffle with a
// std::mt19937 seeded with `seed` over the E mask entries.  std::shuffle's swaps
// depend only on the length and the generator, so the shuffled entry positions
// are the reference's order of its (row, col, label) tuples.  seed 0 keeps the
// mask order.  hp is host work space.
void shuffle_positions(uint32_t* a, int64_t E, uint64_t seed) {
    std::iota(a, a + E, 0u);
    if (seed) {
        std::mt19937 g((std::mt19937::result_type)seed);
        if (E > SHUFFLE_PAIRED_MAX && E <= (int64_t)UINT32_MAX && prefetched_shuffle_matches())
            shuffle_prefetched(a, E, g);
        else
            std::shuffle(a, a + E, g);
    }
}

void shuffle_positions(std::vector<uint32_t>& hp, int64_t E, uint64_t seed) {
    hp.resize((size_t)E);
    shuffle_positions(hp.data(), E, seed);
}

int split_perm(mcpg_handle* h, int64_t E, uint64_t seed, std::vector<uint32_t>& hp, uint32_t* dperm) {
    shuffle_positions(hp, E, seed);
    if (E > 0)
        CK(h, cudaMemcpyAsync(dperm, hp.data(), (size_t)E * 4, cudaMemcpyHostToDevice, h->stream),
           "host-to-device copy");
    return MCPG_OK;
}

// The permutations of iterations i0 .. i0 + n - 1 are independent of one
// another, so a batch is made on several host threads at once (each its own
// std::mt19937), and the next batch is made on a background thread while the
// GPU evaluates the current one.  A batch holds at most 1/16 of the host's
// memory (64 GiB at most) in positions.
struct PermBatch {
    std::vector<std::vector<uint32_t>> p;
    int64_t i0 = 0;
};

int64_t perm_batch_size(int64_t E, int64_t left) {
    int64_t b = (int64_t)omp_get_max_threads();
    const long pages = sysconf(_SC_PHYS_PAGES), psz = sysconf(_SC_PAGESIZE);
    int64_t budget = (pages > 0 && psz > 0) ? (int64_t)pages * psz / 16 : ((int64_t)8 << 30);
    if (budget > ((int64_t)64 << 30)) budget = (int64_t)64 << 30;
    const int64_t cap = budget / ((E > 0 ? E : 1) * 4);
    if (b > cap) b = cap;
    if (b > left) b = left;
    return b < 1 ? 1 : b;
}

void make_perm_batch(PermBatch& pb, int64_t E, int64_t i0, int64_t n) {
    pb.p.resize((size_t)n);
    pb.i0 = i0;
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t b = 0; b < n; ++b) shuffle_positions(pb.p[(size_t)b], E, (uint64_t)(i0 + b));
}

class PermSource {
  public:
    PermSource(int64_t E, int64_t iters) : E_(E), iters_(iters) {}
    ~PermSource() {
        if (worker_.joinable()) worker_.join();
    }
    // The positions of iteration i (called for i = 1, 2, ... in order).
    const std::vector<uint32_t>& get(int64_t i) {
        if (i >= cur_.i0 + (int64_t)cur_.p.size()) {
            if (worker_.joinable()) {
                worker_.join();
                std::swap(cur_, nxt_);
            } else {
                const int64_t n = perm_batch_size(E_, iters_ - next_ + 1);
                make_perm_batch(cur_, E_, next_, n);
                next_ += n;
            }
            if (next_ <= iters_) {  // the batch after this one, in the background
                const int64_t i0 = next_, n = perm_batch_size(E_, iters_ - next_ + 1);
                next_ += n;
                worker_ = std::thread([this, i0, n] { make_perm_batch(nxt_, E_, i0, n); });
            }
        }
        return cur_.p[(size_t)(i - cur_.i0)];
    }

  private:
    int64_t E_, iters_, next_ = 1;
    PermBatch cur_, nxt_;
    std::thread worker_;
};

int upload_perm(mcpg_handle* h, const std::vector<uint32_t>& hp, uint32_t* dperm) {
    if (!hp.empty())
        CK(h, cudaMemcpyAsync(dperm, hp.data(), hp.size() * 4, cudaMemcpyHostToDevice, h->stream),
           "host-to-device copy");
    return MCPG_OK;
}

// compute_aupr2 (mcpnet_helper.hpp:1017-1035) over the shuffled entries
// perm[a..b): their scores (vals, or the combo of *c) split by label into
// positive and negative keys, then the AUPR of aupr_kernel.
int split_aupr_range(mcpg_handle* h, const EvalWs& w, const SplitEntries& se, const uint32_t* perm, int64_t a,
                     int64_t b, const float* vals, const mcpg::ComboSrc* c, double* aupr) {
    void *kp, *kn, *cnt;
    int rc;
    const size_t cap = (size_t)(se.E > 0 ? se.E : 1) * 4;  // sized once for every range
    if ((rc = scratch(h, S_EV_KP, cap, &kp))) return rc;
    if ((rc = scratch(h, S_EV_KN, cap, &kn))) return rc;
    if ((rc = scratch(h, S_SP_CNT, 16, &cnt))) return rc;
    CK(h, cudaMemsetAsync(cnt, 0, 16, h->stream), "memset");
    const mcpg::ComboSrc none{};
    {
        PROF(h, "split_keys");
        CK(h, mcpg::launch_split_keys(perm, a, b, vals, c ? *c : none, c != nullptr, se.lab, (uint32_t*)kp,
                                      (uint32_t*)kn, (unsigned long long*)cnt, w.flag, h->stream, &h->launches),
           "split keys");
    }
    unsigned long long n[2] = {0, 0};
    CK(h, cudaMemcpyAsync(n, cnt, 16, cudaMemcpyDeviceToHost, h->stream), "device-to-host copy");
    CK(h, cudaStreamSynchronize(h->stream), "stream synchronize");
    const int64_t P = (int64_t)n[0], N = (int64_t)n[1];
    uint32_t* knk = (uint32_t*)kn;
    double roc = 0.0;
    return ev_aupr_auroc(
        h, w, (uint32_t*)kp, P, N,
        [&](const uint32_t* X, int64_t nX, uint64_t* lt, uint64_t* eq, uint32_t* dir) {
            return mcpg::launch_rank_count_keys(X, nX, knk, N, lt, eq, dir, h->stream, &h->launches);
        },
        [&](uint32_t** out) {
            *out = knk;
            return MCPG_OK;
        },
        aupr, &roc);
}

int split_check(mcpg_handle* h, const char* who, int64_t iters, const int64_t* tc, int64_t parts, int64_t E) {
    if (iters < 0 || parts < 0) return fail(h, MCPG_ERR_ARG, "%s: negative iteration or part count", who);
    if (parts > 0 && !tc) return fail(h, MCPG_ERR_ARG, "%s: null train counts", who);
    for (int64_t j = 0; j < parts; ++j)
        if (tc[j] < 0 || tc[j] > E)
            return fail(h, MCPG_ERR_ARG, "%s: train count %lld outside 0..%lld labelled entries", who,
                        (long long)tc[j], (long long)E);
    return MCPG_OK;
}

// eval_aupr_mcp (apps/pipeline/eval_mcpnet.cpp:227-301): the AUPR of all
// labelled entries, then for iterations i = 1..iters the entries shuffled with
// seed i and, per train count k, the AUPR of the first k (train) and of the
// rest (test).  train / test: iters x parts, row-major.
int split_aupr_dev(mcpg_handle* h, const float* values, int64_t ldv, const mcpg::TruthRegion& r, int64_t iters,
                   const int64_t* tc, int64_t parts, double* full, double* train, double* test) {
    if (r.rows > 0 && r.cols > 0 && (!values || ldv < r.cols))
        return fail(h, MCPG_ERR_ARG, "split_aupr: null values or leading dimension too small");
    EvalWs w;
    int rc;
    if ((rc = ev_ws(h, w))) return rc;
    SplitEntries se;
    const float* src[4] = {values, nullptr, nullptr, nullptr};
    const int64_t lds[4] = {ldv, 0, 0, 0};
    if ((rc = split_entries(h, r, src, lds, se, w.flag))) return rc;
    if ((rc = split_check(h, "split_aupr", iters, tc, parts, se.E))) return rc;
    void* perm;
    if ((rc = scratch(h, S_SP_PERM, (size_t)(se.E > 0 ? se.E : 1) * 4, &perm))) return rc;
    std::vector<uint32_t> hp;
    const uint32_t* dp = (const uint32_t*)perm;
    if ((rc = split_perm(h, se.E, 0, hp, (uint32_t*)perm))) return rc;
    double a = 0.0;
    if ((rc = split_aupr_range(h, w, se, dp, 0, se.E, se.vals[0], nullptr, &a))) return rc;
    if (full) *full = a;
    PermSource ps(se.E, iters);
    for (int64_t i = 1; i <= iters; ++i) {
        if ((rc = upload_perm(h, ps.get(i), (uint32_t*)perm))) return rc;
        for (int64_t j = 0; j < parts; ++j) {
            double tr = 0.0, te = 0.0;
            if ((rc = split_aupr_range(h, w, se, dp, 0, tc[j], se.vals[0], nullptr, &tr))) return rc;
            if ((rc = split_aupr_range(h, w, se, dp, tc[j], se.E, se.vals[0], nullptr, &te))) return rc;
            if (train) train[(i - 1) * parts + j] = tr;
            if (test) test[(i - 1) * parts + j] = te;
        }
    }
    return MCPG_OK;
}

// eval_combos over the shuffled splits (apps/pipeline/eval_mcpnet.cpp:319-462,
// 814-893): per iteration i (seed i) and train count k, the coefficient row of
// highest AUPR on the first k entries (the first strictly larger, row 0 when
// none is), its AUPR on the rest and on all entries, and the same for the
// Stouffer-transformed combos (stouffer: MCPG_STOUFFER_NONE, a row-statistics
// mode for square matrices, or MCPG_STOUFFER_TF).  Rows (1, 0, 0, 0) are
// skipped.  res: iters x parts x 6 (train, test, Stouffer train, Stouffer test,
// full, Stouffer full; Stouffer values 0 without it); best: iters x parts x 2.
// The scores of every row at the entries do not depend on the split: the
// combos are formed from the gathered matrices on the fly, the Stouffer scores
// (a full matrix transform per row) once per row and kept.
int split_combo_dev(mcpg_handle* h, const float* const mats[4], const int64_t lds[4], const mcpg::TruthRegion& r,
                    const double* coeffs, int64_t nc, int stouffer, int64_t iters, const int64_t* tc, int64_t parts,
                    double* res, int64_t* best) {
    const int64_t rows = r.rows, cols = r.cols;
    if (nc < 1 || !coeffs) return fail(h, MCPG_ERR_ARG, "split_combo_eval: need at least one coefficient row");
    if (stouffer != MCPG_STOUFFER_NONE && stouffer != MCPG_ROWSTATS_ALL && stouffer != MCPG_ROWSTATS_EXCLUDE_DIAGONAL &&
        stouffer != MCPG_STOUFFER_TF)
        return fail(h, MCPG_ERR_ARG, "split_combo_eval: unknown Stouffer mode %d", stouffer);
    if ((stouffer == MCPG_ROWSTATS_ALL || stouffer == MCPG_ROWSTATS_EXCLUDE_DIAGONAL) && rows != cols)
        return fail(h, MCPG_ERR_ARG, "split_combo_eval: the square Stouffer transform needs square matrices");
    if (rows > 0 && cols > 0) {
        if (!mats[0] || lds[0] < cols) return fail(h, MCPG_ERR_ARG, "split_combo_eval: null mi or leading dimension");
        for (int k = 1; k < 4; ++k) {
            if (mats[k] && lds[k] < cols) return fail(h, MCPG_ERR_ARG, "split_combo_eval: leading dimension too small");
            for (int64_t c = 0; c < nc; ++c)
                if (!mats[k] && coeffs[4 * c + k] != 0.0)
                    return fail(h, MCPG_ERR_ARG, "split_combo_eval: coefficient row %lld uses a null matrix",
                                (long long)c);
        }
    }
    EvalWs w;
    int rc;
    if ((rc = ev_ws(h, w))) return rc;
    SplitEntries se;
    if ((rc = split_entries(h, r, mats, lds, se, w.flag))) return rc;
    if ((rc = split_check(h, "split_combo_eval", iters, tc, parts, se.E))) return rc;
    const int64_t E = se.E;
    auto combo_src = [&](int64_t c) {
        mcpg::ComboSrc s{};
        for (int k = 0; k < 4; ++k) {
            s.g[k] = se.vals[k];
            s.cs[k] = coeffs[4 * c + k];
        }
        s.kc = mcpg::make_combo_coef(coeffs + 4 * c);
        s.n = E;
        return s;
    };
    auto skipped = [&](int64_t c) {
        const double* cs = coeffs + 4 * c;
        return cs[0] == 1.0 && cs[1] == 0.0 && cs[2] == 0.0 && cs[3] == 0.0;  // mcpnet.cpp:589
    };
    const bool with_st = stouffer != MCPG_STOUFFER_NONE;
    float* st = nullptr;  // Stouffer scores of row c at the entries: st + c * E
    if (with_st && E > 0) {
        void* p;
        if ((rc = scratch(h, S_SP_ST, (size_t)nc * (size_t)E * 4, &p))) return rc;
        st = (float*)p;
        float *cm = nullptr, *tm = nullptr;
        int64_t ldc = 0;
        if ((rc = stage_out_alloc(h, S_ST_A, rows, cols, &cm, &ldc))) return rc;
        if ((rc = stage_out_alloc(h, S_ST_B, rows, cols, &tm, &ldc))) return rc;
        for (int64_t c = 0; c < nc; ++c) {
            {
                PROF(h, "combo");
                CK(h, mcpg::launch_combo(mats[0], lds[0], mats[1], lds[1], mats[2], lds[2], mats[3], lds[3], rows,
                                         cols, coeffs + 4 * c, cm, ldc, h->stream, &h->launches),
                   "combo kernel");
            }
            rc = stouffer == MCPG_STOUFFER_TF
                     ? stouffer_tf_dev(h, cm, rows, cols, ldc, tm, ldc)
                     : transform_dev(h, cm, rows, ldc, MCPG_TRANSFORM_STOUFFER, stouffer, tm, ldc);
            if (rc) return rc;
            mcpg::GatherSrc g{};
            g.n = 1;
            g.src[0] = tm;
            g.lds[0] = ldc;
            g.dst[0] = st + (size_t)c * (size_t)E;
            PROF(h, "truth_gather");
            CK(h, mcpg::launch_truth_gather(r, -1, se.off, g, w.flag, h->stream, &h->launches), "truth gather");
        }
    }
    void* perm;
    if ((rc = scratch(h, S_SP_PERM, (size_t)(E > 0 ? E : 1) * 4, &perm))) return rc;
    const uint32_t* dp = (const uint32_t*)perm;
    std::vector<uint32_t> hp;
    // AUPR of every row over all entries (the split does not change it)
    if ((rc = split_perm(h, E, 0, hp, (uint32_t*)perm))) return rc;
    std::vector<double> full_p((size_t)nc, 0.0), full_s((size_t)nc, 0.0);
    for (int64_t c = 0; c < nc; ++c) {
        const mcpg::ComboSrc cs = combo_src(c);
        if ((rc = split_aupr_range(h, w, se, dp, 0, E, nullptr, &cs, &full_p[(size_t)c]))) return rc;
        if (with_st && (rc = split_aupr_range(h, w, se, dp, 0, E, st + (size_t)c * (size_t)E, nullptr,
                                              &full_s[(size_t)c])))
            return rc;
    }
    PermSource ps(E, iters);
    for (int64_t i = 1; i <= iters; ++i) {
        if ((rc = upload_perm(h, ps.get(i), (uint32_t*)perm))) return rc;
        for (int64_t j = 0; j < parts; ++j) {
            const int64_t k = tc[j];
            double max_p = 0.0, max_s = 0.0, a = 0.0;
            int64_t co = 0, sco = 0;
            for (int64_t c = 0; c < nc; ++c) {
                if (skipped(c)) continue;
                const mcpg::ComboSrc cs = combo_src(c);
                if ((rc = split_aupr_range(h, w, se, dp, 0, k, nullptr, &cs, &a))) return rc;
                if (a > max_p) {  // eval_mcpnet.cpp:370-373
                    max_p = a;
                    co = c;
                }
                if (!with_st) continue;
                if ((rc = split_aupr_range(h, w, se, dp, 0, k, st + (size_t)c * (size_t)E, nullptr, &a))) return rc;
                if (a > max_s) {
                    max_s = a;
                    sco = c;
                }
            }
            double test_p = 0.0, test_s = 0.0;
            const mcpg::ComboSrc cs = combo_src(co);
            if ((rc = split_aupr_range(h, w, se, dp, k, E, nullptr, &cs, &test_p))) return rc;
            if (with_st &&
                (rc = split_aupr_range(h, w, se, dp, k, E, st + (size_t)sco * (size_t)E, nullptr, &test_s)))
                return rc;
            double* o = res ? res + ((i - 1) * parts + j) * 6 : nullptr;
            if (o) {
                o[0] = max_p;
                o[1] = test_p;
                o[2] = with_st ? max_s : 0.0;
                o[3] = with_st ? test_s : 0.0;
                o[4] = full_p[(size_t)co];
                o[5] = with_st ? full_s[(size_t)sco] : 0.0;
            }
            if (best) {
                best[((i - 1) * parts + j) * 2] = co;
                best[((i - 1) * parts + j) * 2 + 1] = with_st ? sco : 0;
            }
        }
    }
    return MCPG_OK;
}

// Host inputs of the coefficient searches (mi, M1..M3, labels and the TF
// region's row_gene / col_tf) copied to the device; r gets the device region.
int stage_search(mcpg_handle* h, const char* name, const float* const src[4], const int64_t lds[4], int64_t rows,
                 int64_t cols, const int8_t* labels, int64_t ldl, int region, const int32_t* row_gene,
                 const uint8_t* col_tf, const float* d[4], int64_t dl[4], mcpg::TruthRegion* r) {
    int rc;
    if ((rc = truth_region(h, name, labels, rows, cols, ldl, region, row_gene, col_tf, r))) return rc;
    const int slots[4] = {S_IN1, S_IN2, S_IN3, S_IN4};
    for (int k = 0; k < 4; ++k) {
        d[k] = nullptr;
        dl[k] = cols;
        if (!src[k] || rows <= 0 || cols <= 0) continue;
        if (lds[k] < cols) return fail(h, MCPG_ERR_ARG, "%s: leading dimension too small", name);
        float* p;
        if ((rc = stage_in(h, slots[k], src[k], lds[k], rows, cols, &p, &dl[k]))) return rc;
        d[k] = p;
    }
    void *lab, *aux;
    if ((rc = scratch(h, S_EV_LAB, (size_t)(rows * cols), &lab))) return rc;
    if (rows > 0 && cols > 0)
        CK(h, cudaMemcpy2DAsync(lab, (size_t)cols, labels, (size_t)ldl, (size_t)cols, (size_t)rows,
                                cudaMemcpyHostToDevice, h->stream),
           "host-to-device copy");
    r->labels = (const int8_t*)lab;
    r->ldl = cols;
    if (region == MCPG_TRUTH_TF && rows > 0 && cols > 0) {
        if ((rc = scratch(h, S_EV_AUX, (size_t)(rows * 4 + cols), &aux))) return rc;
        CK(h, cudaMemcpyAsync(aux, row_gene, (size_t)rows * 4, cudaMemcpyHostToDevice, h->stream),
           "host-to-device copy");
        CK(h, cudaMemcpyAsync((char*)aux + rows * 4, col_tf, (size_t)cols, cudaMemcpyHostToDevice, h->stream),
           "host-to-device copy");
        r->row_gene = (const int32_t*)aux;
        r->col_tf = (const uint8_t*)aux + rows * 4;
    }
    return MCPG_OK;
}

}  // namespace

using namespace mcpg_api;

extern "C" {

int mcpg_combo_dev(mcpg_handle* h, const float* mi, int64_t ldm, const float* M1, int64_t ld1, const float* M2,
                   int64_t ld2, const float* M3, int64_t ld3, int64_t rows, int64_t cols, const double* coeffs,
                   float* out, int64_t ldo) {
    int rc = check_handle(h);
    if (rc) return rc;
    if (rows < 0 || cols < 0) return fail(h, MCPG_ERR_ARG, "combo: negative size");
    if (rows == 0 || cols == 0) return MCPG_OK;
    if (!mi || !out || !coeffs) return fail(h, MCPG_ERR_ARG, "combo: null pointer");
    if ((coeffs[1] != 0.0 && !M1) || (coeffs[2] != 0.0 && !M2) || (coeffs[3] != 0.0 && !M3))
        return fail(h, MCPG_ERR_ARG, "combo: a matrix with a nonzero coefficient is null");
    if (ldm < cols || ldo < cols || (M1 && ld1 < cols) || (M2 && ld2 < cols) || (M3 && ld3 < cols))
        return fail(h, MCPG_ERR_ARG, "combo: leading dimension too small");
    PROF(h, "combo");
    CK(h, mcpg::launch_combo(mi, ldm, M1, ld1, M2, ld2, M3, ld3, rows, cols, coeffs, out, ldo, h->stream,
                             &h->launches),
       "combo kernel");
    return MCPG_OK;
}

int mcpg_aupr_auroc_dev(mcpg_handle* h, const float* pos, int64_t n_pos, const float* neg, int64_t n_neg,
                        double* aupr, double* auroc) {
    int rc = check_handle(h);
    if (rc) return rc;
    return aupr_auroc_dev(h, pos, n_pos, neg, n_neg, aupr, auroc);
}

int mcpg_aupr_auroc(mcpg_handle* h, const float* pos, int64_t n_pos, const float* neg, int64_t n_neg, double* aupr,
                    double* auroc) {
    int rc = check_handle(h);
    if (rc) return rc;
    if (n_pos < 0 || n_neg < 0) return fail(h, MCPG_ERR_ARG, "aupr_auroc: negative count");
    if ((n_pos > 0 && !pos) || (n_neg > 0 && !neg)) return fail(h, MCPG_ERR_ARG, "aupr_auroc: null score vector");
    float *dp = nullptr, *dn = nullptr;
    int64_t ld;
    if ((rc = stage_in(h, S_IN0, pos, n_pos, 1, n_pos, &dp, &ld))) return rc;
    if ((rc = stage_in(h, S_IN1, neg, n_neg, 1, n_neg, &dn, &ld))) return rc;
    return aupr_auroc_dev(h, dp, n_pos, dn, n_neg, aupr, auroc);
}

int mcpg_eval_truth_dev(mcpg_handle* h, const float* values, int64_t rows, int64_t cols, int64_t ldv,
                        const int8_t* labels, int64_t ldl, int region, const int32_t* row_gene, const uint8_t* col_tf,
                        double* aupr, double* auroc, int64_t* n_pos, int64_t* n_neg) {
    int rc = check_handle(h);
    if (rc) return rc;
    mcpg::TruthRegion r{};
    if ((rc = truth_region(h, "eval_truth", labels, rows, cols, ldl, region, row_gene, col_tf, &r))) return rc;
    return eval_truth_dev(h, values, ldv, r, aupr, auroc, n_pos, n_neg);
}

int mcpg_eval_truth(mcpg_handle* h, const float* values, int64_t rows, int64_t cols, int64_t ldv, const int8_t* labels,
                    int64_t ldl, int region, const int32_t* row_gene, const uint8_t* col_tf, double* aupr,
                    double* auroc, int64_t* n_pos, int64_t* n_neg) {
    int rc = check_handle(h);
    if (rc) return rc;
    mcpg::TruthRegion r{};
    if ((rc = truth_region(h, "eval_truth", labels, rows, cols, ldl, region, row_gene, col_tf, &r))) return rc;
    if (rows > 0 && cols > 0 && (!values || ldv < cols))
        return fail(h, MCPG_ERR_ARG, "eval_truth: null values or leading dimension too small");
    float* dv = nullptr;
    int64_t ld = 0;
    if ((rc = stage_in(h, S_IN0, values, ldv, rows, cols, &dv, &ld))) return rc;
    void *lab, *aux;
    if ((rc = scratch(h, S_EV_LAB, (size_t)(rows * cols), &lab))) return rc;
    if (rows > 0 && cols > 0)
        CK(h, cudaMemcpy2DAsync(lab, (size_t)cols, labels, (size_t)ldl, (size_t)cols, (size_t)rows,
                                cudaMemcpyHostToDevice, h->stream),
           "host-to-device copy");
    r.labels = (const int8_t*)lab;
    r.ldl = cols;
    if (region == MCPG_TRUTH_TF && rows > 0 && cols > 0) {
        if ((rc = scratch(h, S_EV_AUX, (size_t)(rows * 4 + cols), &aux))) return rc;
        CK(h, cudaMemcpyAsync(aux, row_gene, (size_t)rows * 4, cudaMemcpyHostToDevice, h->stream),
           "host-to-device copy");
        CK(h, cudaMemcpyAsync((char*)aux + rows * 4, col_tf, (size_t)cols, cudaMemcpyHostToDevice, h->stream),
           "host-to-device copy");
        r.row_gene = (const int32_t*)aux;
        r.col_tf = (const uint8_t*)aux + rows * 4;
    }
    return eval_truth_dev(h, dv, ld, r, aupr, auroc, n_pos, n_neg);
}

int mcpg_select_truth_dev(mcpg_handle* h, const float* values, int64_t rows, int64_t cols, int64_t ldv,
                          const int8_t* labels, int64_t ldl, int region, const int32_t* row_gene,
                          const uint8_t* col_tf, float* pos, int64_t pos_cap, float* neg, int64_t neg_cap,
                          int64_t* n_pos, int64_t* n_neg) {
    int rc = check_handle(h);
    if (rc) return rc;
    mcpg::TruthRegion r{};
    if ((rc = truth_region(h, "select_truth", labels, rows, cols, ldl, region, row_gene, col_tf, &r))) return rc;
    return select_truth_dev(h, values, ldv, r, pos, pos_cap, neg, neg_cap, n_pos, n_neg);
}

int mcpg_combo_eval_dev(mcpg_handle* h, const float* mi, int64_t ldm, const float* M1, int64_t ld1, const float* M2,
                        int64_t ld2, const float* M3, int64_t ld3, int64_t rows, int64_t cols, const int8_t* labels,
                        int64_t ldl, int region, const int32_t* row_gene, const uint8_t* col_tf, const double* coeffs,
                        int64_t n_coeffs, double* aupr, double* auroc, int64_t* best) {
    int rc = check_handle(h);
    if (rc) return rc;
    mcpg::TruthRegion r{};
    if ((rc = truth_region(h, "combo_eval", labels, rows, cols, ldl, region, row_gene, col_tf, &r))) return rc;
    const float* mats[4] = {mi, M1, M2, M3};
    const int64_t lds[4] = {ldm, ld1, ld2, ld3};
    return combo_eval_dev(h, mats, lds, r, coeffs, n_coeffs, aupr, auroc, best);
}

int mcpg_combo(mcpg_handle* h, const float* mi, int64_t ldm, const float* M1, int64_t ld1, const float* M2, int64_t ld2,
               const float* M3, int64_t ld3, int64_t rows, int64_t cols, const double* coeffs, float* out, int64_t ldo) {
    int rc = check_handle(h);
    if (rc) return rc;
    if (rows < 0 || cols < 0) return fail(h, MCPG_ERR_ARG, "combo: negative size");
    if (rows == 0 || cols == 0) return MCPG_OK;
    if (!mi || !out || !coeffs) return fail(h, MCPG_ERR_ARG, "combo: null pointer");
    if ((coeffs[1] != 0.0 && !M1) || (coeffs[2] != 0.0 && !M2) || (coeffs[3] != 0.0 && !M3))
        return fail(h, MCPG_ERR_ARG, "combo: a matrix with a nonzero coefficient is null");
    const float* src[4] = {mi, M1, M2, M3};
    const int64_t lds[4] = {ldm, ld1, ld2, ld3};
    const int slots[4] = {S_IN1, S_IN2, S_IN3, S_IN4};
    float* d[4] = {};
    int64_t dl[4] = {cols, cols, cols, cols};
    for (int k = 0; k < 4; ++k) {
        if (!src[k] || (k > 0 && coeffs[k] == 0.0)) continue;
        if (lds[k] < cols) return fail(h, MCPG_ERR_ARG, "combo: leading dimension too small");
        if ((rc = in_view(h, slots[k], src[k], lds[k], rows, cols, &d[k], &dl[k]))) return rc;
    }
    float* dout;
    int64_t ld;
    if ((rc = out_view(h, S_OUT0, out, ldo, rows, cols, &dout, &ld))) return rc;
    {
        PROF(h, "combo");
        CK(h, mcpg::launch_combo(d[0], dl[0], d[1], dl[1], d[2], dl[2], d[3], dl[3], rows, cols, coeffs, dout, ld,
                                 h->stream, &h->launches),
           "combo kernel");
    }
    if ((rc = copy_out(h, out, ldo, dout, ld, rows, cols))) return rc;
    return finish(h);
}

int mcpg_combo_eval(mcpg_handle* h, const float* mi, int64_t ldm, const float* M1, int64_t ld1, const float* M2,
                    int64_t ld2, const float* M3, int64_t ld3, int64_t rows, int64_t cols, const int8_t* labels,
                    int64_t ldl, int region, const int32_t* row_gene, const uint8_t* col_tf, const double* coeffs,
                    int64_t n_coeffs, double* aupr, double* auroc, int64_t* best) {
    int rc = check_handle(h);
    if (rc) return rc;
    const float* src[4] = {mi, M1, M2, M3};
    const int64_t lds[4] = {ldm, ld1, ld2, ld3};
    const float* d[4];
    int64_t dl[4];
    mcpg::TruthRegion r{};
    if ((rc = stage_search(h, "combo_eval", src, lds, rows, cols, labels, ldl, region, row_gene, col_tf, d, dl, &r)))
        return rc;
    return combo_eval_dev(h, d, dl, r, coeffs, n_coeffs, aupr, auroc, best);
}

int mcpg_row_stats_dev(mcpg_handle* h, const float* A, int64_t rows, int64_t cols, int64_t lda, int stats_mode,
                       float* mean, float* sd) {
    int rc = check_handle(h);
    if (rc) return rc;
    if (rows < 0 || cols < 0) return fail(h, MCPG_ERR_ARG, "row_stats: negative size");
    if (rows == 0) return MCPG_OK;
    if (!A || !mean || !sd || lda < cols) return fail(h, MCPG_ERR_ARG, "row_stats: null pointer or leading dimension");
    if (stats_mode != MCPG_ROWSTATS_ALL && stats_mode != MCPG_ROWSTATS_EXCLUDE_DIAGONAL)
        return fail(h, MCPG_ERR_ARG, "row_stats: unknown statistics mode %d", stats_mode);
    PROF(h, "row_stats");
    CK(h, mcpg::launch_row_stats(A, rows, cols, lda, stats_mode == MCPG_ROWSTATS_EXCLUDE_DIAGONAL, 1, mean, sd,
                                 h->stream, &h->launches),
       "row stats");
    return MCPG_OK;
}

int mcpg_transform_dev(mcpg_handle* h, const float* A, int64_t n, int64_t lda, int transform, int stats_mode,
                       float* out, int64_t ldo) {
    int rc = check_handle(h);
    if (rc) return rc;
    return transform_dev(h, A, n, lda, transform, stats_mode, out, ldo);
}

int mcpg_transform(mcpg_handle* h, const float* A, int64_t n, int64_t lda, int transform, int stats_mode, float* out,
                   int64_t ldo) {
    int rc = check_handle(h);
    if (rc) return rc;
    if (n < 0) return fail(h, MCPG_ERR_ARG, "transform: negative size");
    if (n == 0) return MCPG_OK;
    if (!A || !out || lda < n || ldo < n) return fail(h, MCPG_ERR_ARG, "transform: null pointer or leading dimension");
    float *da, *dout;
    int64_t la, lo;
    if ((rc = stage_in(h, S_IN0, A, lda, n, n, &da, &la))) return rc;
    if ((rc = out_view(h, S_OUT0, out, ldo, n, n, &dout, &lo))) return rc;
    if ((rc = transform_dev(h, da, n, la, transform, stats_mode, dout, lo))) return rc;
    if ((rc = copy_out(h, out, ldo, dout, lo, n, n))) return rc;
    return finish(h);
}

int mcpg_combo_stouffer_eval_dev(mcpg_handle* h, const float* mi, int64_t ldm, const float* M1, int64_t ld1,
                                 const float* M2, int64_t ld2, const float* M3, int64_t ld3, int64_t n,
                                 const int8_t* labels, int64_t ldl, int region, const int32_t* row_gene,
                                 const uint8_t* col_tf, const double* coeffs, int64_t n_coeffs, int stats_mode,
                                 double* aupr, double* auroc, int64_t* best) {
    int rc = check_handle(h);
    if (rc) return rc;
    mcpg::TruthRegion r{};
    if ((rc = truth_region(h, "combo_stouffer_eval", labels, n, n, ldl, region, row_gene, col_tf, &r))) return rc;
    const float* mats[4] = {mi, M1, M2, M3};
    const int64_t lds[4] = {ldm, ld1, ld2, ld3};
    return combo_stouffer_eval_dev(h, mats, lds, r, coeffs, n_coeffs, stats_mode, aupr, auroc, best);
}

int mcpg_combo_stouffer_eval(mcpg_handle* h, const float* mi, int64_t ldm, const float* M1, int64_t ld1,
                             const float* M2, int64_t ld2, const float* M3, int64_t ld3, int64_t n,
                             const int8_t* labels, int64_t ldl, int region, const int32_t* row_gene,
                             const uint8_t* col_tf, const double* coeffs, int64_t n_coeffs, int stats_mode,
                             double* aupr, double* auroc, int64_t* best) {
    int rc = check_handle(h);
    if (rc) return rc;
    if (stats_mode != MCPG_ROWSTATS_ALL && stats_mode != MCPG_ROWSTATS_EXCLUDE_DIAGONAL)
        return fail(h, MCPG_ERR_ARG, "combo_stouffer_eval: unknown statistics mode %d", stats_mode);
    const float* src[4] = {mi, M1, M2, M3};
    const int64_t lds[4] = {ldm, ld1, ld2, ld3};
    const float* d[4];
    int64_t dl[4];
    mcpg::TruthRegion r{};
    if ((rc = stage_search(h, "combo_stouffer_eval", src, lds, n, n, labels, ldl, region, row_gene, col_tf, d, dl,
                           &r)))
        return rc;
    return combo_stouffer_eval_dev(h, d, dl, r, coeffs, n_coeffs, stats_mode, aupr, auroc, best);
}

int mcpg_combo_stouffer_tf_eval_dev(mcpg_handle* h, const float* mi, int64_t ldm, const float* M1, int64_t ld1,
                                    const float* M2, int64_t ld2, const float* M3, int64_t ld3, int64_t rows,
                                    int64_t cols, const int8_t* labels, int64_t ldl, int region,
                                    const int32_t* row_gene, const uint8_t* col_tf, const double* coeffs,
                                    int64_t n_coeffs, double* aupr, double* auroc, int64_t* best) {
    int rc = check_handle(h);
    if (rc) return rc;
    mcpg::TruthRegion r{};
    if ((rc = truth_region(h, "combo_stouffer_tf_eval", labels, rows, cols, ldl, region, row_gene, col_tf, &r)))
        return rc;
    const float* mats[4] = {mi, M1, M2, M3};
    const int64_t lds[4] = {ldm, ld1, ld2, ld3};
    return combo_stouffer_eval_dev(h, mats, lds, r, coeffs, n_coeffs, ST_TF, aupr, auroc, best);
}

int mcpg_combo_stouffer_tf_eval(mcpg_handle* h, const float* mi, int64_t ldm, const float* M1, int64_t ld1,
                                const float* M2, int64_t ld2, const float* M3, int64_t ld3, int64_t rows, int64_t cols,
                                const int8_t* labels, int64_t ldl, int region, const int32_t* row_gene,
                                const uint8_t* col_tf, const double* coeffs, int64_t n_coeffs, double* aupr,
                                double* auroc, int64_t* best) {
    int rc = check_handle(h);
    if (rc) return rc;
    const float* src[4] = {mi, M1, M2, M3};
    const int64_t lds[4] = {ldm, ld1, ld2, ld3};
    const float* d[4];
    int64_t dl[4];
    mcpg::TruthRegion r{};
    if ((rc = stage_search(h, "combo_stouffer_tf_eval", src, lds, rows, cols, labels, ldl, region, row_gene, col_tf,
                           d, dl, &r)))
        return rc;
    return combo_stouffer_eval_dev(h, d, dl, r, coeffs, n_coeffs, ST_TF, aupr, auroc, best);
}

int mcpg_split_aupr_dev(mcpg_handle* h, const float* values, int64_t rows, int64_t cols, int64_t ldv,
                        const int8_t* labels, int64_t ldl, int region, const int32_t* row_gene, const uint8_t* col_tf,
                        int64_t iterations, const int64_t* train_counts, int64_t parts, double* full_aupr,
                        double* train_aupr, double* test_aupr) {
    int rc = check_handle(h);
    if (rc) return rc;
    mcpg::TruthRegion r{};
    if ((rc = truth_region(h, "split_aupr", labels, rows, cols, ldl, region, row_gene, col_tf, &r))) return rc;
    return split_aupr_dev(h, values, ldv, r, iterations, train_counts, parts, full_aupr, train_aupr, test_aupr);
}

int mcpg_split_aupr(mcpg_handle* h, const float* values, int64_t rows, int64_t cols, int64_t ldv,
                    const int8_t* labels, int64_t ldl, int region, const int32_t* row_gene, const uint8_t* col_tf,
                    int64_t iterations, const int64_t* train_counts, int64_t parts, double* full_aupr,
                    double* train_aupr, double* test_aupr) {
    int rc = check_handle(h);
    if (rc) return rc;
    const float* src[4] = {values, nullptr, nullptr, nullptr};
    const int64_t lds[4] = {ldv, 0, 0, 0};
    const float* d[4];
    int64_t dl[4];
    mcpg::TruthRegion r{};
    if ((rc = stage_search(h, "split_aupr", src, lds, rows, cols, labels, ldl, region, row_gene, col_tf, d, dl, &r)))
        return rc;
    return split_aupr_dev(h, d[0], dl[0], r, iterations, train_counts, parts, full_aupr, train_aupr, test_aupr);
}

int mcpg_shuffle_positions(uint32_t* out, int64_t entries, uint64_t seed) {
    if (entries < 0 || entries > (int64_t)UINT32_MAX || (entries > 0 && !out)) return MCPG_ERR_ARG;
    shuffle_positions(out, entries, seed);
    return MCPG_OK;
}

int mcpg_split_combo_eval_dev(mcpg_handle* h, const float* mi, int64_t ldm, const float* M1, int64_t ld1,
                              const float* M2, int64_t ld2, const float* M3, int64_t ld3, int64_t rows, int64_t cols,
                              const int8_t* labels, int64_t ldl, int region, const int32_t* row_gene,
                              const uint8_t* col_tf, const double* coeffs, int64_t n_coeffs, int stouffer,
                              int64_t iterations, const int64_t* train_counts, int64_t parts, double* results,
                              int64_t* best) {
    int rc = check_handle(h);
    if (rc) return rc;
    mcpg::TruthRegion r{};
    if ((rc = truth_region(h, "split_combo_eval", labels, rows, cols, ldl, region, row_gene, col_tf, &r))) return rc;
    const float* mats[4] = {mi, M1, M2, M3};
    const int64_t lds[4] = {ldm, ld1, ld2, ld3};
    return split_combo_dev(h, mats, lds, r, coeffs, n_coeffs, stouffer, iterations, train_counts, parts, results,
                           best);
}

int mcpg_split_combo_eval(mcpg_handle* h, const float* mi, int64_t ldm, const float* M1, int64_t ld1, const float* M2,
                          int64_t ld2, const float* M3, int64_t ld3, int64_t rows, int64_t cols, const int8_t* labels,
                          int64_t ldl, int region, const int32_t* row_gene, const uint8_t* col_tf,
                          const double* coeffs, int64_t n_coeffs, int stouffer, int64_t iterations,
                          const int64_t* train_counts, int64_t parts, double* results, int64_t* best) {
    int rc = check_handle(h);
    if (rc) return rc;
    const float* src[4] = {mi, M1, M2, M3};
    const int64_t lds[4] = {ldm, ld1, ld2, ld3};
    const float* d[4];
    int64_t dl[4];
    mcpg::TruthRegion r{};
    if ((rc = stage_search(h, "split_combo_eval", src, lds, rows, cols, labels, ldl, region, row_gene, col_tf, d, dl,
                           &r)))
        return rc;
    return split_combo_dev(h, d, dl, r, coeffs, n_coeffs, stouffer, iterations, train_counts, parts, results, best);
}

int mcpg_stouffer_tf_stats_dev(mcpg_handle* h, const float* A, int64_t rows, int64_t cols, int64_t lda,
                               float* row_mean, float* row_sd, float* col_mean, float* col_sd) {
    int rc = check_handle(h);
    if (rc) return rc;
    if (rows < 0 || cols < 0) return fail(h, MCPG_ERR_ARG, "stouffer_tf_stats: negative size");
    if (rows == 0 || cols == 0) return MCPG_OK;
    if (!A || !row_mean || !row_sd || !col_mean || !col_sd || lda < cols)
        return fail(h, MCPG_ERR_ARG, "stouffer_tf_stats: null pointer or leading dimension");
    return tf_stats_dev(h, A, rows, cols, lda, row_mean, row_sd, col_mean, col_sd);
}

int mcpg_stouffer_tf_dev(mcpg_handle* h, const float* A, int64_t rows, int64_t cols, int64_t lda, float* out,
                         int64_t ldo) {
    int rc = check_handle(h);
    if (rc) return rc;
    return stouffer_tf_dev(h, A, rows, cols, lda, out, ldo);
}

int mcpg_transform_tf_dev(mcpg_handle* h, const float* A, int64_t rows, int64_t cols, int64_t lda, int transform,
                          float* out, int64_t ldo) {
    int rc = check_handle(h);
    if (rc) return rc;
    if (transform != MCPG_TRANSFORM_STOUFFER && transform != MCPG_TRANSFORM_CLR)
        return fail(h, MCPG_ERR_ARG, "transform_tf: unknown transform %d", transform);
    return stouffer_tf_dev(h, A, rows, cols, lda, out, ldo, transform == MCPG_TRANSFORM_CLR);
}

int mcpg_transform_tf(mcpg_handle* h, const float* A, int64_t rows, int64_t cols, int64_t lda, int transform,
                      float* out, int64_t ldo) {
    int rc = check_handle(h);
    if (rc) return rc;
    if (transform != MCPG_TRANSFORM_STOUFFER && transform != MCPG_TRANSFORM_CLR)
        return fail(h, MCPG_ERR_ARG, "transform_tf: unknown transform %d", transform);
    if (rows < 0 || cols < 0) return fail(h, MCPG_ERR_ARG, "transform_tf: negative size");
    if (rows == 0 || cols == 0) return MCPG_OK;
    if (!A || !out || lda < cols || ldo < cols)
        return fail(h, MCPG_ERR_ARG, "transform_tf: null pointer or leading dimension");
    float *da, *dout;
    int64_t la, lo;
    if ((rc = stage_in(h, S_IN0, A, lda, rows, cols, &da, &la))) return rc;
    if ((rc = out_view(h, S_OUT0, out, ldo, rows, cols, &dout, &lo))) return rc;
    if ((rc = stouffer_tf_dev(h, da, rows, cols, la, dout, lo, transform == MCPG_TRANSFORM_CLR))) return rc;
    if ((rc = copy_out(h, out, ldo, dout, lo, rows, cols))) return rc;
    return finish(h);
}

int mcpg_stouffer_tf(mcpg_handle* h, const float* A, int64_t rows, int64_t cols, int64_t lda, float* out,
                     int64_t ldo) {
    int rc = check_handle(h);
    if (rc) return rc;
    if (rows < 0 || cols < 0) return fail(h, MCPG_ERR_ARG, "stouffer_tf: negative size");
    if (rows == 0 || cols == 0) return MCPG_OK;
    if (!A || !out || lda < cols || ldo < cols)
        return fail(h, MCPG_ERR_ARG, "stouffer_tf: null pointer or leading dimension");
    float *da, *dout;
    int64_t la, lo;
    if ((rc = stage_in(h, S_IN0, A, lda, rows, cols, &da, &la))) return rc;
    if ((rc = out_view(h, S_OUT0, out, ldo, rows, cols, &dout, &lo))) return rc;
    if ((rc = stouffer_tf_dev(h, da, rows, cols, la, dout, lo))) return rc;
    if ((rc = copy_out(h, out, ldo, dout, lo, rows, cols))) return rc;
    return finish(h);
}

}  // extern "C"
