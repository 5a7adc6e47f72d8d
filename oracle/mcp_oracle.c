/* CPU oracle for the MCPNet compute core: a C restatement of the reference's
 * B-spline MI, max-min (MCP), ratio, DPI and closure arithmetic.
 *
 * TEST INFRASTRUCTURE ONLY -- the checker, never the thing measured or
 * shipped.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * leg load it (through oracle/oracle.py).  Its fidelity to the reference is
 * pinned by tests/test_oracle_golden.py against fixtures produced by MCPNet's
 * own kernels (oracle/ref/ref_driver.cpp, tests/golden/make_golden.py).
 *
 * Build: oracle/Makefile -> oracle/_build/libmcporacle.so
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <float.h>

#define REAL float
#define SFX f32
#include "mcp_oracle_impl.h"
#undef REAL
#undef SFX

#define REAL double
#define SFX f64
#include "mcp_oracle_impl.h"
#undef REAL
#undef SFX

int orc_num_threads(void) {
#ifdef _OPENMP
    extern int omp_get_max_threads(void);
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ---------------- gold-standard evaluation ----------------
 * Scores arrive as doubles (float scores convert exactly, so order and
 * equality are those of the float comparisons of the reference's IT = float
 * instantiation); every curve is accumulated in double left to right over the
 * distinct thresholds in ascending order, as the reference loops do. */

static int orc_cmp_double(const void* a, const void* b) {
    const double x = *(const double*)a, y = *(const double*)b;
    return (x > y) - (x < y);
}

/* Sorts X (copied) and places every Y by lower_bound: lt[i] counts y with
 * X[i-1] < y < X[i], eq[i] counts y == X[i] (i = first index of an equal run),
 * lt[nx] counts y above all of X -- aupr_kernel::ordering (aupr.hpp:84-125) and
 * auroc_kernel::count_le (auroc.hpp:107-146). */
static double* orc_sorted_rank(const double* X, int64_t nx, const double* Y, int64_t ny, uint64_t** lt_out,
                               uint64_t** eq_out) {
    double* s = (double*)malloc((size_t)(nx > 0 ? nx : 1) * sizeof(double));
    uint64_t* lt = (uint64_t*)calloc((size_t)nx + 1, sizeof(uint64_t));
    uint64_t* eq = (uint64_t*)calloc((size_t)nx + 1, sizeof(uint64_t));
    memcpy(s, X, (size_t)nx * sizeof(double));
    qsort(s, (size_t)nx, sizeof(double), orc_cmp_double);
    for (int64_t k = 0; k < ny; ++k) {
        const double y = Y[k];
        int64_t lo = 0, hi = nx;
        while (lo < hi) {
            const int64_t mid = lo + (hi - lo) / 2;
            if (s[mid] < y) lo = mid + 1; else hi = mid;
        }
        if (lo < nx && s[lo] == y) ++eq[lo]; else ++lt[lo];
    }
    *lt_out = lt;
    *eq_out = eq;
    return s;
}

/* aupr_kernel::average_compute_1sort (aupr.hpp:127-236): per distinct positive
 * score t, ascending, add TP(>=t)/(TP(>=t)+FP(>=t)) * (#pos == t)/n_pos. */
double orc_aupr(const double* pos, int64_t np, const double* neg, int64_t nn) {
    if (np == 0) return 0.0;
    uint64_t *lt, *eq;
    double* s = orc_sorted_rank(pos, np, neg, nn, &lt, &eq);
    const double inv = 1.0 / (double)np;
    double aupr = 0.0;
    uint64_t below = 0; /* negatives below the current threshold */
    for (int64_t f = 0, e; f < np; f = e) {
        for (e = f + 1; e < np && s[e] == s[f]; ++e) {}
        below += lt[f];
        const uint64_t tp = (uint64_t)(np - f), fp = (uint64_t)nn - below;
        const double prec = (tp > 0 || fp > 0) ? (double)tp / (double)(tp + fp) : 1.0;
        aupr += prec * ((double)(e - f) * inv);
        below += eq[f];
    }
    free(s);
    free(lt);
    free(eq);
    return aupr;
}

/* auroc_kernel::average_compute_1sort(YV, XV) (auroc.hpp:151-252): per
 * distinct X score t, ascending, add (#Y >= t)/|Y| * (#X == t)/|X|. */
static double orc_roc_avg(const double* Y, int64_t ny, const double* X, int64_t nx) {
    if (nx == 0 || ny == 0) return 0.0;
    uint64_t *lt, *eq;
    double* s = orc_sorted_rank(X, nx, Y, ny, &lt, &eq);
    const double invy = 1.0 / (double)ny, invx = 1.0 / (double)nx;
    double roc = 0.0;
    uint64_t below = 0;
    for (int64_t f = 0, e; f < nx; f = e) {
        for (e = f + 1; e < nx && s[e] == s[f]; ++e) {}
        below += lt[f];
        roc += ((double)((uint64_t)ny - below) * invy) * ((double)(e - f) * invx);
        below += eq[f];
    }
    free(s);
    free(lt);
    free(eq);
    return roc;
}

/* auroc_kernel::operator()(pos, pos_count, neg, neg_count) (auroc.hpp:562-579):
 * the smaller set is the sorted one. */
double orc_auroc(const double* pos, int64_t np, const double* neg, int64_t nn) {
    return np < nn ? 1.0 - orc_roc_avg(neg, nn, pos, np) : orc_roc_avg(pos, np, neg, nn);
}

/* select_lower_triangle (mcpnet_helper.hpp:862-891), select_tfs_from_mat
 * (893-940) or every entry, then select_values2 (947-998): labelled scores in
 * row-major order.  region 0 = lower triangle, 1 = all, 2 = TF rows. */
void orc_select_truth(const float* V, int64_t rows, int64_t cols, int64_t ldv, const int8_t* L, int64_t ldl,
                      int region, const int32_t* row_gene, const uint8_t* col_tf, float* pos, int64_t* np,
                      float* neg, int64_t* nn) {
    int64_t p = 0, q = 0;
    for (int64_t i = 0; i < rows; ++i) {
        const int64_t last = (region == 0) ? (cols < i ? cols : i) : cols;
        for (int64_t j = 0; j < last; ++j) {
            if (region == 2) {
                const int64_t g = row_gene[i];
                if (g == j || (g > j && col_tf[j])) continue;
            }
            const int8_t l = L[i * ldl + j];
            if (l == 1) pos[p++] = V[i * ldv + j];
            else if (l == 0) neg[q++] = V[i * ldv + j];
        }
    }
    *np = p;
    *nn = q;
}

/* ---------------- adaptive-partitioning MI ----------------
 * Rank transform: stands in for splash::kernel::Rank<T, size_t, 0, false>
 * (apps/pipeline/mcpnet_helper.hpp:122-131), whose source is not in the
 * reference snapshot: descending order (the largest value gets rank 0), tied
 * values share the lowest rank of their group.  Parity of this step is
 * unpinned; the MI below is pinned against the reference's own kernels given
 * the ranks. */
typedef struct { float v; int64_t i; } orc_vi;
static int orc_cmp_desc(const void* a, const void* b) {
    const orc_vi* x = (const orc_vi*)a;
    const orc_vi* y = (const orc_vi*)b;
    if (x->v > y->v) return -1;
    if (x->v < y->v) return 1;
    return (x->i > y->i) - (x->i < y->i);
}
void orc_ranks_desc(const float* X, int64_t n, int64_t m, int64_t ldx, int64_t* R) {
#pragma omp parallel for schedule(static)
    for (int64_t g = 0; g < n; ++g) {
        orc_vi* t = (orc_vi*)malloc((size_t)(m > 0 ? m : 1) * sizeof(orc_vi));
        for (int64_t s = 0; s < m; ++s) {
            t[s].v = X[g * ldx + s];
            t[s].i = s;
        }
        qsort(t, (size_t)m, sizeof(orc_vi), orc_cmp_desc);
        int64_t head = 0;
        for (int64_t p = 0; p < m; ++p) {
            if (p > 0 && t[p].v != t[p - 1].v) head = p;
            R[g * m + t[p].i] = head;
        }
        free(t);
    }
}

/* One pair of AdaptivePartitionRankMIKernel2::operator() (AdaptivePartitioningMI.hpp:535-648)
 * with x-ranks grouped by y-rank as _createSparseMatrix (:461-491) builds them.
 * cx / cy: cumulative rank histograms (IntegralCumulativeHistogramKernel, :414-438):
 * c[k] = number of samples with rank < k, k = 0..m. */
typedef struct { int64_t x1, y1, x2, y2, npts; int whole; } orc_win;

static double orc_ap_term(const int64_t* cx, const int64_t* cy, const orc_win* w) {
    /* compute_for_window (:518-531) */
    const int64_t nx = cx[w->x2] - cx[w->x1], ny = cy[w->y2] - cy[w->y1];
    return (double)w->npts * log2((double)w->npts / (double)(nx * ny));
}

static double orc_ap_pair(const int64_t* rx, const int64_t* ry, const int64_t* cx, const int64_t* cy, int64_t m,
                          int64_t* xg, int64_t* fill, orc_win* stack) {
    for (int64_t k = 0; k <= m; ++k) fill[k] = 0;
    for (int64_t s = 0; s < m; ++s) xg[cy[ry[s]] + fill[ry[s]]++] = rx[s];
    int64_t top = 0;
    stack[top++] = (orc_win){0, 0, m, m, m, 1};
    double mi = 0.0;
    while (top > 0) {
        orc_win w = stack[top - 1];
        const int64_t mx = (w.x1 + w.x2) >> 1, my = (w.y1 + w.y2) >> 1;
        orc_win sub[4] = {{w.x1, w.y1, mx, my, 0, 0}, {mx, w.y1, w.x2, my, 0, 0},
                          {w.x1, my, mx, w.y2, 0, 0}, {mx, my, w.x2, w.y2, 0, 0}};
        for (int q = 0; q < 4; ++q) { /* _getNumPointsInWindow (:493-516) */
            orc_win* s = &sub[q];
            if (s->x1 >= s->x2 || s->y1 >= s->y2) continue;
            if (cx[s->x2] - cx[s->x1] == 0 || cy[s->y2] - cy[s->y1] == 0) continue;
            for (int64_t k = cy[s->y1]; k < cy[s->y2]; ++k) s->npts += (xg[k] >= s->x1 && xg[k] < s->x2);
        }
        const double e = (double)w.npts / 4.0;
        double chi = 0.0;
        for (int q = 0; q < 4; ++q) {
            const double d = (double)sub[q].npts - e;
            chi += d * d;
        }
        chi /= e;
        --top; /* the window is consumed either way */
        if (chi > 7.815 || w.whole) {
            for (int q = 0; q < 4; ++q) {
                const orc_win* s = &sub[q];
                const int split = ((s->x1 + 1) < s->x2 || (s->y1 + 1) < s->y2) && s->npts > 2;
                if (split) stack[top++] = *s;
                else if (s->npts > 0) mi += orc_ap_term(cx, cy, s);
            }
        } else if (w.npts > 0) {
            mi += orc_ap_term(cx, cy, &w);
        }
    }
    return mi / (double)m + log2((double)m);
}

void orc_ap_mi(const int64_t* R, int64_t n, int64_t m, float* out, int64_t ldo) {
    int64_t* C = (int64_t*)calloc((size_t)(n * (m + 1)), sizeof(int64_t));
    for (int64_t g = 0; g < n; ++g) {
        int64_t* c = C + g * (m + 1);
        for (int64_t s = 0; s < m; ++s) ++c[R[g * m + s] + 1];
        for (int64_t k = 1; k <= m; ++k) c[k] += c[k - 1];
    }
#pragma omp parallel
    {
        int64_t* xg = (int64_t*)malloc((size_t)(m + 1) * sizeof(int64_t));
        int64_t* fill = (int64_t*)malloc((size_t)(m + 1) * sizeof(int64_t));
        orc_win* stack = (orc_win*)malloc((size_t)(4 * 64 + 4 * m + 8) * sizeof(orc_win));
#pragma omp for schedule(dynamic, 1)
        for (int64_t i = 0; i < n; ++i)
            for (int64_t j = i; j < n; ++j) {
                const float v = (float)orc_ap_pair(R + i * m, R + j * m, C + i * (m + 1), C + j * (m + 1), m, xg,
                                                   fill, stack);
                out[i * ldo + j] = v;
                out[j * ldo + i] = v;
            }
        free(xg);
        free(fill);
        free(stack);
    }
    free(C);
}

/* ---------------- Stouffer / CLR ----------------
 * Row statistics standing in for splash::kernel::GaussianParamsExclude1<T,T,true>
 * (the splash source is absent from the reference; parity unpinned): FP64
 * mean and unbiased (N - 1) standard deviation of each row, two passes,
 * without the diagonal entry when excl_diag; rounded to float. */
void orc_row_stats(const float* A, int64_t rows, int64_t cols, int64_t lda, int excl_diag, float* mean, float* sd) {
    for (int64_t i = 0; i < rows; ++i) {
        const float* r = A + i * lda;
        const int64_t N = cols - ((excl_diag && i < cols) ? 1 : 0);
        double s = 0.0;
        for (int64_t j = 0; j < cols; ++j)
            if (!(excl_diag && j == i)) s += (double)r[j];
        const double mu = N > 0 ? s / (double)N : 0.0;
        double q = 0.0;
        for (int64_t j = 0; j < cols; ++j)
            if (!(excl_diag && j == i)) {
                const double d = (double)r[j] - mu;
                q += d * d;
            }
        mean[i] = (float)mu;
        sd[i] = N > 1 ? (float)sqrt(q / (double)(N - 1)) : 0.0f;
    }
}

/* orc_row_stats with the population (N) variance, the row half of
 * compute_stouffer_tf (StandardScore<T,T,false>). */
void orc_row_stats_pop(const float* A, int64_t rows, int64_t cols, int64_t lda, float* mean, float* sd) {
    for (int64_t i = 0; i < rows; ++i) {
        const float* r = A + i * lda;
        double s = 0.0;
        for (int64_t j = 0; j < cols; ++j) s += (double)r[j];
        const double mu = cols > 0 ? s / (double)cols : 0.0;
        double q = 0.0;
        for (int64_t j = 0; j < cols; ++j) {
            const double d = (double)r[j] - mu;
            q += d * d;
        }
        mean[i] = (float)mu;
        sd[i] = cols > 0 ? (float)sqrt(q / (double)cols) : 0.0f;
    }
}

/* Population statistics of each column of a rows x cols matrix (FP64
 * two-pass, rounded to float): the column half of compute_stouffer_tf
 * (mcpnet_helper.hpp:600-614; StandardScore<T,T,false> on the transpose). */
void orc_col_stats(const float* A, int64_t rows, int64_t cols, int64_t lda, float* mean, float* sd) {
    for (int64_t j = 0; j < cols; ++j) {
        double s = 0.0;
        for (int64_t i = 0; i < rows; ++i) s += (double)A[i * lda + j];
        const double mu = rows > 0 ? s / (double)rows : 0.0;
        double q = 0.0;
        for (int64_t i = 0; i < rows; ++i) {
            const double d = (double)A[i * lda + j] - mu;
            q += d * d;
        }
        mean[j] = (float)mu;
        sd[j] = rows > 0 ? (float)sqrt(q / (double)rows) : 0.0f;
    }
}

/* compute_stouffer_tf (mcpnet_helper.hpp:589-634) given the row statistics
 * (population, over each row's cols entries) and the column statistics: the
 * z-scores in float, |sd| < FLT_EPSILON -> 0, then zscored_stouffer_kernel
 * (include/mcp/transform/stouffer.hpp:84-100): (z_row + z_col) * sqrt(1/2), or
 * with clr zscored_clr_kernel (clr.hpp:75-88): sqrt(z_row^2 + z_col^2).
 * The z matrices go to zr / zc when those are not null (rows x cols, ld cols). */
void orc_stouffer_tf(const float* A, int64_t rows, int64_t cols, int64_t lda, const float* rmean, const float* rsd,
                     const float* cmean, const float* csd, int clr, float* out, int64_t ldo, float* zr, float* zc) {
    const float isqrt2 = 0.70710678118654752440f;
    for (int64_t i = 0; i < rows; ++i)
        for (int64_t j = 0; j < cols; ++j) {
            const float x = A[i * lda + j];
            const float zi = (fabsf(rsd[i]) < FLT_EPSILON) ? 0.0f : (x - rmean[i]) / rsd[i];
            const float zj = (fabsf(csd[j]) < FLT_EPSILON) ? 0.0f : (x - cmean[j]) / csd[j];
            if (zr) zr[i * cols + j] = zi;
            if (zc) zc[i * cols + j] = zj;
            out[i * ldo + j] = clr ? sqrtf(zi * zi + zj * zj) : (zi + zj) * isqrt2;
        }
}

/* stouffer_vector_kernel (include/mcp/transform/stouffer.hpp:57-82) and
 * clr_vector_kernel (include/mcp/transform/clr.hpp:52-73) for every row, with
 * row i's statistics as aux1 and every row's as aux2; float arithmetic. */
void orc_transform(const float* A, int64_t n, int64_t lda, const float* mean, const float* sd, int clr, float* out,
                   int64_t ldo) {
    const float isqrt2 = 0.70710678118654752440f;
    for (int64_t i = 0; i < n; ++i) {
        const float denom = (fabsf(sd[i]) < FLT_EPSILON) ? 0.0f : (float)(1.0 / (double)sd[i]);
        for (int64_t j = 0; j < n; ++j) {
            const float x = A[i * lda + j];
            const float zi = (x - mean[i]) * denom;
            const float zj = (fabsf(sd[j]) < FLT_EPSILON) ? 0.0f : (x - mean[j]) / sd[j];
            out[i * ldo + j] = clr ? sqrtf(zi * zi + zj * zj) : (zi + zj) * isqrt2;
        }
    }
}
