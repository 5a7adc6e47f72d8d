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
