/* CPU restatement of MCPNet's hot-path arithmetic, instantiated once per
 * precision by mcp_oracle.c (REAL = float or double, SFX = f32 or f64).
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle: tests, the smoke check and
 * the CPU-baseline leg of the benchmark call it as the checker; the product
 * never links or calls it.
 *
 * Every routine names the reference lines it restates (paths relative to the
 * MCPNet source tree).  The reference's mixed-precision details are kept:
 * where the reference multiplies a float by a double and stores into a float,
 * so does this code.
 */

#define CAT2(a, b) a##_##b
#define CAT(a, b) CAT2(a, b)
#define FN(name) CAT(name, SFX)

/* MinMaxScale::operator() -- include/mcp/correlation/BSplineMI.hpp:81-115 */
static void FN(scale_row)(const REAL* in, int64_t m, REAL* out) {
    REAL mn = m > 0 ? in[0] : (REAL)0;
    REAL mx = m > 0 ? in[0] : (REAL)0;
    for (int64_t j = 1; j < m; ++j) {
        REAL x = in[j];
        mn = (x < mn) ? x : mn; /* std::min(minX, x) */
        mx = (mx < x) ? x : mx; /* std::max(maxX, x) */
    }
    REAL scale = (mx > mn) ? (REAL)(1.0 / (double)(mx - mn)) : (REAL)1.0;
    REAL offset = (mx > mn) ? mn : (REAL)0.0;
    for (int64_t j = 0; j < m; ++j) out[j] = scale * (in[j] - offset);
}

/* buildKnotVector<KT> -- BSplineMI.hpp:35-71.  knots has bins+order entries. */
static void FN(knots)(int bins, int order, REAL* kv) {
    int nint = bins - order;
    double nf = 1.0 / (double)(nint + 1);
    int i;
    for (i = 0; i < order; ++i) kv[i] = (REAL)0;
    for (i = order; i < order + nint; ++i) kv[i] = (REAL)((double)(REAL)(i - order + 1) * nf);
    for (i = order + nint; i < 2 * order + nint; ++i) kv[i] = (REAL)1;
}

/* BSplineWeightsKernel::basisFunction (Cox-de Boor) -- BSplineMI.hpp:130-164 */
static REAL FN(basis)(const REAL* kv, int bins, int i, int p, REAL t) {
    REAL d1, n1, d2, n2, e1, e2;
    if (p == 1) {
        if ((t >= kv[i] && t < kv[i + 1] && kv[i] < kv[i + 1]) ||
            (fabs((double)(REAL)(t - kv[i + 1])) < 1e-10 && (i + 1 == bins)))
            return (REAL)1;
        return (REAL)0;
    }
    d1 = kv[i + p - 1] - kv[i];
    n1 = t - kv[i];
    d2 = kv[i + p] - kv[i + 1];
    n2 = kv[i + p] - t;
    if (d1 < 1e-10 && d2 < 1e-10) {
        return (REAL)0;
    } else if (d1 < 1e-10) {
        e1 = (REAL)0;
        e2 = n2 / d2 * FN(basis)(kv, bins, i + 1, p - 1, t);
    } else if (d2 < 1e-10) {
        e2 = (REAL)0;
        e1 = n1 / d1 * FN(basis)(kv, bins, i, p - 1, t);
    } else {
        e1 = n1 / d1 * FN(basis)(kv, bins, i, p - 1, t);
        e2 = n2 / d2 * FN(basis)(kv, bins, i + 1, p - 1, t);
    }
    if (e1 + e2 < 0) return (REAL)0;
    return e1 + e2;
}

/* BSplineWeightsKernel::operator() + entropy1d_2 -- BSplineMI.hpp:204-224,248-273.
 * Row layout per gene: w[bin*m + s] (bin-major), then w[bins*m] = H_g in bits. */
static void FN(weights_row)(const REAL* kv, const REAL* x, int64_t m, int bins, int order, REAL* w) {
    int64_t nw = (int64_t)bins * m;
    double nf = 1.0 / (double)m;
    for (int64_t i = 0; i < nw; ++i) {
        int64_t b = i / m, s = i - b * m;
        w[i] = FN(basis)(kv, bins, (int)b, order, x[s]);
    }
    REAL H = 0;
    int64_t idx = 0;
    for (int b = 0; b < bins; ++b) {
        REAL ex = 0;
        for (int64_t s = 0; s < m; ++s) { ex = (REAL)((double)ex + (double)w[idx] * nf); ++idx; }
        if (ex > 0.0) H = (REAL)((double)H + (double)ex * log2((double)ex));
    }
    w[nw] = (REAL)(0.0 - (double)H);
}

/* compute_mi steps 1-2: scale then weights -- apps/pipeline/mcpnet_helper.hpp:58-80 */
void FN(orc_bspline_weights)(const REAL* X, int64_t n, int64_t m, int64_t ldx, int bins, int order, REAL* W) {
    int64_t ldw = (int64_t)bins * m + 1;
    REAL kv[64];
    FN(knots)(bins, order, kv);
#pragma omp parallel
    {
        REAL* sc = (REAL*)malloc(sizeof(REAL) * (size_t)(m > 0 ? m : 1));
#pragma omp for schedule(dynamic, 4)
        for (int64_t g = 0; g < n; ++g) {
            FN(scale_row)(X + g * ldx, m, sc);
            FN(weights_row)(kv, sc, m, bins, order, W + g * ldw);
        }
        free(sc);
    }
}

/* BSplineEntropyKernel::entropy2d_simd + BSplineMIKernel::operator()
 * -- BSplineMI.hpp:288-315,492-499.  The splash dot product is restated as a
 * sequential accumulation in REAL (its real summation order is not in the
 * reference snapshot).  norm_factor is REAL(1)/REAL(m) (BSplineMI.hpp:321). */
static REAL FN(pair_mi)(const REAL* wx, const REAL* wy, int64_t m, int bins) {
    REAL nf = (REAL)1 / (REAL)m;
    REAL H = 0;
    for (int bx = 0; bx < bins; ++bx) {
        for (int by = 0; by < bins; ++by) {
            const REAL* a = wx + (int64_t)bx * m;
            const REAL* b = wy + (int64_t)by * m;
            REAL hx = 0;
            for (int64_t s = 0; s < m; ++s) hx += a[s] * b[s];
            hx *= nf;
            if (hx > 0.0) H = (REAL)((double)H + (double)hx * log2((double)hx));
        }
    }
    REAL e2d = (REAL)(0.0 - (double)H);
    int64_t e1 = (int64_t)bins * m;
    return wx[e1] + wy[e1] - e2d;
}

/* compute_mi step 4: InnerProduct<..., SYMM=true> -- mcpnet_helper.hpp:88-98 */
void FN(orc_bspline_mi_from_weights)(const REAL* W, int64_t n, int64_t m, int bins, REAL* MI, int64_t ldmi) {
    int64_t ldw = (int64_t)bins * m + 1;
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t i = 0; i < n; ++i)
        for (int64_t j = i; j < n; ++j) {
            REAL v = FN(pair_mi)(W + i * ldw, W + j * ldw, m, bins);
            MI[i * ldmi + j] = v;
            MI[j * ldmi + i] = v;
        }
}

void FN(orc_bspline_mi)(const REAL* X, int64_t n, int64_t m, int64_t ldx, int bins, int order, REAL* MI, int64_t ldmi) {
    int64_t ldw = (int64_t)bins * m + 1;
    REAL* W = (REAL*)malloc(sizeof(REAL) * (size_t)(n * ldw > 0 ? n * ldw : 1));
    FN(orc_bspline_weights)(X, n, m, ldx, bins, order, W);
    FN(orc_bspline_mi_from_weights)(W, n, m, bins, MI, ldmi);
    free(W);
}

/* Mutual information of the gene pairs (i, j) with i in [r0, r1), all j, into
 * MI rows r0..r1-1 (a row slab, used to time a bounded CPU sample). */
void FN(orc_bspline_mi_rows)(const REAL* W, int64_t n, int64_t m, int bins, int64_t r0, int64_t r1, REAL* MI, int64_t ldmi) {
    int64_t ldw = (int64_t)bins * m + 1;
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t i = r0; i < r1; ++i)
        for (int64_t j = 0; j < n; ++j)
            MI[(i - r0) * ldmi + j] = FN(pair_mi)(W + i * ldw, W + j * ldw, m, bins);
}

/* max_of_pairmin_scalar -- include/mcp/filter/simd_maxmin.hpp:30-46 (the float
 * dispatch at :447-450 always takes this scalar form). */
static REAL FN(max_of_pairmin)(const REAL* xx, const REAL* yy, int64_t count) {
    REAL val = (REAL)(-DBL_MAX); /* numeric_limits<double>::lowest(), -inf for float */
    for (int64_t i = 0; i < count; ++i) {
        REAL a = xx[i], b = yy[i];
        REAL mn = (b < a) ? b : a;   /* std::min(a, b) */
        val = (val < mn) ? mn : val; /* std::max(val, mn) */
    }
    return val;
}

/* mcp2_maxmin_kernel<IT,false,true> over all (i, j): C = A (x) B, the
 * InnerProduct convention C[i][j] = kernel(row A_i, row B_j) -- filter/mcp.hpp:72-93 */
void FN(orc_maxmin)(const REAL* A, int64_t lda, const REAL* B, int64_t ldb, int64_t rows, int64_t cols,
                    int64_t k, REAL* C, int64_t ldc) {
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t i = 0; i < rows; ++i)
        for (int64_t j = 0; j < cols; ++j)
            C[i * ldc + j] = FN(max_of_pairmin)(A + i * lda, B + j * ldb, k);
}

/* max_of_pairmin_scalar with a mask -- simd_maxmin.hpp:30-46 (mask branch,
 * :35-38): val = max(val, min(mask[i], min(xx[i], yy[i]))). */
static REAL FN(max_of_pairmin_masked)(const REAL* xx, const REAL* yy, const REAL* mask, int64_t count) {
    REAL val = (REAL)(-DBL_MAX);
    for (int64_t i = 0; i < count; ++i) {
        REAL a = xx[i], b = yy[i];
        REAL mn = (b < a) ? b : a;
        REAL mk = mask[i];
        REAL m2 = (mn < mk) ? mn : mk; /* std::min(mask[i], mn) */
        val = (val < m2) ? m2 : val;
    }
    return val;
}

/* mcp2_maxmin_kernel<IT,true,true> over all (i, j) -- filter/mcp.hpp:72-93 */
void FN(orc_maxmin_masked)(const REAL* A, int64_t lda, const REAL* B, int64_t ldb, int64_t rows, int64_t cols,
                           int64_t k, const REAL* mask, REAL* C, int64_t ldc) {
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t i = 0; i < rows; ++i)
        for (int64_t j = 0; j < cols; ++j)
            C[i * ldc + j] = FN(max_of_pairmin_masked)(A + i * lda, B + j * ldb, mask, k);
}

/* ratio_kernel<T,T> -- include/mcp/transform/combine.hpp:210-222 */
void FN(orc_ratio)(const REAL* A, int64_t lda, const REAL* M, int64_t ldm, int64_t rows, int64_t cols,
                   REAL* R, int64_t ldr) {
    const REAL eps = (sizeof(REAL) == 4) ? (REAL)FLT_EPSILON : (REAL)DBL_EPSILON;
    const REAL big = (sizeof(REAL) == 4) ? (REAL)FLT_MAX : (REAL)DBL_MAX;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < rows; ++i)
        for (int64_t j = 0; j < cols; ++j) {
            REAL a = A[i * lda + j], mm = M[i * ldm + j];
            R[i * ldr + j] = (fabs((double)a) < eps) ? (REAL)0
                           : (fabs((double)mm) < eps) ? big
                           : (REAL)((double)a / (double)mm);
        }
}

/* compute_combo -- apps/pipeline/mcpnet_helper.hpp:507-573: the ensemble
 * score mi / (a mi + b M1 + c M2 + d M3), the combination summed in double in
 * that order (a term skipped when its coefficient is 0, added unscaled when it
 * is 1), with ratio_kernel's epsilon guards.  M1..M3 may be NULL when their
 * coefficient is 0. */
void FN(orc_combo)(const REAL* mi, const REAL* M1, const REAL* M2, const REAL* M3, int64_t rows, int64_t cols,
                   int64_t ld, const double* cs, REAL* out, int64_t ldo) {
    const REAL eps = (sizeof(REAL) == 4) ? (REAL)FLT_EPSILON : (REAL)DBL_EPSILON;
    const REAL big = (sizeof(REAL) == 4) ? (REAL)FLT_MAX : (REAL)DBL_MAX;
    const double a = cs[0], b = cs[1], c = cs[2], d = cs[3];
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < rows; ++i)
        for (int64_t j = 0; j < cols; ++j) {
            const int64_t o = i * ld + j;
            double mm = 0.0;
            if (a == 1.0) mm += mi[o]; else if (a != 0.0) mm += a * mi[o];
            if (b == 1.0) mm += M1[o]; else if (b != 0.0) mm += b * M1[o];
            if (c == 1.0) mm += M2[o]; else if (c != 0.0) mm += c * M2[o];
            if (d == 1.0) mm += M3[o]; else if (d != 0.0) mm += d * M3[o];
            out[i * ldo + j] = (fabs((double)mi[o]) < eps) ? (REAL)0
                             : (fabs(mm) < eps) ? big
                             : (REAL)((double)mi[o] / mm);
        }
}

/* max_kernel over (M, M^T) -- combine.hpp:42-58 as used by apps/filter/mcp.cpp:463-476 */
void FN(orc_max_transpose)(const REAL* M, int64_t n, int64_t ldm, REAL* out, int64_t ldo) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i)
        for (int64_t j = 0; j < n; ++j) {
            REAL a = M[i * ldm + j], b = M[j * ldm + i];
            out[i * ldo + j] = (a < b) ? b : a;
        }
}

/* dpi_kernel<IT,true,true>::operator()(x, z, row_x, row_z, count) --
 * include/mcp/filter/dpi.hpp:56-68: delete (x, z) if x == z, or if some
 * y not in {x, z} has row_x[y] >= i_xz and row_z[y] >= i_xz, with
 * i_xz = (IT)(row_x[z] * tol_multiplier) and tol_multiplier = 1/(1 - tol) in
 * double (dpi.hpp:47). */
static int FN(dpi_delete)(const REAL* A, int64_t n, int64_t lda, double tm, int64_t x, int64_t z) {
    if (x == z) return 1;
    const REAL* rx = A + x * lda;
    const REAL* rz = A + z * lda;
    REAL ixz = (REAL)((double)rx[z] * tm);
    int64_t y = 0;
    for (; y < n && (y == x || y == z || rx[y] < ixz || rz[y] < ixz); ++y) {}
    return y < n;
}

/* The dpi app's filter: dpi_kernel over every (x, z) -- as driven by
 * apps/filter/dpi.cpp:236-287 -- followed by mask<IT,true> --
 * include/mcp/filter/threshold.hpp:33-54.  Returns the "removed" count
 * (mask.processed). */
int64_t FN(orc_dpi)(const REAL* A, int64_t n, int64_t lda, double tol, REAL* out, int64_t ldo, uint8_t* mask) {
    double tm = 1.0 / (1.0 - tol);
    int64_t removed = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(+:removed)
    for (int64_t x = 0; x < n; ++x) {
        for (int64_t z = 0; z < n; ++z) {
            int del = FN(dpi_delete)(A, n, lda, tm, x, z);
            if (mask) mask[x * n + z] = (uint8_t)del;
            REAL in = A[x * lda + z];
            REAL o = del ? (REAL)0 : in;
            out[x * ldo + z] = o;
            removed += (o != in);
        }
    }
    return removed;
}

/* orc_dpi restricted to the rows x = rows[0..nr) of the output: row r of out and
 * mask (mask row stride n) is row rows[r] of the full filter; returns the removed
 * count of these rows.  For sampled-row checks of matrices too large to filter
 * whole on the CPU. */
int64_t FN(orc_dpi_rows)(const REAL* A, int64_t n, int64_t lda, double tol, const int64_t* rows, int64_t nr,
                         REAL* out, int64_t ldo, uint8_t* mask) {
    double tm = 1.0 / (1.0 - tol);
    int64_t removed = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+:removed)
    for (int64_t q = 0; q < nr * n; ++q) {
        const int64_t r = q / n, z = q - r * n, x = rows[r];
        int del = FN(dpi_delete)(A, n, lda, tm, x, z);
        if (mask) mask[r * n + z] = (uint8_t)del;
        REAL in = A[x * lda + z];
        REAL o = del ? (REAL)0 : in;
        out[r * ldo + z] = o;
        removed += (o != in);
    }
    return removed;
}

/* dpi_tf_kernel<IT,true> -- include/mcp/filter/dpi.hpp:74-110 (note its
 * multiplier is stored in IT, so i_xz is an IT product): is (x, z) deleted?
 * tfs: the reference's TF vector (> 0 = TF). */
static int FN(dpi_tf_delete)(const REAL* A, int64_t n, int64_t lda, REAL tm, const REAL* tfs, int64_t x, int64_t z) {
    if (x == z) return 1;
    const REAL* rx = A + x * lda;
    const REAL* rz = A + z * lda;
    REAL ixz = rx[z] * tm;
    int tfxz = (tfs[x] > 0) ^ (tfs[z] > 0);
    int64_t y = 0;
    for (; y < n && (y == x || y == z || rx[y] < ixz || rz[y] < ixz || ((tfs[y] <= 0) && tfxz)); ++y) {}
    return y < n;
}

/* dpi_tf_kernel over all (x, z), then mask<IT,true> as apps/filter/dpi.cpp:276-287. */
int64_t FN(orc_dpi_tf)(const REAL* A, int64_t n, int64_t lda, REAL tol, const REAL* tfs, REAL* out, int64_t ldo,
                       uint8_t* mask) {
    const REAL tm = (REAL)(1.0 / (1.0 - (double)tol));
    int64_t removed = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(+:removed)
    for (int64_t x = 0; x < n; ++x) {
        for (int64_t z = 0; z < n; ++z) {
            int del = FN(dpi_tf_delete)(A, n, lda, tm, tfs, x, z);
            if (mask) mask[x * n + z] = (uint8_t)del;
            REAL in = A[x * lda + z];
            REAL o = del ? (REAL)0 : in;
            out[x * ldo + z] = o;
            removed += (o != in);
        }
    }
    return removed;
}

/* orc_dpi_tf restricted to the rows x = rows[0..nr) of the output (row r of out and
 * mask is row rows[r] of the full filter); returns the removed count of these rows. */
int64_t FN(orc_dpi_tf_rows)(const REAL* A, int64_t n, int64_t lda, REAL tol, const REAL* tfs, const int64_t* rows,
                            int64_t nr, REAL* out, int64_t ldo, uint8_t* mask) {
    const REAL tm = (REAL)(1.0 / (1.0 - (double)tol));
    int64_t removed = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+:removed)
    for (int64_t q = 0; q < nr * n; ++q) {
        const int64_t r = q / n, z = q - r * n, x = rows[r];
        int del = FN(dpi_tf_delete)(A, n, lda, tm, tfs, x, z);
        if (mask) mask[r * n + z] = (uint8_t)del;
        REAL in = A[x * lda + z];
        REAL o = del ? (REAL)0 : in;
        out[r * ldo + z] = o;
        removed += (o != in);
    }
    return removed;
}

/* Maximum-capacity closure by repeated squaring: B <- max(B, B (x) B) until no
 * entry changes.  The reference has no closure routine; this is the oracle of
 * the max-capacity-path form, built from the reference's max_of_pairmin
 * (simd_maxmin.hpp:30-46).  Returns the number of products computed, or -1 if
 * max_iter products left it still changing. */
int FN(orc_closure)(const REAL* A, int64_t n, int64_t lda, REAL* out, int64_t ldo, int max_iter) {
    REAL* cur = (REAL*)malloc(sizeof(REAL) * (size_t)(n * n > 0 ? n * n : 1));
    REAL* nxt = (REAL*)malloc(sizeof(REAL) * (size_t)(n * n > 0 ? n * n : 1));
    for (int64_t i = 0; i < n; ++i) memcpy(cur + i * n, A + i * lda, sizeof(REAL) * (size_t)n);
    int it = 0, changed = 1;
    while (changed && it < max_iter) {
        changed = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(|:changed)
        for (int64_t i = 0; i < n; ++i)
            for (int64_t j = 0; j < n; ++j) {
                REAL p = FN(max_of_pairmin)(cur + i * n, cur + j * n, n);
                REAL c = cur[i * n + j];
                REAL v = (c < p) ? p : c;
                nxt[i * n + j] = v;
                changed |= (v != c);
            }
        REAL* t = cur; cur = nxt; nxt = t;
        ++it;
    }
    for (int64_t i = 0; i < n; ++i) memcpy(out + i * ldo, cur + i * n, sizeof(REAL) * (size_t)n);
    free(cur); free(nxt);
    return changed ? -1 : it;
}

/* Rows rows[0..nr) of the maximum-capacity closure of a SYMMETRIC matrix, by a
 * widest-path search from each row (a bottleneck form of Dijkstra's algorithm),
 * independent of orc_closure's repeated squaring.  For x = rows[r]:
 * out[r][j] (j != x) = max over paths x -> j of the smallest entry on the path
 * (the direct entry included); out[r][x] = max(A[x][x], max over j != x of
 * out[r][j]), the value the squaring B <- max(B, B (x) B) leaves on the diagonal
 * of a symmetric matrix.  Only min and max are taken, so every output is an
 * input entry and the comparison with the squaring is exact.  O(n^2) per row. */
void FN(orc_widest_rows)(const REAL* A, int64_t n, int64_t lda, const int64_t* rows, int64_t nr, REAL* out,
                         int64_t ldo) {
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t r = 0; r < nr; ++r) {
        const int64_t x = rows[r];
        REAL* cap = out + r * ldo;
        uint8_t* done = (uint8_t*)calloc((size_t)(n > 0 ? n : 1), 1);
        for (int64_t j = 0; j < n; ++j) cap[j] = A[x * lda + j];
        done[x] = 1;
        for (int64_t it = 1; it < n; ++it) {
            int64_t u = -1;
            for (int64_t j = 0; j < n; ++j)
                if (!done[j] && (u < 0 || cap[u] < cap[j])) u = j;
            done[u] = 1;
            const REAL cu = cap[u];
            const REAL* au = A + u * lda;
            for (int64_t v = 0; v < n; ++v) {
                if (done[v]) continue;
                const REAL c = (au[v] < cu) ? au[v] : cu;
                if (cap[v] < c) cap[v] = c;
            }
        }
        REAL d = A[x * lda + x];
        for (int64_t j = 0; j < n; ++j)
            if (j != x && d < cap[j]) d = cap[j];
        cap[x] = d;
        free(done);
    }
}

/* ================= adjoints (no reference routine; oracle of this build's
 * definitions, restated in plain loops) =================
 *
 * B-spline basis derivative: d/dt N_{a,p}(t) = (p-1) [ N_{a,p-1}(t) / (t_{a+p-1} - t_a)
 *   - N_{a+1,p-1}(t) / (t_{a+p} - t_{a+1}) ], a term dropped when its knot span
 *   is below 1e-10 (the reference basis's own guard, BSplineMI.hpp:146-157). */
static REAL FN(basis_deriv)(const REAL* kv, int bins, int a, int p, REAL t) {
    if (p <= 1) return (REAL)0;
    REAL d1 = kv[a + p - 1] - kv[a], d2 = kv[a + p] - kv[a + 1];
    REAL r = 0;
    if (!(d1 < 1e-10)) r += FN(basis)(kv, bins, a, p - 1, t) / d1;
    if (!(d2 < 1e-10)) r -= FN(basis)(kv, bins, a + 1, p - 1, t) / d2;
    return (REAL)(p - 1) * r;
}

/* Gradient of L with respect to the expression X, given G = dL/dMI (n x n,
 * every ordered entry; the diagonal is ignored because the pipeline resets it).
 * MI_ij = H_i + H_j - H_ij with p_ia = (1/m) sum_s w_ia(s),
 * P_ab = (1/m) sum_s w_ia(s) w_jb(s), c = 1/ln 2:
 *   dMI_ij/dw_ia(s) = (1/m) [ -(log2 p_ia + c) + sum_b (log2 P_ab + c) w_jb(s) ]
 * (cells with p = 0 contribute 0), then w = N(t), t = (x - min)/(max - min)
 * including the dependence of min and max (first arg-min / arg-max sample). */
void FN(orc_mi_bwd)(const REAL* X, int64_t n, int64_t m, int64_t ldx, int bins, int order, const REAL* G,
                    int64_t ldg, REAL* dX, int64_t lddx) {
    const double c = 1.0 / log(2.0);
    REAL kv[64];
    FN(knots)(bins, order, kv);
    const int64_t ldw = (int64_t)bins * m;
    REAL* T = (REAL*)malloc(sizeof(REAL) * (size_t)(n * m));
    REAL* W = (REAL*)malloc(sizeof(REAL) * (size_t)(n * ldw));
    REAL* Hc = (REAL*)malloc(sizeof(REAL) * (size_t)(n * bins));
    REAL* gsum = (REAL*)malloc(sizeof(REAL) * (size_t)n);
#pragma omp parallel for schedule(static)
    for (int64_t g = 0; g < n; ++g) {
        FN(scale_row)(X + g * ldx, m, T + g * m);
        for (int a = 0; a < bins; ++a) {
            double p = 0;
            for (int64_t s = 0; s < m; ++s) {
                REAL w = FN(basis)(kv, bins, a, order, T[g * m + s]);
                W[g * ldw + a * m + s] = w;
                p += w;
            }
            p /= (double)m;
            Hc[g * bins + a] = p > 0 ? (REAL)(log2(p) + c) : (REAL)0;
        }
        double gs = 0;
        for (int64_t j = 0; j < n; ++j)
            if (j != g) gs += (double)G[g * ldg + j] + (double)G[j * ldg + g];
        gsum[g] = (REAL)gs;
    }
#pragma omp parallel
    {
        REAL* dW = (REAL*)malloc(sizeof(REAL) * (size_t)ldw);
        REAL* Q = (REAL*)malloc(sizeof(REAL) * (size_t)(bins * bins));
#pragma omp for schedule(dynamic, 1)
        for (int64_t i = 0; i < n; ++i) {
            const REAL* wi = W + i * ldw;
            for (int a = 0; a < bins; ++a)
                for (int64_t s = 0; s < m; ++s) dW[a * m + s] = -Hc[i * bins + a] * gsum[i];
            for (int64_t j = 0; j < n; ++j) {
                if (j == i) continue;
                const REAL gs = G[i * ldg + j] + G[j * ldg + i];
                if (gs == 0) continue;
                const REAL* wj = W + j * ldw;
                for (int a = 0; a < bins; ++a)
                    for (int b = 0; b < bins; ++b) {
                        double P = 0;
                        for (int64_t s = 0; s < m; ++s) P += (double)wi[a * m + s] * wj[b * m + s];
                        P /= (double)m;
                        Q[a * bins + b] = P > 0 ? (REAL)(gs * (log2(P) + c)) : (REAL)0;
                    }
                for (int a = 0; a < bins; ++a)
                    for (int b = 0; b < bins; ++b) {
                        const REAL q = Q[a * bins + b];
                        if (q == 0) continue;
                        for (int64_t s = 0; s < m; ++s) dW[a * m + s] += q * wj[b * m + s];
                    }
            }
            /* through the weights, the scaling and its min / max */
            const REAL* x = X + i * ldx;
            int64_t amin = 0, amax = 0;
            for (int64_t s = 1; s < m; ++s) {
                if (x[s] < x[amin]) amin = s;
                if (x[amax] < x[s]) amax = s;
            }
            const REAL mn = x[amin], mx = x[amax];
            const int ranged = mx > mn;
            const REAL scale = ranged ? (REAL)(1.0 / (double)(mx - mn)) : (REAL)1;
            double s1 = 0, s2 = 0;
            for (int64_t s = 0; s < m; ++s) {
                const REAL t = T[i * m + s];
                double dt = 0;
                for (int a = 0; a < bins; ++a) dt += (double)dW[a * m + s] * FN(basis_deriv)(kv, bins, a, order, t);
                dt /= (double)m;
                dX[i * lddx + s] = (REAL)(scale * dt);
                s1 += dt * ((double)t - 1.0);
                s2 += dt * (double)t;
            }
            if (ranged) {
                dX[i * lddx + amin] += (REAL)(scale * s1);
                dX[i * lddx + amax] -= (REAL)(scale * s2);
            }
        }
        free(dW);
        free(Q);
    }
    free(T); free(W); free(Hc); free(gsum);
}

/* Adjoint of C = A (x) B (C[i][j] = max_k min(A[i][k], B[j][k])): for every
 * (i, j) with dC != 0, the witness k* is the first k with min(A[i][k], B[j][k])
 * == C[i][j]; the gradient goes to A[i][k*] when A[i][k*] <= B[j][k*] (the
 * operand std::min returns on a tie), else to B[j][k*].  Accumulates into dA,
 * dB (which may alias when A and B are the same matrix).  Where C is -inf there
 * is no witness (-1) and no gradient.  Sequential, so the sums are
 * deterministic. */
void FN(orc_maxmin_bwd)(const REAL* A, int64_t lda, const REAL* B, int64_t ldb, int64_t rows, int64_t cols,
                        int64_t k, const REAL* Cm, int64_t ldc, const REAL* dC, int64_t lddc, REAL* dA, int64_t ldda,
                        REAL* dB, int64_t lddb, int32_t* witness) {
    for (int64_t i = 0; i < rows; ++i)
        for (int64_t j = 0; j < cols; ++j) {
            const REAL g = dC[i * lddc + j];
            if (!witness && g == 0) continue;  /* nothing to route and no witness asked for */
            int64_t ks = -1;
            /* no witness (and no gradient) where the product is -inf */
            for (int64_t q = 0; q < k && Cm[i * ldc + j] > (REAL)(-DBL_MAX); ++q) {
                REAL a = A[i * lda + q], b = B[j * ldb + q];
                REAL mn = (b < a) ? b : a;
                if (mn == Cm[i * ldc + j]) { ks = q; break; }
            }
            if (witness) witness[i * cols + j] = (int32_t)ks;
            if (g == 0 || ks < 0) continue;
            if (A[i * lda + ks] <= B[j * ldb + ks]) dA[i * ldda + ks] += g;
            else dB[j * lddb + ks] += g;
        }
}

/* Adjoint of R = ratio(A, M) (combine.hpp:210-222): where both |a| and |m| are
 * at least epsilon, dA += dR / m and dM -= dR * a / m^2; elsewhere R is constant. */
void FN(orc_ratio_bwd)(const REAL* A, int64_t lda, const REAL* M, int64_t ldm, int64_t rows, int64_t cols,
                       const REAL* dR, int64_t lddr, REAL* dA, int64_t ldda, REAL* dM, int64_t lddm) {
    const REAL eps = (sizeof(REAL) == 4) ? (REAL)FLT_EPSILON : (REAL)DBL_EPSILON;
    for (int64_t i = 0; i < rows; ++i)
        for (int64_t j = 0; j < cols; ++j) {
            const REAL a = A[i * lda + j], mm = M[i * ldm + j], g = dR[i * lddr + j];
            if (fabs((double)a) < eps || fabs((double)mm) < eps) continue;
            dA[i * ldda + j] += g / mm;
            dM[i * lddm + j] -= g * a / (mm * mm);
        }
}

#undef FN
#undef CAT
#undef CAT2
