// C ABI: max-min products and their compositions -- MCP2/3/4 with their ratios
// (mcpnet_helper.hpp:188-365), the DPI filter (apps/filter/dpi.cpp:236-287), the
// max-capacity closure, the TF-restricted variants (mcpnet_helper.hpp:209-505,
// include/mcp/filter/dpi.hpp:74-110) and the max-min / ratio adjoints.
#include "api_internal.h"

#ifndef MCPG_DPI_K0
#define MCPG_DPI_K0 512
#endif

namespace {

using namespace mcpg_api;

int maxmin_dev(mcpg_handle* h, const float* A, int64_t lda, const float* B, int64_t ldb, int64_t rows, int64_t cols,
               int64_t k, float* C, int64_t ldc) {
    if (rows < 0 || cols < 0 || k < 0) return fail(h, MCPG_ERR_ARG, "maxmin: negative size");
    if (rows == 0 || cols == 0) return MCPG_OK;
    if (!A || !B || !C) return fail(h, MCPG_ERR_ARG, "maxmin: null pointer");
    if (lda < k || ldb < k || ldc < cols) return fail(h, MCPG_ERR_ARG, "maxmin: leading dimension too small");
    const bool symm = (A == B) && (lda == ldb) && (rows == cols);
    const float *a, *b;
    int64_t la, lb;
    int rc = aligned_view(h, A, lda, rows, k, S_IN0, &a, &la);
    if (rc) return rc;
    if (symm) {
        b = a;
        lb = la;
    } else {
        rc = aligned_view(h, B, ldb, cols, k, S_IN1, &b, &lb);
        if (rc) return rc;
    }
    mcpg::MaxminParams p{};
    p.A = a; p.lda = la; p.B = b; p.ldb = lb;
    p.rows = rows; p.cols = cols; p.k_len = k;
    p.C = C; p.ldc = ldc;
    {
        PROF(h, "maxmin");
        CK(h, mcpg::launch_maxmin(p, mcpg::MM_PLAIN, symm ? 1 : 0, h->stream, &h->launches), "maxmin kernel");
    }
    return MCPG_OK;
}

int mcp_dev(mcpg_handle* h, const float* A, int64_t n, int64_t lda, int path_len, int symmetrize, float* Mout,
            int64_t ldm, float* Rout, int64_t ldr) {
    if (n < 0) return fail(h, MCPG_ERR_ARG, "mcp: negative size");
    if (n == 0) return MCPG_OK;
    if (!A) return fail(h, MCPG_ERR_ARG, "mcp: null input");
    if (path_len < 2 || path_len > 4) return fail(h, MCPG_ERR_ARG, "mcp: path_len must be 2, 3 or 4 (got %d)", path_len);
    if (!Mout && !Rout) return MCPG_OK;
    if (lda < n || (Mout && ldm < n) || (Rout && ldr < n)) return fail(h, MCPG_ERR_ARG, "mcp: leading dimension too small");
    const float* a;
    int64_t la;
    int rc = aligned_view(h, A, lda, n, n, S_IN0, &a, &la);
    if (rc) return rc;
    const int64_t ldt = round_up(n, 32);
    mcpg::MaxminParams p{};
    p.rows = n; p.cols = n; p.k_len = n;
    if (path_len == 2) {
        p.A = a; p.lda = la; p.B = a; p.ldb = la;
        p.C = Mout; p.ldc = ldm; p.E = a; p.lde = la; p.R = Rout; p.ldr = ldr;
        if (Rout) {
            {
                PROF(h, "maxmin");
                CK(h, mcpg::launch_maxmin(p, mcpg::MM_RATIO, 1, h->stream, &h->launches), "maxmin+ratio kernel");
            }
        } else {
            {
                PROF(h, "maxmin");
                CK(h, mcpg::launch_maxmin(p, mcpg::MM_PLAIN, 1, h->stream, &h->launches), "maxmin kernel");
            }
        }
        return MCPG_OK;
    }
    // M1 = A (x) A (symmetric)
    void* m1;
    rc = scratch(h, S_M1, (size_t)(n * ldt) * sizeof(float), &m1);
    if (rc) return rc;
    p.A = a; p.lda = la; p.B = a; p.ldb = la; p.C = (float*)m1; p.ldc = ldt;
    {
        PROF(h, "maxmin");
        CK(h, mcpg::launch_maxmin(p, mcpg::MM_PLAIN, 1, h->stream, &h->launches), "maxmin kernel (M1)");
    }
    const float* X1 = (const float*)m1;
    mcpg::MaxminParams q{};
    q.rows = n; q.cols = n; q.k_len = n;
    int sym2;
    if (path_len == 3) {  // A (x) M1, InnerProduct(A, M1), not assumed symmetric
        q.A = a; q.lda = la; q.B = X1; q.ldb = ldt; sym2 = 0;
    } else {              // M1 (x) M1, symmetric
        q.A = X1; q.lda = ldt; q.B = X1; q.ldb = ldt; sym2 = 1;
    }
    if (path_len == 3 && symmetrize) {
        void* m2;
        rc = scratch(h, S_M2, (size_t)(n * ldt) * sizeof(float), &m2);
        if (rc) return rc;
        q.C = (float*)m2; q.ldc = ldt;
        {
            PROF(h, "maxmin");
            CK(h, mcpg::launch_maxmin(q, mcpg::MM_PLAIN, sym2, h->stream, &h->launches), "maxmin kernel (M2)");
        }
        float* sym = Mout;
        int64_t lds = ldm;
        if (!sym) {  // reuse M1's slot: M1 is no longer needed
            sym = (float*)m1;
            lds = ldt;
        }
        {
            PROF(h, "max_transpose");
            CK(h, mcpg::launch_max_transpose((const float*)m2, n, ldt, sym, lds, h->stream, &h->launches),
           "max(M, M^T) kernel");
        }
        if (Rout) {
            PROF(h, "ratio");
            CK(h, mcpg::launch_ratio(a, la, sym, lds, n, n, Rout, ldr, h->stream, &h->launches), "ratio kernel");
        }
        return MCPG_OK;
    }
    q.C = Mout; q.ldc = ldm; q.E = a; q.lde = la; q.R = Rout; q.ldr = ldr;
    if (Rout) {
        {
            PROF(h, "maxmin");
            CK(h, mcpg::launch_maxmin(q, mcpg::MM_RATIO, sym2, h->stream, &h->launches), "maxmin+ratio kernel");
        }
    } else {
        {
            PROF(h, "maxmin");
            CK(h, mcpg::launch_maxmin(q, mcpg::MM_PLAIN, sym2, h->stream, &h->launches), "maxmin kernel");
        }
    }
    return MCPG_OK;
}

// Intermediates of the first phase of the two-phase DPI (a multiple of the max-min
// kernel's 64-wide k slices).
constexpr int64_t DPI_K0 = MCPG_DPI_K0;

int dpi_dev(mcpg_handle* h, const float* A, int64_t n, int64_t lda, float tol, float* out, int64_t ldo, uint8_t* mask,
            int64_t* removed) {
    if (n < 0) return fail(h, MCPG_ERR_ARG, "dpi: negative size");
    if (removed) *removed = 0;
    if (n == 0) return MCPG_OK;
    if (!A || !out) return fail(h, MCPG_ERR_ARG, "dpi: null pointer");
    if (lda < n || ldo < n) return fail(h, MCPG_ERR_ARG, "dpi: leading dimension too small");
    if (!(tol >= 0.0f && tol <= 1.0f)) return fail(h, MCPG_ERR_ARG, "dpi: tolerance must be in [0, 1]");
    const float* a = A;
    int64_t la = lda;
    // the output must not alias the input (other tiles still read it)
    const bool alias = (const void*)out < (const void*)(A + n * lda) && (const void*)A < (const void*)(out + n * ldo);
    if (alias || !aligned16(A) || (lda % 4) != 0) {
        const int64_t ld = round_up(n, 32);
        void* p;
        int rc = scratch(h, S_IN0, (size_t)(n * ld) * sizeof(float), &p);
        if (rc) return rc;
        CK(h, mcpg::launch_copy2d(A, lda, (float*)p, ld, n, n, h->stream), "copy2d");
        a = (const float*)p;
        la = ld;
    }
    void* cnt;
    int rc = scratch(h, S_SMALL, 64, &cnt);
    if (rc) return rc;
    unsigned long long* cnt_removed = (unsigned long long*)cnt;
    unsigned long long* cnt_pending = cnt_removed + 1;
    CK(h, cudaMemsetAsync(cnt, 0, 2 * sizeof(unsigned long long), h->stream), "memset counters");
    mcpg::MaxminParams p{};
    p.A = a; p.lda = la; p.B = a; p.ldb = la; p.rows = n; p.cols = n; p.k_len = n;
    p.C = out; p.ldc = ldo; p.E = a; p.lde = la;
    p.tol_mult = 1.0 / (1.0 - (double)tol);  // dpi_kernel ctor, dpi.hpp:47
    p.mask = mask; p.ldmask = n;
    p.removed = cnt_removed;
    // Two phases for larger matrices: the tiled max-min over the first DPI_K0
    // intermediates decides most outputs (on MI matrices ~98 % are deleted by then);
    // the rest continue the scan one warp per output pair with the reference's early
    // exit.  If more outputs stay undecided than the pending list holds, the one-phase
    // product runs instead.  Both give the same bits.
    bool done = false;
    if (n > 2 * DPI_K0) {
        const int64_t cap = std::max<int64_t>(int64_t(1) << 16, n * n / 32);
        void* pend;
        if ((rc = scratch(h, S_DPI_PEND, (size_t)cap * sizeof(mcpg::DpiPending), &pend))) return rc;
        mcpg::MaxminParams p1 = p;
        p1.k_len = DPI_K0;
        p1.pending = (mcpg::DpiPending*)pend;
        p1.pending_cap = cap;
        p1.pending_n = cnt_pending;
        {
            PROF(h, "maxmin");
            CK(h, mcpg::launch_maxmin(p1, mcpg::MM_DPI1, 1, h->stream, &h->launches), "DPI kernel (first phase)");
        }
        unsigned long long np = 0;
        CK(h, cudaMemcpyAsync(&np, cnt_pending, sizeof np, cudaMemcpyDeviceToHost, h->stream), "read pending");
        CK(h, cudaStreamSynchronize(h->stream), "stream synchronize");
        if (np <= (unsigned long long)cap) {
            PROF(h, "dpi_pending");
            CK(h, mcpg::launch_dpi_pending(a, la, n, DPI_K0, p1.pending, (int64_t)np, p.tol_mult, out, ldo, mask, n,
                                           cnt_removed, h->stream, &h->launches),
               "DPI kernel (second phase)");
            done = true;
        } else {
            CK(h, cudaMemsetAsync(cnt_removed, 0, sizeof(unsigned long long), h->stream), "memset counter");
        }
    }
    if (!done) {
        PROF(h, "maxmin");
        CK(h, mcpg::launch_maxmin(p, mcpg::MM_DPI, 1, h->stream, &h->launches), "DPI kernel");
    }
    if (removed) {
        unsigned long long r = 0;
        CK(h, cudaMemcpyAsync(&r, cnt, sizeof r, cudaMemcpyDeviceToHost, h->stream), "read removed");
        CK(h, cudaStreamSynchronize(h->stream), "stream synchronize");
        *removed = (int64_t)r;
    }
    return MCPG_OK;
}

int closure_dev(mcpg_handle* h, const float* A, int64_t n, int64_t lda, int max_iter, float* out, int64_t ldo,
                int* iterations) {
    if (iterations) *iterations = 0;
    if (n < 0 || max_iter < 0) return fail(h, MCPG_ERR_ARG, "closure: negative size or max_iter");
    if (n == 0) return MCPG_OK;
    if (!A || !out) return fail(h, MCPG_ERR_ARG, "closure: null pointer");
    if (lda < n || ldo < n) return fail(h, MCPG_ERR_ARG, "closure: leading dimension too small");
    const int64_t ldt = round_up(n, 32);
    void *b0, *b1, *flag;
    int rc = scratch(h, S_M1, (size_t)(n * ldt) * sizeof(float), &b0);
    if (rc) return rc;
    rc = scratch(h, S_M2, (size_t)(n * ldt) * sizeof(float), &b1);
    if (rc) return rc;
    rc = scratch(h, S_SMALL, 64, &flag);
    if (rc) return rc;
    CK(h, mcpg::launch_copy2d(A, lda, (float*)b0, ldt, n, n, h->stream), "copy2d");
    float* cur = (float*)b0;
    float* nxt = (float*)b1;
    int it = 0, changed = 1;
    while (changed && it < max_iter) {
        CK(h, cudaMemsetAsync(flag, 0, sizeof(int), h->stream), "memset flag");
        mcpg::MaxminParams p{};
        p.A = cur; p.lda = ldt; p.B = cur; p.ldb = ldt; p.rows = n; p.cols = n; p.k_len = n;
        p.C = nxt; p.ldc = ldt; p.E = cur; p.lde = ldt; p.changed = (int*)flag;
        {
            PROF(h, "maxmin");
            CK(h, mcpg::launch_maxmin(p, mcpg::MM_CLOSURE, 1, h->stream, &h->launches), "closure kernel");
        }
        CK(h, cudaMemcpyAsync(&changed, flag, sizeof(int), cudaMemcpyDeviceToHost, h->stream), "read flag");
        CK(h, cudaStreamSynchronize(h->stream), "stream synchronize");
        float* t = cur; cur = nxt; nxt = t;
        ++it;
    }
    CK(h, mcpg::launch_copy2d(cur, ldt, out, ldo, n, n, h->stream), "copy2d");
    if (iterations) *iterations = it;
    if (changed) return fail(h, MCPG_ERR_NOT_CONVERGED, "closure: still changing after %d products", it);
    return MCPG_OK;
}

// mcp2_maxmin_kernel<float,true,true> (mcp.hpp:72-93) as a whole-matrix call:
// C[i][j] = max_k min(mask[k], min(A[i][k], B[j][k])), mask on the host.
// A pure TF mask (+-inf) restricts k to the TF columns (gathered, exact); any
// other mask is folded into A: min(mask, min(a, b)) == min(min(a, mask), b).
int maxmin_masked_dev(mcpg_handle* h, const float* A, int64_t lda, const float* B, int64_t ldb, int64_t rows,
                      int64_t cols, int64_t k, const float* mask, float* C, int64_t ldc) {
    if (rows < 0 || cols < 0 || k < 0) return fail(h, MCPG_ERR_ARG, "maxmin_masked: negative size");
    if (rows == 0 || cols == 0) return MCPG_OK;
    if (!A || !B || !C || (k > 0 && !mask)) return fail(h, MCPG_ERR_ARG, "maxmin_masked: null pointer");
    if (lda < k || ldb < k || ldc < cols) return fail(h, MCPG_ERR_ARG, "maxmin_masked: leading dimension too small");
    const bool same = (A == B) && (lda == ldb) && (rows == cols);
    TfSet ts = tf_set(mask, k);
    mcpg::MaxminParams p{};
    p.rows = rows; p.cols = cols; p.C = C; p.ldc = ldc;
    if (ts.pm_inf) {
        const int64_t t = (int64_t)ts.idx.size();
        const int64_t ldt = round_up(t > 0 ? t : 1, 4);
        void *idx, *a, *b;
        int rc;
        if ((rc = upload(h, S_TFIDX, ts.idx.data(), ts.idx.size() * sizeof(int), &idx))) return rc;
        if ((rc = scratch(h, S_TFA, (size_t)(rows * ldt) * sizeof(float), &a))) return rc;
        CK(h, mcpg::launch_gather(A, lda, nullptr, (const int*)idx, rows, t, (float*)a, ldt, h->stream, &h->launches),
           "gather kernel");
        if (same) {
            b = a;
        } else {
            if ((rc = scratch(h, S_TFB, (size_t)(cols * ldt) * sizeof(float), &b))) return rc;
            CK(h, mcpg::launch_gather(B, ldb, nullptr, (const int*)idx, cols, t, (float*)b, ldt, h->stream,
                                      &h->launches),
               "gather kernel");
        }
        p.A = (const float*)a; p.lda = ldt; p.B = (const float*)b; p.ldb = ldt; p.k_len = t;
    } else {
        const int64_t ldk = round_up(k, 4);
        void *mk, *a;
        int rc;
        if ((rc = upload(h, S_TFIDX, mask, (size_t)k * sizeof(float), &mk))) return rc;
        if ((rc = scratch(h, S_TFA, (size_t)(rows * ldk) * sizeof(float), &a))) return rc;
        CK(h, mcpg::launch_fold_mask(A, lda, (const float*)mk, rows, k, (float*)a, ldk, h->stream, &h->launches),
           "fold_mask kernel");
        const float* bb;
        int64_t lb;
        if ((rc = aligned_view(h, B, ldb, cols, k, S_TFB, &bb, &lb))) return rc;
        p.A = (const float*)a; p.lda = ldk; p.B = bb; p.ldb = lb; p.k_len = k;
    }
    {
        PROF(h, "maxmin");
        CK(h, mcpg::launch_maxmin(p, mcpg::MM_PLAIN, (same && ts.pm_inf) ? 1 : 0, h->stream, &h->launches),
           "maxmin kernel");
    }
    return MCPG_OK;
}

// compute_mcp{2,3,4}_tfs (mcpnet_helper.hpp:209-243, 281-333, 367-434):
// outputs are t x n (t = number of TFs, rows in gene order).
int mcp_tf_dev(mcpg_handle* h, const float* A, int64_t n, int64_t lda, const float* tfs, int path_len,
               int transition, float* Mout, int64_t ldm, float* Rout, int64_t ldr) {
    if (n < 0) return fail(h, MCPG_ERR_ARG, "mcp_tf: negative size");
    if (n == 0) return MCPG_OK;
    if (!A || !tfs) return fail(h, MCPG_ERR_ARG, "mcp_tf: null pointer");
    if (path_len < 2 || path_len > 4) return fail(h, MCPG_ERR_ARG, "mcp_tf: path_len must be 2, 3 or 4");
    const int tmax = path_len == 2 ? 1 : (path_len == 3 ? 2 : 3);
    if (transition < 0 || transition > tmax)
        return fail(h, MCPG_ERR_ARG, "mcp_tf: tf_gene_transition %d out of range 0..%d for path length %d",
                    transition, tmax, path_len);
    if (lda < n || (Mout && ldm < n) || (Rout && ldr < n)) return fail(h, MCPG_ERR_ARG, "mcp_tf: leading dimension too small");
    TfSet ts = tf_set(tfs, n);
    const int64_t t = (int64_t)ts.idx.size();
    if (t == 0 || (!Mout && !Rout)) return MCPG_OK;
    const int64_t ldt = round_up(n, 32);
    int rc;
    void *idx, *tg;
    if ((rc = upload(h, S_TFEX, ts.idx.data(), (size_t)t * sizeof(int), &idx))) return rc;
    if ((rc = scratch(h, S_TFROWS, (size_t)(t * ldt) * sizeof(float), &tg))) return rc;
    CK(h, mcpg::launch_gather(A, lda, (const int*)idx, nullptr, t, n, (float*)tg, ldt, h->stream, &h->launches),
       "gather kernel");
    const float* TG = (const float*)tg;
    auto prod = [&](const float* X, int64_t ldx, int64_t rx, const float* Y, int64_t ldy, int64_t ry, bool masked,
                    float* out, int64_t ldo) -> int {
        if (masked) return maxmin_masked_dev(h, X, ldx, Y, ldy, rx, ry, n, tfs, out, ldo);
        return maxmin_dev(h, X, ldx, Y, ldy, rx, ry, n, out, ldo);
    };
    float* M = Mout;
    int64_t lm = ldm;
    void* mbuf = nullptr;
    if (!M) {
        if ((rc = scratch(h, S_M3, (size_t)(t * ldt) * sizeof(float), &mbuf))) return rc;
        M = (float*)mbuf;
        lm = ldt;
    }
    if (path_len == 2) {
        if ((rc = prod(TG, ldt, t, A, lda, n, transition == 1, M, lm))) return rc;
    } else {
        void* m1;
        if ((rc = scratch(h, S_M1, (size_t)(n * ldt) * sizeof(float), &m1))) return rc;
        const bool m1_masked = (path_len == 3) ? (transition == 2) : (transition == 3);
        if ((rc = prod(A, lda, n, A, lda, n, m1_masked, (float*)m1, ldt))) return rc;
        if (path_len == 3) {
            if ((rc = prod(TG, ldt, t, (const float*)m1, ldt, n, transition == 1 || transition == 2, M, lm))) return rc;
        } else {
            void* m2;
            if ((rc = scratch(h, S_M2, (size_t)(t * ldt) * sizeof(float), &m2))) return rc;
            if ((rc = prod(TG, ldt, t, A, lda, n, transition != 0, (float*)m2, ldt))) return rc;
            if ((rc = prod((const float*)m2, ldt, t, (const float*)m1, ldt, n, transition == 2 || transition == 3, M,
                           lm)))
                return rc;
        }
    }
    if (Rout) {
        PROF(h, "ratio");
        CK(h, mcpg::launch_ratio(TG, ldt, M, lm, t, n, Rout, ldr, h->stream, &h->launches), "ratio kernel");
    }
    return MCPG_OK;
}

// compute_maxmins_tfs (mcpnet_helper.hpp:470-505): with T the TF rows of A
// (t x n, gene order) and (x)m the TF-masked product,
//   M1 = T (x)m A,  M2 = M1 (x)m A,  M3 = M1 (x)m (A (x)m A).
// Every output is t x n and nullable (M1 is kept in scratch when M2 or M3 needs
// it); T_out, when given, gets T.
int maxmins_tf_dev(mcpg_handle* h, const float* A, int64_t n, int64_t lda, const float* tfs, float* T_out,
                   int64_t ldto, float* M1, int64_t ld1, float* M2, int64_t ld2, float* M3, int64_t ld3) {
    if (n < 0) return fail(h, MCPG_ERR_ARG, "maxmins_tf: negative size");
    if (n == 0) return MCPG_OK;
    if (!A || !tfs) return fail(h, MCPG_ERR_ARG, "maxmins_tf: null pointer");
    if (lda < n || (T_out && ldto < n) || (M1 && ld1 < n) || (M2 && ld2 < n) || (M3 && ld3 < n))
        return fail(h, MCPG_ERR_ARG, "maxmins_tf: leading dimension too small");
    TfSet ts = tf_set(tfs, n);
    const int64_t t = (int64_t)ts.idx.size();
    if (t == 0) return MCPG_OK;
    const int64_t ldt = round_up(n, 32);
    int rc;
    void *idx, *tg;
    if ((rc = upload(h, S_TFEX, ts.idx.data(), (size_t)t * sizeof(int), &idx))) return rc;
    if ((rc = scratch(h, S_TFROWS, (size_t)(t * ldt) * sizeof(float), &tg))) return rc;
    CK(h, mcpg::launch_gather(A, lda, (const int*)idx, nullptr, t, n, (float*)tg, ldt, h->stream, &h->launches),
       "gather kernel");
    const float* TG = (const float*)tg;
    if (T_out) CK(h, mcpg::launch_copy2d(TG, ldt, T_out, ldto, t, n, h->stream), "copy2d");
    if (!M1 && !M2 && !M3) return MCPG_OK;
    float* m1 = M1;
    int64_t l1 = ld1;
    if (!m1) {
        void* p;
        if ((rc = scratch(h, S_M3, (size_t)(t * ldt) * sizeof(float), &p))) return rc;
        m1 = (float*)p;
        l1 = ldt;
    }
    if ((rc = maxmin_masked_dev(h, TG, ldt, A, lda, t, n, n, tfs, m1, l1))) return rc;   // ttg
    if (M2 && (rc = maxmin_masked_dev(h, m1, l1, A, lda, t, n, n, tfs, M2, ld2))) return rc;  // tttg
    if (M3) {
        void* g2;  // gtg = A (x)m A, symmetric
        if ((rc = scratch(h, S_M1, (size_t)(n * ldt) * sizeof(float), &g2))) return rc;
        if ((rc = maxmin_masked_dev(h, A, lda, A, lda, n, n, n, tfs, (float*)g2, ldt))) return rc;
        if ((rc = maxmin_masked_dev(h, m1, l1, (const float*)g2, ldt, t, n, n, tfs, M3, ld3))) return rc;  // ttttg
    }
    return MCPG_OK;
}

// dpi_tf_kernel (dpi.hpp:74-110) over all (x, z), then mask<float,true>: two phases on the
// TF-first permutation where they apply, else the all-y and TF-y products and one apply pass.
int dpi_tf_dev(mcpg_handle* h, const float* A, int64_t n, int64_t lda, float tol, const float* tfs, float* out,
               int64_t ldo, uint8_t* mask, int64_t* removed) {
    if (n < 0) return fail(h, MCPG_ERR_ARG, "dpi_tf: negative size");
    if (removed) *removed = 0;
    if (n == 0) return MCPG_OK;
    if (!A || !out || !tfs) return fail(h, MCPG_ERR_ARG, "dpi_tf: null pointer");
    if (lda < n || ldo < n) return fail(h, MCPG_ERR_ARG, "dpi_tf: leading dimension too small");
    if (!(tol >= 0.0f && tol <= 1.0f)) return fail(h, MCPG_ERR_ARG, "dpi_tf: tolerance must be in [0, 1]");
    const int64_t ldt = round_up(n, 32);
    int rc;
    const float* a = A;
    int64_t la = lda;
    const bool alias = (const void*)out < (const void*)(A + n * lda) && (const void*)A < (const void*)(out + n * ldo);
    if (alias || !aligned16(A) || (lda % 4) != 0) {
        void* p;
        if ((rc = scratch(h, S_IN0, (size_t)(n * ldt) * sizeof(float), &p))) return rc;
        CK(h, mcpg::launch_copy2d(A, lda, (float*)p, ldt, n, n, h->stream), "copy2d");
        a = (const float*)p;
        la = ldt;
    }
    TfSet ts = tf_set(tfs, n);
    const int64_t t = (int64_t)ts.idx.size();
    const float tm = (float)(1.0 / (1.0 - (double)tol));  // dpi_tf_kernel stores it as IT
    // Two phases on B = P A P^T with the t TFs first (P: TFs ascending, then the rest).
    // In that order the x, z exclusion is the diagonal again, a pair of one TF and one
    // non-TF admits exactly the intermediates y < t, any other pair all y; the deletion
    // test is an existential one, so the order of the y does not change it.  The first
    // phase scans the first K1 = min(DPI_K0, t) intermediates, TFs only, which are
    // admissible for every pair; the pending scan continues each undecided pair to its
    // own end (t or n).  Outputs go back through P.  On pending-list overflow the
    // product form below runs and rewrites every output.
    if (n > 2 * DPI_K0 && t >= 128) {
        std::vector<int> perm;
        perm.reserve((size_t)n);
        {
            std::vector<uint8_t> is_tf((size_t)n, 0);
            for (int i : ts.idx) is_tf[(size_t)i] = 1;
            for (int64_t g = 0; g < n; ++g)
                if (is_tf[(size_t)g]) perm.push_back((int)g);
            for (int64_t g = 0; g < n; ++g)
                if (!is_tf[(size_t)g]) perm.push_back((int)g);
        }
        void *pd, *bp, *pend, *cnt;
        if ((rc = upload(h, S_TFIDX, perm.data(), (size_t)n * sizeof(int), &pd))) return rc;
        if ((rc = scratch(h, S_M1, (size_t)(n * ldt) * sizeof(float), &bp))) return rc;
        CK(h, mcpg::launch_gather(a, la, (const int*)pd, (const int*)pd, n, n, (float*)bp, ldt, h->stream,
                                  &h->launches),
           "gather kernel (TF-first order)");
        const int64_t cap = std::max<int64_t>(int64_t(1) << 16, n * n / 32);
        if ((rc = scratch(h, S_DPI_PEND, (size_t)cap * sizeof(mcpg::DpiPending), &pend))) return rc;
        if ((rc = scratch(h, S_SMALL, 64, &cnt))) return rc;
        unsigned long long* cnt_removed = (unsigned long long*)cnt;
        CK(h, cudaMemsetAsync(cnt, 0, 2 * sizeof(unsigned long long), h->stream), "memset counters");
        const int64_t k1 = std::min<int64_t>(DPI_K0, t & ~int64_t(3));
        mcpg::MaxminParams p1{};
        p1.A = (const float*)bp; p1.lda = ldt; p1.B = (const float*)bp; p1.ldb = ldt;
        p1.rows = n; p1.cols = n; p1.k_len = k1;
        p1.C = out; p1.ldc = ldo; p1.E = (const float*)bp; p1.lde = ldt;
        p1.tm_float = 1; p1.tol_mult_f = tm; p1.perm = (const int*)pd;
        p1.mask = mask; p1.ldmask = n;
        p1.removed = cnt_removed;
        p1.pending = (mcpg::DpiPending*)pend; p1.pending_cap = cap; p1.pending_n = cnt_removed + 1;
        {
            PROF(h, "maxmin");
            CK(h, mcpg::launch_maxmin(p1, mcpg::MM_DPI1, 1, h->stream, &h->launches), "TF DPI kernel (first phase)");
        }
        unsigned long long np = 0;
        CK(h, cudaMemcpyAsync(&np, cnt_removed + 1, sizeof np, cudaMemcpyDeviceToHost, h->stream), "read pending");
        CK(h, cudaStreamSynchronize(h->stream), "stream synchronize");
        if (np <= (unsigned long long)cap) {
            mcpg::DpiPendingTf tf;
            tf.tsplit = t; tf.perm = (const int*)pd; tf.tol_mult_f = tm; tf.tm_float = 1;
            {
                PROF(h, "dpi_pending");
                CK(h, mcpg::launch_dpi_pending((const float*)bp, ldt, n, k1, p1.pending, (int64_t)np, 0.0, out, ldo,
                                               mask, n, cnt_removed, h->stream, &h->launches, tf),
                   "TF DPI kernel (second phase)");
            }
            if (removed) {
                unsigned long long r = 0;
                CK(h, cudaMemcpyAsync(&r, cnt_removed, sizeof r, cudaMemcpyDeviceToHost, h->stream), "read removed");
                CK(h, cudaStreamSynchronize(h->stream), "stream synchronize");
                *removed = (int64_t)r;
            }
            return MCPG_OK;
        }
    }
    // all-y value (y not in {x, z})
    void* call;
    if ((rc = scratch(h, S_M1, (size_t)(n * ldt) * sizeof(float), &call))) return rc;
    mcpg::MaxminParams p{};
    p.A = a; p.lda = la; p.B = a; p.ldb = la; p.rows = n; p.cols = n; p.k_len = n;
    p.C = (float*)call; p.ldc = ldt;
    {
        PROF(h, "maxmin");
        CK(h, mcpg::launch_maxmin(p, mcpg::MM_EXCL, 1, h->stream, &h->launches), "maxmin kernel (all y)");
    }
    // TF-y value: k over the TF columns only, excluding x's and z's own TF column
    const float* ctf = (const float*)call;
    if (t > 0) {
        std::vector<int> ex((size_t)n, -1);
        for (int64_t c = 0; c < t; ++c) ex[(size_t)ts.idx[(size_t)c]] = (int)c;
        void *idx, *exd, *atf, *c2;
        const int64_t ldk = round_up(t, 4);
        if ((rc = upload(h, S_TFIDX, ts.idx.data(), (size_t)t * sizeof(int), &idx))) return rc;
        if ((rc = upload(h, S_TFEX, ex.data(), (size_t)n * sizeof(int), &exd))) return rc;
        if ((rc = scratch(h, S_TFA, (size_t)(n * ldk) * sizeof(float), &atf))) return rc;
        if ((rc = scratch(h, S_M2, (size_t)(n * ldt) * sizeof(float), &c2))) return rc;
        CK(h, mcpg::launch_gather(a, la, nullptr, (const int*)idx, n, t, (float*)atf, ldk, h->stream, &h->launches),
           "gather kernel");
        mcpg::MaxminParams q{};
        q.A = (const float*)atf; q.lda = ldk; q.B = (const float*)atf; q.ldb = ldk;
        q.rows = n; q.cols = n; q.k_len = t; q.C = (float*)c2; q.ldc = ldt;
        q.excl_row = (const int*)exd; q.excl_col = (const int*)exd;
        {
            PROF(h, "maxmin");
            CK(h, mcpg::launch_maxmin(q, mcpg::MM_EXCL, 1, h->stream, &h->launches), "maxmin kernel (TF y)");
        }
        ctf = (const float*)c2;
    }
    std::vector<uint8_t> flag((size_t)n, 0);
    for (int i : ts.idx) flag[(size_t)i] = 1;
    void *fl, *cnt;
    if ((rc = upload(h, S_MASK + 0, flag.data(), (size_t)n, &fl))) return rc;
    if ((rc = scratch(h, S_SMALL, 64, &cnt))) return rc;
    CK(h, cudaMemsetAsync(cnt, 0, sizeof(unsigned long long), h->stream), "memset counter");
    {
        PROF(h, "dpi_tf_apply");
        CK(h, mcpg::launch_dpi_tf_apply(a, la, (const float*)call, ldt, ctf, ldt, (const uint8_t*)fl, n, tm, out, ldo,
                                        mask, (unsigned long long*)cnt, h->stream, &h->launches),
           "dpi_tf_apply kernel");
    }
    if (removed) {
        unsigned long long r = 0;
        CK(h, cudaMemcpyAsync(&r, cnt, sizeof r, cudaMemcpyDeviceToHost, h->stream), "read removed");
        CK(h, cudaStreamSynchronize(h->stream), "stream synchronize");
        *removed = (int64_t)r;
    }
    return MCPG_OK;
}

// ---------------- adjoints ----------------
int maxmin_witness_dev(mcpg_handle* h, const float* A, int64_t lda, const float* B, int64_t ldb, int64_t rows,
                       int64_t cols, int64_t k, float* C, int64_t ldc, int32_t* K, int64_t ldk) {
    if (rows < 0 || cols < 0 || k < 0) return fail(h, MCPG_ERR_ARG, "maxmin_witness: negative size");
    if (rows == 0 || cols == 0) return MCPG_OK;
    if (!A || !B || !C || !K) return fail(h, MCPG_ERR_ARG, "maxmin_witness: null pointer");
    if (lda < k || ldb < k || ldc < cols || ldk < cols)
        return fail(h, MCPG_ERR_ARG, "maxmin_witness: leading dimension too small");
    const bool symm = (A == B) && (lda == ldb) && (rows == cols);
    const float *a, *b;
    int64_t la, lb;
    int rc = aligned_view(h, A, lda, rows, k, S_IN0, &a, &la);
    if (rc) return rc;
    if (symm) {
        b = a; lb = la;
    } else if ((rc = aligned_view(h, B, ldb, cols, k, S_IN1, &b, &lb))) {
        return rc;
    }
    mcpg::MaxminParams p{};
    p.A = a; p.lda = la; p.B = b; p.ldb = lb; p.rows = rows; p.cols = cols; p.k_len = k;
    p.C = C; p.ldc = ldc; p.K = K; p.ldk = ldk;
    PROF(h, "maxmin_witness");
    CK(h, mcpg::launch_maxmin(p, mcpg::MM_WITNESS, symm ? 1 : 0, h->stream, &h->launches), "maxmin witness kernel");
    return MCPG_OK;
}

int maxmin_bwd_dev(mcpg_handle* h, const float* A, int64_t lda, const float* B, int64_t ldb, int64_t rows,
                   int64_t cols, int64_t k, const float* C, int64_t ldc, const float* dC, int64_t lddc,
                   const int32_t* K, int64_t ldk, float* dA, int64_t ldda, float* dB, int64_t lddb) {
    if (rows < 0 || cols < 0 || k < 0) return fail(h, MCPG_ERR_ARG, "maxmin_bwd: negative size");
    if (rows == 0 || cols == 0) return MCPG_OK;
    if (!A || !B || !dC || !dA || !dB || (!K && !C)) return fail(h, MCPG_ERR_ARG, "maxmin_bwd: null pointer");
    if (lda < k || ldb < k || lddc < cols || ldda < k || lddb < k || (K && ldk < cols) || (!K && ldc < cols))
        return fail(h, MCPG_ERR_ARG, "maxmin_bwd: leading dimension too small");
    PROF(h, "maxmin_route");
    CK(h, mcpg::launch_maxmin_route(A, lda, B, ldb, rows, cols, k, C, ldc, dC, lddc, K, ldk, dA, ldda, dB, lddb,
                                    h->stream, &h->launches),
       "maxmin route kernel");
    return MCPG_OK;
}

int ratio_bwd_dev(mcpg_handle* h, const float* A, int64_t lda, const float* M, int64_t ldm, int64_t rows, int64_t cols,
                  const float* dR, int64_t lddr, float* dA, int64_t ldda, float* dM, int64_t lddm) {
    if (rows < 0 || cols < 0) return fail(h, MCPG_ERR_ARG, "ratio_bwd: negative size");
    if (rows == 0 || cols == 0) return MCPG_OK;
    if (!A || !M || !dR || !dA || !dM) return fail(h, MCPG_ERR_ARG, "ratio_bwd: null pointer");
    if (lda < cols || ldm < cols || lddr < cols || ldda < cols || lddm < cols)
        return fail(h, MCPG_ERR_ARG, "ratio_bwd: leading dimension too small");
    PROF(h, "ratio_bwd");
    CK(h, mcpg::launch_ratio_bwd(A, lda, M, ldm, rows, cols, dR, lddr, dA, ldda, dM, lddm, h->stream, &h->launches),
       "ratio_bwd kernel");
    return MCPG_OK;
}

// compute_maxmins (mcpnet_helper.hpp:437-460): M1 = A (x) A, M2 = A (x) M1,
// M3 = M1 (x) M1 with M1 computed once, plus the MCP2/3/4 ratios ratio(A, Mk)
// fused into the products' epilogues.  Every output is nullable; M1 lives in
// scratch when not requested.
int maxmins_dev(mcpg_handle* h, const float* A, int64_t n, int64_t lda, float* M1, int64_t ld1, float* M2,
                int64_t ld2, float* M3, int64_t ld3, float* R2, int64_t ldr2, float* R3, int64_t ldr3, float* R4,
                int64_t ldr4) {
    if (n < 0) return fail(h, MCPG_ERR_ARG, "maxmins: negative size");
    if (n == 0) return MCPG_OK;
    if (!A) return fail(h, MCPG_ERR_ARG, "maxmins: null input");
    if (lda < n || (M1 && ld1 < n) || (M2 && ld2 < n) || (M3 && ld3 < n) || (R2 && ldr2 < n) || (R3 && ldr3 < n) ||
        (R4 && ldr4 < n))
        return fail(h, MCPG_ERR_ARG, "maxmins: leading dimension too small");
    const float* a;
    int64_t la;
    int rc = aligned_view(h, A, lda, n, n, S_IN0, &a, &la);
    if (rc) return rc;
    float* m1 = M1;
    int64_t l1 = ld1;
    if (!m1 || (l1 % 4) != 0 || ((uintptr_t)m1 & 15u)) {
        void* p;
        l1 = round_up(n, 32);
        if ((rc = scratch(h, S_M1, (size_t)(n * l1) * sizeof(float), &p))) return rc;
        m1 = (float*)p;
    }
    mcpg::MaxminParams p{};
    p.rows = n; p.cols = n; p.k_len = n;
    p.A = a; p.lda = la; p.B = a; p.ldb = la; p.C = m1; p.ldc = l1; p.E = a; p.lde = la; p.R = R2; p.ldr = ldr2;
    {
        PROF(h, "maxmin");
        CK(h, mcpg::launch_maxmin(p, R2 ? mcpg::MM_RATIO : mcpg::MM_PLAIN, 1, h->stream, &h->launches),
           "maxmin kernel (M1)");
    }
    if (M2 || R3) {
        mcpg::MaxminParams q{};
        q.rows = n; q.cols = n; q.k_len = n;
        q.A = a; q.lda = la; q.B = m1; q.ldb = l1; q.C = M2; q.ldc = ld2; q.E = a; q.lde = la; q.R = R3; q.ldr = ldr3;
        PROF(h, "maxmin");
        CK(h, mcpg::launch_maxmin(q, R3 ? mcpg::MM_RATIO : mcpg::MM_PLAIN, 0, h->stream, &h->launches),
           "maxmin kernel (M2)");
    }
    if (M3 || R4) {
        mcpg::MaxminParams q{};
        q.rows = n; q.cols = n; q.k_len = n;
        q.A = m1; q.lda = l1; q.B = m1; q.ldb = l1; q.C = M3; q.ldc = ld3; q.E = a; q.lde = la; q.R = R4; q.ldr = ldr4;
        PROF(h, "maxmin");
        CK(h, mcpg::launch_maxmin(q, R4 ? mcpg::MM_RATIO : mcpg::MM_PLAIN, 1, h->stream, &h->launches),
           "maxmin kernel (M3)");
    }
    if (M1 && m1 != M1) CK(h, mcpg::launch_copy2d(m1, l1, M1, ld1, n, n, h->stream), "copy2d");
    return MCPG_OK;
}

}  // namespace

using namespace mcpg_api;

extern "C" {

// ---- max-min ----
int mcpg_maxmin_dev(mcpg_handle* h, const float* A, int64_t lda, const float* B, int64_t ldb, int64_t rows,
                    int64_t cols, int64_t k, float* C, int64_t ldc) {
    int rc = check_handle(h);
    if (rc) return rc;
    return maxmin_dev(h, A, lda, B, ldb, rows, cols, k, C, ldc);
}

int mcpg_maxmin(mcpg_handle* h, const float* A, int64_t lda, const float* B, int64_t ldb, int64_t rows, int64_t cols,
                int64_t k, float* C, int64_t ldc) {
    int rc = check_handle(h);
    if (rc) return rc;
    if (rows < 0 || cols < 0 || k < 0) return fail(h, MCPG_ERR_ARG, "maxmin: negative size");
    if (rows == 0 || cols == 0) return MCPG_OK;
    if (!A || !B || !C) return fail(h, MCPG_ERR_ARG, "maxmin: null pointer");
    if (lda < k || ldb < k || ldc < cols) return fail(h, MCPG_ERR_ARG, "maxmin: leading dimension too small");
    const bool same = (A == B) && (lda == ldb) && (rows == cols);
    float *dA, *dB, *dC;
    int64_t la, lb, lc;
    if ((rc = stage_in(h, S_IN0, A, lda, rows, k, &dA, &la))) return rc;
    if (same) {
        dB = dA; lb = la;
    } else if ((rc = stage_in(h, S_IN1, B, ldb, cols, k, &dB, &lb))) {
        return rc;
    }
    if ((rc = out_view(h, S_OUT0, C, ldc, rows, cols, &dC, &lc))) return rc;
    if ((rc = maxmin_dev(h, dA, la, dB, lb, rows, cols, k, dC, lc))) return rc;
    if ((rc = copy_out(h, C, ldc, dC, lc, rows, cols))) return rc;
    return finish(h);
}

// ---- ratio ----
int mcpg_ratio_dev(mcpg_handle* h, const float* A, int64_t lda, const float* M, int64_t ldm, int64_t rows,
                   int64_t cols, float* R, int64_t ldr) {
    int rc = check_handle(h);
    if (rc) return rc;
    if (rows < 0 || cols < 0) return fail(h, MCPG_ERR_ARG, "ratio: negative size");
    if (rows == 0 || cols == 0) return MCPG_OK;
    if (!A || !M || !R) return fail(h, MCPG_ERR_ARG, "ratio: null pointer");
    if (lda < cols || ldm < cols || ldr < cols) return fail(h, MCPG_ERR_ARG, "ratio: leading dimension too small");
    {
        PROF(h, "ratio");
        CK(h, mcpg::launch_ratio(A, lda, M, ldm, rows, cols, R, ldr, h->stream, &h->launches), "ratio kernel");
    }
    return MCPG_OK;
}

int mcpg_ratio(mcpg_handle* h, const float* A, int64_t lda, const float* M, int64_t ldm, int64_t rows, int64_t cols,
               float* R, int64_t ldr) {
    int rc = check_handle(h);
    if (rc) return rc;
    if (rows < 0 || cols < 0) return fail(h, MCPG_ERR_ARG, "ratio: negative size");
    if (rows == 0 || cols == 0) return MCPG_OK;
    if (!A || !M || !R) return fail(h, MCPG_ERR_ARG, "ratio: null pointer");
    if (lda < cols || ldm < cols || ldr < cols) return fail(h, MCPG_ERR_ARG, "ratio: leading dimension too small");
    float *dA, *dM, *dR;
    int64_t la, lm, lr;
    if ((rc = in_view(h, S_IN0, A, lda, rows, cols, &dA, &la))) return rc;   // each read once
    if ((rc = in_view(h, S_IN1, M, ldm, rows, cols, &dM, &lm))) return rc;
    if ((rc = out_view(h, S_OUT0, R, ldr, rows, cols, &dR, &lr))) return rc;
    {
        PROF(h, "ratio");
        CK(h, mcpg::launch_ratio(dA, la, dM, lm, rows, cols, dR, lr, h->stream, &h->launches), "ratio kernel");
    }
    if ((rc = copy_out(h, R, ldr, dR, lr, rows, cols))) return rc;
    return finish(h);
}

int mcpg_set_diagonal_dev(mcpg_handle* h, float* A, int64_t rows, int64_t cols, int64_t lda, float value) {
    int rc = check_handle(h);
    if (rc) return rc;
    if (rows < 0 || cols < 0) return fail(h, MCPG_ERR_ARG, "set_diagonal: negative size");
    if (rows == 0 || cols == 0) return MCPG_OK;
    if (!A || lda < cols) return fail(h, MCPG_ERR_ARG, "set_diagonal: bad arguments");
    CK(h, mcpg::launch_set_diagonal(A, rows, cols, lda, value, h->stream, &h->launches), "set_diagonal kernel");
    return MCPG_OK;
}

// ---- MCP ----
int mcpg_mcp_dev(mcpg_handle* h, const float* A, int64_t n, int64_t lda, int path_len, int symmetrize, float* Mout,
                 int64_t ldm, float* Rout, int64_t ldr) {
    int rc = check_handle(h);
    if (rc) return rc;
    return mcp_dev(h, A, n, lda, path_len, symmetrize, Mout, ldm, Rout, ldr);
}

int mcpg_mcp(mcpg_handle* h, const float* A, int64_t n, int64_t lda, int path_len, int symmetrize, float* Mout,
             int64_t ldm, float* Rout, int64_t ldr) {
    int rc = check_handle(h);
    if (rc) return rc;
    if (n < 0) return fail(h, MCPG_ERR_ARG, "mcp: negative size");
    if (n == 0) return MCPG_OK;
    if (!A) return fail(h, MCPG_ERR_ARG, "mcp: null input");
    if (path_len < 2 || path_len > 4) return fail(h, MCPG_ERR_ARG, "mcp: path_len must be 2, 3 or 4 (got %d)", path_len);
    if (lda < n || (Mout && ldm < n) || (Rout && ldr < n)) return fail(h, MCPG_ERR_ARG, "mcp: leading dimension too small");
    float *dA, *dM = nullptr, *dR = nullptr;
    int64_t la, lm = 0, lr = 0;
    if ((rc = stage_in(h, S_IN0, A, lda, n, n, &dA, &la))) return rc;
    if (Mout && (rc = out_view(h, S_OUT0, Mout, ldm, n, n, &dM, &lm))) return rc;
    if (Rout && (rc = out_view(h, S_OUT1, Rout, ldr, n, n, &dR, &lr))) return rc;
    if ((rc = mcp_dev(h, dA, n, la, path_len, symmetrize, dM, lm, dR, lr))) return rc;
    if ((rc = copy_out(h, Mout, ldm, dM, lm, n, n))) return rc;
    if ((rc = copy_out(h, Rout, ldr, dR, lr, n, n))) return rc;
    return finish(h);
}

// ---- DPI ----
int mcpg_dpi_dev(mcpg_handle* h, const float* A, int64_t n, int64_t lda, float tol, float* out, int64_t ldo,
                 uint8_t* mask, int64_t* removed) {
    int rc = check_handle(h);
    if (rc) return rc;
    return dpi_dev(h, A, n, lda, tol, out, ldo, mask, removed);
}

int mcpg_dpi(mcpg_handle* h, const float* A, int64_t n, int64_t lda, float tol, float* out, int64_t ldo, uint8_t* mask,
             int64_t* removed) {
    int rc = check_handle(h);
    if (rc) return rc;
    if (removed) *removed = 0;
    if (n < 0) return fail(h, MCPG_ERR_ARG, "dpi: negative size");
    if (n == 0) return MCPG_OK;
    if (!A || !out) return fail(h, MCPG_ERR_ARG, "dpi: null pointer");
    if (lda < n || ldo < n) return fail(h, MCPG_ERR_ARG, "dpi: leading dimension too small");
    float *dA, *dO;
    int64_t la, lo;
    if ((rc = stage_in(h, S_IN0, A, lda, n, n, &dA, &la))) return rc;
    if ((rc = out_view(h, S_OUT0, out, ldo, n, n, &dO, &lo))) return rc;
    uint8_t* dMask = nullptr;
    const bool mask_direct = mask && host_direct(h, mask, (size_t)(n * n), true);
    if (mask_direct) {
        dMask = mask;
    } else if (mask) {
        void* p;
        if ((rc = scratch(h, S_MASK, (size_t)(n * n), &p))) return rc;
        dMask = (uint8_t*)p;
    }
    if ((rc = dpi_dev(h, dA, n, la, tol, dO, lo, dMask, removed))) return rc;
    if ((rc = copy_out(h, out, ldo, dO, lo, n, n))) return rc;
    if (mask && !mask_direct)
        CK(h, cudaMemcpyAsync(mask, dMask, (size_t)(n * n), cudaMemcpyDeviceToHost, h->stream), "copy mask");
    return finish(h);
}

// ---- closure ----
int mcpg_closure_dev(mcpg_handle* h, const float* A, int64_t n, int64_t lda, int max_iter, float* out, int64_t ldo,
                     int* iterations) {
    int rc = check_handle(h);
    if (rc) return rc;
    return closure_dev(h, A, n, lda, max_iter, out, ldo, iterations);
}

int mcpg_closure(mcpg_handle* h, const float* A, int64_t n, int64_t lda, int max_iter, float* out, int64_t ldo,
                 int* iterations) {
    int rc = check_handle(h);
    if (rc) return rc;
    if (iterations) *iterations = 0;
    if (n < 0 || max_iter < 0) return fail(h, MCPG_ERR_ARG, "closure: negative size or max_iter");
    if (n == 0) return MCPG_OK;
    if (!A || !out) return fail(h, MCPG_ERR_ARG, "closure: null pointer");
    if (lda < n || ldo < n) return fail(h, MCPG_ERR_ARG, "closure: leading dimension too small");
    float *dA, *dO;
    int64_t la, lo;
    if ((rc = stage_in(h, S_IN0, A, lda, n, n, &dA, &la))) return rc;
    if ((rc = out_view(h, S_OUT0, out, ldo, n, n, &dO, &lo))) return rc;
    int crc = closure_dev(h, dA, n, la, max_iter, dO, lo, iterations);
    if (crc && crc != MCPG_ERR_NOT_CONVERGED) return crc;
    std::string keep = h->err;
    if ((rc = copy_out(h, out, ldo, dO, lo, n, n))) return rc;
    if ((rc = finish(h))) return rc;
    h->err = keep;
    return crc;
}

// ---- TF-restricted variants ----
int mcpg_maxmin_masked_dev(mcpg_handle* h, const float* A, int64_t lda, const float* B, int64_t ldb, int64_t rows,
                           int64_t cols, int64_t k, const float* mask, float* C, int64_t ldc) {
    int rc = check_handle(h);
    if (rc) return rc;
    return maxmin_masked_dev(h, A, lda, B, ldb, rows, cols, k, mask, C, ldc);
}

int mcpg_maxmin_masked(mcpg_handle* h, const float* A, int64_t lda, const float* B, int64_t ldb, int64_t rows,
                       int64_t cols, int64_t k, const float* mask, float* C, int64_t ldc) {
    int rc = check_handle(h);
    if (rc) return rc;
    if (rows < 0 || cols < 0 || k < 0) return fail(h, MCPG_ERR_ARG, "maxmin_masked: negative size");
    if (rows == 0 || cols == 0) return MCPG_OK;
    if (!A || !B || !C || (k > 0 && !mask)) return fail(h, MCPG_ERR_ARG, "maxmin_masked: null pointer");
    if (lda < k || ldb < k || ldc < cols) return fail(h, MCPG_ERR_ARG, "maxmin_masked: leading dimension too small");
    const bool same = (A == B) && (lda == ldb) && (rows == cols);
    float *dA, *dB, *dC;
    int64_t la, lb, lc;
    if ((rc = stage_in(h, S_IN0, A, lda, rows, k, &dA, &la))) return rc;
    if (same) {
        dB = dA; lb = la;
    } else if ((rc = stage_in(h, S_IN1, B, ldb, cols, k, &dB, &lb))) {
        return rc;
    }
    if ((rc = out_view(h, S_OUT0, C, ldc, rows, cols, &dC, &lc))) return rc;
    if ((rc = maxmin_masked_dev(h, dA, la, dB, lb, rows, cols, k, mask, dC, lc))) return rc;
    if ((rc = copy_out(h, C, ldc, dC, lc, rows, cols))) return rc;
    return finish(h);
}

int mcpg_mcp_tf_dev(mcpg_handle* h, const float* A, int64_t n, int64_t lda, const float* tfs, int path_len,
                    int tf_gene_transition, float* Mout, int64_t ldm, float* Rout, int64_t ldr) {
    int rc = check_handle(h);
    if (rc) return rc;
    return mcp_tf_dev(h, A, n, lda, tfs, path_len, tf_gene_transition, Mout, ldm, Rout, ldr);
}

int mcpg_mcp_tf(mcpg_handle* h, const float* A, int64_t n, int64_t lda, const float* tfs, int path_len,
                int tf_gene_transition, float* Mout, int64_t ldm, float* Rout, int64_t ldr) {
    int rc = check_handle(h);
    if (rc) return rc;
    if (n < 0) return fail(h, MCPG_ERR_ARG, "mcp_tf: negative size");
    if (n == 0) return MCPG_OK;
    if (!A || !tfs) return fail(h, MCPG_ERR_ARG, "mcp_tf: null pointer");
    if (lda < n || (Mout && ldm < n) || (Rout && ldr < n)) return fail(h, MCPG_ERR_ARG, "mcp_tf: leading dimension too small");
    int64_t t = 0;
    for (int64_t i = 0; i < n; ++i) t += tfs[i] > 0.0f;
    float *dA, *dM = nullptr, *dR = nullptr;
    int64_t la, lm = 0, lr = 0;
    if ((rc = stage_in(h, S_IN0, A, lda, n, n, &dA, &la))) return rc;
    if (Mout && t > 0 && (rc = out_view(h, S_OUT0, Mout, ldm, t, n, &dM, &lm))) return rc;
    if (Rout && t > 0 && (rc = out_view(h, S_OUT1, Rout, ldr, t, n, &dR, &lr))) return rc;
    if ((rc = mcp_tf_dev(h, dA, n, la, tfs, path_len, tf_gene_transition, dM, lm, dR, lr))) return rc;
    if (t > 0) {
        if ((rc = copy_out(h, Mout, ldm, dM, lm, t, n))) return rc;
        if ((rc = copy_out(h, Rout, ldr, dR, lr, t, n))) return rc;
    }
    return finish(h);
}

int mcpg_dpi_tf_dev(mcpg_handle* h, const float* A, int64_t n, int64_t lda, float tol, const float* tfs, float* out,
                    int64_t ldo, uint8_t* mask, int64_t* removed) {
    int rc = check_handle(h);
    if (rc) return rc;
    return dpi_tf_dev(h, A, n, lda, tol, tfs, out, ldo, mask, removed);
}

int mcpg_dpi_tf(mcpg_handle* h, const float* A, int64_t n, int64_t lda, float tol, const float* tfs, float* out,
                int64_t ldo, uint8_t* mask, int64_t* removed) {
    int rc = check_handle(h);
    if (rc) return rc;
    if (removed) *removed = 0;
    if (n < 0) return fail(h, MCPG_ERR_ARG, "dpi_tf: negative size");
    if (n == 0) return MCPG_OK;
    if (!A || !out || !tfs) return fail(h, MCPG_ERR_ARG, "dpi_tf: null pointer");
    if (lda < n || ldo < n) return fail(h, MCPG_ERR_ARG, "dpi_tf: leading dimension too small");
    float *dA, *dO;
    int64_t la, lo;
    if ((rc = stage_in(h, S_IN2, A, lda, n, n, &dA, &la))) return rc;
    if ((rc = out_view(h, S_OUT0, out, ldo, n, n, &dO, &lo))) return rc;
    uint8_t* dMask = nullptr;
    const bool mask_direct = mask && host_direct(h, mask, (size_t)(n * n), true);
    if (mask_direct) {
        dMask = mask;
    } else if (mask) {
        void* p;
        if ((rc = scratch(h, S_OUT1, (size_t)(n * n), &p))) return rc;
        dMask = (uint8_t*)p;
    }
    if ((rc = dpi_tf_dev(h, dA, n, la, tol, tfs, dO, lo, dMask, removed))) return rc;
    if ((rc = copy_out(h, out, ldo, dO, lo, n, n))) return rc;
    if (mask && !mask_direct)
        CK(h, cudaMemcpyAsync(mask, dMask, (size_t)(n * n), cudaMemcpyDeviceToHost, h->stream), "copy mask");
    return finish(h);
}

// ---- adjoints ----
int mcpg_maxmin_witness_dev(mcpg_handle* h, const float* A, int64_t lda, const float* B, int64_t ldb, int64_t rows,
                            int64_t cols, int64_t k, float* C, int64_t ldc, int32_t* K, int64_t ldk) {
    int rc = check_handle(h);
    if (rc) return rc;
    return maxmin_witness_dev(h, A, lda, B, ldb, rows, cols, k, C, ldc, K, ldk);
}

int mcpg_maxmin_witness(mcpg_handle* h, const float* A, int64_t lda, const float* B, int64_t ldb, int64_t rows,
                        int64_t cols, int64_t k, float* C, int64_t ldc, int32_t* K, int64_t ldk) {
    int rc = check_handle(h);
    if (rc) return rc;
    if (rows < 0 || cols < 0 || k < 0) return fail(h, MCPG_ERR_ARG, "maxmin_witness: negative size");
    if (rows == 0 || cols == 0) return MCPG_OK;
    if (!A || !B || !C || !K) return fail(h, MCPG_ERR_ARG, "maxmin_witness: null pointer");
    if (lda < k || ldb < k || ldc < cols || ldk < cols)
        return fail(h, MCPG_ERR_ARG, "maxmin_witness: leading dimension too small");
    const bool same = (A == B) && (lda == ldb) && (rows == cols);
    float *dA, *dB, *dC, *dK;
    int64_t la, lb, lc, lk;
    if ((rc = stage_in(h, S_IN0, A, lda, rows, k, &dA, &la))) return rc;
    if (same) {
        dB = dA; lb = la;
    } else if ((rc = stage_in(h, S_IN1, B, ldb, cols, k, &dB, &lb))) {
        return rc;
    }
    if ((rc = stage_out_alloc(h, S_OUT0, rows, cols, &dC, &lc))) return rc;
    if ((rc = stage_out_alloc(h, S_OUT1, rows, cols, &dK, &lk))) return rc;
    if ((rc = maxmin_witness_dev(h, dA, la, dB, lb, rows, cols, k, dC, lc, (int32_t*)dK, lk))) return rc;
    if ((rc = copy_out(h, C, ldc, dC, lc, rows, cols))) return rc;
    if ((rc = copy_out(h, (float*)K, ldk, dK, lk, rows, cols))) return rc;
    return finish(h);
}

int mcpg_maxmin_bwd_dev(mcpg_handle* h, const float* A, int64_t lda, const float* B, int64_t ldb, int64_t rows,
                        int64_t cols, int64_t k, const float* C, int64_t ldc, const float* dC, int64_t lddc,
                        const int32_t* K, int64_t ldk, float* dA, int64_t ldda, float* dB, int64_t lddb) {
    int rc = check_handle(h);
    if (rc) return rc;
    return maxmin_bwd_dev(h, A, lda, B, ldb, rows, cols, k, C, ldc, dC, lddc, K, ldk, dA, ldda, dB, lddb);
}

int mcpg_maxmin_bwd(mcpg_handle* h, const float* A, int64_t lda, const float* B, int64_t ldb, int64_t rows,
                    int64_t cols, int64_t k, const float* C, int64_t ldc, const float* dC, int64_t lddc,
                    const int32_t* K, int64_t ldk, float* dA, int64_t ldda, float* dB, int64_t lddb) {
    int rc = check_handle(h);
    if (rc) return rc;
    if (rows < 0 || cols < 0 || k < 0) return fail(h, MCPG_ERR_ARG, "maxmin_bwd: negative size");
    if (rows == 0 || cols == 0) return MCPG_OK;
    if (!A || !B || !dC || !dA || !dB || (!K && !C)) return fail(h, MCPG_ERR_ARG, "maxmin_bwd: null pointer");
    if (lda < k || ldb < k || lddc < cols || ldda < k || lddb < k || (K && ldk < cols) || (!K && ldc < cols))
        return fail(h, MCPG_ERR_ARG, "maxmin_bwd: leading dimension too small");
    const bool same_in = (A == B) && (lda == ldb) && (rows == cols);
    const bool same_out = (dA == dB) && (ldda == lddb) && (rows == cols);
    float *a, *b, *c = nullptr, *g, *ga, *gb, *kk = nullptr;
    int64_t la, lb, lc = 0, lg, lga, lgb, lk = 0;
    if ((rc = stage_in(h, S_IN0, A, lda, rows, k, &a, &la))) return rc;
    if (same_in) {
        b = a; lb = la;
    } else if ((rc = stage_in(h, S_IN1, B, ldb, cols, k, &b, &lb))) {
        return rc;
    }
    if (K) {
        if ((rc = stage_in(h, S_IN2, (const float*)K, ldk, rows, cols, &kk, &lk))) return rc;
    } else if ((rc = stage_in(h, S_IN2, C, ldc, rows, cols, &c, &lc))) {
        return rc;
    }
    if ((rc = stage_in(h, S_IN3, dC, lddc, rows, cols, &g, &lg))) return rc;
    if ((rc = stage_in(h, S_OUT0, dA, ldda, rows, k, &ga, &lga))) return rc;
    if (same_out) {
        gb = ga; lgb = lga;
    } else if ((rc = stage_in(h, S_OUT1, dB, lddb, cols, k, &gb, &lgb))) {
        return rc;
    }
    if ((rc = maxmin_bwd_dev(h, a, la, b, lb, rows, cols, k, c, lc, g, lg, (const int32_t*)kk, lk, ga, lga, gb, lgb)))
        return rc;
    if ((rc = copy_out(h, dA, ldda, ga, lga, rows, k))) return rc;
    if (!same_out && (rc = copy_out(h, dB, lddb, gb, lgb, cols, k))) return rc;
    return finish(h);
}

int mcpg_ratio_bwd_dev(mcpg_handle* h, const float* A, int64_t lda, const float* M, int64_t ldm, int64_t rows,
                       int64_t cols, const float* dR, int64_t lddr, float* dA, int64_t ldda, float* dM, int64_t lddm) {
    int rc = check_handle(h);
    if (rc) return rc;
    return ratio_bwd_dev(h, A, lda, M, ldm, rows, cols, dR, lddr, dA, ldda, dM, lddm);
}

int mcpg_maxmins_dev(mcpg_handle* h, const float* A, int64_t n, int64_t lda, float* M1, int64_t ld1, float* M2,
                     int64_t ld2, float* M3, int64_t ld3, float* R2, int64_t ldr2, float* R3, int64_t ldr3, float* R4,
                     int64_t ldr4) {
    int rc = check_handle(h);
    if (rc) return rc;
    return maxmins_dev(h, A, n, lda, M1, ld1, M2, ld2, M3, ld3, R2, ldr2, R3, ldr3, R4, ldr4);
}

int mcpg_maxmins(mcpg_handle* h, const float* A, int64_t n, int64_t lda, float* M1, int64_t ld1, float* M2,
                 int64_t ld2, float* M3, int64_t ld3, float* R2, int64_t ldr2, float* R3, int64_t ldr3, float* R4,
                 int64_t ldr4) {
    int rc = check_handle(h);
    if (rc) return rc;
    if (n < 0) return fail(h, MCPG_ERR_ARG, "maxmins: negative size");
    if (n == 0) return MCPG_OK;
    if (!A || lda < n) return fail(h, MCPG_ERR_ARG, "maxmins: null input or leading dimension");
    float* dA;
    int64_t la;
    if ((rc = stage_in(h, S_IN2, A, lda, n, n, &dA, &la))) return rc;
    // device outputs for the requested host outputs (each in its own scratch slot)
    float* host[6] = {M1, M2, M3, R2, R3, R4};
    const int64_t hld[6] = {ld1, ld2, ld3, ldr2, ldr3, ldr4};
    const int slots[6] = {S_OUT0, S_OUT1, S_IN3, S_IN4, S_TFA, S_TFB};
    float* dev[6] = {};
    int64_t dld[6] = {};
    for (int k = 0; k < 6; ++k) {
        if (!host[k]) continue;
        if (hld[k] < n) return fail(h, MCPG_ERR_ARG, "maxmins: leading dimension too small");
        // M1 is an operand of the later products: it stays in device memory
        rc = k == 0 ? stage_out_alloc(h, slots[k], n, n, &dev[k], &dld[k])
                    : out_view(h, slots[k], host[k], hld[k], n, n, &dev[k], &dld[k]);
        if (rc) return rc;
    }
    if ((rc = maxmins_dev(h, dA, n, la, dev[0], dld[0], dev[1], dld[1], dev[2], dld[2], dev[3], dld[3], dev[4], dld[4],
                          dev[5], dld[5])))
        return rc;
    for (int k = 0; k < 6; ++k)
        if (host[k] && (rc = copy_out(h, host[k], hld[k], dev[k], dld[k], n, n))) return rc;
    return finish(h);
}

int mcpg_maxmins_tf_dev(mcpg_handle* h, const float* A, int64_t n, int64_t lda, const float* tfs, float* T,
                        int64_t ldt, float* M1, int64_t ld1, float* M2, int64_t ld2, float* M3, int64_t ld3) {
    int rc = check_handle(h);
    if (rc) return rc;
    return maxmins_tf_dev(h, A, n, lda, tfs, T, ldt, M1, ld1, M2, ld2, M3, ld3);
}

int mcpg_maxmins_tf(mcpg_handle* h, const float* A, int64_t n, int64_t lda, const float* tfs, float* T, int64_t ldt,
                    float* M1, int64_t ld1, float* M2, int64_t ld2, float* M3, int64_t ld3) {
    int rc = check_handle(h);
    if (rc) return rc;
    if (n < 0) return fail(h, MCPG_ERR_ARG, "maxmins_tf: negative size");
    if (n == 0) return MCPG_OK;
    if (!A || !tfs) return fail(h, MCPG_ERR_ARG, "maxmins_tf: null pointer");
    if (lda < n || (T && ldt < n) || (M1 && ld1 < n) || (M2 && ld2 < n) || (M3 && ld3 < n))
        return fail(h, MCPG_ERR_ARG, "maxmins_tf: leading dimension too small");
    const int64_t t = (int64_t)tf_set(tfs, n).idx.size();
    if (t == 0) return MCPG_OK;
    float *da, *o[4] = {};
    int64_t la, lo[4] = {};
    // (the masked products use only the TF slots)
    if ((rc = stage_in(h, S_IN2, A, lda, n, n, &da, &la))) return rc;
    float* const host[4] = {T, M1, M2, M3};
    const int64_t hld[4] = {ldt, ld1, ld2, ld3};
    const int slots[4] = {S_OUT0, S_OUT1, S_IN3, S_IN4};
    for (int k = 0; k < 4; ++k) {  // M1 (k = 1) is an operand of M2 and M3: it stays in device memory
        if (!host[k]) continue;
        rc = k == 1 ? stage_out_alloc(h, slots[k], t, n, &o[k], &lo[k])
                    : out_view(h, slots[k], host[k], hld[k], t, n, &o[k], &lo[k]);
        if (rc) return rc;
    }
    if ((rc = maxmins_tf_dev(h, da, n, la, tfs, o[0], lo[0], o[1], lo[1], o[2], lo[2], o[3], lo[3]))) return rc;
    for (int k = 0; k < 4; ++k)
        if (host[k] && (rc = copy_out(h, host[k], hld[k], o[k], lo[k], t, n))) return rc;
    return finish(h);
}

}  // extern "C"
