// C ABI: B-spline MI (compute_mi, apps/pipeline/mcpnet_helper.hpp:56-99) on the
// CUDA cores or the tensor cores, its weights, its adjoint, and adaptive-partitioning
// MI (mcpnet_helper.hpp:102-167).
#include "api_internal.h"

namespace {

using namespace mcpg_api;

// ---------------- device implementations ----------------
// ---- B-spline MI in three steps: weights (prepare), gene-range launches, finish ----
struct MiPlan {
    int precision = 0, fmt = 0, split = 0, bins = 0;  // split: mcpg::TcMode
    int64_t n = 0, m = 0;
    const void* w0 = nullptr;  // FP32 sample-major or 16-bit hi weights
    const void* w1 = nullptr;  // 16-bit lo weights, or the interleaved E4M3 H8|L8 plane (split 2)
    int64_t ld = 0;            // weight leading dimension
    double* H = nullptr;
    float* MI = nullptr;
    int64_t ldmi = 0;
    int* flag = nullptr;       // tensor-core timeout flag
};

int mi_prepare(mcpg_handle* h, const float* X, int64_t n, int64_t m, int64_t ldx, int bins, int order, int precision,
               float* MI, int64_t ldmi, double* H, MiPlan& pl) {
    if (n < 1 || m < 1) return fail(h, MCPG_ERR_ARG, "bspline_mi: need n >= 1 and m >= 1 (got %lld, %lld)",
                                    (long long)n, (long long)m);
    if (ldx < m || ldmi < n) return fail(h, MCPG_ERR_ARG, "bspline_mi: leading dimension too small");
    if (!X || !MI) return fail(h, MCPG_ERR_ARG, "bspline_mi: null pointer");
    if (bins < 1 || bins > 32 || order < 1 || order > 8 || bins < order)
        return fail(h, MCPG_ERR_ARG, "bspline_mi: need 1 <= order <= bins <= 32, order <= 8 (got bins=%d order=%d)",
                    bins, order);
    if (precision < MCPG_MI_FP32 || precision > MCPG_MI_BF16F8)
        return fail(h, MCPG_ERR_ARG, "bspline_mi: unknown precision %d", precision);
    pl = MiPlan{};
    pl.precision = precision; pl.bins = bins; pl.n = n; pl.m = m; pl.MI = MI; pl.ldmi = ldmi; pl.H = H;
    int rc;
    if (!pl.H) {
        void* p;
        if ((rc = scratch(h, S_H, (size_t)n * sizeof(double), &p))) return rc;
        pl.H = (double*)p;
    }
    if (precision == MCPG_MI_FP32) {
        if (bins < 2 || bins > 12)
            return fail(h, MCPG_ERR_UNSUPPORTED, "bspline_mi FP32: bins must be 2..12 (got %d)", bins);
        const int64_t ldwt = round_up(n, 16) * bins;
        const int64_t m_pad = round_up(m, 16);
        void* p;
        if ((rc = scratch(h, S_W0, (size_t)(m_pad * ldwt) * sizeof(float), &p))) return rc;
        CK(h, cudaMemsetAsync(p, 0, (size_t)(m_pad * ldwt) * sizeof(float), h->stream), "memset weights");
        PROF(h, "bspline_weights");
        CK(h, mcpg::launch_bspline_weights_fp32(X, n, m, ldx, bins, order, (float*)p, ldwt, pl.H, h->stream,
                                                 &h->launches),
           "bspline weights kernel");
        pl.w0 = p;
        pl.ld = ldwt;
        return MCPG_OK;
    }
    if (bins != 10) return fail(h, MCPG_ERR_UNSUPPORTED, "bspline_mi tensor-core path: only 10 bins (got %d)", bins);
    pl.fmt = (precision == MCPG_MI_FP16 || precision == MCPG_MI_FP16X3) ? 1 : 0;
    pl.split = (precision == MCPG_MI_BF16X3 || precision == MCPG_MI_FP16X3) ? mcpg::TC_SPLIT16
               : precision == MCPG_MI_BF16F8                                ? mcpg::TC_F8C
                                                                            : mcpg::TC_SINGLE;
    const int64_t ldw = mcpg::mi_tc_pitch(m);
    const int64_t rows = round_up(n * bins, 256) + 256;  // whole tiles stay in bounds
    // S_W1: the 16-bit lo plane, or the interleaved 8-bit plane H8|L8 (rows of 2 * ldw bytes: the same bytes)
    void *hi, *lo = nullptr;
    if ((rc = scratch(h, S_W0, (size_t)(rows * ldw) * 2, &hi))) return rc;
    if (pl.split && (rc = scratch(h, S_W1, (size_t)(rows * ldw) * 2, &lo))) return rc;
    const bool f8 = pl.split == mcpg::TC_F8C;
    // rows beyond n*bins must be zero (they are read by the last tiles)
    const size_t done = (size_t)(n * bins * ldw), tail = (size_t)((rows - n * bins) * ldw);
    CK(h, cudaMemsetAsync((char*)hi + done * 2, 0, tail * 2, h->stream), "memset weights");
    if (pl.split) CK(h, cudaMemsetAsync((char*)lo + done * 2, 0, tail * 2, h->stream), "memset weights");
    if (f8) {
        PROF(h, "bspline_weights_f8");
        CK(h, mcpg::launch_bspline_weights_f8(X, n, m, ldx, bins, order, (uint16_t*)hi, (uint8_t*)lo, ldw, pl.H,
                                               h->stream, &h->launches),
           "bspline weights kernel");
    } else {
        PROF(h, "bspline_weights16");
        CK(h, mcpg::launch_bspline_weights_16(X, n, m, ldx, bins, order, pl.fmt, (uint16_t*)hi, (uint16_t*)lo, ldw,
                                               pl.H, h->stream, &h->launches),
           "bspline weights kernel");
    }
    void* flag;
    if ((rc = scratch(h, S_SMALL, 64, &flag))) return rc;
    CK(h, cudaMemsetAsync(flag, 0, sizeof(int), h->stream), "memset flag");
    pl.w0 = hi; pl.w1 = lo; pl.ld = ldw; pl.flag = (int*)flag;
    return MCPG_OK;
}

// Pairs (i, j >= i) with i in [g0, g1); g0 a multiple of 48 (both kernels' gene tiles).
int mi_launch(mcpg_handle* h, const MiPlan& pl, int64_t g0, int64_t g1) {
    if (pl.precision == MCPG_MI_FP32) {
        PROF(h, "mi_fp32");
        CK(h, mcpg::launch_mi_fp32((const float*)pl.w0, pl.ld, pl.H, pl.n, pl.m, pl.bins, pl.MI, pl.ldmi, h->stream,
                                   &h->launches, g0, g1),
           "MI FP32 kernel");
        return MCPG_OK;
    }
    // the 2-SM form's tile counters
    void* work = nullptr;
    {
        int rc = scratch(h, S_TCWORK, (size_t)mcpg::mi_tc_work_bytes(pl.n, pl.bins), &work);
        if (rc) return rc;
    }
    cudaError_t e;
    {
        PROF(h, "mi_tc");
        const bool f8 = pl.split == mcpg::TC_F8C;
        const mcpg::TcWaitHook* hook = h->tc_hook_armed ? &h->tc_hook : nullptr;
        h->tc_hook_armed = false;  // one launch only
        e = mcpg::launch_mi_tc((const uint16_t*)pl.w0, f8 ? nullptr : (const uint16_t*)pl.w1,
                               f8 ? (const uint8_t*)pl.w1 : nullptr, pl.ld, pl.H, pl.n, pl.m,
                               pl.bins, pl.fmt, pl.split, pl.MI, pl.ldmi, pl.flag, h->stream, &h->launches, g0, g1,
                               hook, work);
    }
    if (e == cudaErrorNotSupported)
        return fail(h, MCPG_ERR_UNSUPPORTED, "bspline_mi tensor-core path: unsupported shape or device");
    CK(h, e, "MI tensor-core kernel");
    return MCPG_OK;
}

// Synchronises the stream and reports a tensor-core timeout, if any.
int mi_finish(mcpg_handle* h, const MiPlan& pl) {
    if (!pl.flag) return MCPG_OK;
    int timed_out = 0;
    CK(h, cudaMemcpyAsync(&timed_out, pl.flag, sizeof(int), cudaMemcpyDeviceToHost, h->stream), "read flag");
    CK(h, cudaStreamSynchronize(h->stream), "stream synchronize");
    if (timed_out) return fail(h, MCPG_ERR_DEVICE_TIMEOUT, "MI tensor-core kernel: a bounded barrier wait gave up");
    return MCPG_OK;
}

int mi_dev(mcpg_handle* h, const float* X, int64_t n, int64_t m, int64_t ldx, int bins, int order, int precision,
           float* MI, int64_t ldmi, double* H) {
    MiPlan pl;
    int rc = mi_prepare(h, X, n, m, ldx, bins, order, precision, MI, ldmi, H, pl);
    if (rc) return rc;
    if ((rc = mi_launch(h, pl, 0, n))) return rc;
    return mi_finish(h, pl);
}

// MI adjoint: dX from G = dL/dMI (FP32).  Q = Gs (log2 P + 1/ln 2) is built in
// slabs of gene tiles that fit the slab budget, contracted with the weights on
// the plus-times twin of the max-min kernel, then pushed through the B-spline
// derivative and the min-max scaling per gene.
int mi_bwd_dev(mcpg_handle* h, const float* X, int64_t n, int64_t m, int64_t ldx, int bins, int order,
               const float* G, int64_t ldg, float* dX, int64_t lddx) {
    if (n < 1 || m < 1) return fail(h, MCPG_ERR_ARG, "bspline_mi_bwd: need n >= 1 and m >= 1");
    if (!X || !G || !dX) return fail(h, MCPG_ERR_ARG, "bspline_mi_bwd: null pointer");
    if (ldx < m || ldg < n || lddx < m) return fail(h, MCPG_ERR_ARG, "bspline_mi_bwd: leading dimension too small");
    if (bins < 1 || bins > 12 || order < 1 || order > 8 || bins < order)
        return fail(h, MCPG_ERR_ARG, "bspline_mi_bwd: need 1 <= order <= bins <= 12, order <= 8");
    if (bins < 2) return fail(h, MCPG_ERR_UNSUPPORTED, "bspline_mi_bwd: bins must be 2..12 (got %d)", bins);
    int rc;
    const int64_t ldwt = round_up(n, 16) * bins;
    const int64_t m_pad = round_up(m, 16);
    void *wt, *hd, *gs;
    if ((rc = scratch(h, S_W0, (size_t)(m_pad * ldwt) * sizeof(float), &wt))) return rc;
    if ((rc = scratch(h, S_H, (size_t)n * sizeof(double), &hd))) return rc;
    if ((rc = scratch(h, S_GS, (size_t)n * sizeof(float), &gs))) return rc;
    CK(h, cudaMemsetAsync(wt, 0, (size_t)(m_pad * ldwt) * sizeof(float), h->stream), "memset weights");
    {
        PROF(h, "bspline_weights");
        CK(h, mcpg::launch_bspline_weights_fp32(X, n, m, ldx, bins, order, (float*)wt, ldwt, (double*)hd, h->stream,
                                                 &h->launches),
           "bspline weights kernel");
    }
    {
        PROF(h, "pair_sums");
        CK(h, mcpg::launch_pair_sums(G, ldg, n, (float*)gs, h->stream, &h->launches), "pair sums kernel");
    }
    const int64_t T = (n + 15) / 16;
    const int64_t ldq = ldwt;  // >= n*bins, multiple of 4
    const size_t budget = (size_t)2 << 30;
    int64_t tiles_per_slab = (int64_t)(budget / ((size_t)16 * bins * ldq * sizeof(float)));
    if (tiles_per_slab < 1) tiles_per_slab = 1;
    if (tiles_per_slab > T) tiles_per_slab = T;
    const int64_t lddw = round_up(m, 4);
    void *q, *dw;
    if ((rc = scratch(h, S_Q, (size_t)(tiles_per_slab * 16 * bins * ldq) * sizeof(float), &q))) return rc;
    if ((rc = scratch(h, S_DW, (size_t)(tiles_per_slab * 16 * bins * lddw) * sizeof(float), &dw))) return rc;
    for (int64_t t0 = 0; t0 < T; t0 += tiles_per_slab) {
        const int64_t nt = (t0 + tiles_per_slab <= T) ? tiles_per_slab : T - t0;
        const int64_t g0 = t0 * 16, g1 = (g0 + nt * 16 < n) ? g0 + nt * 16 : n;
        {
            PROF(h, "mi_q");
            CK(h, mcpg::launch_mi_q((const float*)wt, ldwt, G, ldg, n, m, bins, t0, nt, (float*)q, ldq, h->stream,
                                    &h->launches),
               "MI adjoint Q kernel");
        }
        mcpg::MaxminParams p{};
        p.A = (const float*)q; p.lda = ldq; p.B = (const float*)wt; p.ldb = ldwt;
        p.rows = (g1 - g0) * bins; p.cols = m; p.k_len = n * bins;
        p.C = (float*)dw; p.ldc = lddw;
        {
            PROF(h, "gemm");
            CK(h, mcpg::launch_maxmin(p, mcpg::MM_GEMM, 0, h->stream, &h->launches), "adjoint contraction kernel");
        }
        {
            PROF(h, "mi_bwd_x");
            CK(h, mcpg::launch_mi_bwd_x(X, n, m, ldx, bins, order, g0, g1, (const float*)gs, (const float*)dw, lddw,
                                        dX, lddx, h->stream, &h->launches),
               "MI adjoint x kernel");
        }
    }
    return MCPG_OK;
}

// ---- adaptive-partitioning MI ----
int ap_check(mcpg_handle* h, int64_t n, int64_t m, const void* in, int64_t ld, const float* MI, int64_t ldmi) {
    if (n < 0 || m < 0) return fail(h, MCPG_ERR_ARG, "ap_mi: negative size");
    if (n > 0 && m > 0 && (!in || ld < m)) return fail(h, MCPG_ERR_ARG, "ap_mi: null input or leading dimension");
    if (n > 0 && (!MI || ldmi < n)) return fail(h, MCPG_ERR_ARG, "ap_mi: null output or leading dimension");
    if (m > mcpg::ap_max_samples())
        return fail(h, MCPG_ERR_UNSUPPORTED, "ap_mi: at most %lld samples", (long long)mcpg::ap_max_samples());
    if (n > 0 && m == 0) return fail(h, MCPG_ERR_ARG, "ap_mi: no samples");
    return MCPG_OK;
}

int ap_flag_check(mcpg_handle* h, int* dflag) {
    int f = 0;
    CK(h, cudaMemcpyAsync(&f, dflag, sizeof(int), cudaMemcpyDeviceToHost, h->stream), "device-to-host copy");
    CK(h, cudaStreamSynchronize(h->stream), "stream synchronize");
    if (f & 1) return fail(h, MCPG_ERR_ARG, "ap_mi: NaN value or rank outside [0, m)");
    if (f & 2) return fail(h, MCPG_ERR_CUDA, "ap_mi: window walk out of bounds (internal error)");
    return MCPG_OK;
}

int ap_mi_from_ranks(mcpg_handle* h, const int32_t* R, int64_t n, int64_t m, int64_t ldr, float* MI, int64_t ldmi,
                     int* flag, unsigned* counter) {
    const int64_t ldc = round_up(m + 1, 8);
    void* tab;
    int rc = scratch(h, S_AP_TAB, (size_t)(n * (2 * m + ldc)) * 2, &tab);
    if (rc) return rc;
    uint16_t* xr = (uint16_t*)tab;
    uint16_t* order = xr + n * m;
    uint16_t* cH = order + n * m;
    {
        PROF(h, "ap_prep");
        CK(h, mcpg::launch_ap_prep(R, n, m, ldr, xr, order, cH, ldc, flag, h->stream, &h->launches), "ap prep");
    }
    {
        PROF(h, "ap_mi");
        CK(h, mcpg::launch_ap_mi(xr, order, cH, ldc, n, m, MI, ldmi, counter, flag, h->stream, &h->launches),
           "ap mi");
    }
    return ap_flag_check(h, flag);
}

int ap_small(mcpg_handle* h, int** flag, unsigned** counter) {
    void* p;
    int rc = scratch(h, S_SMALL, 64, &p);
    if (rc) return rc;
    *flag = (int*)p;
    *counter = (unsigned*)((char*)p + 16);
    CK(h, cudaMemsetAsync(p, 0, 64, h->stream), "memset");
    return MCPG_OK;
}

int ap_mi_dev(mcpg_handle* h, const float* X, int64_t n, int64_t m, int64_t ldx, float noise, uint64_t seed, float* MI,
              int64_t ldmi) {
    int rc = ap_check(h, n, m, X, ldx, MI, ldmi);
    if (rc || n == 0) return rc;
    if (!(noise >= 0.0f)) return fail(h, MCPG_ERR_ARG, "ap_mi: noise amplitude must be >= 0");
    int* flag;
    unsigned* counter;
    if ((rc = ap_small(h, &flag, &counter))) return rc;
    void* r;
    if ((rc = scratch(h, S_AP_R, (size_t)(n * m) * 4, &r))) return rc;
    {
        PROF(h, "ap_ranks");
        CK(h, mcpg::launch_ap_ranks(X, n, m, ldx, noise, seed, (int32_t*)r, m, flag, h->stream, &h->launches),
           "ap ranks");
    }
    return ap_mi_from_ranks(h, (const int32_t*)r, n, m, m, MI, ldmi, flag, counter);
}

}  // namespace

using namespace mcpg_api;

extern "C" {

// ---- MI ----
int mcpg_bspline_mi_dev(mcpg_handle* h, const float* X, int64_t n, int64_t m, int64_t ldx, int bins, int order,
                        int precision, float* MI, int64_t ldmi, double* H) {
    int rc = check_handle(h);
    if (rc) return rc;
    return mi_dev(h, X, n, m, ldx, bins, order, precision, MI, ldmi, H);
}

int mcpg_bspline_mi(mcpg_handle* h, const float* X, int64_t n, int64_t m, int64_t ldx, int bins, int order,
                    int precision, float* MI, int64_t ldmi, double* H) {
    int rc = check_handle(h);
    if (rc) return rc;
    if (!X || !MI) return fail(h, MCPG_ERR_ARG, "bspline_mi: null pointer");
    if (n < 1 || m < 1 || ldx < m || ldmi < n) return fail(h, MCPG_ERR_ARG, "bspline_mi: bad shape");
    float *dX, *dMI;
    int64_t lx, lmi;
    const bool x_direct = host_direct(h, X, span_bytes(n, m, ldx), false);
    const bool mi_direct = host_direct(h, MI, span_bytes(n, n, ldmi), true);
    h->last_direct = (x_direct ? MCPG_HOST_DIRECT_INPUT : 0) | (mi_direct ? MCPG_HOST_DIRECT_OUTPUT : 0);
    if (x_direct) {
        dX = const_cast<float*>(X);
        lx = ldx;
    } else if ((rc = stage_in(h, S_IN0, X, ldx, n, m, &dX, &lx))) {
        return rc;
    }
    if (mi_direct) {
        dMI = MI;
        lmi = ldmi;
    } else if ((rc = stage_out_alloc(h, S_OUT0, n, n, &dMI, &lmi))) {
        return rc;
    }
    double* dH = nullptr;
    if (H) {
        void* p;
        if ((rc = scratch(h, S_H, (size_t)n * sizeof(double), &p))) return rc;
        dH = (double*)p;
    }
    MiPlan pl;
    if ((rc = mi_prepare(h, dX, n, m, lx, bins, order, precision, dMI, lmi, dH, pl))) return rc;
    if (mi_direct) {  // the kernels write the caller's buffer: one launch, nothing to copy back
        if ((rc = mi_launch(h, pl, 0, n))) return rc;
        if ((rc = mi_finish(h, pl))) return rc;
        if (H) CK(h, cudaMemcpyAsync(H, dH, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, h->stream), "copy H");
        return finish(h);
    }
    // Row slabs of 48-gene multiples: once slab k has run, rows < its end are
    // final (row i's j >= i entries come from its own slab, the j < i ones are
    // mirrors written by earlier slabs), so their copy to the host overlaps
    // the next slabs' compute on a second stream.  The tensor-core forms run one
    // whole-matrix launch instead (its packed tiles give the bits the device and
    // in-place paths give; gene-range launches keep 12-gene tiles).
    if (!h->copy_stream) CK(h, cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking), "create stream");
    const int64_t nslab = (n >= 48 * 16 && precision == MCPG_MI_FP32) ? 16 : 1;
    while ((int64_t)h->slab_events.size() < nslab) {
        cudaEvent_t e;
        CK(h, cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "create event");
        h->slab_events.push_back(e);
    }
    int64_t g0 = 0;
    for (int64_t k = 0; k < nslab; ++k) {
        int64_t g1 = (k + 1 == nslab) ? n : ((n * (k + 1) / nslab) / 48) * 48;
        if (g1 <= g0) continue;
        if ((rc = mi_launch(h, pl, g0, g1))) return rc;
        CK(h, cudaEventRecord(h->slab_events[(size_t)k], h->stream), "record event");
        CK(h, cudaStreamWaitEvent(h->copy_stream, h->slab_events[(size_t)k], 0), "stream wait");
        const int64_t r = g1 - g0;
        if (ldmi == n && lmi == n)
            CK(h, cudaMemcpyAsync(MI + g0 * ldmi, dMI + g0 * lmi, (size_t)(r * n) * sizeof(float),
                                  cudaMemcpyDeviceToHost, h->copy_stream),
               "device-to-host copy");
        else
            CK(h, cudaMemcpy2DAsync(MI + g0 * ldmi, ldmi * sizeof(float), dMI + g0 * lmi, lmi * sizeof(float),
                                    n * sizeof(float), r, cudaMemcpyDeviceToHost, h->copy_stream),
               "device-to-host copy");
        g0 = g1;
    }
    if ((rc = mi_finish(h, pl))) return rc;
    if (H) CK(h, cudaMemcpyAsync(H, dH, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, h->stream), "copy H");
    CK(h, cudaStreamSynchronize(h->copy_stream), "copy stream synchronize");
    return finish(h);
}

// Reference-layout weights: W[g*(bins*m+1) + a*m + s], W[g*(bins*m+1) + bins*m] = H_g.
int mcpg_bspline_weights_dev(mcpg_handle* h, const float* X, int64_t n, int64_t m, int64_t ldx, int bins, int order,
                             float* W, double* H) {
    int rc = check_handle(h);
    if (rc) return rc;
    if (!X || !W || n < 1 || m < 1 || ldx < m) return fail(h, MCPG_ERR_ARG, "bspline_weights: bad arguments");
    if (bins < 1 || bins > 32 || order < 1 || order > 8 || bins < order)
        return fail(h, MCPG_ERR_ARG, "bspline_weights: need 1 <= order <= bins <= 32, order <= 8");
    CK(h, mcpg::launch_bspline_weights_ref(X, n, m, ldx, bins, order, W, H, h->stream, &h->launches),
       "bspline weights kernel");
    return MCPG_OK;
}

int mcpg_bspline_weights(mcpg_handle* h, const float* X, int64_t n, int64_t m, int64_t ldx, int bins, int order,
                         float* W, double* H) {
    int rc = check_handle(h);
    if (rc) return rc;
    if (!X || !W || n < 1 || m < 1 || ldx < m) return fail(h, MCPG_ERR_ARG, "bspline_weights: bad arguments");
    float* dX;
    int64_t lx;
    if ((rc = stage_in(h, S_IN0, X, ldx, n, m, &dX, &lx))) return rc;
    const int64_t ldw = (int64_t)bins * m + 1;
    void *dW, *dH = nullptr;
    if ((rc = scratch(h, S_OUT0, (size_t)(n * ldw) * sizeof(float), &dW))) return rc;
    if (H && (rc = scratch(h, S_H, (size_t)n * sizeof(double), &dH))) return rc;
    if ((rc = mcpg_bspline_weights_dev(h, dX, n, m, lx, bins, order, (float*)dW, (double*)dH))) return rc;
    CK(h, cudaMemcpyAsync(W, dW, (size_t)(n * ldw) * sizeof(float), cudaMemcpyDeviceToHost, h->stream), "copy W");
    if (H) CK(h, cudaMemcpyAsync(H, dH, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, h->stream), "copy H");
    return finish(h);
}

int mcpg_bspline_mi_bwd_dev(mcpg_handle* h, const float* X, int64_t n, int64_t m, int64_t ldx, int bins, int order,
                            const float* G, int64_t ldg, float* dX, int64_t lddx) {
    int rc = check_handle(h);
    if (rc) return rc;
    return mi_bwd_dev(h, X, n, m, ldx, bins, order, G, ldg, dX, lddx);
}

int mcpg_bspline_mi_bwd(mcpg_handle* h, const float* X, int64_t n, int64_t m, int64_t ldx, int bins, int order,
                        const float* G, int64_t ldg, float* dX, int64_t lddx) {
    int rc = check_handle(h);
    if (rc) return rc;
    if (n < 1 || m < 1 || !X || !G || !dX || ldx < m || ldg < n || lddx < m)
        return fail(h, MCPG_ERR_ARG, "bspline_mi_bwd: bad arguments");
    float *dXin, *dG, *dOut;
    int64_t lx, lg, lo;
    if ((rc = stage_in(h, S_IN3, X, ldx, n, m, &dXin, &lx))) return rc;
    if ((rc = stage_in(h, S_IN4, G, ldg, n, n, &dG, &lg))) return rc;
    if ((rc = stage_out_alloc(h, S_OUT0, n, m, &dOut, &lo))) return rc;
    if ((rc = mi_bwd_dev(h, dXin, n, m, lx, bins, order, dG, lg, dOut, lo))) return rc;
    if ((rc = copy_out(h, dX, lddx, dOut, lo, n, m))) return rc;
    return finish(h);
}

int mcpg_ap_ranks_dev(mcpg_handle* h, const float* X, int64_t n, int64_t m, int64_t ldx, float noise, uint64_t seed,
                      int32_t* R, int64_t ldr) {
    int rc = check_handle(h);
    if (rc) return rc;
    if (n < 0 || m < 0) return fail(h, MCPG_ERR_ARG, "ap_ranks: negative size");
    if (n == 0 || m == 0) return MCPG_OK;
    if (!X || !R || ldx < m || ldr < m) return fail(h, MCPG_ERR_ARG, "ap_ranks: null pointer or leading dimension");
    if (m > mcpg::ap_max_samples())
        return fail(h, MCPG_ERR_UNSUPPORTED, "ap_ranks: at most %lld samples", (long long)mcpg::ap_max_samples());
    if (!(noise >= 0.0f)) return fail(h, MCPG_ERR_ARG, "ap_ranks: noise amplitude must be >= 0");
    int* flag;
    unsigned* counter;
    if ((rc = ap_small(h, &flag, &counter))) return rc;
    {
        PROF(h, "ap_ranks");
        CK(h, mcpg::launch_ap_ranks(X, n, m, ldx, noise, seed, R, ldr, flag, h->stream, &h->launches), "ap ranks");
    }
    return ap_flag_check(h, flag);
}

int mcpg_ap_mi_ranks_dev(mcpg_handle* h, const int32_t* R, int64_t n, int64_t m, int64_t ldr, float* MI,
                         int64_t ldmi) {
    int rc = check_handle(h);
    if (rc) return rc;
    if ((rc = ap_check(h, n, m, R, ldr, MI, ldmi)) || n == 0) return rc;
    int* flag;
    unsigned* counter;
    if ((rc = ap_small(h, &flag, &counter))) return rc;
    return ap_mi_from_ranks(h, R, n, m, ldr, MI, ldmi, flag, counter);
}

int mcpg_ap_mi_ranks(mcpg_handle* h, const int32_t* R, int64_t n, int64_t m, int64_t ldr, float* MI, int64_t ldmi) {
    int rc = check_handle(h);
    if (rc) return rc;
    if ((rc = ap_check(h, n, m, R, ldr, MI, ldmi)) || n == 0) return rc;
    void* r;
    if ((rc = scratch(h, S_AP_R, (size_t)(n * m) * 4, &r))) return rc;
    CK(h, cudaMemcpy2DAsync(r, (size_t)m * 4, R, (size_t)ldr * 4, (size_t)m * 4, (size_t)n, cudaMemcpyHostToDevice,
                            h->stream),
       "host-to-device copy");
    float* dmi;
    int64_t ldd;
    if ((rc = stage_out_alloc(h, S_OUT0, n, n, &dmi, &ldd))) return rc;
    int* flag;
    unsigned* counter;
    if ((rc = ap_small(h, &flag, &counter))) return rc;
    if ((rc = ap_mi_from_ranks(h, (const int32_t*)r, n, m, m, dmi, ldd, flag, counter))) return rc;
    if ((rc = copy_out(h, MI, ldmi, dmi, ldd, n, n))) return rc;
    return finish(h);
}

int mcpg_ap_mi_dev(mcpg_handle* h, const float* X, int64_t n, int64_t m, int64_t ldx, float noise, uint64_t seed,
                   float* MI, int64_t ldmi) {
    int rc = check_handle(h);
    if (rc) return rc;
    return ap_mi_dev(h, X, n, m, ldx, noise, seed, MI, ldmi);
}

int mcpg_ap_mi(mcpg_handle* h, const float* X, int64_t n, int64_t m, int64_t ldx, float noise, uint64_t seed, float* MI,
               int64_t ldmi) {
    int rc = check_handle(h);
    if (rc) return rc;
    if ((rc = ap_check(h, n, m, X, ldx, MI, ldmi)) || n == 0) return rc;
    float* dx;
    int64_t lx;
    const bool x_direct = host_direct(h, X, span_bytes(n, m, ldx), false);
    const bool mi_direct = host_direct(h, MI, span_bytes(n, n, ldmi), true);
    h->last_direct = (x_direct ? MCPG_HOST_DIRECT_INPUT : 0) | (mi_direct ? MCPG_HOST_DIRECT_OUTPUT : 0);
    if (x_direct) {
        dx = const_cast<float*>(X);
        lx = ldx;
    } else if ((rc = stage_in(h, S_IN0, X, ldx, n, m, &dx, &lx))) {
        return rc;
    }
    float* dmi;
    int64_t ldd;
    if (mi_direct) {
        dmi = MI;
        ldd = ldmi;
    } else if ((rc = stage_out_alloc(h, S_OUT0, n, n, &dmi, &ldd))) {
        return rc;
    }
    if ((rc = ap_mi_dev(h, dx, n, m, lx, noise, seed, dmi, ldd))) return rc;
    if (!mi_direct && (rc = copy_out(h, MI, ldmi, dmi, ldd, n, n))) return rc;
    return finish(h);
}

}  // extern "C"
