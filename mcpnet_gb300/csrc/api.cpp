// C ABI of the mcpgpu library (include/mcpgpu.h): argument checking, device
// scratch management, host<->device staging and the composition of the
// kernels into MCPNet's helper-level operations (compute_mi, compute_mcp2/3/4,
// the DPI filter).  No CPU fallback exists: every operation runs the CUDA
// kernels or returns an error status.
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <numeric>
#include <random>
#include <string>
#include <thread>
#include <vector>

#include <omp.h>
#include <sys/mman.h>
#include <unistd.h>

#include "../../include/mcpgpu.h"
#include "internal.h"

namespace mcpg {
cudaError_t launch_bspline_weights_ref(const float* X, int64_t n, int64_t m, int64_t ldx, int bins, int order,
                                       float* W, double* H, cudaStream_t stream, int64_t* launches);
}

namespace {

enum Slot {
    S_IN0 = 0,   // staged host input / aligned copy of input 0
    S_IN1,       // staged host input 1
    S_OUT0,      // staged output 0
    S_OUT1,      // staged output 1
    S_W0,        // weights (FP32 sample-major or 16-bit hi)
    S_W1,        // weights lo
    S_H,         // marginal entropies (double)
    S_M1,        // intermediate max-min product
    S_M2,        // second intermediate
    S_SMALL,     // flags and counters
    S_MASK,      // staged mask
    S_TFA,       // TF-compacted / mask-folded operand A
    S_TFB,       // TF-compacted operand B
    S_TFIDX,     // TF column indices (int)
    S_TFEX,      // TF exclusion indices / flags
    S_TFROWS,    // TF rows of the MI matrix (tfs_to_genes)
    S_M3,        // third intermediate (TF MCP4)
    S_IN2,       // staged host input 2
    S_Q,         // MI adjoint slab Q
    S_DW,        // MI adjoint dW slab
    S_GS,        // MI adjoint pair sums
    S_IN3,       // staged host input 3
    S_IN4,       // staged host input 4
    S_EV_CNT,    // evaluation: per-item label counts
    S_EV_OFF,    // evaluation: scanned per-item counts
    S_EV_KP,     // evaluation: positive keys
    S_EV_KN,     // evaluation: negative keys
    S_EV_ALT,    // evaluation: radix-sort ping-pong buffer
    S_EV_BH,     // evaluation: radix-sort block histograms
    S_EV_BHOFF,  // evaluation: scanned block histograms
    S_EV_TMP,    // evaluation: scan partials
    S_EV_HIST,   // evaluation: lt / eq histograms and their prefix sums
    S_EV_RED,    // evaluation: flag, curve sums and partials
    S_EV_GP,     // evaluation: gathered positive (mi, M1, M2, M3)
    S_EV_GN,     // evaluation: gathered negative (mi, M1, M2, M3)
    S_EV_LAB,    // evaluation: staged labels
    S_EV_AUX,    // evaluation: staged row_gene / col_tf
    S_AP_R,      // AP MI: int32 ranks
    S_AP_TAB,    // AP MI: uint16 ranks, order and cumulative histograms
    S_ST_STATS,  // Stouffer: row means and standard deviations
    S_ST_A,      // Stouffer ensemble: the combo matrix
    S_ST_B,      // Stouffer ensemble: its transform
    S_SP_VAL,    // split evaluation: the entries' scores (up to four sources) in mask order
    S_SP_LAB,    // split evaluation: the entries' labels
    S_SP_PERM,   // split evaluation: the shuffled entry order
    S_SP_CNT,    // split evaluation: subset counters
    S_SP_ST,     // split evaluation: Stouffer scores of every coefficient row at the entries
    NSLOTS
};

}  // namespace

struct mcpg_handle {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    std::string err;
    int64_t launches = 0;
    void* buf[NSLOTS] = {};
    size_t cap[NSLOTS] = {};
    int fail_allocs = 0;  // test hook: number of upcoming scratch allocations to fail
    mcpg::TcWaitHook tc_hook;  // test hook: wait limit / starved producers of the next tensor-core MI launch
    bool tc_hook_armed = false;
    // host MI: a second stream copies finished row slabs back while later slabs compute
    cudaStream_t copy_stream = nullptr;
    std::vector<cudaEvent_t> slab_events;
    // host entry points: kernels address the caller's buffers in place when the
    // device reads host memory through the host page tables (-1: not queried)
    int ats = -1;
    int host_access = MCPG_HOST_ACCESS_AUTO;
    int last_direct = 0;  // MCPG_HOST_DIRECT_* of the last host call that can use them
    // optional per-kernel timing (mcpg_profile): CUDA events around each launch
    bool prof = false;
    struct Span { const char* name; cudaEvent_t a, b; };
    std::vector<Span> spans;
};

namespace {

int fail(mcpg_handle* h, int code, const char* fmt, ...) {
    char b[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(b, sizeof b, fmt, ap);
    va_end(ap);
    if (h) h->err = b;
    return code;
}

int cuda_fail(mcpg_handle* h, cudaError_t e, const char* what) {
    return fail(h, MCPG_ERR_CUDA, "%s: %s (%s)", what, cudaGetErrorString(e), cudaGetErrorName(e));
}

#define CK(h, expr, what)                                   \
    do {                                                    \
        cudaError_t _e = (expr);                            \
        if (_e != cudaSuccess) return cuda_fail(h, _e, what); \
    } while (0)

// Grow-only scratch slot.
int scratch(mcpg_handle* h, int slot, size_t bytes, void** out) {
    if (bytes == 0) bytes = 16;
    if (h->cap[slot] < bytes) {
        if (h->buf[slot]) {
            cudaStreamSynchronize(h->stream);
            cudaFree(h->buf[slot]);
            h->buf[slot] = nullptr;
            h->cap[slot] = 0;
        }
        if (h->fail_allocs > 0) {
            --h->fail_allocs;
            return fail(h, MCPG_ERR_OOM, "device scratch allocation of %zu bytes failed (injected)", bytes);
        }
        void* p = nullptr;
        cudaError_t e = cudaMalloc(&p, bytes);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return fail(h, MCPG_ERR_OOM, "device scratch allocation of %zu bytes failed: %s", bytes,
                        cudaGetErrorString(e));
        }
        h->buf[slot] = p;
        h->cap[slot] = bytes;
    }
    *out = h->buf[slot];
    return MCPG_OK;
}

inline bool aligned16(const void* p) { return ((uintptr_t)p & 15u) == 0; }
inline int64_t round_up(int64_t a, int64_t b) { return (a + b - 1) / b * b; }

// Returns a device view of a rows x cols float matrix whose rows are 16-byte
// aligned (lda % 4 == 0, base 16-byte aligned), copying into scratch if needed.
int aligned_view(mcpg_handle* h, const float* A, int64_t lda, int64_t rows, int64_t cols, int slot,
                 const float** out, int64_t* ld_out) {
    if (aligned16(A) && (lda % 4) == 0) {
        *out = A;
        *ld_out = lda;
        return MCPG_OK;
    }
    const int64_t ld = round_up(cols > 0 ? cols : 1, 4);
    void* p;
    int rc = scratch(h, slot, (size_t)(rows * ld) * sizeof(float), &p);
    if (rc) return rc;
    CK(h, mcpg::launch_copy2d(A, lda, (float*)p, ld, rows, cols, h->stream), "copy2d");
    *out = (const float*)p;
    *ld_out = ld;
    return MCPG_OK;
}

// Records CUDA events around one launch when profiling is on.
struct ProfScope {
    mcpg_handle* h;
    const char* name;
    cudaEvent_t a = nullptr, b = nullptr;
    ProfScope(mcpg_handle* h_, const char* n) : h(h_), name(n) {
        if (h->prof && cudaEventCreate(&a) == cudaSuccess && cudaEventCreate(&b) == cudaSuccess)
            cudaEventRecord(a, h->stream);
    }
    ~ProfScope() {
        if (a && b) {
            cudaEventRecord(b, h->stream);
            h->spans.push_back({name, a, b});
        }
    }
};
#define PROF(h, name) ProfScope _prof_scope(h, name)

int check_handle(mcpg_handle* h) {
    if (!h) return MCPG_ERR_ARG;
    h->last_direct = 0;  // the host buffers this call addresses in place, if any
    cudaError_t e = cudaSetDevice(h->device);
    if (e != cudaSuccess) return cuda_fail(h, e, "cudaSetDevice");
    return MCPG_OK;
}

// ---------------- staging helpers for the host entry points ----------------
bool host_direct(mcpg_handle* h, const void* p, size_t bytes, bool for_write);
size_t span_bytes(int64_t rows, int64_t cols, int64_t ld);

int stage_in(mcpg_handle* h, int slot, const float* src, int64_t ld_src, int64_t rows, int64_t cols, float** dev,
             int64_t* ld_dev) {
    const int64_t ld = round_up(cols > 0 ? cols : 1, 4);  // 16-byte rows for the vectorised kernels
    void* p;
    int rc = scratch(h, slot, (size_t)(rows * ld) * sizeof(float), &p);
    if (rc) return rc;
    if (rows > 0 && cols > 0) {
        if (ld == cols && ld_src == cols)  // contiguous on both sides: one linear copy
            CK(h, cudaMemcpyAsync(p, src, (size_t)(rows * cols) * sizeof(float), cudaMemcpyHostToDevice, h->stream),
               "host-to-device copy");
        else
            CK(h, cudaMemcpy2DAsync(p, ld * sizeof(float), src, ld_src * sizeof(float), cols * sizeof(float), rows,
                                    cudaMemcpyHostToDevice, h->stream),
               "host-to-device copy");
    }
    *dev = (float*)p;
    *ld_dev = ld;
    return MCPG_OK;
}

int stage_out_alloc(mcpg_handle* h, int slot, int64_t rows, int64_t cols, float** dev, int64_t* ld_dev) {
    const int64_t ld = round_up(cols > 0 ? cols : 1, 4);
    void* p;
    int rc = scratch(h, slot, (size_t)(rows * ld) * sizeof(float), &p);
    if (rc) return rc;
    *dev = (float*)p;
    *ld_dev = ld;
    return MCPG_OK;
}

// A host input matrix that the kernels read exactly once: the caller's buffer
// itself when host_direct allows, else a staged device copy.
int in_view(mcpg_handle* h, int slot, const float* host, int64_t ld_host, int64_t rows, int64_t cols, float** dev,
            int64_t* ld_dev) {
    if (host && rows > 0 && cols > 0 && host_direct(h, host, span_bytes(rows, cols, ld_host), false)) {
        *dev = const_cast<float*>(host);
        *ld_dev = ld_host;
        h->last_direct |= MCPG_HOST_DIRECT_INPUT;
        return MCPG_OK;
    }
    return stage_in(h, slot, host, ld_host, rows, cols, dev, ld_dev);
}

// A host output matrix: the caller's buffer itself when the kernels can write it
// in place (host_direct; the result is written once), else device scratch that
// copy_out brings back.
int out_view(mcpg_handle* h, int slot, float* host, int64_t ld_host, int64_t rows, int64_t cols, float** dev,
             int64_t* ld_dev) {
    if (host && rows > 0 && cols > 0 && host_direct(h, host, span_bytes(rows, cols, ld_host), true)) {
        *dev = host;
        *ld_dev = ld_host;
        h->last_direct |= MCPG_HOST_DIRECT_OUTPUT;
        return MCPG_OK;
    }
    return stage_out_alloc(h, slot, rows, cols, dev, ld_dev);
}

int copy_out(mcpg_handle* h, float* dst, int64_t ld_dst, const float* src, int64_t ld_src, int64_t rows,
             int64_t cols) {
    if (!dst || rows <= 0 || cols <= 0 || dst == src) return MCPG_OK;  // dst == src: written in place
    if (ld_dst == cols && ld_src == cols)
        CK(h, cudaMemcpyAsync(dst, src, (size_t)(rows * cols) * sizeof(float), cudaMemcpyDeviceToHost, h->stream),
           "device-to-host copy");
    else
        CK(h, cudaMemcpy2DAsync(dst, ld_dst * sizeof(float), src, ld_src * sizeof(float), cols * sizeof(float), rows,
                                cudaMemcpyDeviceToHost, h->stream),
           "device-to-host copy");
    return MCPG_OK;
}

int finish(mcpg_handle* h) {
    CK(h, cudaStreamSynchronize(h->stream), "stream synchronize");
    return MCPG_OK;
}

// ---------------- device implementations ----------------
// ---- B-spline MI in three steps: weights (prepare), gene-range launches, finish ----
struct MiPlan {
    int precision = 0, fmt = 0, split = 0, bins = 0;  // split: mcpg::TcMode
    int64_t n = 0, m = 0;
    const void* w0 = nullptr;  // FP32 sample-major or 16-bit hi weights
    const void* w1 = nullptr;  // 16-bit lo weights, or the E4M3 H8 plane (split 2)
    const void* w2 = nullptr;  // E4M3 L8 plane (split 2)
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
    const int64_t ldw = round_up(m, 64);
    const int64_t rows = round_up(n * bins, 256) + 256;  // whole tiles stay in bounds
    // S_W1: the 16-bit lo plane, or the two 8-bit planes H8 | L8 (the same bytes)
    void *hi, *lo = nullptr;
    if ((rc = scratch(h, S_W0, (size_t)(rows * ldw) * 2, &hi))) return rc;
    if (pl.split && (rc = scratch(h, S_W1, (size_t)(rows * ldw) * 2, &lo))) return rc;
    uint8_t* l8 = pl.split == mcpg::TC_F8C ? (uint8_t*)lo + (size_t)(rows * ldw) : nullptr;
    // rows beyond n*bins must be zero (they are read by the last tiles)
    const size_t done = (size_t)(n * bins * ldw), tail = (size_t)((rows - n * bins) * ldw);
    CK(h, cudaMemsetAsync((char*)hi + done * 2, 0, tail * 2, h->stream), "memset weights");
    if (pl.split == mcpg::TC_SPLIT16)
        CK(h, cudaMemsetAsync((char*)lo + done * 2, 0, tail * 2, h->stream), "memset weights");
    if (l8) {
        CK(h, cudaMemsetAsync((char*)lo + done, 0, tail, h->stream), "memset weights");
        CK(h, cudaMemsetAsync(l8 + done, 0, tail, h->stream), "memset weights");
    }
    if (l8) {
        PROF(h, "bspline_weights_f8");
        CK(h, mcpg::launch_bspline_weights_f8(X, n, m, ldx, bins, order, (uint16_t*)hi, (uint8_t*)lo, l8, ldw, pl.H,
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
    pl.w0 = hi; pl.w1 = lo; pl.w2 = l8; pl.ld = ldw; pl.flag = (int*)flag;
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
    cudaError_t e;
    {
        PROF(h, "mi_tc");
        const bool f8 = pl.split == mcpg::TC_F8C;
        const mcpg::TcWaitHook* hook = h->tc_hook_armed ? &h->tc_hook : nullptr;
        h->tc_hook_armed = false;  // one launch only
        e = mcpg::launch_mi_tc((const uint16_t*)pl.w0, f8 ? nullptr : (const uint16_t*)pl.w1,
                               f8 ? (const uint8_t*)pl.w1 : nullptr, (const uint8_t*)pl.w2, pl.ld, pl.H, pl.n, pl.m,
                               pl.bins, pl.fmt, pl.split, pl.MI, pl.ldmi, pl.flag, h->stream, &h->launches, g0, g1,
                               hook);
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
    CK(h, cudaMemsetAsync(cnt, 0, sizeof(unsigned long long), h->stream), "memset counter");
    mcpg::MaxminParams p{};
    p.A = a; p.lda = la; p.B = a; p.ldb = la; p.rows = n; p.cols = n; p.k_len = n;
    p.C = out; p.ldc = ldo; p.E = a; p.lde = la;
    p.tol_mult = 1.0 / (1.0 - (double)tol);  // dpi_kernel ctor, dpi.hpp:47
    p.mask = mask; p.ldmask = n;
    p.removed = (unsigned long long*)cnt;
    {
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


// ---------------- TF-restricted variants ----------------
struct TfSet {
    std::vector<int> idx;  // positions with value > 0 (the reference's TF test)
    bool pm_inf = true;    // every value is +inf or -inf (a pure TF mask)
};

TfSet tf_set(const float* v, int64_t n) {
    TfSet t;
    for (int64_t i = 0; i < n; ++i) {
        if (v[i] > 0.0f) t.idx.push_back((int)i);
        if (!(v[i] == INFINITY || v[i] == -INFINITY)) t.pm_inf = false;
    }
    return t;
}

// ---------------- host buffers addressed in place ----------------
// On a device that reads and writes pageable memory coherently through the
// host's page tables (Grace + Blackwell over NVLink-C2C: ATS), a kernel can use
// the caller's host buffer itself -- no staging copy, no host-to-device or
// device-to-host transfer.  host_direct says whether [p, p + bytes) qualifies:
// every page must be mapped (mincore), and resident, because a first touch by
// the GPU is a slow IOMMU fault; an output whose pages are not yet populated is
// populated writable by the host first (MADV_POPULATE_WRITE leaves the contents
// as they are), in parallel.  Anything else is staged as before.
#ifndef MADV_POPULATE_WRITE
#define MADV_POPULATE_WRITE 23
#endif

bool ats_device(mcpg_handle* h) {
    if (h->ats < 0) {
        int a = 0, b = 0;
        h->ats = (cudaDeviceGetAttribute(&a, cudaDevAttrPageableMemoryAccess, h->device) == cudaSuccess &&
                  cudaDeviceGetAttribute(&b, cudaDevAttrPageableMemoryAccessUsesHostPageTables, h->device) ==
                      cudaSuccess &&
                  a == 1 && b == 1)
                     ? 1
                     : 0;
        cudaGetLastError();
    }
    return h->ats == 1;
}

bool host_direct(mcpg_handle* h, const void* p, size_t bytes, bool for_write) {
    if (h->host_access != MCPG_HOST_ACCESS_AUTO || !p || bytes == 0 || !ats_device(h)) return false;
    const long ps = sysconf(_SC_PAGESIZE);
    if (ps <= 0) return false;
    const uintptr_t page = (uintptr_t)ps;
    const uintptr_t b = (uintptr_t)p & ~(page - 1);
    const uintptr_t e = ((uintptr_t)p + bytes + page - 1) & ~(page - 1);
    std::vector<unsigned char> vec((size_t)((e - b) / page));
    if (mincore((void*)b, (size_t)(e - b), vec.data()) != 0) return false;  // a page is not mapped
    bool resident = true;
    for (unsigned char v : vec)
        if (!(v & 1)) {
            resident = false;
            break;
        }
    if (resident) return true;
    if (!for_write) return false;
    const size_t chunk = (size_t)16 << 20;  // 16 MiB per task, page-aligned
    const int64_t nchunks = (int64_t)(((e - b) + chunk - 1) / chunk);
    int bad = 0;
#pragma omp parallel for schedule(dynamic) reduction(| : bad)
    for (int64_t c = 0; c < nchunks; ++c) {
        const uintptr_t c0 = b + (uintptr_t)c * chunk;
        const uintptr_t c1 = c0 + chunk < e ? c0 + chunk : e;
        if (madvise((void*)c0, (size_t)(c1 - c0), MADV_POPULATE_WRITE) != 0) bad |= 1;
    }
    return bad == 0;
}

// Bytes spanned by a rows x cols float matrix with leading dimension ld.
size_t span_bytes(int64_t rows, int64_t cols, int64_t ld) {
    return rows > 0 && cols > 0 ? (size_t)((rows - 1) * ld + cols) * sizeof(float) : 0;
}

int upload(mcpg_handle* h, int slot, const void* src, size_t bytes, void** dev) {
    int rc = scratch(h, slot, bytes, dev);
    if (rc) return rc;
    if (bytes) CK(h, cudaMemcpyAsync(*dev, src, bytes, cudaMemcpyHostToDevice, h->stream), "upload");
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

// dpi_tf_kernel (dpi.hpp:74-110) over all (x, z), then mask<float,true>.
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
    const float tm = (float)(1.0 / (1.0 - (double)tol));  // dpi_tf_kernel stores it as IT
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

// =====================================================================
extern "C" {

int mcpg_version(void) { return 100; }

const char* mcpg_status_string(int s) {
    switch (s) {
        case MCPG_OK: return "ok";
        case MCPG_ERR_ARG: return "invalid argument";
        case MCPG_ERR_OOM: return "out of memory";
        case MCPG_ERR_CUDA: return "CUDA error";
        case MCPG_ERR_NOT_CONVERGED: return "not converged";
        case MCPG_ERR_UNSUPPORTED: return "unsupported";
        case MCPG_ERR_DEVICE_TIMEOUT: return "device wait timed out";
        case MCPG_ERR_SCRATCH_LIMIT: return "problem exceeds the 32 MiB static scratch of the no-allocation entry point";
        default: return "unknown status";
    }
}

int mcpg_create(mcpg_handle** out, int device) {
    if (!out) return MCPG_ERR_ARG;
    *out = nullptr;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return MCPG_ERR_CUDA;
    }
    if (device < 0 || device >= count) return MCPG_ERR_ARG;
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return MCPG_ERR_CUDA;
    if (prop.major < 10) return MCPG_ERR_UNSUPPORTED;  // built for sm_103a only
    if (cudaSetDevice(device) != cudaSuccess) return MCPG_ERR_CUDA;
    mcpg_handle* h = new (std::nothrow) mcpg_handle;
    if (!h) return MCPG_ERR_OOM;
    h->device = device;
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete h;
        return MCPG_ERR_CUDA;
    }
    h->own_stream = true;
    *out = h;
    return MCPG_OK;
}

int mcpg_destroy(mcpg_handle* h) {
    if (!h) return MCPG_OK;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    mcpg_profile(h, 0);
    for (cudaEvent_t e : h->slab_events) cudaEventDestroy(e);
    if (h->copy_stream) cudaStreamDestroy(h->copy_stream);
    for (int i = 0; i < NSLOTS; ++i)
        if (h->buf[i]) cudaFree(h->buf[i]);
    if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return MCPG_OK;
}

const char* mcpg_last_error(const mcpg_handle* h) { return h ? h->err.c_str() : "null handle"; }

int mcpg_set_stream(mcpg_handle* h, void* s) {
    if (!h) return MCPG_ERR_ARG;
    if (h->own_stream && h->stream) {
        cudaStreamSynchronize(h->stream);
        cudaStreamDestroy(h->stream);
    }
    h->stream = (cudaStream_t)s;
    h->own_stream = false;
    return MCPG_OK;
}

int mcpg_synchronize(mcpg_handle* h) {
    int rc = check_handle(h);
    if (rc) return rc;
    return finish(h);
}

int64_t mcpg_kernel_launches(const mcpg_handle* h) { return h ? h->launches : 0; }

int mcpg_profile(mcpg_handle* h, int enable) {
    if (!h) return MCPG_ERR_ARG;
    for (auto& sp : h->spans) {
        cudaEventDestroy(sp.a);
        cudaEventDestroy(sp.b);
    }
    h->spans.clear();
    h->prof = enable != 0;
    return MCPG_OK;
}

int64_t mcpg_profile_report(mcpg_handle* h, char* buf, int64_t len) {
    if (!h) return MCPG_ERR_ARG;
    if (cudaStreamSynchronize(h->stream) != cudaSuccess) return MCPG_ERR_CUDA;
    std::map<std::string, std::pair<int64_t, double>> agg;
    for (auto& sp : h->spans) {
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, sp.a, sp.b) == cudaSuccess) {
            auto& e = agg[sp.name];
            e.first += 1;
            e.second += ms;
        }
    }
    std::string js = "{";
    bool first = true;
    for (auto& kv : agg) {
        char tmp[256];
        snprintf(tmp, sizeof tmp, "%s\"%s\": {\"launches\": %lld, \"ms\": %.6f}", first ? "" : ", ", kv.first.c_str(),
                 (long long)kv.second.first, kv.second.second);
        js += tmp;
        first = false;
    }
    js += "}";
    if (buf && len > 0) {
        const size_t c = std::min((size_t)(len - 1), js.size());
        memcpy(buf, js.data(), c);
        buf[c] = 0;
    }
    return (int64_t)js.size() + 1;
}

int mcpg_test_fail_allocs(mcpg_handle* h, int count) {
    if (!h) return MCPG_ERR_ARG;
    h->fail_allocs = count;
    return MCPG_OK;
}

int mcpg_test_tc_timeout(mcpg_handle* h, int64_t wait_ns, int starve) {
    if (!h) return MCPG_ERR_ARG;
    if (wait_ns < 1000 || wait_ns > (int64_t)mcpg::TC_WAIT_NS_DEFAULT)
        return fail(h, MCPG_ERR_ARG, "test_tc_timeout: wait_ns must be 1e3..2e9 (got %lld)", (long long)wait_ns);
    h->tc_hook.wait_ns = (unsigned long long)wait_ns;
    h->tc_hook.starve = starve ? 1 : 0;
    h->tc_hook_armed = true;
    return MCPG_OK;
}

int mcpg_set_host_access(mcpg_handle* h, int mode) {
    int rc = check_handle(h);
    if (rc) return rc;
    if (mode != MCPG_HOST_ACCESS_AUTO && mode != MCPG_HOST_ACCESS_STAGED)
        return fail(h, MCPG_ERR_ARG, "set_host_access: unknown mode %d", mode);
    h->host_access = mode;
    return MCPG_OK;
}

int mcpg_last_host_access(const mcpg_handle* h) { return h ? h->last_direct : 0; }

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
    // the next slabs' compute on a second stream.
    if (!h->copy_stream) CK(h, cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking), "create stream");
    const int64_t nslab = n >= 48 * 16 ? 16 : 1;
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


int mcpg_maxmins_dev(mcpg_handle* h, const float* A, int64_t n, int64_t lda, float* M1, int64_t ld1, float* M2,
                     int64_t ld2, float* M3, int64_t ld3, float* R2, int64_t ldr2, float* R3, int64_t ldr3, float* R4,
                     int64_t ldr4) {
    int rc = check_handle(h);
    if (rc) return rc;
    return maxmins_dev(h, A, n, lda, M1, ld1, M2, ld2, M3, ld3, R2, ldr2, R3, ldr3, R4, ldr4);
}


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
