// C ABI of the mcpgpu library (include/mcpgpu.h): argument checking, device
// scratch management, host<->device staging and the composition of the kernels
// into MCPNet's helper-level operations.  No CPU fallback exists: every
// operation runs the CUDA kernels or returns an error status.
//
// This header is the internal interface shared by the translation units of the C ABI
// (api_core.cpp: handles, streams, profiling and test hooks; api_mi.cpp: B-spline
// and adaptive-partitioning MI and the MI adjoint; api_maxmin.cpp: max-min
// products, MCP, DPI, closure, TF variants and the max-min adjoints; api_eval.cpp:
// ensembles, Stouffer / CLR, the AUPR / AUROC evaluator and the split
// evaluation): the handle, its device scratch slots, error reporting, per-launch
// profiling and host-buffer staging / in-place access.
#pragma once

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

namespace mcpg_api {

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
    S_DPI_PEND,  // two-phase DPI: outputs the first phase left undecided
    S_TCWORK,    // tensor-core MI: the 2-SM form's tile counters
    NSLOTS
};

}  // namespace mcpg_api

using mcpg_api::NSLOTS;

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

namespace mcpg_api {

inline int fail(mcpg_handle* h, int code, const char* fmt, ...) {
    char b[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(b, sizeof b, fmt, ap);
    va_end(ap);
    if (h) h->err = b;
    return code;
}
inline int cuda_fail(mcpg_handle* h, cudaError_t e, const char* what) {
    return fail(h, MCPG_ERR_CUDA, "%s: %s (%s)", what, cudaGetErrorString(e), cudaGetErrorName(e));
}
#define CK(h, expr, what)                                   \
    do {                                                    \
        cudaError_t _e = (expr);                            \
        if (_e != cudaSuccess) return cuda_fail(h, _e, what); \
    } while (0)
// Grow-only scratch slot.
inline int scratch(mcpg_handle* h, int slot, size_t bytes, void** out) {
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
inline int aligned_view(mcpg_handle* h, const float* A, int64_t lda, int64_t rows, int64_t cols, int slot,
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
inline int check_handle(mcpg_handle* h) {
    if (!h) return MCPG_ERR_ARG;
    h->last_direct = 0;  // the host buffers this call addresses in place, if any
    cudaError_t e = cudaSetDevice(h->device);
    if (e != cudaSuccess) return cuda_fail(h, e, "cudaSetDevice");
    return MCPG_OK;
}
// ---------------- staging helpers for the host entry points ----------------
inline bool host_direct(mcpg_handle* h, const void* p, size_t bytes, bool for_write);
inline size_t span_bytes(int64_t rows, int64_t cols, int64_t ld);
inline int stage_in(mcpg_handle* h, int slot, const float* src, int64_t ld_src, int64_t rows, int64_t cols, float** dev,
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
inline int stage_out_alloc(mcpg_handle* h, int slot, int64_t rows, int64_t cols, float** dev, int64_t* ld_dev) {
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
inline int in_view(mcpg_handle* h, int slot, const float* host, int64_t ld_host, int64_t rows, int64_t cols, float** dev,
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
inline int out_view(mcpg_handle* h, int slot, float* host, int64_t ld_host, int64_t rows, int64_t cols, float** dev,
             int64_t* ld_dev) {
    if (host && rows > 0 && cols > 0 && host_direct(h, host, span_bytes(rows, cols, ld_host), true)) {
        *dev = host;
        *ld_dev = ld_host;
        h->last_direct |= MCPG_HOST_DIRECT_OUTPUT;
        return MCPG_OK;
    }
    return stage_out_alloc(h, slot, rows, cols, dev, ld_dev);
}
inline int copy_out(mcpg_handle* h, float* dst, int64_t ld_dst, const float* src, int64_t ld_src, int64_t rows,
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
inline int finish(mcpg_handle* h) {
    CK(h, cudaStreamSynchronize(h->stream), "stream synchronize");
    return MCPG_OK;
}
// ---------------- TF-restricted variants ----------------
struct TfSet {
    std::vector<int> idx;  // positions with value > 0 (the reference's TF test)
    bool pm_inf = true;    // every value is +inf or -inf (a pure TF mask)
};
inline TfSet tf_set(const float* v, int64_t n) {
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
inline bool ats_device(mcpg_handle* h) {
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
inline bool host_direct(mcpg_handle* h, const void* p, size_t bytes, bool for_write) {
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
inline size_t span_bytes(int64_t rows, int64_t cols, int64_t ld) {
    return rows > 0 && cols > 0 ? (size_t)((rows - 1) * ld + cols) * sizeof(float) : 0;
}
inline int upload(mcpg_handle* h, int slot, const void* src, size_t bytes, void** dev) {
    int rc = scratch(h, slot, bytes, dev);
    if (rc) return rc;
    if (bytes) CK(h, cudaMemcpyAsync(*dev, src, bytes, cudaMemcpyHostToDevice, h->stream), "upload");
    return MCPG_OK;
}

}  // namespace mcpg_api
