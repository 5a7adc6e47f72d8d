// B-spline MI (FP32 CUDA-core path) for callers that cannot allocate device
// memory.
//
// Some callers cannot call cudaMalloc: an application whose device memory is
// owned entirely by its own pool allocator (extra cudaMalloc calls fail or
// break its memory budget), or a latency-critical loop that cannot afford the
// implicit device synchronisation and latency of cudaMalloc / cudaFree.  The
// regular entry points keep their weight tables in per-handle scratch that the
// library allocates; this one instead uses one file-scope device array of a
// fixed size, so it allocates nothing.  The caller passes inputs and outputs.
//
// Properties a caller must know:
//  - the array is NOALLOC_SCRATCH_BYTES (32 MiB); every GPU that loads this
//    library holds it until the process exits;
//  - problems whose FP32 weight table (ceil(m/16)*16 x ceil(n/16)*16*bins
//    floats) plus n doubles of marginal entropies exceed it are rejected with
//    MCPG_ERR_SCRATCH_LIMIT before any device work;
//  - the first call on each device looks up the array's device address
//    (cudaGetSymbolAddress) with that device current; make that first call
//    before any stream capture.  The address is kept per device together with
//    the identity of the device's CUDA context: after cudaDeviceReset (or any
//    other teardown of the primary context) the module is loaded again, the
//    array may sit elsewhere, and the next call looks the address up again --
//    so the first call after a reset, too, belongs before any stream capture;
//  - bins must be 2..12 (the compiled FP32 kernels); other values are rejected
//    with MCPG_ERR_ARG before any device work;
//  - every call shares the array and it keeps the last call's contents: the
//    call clears the zero padding it relies on itself, but calls that overlap
//    on the GPU (different streams, or other host threads) race on it.
#include <cuda.h>
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/mcpgpu.h"
#include "internal.h"

namespace {

constexpr size_t NOALLOC_SCRATCH_BYTES = size_t(32) << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

constexpr int MAX_DEVICES = 64;
std::mutex g_mu;
struct CachedAddress {
    void* ptr = nullptr;
    unsigned long long ctx_id = 0;  // identity of the context the address belongs to (0: none yet)
};
CachedAddress g_addr[MAX_DEVICES];

typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long*);

// Identity of the calling thread's current context, 0 when there is none (or the
// driver cannot tell).  Unique for the life of the process, unlike the CUcontext
// handle, which a new context may reuse.
unsigned long long current_context_id() {
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = (CtxGetCurrentFn)p;
        p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = (CtxGetIdFn)p;
    });
    if (!get_current || !get_id) return 0;
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (get_current(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, &id) != CUDA_SUCCESS) return 0;
    return id;
}

// Device address of the scratch array on the current device.  Looked up once per
// device and context: a different (or no) current context means the device was
// reset since, and the address is looked up again with the device current.
cudaError_t scratch_address(void** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= MAX_DEVICES) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_mu);
    CachedAddress& c = g_addr[dev];
    const unsigned long long id = current_context_id();
    if (!c.ptr || id == 0 || id != c.ctx_id) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);  // makes the device's primary context current
        if (e != cudaSuccess) return e;
        c.ptr = p;
        c.ctx_id = current_context_id();
    }
    *out = c.ptr;
    return cudaSuccess;
}

inline int64_t round_up(int64_t a, int64_t b) { return (a + b - 1) / b * b; }

}  // namespace

extern "C" int mcpg_bspline_mi_fp32_noalloc(const float* X, int64_t n, int64_t m, int64_t ldx, int bins, int order,
                                            float* MI, int64_t ldmi, double* H, void* stream) {
    if (!X || !MI || n < 1 || m < 1 || ldx < m || ldmi < n) return MCPG_ERR_ARG;
    if (bins < 2 || bins > 12 || order < 1 || order > 8 || bins < order) return MCPG_ERR_ARG;
    const int64_t ldwt = round_up(n, 16) * bins;
    const int64_t m_pad = round_up(m, 16);
    const size_t wt_bytes = (size_t)round_up(m_pad * ldwt * (int64_t)sizeof(float), 256);
    const size_t h_bytes = H ? 0 : (size_t)n * sizeof(double);
    if (wt_bytes + h_bytes > NOALLOC_SCRATCH_BYTES) return MCPG_ERR_SCRATCH_LIMIT;
    void* base = nullptr;
    if (scratch_address(&base) != cudaSuccess) {
        cudaGetLastError();
        return MCPG_ERR_CUDA;
    }
    cudaStream_t s = (cudaStream_t)stream;
    float* Wt = (float*)base;
    double* Hd = H ? H : (double*)((unsigned char*)base + wt_bytes);
    // the sample and gene padding of the weight table must read as zero
    if (cudaMemsetAsync(Wt, 0, wt_bytes, s) != cudaSuccess) return MCPG_ERR_CUDA;
    if (mcpg::launch_bspline_weights_fp32(X, n, m, ldx, bins, order, Wt, ldwt, Hd, s, nullptr) != cudaSuccess)
        return MCPG_ERR_CUDA;
    if (mcpg::launch_mi_fp32(Wt, ldwt, Hd, n, m, bins, MI, ldmi, s, nullptr) != cudaSuccess) return MCPG_ERR_CUDA;
    return MCPG_OK;
}
