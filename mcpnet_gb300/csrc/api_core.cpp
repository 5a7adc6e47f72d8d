// C ABI: handle lifetime, streams, status strings, per-launch profiling, the
// host-access policy and the test hooks.
#include "api_internal.h"

using namespace mcpg_api;

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

}  // extern "C"
