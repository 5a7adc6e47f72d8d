// Adaptive-partitioning MI (MCPNet's default MI method), GPU form of
//   rank transform            splash::kernel::Rank<T, size_t, 0, false> as called by
//                             apps/pipeline/mcpnet_helper.hpp:122-131 (descending; the splash
//                             source is absent: tied values share the lowest rank here)
//   cumulative histograms     IntegralCumulativeHistogramKernel
//                             include/mcp/correlation/AdaptivePartitioningMI.hpp:414-438
//   per-pair MI               AdaptivePartitionRankMIKernel2::operator() (:535-648) over the
//                             symmetric InnerProduct (mcpnet_helper.hpp:152-163)
//
// Layout (all per gene, rows of n): xr = ranks (uint16), order = sample indices
// sorted by rank (uint16), cH = cumulative rank histogram, m + 1 entries
// (uint16; cH[k] = samples with rank < k).  m <= 16384.
//
// ap_mi_kernel: persistent blocks take the next X gene i from a global
// counter; X's ranks sit in shared memory; each warp takes the next Y gene
// j >= i and walks the reference's window quadtree for the pair:
//   * x ranks grouped by y rank: xg[k] = xr[order_Y[k]] (warp-private shared)
//   * a window's four sub-window counts come from one warp-strided scan of
//     its y band, reduced with redux.sync
//   * the chi-square split test `fl(S / e) > 7.815` is decided exactly in
//     128-bit integers (S and e are exact in double, so only the rounding of
//     the quotient matters, and it is reproduced against the midpoint of
//     7.815 and its successor)
//   * the depth-first order of the reference (a LIFO of pushed windows) is
//     kept, leaves are queued in that order; 32 queued leaves are evaluated
//     one per lane (nxy * log2(nxy / (nx*ny)) in double) and added to the sum
//     in queue order, so the sum has the reference's order.
// The only source of difference from the reference is log2 (CUDA's vs the
// C library's, each within an ulp).
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"
#include "internal.h"

namespace mcpg {
namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int AP_MAX_M = 16384;
constexpr int AP_STACK = 64;   // the LIFO holds at most 3 * depth + 1 <= 46 windows for m <= 16384
constexpr int AP_LEAVES = 32;
constexpr int AP_WARPS = 8;

__device__ __forceinline__ uint32_t order_key_desc(float f) {
    uint32_t u = __float_as_uint(f);
    if ((u & 0x7fffffffu) == 0) u = 0;                      // -0 == +0
    u = (u & 0x80000000u) ? ~u : (u | 0x80000000u);          // ascending order key
    return ~u;                                               // descending
}

// splitmix64 of (seed, gene, sample): U[0, amp) noise, the reference's tie breaker
// (mi.cpp:121-131 adds U[0, 1e-5) with its own generator).
__device__ __forceinline__ float noise_at(uint64_t seed, int64_t g, int64_t s, float amp) {
    uint64_t z = seed + 0x9E3779B97F4A7C15ull * (uint64_t)(g * 1000003 + s + 1);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (float)((double)(z >> 40) * (1.0 / 16777216.0)) * amp;
}

// One gene per block iteration: bitonic sort of (descending key, sample) in
// shared memory, rank = first sorted position of the value's tie group.
__global__ void __launch_bounds__(1024, 1) ap_rank_kernel(const float* X, int64_t n, int64_t m, int64_t ldx, float amp,
                                                       uint64_t seed, int32_t* R, int64_t ldr, int* flag) {
    extern __shared__ unsigned long long ap_keys[];
    int64_t mp = 1;
    while (mp < m) mp <<= 1;
    for (int64_t g = blockIdx.x; g < n; g += gridDim.x) {
        bool bad = false;
        for (int64_t s = threadIdx.x; s < mp; s += blockDim.x) {
            unsigned long long k = ~0ull;
            if (s < m) {
                float v = X[g * ldx + s];
                if (amp > 0.0f) v = v + noise_at(seed, g, s, amp);
                bad |= (__float_as_uint(v) & 0x7fffffffu) > 0x7f800000u;
                k = ((unsigned long long)order_key_desc(v) << 32) | (unsigned long long)s;
            }
            ap_keys[s] = k;
        }
        if (bad) atomicOr(flag, 1);
        __syncthreads();
        for (int64_t k = 2; k <= mp; k <<= 1)
            for (int64_t j = k >> 1; j > 0; j >>= 1) {
                for (int64_t i = threadIdx.x; i < mp; i += blockDim.x) {
                    const int64_t ixj = i ^ j;
                    if (ixj > i) {
                        const unsigned long long a = ap_keys[i], b = ap_keys[ixj];
                        if ((a > b) == ((i & k) == 0)) {
                            ap_keys[i] = b;
                            ap_keys[ixj] = a;
                        }
                    }
                }
                __syncthreads();
            }
        for (int64_t p = threadIdx.x; p < m; p += blockDim.x) {
            const unsigned long long k = ap_keys[p];
            const unsigned long long hi = k & 0xffffffff00000000ull;
            int64_t lo = 0, up = p;  // first position whose value equals this one
            while (lo < up) {
                const int64_t mid = (lo + up) >> 1;
                if ((ap_keys[mid] & 0xffffffff00000000ull) < hi) lo = mid + 1; else up = mid;
            }
            R[g * ldr + (int64_t)(k & 0xffffffffull)] = (int32_t)lo;
        }
        __syncthreads();
    }
}

// Ranks -> uint16 ranks, the cumulative histogram and the samples ordered by rank.
__global__ void __launch_bounds__(1024) ap_prep_kernel(const int32_t* R, int64_t n, int64_t m, int64_t ldr,
                                                       uint16_t* xr, uint16_t* order, uint16_t* cH, int64_t ldc,
                                                       int* flag) {
    extern __shared__ uint32_t ap_cnt[];  // m + 1 counts, then m + 1 fill cursors
    uint32_t* fillc = ap_cnt + (m + 1);
    __shared__ uint32_t wsum[32];
    for (int64_t g = blockIdx.x; g < n; g += gridDim.x) {
        for (int64_t k = threadIdx.x; k <= m; k += blockDim.x) ap_cnt[k] = fillc[k] = 0;
        __syncthreads();
        bool bad = false;
        for (int64_t s = threadIdx.x; s < m; s += blockDim.x) {
            const int32_t r = R[g * ldr + s];
            if (r < 0 || r >= m) { bad = true; continue; }
            atomicAdd(&ap_cnt[r], 1u);
            xr[g * m + s] = (uint16_t)r;
        }
        if (bad) atomicOr(flag, 1);
        __syncthreads();
        // exclusive scan of ap_cnt[0..m] in place: each thread owns a contiguous chunk
        const int64_t chunk = ceil_div(m + 1, blockDim.x);
        const int64_t c0 = threadIdx.x * chunk;
        const int64_t c1 = c0 + chunk < m + 1 ? c0 + chunk : m + 1;
        uint32_t local = 0;
        for (int64_t k = c0; k < c1; ++k) local += ap_cnt[k];
        uint32_t x = local;
        const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(FULL, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) wsum[w] = x;
        __syncthreads();
        if (w == 0) {
            uint32_t t = lane < (int)(blockDim.x >> 5) ? wsum[lane] : 0;
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(FULL, t, o);
                if (lane >= o) t += y;
            }
            wsum[lane] = t;
        }
        __syncthreads();
        uint32_t run = (w > 0 ? wsum[w - 1] : 0) + x - local;
        for (int64_t k = c0; k < c1; ++k) {
            const uint32_t v = ap_cnt[k];
            ap_cnt[k] = run;
            run += v;
        }
        __syncthreads();
        for (int64_t k = threadIdx.x; k <= m; k += blockDim.x) cH[g * ldc + k] = (uint16_t)ap_cnt[k];
        for (int64_t s = threadIdx.x; s < m; s += blockDim.x) {
            const int32_t r = R[g * ldr + s];
            if (r < 0 || r >= m) continue;
            const uint32_t pos = ap_cnt[r] + atomicAdd(&fillc[r], 1u);  // order within a tie is irrelevant
            order[g * m + pos] = (uint16_t)s;
        }
        __syncthreads();
    }
}

struct ApWin {
    uint16_t x1, y1, x2, y2;  // exclusive upper bounds
    uint32_t npts;
};

// fl((sum_q (c_q - n/4)^2) / (n/4)) > 7.815 in IEEE double, decided exactly:
// with A = sum_q (4 c_q - n)^2 the quotient is A / (4n); 7.815 = K * 2^-50 and
// the rounding boundary above it is (2K + 1) * 2^-51 (K odd: a tie rounds up).
__device__ __forceinline__ bool chi_square_above(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t n) {
    const long long d0 = 4ll * c0 - n, d1 = 4ll * c1 - n, d2 = 4ll * c2 - n, d3 = 4ll * c3 - n;
    const unsigned long long A = (unsigned long long)(d0 * d0 + d1 * d1 + d2 * d2 + d3 * d3);
    constexpr unsigned long long K = 8798907771975107ull;  // 7.815 * 2^50, exact
    const unsigned __int128 lhs = (unsigned __int128)A << 49;
    const unsigned __int128 rhs = (unsigned __int128)(2 * K + 1) * n;
    return lhs > rhs || (lhs == rhs && (K & 1));
}

struct ApArgs {
    const uint16_t* xr;
    const uint16_t* order;
    const uint16_t* cH;
    int64_t ldc;
    int64_t n, m;
    float* MI;
    int64_t ldmi;
    unsigned* next_i;
    int* flag;
    int warp_bytes;  // shared bytes per warp
};

__device__ __forceinline__ void ap_flush(const uint32_t* lnxy, const uint32_t* lnxny, int& nleaf, double& mi,
                                         int lane) {
    __syncwarp();
    double t = 0.0;
    if (lane < nleaf) {
        const double nxy = (double)lnxy[lane];
        t = nxy * log2(nxy / (double)lnxny[lane]);
    }
    for (int k = 0; k < nleaf; ++k) mi += __shfl_sync(FULL, t, k);  // queue order = the reference's order
    nleaf = 0;
    __syncwarp();
}

__global__ void __launch_bounds__(AP_WARPS * 32) ap_mi_kernel(ApArgs a) {
    extern __shared__ __align__(16) unsigned char ap_smem[];
    __shared__ int s_i;
    __shared__ int s_next_j;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int m = (int)a.m;
    const int xr_bytes = (int)(((int64_t)m * 2 + 15) / 16 * 16);
    uint16_t* xr = (uint16_t*)ap_smem;
    unsigned char* wbase = ap_smem + xr_bytes + w * a.warp_bytes;
    ApWin* stack = (ApWin*)wbase;
    uint32_t* lnxy = (uint32_t*)(wbase + AP_STACK * sizeof(ApWin));
    uint32_t* lnxny = lnxy + AP_LEAVES;
    uint16_t* xg = (uint16_t*)(lnxny + AP_LEAVES);
    const double logm = log2((double)m);

    for (;;) {
        if (threadIdx.x == 0) {
            s_i = (int)atomicAdd(a.next_i, 1u);
            s_next_j = s_i;
        }
        __syncthreads();
        const int i = s_i;
        if (i >= a.n) break;
        for (int s = threadIdx.x; s < m; s += blockDim.x) xr[s] = a.xr[(int64_t)i * m + s];
        __syncthreads();
        const uint16_t* cX = a.cH + (int64_t)i * a.ldc;
        for (;;) {
            int j = 0;
            if (lane == 0) j = atomicAdd(&s_next_j, 1);
            j = __shfl_sync(FULL, j, 0);
            if (j >= a.n) break;
            const uint16_t* oY = a.order + (int64_t)j * m;
            const uint16_t* cY = a.cH + (int64_t)j * a.ldc;
            for (int k = lane; k < m; k += 32) xg[k] = xr[oY[k]];
            if (lane == 0) stack[0] = ApWin{0, 0, (uint16_t)m, (uint16_t)m, (uint32_t)m};
            __syncwarp();
            int top = 1, nleaf = 0;
            bool root = true, broken = false;
            double mi = 0.0;
            int64_t guard = 0;
            while (top > 0) {
                if (++guard > 16ll * m + 64) {  // cannot happen: every pushed window is smaller than its parent
                    broken = true;
                    break;
                }
                const ApWin wv = stack[top - 1];
                __syncwarp();
                const int mx = (wv.x1 + wv.x2) >> 1, my = (wv.y1 + wv.y2) >> 1;
                const int b0 = cY[wv.y1], b1 = cY[my], b2 = cY[wv.y2];
                uint32_t c0 = 0, c1 = 0, c2 = 0, c3 = 0;
                for (int k = b0 + lane; k < b1; k += 32) {
                    const int x = xg[k];
                    c0 += (x >= wv.x1 && x < mx);
                    c1 += (x >= mx && x < wv.x2);
                }
                for (int k = b1 + lane; k < b2; k += 32) {
                    const int x = xg[k];
                    c2 += (x >= wv.x1 && x < mx);
                    c3 += (x >= mx && x < wv.x2);
                }
                c0 = __reduce_add_sync(FULL, c0);
                c1 = __reduce_add_sync(FULL, c1);
                c2 = __reduce_add_sync(FULL, c2);
                c3 = __reduce_add_sync(FULL, c3);
                --top;
                if (root || chi_square_above(c0, c1, c2, c3, wv.npts)) {
                    const int sx1[4] = {wv.x1, mx, wv.x1, mx}, sx2[4] = {mx, wv.x2, mx, wv.x2};
                    const int sy1[4] = {wv.y1, wv.y1, my, my}, sy2[4] = {my, my, wv.y2, wv.y2};
                    const uint32_t cc[4] = {c0, c1, c2, c3};
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        const bool split = ((sx1[q] + 1) < sx2[q] || (sy1[q] + 1) < sy2[q]) && cc[q] > 2;
                        if (split) {
                            if (top >= AP_STACK) {
                                broken = true;
                                continue;
                            }
                            if (lane == 0)
                                stack[top] = ApWin{(uint16_t)sx1[q], (uint16_t)sy1[q], (uint16_t)sx2[q],
                                                   (uint16_t)sy2[q], cc[q]};
                            ++top;
                        } else if (cc[q] > 0) {
                            if (lane == 0) {
                                lnxy[nleaf] = cc[q];
                                lnxny[nleaf] = (uint32_t)(cX[sx2[q]] - cX[sx1[q]]) * (uint32_t)(cY[sy2[q]] - cY[sy1[q]]);
                            }
                            if (++nleaf == AP_LEAVES) ap_flush(lnxy, lnxny, nleaf, mi, lane);
                        }
                    }
                } else {
                    if (lane == 0) {
                        lnxy[nleaf] = wv.npts;
                        lnxny[nleaf] = (uint32_t)(cX[wv.x2] - cX[wv.x1]) * (uint32_t)(cY[wv.y2] - cY[wv.y1]);
                    }
                    if (++nleaf == AP_LEAVES) ap_flush(lnxy, lnxny, nleaf, mi, lane);
                }
                root = false;
                __syncwarp();
                if (broken) break;
            }
            ap_flush(lnxy, lnxny, nleaf, mi, lane);
            if (lane == 0) {
                float v = (float)(mi / (double)m + logm);
                if (broken) {
                    v = __int_as_float(0x7fc00000);
                    atomicOr(a.flag, 2);
                }
                a.MI[(int64_t)i * a.ldmi + j] = v;
                a.MI[(int64_t)j * a.ldmi + i] = v;
            }
            __syncwarp();
        }
        __syncthreads();
    }
}

}  // namespace

int64_t ap_max_samples() { return AP_MAX_M; }

cudaError_t launch_ap_ranks(const float* X, int64_t n, int64_t m, int64_t ldx, float noise, uint64_t seed,
                            int32_t* R, int64_t ldr, int* flag, cudaStream_t st, int64_t* launches) {
    if (n <= 0 || m <= 0) return cudaSuccess;
    if (m > AP_MAX_M) return cudaErrorNotSupported;
    int64_t mp = 1;
    while (mp < m) mp <<= 1;
    const size_t smem = (size_t)mp * 8;
    cudaError_t e = cudaFuncSetAttribute(ap_rank_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const int threads = mp >= 1024 ? 1024 : (int)(mp < 32 ? 32 : mp);
    const int64_t grid = n < 152 * 2 ? n : 152 * 2;
    ap_rank_kernel<<<(unsigned)grid, threads, smem, st>>>(X, n, m, ldx, noise, seed, R, ldr, flag);
    if (launches) ++*launches;
    return cudaGetLastError();
}

cudaError_t launch_ap_prep(const int32_t* R, int64_t n, int64_t m, int64_t ldr, uint16_t* xr, uint16_t* order,
                           uint16_t* cH, int64_t ldc, int* flag, cudaStream_t st, int64_t* launches) {
    if (n <= 0 || m <= 0) return cudaSuccess;
    if (m > AP_MAX_M) return cudaErrorNotSupported;
    const size_t smem = (size_t)(m + 1) * 2 * sizeof(uint32_t);
    cudaError_t e = cudaFuncSetAttribute(ap_prep_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const int64_t grid = n < 152 * 4 ? n : 152 * 4;
    ap_prep_kernel<<<(unsigned)grid, 512, smem, st>>>(R, n, m, ldr, xr, order, cH, ldc, flag);
    if (launches) ++*launches;
    return cudaGetLastError();
}

cudaError_t launch_ap_mi(const uint16_t* xr, const uint16_t* order, const uint16_t* cH, int64_t ldc, int64_t n,
                         int64_t m, float* MI, int64_t ldmi, unsigned* next_i, int* flag, cudaStream_t st,
                         int64_t* launches) {
    if (n <= 0 || m <= 0) return cudaSuccess;
    if (m > AP_MAX_M) return cudaErrorNotSupported;
    ApArgs a;
    a.xr = xr;
    a.order = order;
    a.cH = cH;
    a.ldc = ldc;
    a.n = n;
    a.m = m;
    a.MI = MI;
    a.ldmi = ldmi;
    a.next_i = next_i;
    a.flag = flag;
    a.warp_bytes = (int)(AP_STACK * sizeof(ApWin) + 2 * AP_LEAVES * sizeof(uint32_t) + ((int64_t)m * 2 + 15) / 16 * 16);
    int dev = 0, sms = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    const size_t xr_bytes = (size_t)((m * 2 + 15) / 16 * 16);
    // warps per block: up to AP_WARPS, as many as the shared memory holds (m = 16384: 5)
    int64_t warps = ((int64_t)optin - 1024 - (int64_t)xr_bytes) / a.warp_bytes;
    if (warps > AP_WARPS) warps = AP_WARPS;
    if (warps < 1) return cudaErrorNotSupported;
    const size_t smem = xr_bytes + (size_t)warps * a.warp_bytes;
    cudaError_t e = cudaFuncSetAttribute(ap_mi_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ap_mi_kernel, (int)warps * 32, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorNotSupported;
    e = cudaMemsetAsync(next_i, 0, sizeof(unsigned), st);
    if (e != cudaSuccess) return e;
    int64_t grid = (int64_t)sms * per_sm;
    if (grid > n) grid = n;
    ap_mi_kernel<<<(unsigned)grid, (unsigned)(warps * 32), smem, st>>>(a);
    if (launches) ++*launches;
    return cudaGetLastError();
}

}  // namespace mcpg
