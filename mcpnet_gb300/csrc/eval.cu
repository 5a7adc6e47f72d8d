// Evaluation of score matrices against a gold standard, as MCPNet's pipeline
// does it (apps/pipeline/mcpnet_helper.hpp:1050-1071 compute_aupr_auroc):
//   * truth selection   select_lower_triangle   mcpnet_helper.hpp:862-891
//                       select_tfs_from_mat     mcpnet_helper.hpp:893-940
//                       select_values2          mcpnet_helper.hpp:947-998
//   * AUPR              aupr_kernel::ordering + average_compute_1sort
//                       include/mcp/transform/aupr.hpp:84-236
//   * AUROC             auroc_kernel::count_le + average_compute_1sort
//                       include/mcp/transform/auroc.hpp:107-252, 562-579
//
// GPU formulation.  Both curves reduce to one primitive: with the smaller
// score set X sorted ascending and every score y of the other set Y placed by
// lower_bound into X (lt[i] = #y strictly between X[i-1] and X[i], eq[i] =
// #y == X[i], both landing on the first index of an equal run), the number of
// Y scores >= the threshold X[f] is |Y| - S[f] - lt[f], S the exclusive prefix
// sum of lt + eq.  One term per distinct threshold then gives
//   AUPR  term = TP / (TP + FP) * (run length / |X|)      (X = positives)
//   AUROC term = (#Y >= t / |Y|) * (run length / |X|)
// exactly as the reference rounds each term; the terms are summed with a
// deterministic compensated reduction instead of the reference's sequential
// loop (the only difference: the order of a double sum).
//
// Scores are compared through an order-preserving 32-bit key of the float
// (-0 folded onto +0, as float comparison treats them); NaN scores are
// rejected through a flag, since the reference's sort has no order for them.
//
// Kernels: truth_count (labels only, 1 byte/entry), truth_gather (order-
// preserving compaction), keys_from_floats / combo_keys, an LSD radix sort
// (4 passes of 8 bits: block histogram, scan, stable warp-match ranked
// scatter), rank_count (binary search in shared memory, aggregated atomics)
// and curve (distinct-threshold terms + reduction).
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"
#include "internal.h"

namespace mcpg {
namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int EV_THREADS = 256;
constexpr int EV_CHUNK = 4096;                       // row segment per block iteration
constexpr int EV_PER_THREAD = EV_CHUNK / EV_THREADS;  // 16
constexpr int SC_THREADS = 1024;                     // scan
constexpr int SC_ITEMS = 4;
constexpr int SC_TILE = SC_THREADS * SC_ITEMS;
constexpr int RS_THREADS = 256;                      // radix sort
constexpr int RS_WARPS = RS_THREADS / 32;
constexpr int RS_ITEMS = 16;
constexpr int RS_TILE = RS_THREADS * RS_ITEMS;
// Directory width and CTAs per SM: 20 bits (a 4 MB directory, L2-resident) and 4 CTAs
// measured best of 16/18/20 bits x 3/4 CTAs on the evaluations of a 32,768-gene network.
#ifndef MCPG_RC_DIR_BITS
#define MCPG_RC_DIR_BITS 20
#endif
#ifndef MCPG_RC_MINB
#define MCPG_RC_MINB 4
#endif
constexpr int RC_DIR_BITS = MCPG_RC_DIR_BITS;        // key prefix bits of the directory of X
constexpr int64_t RC_DIR = ((int64_t)1 << RC_DIR_BITS) + 1;  // its entries
constexpr int RC_SBINS = 4096;                       // histogram bins held in shared memory
constexpr int RC_SLOW = 3072;                        // ... when |X| + 1 > RC_SBINS: the lowest bins
constexpr int RC_SHIGH = RC_SBINS - RC_SLOW;         //     and the highest (scores below / above most of X)
// Keys per thread per step: 8 (with 4 CTAs) measured best of 16 / 8 / 4 keys x 4-6 CTAs per SM on
// a 32,768-gene network (MI 9.8 ms, MCP2 11.6 ms, combo search 8.6 ms per row).
#ifndef MCPG_RC_BATCH
#define MCPG_RC_BATCH 8
#endif
constexpr int RC_BATCH = MCPG_RC_BATCH;              // keys placed per thread per call (divides EV_PER_THREAD)
static_assert(EV_PER_THREAD % RC_BATCH == 0, "rank-count batch");

__device__ __forceinline__ uint32_t order_key(float f) {
    uint32_t u = __float_as_uint(f);
    if ((u & 0x7fffffffu) == 0) u = 0;  // -0 == +0
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ bool is_nan(float f) { return (__float_as_uint(f) & 0x7fffffffu) > 0x7f800000u; }
__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// ---- truth region geometry: item t = (row, 4096-column segment) ----
struct Seg {
    int64_t row, c0, c1;
};
__device__ __forceinline__ Seg item_seg(const TruthRegion& r, int64_t cpr, int64_t t) {
    Seg s;
    s.row = t / cpr;
    s.c0 = (t - s.row * cpr) * EV_CHUNK;
    s.c1 = s.c0 + EV_CHUNK < r.cols ? s.c0 + EV_CHUNK : r.cols;
    if (r.mode == TRUTH_LOWER && s.c1 > s.row) s.c1 = s.row;  // j < min(cols, i)
    return s;
}
__device__ __forceinline__ bool in_region(const TruthRegion& r, int64_t row, int64_t col) {
    if (r.mode != TRUTH_TF) return true;  // lower triangle is bounded by the segment
    const int64_t g = r.row_gene[row];
    return col != g && !(g > col && r.col_tf[col] != 0);
}

__device__ __forceinline__ void block_sum2(uint32_t& a, uint32_t& b, uint32_t* sh /*2*32*/) {
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(FULL, a, o);
        b += __shfl_down_sync(FULL, b, o);
    }
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    if (lane == 0) { sh[w] = a; sh[32 + w] = b; }
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t x = 0, y = 0;
        for (int i = 0; i < nw; ++i) { x += sh[i]; y += sh[32 + i]; }
        a = x;
        b = y;
    }
    __syncthreads();
}

__global__ void __launch_bounds__(EV_THREADS) truth_count_kernel(TruthRegion r, int64_t cpr, int64_t items,
                                                                 uint32_t* cpos, uint32_t* cneg) {
    __shared__ uint32_t sh[64];
    for (int64_t t = blockIdx.x; t < items; t += gridDim.x) {
        const Seg s = item_seg(r, cpr, t);
        uint32_t np = 0, nn = 0;
        const int8_t* lrow = r.labels + s.row * r.ldl;
        for (int k = 0; k < EV_PER_THREAD; ++k) {
            const int64_t col = s.c0 + k * EV_THREADS + threadIdx.x;
            if (col < s.c1 && in_region(r, s.row, col)) {
                const int8_t l = lrow[col];
                np += (l == 1);
                nn += (l == 0);
            }
        }
        block_sum2(np, nn, sh);
        if (threadIdx.x == 0) {
            cpos[t] = np;
            cneg[t] = nn;
        }
    }
}

// ---- exclusive scan (u32 / u64 in, u64 out) ----
__device__ __forceinline__ uint64_t block_excl_scan(uint64_t v, uint64_t* sw /*32*/, uint64_t& total) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    uint64_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const uint64_t y = __shfl_up_sync(FULL, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sw[w] = x;
    __syncthreads();
    if (w == 0) {
        uint64_t t = lane < nw ? sw[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            const uint64_t y = __shfl_up_sync(FULL, t, o);
            if (lane >= o) t += y;
        }
        if (lane < nw) sw[lane] = t;
    }
    __syncthreads();
    const uint64_t before = w > 0 ? sw[w - 1] : 0;
    total = sw[nw - 1];
    __syncthreads();
    return before + x - v;
}

template <typename T>
__global__ void __launch_bounds__(SC_THREADS) scan_tile_sums(const T* in, int64_t n, uint64_t* part) {
    __shared__ uint64_t sw[32];
    const int64_t base = (int64_t)blockIdx.x * SC_TILE + (int64_t)threadIdx.x * SC_ITEMS;
    uint64_t s = 0;
#pragma unroll
    for (int k = 0; k < SC_ITEMS; ++k)
        if (base + k < n) s += (uint64_t)in[base + k];
    uint64_t total;
    block_excl_scan(s, sw, total);
    if (threadIdx.x == 0) part[blockIdx.x] = total;
}

// In-place exclusive scan of the tile sums (one block); the grand total goes to *total_out.
__global__ void __launch_bounds__(SC_THREADS) scan_parts(uint64_t* part, int64_t nb, uint64_t* total_out) {
    __shared__ uint64_t sw[32];
    uint64_t carry = 0;
    for (int64_t c0 = 0; c0 < nb; c0 += SC_TILE) {
        const int64_t base = c0 + (int64_t)threadIdx.x * SC_ITEMS;
        uint64_t v[SC_ITEMS], s = 0;
#pragma unroll
        for (int k = 0; k < SC_ITEMS; ++k) {
            v[k] = base + k < nb ? part[base + k] : 0;
            s += v[k];
        }
        uint64_t total;
        uint64_t run = carry + block_excl_scan(s, sw, total);
#pragma unroll
        for (int k = 0; k < SC_ITEMS; ++k) {
            if (base + k < nb) part[base + k] = run;
            run += v[k];
        }
        carry += total;
    }
    if (threadIdx.x == 0) *total_out = carry;
}

template <typename T>
__global__ void __launch_bounds__(SC_THREADS) scan_tile_down(const T* in, int64_t n, const uint64_t* part,
                                                              uint64_t* out) {
    __shared__ uint64_t sw[32];
    const int64_t base = (int64_t)blockIdx.x * SC_TILE + (int64_t)threadIdx.x * SC_ITEMS;
    uint64_t v[SC_ITEMS], s = 0;
#pragma unroll
    for (int k = 0; k < SC_ITEMS; ++k) {
        v[k] = base + k < n ? (uint64_t)in[base + k] : 0;
        s += v[k];
    }
    uint64_t total;
    uint64_t run = part[blockIdx.x] + block_excl_scan(s, sw, total);
#pragma unroll
    for (int k = 0; k < SC_ITEMS; ++k) {
        if (base + k < n) out[base + k] = run;
        run += v[k];
    }
}

template <typename T>
cudaError_t scan_any(const T* in, int64_t n, uint64_t* out, uint64_t* tmp, cudaStream_t st, int64_t* launches) {
    if (n <= 0) return cudaMemsetAsync(out, 0, sizeof(uint64_t), st);
    const int64_t nb = ceil_div(n, SC_TILE);
    scan_tile_sums<T><<<(unsigned)nb, SC_THREADS, 0, st>>>(in, n, tmp);
    scan_parts<<<1, SC_THREADS, 0, st>>>(tmp, nb, out + n);
    scan_tile_down<T><<<(unsigned)nb, SC_THREADS, 0, st>>>(in, n, tmp, out);
    if (launches) *launches += 3;
    return cudaGetLastError();
}

// ---- order-preserving gather of the selected entries with one label ----
__global__ void __launch_bounds__(EV_THREADS) truth_gather_kernel(TruthRegion r, int64_t cpr, int64_t items, int lab,
                                                                  const uint64_t* off, GatherSrc g, int* nan_flag) {
    __shared__ uint32_t swarp[EV_THREADS / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int64_t t = blockIdx.x; t < items; t += gridDim.x) {
        const Seg s = item_seg(r, cpr, t);
        if (s.c0 >= s.c1 || off[t + 1] == off[t]) continue;  // uniform over the block
        uint64_t pos = off[t];
        const int8_t* lrow = r.labels + s.row * r.ldl;
        bool bad = false;
        for (int k = 0; k < EV_PER_THREAD; ++k) {
            const int64_t col = s.c0 + k * EV_THREADS + threadIdx.x;
            const int8_t l = (col < s.c1 && in_region(r, s.row, col)) ? lrow[col] : (int8_t)-1;
            const bool sel = lab < 0 ? (l == 0 || l == 1) : (l == lab);
            const uint32_t b = __ballot_sync(FULL, sel);
            if (lane == 0) swarp[w] = __popc(b);
            __syncthreads();
            uint32_t before = 0, tot = 0;
#pragma unroll
            for (int i = 0; i < EV_THREADS / 32; ++i) {
                const uint32_t v = swarp[i];
                before += (i < w) ? v : 0;
                tot += v;
            }
            if (sel) {
                const uint64_t p = pos + before + __popc(b & lanemask_lt());
                for (int q = 0; q < g.n; ++q) {
                    const float v = g.src[q][s.row * g.lds[q] + col];
                    bad |= is_nan(v);
                    g.dst[q][p] = v;
                }
                if (g.lab_dst) g.lab_dst[p] = l;
            }
            pos += tot;
            __syncthreads();
        }
        if (bad) atomicOr(nan_flag, 1);
    }
}

__global__ void keys_from_floats_kernel(const float* v, int64_t n, uint32_t* keys, int* nan_flag) {
    bool bad = false;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float f = v[i];
        bad |= is_nan(f);
        keys[i] = order_key(f);
    }
    if (bad) atomicOr(nan_flag, 1);
}

__device__ __forceinline__ float combo_at(const ComboSrc& c, int64_t i) {
    return combo_value_ff(c.g[0][i], c.cs[1] != 0.0 ? c.g[1][i] : 0.0f, c.cs[2] != 0.0 ? c.g[2][i] : 0.0f,
                          c.cs[3] != 0.0 ? c.g[3][i] : 0.0f, c.kc);
}

__global__ void combo_keys_kernel(ComboSrc c, uint32_t* keys, int* nan_flag) {
    bool bad = false;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < c.n; i += (int64_t)gridDim.x * blockDim.x) {
        const float f = combo_at(c, i);
        bad |= is_nan(f);
        keys[i] = order_key(f);
    }
    if (bad) atomicOr(nan_flag, 1);
}

// ---- LSD radix sort of 32-bit keys ----
__global__ void __launch_bounds__(RS_THREADS) radix_hist_kernel(const uint32_t* keys, int64_t n, int shift,
                                                                uint32_t* bh, int64_t nblk) {
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const int64_t base = (int64_t)blockIdx.x * RS_TILE;
#pragma unroll 4
    for (int k = 0; k < RS_ITEMS; ++k) {
        const int64_t i = base + k * RS_THREADS + threadIdx.x;
        if (i < n) atomicAdd(&h[(keys[i] >> shift) & 255u], 1u);
    }
    __syncthreads();
    bh[(int64_t)threadIdx.x * nblk + blockIdx.x] = h[threadIdx.x];  // digit-major: scan gives global offsets
}


// Stable scatter: warp w owns tile elements [w*512, (w+1)*512) read as 16 rows
// of 32 lanes; equal digits are ranked in (row, lane) order with
// __match_any_sync, then offset by the same digit in earlier warps of the block
// and in earlier blocks (the digit-major scanned histogram).
__global__ void __launch_bounds__(RS_THREADS) radix_scatter_kernel(const uint32_t* in, uint32_t* out, int64_t n,
                                                                   int shift, const uint64_t* off, int64_t nblk) {
    __shared__ uint32_t wc[RS_WARPS][256];
    __shared__ uint64_t boff[256];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int d = threadIdx.x; d < RS_WARPS * 256; d += RS_THREADS) (&wc[0][0])[d] = 0;
    boff[threadIdx.x] = off[(int64_t)threadIdx.x * nblk + blockIdx.x];
    __syncthreads();
    const int64_t base = (int64_t)blockIdx.x * RS_TILE + (int64_t)w * (RS_ITEMS * 32);
    uint32_t key[RS_ITEMS], rank[RS_ITEMS];
    const uint32_t lt = lanemask_lt();
#pragma unroll
    for (int k = 0; k < RS_ITEMS; ++k) {
        const int64_t i = base + k * 32 + lane;
        const bool valid = i < n;
        key[k] = valid ? in[i] : 0u;
        const uint32_t act = __ballot_sync(FULL, valid);
        uint32_t peers = 0, d = 0;
        rank[k] = 0;
        if (valid) {
            d = (key[k] >> shift) & 255u;
            peers = __match_any_sync(act, d);
            rank[k] = wc[w][d] + __popc(peers & lt);
        }
        __syncwarp();
        if (valid && lane == __ffs(peers) - 1) wc[w][d] += __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    {   // per digit: exclusive prefix over the warps of this block
        const int d = threadIdx.x;  // RS_THREADS == 256 digits
        uint32_t s = 0;
        for (int q = 0; q < RS_WARPS; ++q) {
            const uint32_t c = wc[q][d];
            wc[q][d] = s;
            s += c;
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < RS_ITEMS; ++k) {
        const int64_t i = base + k * 32 + lane;
        if (i < n) {
            const uint32_t d = (key[k] >> shift) & 255u;
            out[boff[d] + wc[w][d] + rank[k]] = key[k];
        }
    }
}

// ---- rank counting: place every Y score into the sorted X by lower_bound ----
// The directory D[b] = lower_bound(X, b << (32 - RC_DIR_BITS)), b = 0 .. 2^RC_DIR_BITS,
// places a key in one look-up when no X key shares its prefix, and otherwise
// narrows its search to the X keys of that prefix.
__global__ void rank_dir_kernel(const uint32_t* X, int64_t nX, uint32_t* D) {
    for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b < RC_DIR; b += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t key = (uint64_t)b << (32 - RC_DIR_BITS);
        int64_t lo = 0, n = nX;
        while (n > 0) {
            const int64_t half = n >> 1;
            if ((uint64_t)X[lo + half] < key) {
                lo += half + 1;
                n -= half + 1;
            } else {
                n = half;
            }
        }
        D[b] = (uint32_t)lo;
    }
}

struct RankCtx {
    const uint32_t* X;
    int64_t nX;
    uint64_t* lt;
    uint64_t* eq;
    const uint32_t* D;   // directory of X
    uint32_t* shl;       // shared histogram windows (RC_SBINS bins each)
    uint32_t* she;
    int64_t hi0;         // first bin of the high window (bins >= hi0 map to RC_SLOW + bin - hi0)

    // Shared-memory slot of a bin, or -1 for the global histogram.  Scores of
    // the negatives of a network pile up below (or above) most positives, so
    // the windows take the contended bins; with |X| + 1 <= RC_SBINS every bin
    // is in shared memory.
    __device__ __forceinline__ int slot(uint32_t bin) const {
        if ((int64_t)bin < RC_SLOW) return (int)bin;
        if ((int64_t)bin >= hi0) return RC_SLOW + (int)((int64_t)bin - hi0);
        return -1;
    }

    // Places RC_BATCH keys per thread (has[j] false: no key): the directory
    // gives each key's range of X keys with the same prefix, and lower_bound
    // searches those ranges interleaved over the batch (the loads of one step
    // are independent).  Every lane of the warp calls this (ballot / match inside).
    __device__ __forceinline__ void place(const bool (&has)[RC_BATCH], const uint32_t (&key)[RC_BATCH]) const {
        int lo[RC_BATCH], n[RC_BATCH];
#pragma unroll
        for (int j = 0; j < RC_BATCH; ++j) {
            const uint32_t b = key[j] >> (32 - RC_DIR_BITS);
            lo[j] = (int)__ldg(D + b);
            n[j] = has[j] ? (int)__ldg(D + b + 1) - lo[j] : 0;
        }
        for (;;) {
            bool any = false;
#pragma unroll
            for (int j = 0; j < RC_BATCH; ++j) {
                if (n[j] > 0) {
                    const int half = n[j] >> 1;
                    const bool below = __ldg(X + lo[j] + half) < key[j];
                    lo[j] = below ? lo[j] + half + 1 : lo[j];
                    n[j] = below ? n[j] - half - 1 : half;
                    any = true;
                }
            }
            if (!any) break;
        }
#pragma unroll
        for (int j = 0; j < RC_BATCH; ++j) {
            const bool e = has[j] && lo[j] < (int)nX && __ldg(X + lo[j]) == key[j];
            const uint32_t b = (uint32_t)lo[j];
            const uint32_t act = __ballot_sync(FULL, has[j]);
            if (has[j]) {
                const uint32_t peers = __match_any_sync(act, (b << 1) | (e ? 1u : 0u));
                if ((threadIdx.x & 31) == __ffs(peers) - 1) {
                    const uint32_t c = __popc(peers);
                    const int sl = slot(b);
                    if (sl >= 0) atomicAdd(e ? she + sl : shl + sl, c);
                    else atomicAdd((unsigned long long*)(e ? eq + b : lt + b), (unsigned long long)c);
                }
            }
        }
    }
};

struct YMatrix {  // selected entries of one label in a score matrix
    TruthRegion r;
    int64_t cpr, items;
    const float* v;
    int64_t ldv;
    int lab;
    __device__ __forceinline__ bool run(const RankCtx& c) const {
        bool bad = false;
        for (int64_t t = blockIdx.x; t < items; t += gridDim.x) {
            const Seg s = item_seg(r, cpr, t);
            if (s.c0 >= s.c1) continue;  // uniform over the block
            const int8_t* lrow = r.labels + s.row * r.ldl;
            const float* vrow = v + s.row * ldv;
            for (int k0 = 0; k0 < EV_PER_THREAD; k0 += RC_BATCH) {  // the thread's segment, a batch at a time
                bool has[RC_BATCH];
                uint32_t key[RC_BATCH];
#pragma unroll
                for (int k = 0; k < RC_BATCH; ++k) {
                    const int64_t col = s.c0 + (k0 + k) * EV_THREADS + threadIdx.x;
                    has[k] = col < s.c1 && in_region(r, s.row, col) && lrow[col] == lab;
                    const float f = has[k] ? vrow[col] : 0.0f;
                    bad |= has[k] && is_nan(f);
                    key[k] = order_key(f);
                }
                c.place(has, key);
            }
        }
        return bad;
    }
};

struct YKeys {  // a compact array of keys
    const uint32_t* k;
    int64_t n;
    __device__ __forceinline__ bool run(const RankCtx& c) const {
        const int64_t step = (int64_t)gridDim.x * EV_CHUNK;
        for (int64_t i0 = (int64_t)blockIdx.x * EV_CHUNK; i0 < n; i0 += step) {
            for (int k0 = 0; k0 < EV_PER_THREAD; k0 += RC_BATCH) {
                bool has[RC_BATCH];
                uint32_t key[RC_BATCH];
#pragma unroll
                for (int j = 0; j < RC_BATCH; ++j) {
                    const int64_t i = i0 + (k0 + j) * EV_THREADS + threadIdx.x;
                    has[j] = i < n;
                    key[j] = has[j] ? k[i] : 0u;
                }
                c.place(has, key);
            }
        }
        return false;
    }
};

struct YCombo {  // combo values of gathered (mi, M1, M2, M3) tuples
    ComboSrc s;
    __device__ __forceinline__ bool run(const RankCtx& c) const {
        bool bad = false;
        const int64_t step = (int64_t)gridDim.x * EV_CHUNK;
        for (int64_t i0 = (int64_t)blockIdx.x * EV_CHUNK; i0 < s.n; i0 += step) {
            for (int k0 = 0; k0 < EV_PER_THREAD; k0 += RC_BATCH) {
                bool has[RC_BATCH];
                uint32_t key[RC_BATCH];
#pragma unroll
                for (int j = 0; j < RC_BATCH; ++j) {
                    const int64_t i = i0 + (k0 + j) * EV_THREADS + threadIdx.x;
                    has[j] = i < s.n;
                    const float f = has[j] ? combo_at(s, i) : 0.0f;
                    bad |= has[j] && is_nan(f);
                    key[j] = order_key(f);
                }
                c.place(has, key);
            }
        }
        return bad;
    }
};

template <class Y>
__global__ void __launch_bounds__(EV_THREADS, MCPG_RC_MINB) rank_count_kernel(const uint32_t* X, int64_t nX, const uint32_t* D,
                                                                Y y, uint64_t* lt, uint64_t* eq, int* nan_flag) {
    __shared__ uint32_t shl[RC_SBINS], she[RC_SBINS];
    RankCtx c;
    c.X = X;
    c.nX = nX;
    c.lt = lt;
    c.eq = eq;
    c.D = D;
    c.shl = shl;
    c.she = she;
    c.hi0 = nX + 1 <= RC_SBINS ? (int64_t)RC_SLOW : nX + 1 - RC_SHIGH;
    const int nsb = nX + 1 <= RC_SBINS ? (int)(nX + 1) : RC_SBINS;  // used slots
    for (int i = threadIdx.x; i < RC_SBINS; i += blockDim.x) shl[i] = she[i] = 0;
    __syncthreads();
    const bool bad = y.run(c);
    if (bad) atomicOr(nan_flag, 1);
    __syncthreads();
    for (int i = threadIdx.x; i < nsb; i += blockDim.x) {
        const int64_t bin = i < RC_SLOW ? i : c.hi0 + (i - RC_SLOW);
        if (shl[i]) atomicAdd((unsigned long long*)(lt + bin), (unsigned long long)shl[i]);
        if (she[i]) atomicAdd((unsigned long long*)(eq + bin), (unsigned long long)she[i]);
    }
}

// ---- curve terms over the distinct thresholds of X, compensated deterministic sum ----
struct Neu {  // Neumaier compensated sum
    double s = 0.0, c = 0.0;
    __device__ __forceinline__ void add(double x) {
        const double t = __dadd_rn(s, x);
        if (fabs(s) >= fabs(x)) c = __dadd_rn(c, __dadd_rn(__dadd_rn(s, -t), x));
        else c = __dadd_rn(c, __dadd_rn(__dadd_rn(x, -t), s));
        s = t;
    }
    __device__ __forceinline__ void merge(const Neu& o) {
        add(o.s);
        add(o.c);
    }
};

__global__ void add_u32_kernel(const uint32_t* a, const uint32_t* b, int64_t n, uint32_t* out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = a[i] + b[i];
}

// Warps take 32 consecutive positions of [a, b) (the loop bound is uniform over
// a warp), ballot the positives and negatives and append them with one atomic
// per warp and label.
__global__ void split_keys_kernel(const uint32_t* perm, int64_t a, int64_t b, const float* vals, ComboSrc c, int combo,
                                  const int8_t* lab, uint32_t* kp, uint32_t* kn, unsigned long long* cnt,
                                  int* nan_flag) {
    const int lane = threadIdx.x & 31;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    bool bad = false;
    for (int64_t p0 = a + blockIdx.x * (int64_t)blockDim.x + (threadIdx.x & ~31); p0 < b; p0 += stride) {
        const int64_t p = p0 + lane;
        int8_t l = -1;
        float v = 0.0f;
        if (p < b) {
            const int64_t e = perm[p];
            l = lab[e];
            v = combo ? combo_at(c, e) : vals[e];
        }
        const bool isp = l == 1, isn = l == 0;
        bad |= (isp || isn) && is_nan(v);
        const uint32_t bp = __ballot_sync(FULL, isp), bn = __ballot_sync(FULL, isn);
        unsigned long long basep = 0, basen = 0;
        if (lane == 0) {
            if (bp) basep = atomicAdd(&cnt[0], (unsigned long long)__popc(bp));
            if (bn) basen = atomicAdd(&cnt[1], (unsigned long long)__popc(bn));
        }
        basep = __shfl_sync(FULL, basep, 0);
        basen = __shfl_sync(FULL, basen, 0);
        const uint32_t below = lanemask_lt();
        if (isp) kp[basep + __popc(bp & below)] = order_key(v);
        if (isn) kn[basen + __popc(bn & below)] = order_key(v);
    }
    if (bad) atomicOr(nan_flag, 1);
}

__global__ void add_u64_kernel(const uint64_t* a, const uint64_t* b, int64_t n, uint64_t* out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = a[i] + b[i];
}

constexpr int CV_THREADS = 256;
constexpr int CV_MAX_BLOCKS = 256;

__global__ void __launch_bounds__(CV_THREADS) curve_kernel(const uint32_t* X, int64_t nX, int64_t nY,
                                                           const uint64_t* lt, const uint64_t* S, double* part,
                                                           unsigned* ticket, double* out) {
    __shared__ double sh[CV_THREADS / 32][4];
    __shared__ bool last;
    const double invX = __ddiv_rn(1.0, (double)nX);
    const double invY = nY > 0 ? __ddiv_rn(1.0, (double)nY) : 0.0;
    Neu pr, roc;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nX; k += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t x = X[k];
        if (k > 0 && X[k - 1] == x) continue;  // not the first of an equal run
        int64_t lo = k + 1, hi = nX;          // end of the run
        while (lo < hi) {
            const int64_t mid = (lo + hi) >> 1;
            if (X[mid] == x) lo = mid + 1; else hi = mid;
        }
        const double run = __dmul_rn((double)(lo - k), invX);
        const uint64_t ge = (uint64_t)nY - S[k] - lt[k];  // Y scores >= x
        const uint64_t tp = (uint64_t)(nX - k);           // X scores >= x
        pr.add(__dmul_rn(__ddiv_rn((double)tp, (double)(tp + ge)), run));
        roc.add(__dmul_rn(__dmul_rn((double)ge, invY), run));
    }
    // warp, then block, then grid: fixed pairing order, so the result is reproducible
    for (int o = 16; o > 0; o >>= 1) {
        Neu a, b;
        a.s = __shfl_down_sync(FULL, pr.s, o);
        a.c = __shfl_down_sync(FULL, pr.c, o);
        b.s = __shfl_down_sync(FULL, roc.s, o);
        b.c = __shfl_down_sync(FULL, roc.c, o);
        pr.merge(a);
        roc.merge(b);
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) {
        sh[w][0] = pr.s; sh[w][1] = pr.c; sh[w][2] = roc.s; sh[w][3] = roc.c;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        Neu p, r;
        for (int i = 0; i < CV_THREADS / 32; ++i) {
            Neu a, b;
            a.s = sh[i][0]; a.c = sh[i][1]; b.s = sh[i][2]; b.c = sh[i][3];
            p.merge(a);
            r.merge(b);
        }
        double* q = part + 4 * blockIdx.x;
        q[0] = p.s; q[1] = p.c; q[2] = r.s; q[3] = r.c;
        __threadfence();
        last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (last && threadIdx.x == 0) {
        __threadfence();
        Neu p, r;
        for (unsigned i = 0; i < gridDim.x; ++i) {
            Neu a, b;
            a.s = __ldcg(part + 4 * i); a.c = __ldcg(part + 4 * i + 1);
            b.s = __ldcg(part + 4 * i + 2); b.c = __ldcg(part + 4 * i + 3);
            p.merge(a);
            r.merge(b);
        }
        out[0] = __dadd_rn(p.s, p.c);
        out[1] = __dadd_rn(r.s, r.c);
    }
}

unsigned grid_for(int64_t work, int64_t per_block, int64_t cap) {
    int64_t b = ceil_div(work, per_block);
    if (b > cap) b = cap;
    if (b < 1) b = 1;
    return (unsigned)b;
}

}  // namespace

int64_t truth_items(const TruthRegion& r) {
    if (r.rows <= 0 || r.cols <= 0) return 0;
    return r.rows * ceil_div(r.cols, EV_CHUNK);
}
int64_t scan_tmp_elems(int64_t n) { return ceil_div(n > 0 ? n : 1, SC_TILE); }
int64_t radix_blocks(int64_t n) { return ceil_div(n > 0 ? n : 1, RS_TILE); }
int64_t curve_part_elems() { return 4 * CV_MAX_BLOCKS; }
int64_t rank_dir_elems() { return RC_DIR; }

cudaError_t launch_truth_count(const TruthRegion& r, uint32_t* cpos, uint32_t* cneg, cudaStream_t st,
                               int64_t* launches) {
    const int64_t items = truth_items(r);
    if (items == 0) return cudaSuccess;
    truth_count_kernel<<<grid_for(items, 1, 152 * 16), EV_THREADS, 0, st>>>(r, ceil_div(r.cols, EV_CHUNK), items,
                                                                            cpos, cneg);
    if (launches) ++*launches;
    return cudaGetLastError();
}

cudaError_t launch_scan_u32(const uint32_t* in, int64_t n, uint64_t* out, uint64_t* tmp, cudaStream_t st,
                            int64_t* launches) {
    return scan_any<uint32_t>(in, n, out, tmp, st, launches);
}

cudaError_t launch_truth_gather(const TruthRegion& r, int lab, const uint64_t* off, const GatherSrc& g, int* nan_flag,
                                cudaStream_t st, int64_t* launches) {
    const int64_t items = truth_items(r);
    if (items == 0) return cudaSuccess;
    truth_gather_kernel<<<grid_for(items, 1, 152 * 16), EV_THREADS, 0, st>>>(r, ceil_div(r.cols, EV_CHUNK), items,
                                                                             lab, off, g, nan_flag);
    if (launches) ++*launches;
    return cudaGetLastError();
}

cudaError_t launch_add_u32(const uint32_t* a, const uint32_t* b, int64_t n, uint32_t* out, cudaStream_t st,
                           int64_t* launches) {
    if (n <= 0) return cudaSuccess;
    add_u32_kernel<<<grid_for(n, 256, 152 * 8), 256, 0, st>>>(a, b, n, out);
    if (launches) ++*launches;
    return cudaGetLastError();
}

cudaError_t launch_split_keys(const uint32_t* perm, int64_t a, int64_t b, const float* vals, const ComboSrc& c,
                              int combo, const int8_t* lab, uint32_t* kp, uint32_t* kn, unsigned long long* cnt,
                              int* nan_flag, cudaStream_t st, int64_t* launches) {
    if (b <= a) return cudaSuccess;
    split_keys_kernel<<<grid_for(b - a, 256, 152 * 16), 256, 0, st>>>(perm, a, b, vals, c, combo, lab, kp, kn, cnt,
                                                                     nan_flag);
    if (launches) ++*launches;
    return cudaGetLastError();
}

cudaError_t launch_keys_from_floats(const float* v, int64_t n, uint32_t* keys, int* nan_flag, cudaStream_t st,
                                    int64_t* launches) {
    if (n <= 0) return cudaSuccess;
    keys_from_floats_kernel<<<grid_for(n, 256, 152 * 16), 256, 0, st>>>(v, n, keys, nan_flag);
    if (launches) ++*launches;
    return cudaGetLastError();
}

cudaError_t launch_combo_keys(const ComboSrc& c, uint32_t* keys, int* nan_flag, cudaStream_t st, int64_t* launches) {
    if (c.n <= 0) return cudaSuccess;
    combo_keys_kernel<<<grid_for(c.n, 256, 152 * 16), 256, 0, st>>>(c, keys, nan_flag);
    if (launches) ++*launches;
    return cudaGetLastError();
}

cudaError_t launch_radix_sort(uint32_t* keys, uint32_t* alt, int64_t n, uint32_t* bh, uint64_t* bh_off,
                              uint64_t* tmp, cudaStream_t st, int64_t* launches) {
    if (n <= 1) return cudaSuccess;
    const int64_t nblk = radix_blocks(n);
    uint32_t* src = keys;
    uint32_t* dst = alt;
    for (int pass = 0; pass < 4; ++pass) {
        const int shift = 8 * pass;
        radix_hist_kernel<<<(unsigned)nblk, RS_THREADS, 0, st>>>(src, n, shift, bh, nblk);
        cudaError_t e = scan_any<uint32_t>(bh, 256 * nblk, bh_off, tmp, st, launches);
        if (e != cudaSuccess) return e;
        radix_scatter_kernel<<<(unsigned)nblk, RS_THREADS, 0, st>>>(src, dst, n, shift, bh_off, nblk);
        if (launches) *launches += 2;
        uint32_t* t = src;
        src = dst;
        dst = t;
    }
    return cudaGetLastError();  // four passes: the result is back in keys
}

// Zeroes the histograms and builds the directory of X.
static cudaError_t rank_prep(const uint32_t* X, int64_t nX, uint64_t* lt, uint64_t* eq, uint32_t* dir,
                             cudaStream_t st, int64_t* launches) {
    cudaError_t e = cudaMemsetAsync(lt, 0, (size_t)(nX + 1) * sizeof(uint64_t), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(eq, 0, (size_t)(nX + 1) * sizeof(uint64_t), st);
    if (e != cudaSuccess) return e;
    rank_dir_kernel<<<grid_for(RC_DIR, 256, 152 * 2), 256, 0, st>>>(X, nX, dir);
    if (launches) ++*launches;
    return cudaGetLastError();
}

cudaError_t launch_rank_count_matrix(const uint32_t* X, int64_t nX, const TruthRegion& r, const float* v, int64_t ldv,
                                     int lab, uint64_t* lt, uint64_t* eq, uint32_t* dir, int* nan_flag,
                                     cudaStream_t st, int64_t* launches) {
    if (nX <= 0 || nX >= (int64_t)1 << 31) return cudaErrorInvalidValue;
    cudaError_t e = rank_prep(X, nX, lt, eq, dir, st, launches);
    if (e != cudaSuccess) return e;
    const int64_t items = truth_items(r);
    if (items == 0) return cudaSuccess;
    YMatrix y{r, ceil_div(r.cols, EV_CHUNK), items, v, ldv, lab};
    rank_count_kernel<YMatrix><<<grid_for(items, 1, 152 * MCPG_RC_MINB), EV_THREADS, 0, st>>>(X, nX, dir, y, lt, eq, nan_flag);
    if (launches) ++*launches;
    return cudaGetLastError();
}

cudaError_t launch_rank_count_keys(const uint32_t* X, int64_t nX, const uint32_t* Y, int64_t nY, uint64_t* lt,
                                   uint64_t* eq, uint32_t* dir, cudaStream_t st, int64_t* launches) {
    if (nX <= 0 || nX >= (int64_t)1 << 31) return cudaErrorInvalidValue;
    cudaError_t e = rank_prep(X, nX, lt, eq, dir, st, launches);
    if (e != cudaSuccess || nY <= 0) return e;
    YKeys y{Y, nY};
    rank_count_kernel<YKeys><<<grid_for(nY, EV_CHUNK, 152 * MCPG_RC_MINB), EV_THREADS, 0, st>>>(X, nX, dir, y, lt, eq, nullptr);
    if (launches) ++*launches;
    return cudaGetLastError();
}

cudaError_t launch_rank_count_combo(const uint32_t* X, int64_t nX, const ComboSrc& c, uint64_t* lt, uint64_t* eq,
                                    uint32_t* dir, int* nan_flag, cudaStream_t st, int64_t* launches) {
    if (nX <= 0 || nX >= (int64_t)1 << 31) return cudaErrorInvalidValue;
    cudaError_t e = rank_prep(X, nX, lt, eq, dir, st, launches);
    if (e != cudaSuccess || c.n <= 0) return e;
    YCombo y{c};
    rank_count_kernel<YCombo><<<grid_for(c.n, EV_CHUNK, 152 * MCPG_RC_MINB), EV_THREADS, 0, st>>>(X, nX, dir, y, lt, eq,
                                                                                      nan_flag);
    if (launches) ++*launches;
    return cudaGetLastError();
}

cudaError_t launch_curve(const uint32_t* X, int64_t nX, int64_t nY, const uint64_t* lt, const uint64_t* eq,
                         uint64_t* work, uint64_t* tmp, double* part, unsigned* ticket, double* out, cudaStream_t st,
                         int64_t* launches) {
    if (nX <= 0) return cudaErrorInvalidValue;
    uint64_t* sum = work;          // nX
    uint64_t* S = work + nX;       // nX + 1
    add_u64_kernel<<<grid_for(nX, 256, 152 * 8), 256, 0, st>>>(lt, eq, nX, sum);
    cudaError_t e = scan_any<uint64_t>(sum, nX, S, tmp, st, launches);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(ticket, 0, sizeof(unsigned), st);
    if (e != cudaSuccess) return e;
    curve_kernel<<<grid_for(nX, CV_THREADS, CV_MAX_BLOCKS), CV_THREADS, 0, st>>>(X, nX, nY, lt, S, part, ticket, out);
    if (launches) *launches += 2;
    return cudaGetLastError();
}

}  // namespace mcpg
