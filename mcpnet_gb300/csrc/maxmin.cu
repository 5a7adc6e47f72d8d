// Max-min ("maximum-capacity path") products and their fused epilogues.
//
//   C[i][j] = max_k min(A[i][k], B[j][k])
//
// is the whole-matrix form of mcp2_maxmin_kernel<float,false,true>
// (include/mcp/filter/mcp.hpp:72-93) applied by splash InnerProduct(A, B), with
// max_of_pairmin_scalar (include/mcp/filter/simd_maxmin.hpp:30-46) as the
// per-pair reduction.  It is a selection semiring: no rounding anywhere, so the
// result is bit-exact for NaN-free inputs whatever the reduction order.
//
// Kernel shape (FP32 ALU bound, no tensor cores):
//  - CTA tile 128 x 128 outputs, 256 threads, 8 x 8 outputs per thread held in
//    registers; k staged through shared memory in 64-wide slices by a 2-stage
//    cp.async pipeline (operand rows are k-contiguous in HBM, so no transpose).
//  - inner step per thread and 4 k: 16 LDS.128 feed 64 x 2 x (min, min, max3):
//    1.5 FP32 min/max instructions per (i, j, k) triple using the sm_100+
//    3-input max.  (BK 64 / 2 stages / LDS.128 measured best on GB300 of
//    BK 16/32/64, 2-4 stages, LDS.64/128: at n = 20,000 BK 32 / 3 stages ran
//    670.9 ms, BK 64 / 2 stages 656.0 ms; half as many barriers and loader
//    rounds per min/max instruction.  A 512-thread 8 x 4 thread tile, twice the
//    resident warps at 128 registers, ran 665.4 ms.)
//  - fused epilogues: MCP ratio (combine.hpp:210-222), closure step
//    B <- max(B, B (x) B) with a changed flag, DPI mask + apply
//    (dpi.hpp:56-68, threshold.hpp:46-53) with the y in {x, z} exclusion done
//    on the k slices that overlap the tile's rows or columns.
//  - symmetric mode (A == B): only tiles on/above the diagonal run; each writes
//    its tile and the mirrored tile, as InnerProduct<..., SYMM=true> does.
#include <float.h>
#include <math.h>

#include "common.cuh"
#include "internal.h"

namespace mcpg {
namespace {

#ifndef MCPG_MM_BK
#define MCPG_MM_BK 64
#endif
#ifndef MCPG_MM_STAGES
#define MCPG_MM_STAGES 2
#endif
#ifndef MCPG_MM_MINB
#define MCPG_MM_MINB 1
#endif
#ifndef MCPG_MM_KSTEP
#define MCPG_MM_KSTEP 4
#endif
#ifndef MCPG_MM_TN
#define MCPG_MM_TN 8
#endif
// Thread tile 8 x TN: 16 threads down the tile's rows, BN / TN across its columns.
constexpr int TN = MCPG_MM_TN;
constexpr int BM = 128, BN = 128, BK = MCPG_MM_BK, STAGES = MCPG_MM_STAGES, THREADS = 16 * (BN / TN);
constexpr int TXS = BN / TN;  // column step between a thread's outputs
constexpr int NTXB = TXS / 8; // column blocks of 8 threads per warp row
constexpr int KSTEP = MCPG_MM_KSTEP;  // k values per shared-memory load (2: LDS.64, 4: LDS.128)
constexpr int LDS = BK + 4;  // row stride in floats: 16B-aligned, 4 consecutive rows -> 4 distinct bank groups
constexpr int TILE_FLOATS = BM * LDS;
constexpr size_t SMEM_BYTES = (size_t)STAGES * 2 * TILE_FLOATS * sizeof(float);  // 136 KB

// Per-thread view of the operand rows it stages: with CPR = BK/4 chunks of 16
// bytes per row, thread t copies chunk q = t % CPR of rows t / CPR + h * RSTEP
// (h < HPT) of both operand tiles.
constexpr int CPR = BK / 4;
constexpr int RSTEP = THREADS / CPR;    // row step between a thread's rows
constexpr int HPT = BM / RSTEP;         // rows per thread per operand
static_assert(HPT * RSTEP == BM && RSTEP * CPR == THREADS && BM == BN, "loader covers the tile");

struct StageLoader {
    const float* a[HPT];
    const float* b[HPT];
    int64_t k_rem;   // k_len - 4q
    uint32_t soff;   // shared offset (floats) of chunk (r, q)
    uint32_t va, vb; // validity bit per row

    __device__ __forceinline__ void init(const MaxminParams& p, int64_t i0, int64_t j0, int tid) {
        const int r = tid / CPR, q = tid % CPR;
        soff = r * LDS + q * 4;
        k_rem = p.k_len - 4 * q;
        va = vb = 0;
#pragma unroll
        for (int h = 0; h < HPT; ++h) {
            const int64_t gi = i0 + r + h * RSTEP, gj = j0 + r + h * RSTEP;
            const bool oka = gi < p.rows, okb = gj < p.cols;
            va |= (uint32_t)oka << h;
            vb |= (uint32_t)okb << h;
            a[h] = oka ? p.A + gi * p.lda + 4 * q : p.A;
            b[h] = okb ? p.B + gj * p.ldb + 4 * q : p.B;
        }
    }
    __device__ __forceinline__ void load(float* As, float* Bs, int64_t k0) const {
        const int64_t rem = k_rem - k0;
        const int kb = rem >= 4 ? 16 : (rem > 0 ? (int)rem * 4 : 0);
#pragma unroll
        for (int h = 0; h < HPT; ++h) {
            const bool oka = (va >> h) & 1u, okb = (vb >> h) & 1u;
            cp_async16(As + soff + h * RSTEP * LDS, oka ? a[h] + k0 : a[h], oka ? kb : 0);
            cp_async16(Bs + soff + h * RSTEP * LDS, okb ? b[h] + k0 : b[h], okb ? kb : 0);
        }
    }
};

__device__ __forceinline__ float ratio_of(float a, float m) {
    // ratio_kernel<float,float> (combine.hpp:210-222).  The reference divides in
    // double and rounds to float; for float operands that double rounding is
    // innocuous (53 >= 2*24+2), so the correctly rounded float quotient is
    // bit-identical.
    return (fabsf(a) < FLT_EPSILON) ? 0.0f : (fabsf(m) < FLT_EPSILON) ? FLT_MAX : __fdiv_rn(a, m);
}

template <int MODE, bool SYMM>
__global__ void __launch_bounds__(THREADS, MCPG_MM_MINB) maxmin_kernel(const MaxminParams p) {
    extern __shared__ float4 smem_f4[];
    float* smem = reinterpret_cast<float*>(smem_f4);

    int64_t ti = blockIdx.y, tj = blockIdx.x;
    if (SYMM && tj < ti) return;
    const int64_t i0 = ti * BM, j0 = tj * BN;
    const bool mirror = SYMM && (tj != ti);

    const int tid = threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;
    const int ty = ((warp / NTXB) << 2) + (lane >> 3);  // 0..15
    const int tx = ((warp % NTXB) << 3) + (lane & 7);   // 0..TXS-1

    // DPI: NaN is the neutral element of the NaN-ignoring max, so an output with
    // no admissible y stays NaN and compares false (the reference keeps it).
    constexpr bool DPI1 = (MODE == MM_DPI1);
    constexpr bool EXCL = (MODE == MM_DPI || MODE == MM_EXCL || DPI1);
    constexpr bool WIT = (MODE == MM_WITNESS);
    constexpr bool GEMM = (MODE == MM_GEMM);
    const float init = EXCL ? __int_as_float(0x7fc00000) : (GEMM ? 0.0f : -INFINITY);
    int32_t kidx[WIT ? 8 : 1][WIT ? TN : 1];
    if (WIT) {
#pragma unroll
        for (int q = 0; q < (WIT ? 8 : 1); ++q)
#pragma unroll
            for (int r = 0; r < (WIT ? TN : 1); ++r) kidx[q][r] = -1;
    }
    // excluded k per owned row / column (EXCL modes)
    int64_t exr[8], exc[TN];
    if (EXCL) {
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int64_t i = i0 + ty + 16 * q;
            exr[q] = p.excl_row ? (i < p.rows ? (int64_t)p.excl_row[i] : -1) : i;
        }
#pragma unroll
        for (int r = 0; r < TN; ++r) {
            const int64_t j = j0 + tx + TXS * r;
            exc[r] = p.excl_col ? (j < p.cols ? (int64_t)p.excl_col[j] : -1) : j;
        }
    }
    float acc[8][TN];
#pragma unroll
    for (int q = 0; q < 8; ++q)
#pragma unroll
        for (int r = 0; r < TN; ++r) acc[q][r] = init;

    StageLoader ld;
    ld.init(p, i0, j0, tid);
    const int64_t ktiles = ceil_div(p.k_len, BK);
#pragma unroll
    for (int s = 0; s < STAGES - 1; ++s) {
        if (s < ktiles) ld.load(smem + s * 2 * TILE_FLOATS, smem + s * 2 * TILE_FLOATS + TILE_FLOATS, (int64_t)s * BK);
        cp_async_commit();
    }

    for (int64_t t = 0; t < ktiles; ++t) {
        cp_async_wait<STAGES - 2>();
        __syncthreads();
        {
            const int64_t tn = t + STAGES - 1;
            if (tn < ktiles) {
                float* st = smem + (tn % STAGES) * 2 * TILE_FLOATS;
                ld.load(st, st + TILE_FLOATS, tn * BK);
            }
            cp_async_commit();
        }
        const float* As = smem + (t % STAGES) * 2 * TILE_FLOATS;
        const float* Bs = As + TILE_FLOATS;
        const float* a_base = As + ty * LDS;
        const float* b_base = Bs + tx * LDS;
        const int64_t k0 = t * BK;
        const int64_t kmax = min((int64_t)BK, p.k_len - k0);
        bool excl = false;
        if (EXCL) {
            excl = (p.excl_row || p.excl_col) ||
                   (k0 < i0 + BM && k0 + BK > i0) || (k0 < j0 + BN && k0 + BK > j0);
        }
        if (kmax == BK && !excl) {
            if (WIT || GEMM) {
#pragma unroll
                for (int kk = 0; kk < BK; kk += 4) {
                    float4 a[8];
#pragma unroll
                    for (int q = 0; q < 8; ++q) a[q] = *reinterpret_cast<const float4*>(a_base + q * 16 * LDS + kk);
#pragma unroll
                    for (int r = 0; r < TN; ++r) {
                        const float4 b = *reinterpret_cast<const float4*>(b_base + r * TXS * LDS + kk);
#pragma unroll
                        for (int q = 0; q < 8; ++q) {
                            if (GEMM) {
                                float t = fmaf(a[q].x, b.x, acc[q][r]);
                                t = fmaf(a[q].y, b.y, t);
                                t = fmaf(a[q].z, b.z, t);
                                acc[q][r] = fmaf(a[q].w, b.w, t);
                            } else {
                                // first k attaining the running maximum (strict >)
                                const int32_t y0 = (int32_t)(k0 + kk);
                                const float v0 = fmin2(a[q].x, b.x), v1 = fmin2(a[q].y, b.y);
                                const float v2 = fmin2(a[q].z, b.z), v3 = fmin2(a[q].w, b.w);
                                if (v0 > acc[q][r]) { acc[q][r] = v0; kidx[WIT ? q : 0][WIT ? r : 0] = y0; }
                                if (v1 > acc[q][r]) { acc[q][r] = v1; kidx[WIT ? q : 0][WIT ? r : 0] = y0 + 1; }
                                if (v2 > acc[q][r]) { acc[q][r] = v2; kidx[WIT ? q : 0][WIT ? r : 0] = y0 + 2; }
                                if (v3 > acc[q][r]) { acc[q][r] = v3; kidx[WIT ? q : 0][WIT ? r : 0] = y0 + 3; }
                            }
                        }
                    }
                }
            } else if (KSTEP == 2) {
#pragma unroll
                for (int kk = 0; kk < BK; kk += 2) {
                    float2 a[8];
#pragma unroll
                    for (int q = 0; q < 8; ++q) a[q] = *reinterpret_cast<const float2*>(a_base + q * 16 * LDS + kk);
#pragma unroll
                    for (int r = 0; r < TN; ++r) {
                        const float2 b = *reinterpret_cast<const float2*>(b_base + r * TXS * LDS + kk);
#pragma unroll
                        for (int q = 0; q < 8; ++q)
                            acc[q][r] = fmax3(acc[q][r], fmin2(a[q].x, b.x), fmin2(a[q].y, b.y));
                    }
                }
            } else {
#pragma unroll
                for (int kk = 0; kk < BK; kk += 4) {
                    float4 a[8];
#pragma unroll
                    for (int q = 0; q < 8; ++q) a[q] = *reinterpret_cast<const float4*>(a_base + q * 16 * LDS + kk);
#pragma unroll
                    for (int r = 0; r < TN; ++r) {
                        const float4 b = *reinterpret_cast<const float4*>(b_base + r * TXS * LDS + kk);
#pragma unroll
                        for (int q = 0; q < 8; ++q) {
                            acc[q][r] = fmax3(acc[q][r], fmin2(a[q].x, b.x), fmin2(a[q].y, b.y));
                            acc[q][r] = fmax3(acc[q][r], fmin2(a[q].z, b.z), fmin2(a[q].w, b.w));
                        }
                    }
                }
            }
        } else {
            for (int kk = 0; kk < (int)kmax; ++kk) {
                const int64_t y = k0 + kk;
                float a[8], b[TN];
#pragma unroll
                for (int q = 0; q < 8; ++q) a[q] = a_base[q * 16 * LDS + kk];
#pragma unroll
                for (int r = 0; r < TN; ++r) b[r] = b_base[r * TXS * LDS + kk];
#pragma unroll
                for (int q = 0; q < 8; ++q)
#pragma unroll
                    for (int r = 0; r < TN; ++r) {
                        if (GEMM) {
                            acc[q][r] = fmaf(a[q], b[r], acc[q][r]);
                            continue;
                        }
                        float v = fmin2(a[q], b[r]);
                        if (WIT) {
                            if (v > acc[q][r]) { acc[q][r] = v; kidx[WIT ? q : 0][WIT ? r : 0] = (int32_t)y; }
                            continue;
                        }
                        if (EXCL) {
                            if (y == exr[q] || y == exc[r]) v = __int_as_float(0x7fc00000);
                        }
                        acc[q][r] = fmax2(acc[q][r], v);
                    }
            }
        }
    }
    cp_async_wait<0>();

    // ---------------- epilogue ----------------
    int any_changed = 0;
    unsigned long long removed = 0;
    uint64_t pend0 = 0, pend1 = 0;  // MM_DPI1: outputs (and mirrors) the first phase left undecided
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const int64_t i = i0 + ty + 16 * q;
        if (i >= p.rows) continue;
#pragma unroll
        for (int r = 0; r < TN; ++r) {
            const int64_t j = j0 + tx + TXS * r;
            if (j >= p.cols) continue;
            const float m = acc[q][r];
            if (MODE == MM_PLAIN || MODE == MM_EXCL || MODE == MM_GEMM) {
                p.C[i * p.ldc + j] = m;
                if (mirror) p.C[j * p.ldc + i] = m;
            } else if (MODE == MM_WITNESS) {
                const int32_t kw = kidx[WIT ? q : 0][WIT ? r : 0];
                p.C[i * p.ldc + j] = m;
                p.K[i * p.ldk + j] = kw;
                if (mirror) {
                    p.C[j * p.ldc + i] = m;
                    p.K[j * p.ldk + i] = kw;
                }
            } else if (MODE == MM_RATIO) {
                p.R[i * p.ldr + j] = ratio_of(p.E[i * p.lde + j], m);
                if (p.C) p.C[i * p.ldc + j] = m;
                if (mirror) {
                    p.R[j * p.ldr + i] = ratio_of(p.E[j * p.lde + i], m);
                    if (p.C) p.C[j * p.ldc + i] = m;
                }
            } else if (MODE == MM_CLOSURE) {
                const float e = p.E[i * p.lde + j];
                const float v = (e < m) ? m : e;  // std::max(e, m)
                p.C[i * p.ldc + j] = v;
                any_changed |= (v != e);
                if (mirror) {
                    const float e2 = p.E[j * p.lde + i];
                    const float v2 = (e2 < m) ? m : e2;
                    p.C[j * p.ldc + i] = v2;
                    any_changed |= (v2 != e2);
                }
            } else {  // MM_DPI; MM_DPI1 writes only what the first phase decides (deleted)
                const int64_t oi = p.perm ? (int64_t)p.perm[i] : i, oj = p.perm ? (int64_t)p.perm[j] : j;
                {
                    const float e = p.E[i * p.lde + j];
                    const float ixz = p.tm_float ? __fmul_rn(e, p.tol_mult_f) : (float)((double)e * p.tol_mult);
                    const bool del = (i == j) || (m >= ixz);
                    if (!DPI1 || del) {
                        const float o = del ? 0.0f : e;
                        p.C[oi * p.ldc + oj] = o;
                        removed += (o != e);
                        if (p.mask) p.mask[oi * p.ldmask + oj] = del ? 1 : 0;
                    } else {
                        pend0 |= 1ull << (q * TN + r);
                    }
                }
                if (mirror) {
                    const float e = p.E[j * p.lde + i];
                    const float ixz = p.tm_float ? __fmul_rn(e, p.tol_mult_f) : (float)((double)e * p.tol_mult);
                    const bool del = (m >= ixz);
                    if (!DPI1 || del) {
                        const float o = del ? 0.0f : e;
                        p.C[oj * p.ldc + oi] = o;
                        removed += (o != e);
                        if (p.mask) p.mask[oj * p.ldmask + oi] = del ? 1 : 0;
                    } else {
                        pend1 |= 1ull << (q * TN + r);
                    }
                }
            }
        }
    }
    if (MODE == MM_CLOSURE) {
        if (__syncthreads_or(any_changed) && tid == 0) atomicOr(p.changed, 1);
    }
    if (DPI1) {
        // append the undecided outputs: one atomic per warp, then each lane writes its own
        const uint64_t any = pend0 | pend1;
        const unsigned cnt = (unsigned)__popcll(any);
        unsigned incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        unsigned long long base = 0;
        if (lane == 31 && incl) base = atomicAdd(p.pending_n, (unsigned long long)incl);
        base = __shfl_sync(0xffffffffu, base, 31);
        if (any) {
            unsigned long long idx = base + incl - cnt;
#pragma unroll
            for (int q = 0; q < 8; ++q)
#pragma unroll
                for (int r = 0; r < TN; ++r) {
                    const uint64_t bit = 1ull << (q * TN + r);
                    if (!(any & bit)) continue;
                    if (idx < (unsigned long long)p.pending_cap) {
                        DpiPending d;
                        d.x = (int32_t)(i0 + ty + 16 * q);
                        d.z = (int32_t)(j0 + tx + TXS * r);
                        d.m = acc[q][r];
                        d.flags = ((pend0 & bit) ? 1u : 0u) | ((pend1 & bit) ? 2u : 0u);
                        p.pending[idx] = d;
                    }
                    ++idx;
                }
        }
    }
    if ((MODE == MM_DPI || DPI1) && p.removed) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) removed += __shfl_xor_sync(0xffffffffu, removed, o);
        if (lane == 0 && removed) atomicAdd(p.removed, removed);
    }
}

template <int MODE, bool SYMM>
cudaError_t launch_one(const MaxminParams& p, cudaStream_t stream) {
    auto kern = maxmin_kernel<MODE, SYMM>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_BYTES);
    if (e != cudaSuccess) return e;
    dim3 grid((unsigned)ceil_div(p.cols, BN), (unsigned)ceil_div(p.rows, BM));
    kern<<<grid, THREADS, SMEM_BYTES, stream>>>(p);
    return cudaGetLastError();
}

// ---------------- element-wise helpers ----------------
__global__ void __launch_bounds__(EW_TPB) ratio_kernel_ew(const float* __restrict__ A, int64_t lda,
                                                         const float* __restrict__ M, int64_t ldm, int64_t rows,
                                                         int64_t cols, float* __restrict__ R, int64_t ldr) {
    for_each_entry(rows, cols, [&](int64_t i, int64_t j) { R[i * ldr + j] = ratio_of(A[i * lda + j], M[i * ldm + j]); });
}

__global__ void set_diag_kernel(float* A, int64_t nd, int64_t lda, float v) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < nd) A[i * lda + i] = v;
}

// out = max(M, M^T) through a 32x32 shared-memory tile (max_kernel, combine.hpp:42-58).
__global__ void max_transpose_kernel(const float* M, int64_t n, int64_t ldm, float* out, int64_t ldo) {
    __shared__ float tile[32][33];
    const int64_t bi = (int64_t)blockIdx.y * 32, bj = (int64_t)blockIdx.x * 32;
    // load the transposed block M[bj.., bi..]
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const int64_t gi = bj + r, gj = bi + threadIdx.x;
        tile[r][threadIdx.x] = (gi < n && gj < n) ? M[gi * ldm + gj] : 0.0f;
    }
    __syncthreads();
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const int64_t i = bi + r, j = bj + threadIdx.x;
        if (i < n && j < n) {
            const float a = M[i * ldm + j];
            const float b = tile[threadIdx.x][r];  // = M[j][i]
            out[i * ldo + j] = (a < b) ? b : a;    // std::max(in, aux)
        }
    }
}

__global__ void __launch_bounds__(EW_TPB) copy2d_kernel(const float* __restrict__ src, int64_t lds,
                                                       float* __restrict__ dst, int64_t ldd, int64_t rows,
                                                       int64_t cols) {
    for_each_entry(rows, cols, [&](int64_t i, int64_t j) { dst[i * ldd + j] = src[i * lds + j]; });
}

__global__ void gather_kernel(const float* src, int64_t lds, const int* ri, const int* ci, int64_t rows, int64_t cols,
                              float* dst, int64_t ldd) {
    for_each_entry(rows, cols, [&](int64_t r, int64_t c) {
        const int64_t sr = ri ? ri[r] : r, sc = ci ? ci[c] : c;
        dst[r * ldd + c] = src[sr * lds + sc];
    });
}

__global__ void fold_mask_kernel(const float* src, int64_t lds, const float* mask, int64_t rows, int64_t cols,
                                 float* dst, int64_t ldd) {
    for_each_entry(rows, cols, [&](int64_t r, int64_t c) {
        const float a = src[r * lds + c], mk = mask[c];
        dst[r * ldd + c] = (mk < a) ? mk : a;  // min(a, mask[c]); min is exact, so folding the mask
                                               // into one operand equals the reference's 3-way min
    });
}

__global__ void dpi_tf_apply_kernel(const float* A, int64_t lda, const float* Call, int64_t ld1, const float* Ctf,
                                    int64_t ld2, const uint8_t* tf, int64_t n, float tm, float* out, int64_t ldo,
                                    uint8_t* mask, unsigned long long* removed) {
    unsigned long long cnt = 0;
    for_each_entry(n, n, [&](int64_t x, int64_t z) {
        const float e = A[x * lda + z];
        const float ixz = __fmul_rn(e, tm);  // dpi_tf_kernel keeps its multiplier in IT (float)
        const bool tfxz = (tf[x] != 0) != (tf[z] != 0);
        const float c = tfxz ? Ctf[x * ld2 + z] : Call[x * ld1 + z];
        const bool del = (x == z) || (c >= ixz);
        const float o = del ? 0.0f : e;
        out[x * ldo + z] = o;
        cnt += (o != e);
        if (mask) mask[x * n + z] = del ? 1 : 0;
    });
    if (removed) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
        if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(removed, cnt);
    }
}

__global__ void maxmin_route_kernel(const float* A, int64_t lda, const float* B, int64_t ldb, int64_t rows,
                                    int64_t cols, int64_t k, const float* C, int64_t ldc, const float* dC,
                                    int64_t lddc, const int32_t* K, int64_t ldk, float* dA, int64_t ldda, float* dB,
                                    int64_t lddb) {
    for_each_entry(rows, cols, [&](int64_t i, int64_t j) {
        const float g = dC[i * lddc + j];
        if (g == 0.0f) return;
        int64_t ks = -1;
        if (K) {
            ks = K[i * ldk + j];
        } else {
            const float c = C[i * ldc + j];
            if (c > -INFINITY)
                for (int64_t q = 0; q < k; ++q)
                    if (fmin2(A[i * lda + q], B[j * ldb + q]) == c) {
                        ks = q;
                        break;
                    }
        }
        if (ks < 0) return;
        const float a = A[i * lda + ks], b = B[j * ldb + ks];
        if (a <= b) atomicAdd(dA + i * ldda + ks, g);  // std::min(a, b) returns a on a tie
        else atomicAdd(dB + j * lddb + ks, g);
    });
}

__global__ void ratio_bwd_kernel(const float* A, int64_t lda, const float* M, int64_t ldm, int64_t rows, int64_t cols,
                                 const float* dR, int64_t lddr, float* dA, int64_t ldda, float* dM, int64_t lddm) {
    for_each_entry(rows, cols, [&](int64_t i, int64_t j) {
        const float a = A[i * lda + j], m = M[i * ldm + j], g = dR[i * lddr + j];
        if (g == 0.0f || fabsf(a) < FLT_EPSILON || fabsf(m) < FLT_EPSILON) return;
        dA[i * ldda + j] += g / m;
        dM[i * lddm + j] -= g * a / (m * m);
    });
}

// Second phase of the two-phase DPI: one warp per pending pair continues
// dpi_kernel's scan (dpi.hpp:56-68) over the intermediates y in [k0, n), 128 per
// step (float4 per lane, rows x and z coalesced), and stops as soon as the running
// max-min reaches every undecided orientation's threshold -- the reference's own
// early exit, at warp granularity.  Excluded y (x and z) contribute NaN, which the
// NaN-ignoring max drops, exactly as in the tiled kernel.
// TF form (dpi_tf_kernel, dpi.hpp:74-110, on P A P^T with the t TFs first): a pair
// with exactly one TF admits only TF intermediates, i.e. y < t.
__global__ void __launch_bounds__(256) dpi_pending_kernel(const float* __restrict__ A, int64_t lda, int64_t n,
                                                          int64_t k0, const DpiPending* __restrict__ list,
                                                          int64_t count, double tm, float* __restrict__ out,
                                                          int64_t ldo, uint8_t* __restrict__ mask, int64_t ldmask,
                                                          unsigned long long* removed, const DpiPendingTf tf) {
    const int lane = threadIdx.x & 31;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const float qnan = __int_as_float(0x7fc00000);
    unsigned long long cnt = 0;
    for (int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < count; w += nw) {
        const DpiPending d = list[w];
        const int64_t x = d.x, z = d.z;
        const float* rx = A + x * lda;
        const float* rz = A + z * lda;
        const float exz = rx[z], ezx = rz[x];
        const float t0 = tf.tm_float ? __fmul_rn(exz, tf.tol_mult_f) : (float)((double)exz * tm);
        const float t1 = tf.tm_float ? __fmul_rn(ezx, tf.tol_mult_f) : (float)((double)ezx * tm);
        const int64_t kend = (tf.tsplit >= 0 && ((x < tf.tsplit) != (z < tf.tsplit))) ? tf.tsplit : n;
        const bool u0 = (d.flags & 1u) != 0, u1 = (d.flags & 2u) != 0;
        const float target = u0 ? (u1 ? fmaxf(t0, t1) : t0) : t1;
        float mm = d.m;
        for (int64_t y0 = k0; y0 < kend; y0 += 128) {
            const int64_t y = y0 + 4 * lane;
            if (y + 3 < kend) {
                const float4 a = __ldg(reinterpret_cast<const float4*>(rx + y));
                const float4 b = __ldg(reinterpret_cast<const float4*>(rz + y));
                const float v0 = (y == x || y == z) ? qnan : fmin2(a.x, b.x);
                const float v1 = (y + 1 == x || y + 1 == z) ? qnan : fmin2(a.y, b.y);
                const float v2 = (y + 2 == x || y + 2 == z) ? qnan : fmin2(a.z, b.z);
                const float v3 = (y + 3 == x || y + 3 == z) ? qnan : fmin2(a.w, b.w);
                mm = fmax2(fmax2(mm, v0), fmax2(v1, fmax2(v2, v3)));
            } else {
                for (int64_t c = y; c < kend && c < y + 4; ++c)
                    if (c != x && c != z) mm = fmax2(mm, fmin2(rx[c], rz[c]));
            }
            if (__any_sync(0xffffffffu, mm >= target)) break;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) mm = fmax2(mm, __shfl_xor_sync(0xffffffffu, mm, o));
        if (lane == 0) {
            const int64_t ox = tf.perm ? (int64_t)tf.perm[x] : x, oz = tf.perm ? (int64_t)tf.perm[z] : z;
            if (u0) {
                const bool del = mm >= t0;
                const float o = del ? 0.0f : exz;
                out[ox * ldo + oz] = o;
                cnt += (o != exz);
                if (mask) mask[ox * ldmask + oz] = del ? 1 : 0;
            }
            if (u1) {
                const bool del = mm >= t1;
                const float o = del ? 0.0f : ezx;
                out[oz * ldo + ox] = o;
                cnt += (o != ezx);
                if (mask) mask[oz * ldmask + ox] = del ? 1 : 0;
            }
        }
    }
    if (removed) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
        if (lane == 0 && cnt) atomicAdd(removed, cnt);
    }
}

// compute_combo (mcpnet_helper.hpp:507-573): combo_value_ff gives the
// reference's double-precision result, mostly without the FP64 pipe.
__global__ void __launch_bounds__(EW_TPB) combo_kernel(const float* __restrict__ mi, int64_t ldm,
                                                      const float* __restrict__ M1, int64_t ld1,
                                                      const float* __restrict__ M2, int64_t ld2,
                                                      const float* __restrict__ M3, int64_t ld3, int64_t rows,
                                                      int64_t cols, const ComboCoef k, float* __restrict__ out,
                                                      int64_t ldo) {
    for_each_entry(rows, cols, [&](int64_t i, int64_t j) {
        const float v = mi[i * ldm + j];
        const float m1 = k.kind[1] ? M1[i * ld1 + j] : 0.0f;
        const float m2 = k.kind[2] ? M2[i * ld2 + j] : 0.0f;
        const float m3 = k.kind[3] ? M3[i * ld3 + j] : 0.0f;
        out[i * ldo + j] = combo_value_ff(v, m1, m2, m3, k);
    });
}

}  // namespace

cudaError_t launch_maxmin(const MaxminParams& p, int mode, int symmetric, cudaStream_t stream, int64_t* launches) {
    if (p.rows <= 0 || p.cols <= 0) return cudaSuccess;
    if (launches) ++*launches;
    const bool s = symmetric != 0;
    switch (mode) {
        case MM_PLAIN: return s ? launch_one<MM_PLAIN, true>(p, stream) : launch_one<MM_PLAIN, false>(p, stream);
        case MM_RATIO: return s ? launch_one<MM_RATIO, true>(p, stream) : launch_one<MM_RATIO, false>(p, stream);
        case MM_CLOSURE: return s ? launch_one<MM_CLOSURE, true>(p, stream) : launch_one<MM_CLOSURE, false>(p, stream);
        case MM_DPI: return s ? launch_one<MM_DPI, true>(p, stream) : launch_one<MM_DPI, false>(p, stream);
        case MM_EXCL: return s ? launch_one<MM_EXCL, true>(p, stream) : launch_one<MM_EXCL, false>(p, stream);
        case MM_WITNESS:
            return s ? launch_one<MM_WITNESS, true>(p, stream) : launch_one<MM_WITNESS, false>(p, stream);
        case MM_GEMM: return launch_one<MM_GEMM, false>(p, stream);
        case MM_DPI1: return s ? launch_one<MM_DPI1, true>(p, stream) : launch_one<MM_DPI1, false>(p, stream);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_ratio(const float* A, int64_t lda, const float* M, int64_t ldm, int64_t rows, int64_t cols,
                         float* R, int64_t ldr, cudaStream_t stream, int64_t* launches) {
    if (rows <= 0 || cols <= 0) return cudaSuccess;
    if (launches) ++*launches;
    ratio_kernel_ew<<<ew_grid2d(rows, cols), 256, 0, stream>>>(A, lda, M, ldm, rows, cols, R, ldr);
    return cudaGetLastError();
}

cudaError_t launch_dpi_pending(const float* A, int64_t lda, int64_t n, int64_t k0, const DpiPending* list,
                               int64_t count, double tol_mult, float* out, int64_t ldo, uint8_t* mask,
                               int64_t ldmask, unsigned long long* removed, cudaStream_t stream, int64_t* launches,
                               const DpiPendingTf& tf) {
    if (count <= 0 || n <= 0) return cudaSuccess;
    if ((lda % 4) != 0 || ((uintptr_t)A & 15u) || (k0 % 4) != 0) return cudaErrorInvalidValue;
    if (launches) ++*launches;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t want = ceil_div(count, (int64_t)8);  // 8 warps per block
    const int64_t grid = want < (int64_t)sms * 8 ? want : (int64_t)sms * 8;
    dpi_pending_kernel<<<(unsigned)grid, 256, 0, stream>>>(A, lda, n, k0, list, count, tol_mult, out, ldo, mask,
                                                           ldmask, removed, tf);
    return cudaGetLastError();
}

cudaError_t launch_set_diagonal(float* A, int64_t rows, int64_t cols, int64_t lda, float value, cudaStream_t stream,
                                int64_t* launches) {
    const int64_t nd = rows < cols ? rows : cols;
    if (nd <= 0 || value < 0.0f) return cudaSuccess;
    if (launches) ++*launches;
    set_diag_kernel<<<(unsigned)ceil_div(nd, 256), 256, 0, stream>>>(A, nd, lda, value);
    return cudaGetLastError();
}

cudaError_t launch_max_transpose(const float* M, int64_t n, int64_t ldm, float* out, int64_t ldo, cudaStream_t stream,
                                 int64_t* launches) {
    if (n <= 0) return cudaSuccess;
    if (launches) ++*launches;
    dim3 grid((unsigned)ceil_div(n, 32), (unsigned)ceil_div(n, 32));
    max_transpose_kernel<<<grid, dim3(32, 8), 0, stream>>>(M, n, ldm, out, ldo);
    return cudaGetLastError();
}

cudaError_t launch_gather(const float* src, int64_t lds, const int* ri, const int* ci, int64_t rows, int64_t cols,
                          float* dst, int64_t ldd, cudaStream_t stream, int64_t* launches) {
    if (rows <= 0 || cols <= 0) return cudaSuccess;
    if (launches) ++*launches;
    gather_kernel<<<ew_grid2d(rows, cols), 256, 0, stream>>>(src, lds, ri, ci, rows, cols, dst, ldd);
    return cudaGetLastError();
}

cudaError_t launch_fold_mask(const float* src, int64_t lds, const float* mask, int64_t rows, int64_t cols, float* dst,
                             int64_t ldd, cudaStream_t stream, int64_t* launches) {
    if (rows <= 0 || cols <= 0) return cudaSuccess;
    if (launches) ++*launches;
    fold_mask_kernel<<<ew_grid2d(rows, cols), 256, 0, stream>>>(src, lds, mask, rows, cols, dst, ldd);
    return cudaGetLastError();
}

cudaError_t launch_dpi_tf_apply(const float* A, int64_t lda, const float* Call, int64_t ld1, const float* Ctf,
                                int64_t ld2, const uint8_t* tf, int64_t n, float tm, float* out, int64_t ldo,
                                uint8_t* mask, unsigned long long* removed, cudaStream_t stream, int64_t* launches) {
    if (n <= 0) return cudaSuccess;
    if (launches) ++*launches;
    dpi_tf_apply_kernel<<<ew_grid2d(n, n), 256, 0, stream>>>(A, lda, Call, ld1, Ctf, ld2, tf, n, tm, out, ldo, mask,
                                                             removed);
    return cudaGetLastError();
}

cudaError_t launch_maxmin_route(const float* A, int64_t lda, const float* B, int64_t ldb, int64_t rows, int64_t cols,
                                int64_t k, const float* C, int64_t ldc, const float* dC, int64_t lddc,
                                const int32_t* K, int64_t ldk, float* dA, int64_t ldda, float* dB, int64_t lddb,
                                cudaStream_t stream, int64_t* launches) {
    if (rows <= 0 || cols <= 0) return cudaSuccess;
    if (launches) ++*launches;
    maxmin_route_kernel<<<ew_grid2d(rows, cols), 256, 0, stream>>>(A, lda, B, ldb, rows, cols, k, C, ldc, dC, lddc, K,
                                                                   ldk, dA, ldda, dB, lddb);
    return cudaGetLastError();
}

cudaError_t launch_ratio_bwd(const float* A, int64_t lda, const float* M, int64_t ldm, int64_t rows, int64_t cols,
                             const float* dR, int64_t lddr, float* dA, int64_t ldda, float* dM, int64_t lddm,
                             cudaStream_t stream, int64_t* launches) {
    if (rows <= 0 || cols <= 0) return cudaSuccess;
    if (launches) ++*launches;
    ratio_bwd_kernel<<<ew_grid2d(rows, cols), 256, 0, stream>>>(A, lda, M, ldm, rows, cols, dR, lddr, dA, ldda, dM,
                                                                lddm);
    return cudaGetLastError();
}

cudaError_t launch_combo(const float* mi, int64_t ldm, const float* M1, int64_t ld1, const float* M2, int64_t ld2,
                         const float* M3, int64_t ld3, int64_t rows, int64_t cols, const double* cs, float* out,
                         int64_t ldo, cudaStream_t stream, int64_t* launches) {
    if (rows <= 0 || cols <= 0) return cudaSuccess;
    if (launches) ++*launches;
    combo_kernel<<<ew_grid2d(rows, cols), 256, 0, stream>>>(mi, ldm, M1, ld1, M2, ld2, M3, ld3, rows, cols,
                                                            make_combo_coef(cs), out, ldo);
    return cudaGetLastError();
}

cudaError_t launch_copy2d(const float* src, int64_t lds, float* dst, int64_t ldd, int64_t rows, int64_t cols,
                          cudaStream_t stream) {
    if (rows <= 0 || cols <= 0) return cudaSuccess;
    copy2d_kernel<<<ew_grid2d(rows, cols), 256, 0, stream>>>(src, lds, dst, ldd, rows, cols);
    return cudaGetLastError();
}

}  // namespace mcpg
