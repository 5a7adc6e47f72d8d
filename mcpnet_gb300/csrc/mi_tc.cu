// Tensor-core B-spline MI (K2) on tcgen05: the all-pairs joint histogram as a
// tiled W W^T contraction over samples, with the entropy and the MI combine
// fused into the epilogue so the (n*bins)^2 joint tables never reach HBM.
//
// Whole-matrix form of BSplineEntropyKernel::entropy2d_simd +
// BSplineMIKernel::operator() (include/mcp/correlation/BSplineMI.hpp:288-315,
// 492-499) under InnerProduct<..., SYMM=true> (mcpnet_helper.hpp:88-98).
//
// Operands: 16-bit weights Whi (and Wlo = round16(w - Whi) for the hi+lo
// split), gene-bin-major rows (row = gene*BINS + bin), K = samples contiguous,
// zero-padded to a multiple of 64.  The split computes
//   P = Whi Whi' + Whi Wlo' + Wlo Whi'      (the lo*lo term is below FP32 noise)
// into one FP32 accumulator.
//
// CTA tile: A = 12 genes (120 of the 128 MMA rows), B = 24 genes (N = 240);
// D = 128 x 240 FP32 in tensor memory (256 columns allocated).
//   warp 0 / one lane : TMA producer (cp.async.bulk.tensor, 128B swizzle, 64-sample slices)
//   warp 1 / one lane : tcgen05.mma issuer (kind::f16, M=128, N=240, K=16)
//   warps 0-3         : epilogue -- tcgen05.ld one row per thread, p*log2(p)
//                       per (row, B gene) in FP32, cross-bin sums and
//                       H_i + H_j - H_ij in FP64, symmetric store.
// Two pipeline stages of 64 samples (92 KB each with the split) are double
// buffered through mbarriers.  Only gene-tile pairs that contain some j >= i
// run; tiles are visited in groups of GI A-tiles so that the A and B tiles in
// flight stay resident in L2.
//
// Every mbarrier wait is bounded (2 s of %globaltimer): on expiry the kernel
// raises *err, stops issuing work, drains what it issued (bounded), frees its
// tensor memory and returns.
#include <cuda.h>
#include <cuda_runtime.h>
#include <math.h>

#include "common.cuh"
#include "internal.h"

namespace mcpg {
namespace {

constexpr int BINS = 10;
constexpr int GA = 12;                 // genes per A tile
constexpr int GBN = 24;                // genes per B tile
constexpr int MROWS = 128;             // MMA M
constexpr int NCOLS = GBN * BINS;      // MMA N = 240
constexpr int BK = 64;                 // samples per stage (128 bytes of 16-bit)
constexpr int STAGES = 2;
constexpr int THREADS = 128;
constexpr int TMEM_COLS = 256;
constexpr int GI = 8;                  // A tiles per rasterization group
constexpr uint32_t A_BYTES = MROWS * BK * 2;   // 16 KB
constexpr uint32_t B_BYTES = NCOLS * BK * 2;   // 30 KB
constexpr int PSTRIDE = GBN + 1;       // epilogue partials row stride (floats)
constexpr unsigned long long WAIT_NS = 2000000000ull;

// ---------------------------------------------------------------- PTX wrappers
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long gtimer() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait: false (and *err raised) if the phase did not complete in WAIT_NS.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, int* err) {
    if (mbar_try(bar, parity)) return true;
    const unsigned long long t0 = gtimer();
    for (;;) {
        for (int i = 0; i < 256; ++i)
            if (mbar_try(bar, parity)) return true;
        if (gtimer() - t0 > WAIT_NS) {
            atomicExch(err, 1);
            return false;
        }
    }
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
        "l"((unsigned long long)map), "r"(x), "r"(y), "r"(bar)
        : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_alloc(uint32_t dst_smem, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst_smem), "r"(ncols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols));
}

// D[tmem] (+)= A[smem] * B[smem]^T, kind::f16, one elected thread.
__device__ __forceinline__ void mma_f16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                        uint32_t accum) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accum));
}
__device__ __forceinline__ void mma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

// 32 lanes x 32 bits, 16 consecutive columns per thread.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, rows of 128 bytes,
// 8-row groups 1024 bytes apart (SBO), descriptor version 1.
__device__ __forceinline__ uint64_t sdesc_sw128(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);          // start address
    d |= (uint64_t)1 << 16;                            // LBO (unused for swizzled K-major)
    d |= (uint64_t)(1024 >> 4) << 32;                  // SBO
    d |= (uint64_t)1 << 46;                            // version
    d |= (uint64_t)2 << 61;                            // SWIZZLE_128B
    return d;
}

// Instruction descriptor, kind::f16: F32 accumulate, A/B fmt (0 = F16, 1 = BF16),
// both K-major, N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t idesc_f16(uint32_t fmt, uint32_t M, uint32_t N) {
    return (1u << 4) | (fmt << 7) | (fmt << 10) | ((N >> 3) << 17) | ((M >> 4) << 24);
}

struct TcArgs {
    const double* H;
    float* MI;
    int64_t ldmi;
    int64_t n;
    int TI, TJ;        // A tiles (12 genes), B tiles (24 genes)
    int ktiles;        // K / 64
    float inv_m;
    uint32_t idesc;
    int* err;
    float* dbg;        // nullable: tile (0, 0) stores its raw 128 x 240 accumulator here
};

// Raw-accumulator dump target for kernel bring-up harnesses (null in the library).
float* g_tc_debug_dump = nullptr;

__device__ __forceinline__ int j_min_for(int I) {
    // first B tile with some j >= i for A tile I: 24 J + 23 >= 12 I
    const int v = 12 * I - 23;
    return v <= 0 ? 0 : (v + 23) / 24;
}

template <bool SPLIT>
__global__ void __launch_bounds__(THREADS, 1)
    mi_tc_kernel(const __grid_constant__ CUtensorMap map_hi, const __grid_constant__ CUtensorMap map_lo,
                 const __grid_constant__ CUtensorMap mapb_hi, const __grid_constant__ CUtensorMap mapb_lo,
                 const TcArgs args) {
    // ---- tile of this CTA: grouped rasterization over the TI x TJ rectangle ----
    const int64_t b = (int64_t)blockIdx.x;
    const int64_t per_group = (int64_t)GI * args.TJ;
    const int g = (int)(b / per_group);
    const int r = (int)(b - (int64_t)g * per_group);
    const int J = r / GI;
    const int I = g * GI + (r - J * GI);
    if (I >= args.TI || J < j_min_for(I)) return;

    extern __shared__ uint8_t smem_raw[];
    const uint32_t raw = smem_u32(smem_raw);
    const uint32_t base = (raw + 1023u) & ~1023u;
    uint8_t* gbase = smem_raw + (base - raw);
    constexpr uint32_t STAGE_BYTES = (SPLIT ? 2 : 1) * (A_BYTES + B_BYTES);
    // layout per stage: A_hi, B_hi, [A_lo, B_lo]
    const uint32_t bar_base = base + STAGES * STAGE_BYTES;  // full[S], empty[S], done
    const uint32_t full0 = bar_base, empty0 = bar_base + 8 * STAGES, done = bar_base + 16 * STAGES;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(gbase + STAGES * STAGE_BYTES + 16 * STAGES + 16);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(full0 + 8 * s, 1);
            mbar_init(empty0 + 8 * s, 1);
        }
        mbar_init(done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if (warp == 0) tmem_alloc(smem_u32(tmem_slot), TMEM_COLS);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *reinterpret_cast<volatile uint32_t*>(tmem_slot);

    const int rowA = I * GA * BINS;
    const int rowB = J * GBN * BINS;
    const int KT = args.ktiles;

    if (warp == 0 && lane == 0) {
        // ---------------- TMA producer ----------------
        bool ok = true;
        for (int kt = 0; kt < KT && ok; ++kt) {
            const int s = kt % STAGES;
            const int u = kt / STAGES;
            if (u > 0) ok = mbar_wait(empty0 + 8 * s, (u - 1) & 1, args.err);
            if (!ok) break;
            const uint32_t st = base + s * STAGE_BYTES;
            mbar_expect_tx(full0 + 8 * s, STAGE_BYTES);
            tma_load_2d(st, &map_hi, kt * BK, rowA, full0 + 8 * s);
            tma_load_2d(st + A_BYTES, &mapb_hi, kt * BK, rowB, full0 + 8 * s);
            if (SPLIT) {
                tma_load_2d(st + A_BYTES + B_BYTES, &map_lo, kt * BK, rowA, full0 + 8 * s);
                tma_load_2d(st + 2 * A_BYTES + B_BYTES, &mapb_lo, kt * BK, rowB, full0 + 8 * s);
            }
        }
        // drain: the last phase issued on each stage must complete before smem goes away
        for (int s = 0; s < STAGES && s < KT; ++s) {
            const int last = ((KT - 1 - s) / STAGES);
            mbar_wait(full0 + 8 * s, last & 1, args.err);
        }
    } else if (warp == 1 && lane == 0) {
        // ---------------- MMA issuer ----------------
        bool ok = true;
        for (int kt = 0; kt < KT && ok; ++kt) {
            const int s = kt % STAGES;
            ok = mbar_wait(full0 + 8 * s, (kt / STAGES) & 1, args.err);
            if (!ok) break;
            tc_fence_after();
            const uint32_t st = base + s * STAGE_BYTES;
#pragma unroll
            for (int k = 0; k < BK / 16; ++k) {
                const uint64_t ahi = sdesc_sw128(st + 32 * k);
                const uint64_t bhi = sdesc_sw128(st + A_BYTES + 32 * k);
                const uint32_t acc0 = (kt > 0 || k > 0) ? 1u : 0u;
                mma_f16(tmem, ahi, bhi, args.idesc, acc0);
                if (SPLIT) {
                    const uint64_t alo = sdesc_sw128(st + A_BYTES + B_BYTES + 32 * k);
                    const uint64_t blo = sdesc_sw128(st + 2 * A_BYTES + B_BYTES + 32 * k);
                    mma_f16(tmem, ahi, blo, args.idesc, 1u);
                    mma_f16(tmem, alo, bhi, args.idesc, 1u);
                }
            }
            mma_commit(empty0 + 8 * s);  // frees the stage once these MMAs have read it
        }
        mma_commit(done);  // accumulator complete (or, after an abort, nothing in flight)
    }
    __syncwarp();

    // ---------------- epilogue (all 4 warps) ----------------
    const bool got = mbar_wait(done, 0, args.err);
    tc_fence_after();
    float* part = reinterpret_cast<float*>(gbase);  // reuse stage buffers: 128 x PSTRIDE floats
    // CTA-uniform, so the .sync.aligned tensor-memory loads below never diverge;
    // also: every thread is past its last smem-stage access
    const bool have = __syncthreads_and(got) != 0;
    if (have) {
        float acc[GBN];
#pragma unroll
        for (int q = 0; q < GBN; ++q) acc[q] = 0.0f;
        const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll
        for (int c = 0; c < NCOLS / 16; ++c) {
            float v[16];
            tmem_ld16(trow + c * 16, v);
            if (args.dbg && I == 0 && J == 0) {
#pragma unroll
                for (int e = 0; e < 16; ++e) args.dbg[tid * NCOLS + c * 16 + e] = v[e];
            }
#pragma unroll
            for (int e = 0; e < 16; ++e) {
                const int col = c * 16 + e;
                const float p = v[e] * args.inv_m;
                const float t = (p > 0.0f) ? p * __log2f(p) : 0.0f;
                acc[col / BINS] += t;
            }
        }
#pragma unroll
        for (int q = 0; q < GBN; ++q) part[tid * PSTRIDE + q] = acc[q];
    }
    tc_fence_before();
    __syncthreads();
    if (have) {
        const int64_t gi0 = (int64_t)I * GA, gj0 = (int64_t)J * GBN;
        for (int p = tid; p < GA * GBN; p += THREADS) {
            const int il = p / GBN, jl = p - il * GBN;
            const int64_t i = gi0 + il, j = gj0 + jl;
            if (i >= args.n || j >= args.n || j < i) continue;
            double s = 0.0;
#pragma unroll
            for (int a = 0; a < BINS; ++a) s += (double)part[(il * BINS + a) * PSTRIDE + jl];
            const float v = (float)(args.H[i] + args.H[j] + s);  // s = -H_ij
            args.MI[i * args.ldmi + j] = v;
            args.MI[j * args.ldmi + i] = v;
        }
    }
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, TMEM_COLS);
}

// ---------------------------------------------------------------- host side
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
    static EncodeTiledFn fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (EncodeTiledFn)p;
    }
    return fn;
}

bool make_map(CUtensorMap* map, const uint16_t* base, int fmt, int64_t rows, int64_t ldw, uint32_t box_rows) {
    EncodeTiledFn enc = encode_fn();
    if (!enc) return false;
    cuuint64_t dims[2] = {(cuuint64_t)ldw, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)ldw * 2};
    cuuint32_t box[2] = {(cuuint32_t)BK, box_rows};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = enc(map, fmt == 0 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2,
                     (void*)base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                     CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

}  // namespace

// Whi/Wlo: rows >= ceil(n*bins/240)*240 + 256 rows of ldw 16-bit values, zero
// beyond row n*bins and beyond column m; ldw a multiple of 64.
cudaError_t launch_mi_tc(const uint16_t* Whi, const uint16_t* Wlo, int64_t ldw, const double* H, int64_t n, int64_t m,
                         int bins, int fmt, int split, float* MI, int64_t ldmi, int* timeout_flag, cudaStream_t stream,
                         int64_t* launches) {
    if (bins != BINS || (ldw % BK) != 0) return cudaErrorNotSupported;
    if (n <= 0) return cudaSuccess;
    int dev = 0;
    cudaGetDevice(&dev);
    int major = 0;
    cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
    if (major < 10) return cudaErrorNotSupported;
    const int64_t rows = ((n * bins + 255) / 256) * 256 + 256;
    CUtensorMap ma_hi, ma_lo, mb_hi, mb_lo;
    if (!make_map(&ma_hi, Whi, fmt, rows, ldw, MROWS) || !make_map(&mb_hi, Whi, fmt, rows, ldw, NCOLS))
        return cudaErrorNotSupported;
    if (split) {
        if (!Wlo || !make_map(&ma_lo, Wlo, fmt, rows, ldw, MROWS) || !make_map(&mb_lo, Wlo, fmt, rows, ldw, NCOLS))
            return cudaErrorNotSupported;
    } else {
        ma_lo = ma_hi;
        mb_lo = mb_hi;
    }
    TcArgs a;
    a.H = H;
    a.MI = MI;
    a.ldmi = ldmi;
    a.n = n;
    a.TI = (int)((n + GA - 1) / GA);
    a.TJ = (int)((n + GBN - 1) / GBN);
    a.ktiles = (int)(ldw / BK);
    a.inv_m = 1.0f / (float)m;
    a.idesc = idesc_f16(fmt == 0 ? 1u : 0u, MROWS, NCOLS);
    a.err = timeout_flag;
    a.dbg = g_tc_debug_dump;
    const int groups = (a.TI + GI - 1) / GI;
    const int64_t grid = (int64_t)groups * GI * a.TJ;
    const uint32_t stage_bytes = (split ? 2u : 1u) * (A_BYTES + B_BYTES);
    const size_t smem = 1024 + STAGES * stage_bytes + 16 * STAGES + 16 + 16;
    cudaError_t e;
    if (launches) ++*launches;
    if (split) {
        e = cudaFuncSetAttribute(mi_tc_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        mi_tc_kernel<true><<<(unsigned)grid, THREADS, smem, stream>>>(ma_hi, ma_lo, mb_hi, mb_lo, a);
    } else {
        e = cudaFuncSetAttribute(mi_tc_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        mi_tc_kernel<false><<<(unsigned)grid, THREADS, smem, stream>>>(ma_hi, ma_lo, mb_hi, mb_lo, a);
    }
    return cudaGetLastError();
}

}  // namespace mcpg
