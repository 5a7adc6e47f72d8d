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
// into one FP32 accumulator.  The FP8-corrected form keeps the hi*hi term in BF16
// (kind::f16) and computes the two correction terms on the FP8 tensor path
// (kind::f8f6f4, E4M3, twice the kind::f16 rate) from H8 = e4m3(16 hi) and
// L8 = e4m3(4096 lo):  2^16 P = (256 Whi)(256 Whi)' + H8 L8' + L8 H8'.  A tile
// first runs the correction over all samples (while the accumulator is small),
// then the hi*hi term: per 64 samples 4 BF16 MMAs + 4 FP8 MMAs of equal duration,
// against 12 for the BF16 split.  H8 and L8 are stored interleaved (per 64 samples
// of a row: 64 H8 bytes, then 64 L8 bytes), so a correction slice is one 128-byte
// -wide TMA box per operand, 128-byte swizzled like the hi*hi slices and of the
// same size: the MMA descriptors pick H8 at byte offsets 0 / 32 and L8 at 64 / 96
// of the swizzled rows (two K = 32 steps each).  Every TMA instruction costs the
// issuing thread a few hundred cycles, and four 64-byte boxes per slice had made
// the correction pass the producer's bottleneck.
//
// The default is the 2-SM form (mi_tc_pair_kernel, below): clusters of two CTAs
// running tcgen05.mma.cta_group::2 on 25-gene pair tiles, fed by a 7-slice ring and
// scheduled dynamically from per-group tile counters.  The 1-SM form described here
// runs when no cluster of two fits (or MCPG_TC_FORM=1sm).
// 1-SM CTA tile: A = 12 genes (120 of the 128 MMA rows), B = 24 genes (N = 240);
// D = 128 x 240 FP32 in tensor memory (256 columns allocated).
//   warp 0 / one lane : TMA producer (cp.async.bulk.tensor, 128B swizzle, 64-sample slices)
//   warp 1 / one lane : tcgen05.mma issuer (kind::f16 K=16 / kind::f8f6f4 K=32, M=128, N=240)
//   warps 2-5         : epilogue -- tcgen05.ld one row per thread, p*log2(p)
//                       per (row, B gene) in FP32, cross-bin sums and
//                       H_i + H_j - H_ij in FP64, symmetric store.
// Persistent CTAs (one per SM) walk the tile list; a ring of 64-sample stages
// (2 x 92 KB with the BF16 split, 4 x 46 KB otherwise) feeds the MMAs through
// mbarriers, and two TMEM accumulators let the epilogue of one tile overlap the
// main loop of the next.  Only gene-tile pairs that contain some j >= i run;
// tiles are visited in groups of GI A-tiles, B tiles outer, so that a group's
// A tiles stay resident in the 129 MB L2 while the B tiles stream through it
// once per group.  GI is the power of two that keeps a group within
// group_bytes() of tile operands.  Measured with the split (BF16x3): at 20,000
// x 2,000 (1 MB per A tile) GI 8 144.4 ms, 16 134.5 ms, 32 133.3 ms, 64 162.7
// ms; at 32,768 x 4,096 (2 MB per A tile) GI 8 902 ms, 16 972 ms, 32 987 ms.
//
// Every mbarrier wait is bounded (2 s of %globaltimer by default; a test hook sets a
// shorter limit and can starve the producers): on expiry the kernel raises *err,
// stops issuing work, drains what it issued (bounded), frees its tensor memory and
// returns.
#include <cuda.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

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
constexpr int TMEM_COLS = 256;
// 2-SM form: warp 0 and warps 6.. issue the TMA loads (64-sample slices round robin),
// 1 the MMAs, 2-5 the epilogue.  (The 1-SM form keeps one producer warp and 192 threads.)
#ifndef MCPG_TC_PPROD
#define MCPG_TC_PPROD 2
#endif
constexpr int NPROD = MCPG_TC_PPROD;
static_assert(NPROD >= 1 && NPROD <= 3, "producer threads per CTA");
constexpr int PAIR_THREADS = 32 * (6 + NPROD - 1);
constexpr int TQ = 4;                   // tile ring entries (2-SM form)
constexpr int TQ_CONS = 2 * NPROD + 8;  // ring readers: producers but the scheduler, the MMA issuer, 8 epilogue warps
// A-tile bytes of one rasterization group: 32 MB, except 16 MB beyond 2,048 samples
// for the 16-bit forms.  Measured on the 2-SM kernel with dynamic tile scheduling
// (ms): 20,000 x 2,000 bf16f8 16 / 32 / 64 MB 89.5 / 87.1 / 91.7, BF16x3 112.2 /
// 110.3 / 114.5; 32,768 x 4,096 bf16f8 8 / 16 / 32 / 64 MB 519 / 496 / 485 / 499.
// (With a fixed tile sequence per cluster the optimum at 32,768 x 4,096 was 8 MB for
// bf16f8 and 16 MB for BF16x3.)
inline int64_t group_bytes(int64_t ldw, int mode) {
    return (ldw <= 2048 || mode == TC_F8C) ? (32ll << 20) : (16ll << 20);
}
constexpr uint32_t A_BYTES = MROWS * BK * 2;   // 16 KB
constexpr uint32_t B_BYTES = NCOLS * BK * 2;   // 30 KB
constexpr uint32_t HL8_OFF = 64;               // byte offset of L8 within an interleaved 128-byte row

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
// non-blocking: has the phase of this parity completed?
__device__ __forceinline__ bool mbar_test(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
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
// try_wait with cluster-scope acquire: for phases completed by the peer CTA's arrivals.
__device__ __forceinline__ bool mbar_try_cluster(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n"
        "selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
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
// D[tmem] (+)= A[smem] * B[smem]^T, kind::f8f6f4 (E4M3 operands, K = 32).
__device__ __forceinline__ void mma_f8(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                       uint32_t accum) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accum));
}
__device__ __forceinline__ void mma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

// 32 lanes x 32 bits, 16 consecutive columns per thread.
// tcgen05.ld writes its destination registers asynchronously, so the wait sits in the
// same asm statement: the compiler sees the registers defined only once they hold the
// data, and cannot move, spill or reuse them in between.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
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

// Instruction descriptor, kind::f16 / kind::f8f6f4: F32 accumulate, A/B fmt
// (kind::f16: 0 = F16, 1 = BF16; kind::f8f6f4: 0 = E4M3), both K-major,
// N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t idesc_f16(uint32_t fmt, uint32_t M, uint32_t N) {
    return (1u << 4) | (fmt << 7) | (fmt << 10) | ((N >> 3) << 17) | ((M >> 4) << 24);
}

struct TcArgs {
    const double* H;
    float* MI;
    int64_t ldmi;
    int64_t n;
    int TI, TJ;        // A tiles (1-SM: 12 genes; 2-SM: pair tiles of pair_rows rows), B tiles (24 genes)
    int GI;            // A tiles per rasterization group
    int I0, TIr;       // this launch covers A tiles [I0, I0 + TIr)
    int ktiles;        // K / 64
    float inv_m;
    uint32_t idesc;
    uint32_t idesc8;   // kind::f8f6f4 (TC_F8C)
    int* err;
    unsigned long long wait_ns;  // limit of every mbarrier wait
    int starve;                  // test hook: the producers issue no loads
    // 2-SM form: weight rows of a pair tile (240: 24 genes, 120 per CTA; 250: 25 genes,
    // rows [0, 128) for rank 0 and [128, 250) for rank 1, so gene 12 of the pair is cut
    // at row 128 and rank 1 hands its two rows' sums to rank 0 through shared memory)
    // and the first row of rank 1's tile
    int pair_rows, rank1_row;
    // K steps of the last 64-sample slice that hold samples < m (16- and 32-sample MMAs);
    // the rest multiply the zero padding and are skipped
    int klast16, klast32;
    // 2-SM form: one tile counter per rasterization group (zeroed before the launch);
    // a cluster takes its next tile from the current group's counter, so all clusters
    // work on neighbouring tiles
    unsigned long long* sched;
};

__device__ __forceinline__ int j_min_for(int I) {
    // first B tile with some j >= i for A tile I: 24 J + 23 >= 12 I
    const int v = 12 * I - 23;
    return v <= 0 ? 0 : (v + 23) / 24;
}

// Bounded wait that also gives up as soon as another role raised the CTA's
// abort flag (so one timeout does not cascade into a long chain of timeouts).
__device__ __forceinline__ bool mbar_wait_abortable(uint32_t bar, uint32_t parity, int* err, volatile int* abort_flag,
                                                    unsigned long long wait_ns) {
    if (mbar_try(bar, parity)) return true;
    const unsigned long long t0 = gtimer();
    for (;;) {
        for (int i = 0; i < 64; ++i)
            if (mbar_try(bar, parity)) return true;
        if (*abort_flag) return false;
        if (gtimer() - t0 > wait_ns) {
            atomicExch(err, 1);
            *abort_flag = 1;
            return false;
        }
    }
}

__device__ __forceinline__ bool mbar_wait_cluster_abortable(uint32_t bar, uint32_t parity, int* err,
                                                            volatile int* abort_flag, unsigned long long wait_ns) {
    if (mbar_try_cluster(bar, parity)) return true;
    const unsigned long long t0 = gtimer();
    for (;;) {
        for (int i = 0; i < 64; ++i)
            if (mbar_try_cluster(bar, parity)) return true;
        if (*abort_flag) return false;
        if (gtimer() - t0 > wait_ns) {
            atomicExch(err, 1);
            *abort_flag = 1;
            return false;
        }
    }
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// Linear tile index -> (I, J): groups of a.GI A tiles, B tiles outer within a
// group.  Returns false for rectangle slots outside the upper triangle.
__device__ __forceinline__ bool tile_of(int64_t L, const TcArgs& a, int& I, int& J) {
    const int64_t per_group = (int64_t)a.GI * a.TJ;
    const int g = (int)(L / per_group);
    const int r = (int)(L - (int64_t)g * per_group);
    J = r / a.GI;
    I = a.I0 + g * a.GI + (r - J * a.GI);
    return I < a.I0 + a.TIr && I < a.TI && J >= j_min_for(I);
}

// One tile's epilogue (warps 2-5, one accumulator row per thread): reads the
// 128 x 240 accumulator at trow with tcgen05.ld, sums p*log2(p) per (row, B gene)
// in FP32, hands the accumulator back through free_acc(), then forms
// H_i + H_j - H_ij in FP64 for the tile's pairs (j in [gj0, gj0 + 24), j >= i) and
// stores both mirror entries.  The (n*bins)^2 joint table never leaves tensor memory.
// The tile holds weight rows [rowA, rowA + valid) (tile index `tile`); its genes are
// those rows' genes.  The rows (bins) of a gene are summed inside the warp by a
// segmented shuffle reduction (a fixed tree order); only per-gene sums pass through
// shared memory: gsum[0][gene][jl] for the segment that starts at the gene's first
// row, gsum[1][gene][jl] for a segment that starts at a warp's first row (the rest of
// a gene that crosses a 32-row warp boundary, or a gene that began in the tile below).
// In a 25-gene pair tile, gene 12 is cut at the ranks' boundary: rank 1 (role SEND)
// stores its part of that gene's sums into rank 0's exchange buffer and arrives on
// rank 0's barrier; rank 0 (role RECV) waits for it and writes the gene's entries.
constexpr int NGMAX = 14;  // genes a 128-row tile touches at most
constexpr int GSUM_FLOATS = 2 * NGMAX * GBN;  // 2.7 KB
constexpr int XSLOTS = 4;  // exchange slots (tile parity mod 4: rank 1 runs at most two tiles ahead)
struct Exchange {
    int role = 0;                 // 0: none, 1: RECV (rank 0), 2: SEND (rank 1)
    uint32_t buf0 = 0, bar0 = 0;  // this CTA's slot buffers (XSLOTS x GBN floats) and barriers (shared addresses)
    int64_t use = 0;              // the tile's exchange number: slot use % XSLOTS, phase (use / XSLOTS) & 1
};

template <typename FreeAcc>
__device__ __forceinline__ void epilogue_tile(uint32_t trow, float* gsum, int row, int etid, const TcArgs& args,
                                              int rowA, int valid, int gj0, const Exchange& xc,
                                              volatile int* abort_flag, FreeAcc free_acc) {
    float acc[GBN];
#pragma unroll
    for (int q = 0; q < GBN; ++q) acc[q] = 0.0f;
#pragma unroll
    for (int c = 0; c < NCOLS / 16; ++c) {
        float v[16];
        tmem_ld16(trow + c * 16, v);
#pragma unroll
        for (int e = 0; e < 16; ++e) {
            const int col = c * 16 + e;
            const float p = v[e] * args.inv_m;
            const float tt = (p > 0.0f) ? p * __log2f(p) : 0.0f;
            acc[col / BINS] += tt;
        }
    }
    // the accumulator may be overwritten from here on
    tc_fence_before();
    __syncwarp();
    free_acc();
    const int lane = row & 31;
    const int g0 = rowA / BINS;  // weight rows and genes fit in 32 bits
    const int R = rowA + row;
    const int gl = R / BINS - g0, bin = R % BINS;
    const bool same1 = (lane + 1 < 32) && (bin + 1 < BINS);
    const bool same2 = (lane + 2 < 32) && (bin + 2 < BINS);
    const bool same4 = (lane + 4 < 32) && (bin + 4 < BINS);
    const bool same8 = (lane + 8 < 32) && (bin + 8 < BINS);
#pragma unroll
    for (int q = 0; q < GBN; ++q) {
        float a = acc[q], u;
        u = __shfl_down_sync(0xffffffffu, a, 1);
        if (same1) a += u;
        u = __shfl_down_sync(0xffffffffu, a, 2);
        if (same2) a += u;
        u = __shfl_down_sync(0xffffffffu, a, 4);
        if (same4) a += u;
        u = __shfl_down_sync(0xffffffffu, a, 8);
        if (same8) a += u;
        acc[q] = a;
    }
    if (row < valid && (bin == 0 || lane == 0)) {
        float* dst = gsum + (bin == 0 ? 0 : NGMAX * GBN) + gl * GBN;
#pragma unroll
        for (int q = 0; q < GBN; ++q) dst[q] = acc[q];
    }
    asm volatile("bar.sync 1, 128;" ::: "memory");
    // the addresses are formed only here, after the accumulator loads
    const int xs = (int)(xc.use % XSLOTS);
    const uint32_t xbuf = xc.buf0 + 4u * GBN * xs, xbar = xc.bar0 + 8u * xs;
    if (xc.role == 2 && etid == 0) {
        // this tile's first gene (the pair's cut gene): its rows here went to gsum[1][0]
        uint32_t dbuf, dbar;
        asm volatile("mapa.shared::cluster.u32 %0, %1, 0;" : "=r"(dbuf) : "r"(xbuf));
        asm volatile("mapa.shared::cluster.u32 %0, %1, 0;" : "=r"(dbar) : "r"(xbar));
#pragma unroll 1
        for (int q = 0; q < GBN; ++q)
            asm volatile("st.shared::cluster.f32 [%0], %1;" ::"r"(dbuf + 4 * q), "f"(gsum[NGMAX * GBN + q]) : "memory");
        asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(dbar) : "memory");
    }
    bool have_peer = true;
    if (xc.role == 1) {
        if (etid == 0 && !mbar_wait_cluster_abortable(xbar, (uint32_t)((xc.use / XSLOTS) & 1), args.err, abort_flag,
                                                       args.wait_ns))
            *abort_flag = 1;
        asm volatile("bar.sync 1, 128;" ::: "memory");
        have_peer = !*abort_flag;
    }
    const int g_last = (rowA + valid - 1) / BINS;
    for (int p = etid; p < NGMAX * GBN; p += 128) {
        const int il = p / GBN, jl = p - il * GBN;
        const int64_t i = g0 + il, j = gj0 + jl;
        if (i > g_last || i >= args.n || j >= args.n || j < i) continue;
        const int r0 = BINS * (g0 + il) - rowA, r1 = r0 + BINS;  // the gene's rows, tile-relative
        const bool starts_here = r0 >= 0, ends_here = r1 <= valid;
        const int lo = starts_here ? r0 : 0, hi = ends_here ? r1 : valid;
        double sum = (double)gsum[(starts_here ? 0 : NGMAX * GBN) + il * GBN + jl];
        if (lo / 32 != (hi - 1) / 32) sum += (double)gsum[NGMAX * GBN + il * GBN + jl];
        if (!starts_here) continue;  // rank 1's part of the pair's cut gene: rank 0 writes it
        if (!ends_here) {             // rank 0: the cut gene, plus rank 1's two rows
            if (xc.role != 1 || !have_peer) continue;
            float peer;
            asm volatile("ld.shared.f32 %0, [%1];" : "=f"(peer) : "r"(xbuf + 4u * jl) : "memory");
            sum += (double)peer;
        }
        const float val = (float)(args.H[i] + args.H[j] + sum);  // sum = -H_ij
        args.MI[i * args.ldmi + j] = val;
        args.MI[j * args.ldmi + i] = val;
    }
}

// Persistent, warp-specialised CTA (one per SM):
//   warp 0 (one lane)  TMA producer over a STAGES-deep ring of 64-sample slices
//   warp 1 (one lane)  tcgen05.mma issuer; warp 1 also owns the TMEM allocation
//   warps 2-5          epilogue, 128 threads = 128 accumulator rows
// Two TMEM accumulators (2 x 256 columns) let the epilogue of tile t overlap the
// main loop of tile t+1.
// map_lo / mapb_lo carry Wlo (TC_SPLIT16) or the interleaved H8|L8 plane (TC_F8C); map_l8 / mapb_l8 are unused.
template <int MODE, int STAGES, int SUB>
__global__ void __launch_bounds__(192, 1)
    mi_tc_kernel(const __grid_constant__ CUtensorMap map_hi, const __grid_constant__ CUtensorMap map_lo,
                 const __grid_constant__ CUtensorMap mapb_hi, const __grid_constant__ CUtensorMap mapb_lo,
                 const __grid_constant__ CUtensorMap map_l8, const __grid_constant__ CUtensorMap mapb_l8,
                 const TcArgs args, const int64_t n_slots) {
    constexpr bool SPLIT = MODE == TC_SPLIT16;
    constexpr bool F8C = MODE == TC_F8C;
    extern __shared__ uint8_t smem_raw[];
    const uint32_t raw = smem_u32(smem_raw);
    const uint32_t base = (raw + 1023u) & ~1023u;
    uint8_t* gbase = smem_raw + (base - raw);
    constexpr uint32_t SLICE = (SPLIT ? 2 : 1) * (A_BYTES + B_BYTES);  // one 64-sample slice
    constexpr uint32_t STAGE_BYTES = SUB * SLICE;
    constexpr uint32_t PART_BYTES = GSUM_FLOATS * 4;  // per-gene bin sums of the epilogue
    float* part = reinterpret_cast<float*>(gbase + STAGES * STAGE_BYTES);
    const uint32_t bars = base + STAGES * STAGE_BYTES + PART_BYTES;
    const uint32_t full0 = bars, empty0 = bars + 8 * STAGES;
    const uint32_t tfull0 = bars + 16 * STAGES, tempty0 = tfull0 + 16;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(gbase + STAGES * STAGE_BYTES + PART_BYTES + 16 * STAGES + 32);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(full0 + 8 * s, 1);
            mbar_init(empty0 + 8 * s, 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(tfull0 + 8 * b, 1);
            mbar_init(tempty0 + 8 * b, 4);
        }
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if (warp == 1) tmem_alloc(smem_u32(tmem_slot), 2 * TMEM_COLS);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *reinterpret_cast<volatile uint32_t*>(tmem_slot);
    const int KT = args.ktiles;
    const int QP = (KT + SUB - 1) / SUB;  // stages per pass over the samples
    const int QT = F8C ? 2 * QP : QP;     // stages per tile: the correction pass, then hi*hi

    if (warp == 0) {
        if (lane == 0) {
            // ---------------- TMA producer ----------------
            int64_t g = 0;  // running k-slice counter across this CTA's tiles
            bool ok = !args.starve;
            for (int64_t L = blockIdx.x; L < n_slots && ok; L += gridDim.x) {
                int I, J;
                if (!tile_of(L, args, I, J)) continue;
                const int rowA = I * GA * BINS, rowB = J * GBN * BINS;
                for (int q = 0; q < QT; ++q, ++g) {
                    const int s = (int)(g % STAGES);
                    const int64_t u = g / STAGES;
                    if (u > 0 && !(ok = mbar_wait_abortable(empty0 + 8 * s, (uint32_t)((u - 1) & 1), args.err,
                                                            abort_flag, args.wait_ns)))
                        break;
                    const uint32_t st = base + s * STAGE_BYTES, fb = full0 + 8 * s;
                    const bool corr = F8C && q < QP;
                    const int kt0 = (q % QP) * SUB, ns = KT - kt0 < SUB ? KT - kt0 : SUB;
                    mbar_expect_tx(fb, (uint32_t)ns * SLICE);
#pragma unroll
                    for (int j = 0; j < SUB; ++j) {
                        if (j >= ns) break;
                        const uint32_t sl = st + j * SLICE;
                        const int x = (kt0 + j) * BK;
                        if (corr) {  // H8|L8 of 64 samples: one 128-byte box row per operand row
                            tma_load_2d(sl, &map_lo, 2 * x, rowA, fb);
                            tma_load_2d(sl + A_BYTES, &mapb_lo, 2 * x, rowB, fb);
                            continue;
                        }
                        tma_load_2d(sl, &map_hi, x, rowA, fb);
                        tma_load_2d(sl + A_BYTES, &mapb_hi, x, rowB, fb);
                        if (SPLIT) {
                            tma_load_2d(sl + A_BYTES + B_BYTES, &map_lo, x, rowA, fb);
                            tma_load_2d(sl + 2 * A_BYTES + B_BYTES, &mapb_lo, x, rowB, fb);
                        }
                    }
                }
            }
            // drain: the last phase issued on each stage lands before the CTA exits
            for (int s = 0; s < STAGES && (int64_t)s < g; ++s) {
                const int64_t last = (g - 1 - s) / STAGES;
                mbar_wait_abortable(full0 + 8 * s, (uint32_t)(last & 1), args.err, abort_flag, args.wait_ns);
            }
        }
        __syncwarp();
    } else if (warp == 1) {
        if (lane == 0) {
            // ---------------- MMA issuer ----------------
            int64_t g = 0, t = 0;
            bool ok = true;
            for (int64_t L = blockIdx.x; L < n_slots && ok; L += gridDim.x) {
                int I, J;
                if (!tile_of(L, args, I, J)) continue;
                const int ab = (int)(t & 1);
                const int64_t ua = t >> 1;
                if (ua > 0 &&
                    !(ok = mbar_wait_abortable(tempty0 + 8 * ab, (uint32_t)((ua - 1) & 1), args.err, abort_flag, args.wait_ns)))
                    break;
                tc_fence_after();
                const uint32_t dacc = tmem + (uint32_t)(ab * TMEM_COLS);
                for (int q = 0; q < QT; ++q, ++g) {
                    const int s = (int)(g % STAGES);
                    if (!(ok = mbar_wait_abortable(full0 + 8 * s, (uint32_t)((g / STAGES) & 1), args.err,
                                                   abort_flag, args.wait_ns)))
                        break;
                    tc_fence_after();
                    const uint32_t st = base + s * STAGE_BYTES;
                    const bool corr = F8C && q < QP;
                    const int kt0 = (q % QP) * SUB, ns = KT - kt0 < SUB ? KT - kt0 : SUB;
#pragma unroll
                    for (int j = 0; j < SUB; ++j) {
                        if (j >= ns) break;
                        const uint32_t sl = st + j * SLICE;
                        if (corr) {
#pragma unroll
                            for (int k = 0; k < BK / 32; ++k) {
                                const uint64_t ah = sdesc_sw128(sl + 32 * k), al = sdesc_sw128(sl + HL8_OFF + 32 * k);
                                const uint64_t bh = sdesc_sw128(sl + A_BYTES + 32 * k);
                                const uint64_t bl = sdesc_sw128(sl + A_BYTES + HL8_OFF + 32 * k);
                                mma_f8(dacc, ah, bl, args.idesc8, (q > 0 || j > 0 || k > 0) ? 1u : 0u);
                                mma_f8(dacc, al, bh, args.idesc8, 1u);
                            }
                            continue;
                        }
#pragma unroll
                        for (int k = 0; k < BK / 16; ++k) {
                            const uint64_t ahi = sdesc_sw128(sl + 32 * k);
                            const uint64_t bhi = sdesc_sw128(sl + A_BYTES + 32 * k);
                            mma_f16(dacc, ahi, bhi, args.idesc, (F8C || q > 0 || j > 0 || k > 0) ? 1u : 0u);
                            if (SPLIT) {
                                const uint64_t alo = sdesc_sw128(sl + A_BYTES + B_BYTES + 32 * k);
                                const uint64_t blo = sdesc_sw128(sl + 2 * A_BYTES + B_BYTES + 32 * k);
                                mma_f16(dacc, ahi, blo, args.idesc, 1u);
                                mma_f16(dacc, alo, bhi, args.idesc, 1u);
                            }
                        }
                    }
                    mma_commit(empty0 + 8 * s);  // frees the stage once these MMAs have read it
                }
                if (!ok) break;
                mma_commit(tfull0 + 8 * ab);  // accumulator ab complete
                ++t;
            }
        }
        __syncwarp();
    } else {
        // ---------------- epilogue: warps 2..5, 128 rows ----------------
        const int row = ((warp & 3) << 5) + lane;  // TMEM lane quarter of this warp
        const int etid = tid - 64;                  // 0..127
        int64_t t = 0;
        for (int64_t L = blockIdx.x; L < n_slots; L += gridDim.x) {
            int I, J;
            if (!tile_of(L, args, I, J)) continue;
            const int ab = (int)(t & 1);
            const bool got = mbar_wait_abortable(tfull0 + 8 * ab, (uint32_t)((t >> 1) & 1), args.err, abort_flag, args.wait_ns);
            tc_fence_after();
            // uniform across the 128 epilogue threads (.sync.aligned loads below)
            asm volatile("bar.sync 1, 128;" ::: "memory");
            if (!got || *abort_flag) break;
            const uint32_t trow = tmem + (uint32_t)(ab * TMEM_COLS) + ((uint32_t)((warp & 3) * 32) << 16);
            epilogue_tile(trow, part, row, etid, args, I * GA * BINS, GA * BINS, J * GBN, Exchange(), abort_flag, [&] {
                if (lane == 0) mbar_arrive(tempty0 + 8 * ab);
            });
            ++t;
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        tmem_dealloc(tmem, 2 * TMEM_COLS);
    }
}

// ---------------------------------------------------------------- 2-SM form
// A cluster of two CTAs (an SM pair) runs cta_group::2 MMAs of M = 256: each CTA
// holds its own A tile (128 or 122 weight rows of a 25-gene pair, or 12 genes) and HALF of the B tile (12 of its 24
// genes, 120 rows); the MMA reads both CTAs' shared memory and writes each CTA's
// 128 x 240 accumulator into that CTA's tensor memory.  Per SM and per 64
// samples the stages carry 31 KB instead of 46 KB for the same MMA time, which
// is what the L2 -> SM path sustains at the tensor pipe's rate.  Pair tile IP covers
// weight rows [IP pair_rows, (IP + 1) pair_rows) (24 or 25 genes), B tile J genes
// [24 J, 24 J + 24); only pairs with some j >= i run (pair_j_min).
//   leader (rank 0): warps 0 and 6 TMA for its halves (alternate slices; warp 0's lane 0
//                    also takes the tiles and publishes them to both CTAs), warp 1 the
//                    MMA issuer, warps 2-5 epilogue
//   peer   (rank 1): warps 0 and 6 TMA for its halves, warps 2-5 epilogue
// The ring holds SLOTS slices; a stage is SUB consecutive slices (slot (stage*SUB + j)
// mod SLOTS), so the ring length need not be a multiple of the stage.  Full barriers
// (NF = ceil(SLOTS / SUB), one per stage in flight, SUB arrivals) live in the leader:
// each slice's expect_tx covers both CTAs' bytes, the peer's loads signal it through
// the cta_group::2 TMA form, and the MMA issuer waits once per stage.  A producer
// refills a slot only after the MMAs of the slice SLOTS earlier committed, which is in
// stage (g*SUB - SLOTS)/SUB >= g - NF, so a full barrier is never re-armed before the
// issuer has passed its previous phase.  Slot
// empty barriers (one per slice, a multicast commit after that slice's MMAs) and the
// accumulator-full barriers sit in both CTAs; accumulator-empty in the leader (8
// arrivals: both CTAs' epilogue warps).
constexpr uint32_t BH_BYTES = (NCOLS / 2) * BK * 2;   // 15 KB: half a B tile, 16-bit
#ifndef MCPG_TC_PAIR25
#define MCPG_TC_PAIR25 1  // whole-matrix launches on 25-gene pair tiles (0: 24-gene pairs)
#endif

__device__ __forceinline__ uint32_t cluster_rank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
// shared::cluster address of this CTA's shared variable at saddr, in CTA `rank`
__device__ __forceinline__ uint32_t map_to_rank(uint32_t saddr, uint32_t rank) {
    uint32_t d;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(d) : "r"(saddr), "r"(rank));
    return d;
}
__device__ __forceinline__ void cluster_sync_all() {
    asm volatile("barrier.cluster.arrive.release.aligned;\nbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_remote(uint32_t cluster_addr) {
    asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(cluster_addr) : "memory");
}
// TMA into this CTA's shared memory, completing on a barrier of either CTA of the pair
__device__ __forceinline__ void tma_load_2d_pair(uint32_t dst, const CUtensorMap* map, int x, int y,
                                                 uint32_t bar_cluster) {
    asm volatile(
        "cp.async.bulk.tensor.2d.cta_group::2.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, "
        "%3}], [%4];" ::"r"(dst),
        "l"((unsigned long long)map), "r"(x), "r"(y), "r"(bar_cluster)
        : "memory");
}
__device__ __forceinline__ void mma2_f16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accum) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::2.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accum));
}
__device__ __forceinline__ void mma2_f8(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                        uint32_t accum) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::2.kind::f8f6f4 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accum));
}
// arrive on the barrier at this shared offset in both CTAs once the issued MMAs completed
__device__ __forceinline__ void mma2_commit_both(uint32_t bar) {
    const uint16_t mask = 3;
    asm volatile(
        "tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], %1;" ::"r"(bar),
        "h"(mask)
        : "memory");
}

__device__ __forceinline__ void st_cluster_u32(uint32_t cluster_addr, uint32_t v) {
    asm volatile("st.shared::cluster.u32 [%0], %1;" ::"r"(cluster_addr), "r"(v) : "memory");
}

// first B tile with some j >= i for pair tile IP (pair_rows weight rows, whole genes)
__device__ __forceinline__ int pair_j_min(int IP, int pair_rows) {
    const int64_t v = (int64_t)IP * pair_rows / BINS - (GBN - 1);
    return v <= 0 ? 0 : (int)((v + GBN - 1) / GBN);
}

// Rasterization group g of the 2-SM form: pair tiles [ip0, ip0 + gi), B tiles
// [js, TJ) outer; slot v is (IP, J) = (ip0 + v % gi, js + v / gi), a tile with some
// j >= i unless IP's own first B tile lies above J (near the diagonal only).
struct PairGroup {
    int ip0, gi, js;
    int64_t slots;
};
__device__ __forceinline__ PairGroup pair_group(const TcArgs& a, int g) {
    PairGroup G;
    G.ip0 = a.I0 + g * a.GI;
    const int end = min(a.I0 + a.TIr, a.TI);
    G.gi = min(a.GI, end - G.ip0);
    G.js = pair_j_min(G.ip0, a.pair_rows);
    G.slots = G.gi > 0 && a.TJ > G.js ? (int64_t)G.gi * (a.TJ - G.js) : 0;
    return G;
}


// TcArgs in pair units: TI = pair tiles (24 genes), I0 / TIr = the launch's pair range.
template <int MODE, int SLOTS, int SUB>
__global__ void __launch_bounds__(PAIR_THREADS, 1)
    mi_tc_pair_kernel(const __grid_constant__ CUtensorMap map_hi, const __grid_constant__ CUtensorMap map_lo,
                      const __grid_constant__ CUtensorMap mapb_hi, const __grid_constant__ CUtensorMap mapb_lo,
                      const __grid_constant__ CUtensorMap map_l8, const __grid_constant__ CUtensorMap mapb_l8,
                      const TcArgs args, const int64_t n_slots) {
    constexpr bool SPLIT = MODE == TC_SPLIT16;
    constexpr bool F8C = MODE == TC_F8C;
    constexpr uint32_t HALF = A_BYTES + BH_BYTES;                 // 31 KB
    constexpr uint32_t SLICE = (SPLIT ? 2 : 1) * HALF;
    constexpr uint32_t RING_BYTES = SLOTS * SLICE;
    // A box rows: 128 for 25-gene pair tiles (rank 1's last 6 rows are the next pair's), 120 for 24
    const uint32_t a_box = args.rank1_row == GA * BINS ? GA * BINS : MROWS;
    const uint32_t slice_tx = (SPLIT ? 2u : 1u) * (a_box * BK * 2u + BH_BYTES);  // per CTA
    // per-gene bin sums of the epilogue, then the exchange slots of the pair's cut gene
    constexpr uint32_t PART_BYTES = (GSUM_FLOATS + XSLOTS * GBN) * 4;
    // the MMA issuer waits once per stage (full, one arrival per slice), but every slice
    // is released on its own (empty, one commit per slice), so a slot refills while the
    // rest of the ring is consumed
    constexpr int NF = (SLOTS + SUB - 1) / SUB;
    static_assert(NF * SUB >= SLOTS && SLOTS >= SUB, "ring of at least one stage");
    extern __shared__ uint8_t smem_raw[];
    const uint32_t raw = smem_u32(smem_raw);
    const uint32_t base = (raw + 1023u) & ~1023u;
    uint8_t* gbase = smem_raw + (base - raw);
    float* part = reinterpret_cast<float*>(gbase + RING_BYTES);
    const uint32_t bars = base + RING_BYTES + PART_BYTES;
    const uint32_t full0 = bars, empty0 = bars + 8 * NF;
    const uint32_t tfull0 = empty0 + 8 * SLOTS, tempty0 = tfull0 + 16;
    // tile ring: the leader's scheduler thread publishes each tile it takes from the
    // launch's counter into both CTAs (qfull: one arrival); every other role of both
    // CTAs reads it and arrives on the leader's qempty (TQ_CONS arrivals); -1 ends
    const uint32_t qfull0 = tempty0 + 16, qempty0 = qfull0 + 8 * TQ, qtiles = qempty0 + 8 * TQ;
    volatile int32_t* qt = reinterpret_cast<volatile int32_t*>(gbase + (qtiles - base));
    const uint32_t xfull0 = qtiles + 4 * TQ;                      // exchange barriers (rank 0's used)
    const uint32_t xbuf0 = base + RING_BYTES + GSUM_FLOATS * 4;   // exchange slots (XSLOTS x GBN floats)
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(gbase + (xfull0 + 8 * XSLOTS - base));
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t rank = cluster_rank();
    const bool leader = rank == 0;
    if (tid == 0) {
        for (int s = 0; s < NF; ++s) mbar_init(full0 + 8 * s, SUB);  // one arrival per slice
        for (int s = 0; s < TQ; ++s) {
            mbar_init(qfull0 + 8 * s, 1);
            mbar_init(qempty0 + 8 * s, TQ_CONS);
        }
        for (int s = 0; s < XSLOTS; ++s) mbar_init(xfull0 + 8 * s, 1);  // rank 1's arrival
        for (int r = 0; r < SLOTS; ++r) mbar_init(empty0 + 8 * r, 1);
        for (int b = 0; b < 2; ++b) {
            mbar_init(tfull0 + 8 * b, 1);
            mbar_init(tempty0 + 8 * b, 8);
        }
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(2 * TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;");
    }
    tc_fence_before();
    cluster_sync_all();  // both CTAs' barriers initialised and tensor memory allocated
    tc_fence_after();
    const uint32_t tmem = *reinterpret_cast<volatile uint32_t*>(tmem_slot);
    const int KT = args.ktiles;
    const int QP = (KT + SUB - 1) / SUB;
    const int QT = F8C ? 2 * QP : QP;
    // ring entry k of the tile sequence: wait until published, read it, release it
    auto take_tile = [&](int64_t k, int32_t& L) -> bool {
        const int s = (int)(k % TQ);
        if (!mbar_wait_cluster_abortable(qfull0 + 8 * s, (uint32_t)((k / TQ) & 1), args.err, abort_flag,
                                         args.wait_ns))
            return false;
        L = qt[s];
        if (leader) mbar_arrive(qempty0 + 8 * s);
        else mbar_arrive_remote(map_to_rank(qempty0 + 8 * s, 0));
        return true;
    };

    if (warp == 0 || warp >= 6) {
        if (lane == 0) {
            // ---------------- TMA producers (both CTAs: own A tile, own half of B) ----------------
            // NPROD threads take the slices round robin (a thread waits a few hundred cycles
            // per TMA instruction and per barrier wait, so one thread alone falls behind
            // 64-sample slices; two are fastest, measured against one and three).  A slice missing at the end of a pass (KT not a multiple of SUB) is a
            // bare arrival, so every stage takes SUB arrivals and every slot SUB commits a round.
            const int pid = warp == 0 ? 0 : warp - 5;
            const bool scheduler = leader && pid == 0;
            const int ngroups = (args.TIr + args.GI - 1) / args.GI;
            int sg = 0;  // the scheduler's current group, and its next slot in flight
            unsigned long long pend = (scheduler && ngroups > 0) ? atomicAdd(args.sched, 1ull) : 0ull;
            int64_t g = 0;  // stages issued by this CTA (every producer counts all of them)
            bool ok = true;
            for (int64_t k = 0; ok; ++k) {
                int32_t L = -1;
                if (scheduler) {
                    // the next tile with some j >= i as (IP << 16) | J, or -1 past the end;
                    // published to both CTAs
                    while (sg < ngroups) {
                        const PairGroup G = pair_group(args, sg);
                        const unsigned long long v = pend;
                        if ((int64_t)v >= G.slots) {  // this group is taken: the next one
                            if (++sg < ngroups) pend = atomicAdd(args.sched + sg, 1ull);
                            continue;
                        }
                        pend = atomicAdd(args.sched + sg, 1ull);  // in flight while this tile loads
                        const int J = G.js + (int)(v / (unsigned)G.gi), IP = G.ip0 + (int)(v % (unsigned)G.gi);
                        if (J >= pair_j_min(IP, args.pair_rows)) {
                            L = (IP << 16) | J;
                            break;
                        }
                    }
                    const int s = (int)(k % TQ);
                    const int64_t u = k / TQ;
                    if (u > 0 && !(ok = mbar_wait_cluster_abortable(qempty0 + 8 * s, (uint32_t)((u - 1) & 1), args.err,
                                                                    abort_flag, args.wait_ns)))
                        break;
                    qt[s] = L;
                    st_cluster_u32(map_to_rank(qtiles + 4 * s, 1), (uint32_t)L);
                    mbar_arrive(qfull0 + 8 * s);
                    mbar_arrive_remote(map_to_rank(qfull0 + 8 * s, 1));
                } else if (!(ok = take_tile(k, L))) {
                    break;
                }
                if (L < 0) break;
                if (args.starve) continue;  // test hook: no loads, the MMA issuer's first wait runs out
                const int IP = L >> 16, J = L & 0xFFFF;
                const int rowA = IP * args.pair_rows + (int)rank * args.rank1_row;
                const int rowB = J * GBN * BINS + (int)rank * (NCOLS / 2);
                for (int q = 0; q < QT && ok; ++q, ++g) {
                    const int s = (int)(g % NF);
                    const uint32_t fb = map_to_rank(full0 + 8 * s, 0);
                    const bool corr = F8C && q < QP;
                    const int kt0 = (q % QP) * SUB, ns = KT - kt0 < SUB ? KT - kt0 : SUB;
#pragma unroll 1
                    for (int j = 0; j < SUB; ++j) {
                        const int64_t gs = g * SUB + j;  // slice slot sequence
                        if ((int)(gs % NPROD) != pid) continue;
                        const int r = (int)(gs % SLOTS);
                        const int64_t u = gs / SLOTS;
                        if (u > 0 && !(ok = mbar_wait_abortable(empty0 + 8 * r, (uint32_t)((u - 1) & 1), args.err,
                                                                abort_flag, args.wait_ns)))
                            break;
                        if (j >= ns) {
                            if (leader) mbar_arrive(full0 + 8 * s);
                            continue;
                        }
                        if (leader) mbar_expect_tx(full0 + 8 * s, 2u * slice_tx);  // this slice of both CTAs
                        const uint32_t sl = base + (uint32_t)r * SLICE;
                        const int x = (kt0 + j) * BK;
                        if (corr) {  // H8|L8 of 64 samples: one 128-byte box row per operand row
                            tma_load_2d_pair(sl, &map_lo, 2 * x, rowA, fb);
                            tma_load_2d_pair(sl + A_BYTES, &mapb_lo, 2 * x, rowB, fb);
                            continue;
                        }
                        tma_load_2d_pair(sl, &map_hi, x, rowA, fb);
                        tma_load_2d_pair(sl + A_BYTES, &mapb_hi, x, rowB, fb);
                        if (SPLIT) {
                            tma_load_2d_pair(sl + HALF, &map_lo, x, rowA, fb);
                            tma_load_2d_pair(sl + HALF + A_BYTES, &mapb_lo, x, rowB, fb);
                        }
                    }
                }
            }
            // drain: every slot filled has been consumed by the MMAs (the multicast commits
            // reach both CTAs), so no load is still in flight
            const int64_t G = g * SUB;
            for (int r = 0; r < SLOTS && (int64_t)r < G; ++r) {
                const int64_t last = (G - 1 - r) / SLOTS;
                mbar_wait_abortable(empty0 + 8 * r, (uint32_t)(last & 1), args.err, abort_flag, args.wait_ns);
            }
        }
        __syncwarp();
    } else if (warp == 1) {
        if (lane == 0 && leader) {
            // ---------------- MMA issuer (leader only) ----------------
            // The tensor pipe runs only slightly behind this thread, so every pause here
            // (a barrier wait costs ~100 cycles even when the phase is already complete)
            // shows up as idle tensor cycles.  The next stage's full barrier is therefore
            // tested without blocking before the current stage's last slice is issued; the
            // blocking wait runs only when that test found the stage incomplete.  Barrier
            // and slot indices advance incrementally (no 64-bit division per slice).
            int64_t t = 0;
            int fs = 0, rs = 0;    // full barrier of the current stage, slot of its first slice
            uint32_t fph = 0;      // phase parity of that full barrier
            bool ready = false;    // the current stage's full barrier was already seen complete
            bool ok = true;
            for (int64_t k = 0; ok; ++k) {
                int32_t L;
                if (!(ok = take_tile(k, L)) || L < 0) break;
                const int ab = (int)(t & 1);
                const int64_t ua = t >> 1;
                if (ua > 0 && !(ok = mbar_wait_cluster_abortable(tempty0 + 8 * ab, (uint32_t)((ua - 1) & 1),
                                                                 args.err, abort_flag, args.wait_ns)))
                    break;
                tc_fence_after();
                const uint32_t dacc = tmem + (uint32_t)(ab * TMEM_COLS);
                for (int q = 0; q < QT; ++q) {
                    if (!ready && !(ok = mbar_wait_abortable(full0 + 8 * fs, fph, args.err, abort_flag,
                                                             args.wait_ns)))
                        break;
                    tc_fence_after();
                    const int fs1 = fs + 1 == NF ? 0 : fs + 1;
                    const uint32_t fph1 = fs + 1 == NF ? fph ^ 1u : fph;
                    ready = false;
                    const bool corr = F8C && q < QP;
                    const int kt0 = (q % QP) * SUB, ns = KT - kt0 < SUB ? KT - kt0 : SUB;
#pragma unroll
                    for (int j = 0; j < SUB; ++j) {
                        const int r = rs;
                        rs = rs + 1 == SLOTS ? 0 : rs + 1;
                        const uint32_t sl = base + (uint32_t)r * SLICE;
                        // the next stage of this tile: its barrier's previous phase (stage
                        // g + 1 - NF) was waited for already, so the test sees its own phase
                        if (j == SUB - 1 && q + 1 < QT) ready = mbar_test(full0 + 8 * fs1, fph1);
                        if (j < ns) {
                            // every operand of the slice from one descriptor: the start-address
                            // field is addr >> 4 and all shared addresses stay below 2^18, so
                            // desc(sl + off) == desc(sl) + off / 16 with no carry
                            const uint64_t d0 = sdesc_sw128(sl);
                            const bool last = kt0 + j == KT - 1;
                            const int k32 = last ? args.klast32 : BK / 32, k16 = last ? args.klast16 : BK / 16;
                            if (corr) {
#pragma unroll
                                for (int k = 0; k < BK / 32; ++k) {
                                    if (k >= k32) break;
                                    const uint64_t ah = d0 + (uint64_t)((32 * k) >> 4);
                                    const uint64_t al = d0 + (uint64_t)((HL8_OFF + 32 * k) >> 4);
                                    const uint64_t bh = d0 + (uint64_t)((A_BYTES + 32 * k) >> 4);
                                    const uint64_t bl = d0 + (uint64_t)((A_BYTES + HL8_OFF + 32 * k) >> 4);
                                    mma2_f8(dacc, ah, bl, args.idesc8, (q > 0 || j > 0 || k > 0) ? 1u : 0u);
                                    mma2_f8(dacc, al, bh, args.idesc8, 1u);
                                }
                            } else {
#pragma unroll
                                for (int k = 0; k < BK / 16; ++k) {
                                    if (k >= k16) break;
                                    const uint64_t ahi = d0 + (uint64_t)((32 * k) >> 4);
                                    const uint64_t bhi = d0 + (uint64_t)((A_BYTES + 32 * k) >> 4);
                                    mma2_f16(dacc, ahi, bhi, args.idesc, (F8C || q > 0 || j > 0 || k > 0) ? 1u : 0u);
                                    if (SPLIT) {
                                        const uint64_t alo = d0 + (uint64_t)((HALF + 32 * k) >> 4);
                                        const uint64_t blo = d0 + (uint64_t)((HALF + A_BYTES + 32 * k) >> 4);
                                        mma2_f16(dacc, ahi, blo, args.idesc, 1u);
                                        mma2_f16(dacc, alo, bhi, args.idesc, 1u);
                                    }
                                }
                            }
                        }
                        mma2_commit_both(empty0 + 8 * r);  // frees this slot once its MMAs have read it
                    }
                    fs = fs1;
                    fph = fph1;
                }
                if (!ok) break;
                mma2_commit_both(tfull0 + 8 * ab);
                ++t;
            }
        }
        __syncwarp();
    } else {
        // ---------------- epilogue: warps 2..5 of both CTAs, 128 rows each ----------------
        const int row = ((warp & 3) << 5) + lane;
        const int etid = tid - 64;
        const uint32_t te_leader = map_to_rank(tempty0, 0);
        int64_t t = 0;
        for (int64_t k = 0;; ++k) {
            // one ring read per warp (its lane 0), shared with the warp
            int32_t L = -1;
            bool gotq = true;
            if (lane == 0) gotq = take_tile(k, L);
            L = __shfl_sync(0xffffffffu, L, 0);
            gotq = __shfl_sync(0xffffffffu, gotq ? 1 : 0, 0) != 0;
            if (!gotq || L < 0) {
                asm volatile("bar.sync 1, 128;" ::: "memory");
                break;
            }
            const int IP = L >> 16, J = L & 0xFFFF;
            const int ab = (int)(t & 1);
            const bool got = mbar_wait_abortable(tfull0 + 8 * ab, (uint32_t)((t >> 1) & 1), args.err, abort_flag, args.wait_ns);
            tc_fence_after();
            asm volatile("bar.sync 1, 128;" ::: "memory");
            if (!got || *abort_flag) break;
            const uint32_t trow = tmem + (uint32_t)(ab * TMEM_COLS) + ((uint32_t)((warp & 3) * 32) << 16);
            Exchange xc;
            if (args.rank1_row != GA * BINS) {  // 25-gene pair tile: gene 12 is cut at row 128
                xc.role = leader ? 1 : 2;
                xc.buf0 = xbuf0;
                xc.bar0 = xfull0;
                xc.use = t;
            }
            const int rowA = IP * args.pair_rows + (int)rank * args.rank1_row;
            const int valid = rank ? args.pair_rows - args.rank1_row : args.rank1_row;
            epilogue_tile(trow, part, row, etid, args, rowA, valid, J * GBN, xc, abort_flag, [&] {
                if (lane == 0) mbar_arrive_remote(te_leader + 8 * ab);
            });
            ++t;
        }
    }
    tc_fence_before();
    cluster_sync_all();  // no MMA, load or remote arrive of either CTA is outstanding
    if (warp == 1) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * TMEM_COLS));
    }
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

// The interleaved 8-bit correction plane: rows of 2 * ldw bytes, boxes of 128 bytes
// (64 samples of H8 and their 64 of L8) with a 128-byte swizzle.
bool make_map_hl8(CUtensorMap* map, const uint8_t* base, int64_t rows, int64_t ldw, uint32_t box_rows) {
    EncodeTiledFn enc = encode_fn();
    if (!enc) return false;
    cuuint64_t dims[2] = {(cuuint64_t)(2 * ldw), (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)(2 * ldw)};
    cuuint32_t box[2] = {(cuuint32_t)(2 * BK), box_rows};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, (void*)base, dims, strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

// The 2-SM form: clusters of two CTAs, as many as fit at once (persistent).
// Returns cudaErrorNotSupported when no cluster of two fits (the caller then
// runs the 1-SM form).
template <int MODE, int SLOTS, int SUB>
cudaError_t launch_pair(const CUtensorMap& a0, const CUtensorMap& a1, const CUtensorMap& b0, const CUtensorMap& b1,
                        const CUtensorMap& a2, const CUtensorMap& b2, const TcArgs& a, int64_t n_slots,
                        cudaStream_t stream) {
    constexpr uint32_t slice_bytes = (MODE == TC_SPLIT16 ? 2u : 1u) * (A_BYTES + BH_BYTES);
    constexpr int NF = (SLOTS + SUB - 1) / SUB;
    // ring, epilogue gene sums, full (per stage in flight) and empty (per slice) barriers,
    // two accumulator barrier pairs, the tile ring (barriers and entries), the
    // tensor-memory slot and the abort flag
    const size_t smem = 1024 + SLOTS * slice_bytes + (GSUM_FLOATS + XSLOTS * GBN) * 4 + 8 * NF + 8 * SLOTS + 32 +
                        20 * TQ + 8 * XSLOTS + 16;
    cudaError_t e = cudaFuncSetAttribute(mi_tc_pair_kernel<MODE, SLOTS, SUB>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = 2;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.blockDim = dim3(PAIR_THREADS, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int sms = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cfg.gridDim = dim3((unsigned)(sms & ~1), 1, 1);
    int clusters = 0;
    e = cudaOccupancyMaxActiveClusters(&clusters, mi_tc_pair_kernel<MODE, SLOTS, SUB>, &cfg);
    if (e != cudaSuccess || clusters < 1) {
        cudaGetLastError();
        return cudaErrorNotSupported;
    }
    const int64_t nclu = n_slots < clusters ? n_slots : clusters;
    cfg.gridDim = dim3((unsigned)(2 * nclu), 1, 1);
    e = cudaLaunchKernelEx(&cfg, mi_tc_pair_kernel<MODE, SLOTS, SUB>, a0, a1, b0, b1, a2, b2, a, n_slots);
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
}

// 2-SM form unless MCPG_TC_FORM=1sm (the 1-SM form also runs when no pair fits).
bool pair_form_enabled() {
    static int v = -1;
    if (v < 0) {
        const char* e = getenv("MCPG_TC_FORM");
        v = (e && strcmp(e, "1sm") == 0) ? 0 : 1;
    }
    return v == 1;
}

template <int MODE, int STAGES, int SUB>
cudaError_t launch_mode(const CUtensorMap& a0, const CUtensorMap& a1, const CUtensorMap& b0, const CUtensorMap& b1,
                        const CUtensorMap& a2, const CUtensorMap& b2, const TcArgs& a, int64_t n_slots, int64_t grid,
                        cudaStream_t stream) {
    constexpr uint32_t stage_bytes = SUB * (MODE == TC_SPLIT16 ? 2u : 1u) * (A_BYTES + B_BYTES);
    const size_t smem = 1024 + STAGES * stage_bytes + GSUM_FLOATS * 4 + 16 * STAGES + 32 + 16;
    cudaError_t e = cudaFuncSetAttribute(mi_tc_kernel<MODE, STAGES, SUB>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    mi_tc_kernel<MODE, STAGES, SUB><<<(unsigned)grid, 192, smem, stream>>>(a0, a1, b0, b1, a2, b2, a, n_slots);
    return cudaGetLastError();
}

// Slices (64 samples each) per pipeline stage of the 1-SM / 2-SM forms in the
// single-pass and FP8-corrected modes (the BF16 split always runs one slice).
// Measured at 20,000 x 2,000 (weights + MI, ms; FP8-corrected / single BF16):
// 1-SM 1 slice x 4 stages 116.2 / 56.9, 2 x 2 123.6 / 61.6; 2-SM 1 x 6 117.9 /
// 60.7, 2 x 3 112.0 / 54.1, 3 x 2 107.0 / 52.2 (BF16 split: 1-SM 139.4, 2-SM 131.6).
// With per-slice release, two producers and the 2.3 KB epilogue (2-SM ring slots /
// slices per stage): 6 / 3 89.8 / 46.4, 7 / 3 104.1 / 48.2, 7 / 2 105.7 / 50.2,
// 7 / 1 115.4 / 55.3, 6 / 2 106.2 / 51.3; 1-SM 101.5 / 52.1.  The 7-slot ring lost then
// because clusters drifted apart and L2 reuse collapsed (461 GB of DRAM reads per launch);
// with dynamic tile scheduling it wins: bf16f8 6 / 7 slots 88.7 / 86.9 ms at 20,000 x
// 2,000 and 488 / 457 ms at 32,768 x 4,096.
#ifndef MCPG_TC_SUB
#define MCPG_TC_SUB 1
#endif
#ifndef MCPG_TC_PSUB
#define MCPG_TC_PSUB 3
#endif
#ifndef MCPG_TC_PSLOTS
#define MCPG_TC_PSLOTS 7
#endif
constexpr int SUB1 = MCPG_TC_SUB, SUB2 = MCPG_TC_PSUB, SLOTS2 = MCPG_TC_PSLOTS;
static_assert((SUB1 == 1 || SUB1 == 2 || SUB1 == 4) && (SUB2 >= 1 && SUB2 <= 6) && SLOTS2 >= SUB2 && SLOTS2 <= 7,
              "slices per stage, ring slots");

}  // namespace

#ifndef MCPG_TC_PITCH_PAD
#define MCPG_TC_PITCH_PAD 0
#endif
int64_t mi_tc_pitch(int64_t m) { return (m + BK - 1) / BK * BK + MCPG_TC_PITCH_PAD; }
// work: the group tile counters of the 2-SM form (one per rasterization group, at most
// one per pair tile)
int64_t mi_tc_work_bytes(int64_t n, int bins) {
    const int64_t pair_tiles = (n * bins + 2 * GA * BINS - 1) / (2 * GA * BINS) + 1;
    return (pair_tiles * 8 + 255) / 256 * 256;
}

// Whi/Wlo (16-bit) and HL8 (8-bit, 2 * ldw bytes per row): rows >= ceil(n*bins/256)*256
// + 256 rows of ldw samples, zero beyond row n*bins and beyond sample m; ldw a multiple of 64.
cudaError_t launch_mi_tc(const uint16_t* Whi, const uint16_t* Wlo, const uint8_t* HL8, int64_t ldw, const double* H, int64_t n, int64_t m, int bins, int fmt, int mode, float* MI,
                         int64_t ldmi, int* timeout_flag, cudaStream_t stream, int64_t* launches, int64_t gene0,
                         int64_t gene1, const TcWaitHook* hook, void* work) {
    if (bins != BINS || (ldw % BK) != 0) return cudaErrorNotSupported;
    if (mode != TC_SINGLE && mode != TC_SPLIT16 && mode != TC_F8C) return cudaErrorInvalidValue;
    if (mode == TC_F8C && fmt != 0) return cudaErrorInvalidValue;
    if (gene1 < 0 || gene1 > n) gene1 = n;
    if (n <= 0 || gene0 >= gene1) return cudaSuccess;
    if (gene0 % GA) return cudaErrorInvalidValue;
    int dev = 0;
    cudaGetDevice(&dev);
    int major = 0;
    cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
    if (major < 10) return cudaErrorNotSupported;
    const int64_t rows = ((n * bins + 255) / 256) * 256 + 256;
    if (mode == TC_SPLIT16 && !Wlo) return cudaErrorNotSupported;
    if (mode == TC_F8C && !HL8) return cudaErrorNotSupported;
    // A maps with a_rows-row boxes (128: the 1-SM tile; 120: a pair CTA's 12 genes, the MMA's
    // last 8 rows then hold stale shared memory and the epilogue drops them) and B maps with
    // b_rows-row boxes (240: whole B tile; 120: a pair's half)
    CUtensorMap ma_hi, ma_lo, mb_hi, mb_lo, ma_l8, mb_l8;
    auto make_maps = [&](uint32_t a_rows, uint32_t b_rows) -> bool {
        if (!make_map(&ma_hi, Whi, fmt, rows, ldw, a_rows) || !make_map(&mb_hi, Whi, fmt, rows, ldw, b_rows))
            return false;
        ma_lo = ma_l8 = ma_hi;
        mb_lo = mb_l8 = mb_hi;
        if (mode == TC_SPLIT16)
            return make_map(&ma_lo, Wlo, fmt, rows, ldw, a_rows) && make_map(&mb_lo, Wlo, fmt, rows, ldw, b_rows);
        if (mode == TC_F8C)
            return make_map_hl8(&ma_lo, HL8, rows, ldw, a_rows) && make_map_hl8(&mb_lo, HL8, rows, ldw, b_rows);
        return true;
    };
    TcArgs a;
    a.H = H;
    a.MI = MI;
    a.ldmi = ldmi;
    a.n = n;
    a.TI = (int)((n + GA - 1) / GA);
    a.TJ = (int)((n + GBN - 1) / GBN);
    a.I0 = (int)(gene0 / GA);
    a.TIr = (int)((gene1 + GA - 1) / GA) - a.I0;
    a.ktiles = (int)((m + BK - 1) / BK);  // the row pitch ldw may exceed the samples
    // the FP8-corrected form accumulates 2^16 P (power-of-two scale: exact)
    a.inv_m = (1.0f / (float)m) * (mode == TC_F8C ? 1.0f / 65536.0f : 1.0f);
    a.idesc = idesc_f16(fmt == 0 ? 1u : 0u, MROWS, NCOLS);
    a.idesc8 = idesc_f16(0u, MROWS, NCOLS);  // E4M3 x E4M3 (format code 0 in kind::f8f6f4)
    a.err = timeout_flag;
    a.wait_ns = hook ? hook->wait_ns : TC_WAIT_NS_DEFAULT;
    a.starve = hook ? hook->starve : 0;
    a.pair_rows = 2 * GA * BINS;
    a.rank1_row = GA * BINS;
    a.sched = nullptr;
    {
        const int64_t tail_samples = m - (int64_t)(a.ktiles - 1) * BK;  // 1..64
        a.klast16 = (int)((tail_samples + 15) / 16);
        a.klast32 = (int)((tail_samples + 31) / 32);
#if defined(MCPG_TC_NO_PAD_SKIP)
        a.klast16 = BK / 16;  // tuning builds: issue the padding's MMAs too
        a.klast32 = BK / 32;
#endif
    }
    {
        const int64_t tile_bytes = (int64_t)MROWS * ldw * 2 * (mode == TC_SINGLE ? 1 : 2);
        int gi = 1;
        while (gi < 64 && (int64_t)(2 * gi) * tile_bytes <= group_bytes(ldw, mode)) gi *= 2;
#ifdef MCPG_TC_GI
        gi = MCPG_TC_GI;  // fixed group size (tuning builds)
#endif
        a.GI = gi < 4 ? 4 : gi;
    }
    // 2-SM form.  A whole-matrix launch takes pair tiles of 25 genes (250 weight rows:
    // rank 0 rows [0, 128), rank 1 rows [128, 250), so only 6 of the 256 MMA rows idle and
    // rank 1 hands its two rows of the pair's gene 12 to rank 0).  A launch over a gene
    // range keeps 24-gene pair tiles of 120 rows per CTA (the MMA's last 8 rows then read
    // stale shared memory and the epilogue drops them).
    const bool pair25 = MCPG_TC_PAIR25 && gene0 == 0 && gene1 == n;
    const int pair_rows = pair25 ? 25 * BINS : 2 * GA * BINS, rank1_row = pair25 ? MROWS : GA * BINS;
    if (pair_form_enabled() && work && (pair25 || gene0 % (2 * GA) == 0) &&
        make_maps((uint32_t)(pair25 ? MROWS : GA * BINS), NCOLS / 2)) {
        TcArgs p = a;
        p.pair_rows = pair_rows;
        p.rank1_row = rank1_row;
        p.sched = static_cast<unsigned long long*>(work);  // one counter per group, zeroed below
        const int genes_per_pair = pair_rows / BINS;
        p.TI = (int)((n + genes_per_pair - 1) / genes_per_pair);
        p.I0 = (int)(gene0 / genes_per_pair);
        p.TIr = (int)((gene1 + genes_per_pair - 1) / genes_per_pair) - p.I0;
        p.GI = a.GI / 2 < 2 ? 2 : a.GI / 2;
        const int64_t ngroups = (p.TIr + p.GI - 1) / p.GI;
        if (ngroups * 8 > mi_tc_work_bytes(n, bins)) return cudaErrorInvalidValue;
        if (cudaMemsetAsync(p.sched, 0, (size_t)ngroups * 8, stream) != cudaSuccess) return cudaGetLastError();
        p.idesc = idesc_f16(fmt == 0 ? 1u : 0u, 2 * MROWS, NCOLS);
        p.idesc8 = idesc_f16(0u, 2 * MROWS, NCOLS);
        const int64_t pslots = (int64_t)((p.TIr + p.GI - 1) / p.GI) * p.GI * p.TJ;
        cudaError_t e;
        if (mode == TC_SPLIT16)
            e = launch_pair<TC_SPLIT16, 3, 1>(ma_hi, ma_lo, mb_hi, mb_lo, ma_l8, mb_l8, p, pslots, stream);
        else if (mode == TC_F8C)
            e = launch_pair<TC_F8C, SLOTS2, SUB2>(ma_hi, ma_lo, mb_hi, mb_lo, ma_l8, mb_l8, p, pslots, stream);
        else
            e = launch_pair<TC_SINGLE, SLOTS2, SUB2>(ma_hi, ma_lo, mb_hi, mb_lo, ma_l8, mb_l8, p, pslots, stream);
        if (e != cudaErrorNotSupported) {
            if (launches) ++*launches;
            return e;
        }
    }
    if (!make_maps(MROWS, NCOLS)) return cudaErrorNotSupported;
    const int groups = (a.TIr + a.GI - 1) / a.GI;
    const int64_t n_slots = (int64_t)groups * a.GI * a.TJ;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t grid = n_slots < sms ? n_slots : sms;
    if (launches) ++*launches;
    if (mode == TC_SPLIT16)
        return launch_mode<TC_SPLIT16, 2, 1>(ma_hi, ma_lo, mb_hi, mb_lo, ma_l8, mb_l8, a, n_slots, grid, stream);
    if (mode == TC_F8C)
        return launch_mode<TC_F8C, 4 / SUB1, SUB1>(ma_hi, ma_lo, mb_hi, mb_lo, ma_l8, mb_l8, a, n_slots, grid, stream);
    return launch_mode<TC_SINGLE, 4 / SUB1, SUB1>(ma_hi, ma_lo, mb_hi, mb_lo, ma_l8, mb_l8, a, n_slots, grid, stream);
}

}  // namespace mcpg
