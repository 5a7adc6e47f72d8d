// Plain-FP32 B-spline MI on CUDA cores (K2'): the dense contraction
//   P_ij[a][b] = (1/m) sum_s w_i[a](s) w_j[b](s)
// with the joint entropy and Hx + Hy - Hxy fused into the epilogue, so the
// joint tables never leave registers.  Whole-matrix form of
// BSplineEntropyKernel::entropy2d_simd + BSplineMIKernel::operator()
// (include/mcp/correlation/BSplineMI.hpp:288-315,492-499) under
// InnerProduct<..., SYMM=true> (apps/pipeline/mcpnet_helper.hpp:88-98).
//
// Shape: CTA = 16 x 16 genes, 256 threads, one gene pair per thread with its
// BINS x BINS joint counts in registers.  Weights are sample-major
// (Wt[s][gene*BINS + a]) so one sample of 16 genes is one contiguous 640-byte
// row: a 4-stage cp.async pipeline stages 16 samples per step.  Per sample a
// thread loads 2*BINS floats (LDS.64, broadcast across the warp's 4 x 8 pair
// layout) and issues BINS^2 FFMA.  Only tiles with j-block >= i-block run.
// Epilogue: p = count * (1/m) (float, as the reference's norm_factor),
// row sums of p*log2(p) in float, the BINS row sums and the combine
// H_i + H_j - H_ij in double.
#include <math.h>

#include "common.cuh"
#include "internal.h"

namespace mcpg {
namespace {

constexpr int G = 16;          // genes per tile side
constexpr int BKS = 16;        // samples per stage
constexpr int STAGES = 4;
constexpr int THREADS = 256;

template <int BINS>
struct MiCfg {
    static constexpr int ROW = G * BINS;                  // floats per sample per operand tile
    static constexpr int STAGE_FLOATS = 2 * BKS * ROW;    // A and B
    static constexpr size_t SMEM = (size_t)STAGES * STAGE_FLOATS * sizeof(float);
};

// Upper-triangular tile index -> (ti, tj) with tj >= ti, row-major.
__device__ __forceinline__ void tri_tile(int64_t b, int64_t T, int64_t& ti, int64_t& tj) {
    // rows r have (T - r) tiles; start(r) = r*T - r(r-1)/2
    double tt = (double)(2 * T + 1);
    int64_t r = (int64_t)floor((tt - sqrt(tt * tt - 8.0 * (double)b)) * 0.5);
    if (r < 0) r = 0;
    if (r >= T) r = T - 1;
    while (r > 0 && r * T - r * (r - 1) / 2 > b) --r;
    while (r + 1 < T && (r + 1) * T - (r + 1) * r / 2 <= b) ++r;
    ti = r;
    tj = r + (b - (r * T - r * (r - 1) / 2));
}

// Adjoint epilogue arguments (EPI == 1): Q[(i - q_gene0) * BINS + a][j * BINS + b]
// = Gs_ij (log2 P_ab + 1/ln 2) for P_ab > 0 (else 0), Gs_ij = G[i][j] + G[j][i]
// for i != j and 0 on the diagonal; tiles cover A genes [16*q_tile0, ...) x all genes.
struct QArgs {
    const float* G; int64_t ldg;
    float* Q; int64_t ldq;
    int64_t q_tile0;
};

template <int BINS, int EPI>
__global__ void __launch_bounds__(THREADS, 1)
    mi_fp32_kernel(const float* __restrict__ Wt, int64_t ldwt, const double* __restrict__ H, int64_t n,
                   int64_t m_pad, float inv_m, float* __restrict__ MI, int64_t ldmi, int64_t T, const QArgs qa,
                   int64_t tile_base) {
    using C = MiCfg<BINS>;
    extern __shared__ float4 smem_f4[];
    float* smem = reinterpret_cast<float*>(smem_f4);

    int64_t ti, tj;
    if (EPI == 0) {
        tri_tile(tile_base + blockIdx.x, T, ti, tj);
    } else {
        ti = qa.q_tile0 + blockIdx.x / T;
        tj = blockIdx.x % T;
    }
    const int64_t gi0 = ti * G, gj0 = tj * G;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int il = ((warp >> 1) << 2) + (lane >> 3);  // 0..15
    const int jl = ((warp & 1) << 3) + (lane & 7);    // 0..15

    // staging: per sample and operand, ROW floats = ROW/4 chunks of 16 bytes
    constexpr int CHUNKS_PER_ROW = C::ROW / 4;              // 40 for BINS = 10
    constexpr int CHUNKS = 2 * BKS * CHUNKS_PER_ROW;         // per stage
    const float* srcA = Wt + gi0 * BINS;
    const float* srcB = Wt + gj0 * BINS;
    auto load = [&](int stage, int64_t s0) {
        float* dst = smem + stage * C::STAGE_FLOATS;
        for (int c = tid; c < CHUNKS; c += THREADS) {
            const int op = c / (BKS * CHUNKS_PER_ROW);
            const int rem = c - op * (BKS * CHUNKS_PER_ROW);
            const int srow = rem / CHUNKS_PER_ROW, ch = rem - srow * CHUNKS_PER_ROW;
            const float* src = (op ? srcB : srcA) + (s0 + srow) * ldwt + ch * 4;
            cp_async16(dst + op * BKS * C::ROW + srow * C::ROW + ch * 4, src, 16);
        }
    };

    float acc[BINS][BINS];
#pragma unroll
    for (int a = 0; a < BINS; ++a)
#pragma unroll
        for (int b = 0; b < BINS; ++b) acc[a][b] = 0.0f;

    const int64_t ksteps = m_pad / BKS;
#pragma unroll
    for (int s = 0; s < STAGES - 1; ++s) {
        if (s < ksteps) load(s, (int64_t)s * BKS);
        cp_async_commit();
    }
    for (int64_t t = 0; t < ksteps; ++t) {
        cp_async_wait<STAGES - 2>();
        __syncthreads();
        {
            const int64_t tn = t + STAGES - 1;
            if (tn < ksteps) load((int)(tn % STAGES), tn * BKS);
            cp_async_commit();
        }
        const float* As = smem + (t % STAGES) * C::STAGE_FLOATS + il * BINS;
        const float* Bs = smem + (t % STAGES) * C::STAGE_FLOATS + BKS * C::ROW + jl * BINS;
#pragma unroll 2
        for (int s = 0; s < BKS; ++s) {
            float a[BINS], b[BINS];
            if (BINS % 2 == 0) {
#pragma unroll
                for (int q = 0; q < BINS / 2; ++q) {
                    const float2 va = *reinterpret_cast<const float2*>(As + s * C::ROW + 2 * q);
                    const float2 vb = *reinterpret_cast<const float2*>(Bs + s * C::ROW + 2 * q);
                    a[2 * q] = va.x; a[2 * q + 1] = va.y;
                    b[2 * q] = vb.x; b[2 * q + 1] = vb.y;
                }
            } else {
#pragma unroll
                for (int q = 0; q < BINS; ++q) { a[q] = As[s * C::ROW + q]; b[q] = Bs[s * C::ROW + q]; }
            }
#pragma unroll
            for (int x = 0; x < BINS; ++x)
#pragma unroll
                for (int y = 0; y < BINS; ++y) acc[x][y] = fmaf(a[x], b[y], acc[x][y]);
        }
    }
    cp_async_wait<0>();

    const int64_t i = gi0 + il, j = gj0 + jl;
    if (EPI == 1) {
        if (i >= n || j >= n) return;
        const float gs = (i == j) ? 0.0f : qa.G[i * qa.ldg + j] + qa.G[j * qa.ldg + i];
        const float c = 1.4426950408889634f;  // 1 / ln 2
        float* Qr = qa.Q + (i - qa.q_tile0 * G) * BINS * qa.ldq + j * BINS;
#pragma unroll
        for (int x = 0; x < BINS; ++x)
#pragma unroll
            for (int y = 0; y < BINS; ++y) {
                const float pv = acc[x][y] * inv_m;
                Qr[x * qa.ldq + y] = (gs != 0.0f && pv > 0.0f) ? gs * (__log2f(pv) + c) : 0.0f;
            }
        return;
    }
    if (i >= n || j >= n || j < i) return;
    double hxy = 0.0;
#pragma unroll
    for (int x = 0; x < BINS; ++x) {
        float row = 0.0f;
#pragma unroll
        for (int y = 0; y < BINS; ++y) {
            const float pv = acc[x][y] * inv_m;
            if (pv > 0.0f) row += pv * __log2f(pv);
        }
        hxy += (double)row;
    }
    const float v = (float)(H[i] + H[j] + hxy);  // hxy = -H_ij
    MI[i * ldmi + j] = v;
    MI[j * ldmi + i] = v;
}

template <int BINS>
cudaError_t launch_bins(const float* Wt, int64_t ldwt, const double* H, int64_t n, int64_t m, float* MI, int64_t ldmi,
                        cudaStream_t stream, int64_t t0, int64_t t1) {
    using C = MiCfg<BINS>;
    auto kern = mi_fp32_kernel<BINS, 0>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)C::SMEM);
    if (e != cudaSuccess) return e;
    const int64_t T = ceil_div(n, G);
    if (t1 > T) t1 = T;
    if (t0 >= t1) return cudaSuccess;
    // triangle rows [t0, t1): tiles start(t) = t*T - t(t-1)/2
    const int64_t start0 = t0 * T - t0 * (t0 - 1) / 2, start1 = t1 * T - t1 * (t1 - 1) / 2;
    const int64_t tiles = start1 - start0;
    const int64_t m_pad = ceil_div(m, BKS) * BKS;
    const float inv_m = 1.0f / (float)m;  // norm_factor = FT(1) / FT(m), BSplineMI.hpp:321
    kern<<<(unsigned)tiles, THREADS, C::SMEM, stream>>>(Wt, ldwt, H, n, m_pad, inv_m, MI, ldmi, T, QArgs{}, start0);
    return cudaGetLastError();
}

template <int BINS>
cudaError_t launch_q_bins(const float* Wt, int64_t ldwt, int64_t n, int64_t m, const QArgs& qa, int64_t tiles_a,
                          cudaStream_t stream) {
    using C = MiCfg<BINS>;
    auto kern = mi_fp32_kernel<BINS, 1>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)C::SMEM);
    if (e != cudaSuccess) return e;
    const int64_t T = ceil_div(n, G);
    const int64_t m_pad = ceil_div(m, BKS) * BKS;
    const float inv_m = 1.0f / (float)m;
    kern<<<(unsigned)(tiles_a * T), THREADS, C::SMEM, stream>>>(Wt, ldwt, nullptr, n, m_pad, inv_m, nullptr, 0, T,
                                                                qa, 0);
    return cudaGetLastError();
}

}  // namespace

// Adjoint slab: Q for A genes [16*tile0, 16*(tile0 + tiles)) x all genes.
cudaError_t launch_mi_q(const float* Wt, int64_t ldwt, const float* G, int64_t ldg, int64_t n, int64_t m, int bins,
                        int64_t tile0, int64_t tiles, float* Q, int64_t ldq, cudaStream_t stream, int64_t* launches) {
    if (n <= 0 || tiles <= 0) return cudaSuccess;
    if (launches) ++*launches;
    QArgs qa{G, ldg, Q, ldq, tile0};
    switch (bins) {
        case 2: return launch_q_bins<2>(Wt, ldwt, n, m, qa, tiles, stream);
        case 3: return launch_q_bins<3>(Wt, ldwt, n, m, qa, tiles, stream);
        case 4: return launch_q_bins<4>(Wt, ldwt, n, m, qa, tiles, stream);
        case 5: return launch_q_bins<5>(Wt, ldwt, n, m, qa, tiles, stream);
        case 6: return launch_q_bins<6>(Wt, ldwt, n, m, qa, tiles, stream);
        case 7: return launch_q_bins<7>(Wt, ldwt, n, m, qa, tiles, stream);
        case 8: return launch_q_bins<8>(Wt, ldwt, n, m, qa, tiles, stream);
        case 9: return launch_q_bins<9>(Wt, ldwt, n, m, qa, tiles, stream);
        case 10: return launch_q_bins<10>(Wt, ldwt, n, m, qa, tiles, stream);
        case 11: return launch_q_bins<11>(Wt, ldwt, n, m, qa, tiles, stream);
        case 12: return launch_q_bins<12>(Wt, ldwt, n, m, qa, tiles, stream);
        default: return cudaErrorNotSupported;
    }
}

// Wt must be zero-padded: ldwt >= ceil(n/16)*16*bins (multiple of 4), rows
// s in [m, ceil(m/16)*16) zero.
cudaError_t launch_mi_fp32(const float* Wt, int64_t ldwt, const double* H, int64_t n, int64_t m, int bins, float* MI,
                           int64_t ldmi, cudaStream_t stream, int64_t* launches, int64_t gene0, int64_t gene1) {
    if (gene1 < 0 || gene1 > n) gene1 = n;
    if (n <= 0 || gene0 >= gene1) return cudaSuccess;
    if (gene0 % G) return cudaErrorInvalidValue;
    const int64_t t0 = gene0 / G, t1 = ceil_div(gene1, G);
    if (launches) ++*launches;
    switch (bins) {
        case 2: return launch_bins<2>(Wt, ldwt, H, n, m, MI, ldmi, stream, t0, t1);
        case 3: return launch_bins<3>(Wt, ldwt, H, n, m, MI, ldmi, stream, t0, t1);
        case 4: return launch_bins<4>(Wt, ldwt, H, n, m, MI, ldmi, stream, t0, t1);
        case 5: return launch_bins<5>(Wt, ldwt, H, n, m, MI, ldmi, stream, t0, t1);
        case 6: return launch_bins<6>(Wt, ldwt, H, n, m, MI, ldmi, stream, t0, t1);
        case 7: return launch_bins<7>(Wt, ldwt, H, n, m, MI, ldmi, stream, t0, t1);
        case 8: return launch_bins<8>(Wt, ldwt, H, n, m, MI, ldmi, stream, t0, t1);
        case 9: return launch_bins<9>(Wt, ldwt, H, n, m, MI, ldmi, stream, t0, t1);
        case 10: return launch_bins<10>(Wt, ldwt, H, n, m, MI, ldmi, stream, t0, t1);
        case 11: return launch_bins<11>(Wt, ldwt, H, n, m, MI, ldmi, stream, t0, t1);
        case 12: return launch_bins<12>(Wt, ldwt, H, n, m, MI, ldmi, stream, t0, t1);
        default: return cudaErrorNotSupported;
    }
}

}  // namespace mcpg
