// Stouffer and CLR transforms of a gene x gene score matrix
// (compute_stouffer, apps/pipeline/mcpnet_helper.hpp:575-586; the transform
// app, apps/transform/transform.cpp:214-231):
//   * row statistics (mean, standard deviation) per row, in FP64: the
//     reference takes them from splash::kernel::GaussianParamsExclude1<T,T,true>
//     (unbiased variance), whose source is not in the reference snapshot.  Here
//     the mean and the unbiased (N - 1) variance are two-pass FP64 sums over
//     the row, optionally without the diagonal entry; they are rounded to the
//     float pair the reference's kernels take.
//   * per entry exactly stouffer_vector_kernel / clr_vector_kernel
//     (include/mcp/transform/stouffer.hpp:57-82, clr.hpp:52-73) in float:
//       denom_i = |sd_i| < eps ? 0 : (float)(1.0 / sd_i)
//       zi = (x - mean_i) * denom_i,  zj = |sd_j| < eps ? 0 : (x - mean_j) / sd_j
//       Stouffer (zi + zj) * (float)sqrt(1/2),  CLR sqrt(zi^2 + zj^2)
//     with explicit _rn intrinsics so nvcc contracts nothing.
//   * the TF form (compute_stouffer_tf, mcpnet_helper.hpp:589-634) of a t x n
//     matrix: every row z-scored across its n entries and every column across
//     its t entries with splash::kernel::StandardScore<T,T,false> (population
//     statistics; also absent from the snapshot -- here FP64 two-pass mean and
//     population sd rounded to float, z = |sd| < eps ? 0 : (x - mean) / sd in
//     float), then zscored_stouffer_kernel (stouffer.hpp:84-100):
//     (z_row + z_col) * (float)sqrt(1/2), or zscored_clr_kernel (clr.hpp:75-88):
//     sqrt(z_row^2 + z_col^2).
#include <cuda_runtime.h>
#include <float.h>
#include <stdint.h>

#include "common.cuh"
#include "internal.h"

namespace mcpg {
namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int ST_THREADS = 256;

__device__ __forceinline__ double block_sum_d(double v, double* sh /*32*/) {
    for (int o = 16; o > 0; o >>= 1) v = __dadd_rn(v, __shfl_down_sync(FULL, v, o));
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    if (lane == 0) sh[w] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x == 0)
        for (int i = 0; i < nw; ++i) t = __dadd_rn(t, sh[i]);  // fixed order: reproducible
    __syncthreads();
    if (threadIdx.x == 0) sh[0] = t;
    __syncthreads();
    t = sh[0];
    __syncthreads();
    return t;
}

// ---- float-float accumulation on the FP32 pipe (GB300's FP64 rate is low) ----
// (hi, lo) += x by TwoSum, the rounding error gathered in lo.
__device__ __forceinline__ void ff_add(float& hi, float& lo, float x) {
    const float s = __fadd_rn(hi, x);
    const float bb = __fsub_rn(s, hi);
    const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(x, bb));
    hi = s;
    lo = __fadd_rn(lo, e);
}
// (hi, lo) += (bh, bl), renormalised.
__device__ __forceinline__ void ff_add2(float& hi, float& lo, float bh, float bl) {
    const float s = __fadd_rn(hi, bh);
    const float bb = __fsub_rn(s, hi);
    float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(bh, bb));
    e = __fadd_rn(e, __fadd_rn(lo, bl));
    hi = __fadd_rn(s, e);
    lo = __fsub_rn(e, __fsub_rn(hi, s));
}
// Block sum of the threads' (hi, lo) in a fixed order, as a double (every thread).
__device__ __forceinline__ double block_sum_ff(float hi, float lo, float* sh /*64*/) {
    for (int o = 16; o > 0; o >>= 1) {
        const float oh = __shfl_down_sync(FULL, hi, o), ol = __shfl_down_sync(FULL, lo, o);
        ff_add2(hi, lo, oh, ol);
    }
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    if (lane == 0) {
        sh[2 * w] = hi;
        sh[2 * w + 1] = lo;
    }
    __syncthreads();
    double t = 0.0;
    for (int k = 0; k < nw; ++k) t = __dadd_rn(t, __dadd_rn((double)sh[2 * k], (double)sh[2 * k + 1]));
    __syncthreads();
    return t;
}
__device__ __forceinline__ float block_max_f(float v, float* sh /*32*/) {
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_down_sync(FULL, v, o));
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    if (lane == 0) sh[w] = v;
    __syncthreads();
    float t = 0.0f;
    for (int k = 0; k < nw; ++k) t = fmaxf(t, sh[k]);
    __syncthreads();
    return t;
}

// One block per row (grid-stride): the mean and the variance (divided by
// N - ddof; ddof 1 unbiased, 0 population) by two passes over the row.  The
// passes accumulate in float-float and the block's partial sums combine in
// FP64: with c columns per thread the relative error of a sum stays below
// about c^2 * 2^-48 (2^-34 at 32,768 columns), far below the float rounding of
// the results, which can differ from FP64 sums' by one ulp only at a rounding
// boundary -- as another summation order can too.  A row whose sums or
// squared deviations leave float range (|x| near FLT_MAX, as compute_combo
// writes for a vanishing denominator) or whose deviations are all below
// 2^-40 (their squares would lose precision) is summed again in FP64.
__global__ void __launch_bounds__(ST_THREADS) row_stats_kernel(const float* A, int64_t rows, int64_t cols,
                                                               int64_t lda, int excl_diag, int ddof, float* mean,
                                                               float* sd) {
    __shared__ double sh[32];
    __shared__ float shf[64];
    for (int64_t i = blockIdx.x; i < rows; i += gridDim.x) {
        const float* row = A + i * lda;
        const int64_t N = cols - ((excl_diag && i < cols) ? 1 : 0);
        float hi = 0.0f, lo = 0.0f;
        for (int64_t j = threadIdx.x; j < cols; j += blockDim.x)
            if (!(excl_diag && j == i)) ff_add(hi, lo, row[j]);
        double tot = block_sum_ff(hi, lo, shf);
        bool ok = isfinite(tot);
        double mu = N > 0 ? __ddiv_rn(tot, (double)N) : 0.0, ss = 0.0;
        if (ok) {
            const float mh = __double2float_rn(mu);
            const float ml = __double2float_rn(__dadd_rn(mu, -(double)mh));
            float qh = 0.0f, ql = 0.0f, dmax = 0.0f;
            for (int64_t j = threadIdx.x; j < cols; j += blockDim.x)
                if (!(excl_diag && j == i)) {
                    const float x = row[j];
                    // d = x - mu as dh + dl: TwoSum of x and -mh, then -ml
                    const float dh = __fadd_rn(x, -mh);
                    const float bb = __fsub_rn(dh, x);
                    const float dl = __fsub_rn(__fadd_rn(__fsub_rn(x, __fsub_rn(dh, bb)), __fsub_rn(-mh, bb)), ml);
                    const float p = __fmul_rn(dh, dh);
                    const float pe = __fadd_rn(__fmaf_rn(dh, dh, -p), __fmul_rn(__fmul_rn(2.0f, dh), dl));
                    ff_add2(qh, ql, p, pe);
                    dmax = fmaxf(dmax, fabsf(dh));
                }
            ss = block_sum_ff(qh, ql, shf);
            const float spread = block_max_f(dmax, shf);
            ok = isfinite(ss) && (N <= 1 || spread == 0.0f || spread >= 9.094947e-13f);  // 2^-40
        }
        if (!ok) {  // FP64 two-pass
            double s = 0.0;
            for (int64_t j = threadIdx.x; j < cols; j += blockDim.x)
                if (!(excl_diag && j == i)) s = __dadd_rn(s, (double)row[j]);
            tot = block_sum_d(s, sh);
            mu = N > 0 ? __ddiv_rn(tot, (double)N) : 0.0;
            double q = 0.0;
            for (int64_t j = threadIdx.x; j < cols; j += blockDim.x)
                if (!(excl_diag && j == i)) {
                    const double d = __dadd_rn((double)row[j], -mu);
                    q = __dadd_rn(q, __dmul_rn(d, d));
                }
            ss = block_sum_d(q, sh);
        }
        if (threadIdx.x == 0) {
            mean[i] = __double2float_rn(mu);
            sd[i] = N > ddof ? __double2float_rn(__dsqrt_rn(__ddiv_rn(ss, (double)(N - ddof)))) : 0.0f;
        }
    }
}

template <int CLR>
__global__ void __launch_bounds__(EW_TPB) transform_kernel(const float* __restrict__ A, int64_t n, int64_t lda,
                                                          const float* __restrict__ mean, const float* __restrict__ sd,
                                                          float* __restrict__ out, int64_t ldo) {
    const float isqrt2 = 0.70710678118654752440f;
    for_each_entry(n, n, [&](int64_t i, int64_t j) {
        const float x = A[i * lda + j];
        const float si = sd[i], sj = sd[j];
        const float denom = fabsf(si) < FLT_EPSILON ? 0.0f : __frcp_rn(si);  // (float)(1.0 / sd): double rounding innocuous
        const float zi = __fmul_rn(__fsub_rn(x, mean[i]), denom);
        const float zj = fabsf(sj) < FLT_EPSILON ? 0.0f : __fdiv_rn(__fsub_rn(x, mean[j]), sj);
        out[i * ldo + j] = CLR ? __fsqrt_rn(__fadd_rn(__fmul_rn(zi, zi), __fmul_rn(zj, zj)))
                               : __fmul_rn(__fadd_rn(zi, zj), isqrt2);
    });
}

// Population statistics of each column over the rows: blocks of 32 columns x
// CS_Y row strides (coalesced 128-byte row segments), FP64 partial sums
// combined across the strides in a fixed order.
constexpr int CS_Y = 8;
__global__ void __launch_bounds__(32 * CS_Y) col_stats_kernel(const float* A, int64_t rows, int64_t cols, int64_t lda,
                                                              float* mean, float* sd) {
    __shared__ double sh[CS_Y][33];
    const int64_t j = (int64_t)blockIdx.x * 32 + threadIdx.x;
    const bool live = j < cols;
    double s = 0.0;
    if (live)
        for (int64_t i = threadIdx.y; i < rows; i += CS_Y) s = __dadd_rn(s, (double)A[i * lda + j]);
    sh[threadIdx.y][threadIdx.x] = s;
    __syncthreads();
    double tot = 0.0;
    for (int y = 0; y < CS_Y; ++y) tot = __dadd_rn(tot, sh[y][threadIdx.x]);
    const double mu = rows > 0 ? __ddiv_rn(tot, (double)rows) : 0.0;
    __syncthreads();
    double q = 0.0;
    if (live)
        for (int64_t i = threadIdx.y; i < rows; i += CS_Y) {
            const double d = __dadd_rn((double)A[i * lda + j], -mu);
            q = __dadd_rn(q, __dmul_rn(d, d));
        }
    sh[threadIdx.y][threadIdx.x] = q;
    __syncthreads();
    if (threadIdx.y == 0 && live) {
        double ss = 0.0;
        for (int y = 0; y < CS_Y; ++y) ss = __dadd_rn(ss, sh[y][threadIdx.x]);
        mean[j] = __double2float_rn(mu);
        sd[j] = rows > 0 ? __double2float_rn(__dsqrt_rn(__ddiv_rn(ss, (double)rows))) : 0.0f;
    }
}

__device__ __forceinline__ float zscore(float x, float mean, float sd) {
    return fabsf(sd) < FLT_EPSILON ? 0.0f : __fdiv_rn(__fsub_rn(x, mean), sd);
}

// zscored_stouffer_kernel (CLR = 0) or zscored_clr_kernel (CLR = 1) over a rows x
// cols matrix with row and column statistics.
template <int CLR>
__global__ void __launch_bounds__(EW_TPB) stouffer_tf_kernel(const float* __restrict__ A, int64_t rows, int64_t cols,
                                                            int64_t lda, const float* __restrict__ rmean,
                                                            const float* __restrict__ rsd,
                                                            const float* __restrict__ cmean,
                                                            const float* __restrict__ csd, float* __restrict__ out,
                                                            int64_t ldo) {
    const float isqrt2 = 0.70710678118654752440f;
    for_each_entry(rows, cols, [&](int64_t i, int64_t j) {
        const float x = A[i * lda + j];
        const float zi = zscore(x, rmean[i], rsd[i]);
        const float zj = zscore(x, cmean[j], csd[j]);
        out[i * ldo + j] = CLR ? __fsqrt_rn(__fadd_rn(__fmul_rn(zi, zi), __fmul_rn(zj, zj)))
                               : __fmul_rn(__fadd_rn(zi, zj), isqrt2);
    });
}

}  // namespace

cudaError_t launch_row_stats(const float* A, int64_t rows, int64_t cols, int64_t lda, int excl_diag, int ddof,
                             float* mean, float* sd, cudaStream_t st, int64_t* launches) {
    if (rows <= 0) return cudaSuccess;
    const int64_t grid = rows < 152 * 8 ? rows : 152 * 8;
    row_stats_kernel<<<(unsigned)grid, ST_THREADS, 0, st>>>(A, rows, cols, lda, excl_diag, ddof, mean, sd);
    if (launches) ++*launches;
    return cudaGetLastError();
}

cudaError_t launch_transform(const float* A, int64_t n, int64_t lda, const float* mean, const float* sd, int clr,
                             float* out, int64_t ldo, cudaStream_t st, int64_t* launches) {
    if (n <= 0) return cudaSuccess;
    if (clr) transform_kernel<1><<<ew_grid2d(n, n), 256, 0, st>>>(A, n, lda, mean, sd, out, ldo);
    else transform_kernel<0><<<ew_grid2d(n, n), 256, 0, st>>>(A, n, lda, mean, sd, out, ldo);
    if (launches) ++*launches;
    return cudaGetLastError();
}

cudaError_t launch_col_stats(const float* A, int64_t rows, int64_t cols, int64_t lda, float* mean, float* sd,
                             cudaStream_t st, int64_t* launches) {
    if (cols <= 0) return cudaSuccess;
    col_stats_kernel<<<(unsigned)ceil_div(cols, 32), dim3(32, CS_Y), 0, st>>>(A, rows, cols, lda, mean, sd);
    if (launches) ++*launches;
    return cudaGetLastError();
}

cudaError_t launch_stouffer_tf(const float* A, int64_t rows, int64_t cols, int64_t lda, const float* rmean,
                               const float* rsd, const float* cmean, const float* csd, int clr, float* out,
                               int64_t ldo, cudaStream_t st, int64_t* launches) {
    if (rows <= 0 || cols <= 0) return cudaSuccess;
    if (clr)
        stouffer_tf_kernel<1><<<ew_grid2d(rows, cols), 256, 0, st>>>(A, rows, cols, lda, rmean, rsd, cmean, csd, out,
                                                                     ldo);
    else
        stouffer_tf_kernel<0><<<ew_grid2d(rows, cols), 256, 0, st>>>(A, rows, cols, lda, rmean, rsd, cmean, csd, out,
                                                                     ldo);
    if (launches) ++*launches;
    return cudaGetLastError();
}

}  // namespace mcpg
