// Driver that runs MCPNet's OWN hot-path kernels (compiled from the reference
// headers where they lie, see oracle/Makefile) over whole matrices, standing in
// for the splash InnerProduct / Transform / BinaryOp patterns that are absent
// from the reference snapshot.  Output goes to oracle/_ref/libmcpref.so.
//
// Test infrastructure only: used to pin the C restatement (oracle/mcp_oracle.c)
// and to generate the golden fixtures under tests/golden/.  Nothing in the
// product links it.
//
// Loops follow the reference call sites:
//   compute_mi            apps/pipeline/mcpnet_helper.hpp:56-99
//   compute_maxmin1/2/3   apps/pipeline/mcpnet_helper.hpp:188-196,247-268,335-355
//   compute_ratio         apps/pipeline/mcpnet_helper.hpp:172-184
//   DPI mask + apply      apps/filter/dpi.cpp:236-287
//   MCP3 symmetrisation   apps/filter/mcp.cpp:463-476
//   AP MI (ranks given)   IntegralCumulativeHistogramKernel + AdaptivePartitionRankMIKernel2,
//                         as apps/pipeline/mcpnet_helper.hpp:136-163 (InnerProduct SYMM)
//   Stouffer / CLR        stouffer_vector_kernel / clr_vector_kernel per row with given row
//                         statistics (include/mcp/transform/stouffer.hpp:57-82, clr.hpp:52-73)
//   AUPR / AUROC          aupr_kernel / auroc_kernel::operator()(pos, count, neg, count)
//                         include/mcp/transform/aupr.hpp:565-584, auroc.hpp:562-579
// The InnerProduct SYMM=true pattern is restated as "compute j >= i, mirror".
#include <cstdint>
#include <cstring>
#include <vector>
#include <limits>
#include <algorithm>

#include "mcp/correlation/BSplineMI.hpp"
#include "mcp/filter/mcp.hpp"
#include "mcp/filter/dpi.hpp"
#include "mcp/filter/threshold.hpp"
#include "mcp/transform/combine.hpp"
#include "mcp/transform/aupr.hpp"
#include "mcp/transform/auroc.hpp"
#include "mcp/correlation/AdaptivePartitioningMI.hpp"
#include "mcp/transform/stouffer.hpp"
#include "mcp/transform/clr.hpp"

namespace {

template <typename T>
void bspline_weights(T const* X, int64_t n, int64_t m, int64_t ldx, int bins, int order,
                     T* W /* n x (bins*m+1) */) {
    mcp::kernel::MinMaxScale<T> scaler;
    mcp::kernel::BSplineWeightsKernel<T> wk(bins, order, (int)m);
    std::vector<T> scaled(m);
    const int64_t ldw = (int64_t)bins * m + 1;
#pragma omp parallel for firstprivate(scaled) schedule(dynamic, 4)
    for (int64_t g = 0; g < n; ++g) {
        scaler(X + g * ldx, (size_t)m, scaled.data());
        wk(scaled.data(), (size_t)m, W + g * ldw);
    }
}

template <typename T>
void bspline_mi(T const* X, int64_t n, int64_t m, int64_t ldx, int bins, int order,
                T* MI, int64_t ldmi, T* W_out) {
    const int64_t ldw = (int64_t)bins * m + 1;
    std::vector<T> W((size_t)(n * ldw));
    bspline_weights(X, n, m, ldx, bins, order, W.data());
    if (W_out) std::memcpy(W_out, W.data(), W.size() * sizeof(T));
    mcp::kernel::BSplineMIKernel<T> mik(bins, (int)m);
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t i = 0; i < n; ++i) {
        for (int64_t j = i; j < n; ++j) {
            T v = mik(W.data() + i * ldw, W.data() + j * ldw, (size_t)ldw);
            MI[i * ldmi + j] = v;
            MI[j * ldmi + i] = v;
        }
    }
}

template <typename T>
void maxmin(T const* A, int64_t lda, T const* B, int64_t ldb, int64_t rows, int64_t cols,
            int64_t k, T* C, int64_t ldc) {
    mcp::kernel::mcp2_maxmin_kernel<T, false, true> kern;
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t i = 0; i < rows; ++i)
        for (int64_t j = 0; j < cols; ++j)
            C[i * ldc + j] = kern(A + i * lda, B + j * ldb, (size_t)k);
}

template <typename T>
void maxmin_symm(T const* A, int64_t lda, int64_t n, T* C, int64_t ldc) {
    mcp::kernel::mcp2_maxmin_kernel<T, false, true> kern;
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t i = 0; i < n; ++i)
        for (int64_t j = i; j < n; ++j) {
            T v = kern(A + i * lda, A + j * lda, (size_t)n);
            C[i * ldc + j] = v;
            C[j * ldc + i] = v;
        }
}

template <typename T>
void maxmin_masked(T const* A, int64_t lda, T const* B, int64_t ldb, int64_t rows, int64_t cols, int64_t k,
                   T const* mask, T* C, int64_t ldc) {
    std::vector<T> tfs(mask, mask + k);
    mcp::kernel::mcp2_maxmin_kernel<T, true, true> kern(tfs);
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t i = 0; i < rows; ++i)
        for (int64_t j = 0; j < cols; ++j)
            C[i * ldc + j] = kern(A + i * lda, B + j * ldb, (size_t)k);
}

template <typename T>
int64_t dpi_tf(T const* A, int64_t n, int64_t lda, T tol, T const* tfs_in, T* out, int64_t ldo, uint8_t* mask_out) {
    std::vector<T> tfs(tfs_in, tfs_in + n);
    mcp::kernel::dpi_tf_kernel<T> kern(tfs, tol);
    std::vector<uint8_t> mask((size_t)(n * n));
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t x = 0; x < n; ++x)
        for (int64_t z = 0; z < n; ++z)
            mask[x * n + z] = kern((size_t)x, (size_t)z, A + x * lda, A + z * lda, (size_t)n) ? 1 : 0;
    mcp::kernel::mask<T, true> masker;
    bool* b = new bool[n];
    for (int64_t x = 0; x < n; ++x) {
        for (int64_t z = 0; z < n; ++z) b[z] = mask[x * n + z] != 0;
        masker(A + x * lda, b, (size_t)n, out + x * ldo);
    }
    delete[] b;
    if (mask_out) std::memcpy(mask_out, mask.data(), mask.size());
    return (int64_t)masker.processed;
}

template <typename T>
void ratio(T const* A, int64_t lda, T const* M, int64_t ldm, int64_t rows, int64_t cols,
           T* R, int64_t ldr) {
    mcp::kernel::ratio_kernel<T, T> kern;
    for (int64_t i = 0; i < rows; ++i) kern(A + i * lda, M + i * ldm, (size_t)cols, R + i * ldr);
}

template <typename T>
void max_transpose(T const* M, int64_t n, int64_t ldm, T* out, int64_t ldo) {
    mcp::kernel::max_kernel<T> kern;
    std::vector<T> row(n);
    for (int64_t i = 0; i < n; ++i) {
        for (int64_t j = 0; j < n; ++j) row[j] = M[j * ldm + i];
        kern(M + i * ldm, row.data(), (size_t)n, out + i * ldo);
    }
}

template <typename T>
int64_t dpi(T const* A, int64_t n, int64_t lda, double tol, T* out, int64_t ldo, uint8_t* mask_out) {
    mcp::kernel::dpi_kernel<T> kern(tol);
    std::vector<uint8_t> mask((size_t)(n * n));
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t x = 0; x < n; ++x)
        for (int64_t z = 0; z < n; ++z)
            mask[x * n + z] = kern((size_t)x, (size_t)z, A + x * lda, A + z * lda, (size_t)n) ? 1 : 0;
    mcp::kernel::mask<T, true> masker;
    bool* b = new bool[n];
    for (int64_t x = 0; x < n; ++x) {
        for (int64_t z = 0; z < n; ++z) b[z] = mask[x * n + z] != 0;
        masker(A + x * lda, b, (size_t)n, out + x * ldo);
    }
    delete[] b;
    if (mask_out) std::memcpy(mask_out, mask.data(), mask.size());
    return (int64_t)masker.processed;
}

}  // namespace

extern "C" {

void ref_bspline_weights_f32(const float* X, int64_t n, int64_t m, int64_t ldx, int bins, int order, float* W) {
    bspline_weights<float>(X, n, m, ldx, bins, order, W);
}
void ref_bspline_weights_f64(const double* X, int64_t n, int64_t m, int64_t ldx, int bins, int order, double* W) {
    bspline_weights<double>(X, n, m, ldx, bins, order, W);
}
void ref_bspline_mi_f32(const float* X, int64_t n, int64_t m, int64_t ldx, int bins, int order,
                        float* MI, int64_t ldmi, float* W_out) {
    bspline_mi<float>(X, n, m, ldx, bins, order, MI, ldmi, W_out);
}
void ref_bspline_mi_f64(const double* X, int64_t n, int64_t m, int64_t ldx, int bins, int order,
                        double* MI, int64_t ldmi, double* W_out) {
    bspline_mi<double>(X, n, m, ldx, bins, order, MI, ldmi, W_out);
}
// MI of the pairs (i, j), i in [r0, r1), all j, from reference weight rows
// (a row slab of the InnerProduct, used to time a bounded CPU sample).
void ref_bspline_mi_rows_f32(const float* W, int64_t n, int64_t m, int bins, int64_t r0, int64_t r1, float* out,
                             int64_t ldo) {
    const int64_t ldw = (int64_t)bins * m + 1;
    mcp::kernel::BSplineMIKernel<float> mik(bins, (int)m);
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t i = r0; i < r1; ++i)
        for (int64_t j = 0; j < n; ++j) out[(i - r0) * ldo + j] = mik(W + i * ldw, W + j * ldw, (size_t)ldw);
}
void ref_maxmin_f32(const float* A, int64_t lda, const float* B, int64_t ldb, int64_t rows, int64_t cols,
                    int64_t k, float* C, int64_t ldc) {
    maxmin<float>(A, lda, B, ldb, rows, cols, k, C, ldc);
}
void ref_maxmin_symm_f32(const float* A, int64_t lda, int64_t n, float* C, int64_t ldc) {
    maxmin_symm<float>(A, lda, n, C, ldc);
}
void ref_ratio_f32(const float* A, int64_t lda, const float* M, int64_t ldm, int64_t rows, int64_t cols,
                   float* R, int64_t ldr) {
    ratio<float>(A, lda, M, ldm, rows, cols, R, ldr);
}
void ref_max_transpose_f32(const float* M, int64_t n, int64_t ldm, float* out, int64_t ldo) {
    max_transpose<float>(M, n, ldm, out, ldo);
}
void ref_maxmin_masked_f32(const float* A, int64_t lda, const float* B, int64_t ldb, int64_t rows, int64_t cols,
                           int64_t k, const float* mask, float* C, int64_t ldc) {
    maxmin_masked<float>(A, lda, B, ldb, rows, cols, k, mask, C, ldc);
}
int64_t ref_dpi_tf_f32(const float* A, int64_t n, int64_t lda, float tol, const float* tfs, float* out, int64_t ldo,
                       uint8_t* mask) {
    return dpi_tf<float>(A, n, lda, tol, tfs, out, ldo, mask);
}
// tol arrives as float, as under `--single` (apps/filter/dpi.cpp:63,69-74).
int64_t ref_dpi_f32(const float* A, int64_t n, int64_t lda, float tol, float* out, int64_t ldo, uint8_t* mask) {
    return dpi<float>(A, n, lda, (double)tol, out, ldo, mask);
}

// AUPR and AUROC of score vectors with the reference's kernels; IT = float or
// double comparisons, OT = double (the sums before any rounding to float).
void ref_aupr_auroc_f32(const float* pos, int64_t np, const float* neg, int64_t nn, double* out) {
    mcp::kernel::aupr_kernel<float, char, double> pr;
    mcp::kernel::auroc_kernel<float, char, double> roc;
    out[0] = pr(pos, (size_t)np, neg, (size_t)nn);
    out[1] = roc(pos, (size_t)np, neg, (size_t)nn);
}
void ref_aupr_auroc_f64(const double* pos, int64_t np, const double* neg, int64_t nn, double* out) {
    mcp::kernel::aupr_kernel<double, char, double> pr;
    mcp::kernel::auroc_kernel<double, char, double> roc;
    out[0] = pr(pos, (size_t)np, neg, (size_t)nn);
    out[1] = roc(pos, (size_t)np, neg, (size_t)nn);
}

// Adaptive-partitioning MI from integer ranks (n x m, ranks in [0, m)) with the
// reference's cumulative-histogram and MI kernels; out[i][j] = out[j][i] for
// j >= i computed as kernel(i, j), as the symmetric InnerProduct does.
void ref_ap_mi_f32(const int64_t* ranks, int64_t n, int64_t m, float* out, int64_t ldo) {
    std::vector<size_t> R((size_t)(n * m)), H((size_t)(n * (m + 1)), 0);
    for (int64_t i = 0; i < n * m; ++i) R[(size_t)i] = (size_t)ranks[i];
    mcp::kernel::IntegralCumulativeHistogramKernel<size_t, 0> hist;
    for (int64_t i = 0; i < n; ++i) hist(R.data() + i * m, (size_t)m, H.data() + i * (m + 1));
#pragma omp parallel
    {
        mcp::kernel::AdaptivePartitionRankMIKernel2<size_t, float, 0> k(H.data(), (size_t)(m + 1) * sizeof(size_t));
#pragma omp for schedule(dynamic, 1)
        for (int64_t i = 0; i < n; ++i)
            for (int64_t j = i; j < n; ++j) {
                float v = k((size_t)i, (size_t)j, R.data() + i * m, R.data() + j * m, (size_t)m);
                out[i * ldo + j] = v;
                out[j * ldo + i] = v;
            }
    }
}

// The reference's Stouffer (clr = 0) or CLR (clr = 1) vector kernel over every
// row of the n x n matrix A with the given per-row (mean, sd) as float pairs,
// as GlobalReduceTransform hands them to the kernel (aux1 = row i's, aux2 =
// every row's).
void ref_transform_f32(const float* A, int64_t n, int64_t lda, const float* mean, const float* sd, int clr,
                       float* out, int64_t ldo) {
    std::vector<std::pair<float, float>> aux((size_t)n);
    for (int64_t i = 0; i < n; ++i) aux[(size_t)i] = std::make_pair(mean[i], sd[i]);
    mcp::kernel::stouffer_vector_kernel<float> st;
    mcp::kernel::clr_vector_kernel<float> cl;
    for (int64_t i = 0; i < n; ++i) {
        if (clr) cl(A + i * lda, aux.data() + i, aux.data(), (size_t)n, out + i * ldo);
        else st(A + i * lda, aux.data() + i, aux.data(), (size_t)n, out + i * ldo);
    }
}

// zscored_stouffer_kernel<float> (include/mcp/transform/stouffer.hpp:84-100)
// over rows of the row z-scores zi and column z-scores zj (rows x cols, ld
// cols), as the BinaryOp pattern of compute_stouffer_tf hands them over.
void ref_zscored_stouffer_f32(const float* zi, const float* zj, int64_t rows, int64_t cols, float* out) {
    mcp::kernel::zscored_stouffer_kernel<float> k;
    for (int64_t i = 0; i < rows; ++i) k(zi + i * cols, zj + i * cols, (size_t)cols, out + i * cols);
}

// zscored_clr_kernel<float> (include/mcp/transform/clr.hpp:75-88), as the
// transform app's GlobalBinaryOp hands rows over (apps/transform/transform.cpp:192-198).
void ref_zscored_clr_f32(const float* zi, const float* zj, int64_t rows, int64_t cols, float* out) {
    mcp::kernel::zscored_clr_kernel<float> k;
    for (int64_t i = 0; i < rows; ++i) k(zi + i * cols, zj + i * cols, (size_t)cols, out + i * cols);
}

}  // extern "C"
