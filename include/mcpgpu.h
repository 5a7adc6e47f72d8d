/*
 * mcpgpu -- GB300 (sm_103a) implementation of MCPNet's compute core behind a
 * plain C ABI: B-spline mutual information, max-min (maximum-capacity path)
 * products with the MCP ratio, the DPI filter and the max-capacity closure.
 *
 * Conventions
 *  - Matrices are row-major with an explicit leading dimension (elements), the
 *    layout of MCPNet's splash::ds::aligned_matrix (rows may be padded).
 *  - Every call returns an int status (MCPG_OK == 0, negative on error) and
 *    never aborts; mcpg_last_error() gives the message of the last failure on
 *    that handle.
 *  - Host-buffer entry points (no suffix) take HOST pointers, copy in, compute
 *    and copy out; they return when the results are in the caller's buffers.
 *  - Device entry points (suffix _dev) take DEVICE pointers and are
 *    asynchronous on the handle's stream (mcpg_set_stream); call
 *    mcpg_synchronize() before reading results.  Scalars they return (removed
 *    counts, iteration counts) are read back synchronously.
 *  - A handle is not thread-safe: one host thread, one CUDA stream per handle.
 *    The library owns the device scratch memory of a handle.
 *  - MI is in bits (log2), as in the reference.
 *
 * Reference interfaces replaced (paths relative to the MCPNet source tree):
 *  each function names the reference functor / helper whose whole-matrix
 *  application it performs.
 */
#ifndef MCPGPU_H
#define MCPGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define MCPG_API __attribute__((visibility("default")))
#else
#define MCPG_API
#endif

typedef struct mcpg_handle mcpg_handle;

/* ---- status codes ---- */
#define MCPG_OK 0
#define MCPG_ERR_ARG (-1)           /* bad argument: null pointer, bad shape, bad enum */
#define MCPG_ERR_OOM (-2)           /* device or host allocation failed */
#define MCPG_ERR_CUDA (-3)          /* a CUDA runtime/driver call failed */
#define MCPG_ERR_NOT_CONVERGED (-4) /* closure still changing after max_iter products */
#define MCPG_ERR_UNSUPPORTED (-5)   /* feature unavailable on this device / build */
#define MCPG_ERR_DEVICE_TIMEOUT (-6)/* a bounded device-side wait gave up */
#define MCPG_ERR_SCRATCH_LIMIT (-7) /* problem too large for the no-allocation entry point's static scratch */

/* ---- MI contraction precision (mcpg_bspline_mi*) ---- */
#define MCPG_MI_FP32 0   /* FP32 weights, FP32 CUDA-core contraction */
#define MCPG_MI_BF16 1   /* weights rounded once to BF16, tcgen05 tensor cores, FP32 accumulate */
#define MCPG_MI_BF16X3 2 /* hi+lo BF16 split: hi*hi' + hi*lo' + lo*hi' on tcgen05 */
#define MCPG_MI_FP16 3   /* weights rounded once to FP16, tcgen05 */
#define MCPG_MI_FP16X3 4 /* hi+lo FP16 split on tcgen05 */
#define MCPG_MI_BF16F8 5 /* BF16 hi*hi' (tcgen05 kind::f16) plus an E4M3 hi*lo' + lo*hi' correction
                            (kind::f8f6f4, twice the rate) in the same FP32 accumulator */

/* ---- library / handle ---- */
MCPG_API int mcpg_version(void);
MCPG_API const char* mcpg_status_string(int status);
MCPG_API int mcpg_create(mcpg_handle** out, int device);
MCPG_API int mcpg_destroy(mcpg_handle* h);
MCPG_API const char* mcpg_last_error(const mcpg_handle* h);
MCPG_API int mcpg_set_stream(mcpg_handle* h, void* cuda_stream);
MCPG_API int mcpg_synchronize(mcpg_handle* h);
/* Number of kernels this handle has launched since creation (instrumentation). */
MCPG_API int64_t mcpg_kernel_launches(const mcpg_handle* h);
/* Per-kernel timing: with profiling on, the handle records CUDA events around
 * every kernel it launches.  mcpg_profile() (re)starts or stops recording and
 * clears what was recorded; mcpg_profile_report() synchronizes the stream and
 * writes {"<kernel>": {"launches": L, "ms": T}, ...} into buf, returning the
 * bytes needed (including the terminating NUL). */
MCPG_API int mcpg_profile(mcpg_handle* h, int enable);
MCPG_API int64_t mcpg_profile_report(mcpg_handle* h, char* buf, int64_t len);

/* ---- B-spline mutual information ----
 * Replaces compute_mi (apps/pipeline/mcpnet_helper.hpp:56-99): MinMaxScale
 * (include/mcp/correlation/BSplineMI.hpp:74-116) -> BSplineWeightsKernel
 * (:119-274) -> InnerProduct<BSplineMIKernel, SYMM=true> (:276-500).
 * X: n genes x m samples (ldx >= m).  MI: n x n (ldmi >= n), symmetric, bits.
 * H (nullable): n per-gene marginal entropies in bits, computed in FP64.
 * bins >= order >= 1, bins <= 32; order in 1..8. */
MCPG_API int mcpg_bspline_mi(mcpg_handle* h, const float* X, int64_t n, int64_t m, int64_t ldx,
                             int bins, int order, int precision,
                             float* MI, int64_t ldmi, double* H);
MCPG_API int mcpg_bspline_mi_dev(mcpg_handle* h, const float* X, int64_t n, int64_t m, int64_t ldx,
                                 int bins, int order, int precision,
                                 float* MI, int64_t ldmi, double* H);

/* ---- B-spline weights alone (the Transform<BSplineWeightsKernel> step) ----
 * Whole-matrix BSplineWeightsKernel (BSplineMI.hpp:248-273) after MinMaxScale,
 * as mcpnet_helper.hpp:58-80.  W: n rows of bins*m+1 floats in the reference's
 * own row layout W[g][a*m + s], with W[g][bins*m] = H_g (FP64 value rounded to
 * float).  H (nullable): FP64 marginal entropies.  The weights are bit-identical
 * to the reference's float weights when the reference is built without FMA
 * contraction. */
MCPG_API int mcpg_bspline_weights(mcpg_handle* h, const float* X, int64_t n, int64_t m, int64_t ldx,
                                  int bins, int order, float* W, double* H);
MCPG_API int mcpg_bspline_weights_dev(mcpg_handle* h, const float* X, int64_t n, int64_t m, int64_t ldx,
                                      int bins, int order, float* W, double* H);

/* ---- max-min product ----
 * C[i][j] = max_k min(A[i][k], B[j][k]), i < rows, j < cols, k < k_len: the
 * whole-matrix application of mcp2_maxmin_kernel<float,false,true>
 * (include/mcp/filter/mcp.hpp:72-93) under splash InnerProduct(A, B).
 * Bit-exact (every output is one of the inputs).  Empty k range gives -inf. */
MCPG_API int mcpg_maxmin(mcpg_handle* h, const float* A, int64_t lda, const float* B, int64_t ldb,
                         int64_t rows, int64_t cols, int64_t k_len, float* C, int64_t ldc);
MCPG_API int mcpg_maxmin_dev(mcpg_handle* h, const float* A, int64_t lda, const float* B, int64_t ldb,
                             int64_t rows, int64_t cols, int64_t k_len, float* C, int64_t ldc);

/* ---- MCP ratio ----
 * R = ratio_kernel<float,float>(A, M) (include/mcp/transform/combine.hpp:210-222):
 * |a| < FLT_EPSILON -> 0; |m| < FLT_EPSILON -> FLT_MAX; else (float)(a / m). */
MCPG_API int mcpg_ratio(mcpg_handle* h, const float* A, int64_t lda, const float* M, int64_t ldm,
                        int64_t rows, int64_t cols, float* R, int64_t ldr);
MCPG_API int mcpg_ratio_dev(mcpg_handle* h, const float* A, int64_t lda, const float* M, int64_t ldm,
                            int64_t rows, int64_t cols, float* R, int64_t ldr);

/* ---- diagonal reset (apps/pipeline/mcpnet.cpp:299-308) ----
 * A[i][i] = value for i < min(rows, cols); a negative value leaves A untouched. */
MCPG_API int mcpg_set_diagonal_dev(mcpg_handle* h, float* A, int64_t rows, int64_t cols, int64_t lda, float value);

/* ---- MCP scores of path length 2, 3 or 4 ----
 * A: n x n MI matrix with its diagonal already set (0 in the reference default).
 * path_len 2: M = A (x) A                       compute_mcp2 (mcpnet_helper.hpp:199-206)
 * path_len 3: M = A (x) (A (x) A)               compute_mcp3 (mcpnet_helper.hpp:271-278)
 *             symmetrize != 0 additionally takes max(M, M^T) as the mcp app
 *             does (apps/filter/mcp.cpp:463-476)
 * path_len 4: M = (A (x) A) (x) (A (x) A)       compute_mcp4 (mcpnet_helper.hpp:358-365)
 * maxmin_out (nullable) receives M, ratio_out (nullable) receives ratio(A, M). */
MCPG_API int mcpg_mcp(mcpg_handle* h, const float* A, int64_t n, int64_t lda, int path_len, int symmetrize,
                      float* maxmin_out, int64_t ldm, float* ratio_out, int64_t ldr);
MCPG_API int mcpg_mcp_dev(mcpg_handle* h, const float* A, int64_t n, int64_t lda, int path_len, int symmetrize,
                          float* maxmin_out, int64_t ldm, float* ratio_out, int64_t ldr);

/* ---- the three max-min products at once (compute_maxmins, mcpnet_helper.hpp:437-460) ----
 * M1 = A (x) A, M2 = A (x) M1, M3 = M1 (x) M1 with M1 computed once, and the
 * MCP2 / MCP3 / MCP4 scores R2 = ratio(A, M1), R3 = ratio(A, M2),
 * R4 = ratio(A, M3) fused into the products.  Every output is nullable (M1 is
 * kept in scratch when not requested); a product whose outputs are all null
 * is skipped. */
MCPG_API int mcpg_maxmins_dev(mcpg_handle* h, const float* A, int64_t n, int64_t lda, float* M1, int64_t ld1,
                              float* M2, int64_t ld2, float* M3, int64_t ld3, float* R2, int64_t ldr2, float* R3,
                              int64_t ldr3, float* R4, int64_t ldr4);
MCPG_API int mcpg_maxmins(mcpg_handle* h, const float* A, int64_t n, int64_t lda, float* M1, int64_t ld1,
                          float* M2, int64_t ld2, float* M3, int64_t ld3, float* R2, int64_t ldr2, float* R3,
                          int64_t ldr3, float* R4, int64_t ldr4);

/* ---- ensemble combination (compute_combo, mcpnet_helper.hpp:507-573) ----
 * out = mi / (c0 mi + c1 M1 + c2 M2 + c3 M3), the combination summed in
 * double in that order (a term skipped when its coefficient is 0, added
 * unscaled when it is 1), |mi| < FLT_EPSILON -> 0, |combination| <
 * FLT_EPSILON -> FLT_MAX, else the double quotient rounded to float.
 * coeffs: 4 doubles on the host; Mk may be null when ck == 0. */
MCPG_API int mcpg_combo_dev(mcpg_handle* h, const float* mi, int64_t ldm, const float* M1, int64_t ld1,
                            const float* M2, int64_t ld2, const float* M3, int64_t ld3, int64_t rows, int64_t cols,
                            const double* coeffs, float* out, int64_t ldo);
MCPG_API int mcpg_combo(mcpg_handle* h, const float* mi, int64_t ldm, const float* M1, int64_t ld1,
                        const float* M2, int64_t ld2, const float* M3, int64_t ld3, int64_t rows, int64_t cols,
                        const double* coeffs, float* out, int64_t ldo);

/* ---- DPI filter ----
 * dpi_kernel<float> (include/mcp/filter/dpi.hpp:42-69) over all (x, z), then
 * mask<float,true> (include/mcp/filter/threshold.hpp:33-54), as apps/filter/dpi.cpp:236-287.
 * tol is the float tolerance of `dpi --single`; the multiplier 1/(1-tol) is
 * formed in double.  out = deleted ? 0 : A; mask (nullable, n*n bytes, row-major)
 * gets 1 for deleted entries; removed (nullable) gets the reference's
 * "Mask removing N elements" count. */
MCPG_API int mcpg_dpi(mcpg_handle* h, const float* A, int64_t n, int64_t lda, float tol,
                      float* out, int64_t ldo, uint8_t* mask, int64_t* removed);
MCPG_API int mcpg_dpi_dev(mcpg_handle* h, const float* A, int64_t n, int64_t lda, float tol,
                          float* out, int64_t ldo, uint8_t* mask, int64_t* removed);

/* ---- TF-restricted variants ----
 * tfs / mask are HOST arrays of floats.  tfs is the reference's TF vector
 * (load_tfs, apps/pipeline/mcpnet_helper.hpp:1074-1123): one value per gene,
 * > 0 marks a transcription factor (the reference stores +max / lowest, which
 * are +inf / -inf in float).
 *
 * mcpg_maxmin_masked: mcp2_maxmin_kernel<float,true,true> (mcp.hpp:72-93) as a
 * whole-matrix InnerProduct: C[i][j] = max_k min(mask[k], min(A[i][k], B[j][k])),
 * mask of k_len values.  Bit-exact for any mask. */
MCPG_API int mcpg_maxmin_masked(mcpg_handle* h, const float* A, int64_t lda, const float* B, int64_t ldb,
                                int64_t rows, int64_t cols, int64_t k_len, const float* mask, float* C, int64_t ldc);
MCPG_API int mcpg_maxmin_masked_dev(mcpg_handle* h, const float* A, int64_t lda, const float* B, int64_t ldb,
                                    int64_t rows, int64_t cols, int64_t k_len, const float* mask, float* C,
                                    int64_t ldc);
/* compute_mcp{2,3,4}_tfs (mcpnet_helper.hpp:209-243, 281-333, 367-434) with
 * tf_gene_transition in 0..1 (path 2), 0..2 (path 3), 0..3 (path 4).  A is the
 * n x n MI matrix (diagonal already set); outputs are t x n with t = number of
 * TFs, rows in gene order: maxmin_out gets the max-min matrix, ratio_out the
 * MCP score ratio(tfs_to_genes, maxmin).  Nothing is written when t == 0. */
MCPG_API int mcpg_mcp_tf(mcpg_handle* h, const float* A, int64_t n, int64_t lda, const float* tfs, int path_len,
                         int tf_gene_transition, float* maxmin_out, int64_t ldm, float* ratio_out, int64_t ldr);
MCPG_API int mcpg_mcp_tf_dev(mcpg_handle* h, const float* A, int64_t n, int64_t lda, const float* tfs,
                             int path_len, int tf_gene_transition, float* maxmin_out, int64_t ldm,
                             float* ratio_out, int64_t ldr);
/* dpi_tf_kernel (dpi.hpp:74-110) over all (x, z), then mask<float,true>: an
 * edge between a TF and a non-TF is only deleted through TF intermediates; the
 * tolerance multiplier is kept in float as the reference's IT member.  out is
 * n x n (the dpi app then keeps the TF rows); mask / removed as mcpg_dpi. */
MCPG_API int mcpg_dpi_tf(mcpg_handle* h, const float* A, int64_t n, int64_t lda, float tol, const float* tfs,
                         float* out, int64_t ldo, uint8_t* mask, int64_t* removed);
MCPG_API int mcpg_dpi_tf_dev(mcpg_handle* h, const float* A, int64_t n, int64_t lda, float tol, const float* tfs,
                             float* out, int64_t ldo, uint8_t* mask, int64_t* removed);
/* compute_maxmins_tfs (mcpnet_helper.hpp:470-505), the TF form of the
 * ensemble's three products.  With T the TF rows of the n x n MI matrix A
 * (t x n, gene order; filter_local_mat_rows_by_tfs, mcpnet.cpp:317-325) and
 * (x)m the TF-masked product of mcpg_maxmin_masked:
 *   M1 = T (x)m A,  M2 = M1 (x)m A,  M3 = M1 (x)m (A (x)m A).
 * Every output is t x n and nullable; T (nullable) gets the TF rows, which are
 * the mi operand of the TF ensemble.  Nothing is written when t == 0. */
MCPG_API int mcpg_maxmins_tf(mcpg_handle* h, const float* A, int64_t n, int64_t lda, const float* tfs, float* T,
                             int64_t ldt, float* M1, int64_t ld1, float* M2, int64_t ld2, float* M3, int64_t ld3);
MCPG_API int mcpg_maxmins_tf_dev(mcpg_handle* h, const float* A, int64_t n, int64_t lda, const float* tfs,
                                 float* T, int64_t ldt, float* M1, int64_t ld1, float* M2, int64_t ld2, float* M3,
                                 int64_t ld3);

/* ---- adjoints (no counterpart in the reference) ----
 * Forward/backward pairs for sample-level sensitivity of MCP scores.  Every
 * backward ACCUMULATES (+=) into its gradient outputs, except
 * mcpg_bspline_mi_bwd, which writes dX.
 *
 * mcpg_maxmin_witness: the product C = A (x) B plus, per output, the witness
 * K[i][j] = the first k attaining the maximum (-1 where C is -inf).
 * mcpg_maxmin_bwd: routes dC[i][j] to A[i][k*] when A[i][k*] <= B[j][k*] (the
 * operand std::min returns on a tie) else to B[j][k*]; k* from K when given
 * (saved witness), else recomputed from C as the first k with
 * min(A[i][k], B[j][k]) == C[i][j] (cheap when dC is sparse).  dA and dB may be
 * the same buffer when A and B are.  Accumulation uses atomics, so the last
 * bits of a sum can vary between runs. */
MCPG_API int mcpg_maxmin_witness(mcpg_handle* h, const float* A, int64_t lda, const float* B, int64_t ldb,
                                 int64_t rows, int64_t cols, int64_t k_len, float* C, int64_t ldc, int32_t* K,
                                 int64_t ldk);
MCPG_API int mcpg_maxmin_witness_dev(mcpg_handle* h, const float* A, int64_t lda, const float* B, int64_t ldb,
                                     int64_t rows, int64_t cols, int64_t k_len, float* C, int64_t ldc, int32_t* K,
                                     int64_t ldk);
MCPG_API int mcpg_maxmin_bwd(mcpg_handle* h, const float* A, int64_t lda, const float* B, int64_t ldb,
                             int64_t rows, int64_t cols, int64_t k_len, const float* C, int64_t ldc,
                             const float* dC, int64_t lddc, const int32_t* K, int64_t ldk, float* dA, int64_t ldda,
                             float* dB, int64_t lddb);
MCPG_API int mcpg_maxmin_bwd_dev(mcpg_handle* h, const float* A, int64_t lda, const float* B, int64_t ldb,
                                 int64_t rows, int64_t cols, int64_t k_len, const float* C, int64_t ldc,
                                 const float* dC, int64_t lddc, const int32_t* K, int64_t ldk, float* dA,
                                 int64_t ldda, float* dB, int64_t lddb);
/* Adjoint of ratio_kernel: where |A| and |M| are at least FLT_EPSILON,
 * dA += dR / M and dM -= dR * A / M^2 (elsewhere the ratio is constant). */
MCPG_API int mcpg_ratio_bwd_dev(mcpg_handle* h, const float* A, int64_t lda, const float* M, int64_t ldm,
                                int64_t rows, int64_t cols, const float* dR, int64_t lddr, float* dA, int64_t ldda,
                                float* dM, int64_t lddm);
/* Adjoint of mcpg_bspline_mi (FP32): given G = dL/dMI (n x n, all ordered
 * entries; the diagonal is ignored), writes dX = dL/dX (n x m).  Goes through
 * MI_ij = H_i + H_j - H_ij (cells with p = 0 contribute no gradient), the
 * B-spline weight derivatives as a contraction of Gs_ij (log2 P_ab + 1/ln 2)
 * with the weights, and the min-max scaling including its min / max samples.
 * bins <= 12. */
MCPG_API int mcpg_bspline_mi_bwd(mcpg_handle* h, const float* X, int64_t n, int64_t m, int64_t ldx, int bins,
                                 int order, const float* G, int64_t ldg, float* dX, int64_t lddx);
MCPG_API int mcpg_bspline_mi_bwd_dev(mcpg_handle* h, const float* X, int64_t n, int64_t m, int64_t ldx, int bins,
                                     int order, const float* G, int64_t ldg, float* dX, int64_t lddx);

/* ---- maximum-capacity closure (no counterpart routine in the reference) ----
 * Repeated squaring B <- max(B, B (x) B) from B = A until no entry changes,
 * with (x) the reference's max_of_pairmin (include/mcp/filter/simd_maxmin.hpp:30-46).
 * A must be symmetric.  iterations (nullable) gets the number of products.
 * Returns MCPG_ERR_NOT_CONVERGED (out holds the last iterate) if max_iter
 * products did not reach the fixed point. */
MCPG_API int mcpg_closure(mcpg_handle* h, const float* A, int64_t n, int64_t lda, int max_iter,
                          float* out, int64_t ldo, int* iterations);
MCPG_API int mcpg_closure_dev(mcpg_handle* h, const float* A, int64_t n, int64_t lda, int max_iter,
                              float* out, int64_t ldo, int* iterations);

/* ---- adaptive-partitioning MI (the reference's default MI method) ----
 * compute_ap_mi (apps/pipeline/mcpnet_helper.hpp:101-164; apps/correlation/mi.cpp:119-178):
 *   1. optional noise U[0, noise) added to every value (the apps add U[0, 1e-5)
 *      to break ties, mi.cpp:121-131; here a seeded counter-based generator, so
 *      the draw differs from the reference's);
 *   2. rank transform, descending (splash::kernel::Rank<T, size_t, 0, false>;
 *      the splash source is absent from the reference: tied values share the
 *      lowest rank here);
 *   3. IntegralCumulativeHistogramKernel (include/mcp/correlation/
 *      AdaptivePartitioningMI.hpp:414-438) and AdaptivePartitionRankMIKernel2
 *      (:443-648) for every pair j >= i, mirrored (symmetric InnerProduct).
 * MI is n x n float (bits).  Given the same ranks the result equals the
 * reference's kernel except where CUDA's and the C library's log2 differ in
 * the last bit.  m <= 16384 (MCPG_ERR_UNSUPPORTED above).
 * mcpg_ap_ranks_dev: step 1-2 only (ranks: int32, n x ldr).
 * mcpg_ap_mi_ranks[_dev]: step 3 from caller-supplied ranks in [0, m). */
MCPG_API int mcpg_ap_ranks_dev(mcpg_handle* h, const float* X, int64_t n, int64_t m, int64_t ldx, float noise,
                               uint64_t seed, int32_t* R, int64_t ldr);
MCPG_API int mcpg_ap_mi_ranks(mcpg_handle* h, const int32_t* R, int64_t n, int64_t m, int64_t ldr, float* MI,
                              int64_t ldmi);
MCPG_API int mcpg_ap_mi_ranks_dev(mcpg_handle* h, const int32_t* R, int64_t n, int64_t m, int64_t ldr, float* MI,
                                  int64_t ldmi);
MCPG_API int mcpg_ap_mi(mcpg_handle* h, const float* X, int64_t n, int64_t m, int64_t ldx, float noise,
                        uint64_t seed, float* MI, int64_t ldmi);
MCPG_API int mcpg_ap_mi_dev(mcpg_handle* h, const float* X, int64_t n, int64_t m, int64_t ldx, float noise,
                            uint64_t seed, float* MI, int64_t ldmi);

/* ---- Stouffer / CLR transforms ----
 * compute_stouffer (apps/pipeline/mcpnet_helper.hpp:575-586) and the transform
 * app (apps/transform/transform.cpp:214-231): per-row statistics, then per entry
 * stouffer_vector_kernel (include/mcp/transform/stouffer.hpp:57-82):
 *   out = ((x - mean_i) * (|sd_i| < eps ? 0 : 1/sd_i) + (|sd_j| < eps ? 0 : (x - mean_j) / sd_j)) * sqrt(1/2)
 * or clr_vector_kernel (include/mcp/transform/clr.hpp:52-73): sqrt(zi^2 + zj^2),
 * in float exactly as those kernels.  The statistics come, in the reference,
 * from splash::kernel::GaussianParamsExclude1<T,T,true>, which is not in the
 * reference snapshot; here they are the FP64 mean and unbiased (N-1) standard
 * deviation of the row, rounded to float, over every entry
 * (MCPG_ROWSTATS_ALL) or every entry but the diagonal
 * (MCPG_ROWSTATS_EXCLUDE_DIAGONAL) -- the statistics' parity is unpinned.
 * A: n x n.  mcpg_row_stats_dev: rows x cols, mean / sd device float arrays. */
#define MCPG_TRANSFORM_STOUFFER 0
#define MCPG_TRANSFORM_CLR 1
#define MCPG_ROWSTATS_ALL 0
#define MCPG_ROWSTATS_EXCLUDE_DIAGONAL 1
MCPG_API int mcpg_row_stats_dev(mcpg_handle* h, const float* A, int64_t rows, int64_t cols, int64_t lda,
                                int stats_mode, float* mean, float* sd);
MCPG_API int mcpg_transform(mcpg_handle* h, const float* A, int64_t n, int64_t lda, int transform, int stats_mode,
                            float* out, int64_t ldo);
MCPG_API int mcpg_transform_dev(mcpg_handle* h, const float* A, int64_t n, int64_t lda, int transform,
                                int stats_mode, float* out, int64_t ldo);
/* compute_stouffer_tf (mcpnet_helper.hpp:589-634) of a rows x cols (TFs x
 * genes) matrix: z-scores of every row across its cols entries and of every
 * column across its rows entries (splash::kernel::StandardScore<T,T,false>,
 * absent from the reference snapshot: here FP64 two-pass mean and population
 * standard deviation rounded to float, z = |sd| < FLT_EPSILON ? 0 :
 * (x - mean) / sd in float), combined per entry by zscored_stouffer_kernel
 * (include/mcp/transform/stouffer.hpp:84-100): (z_row + z_col) * sqrt(1/2). */
MCPG_API int mcpg_stouffer_tf(mcpg_handle* h, const float* A, int64_t rows, int64_t cols, int64_t lda, float* out,
                              int64_t ldo);
MCPG_API int mcpg_stouffer_tf_dev(mcpg_handle* h, const float* A, int64_t rows, int64_t cols, int64_t lda,
                                  float* out, int64_t ldo);
/* The TF transform of the transform app (apps/transform/transform.cpp:156-209):
 * the same z-scores combined by zscored_stouffer_kernel (MCPG_TRANSFORM_STOUFFER,
 * = mcpg_stouffer_tf) or zscored_clr_kernel (MCPG_TRANSFORM_CLR,
 * include/mcp/transform/clr.hpp:75-88: sqrt(z_row^2 + z_col^2)). */
MCPG_API int mcpg_transform_tf(mcpg_handle* h, const float* A, int64_t rows, int64_t cols, int64_t lda, int transform,
                               float* out, int64_t ldo);
MCPG_API int mcpg_transform_tf_dev(mcpg_handle* h, const float* A, int64_t rows, int64_t cols, int64_t lda,
                                   int transform, float* out, int64_t ldo);
/* The statistics mcpg_stouffer_tf_dev uses, into device float arrays: row_mean /
 * row_sd (rows entries) and col_mean / col_sd (cols entries). */
MCPG_API int mcpg_stouffer_tf_stats_dev(mcpg_handle* h, const float* A, int64_t rows, int64_t cols, int64_t lda,
                                        float* row_mean, float* row_sd, float* col_mean, float* col_sd);

/* ---- gold-standard evaluation: AUPR and AUROC ----
 * mcpg_aupr_auroc: aupr_kernel::operator()(pos, pos_count, neg, neg_count)
 * (include/mcp/transform/aupr.hpp:565-584 -> average_compute_1sort, 127-236)
 * and auroc_kernel::operator() of the same arguments (auroc.hpp:562-579 ->
 * average_compute_1sort, 151-252):
 *   AUPR  = sum over the distinct positive scores t of
 *           TP(>=t) / (TP(>=t) + FP(>=t)) * #pos(==t) / n_pos     (0 if n_pos == 0)
 *   AUROC = n_pos < n_neg ? 1 - sum over distinct positive t of #neg(>=t)/n_neg * #pos(==t)/n_pos
 *                         :     sum over distinct negative t of #pos(>=t)/n_pos * #neg(==t)/n_neg
 *           (an empty sorted side gives a sum of 0, as the reference).
 * Every term is rounded as the reference rounds it; the terms are summed by a
 * deterministic compensated reduction rather than the reference's left-to-right
 * loop, so results agree with it to the rounding of a double sum (a few ulps).
 * NaN scores return MCPG_ERR_ARG.  aupr / auroc: host doubles (either nullable).
 * The _dev form takes device score vectors. */
MCPG_API int mcpg_aupr_auroc(mcpg_handle* h, const float* pos, int64_t n_pos, const float* neg, int64_t n_neg,
                             double* aupr, double* auroc);
MCPG_API int mcpg_aupr_auroc_dev(mcpg_handle* h, const float* pos, int64_t n_pos, const float* neg, int64_t n_neg,
                                 double* aupr, double* auroc);

/* Truth regions of a rows x cols score matrix and its int8 label matrix
 * (1 = positive, 0 = negative, anything else unknown, as the reference's
 * aligned_matrix<char> truth):
 *   MCPG_TRUTH_LOWER  entries (i, j) with j < i     select_lower_triangle, mcpnet_helper.hpp:862-891
 *   MCPG_TRUTH_ALL    every entry                   (aupr_kernel::compute_full_mat, aupr.hpp:356-387)
 *   MCPG_TRUTH_TF     rows are TFs: row i is gene row_gene[i]; (i, j) is kept unless
 *                     j == row_gene[i], or row_gene[i] > j and col_tf[j] != 0
 *                     (select_tfs_from_mat, mcpnet_helper.hpp:893-940)
 * row_gene (int32 per row) and col_tf (uint8 per column) are used by
 * MCPG_TRUTH_TF only (null otherwise). */
#define MCPG_TRUTH_LOWER 0
#define MCPG_TRUTH_ALL 1
#define MCPG_TRUTH_TF 2

/* compute_aupr_auroc (apps/pipeline/mcpnet_helper.hpp:1050-1071): selects the
 * labelled entries of the region (select_values2, mcpnet_helper.hpp:947-998)
 * and returns their AUPR / AUROC as mcpg_aupr_auroc, without materialising the
 * negative scores.  n_pos / n_neg (nullable) get the selected counts.  The
 * host form takes host values / labels / row_gene / col_tf; the _dev form,
 * device ones. */
MCPG_API int mcpg_eval_truth(mcpg_handle* h, const float* values, int64_t rows, int64_t cols, int64_t ldv,
                             const int8_t* labels, int64_t ldl, int region, const int32_t* row_gene,
                             const uint8_t* col_tf, double* aupr, double* auroc, int64_t* n_pos, int64_t* n_neg);
MCPG_API int mcpg_eval_truth_dev(mcpg_handle* h, const float* values, int64_t rows, int64_t cols, int64_t ldv,
                                 const int8_t* labels, int64_t ldl, int region, const int32_t* row_gene,
                                 const uint8_t* col_tf, double* aupr, double* auroc, int64_t* n_pos,
                                 int64_t* n_neg);

/* select_values2 (mcpnet_helper.hpp:947-998) over the region: the positive and
 * negative scores in row-major order into device arrays pos / neg of
 * capacities pos_cap / neg_cap (either nullable with capacity 0 to count only).
 * n_pos / n_neg get the counts; MCPG_ERR_ARG if a capacity is too small (the
 * counts are still set). */
MCPG_API int mcpg_select_truth_dev(mcpg_handle* h, const float* values, int64_t rows, int64_t cols, int64_t ldv,
                                   const int8_t* labels, int64_t ldl, int region, const int32_t* row_gene,
                                   const uint8_t* col_tf, float* pos, int64_t pos_cap, float* neg, int64_t neg_cap,
                                   int64_t* n_pos, int64_t* n_neg);

/* Ensemble coefficient search (apps/pipeline/mcpnet.cpp:575-616): for every
 * row c of coeffs (n_coeffs x 4 host doubles) the AUPR / AUROC of
 * compute_combo(mi, M1, M2, M3, c) (mcpg_combo_dev) over the labelled entries
 * of the region.  The combo values are formed only at the labelled entries
 * (bit-identical to the full matrix's).  Rows equal to (1, 0, 0, 0) are
 * skipped as the reference does (NaN in aupr / auroc).  aupr / auroc: host
 * arrays of n_coeffs (nullable); best (nullable) gets the reference's choice:
 * the first row whose AUPR exceeds every earlier one and 0, else 0.  Mk may be
 * null when column k of every row is 0. */
MCPG_API int mcpg_combo_eval_dev(mcpg_handle* h, const float* mi, int64_t ldm, const float* M1, int64_t ld1,
                                 const float* M2, int64_t ld2, const float* M3, int64_t ld3, int64_t rows,
                                 int64_t cols, const int8_t* labels, int64_t ldl, int region, const int32_t* row_gene,
                                 const uint8_t* col_tf, const double* coeffs, int64_t n_coeffs, double* aupr,
                                 double* auroc, int64_t* best);
/* The Stouffer half of the same loop (mcpnet.cpp:622-661): for every row c the
 * AUPR / AUROC of the Stouffer transform (mcpg_transform_dev, stats_mode) of
 * the full combo matrix over the labelled entries, and the row chosen by the
 * same rule.  Needs two n x n float scratch matrices; rows == cols. */
MCPG_API int mcpg_combo_stouffer_eval_dev(mcpg_handle* h, const float* mi, int64_t ldm, const float* M1,
                                          int64_t ld1, const float* M2, int64_t ld2, const float* M3, int64_t ld3,
                                          int64_t n, const int8_t* labels, int64_t ldl, int region,
                                          const int32_t* row_gene, const uint8_t* col_tf, const double* coeffs,
                                          int64_t n_coeffs, int stats_mode, double* aupr, double* auroc,
                                          int64_t* best);
MCPG_API int mcpg_combo_stouffer_eval(mcpg_handle* h, const float* mi, int64_t ldm, const float* M1, int64_t ld1,
                                      const float* M2, int64_t ld2, const float* M3, int64_t ld3, int64_t n,
                                      const int8_t* labels, int64_t ldl, int region, const int32_t* row_gene,
                                      const uint8_t* col_tf, const double* coeffs, int64_t n_coeffs, int stats_mode,
                                      double* aupr, double* auroc, int64_t* best);
/* The Stouffer half of the TF loop (mcpnet.cpp:622-626 with --tf-input): as
 * mcpg_combo_stouffer_eval_dev with the TF transform (mcpg_stouffer_tf_dev) of
 * each rows x cols (TFs x genes) combo matrix; region is normally
 * MCPG_TRUTH_TF (select_tfs_from_mat) or MCPG_TRUTH_ALL (select_from_list). */
MCPG_API int mcpg_combo_stouffer_tf_eval_dev(mcpg_handle* h, const float* mi, int64_t ldm, const float* M1,
                                             int64_t ld1, const float* M2, int64_t ld2, const float* M3,
                                             int64_t ld3, int64_t rows, int64_t cols, const int8_t* labels,
                                             int64_t ldl, int region, const int32_t* row_gene, const uint8_t* col_tf,
                                             const double* coeffs, int64_t n_coeffs, double* aupr, double* auroc,
                                             int64_t* best);
MCPG_API int mcpg_combo_stouffer_tf_eval(mcpg_handle* h, const float* mi, int64_t ldm, const float* M1, int64_t ld1,
                                         const float* M2, int64_t ld2, const float* M3, int64_t ld3, int64_t rows,
                                         int64_t cols, const int8_t* labels, int64_t ldl, int region,
                                         const int32_t* row_gene, const uint8_t* col_tf, const double* coeffs,
                                         int64_t n_coeffs, double* aupr, double* auroc, int64_t* best);
/* ---- semi-supervised split evaluation (the eval_mcpnet app) ----
 * The labelled entries of the region in the reference's mask order (row-major:
 * select_lower_triangle, select_from_list's sorted mask, select_tfs_from_mat) are
 * shuffled for iteration i = 1..iterations by std::shuffle with a std::mt19937
 * seeded with i (shuffle_truth, apps/pipeline/eval_mcpnet.cpp:214-224); a part j
 * trains on the first train_counts[j] shuffled entries and tests on the rest
 * (the app uses counts (size_t)(f * entries) for f = 0.005, 0.01, 0.02, 0.05,
 * 0.1, and also 0.2 .. 0.5 with TFs).  All AUPRs are aupr_kernel's
 * (compute_aupr2, mcpnet_helper.hpp:1017-1035).  Fewer than 2^32 entries.
 *
 * mcpg_shuffle_positions: iteration `seed`'s shuffled order as mask positions, out[k] =
 * the position of the k-th shuffled entry among `entries` (seed 0: the mask order).
 * Host only (no handle); MCPG_ERR_ARG for a negative count, 2^32 or more, or a null out.
 *
 * mcpg_split_aupr: eval_aupr_mcp (eval_mcpnet.cpp:227-301) of one score matrix:
 * full_aupr (nullable) over all entries; train_aupr / test_aupr (nullable,
 * iterations x parts, row-major). */
MCPG_API int mcpg_shuffle_positions(uint32_t* out, int64_t entries, uint64_t seed);
MCPG_API int mcpg_split_aupr(mcpg_handle* h, const float* values, int64_t rows, int64_t cols, int64_t ldv,
                             const int8_t* labels, int64_t ldl, int region, const int32_t* row_gene,
                             const uint8_t* col_tf, int64_t iterations, const int64_t* train_counts, int64_t parts,
                             double* full_aupr, double* train_aupr, double* test_aupr);
MCPG_API int mcpg_split_aupr_dev(mcpg_handle* h, const float* values, int64_t rows, int64_t cols, int64_t ldv,
                                 const int8_t* labels, int64_t ldl, int region, const int32_t* row_gene,
                                 const uint8_t* col_tf, int64_t iterations, const int64_t* train_counts,
                                 int64_t parts, double* full_aupr, double* train_aupr, double* test_aupr);
/* mcpg_split_combo_eval: eval_combos over the splits (eval_mcpnet.cpp:319-462,
 * 814-893, the app's default --permute-combo): per iteration and part the
 * coefficient row of highest training AUPR (the first strictly larger; row 0
 * when none is; rows (1, 0, 0, 0) skipped), its test AUPR and its AUPR over all
 * entries, and the same for the Stouffer-transformed combos.  stouffer:
 * MCPG_STOUFFER_NONE, a MCPG_ROWSTATS_* mode (square matrices, as
 * mcpg_transform) or MCPG_STOUFFER_TF (as mcpg_stouffer_tf).  results:
 * iterations x parts x 6 host doubles -- train, test, Stouffer train, Stouffer
 * test, full, Stouffer full (the Stouffer ones 0 without it); best (nullable):
 * iterations x parts x 2 chosen rows.  Keeps n_coeffs x entries floats of
 * Stouffer scores in device scratch. */
#define MCPG_STOUFFER_NONE (-1)
#define MCPG_STOUFFER_TF 2
MCPG_API int mcpg_split_combo_eval(mcpg_handle* h, const float* mi, int64_t ldm, const float* M1, int64_t ld1,
                                   const float* M2, int64_t ld2, const float* M3, int64_t ld3, int64_t rows,
                                   int64_t cols, const int8_t* labels, int64_t ldl, int region,
                                   const int32_t* row_gene, const uint8_t* col_tf, const double* coeffs,
                                   int64_t n_coeffs, int stouffer, int64_t iterations, const int64_t* train_counts,
                                   int64_t parts, double* results, int64_t* best);
MCPG_API int mcpg_split_combo_eval_dev(mcpg_handle* h, const float* mi, int64_t ldm, const float* M1, int64_t ld1,
                                       const float* M2, int64_t ld2, const float* M3, int64_t ld3, int64_t rows,
                                       int64_t cols, const int8_t* labels, int64_t ldl, int region,
                                       const int32_t* row_gene, const uint8_t* col_tf, const double* coeffs,
                                       int64_t n_coeffs, int stouffer, int64_t iterations,
                                       const int64_t* train_counts, int64_t parts, double* results, int64_t* best);
/* Host-buffer form of mcpg_combo_eval_dev (matrices, labels, row_gene and col_tf on the host). */
MCPG_API int mcpg_combo_eval(mcpg_handle* h, const float* mi, int64_t ldm, const float* M1, int64_t ld1,
                             const float* M2, int64_t ld2, const float* M3, int64_t ld3, int64_t rows, int64_t cols,
                             const int8_t* labels, int64_t ldl, int region, const int32_t* row_gene,
                             const uint8_t* col_tf, const double* coeffs, int64_t n_coeffs, double* aupr,
                             double* auroc, int64_t* best);

/* ---- B-spline MI without any device allocation (no counterpart in the reference) ----
 * For callers that cannot call cudaMalloc -- an application whose device
 * memory belongs entirely to its own pool allocator, or a latency-critical
 * loop that cannot take cudaMalloc's implicit synchronisation.  Same result as
 * mcpg_bspline_mi_dev(..., MCPG_MI_FP32, ...) with device pointers, enqueued on
 * `cuda_stream` (0 = legacy default stream), no handle.  Its FP32 weight table
 * lives in a file-scope device array of 32 MiB that every GPU loading this
 * library holds until exit; problems whose table (ceil(m/16)*16 x
 * ceil(n/16)*16*bins floats, plus n doubles when H is null) does not fit return
 * MCPG_ERR_SCRATCH_LIMIT.  The first call on a device looks up the array's
 * address with that device current: make it before any stream capture.  The
 * address is kept per device and CUDA context, so after cudaDeviceReset the next
 * call looks it up again (make that call, too, before any stream capture).  All
 * calls share the array and it keeps the last call's contents (the call clears
 * the padding it needs); calls that overlap on the GPU race on it.
 * 2 <= bins <= 12 (else MCPG_ERR_ARG, before any device work). */
MCPG_API int mcpg_bspline_mi_fp32_noalloc(const float* X, int64_t n, int64_t m, int64_t ldx, int bins, int order,
                                          float* MI, int64_t ldmi, double* H, void* cuda_stream);

/* ---- host buffers addressed in place (no counterpart in the reference) ----
 * On a device that accesses pageable host memory coherently through the host's
 * page tables (GB300 / Grace over NVLink-C2C), the host entry points let their
 * kernels use the caller's host buffers directly -- no staging copies -- when
 * every page of the buffer is mapped and resident: every output that is written
 * once (MI, max-min products other than an M1 that later products read again,
 * ratios, DPI outputs and masks, the closure, combos, transforms) and every
 * input that is read once (X of the MI entry points, the combo and ratio
 * operands).  An output buffer whose pages are not populated yet is populated by
 * the host first (its contents, padding included, are left as they are).
 * Other buffers, and other devices, take the staged path (copies through device
 * scratch).  Results are identical either way.  MCPG_HOST_ACCESS_STAGED forces
 * the staged path on this handle; mcpg_last_host_access returns which kinds of
 * buffer the last call used in place (MCPG_HOST_DIRECT_* bits). */
#define MCPG_HOST_ACCESS_AUTO 0
#define MCPG_HOST_ACCESS_STAGED 1
#define MCPG_HOST_DIRECT_INPUT 1
#define MCPG_HOST_DIRECT_OUTPUT 2
MCPG_API int mcpg_set_host_access(mcpg_handle* h, int mode);
MCPG_API int mcpg_last_host_access(const mcpg_handle* h);

/* ---- testing hook: make the next `count` device scratch allocations of this
 * handle fail with MCPG_ERR_OOM (exercises the error path without a GPU fault). */
MCPG_API int mcpg_test_fail_allocs(mcpg_handle* h, int count);

/* ---- testing hook: the next tensor-core MI launch of this handle (precision
 * BF16 / FP16 / BF16X3 / FP16X3 / BF16F8) gives every barrier wait a limit of
 * wait_ns nanoseconds (1e3..2e9; the default limit is 2 s), and with starve != 0
 * its TMA producers issue no loads, so the MMA issuer's first wait runs out with
 * no load or MMA outstanding.  The kernel then raises its timeout flag, frees its
 * tensor memory and returns; the call returns MCPG_ERR_DEVICE_TIMEOUT and the
 * handle stays usable.  Exercises the bounded-wait path without a GPU fault. */
MCPG_API int mcpg_test_tc_timeout(mcpg_handle* h, int64_t wait_ns, int starve);

#ifdef __cplusplus
}
#endif

#endif /* MCPGPU_H */
