// Internal launcher interface between the C ABI (api.cpp) and the kernels.
// Every launcher enqueues work on `stream`, returns the launch status and adds
// the number of kernels it launched to *launches.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace mcpg {

// ---------------- max-min family (maxmin.cu) ----------------
enum MaxminMode : int {
    MM_PLAIN = 0,    // C = A (x) B
    MM_RATIO = 1,    // R = ratio(E, A (x) B); C (nullable) = A (x) B
    MM_CLOSURE = 2,  // C = max(E, A (x) B); *changed |= any entry grew
    MM_DPI = 3,      // C = dpi-mask(E) applied to E; k excluded when k == i or k == j
    MM_EXCL = 4,     // C = max over admissible k of min(A[i][k], B[j][k]); k excluded as in
                     // MM_DPI; an output with no admissible k is NaN
    MM_WITNESS = 5,  // C = A (x) B and K[i][j] = first k attaining it (-1 where C is -inf)
    MM_GEMM = 6,     // C = A B^T in (+, x): the plus-times twin of the kernel (FP32 FFMA)
    MM_DPI1 = 7,     // first phase of the two-phase DPI: k runs over [0, k_len) only; outputs it
                     // decides are written (as MM_DPI), the others appended to `pending`
};

// An output pair of the two-phase DPI that the first k_len intermediates did not
// decide: (x, z) and, when `flags` bit 1 is set, its mirror (z, x), with m the
// max-min over the first phase's admissible intermediates.  flags bit 0: (x, z)
// undecided; bit 1: (z, x) undecided.
struct DpiPending {
    int32_t x, z;
    float m;
    uint32_t flags;
};

struct MaxminParams {
    const float* A; int64_t lda;  // rows x k_len, 16-byte aligned rows
    const float* B; int64_t ldb;  // cols x k_len, 16-byte aligned rows
    int64_t rows, cols, k_len;
    float* C; int64_t ldc;        // product / closure / DPI output (nullable in RATIO mode)
    const float* E; int64_t lde;  // RATIO numerator, CLOSURE current iterate, DPI input
    float* R; int64_t ldr;        // RATIO output
    int* changed;                 // CLOSURE flag (device)
    double tol_mult;              // DPI 1/(1 - tol)
    // DPI threshold in float arithmetic when tm_float != 0: e * tol_mult_f rounded once
    // (dpi_tf_kernel keeps its multiplier in the value type)
    float tol_mult_f; int tm_float;
    uint8_t* mask; int64_t ldmask;  // DPI mask (nullable)
    unsigned long long* removed;  // DPI removed count (device, nullable)
    // MM_DPI / MM_EXCL: the excluded k of output (i, j) are excl_row[i] and
    // excl_col[j] (device, -1 = none) when given, else i and j.
    const int* excl_row;
    const int* excl_col;
    int32_t* K; int64_t ldk;      // MM_WITNESS output
    // MM_DPI1: pending outputs (capacity pending_cap; *pending_n counts every append,
    // so a count above the capacity means the list overflowed)
    DpiPending* pending; int64_t pending_cap; unsigned long long* pending_n;
    // MM_DPI / MM_DPI1 on a permuted input P A P^T: output (i, j) goes to
    // C / mask [perm[i]][perm[j]] (device, nullable = identity)
    const int* perm;
};

// symmetric != 0: A == B (same rows), rows == cols; only tiles on or above the
// diagonal are computed and mirrored (C is symmetric for any A in that case).
cudaError_t launch_maxmin(const MaxminParams& p, int mode, int symmetric, cudaStream_t stream, int64_t* launches);
cudaError_t launch_ratio(const float* A, int64_t lda, const float* M, int64_t ldm, int64_t rows, int64_t cols,
                         float* R, int64_t ldr, cudaStream_t stream, int64_t* launches);
// Second phase of the two-phase DPI: for every pending pair, continue the max-min over
// the intermediates y in [k0, n) (y not in {x, z}) until every undecided orientation is
// deleted or the row ends, then write out / mask and add to *removed as MM_DPI does.
// A: n x n (16-byte aligned rows, lda % 4 == 0), also the DPI input E.
// TF form (dpi_tf_kernel on the permuted input P A P^T, TFs first): tsplit >= 0 is the
// TF count t; a pair with exactly one TF scans only y < t.  perm (nullable) maps the
// permuted indices back for out / mask; tm_float selects the float threshold.
struct DpiPendingTf {
    int64_t tsplit = -1;
    const int* perm = nullptr;
    float tol_mult_f = 0.0f;
    int tm_float = 0;
};
cudaError_t launch_dpi_pending(const float* A, int64_t lda, int64_t n, int64_t k0, const DpiPending* list,
                               int64_t count, double tol_mult, float* out, int64_t ldo, uint8_t* mask,
                               int64_t ldmask, unsigned long long* removed, cudaStream_t stream, int64_t* launches,
                               const DpiPendingTf& tf = DpiPendingTf());
cudaError_t launch_set_diagonal(float* A, int64_t rows, int64_t cols, int64_t lda, float value,
                                cudaStream_t stream, int64_t* launches);
cudaError_t launch_max_transpose(const float* M, int64_t n, int64_t ldm, float* out, int64_t ldo,
                                 cudaStream_t stream, int64_t* launches);
// dst[r][c] = src[rows_idx ? rows_idx[r] : r][cols_idx ? cols_idx[c] : c]  (device index arrays)
cudaError_t launch_gather(const float* src, int64_t lds, const int* rows_idx, const int* cols_idx, int64_t rows,
                          int64_t cols, float* dst, int64_t ldd, cudaStream_t stream, int64_t* launches);
// dst[r][c] = min(src[r][c], mask[c])  (mask: device, cols floats)
cudaError_t launch_fold_mask(const float* src, int64_t lds, const float* mask, int64_t rows, int64_t cols, float* dst,
                             int64_t ldd, cudaStream_t stream, int64_t* launches);
// dpi_tf_kernel decision (dpi.hpp:74-110) + mask<float,true>: per (x, z) pick the
// all-y value Call or the TF-y value Ctf by tf[x] xor tf[z].
cudaError_t launch_dpi_tf_apply(const float* A, int64_t lda, const float* Call, int64_t ld1, const float* Ctf,
                                int64_t ld2, const uint8_t* tf, int64_t n, float tol_mult, float* out, int64_t ldo,
                                uint8_t* mask, unsigned long long* removed, cudaStream_t stream, int64_t* launches);
// Adjoint of C = A (x) B: for every (i, j) with dC != 0 route dC to A[i][k*]
// (if A[i][k*] <= B[j][k*]) or B[j][k*], k* = K[i][j] when K is given, else the
// first k with min(A[i][k], B[j][k]) == C[i][j].  Accumulates with atomics.
cudaError_t launch_maxmin_route(const float* A, int64_t lda, const float* B, int64_t ldb, int64_t rows, int64_t cols,
                                int64_t k, const float* C, int64_t ldc, const float* dC, int64_t lddc,
                                const int32_t* K, int64_t ldk, float* dA, int64_t ldda, float* dB, int64_t lddb,
                                cudaStream_t stream, int64_t* launches);
// Adjoint of ratio_kernel: dA += dR / M, dM -= dR A / M^2 where |A|, |M| >= FLT_EPSILON.
cudaError_t launch_ratio_bwd(const float* A, int64_t lda, const float* M, int64_t ldm, int64_t rows, int64_t cols,
                             const float* dR, int64_t lddr, float* dA, int64_t ldda, float* dM, int64_t lddm,
                             cudaStream_t stream, int64_t* launches);
// compute_combo: out = mi / (cs0 mi + cs1 M1 + cs2 M2 + cs3 M3) in double with the
// ratio's epsilon guards; Mk may be null when csk == 0 (cs: host, 4 values).
cudaError_t launch_combo(const float* mi, int64_t ldm, const float* M1, int64_t ld1, const float* M2, int64_t ld2,
                         const float* M3, int64_t ld3, int64_t rows, int64_t cols, const double* cs, float* out,
                         int64_t ldo, cudaStream_t stream, int64_t* launches);
// Copies a rows x cols matrix between arbitrary leading dimensions (device to device).
cudaError_t launch_copy2d(const float* src, int64_t lds, float* dst, int64_t ldd, int64_t rows, int64_t cols,
                          cudaStream_t stream);

// ---------------- B-spline weights and MI (bspline.cu, mi_fp32.cu, mi_tc.cu) ----------------
// Sample-major FP32 weights for the CUDA-core contraction:
//   Wt[s * ldwt + g * bins + a] = B_a(scaled x_g[s]),  s < m, g < n  (ldwt >= n*bins)
// H[g] (double) = marginal entropy in bits.
cudaError_t launch_bspline_weights_fp32(const float* X, int64_t n, int64_t m, int64_t ldx, int bins, int order,
                                        float* Wt, int64_t ldwt, double* H, cudaStream_t stream, int64_t* launches);
// Gene-bin-major 16-bit weights for tcgen05 (K = samples contiguous):
//   Whi[(g*bins + a) * ldw + s] = round16(w), Wlo[...] = round16(w - Whi) (Wlo nullable)
// fmt: 0 = bf16, 1 = fp16.  Columns s in [m, ldw) are written as zero.
cudaError_t launch_bspline_weights_16(const float* X, int64_t n, int64_t m, int64_t ldx, int bins, int order,
                                      int fmt, uint16_t* Whi, uint16_t* Wlo, int64_t ldw, double* H,
                                      cudaStream_t stream, int64_t* launches);
// The FP8-corrected form: Whi = bf16(w) * 2^8 in the layout above, and the E4M3 planes
// H8 = e4m3(bf16(w) * 2^4), L8 = e4m3((w - bf16(w)) * 2^12) (every product scaled 2^16)
// interleaved in HL8: rows of 2 * ldw bytes, each 64 samples as 64 H8 bytes then 64 L8 bytes.
cudaError_t launch_bspline_weights_f8(const float* X, int64_t n, int64_t m, int64_t ldx, int bins, int order,
                                      uint16_t* Whi, uint8_t* HL8, int64_t ldw, double* H, cudaStream_t stream,
                                      int64_t* launches);
// FP32 MI from sample-major weights (CUDA cores), symmetric output.
// Covers gene pairs (i, j >= i) with i in [gene0, gene1) (gene0 a multiple of 16;
// gene1 = -1 for n): rows i < gene1 of MI are complete once every earlier range ran.
cudaError_t launch_mi_fp32(const float* Wt, int64_t ldwt, const double* H, int64_t n, int64_t m, int bins,
                           float* MI, int64_t ldmi, cudaStream_t stream, int64_t* launches, int64_t gene0 = 0,
                           int64_t gene1 = -1);
// MI adjoint, slab of gene tiles [tile0, tile0 + tiles) (16 genes each) x all genes:
// Q[(i - 16*tile0)*bins + a][j*bins + b] = Gs_ij (log2 P_ab + 1/ln 2) [P_ab > 0],
// Gs_ij = G[i][j] + G[j][i] (i != j), recomputing P from the sample-major weights.
cudaError_t launch_mi_q(const float* Wt, int64_t ldwt, const float* G, int64_t ldg, int64_t n, int64_t m, int bins,
                        int64_t tile0, int64_t tiles, float* Q, int64_t ldq, cudaStream_t stream, int64_t* launches);
// gsum[i] = sum_{j != i} (G[i][j] + G[j][i])
cudaError_t launch_pair_sums(const float* G, int64_t ldg, int64_t n, float* gsum, cudaStream_t stream,
                             int64_t* launches);
// dL/dX for genes [g0, g1) from dWq[(g - g0)*bins + a][s] (= sum_j,b Q w_jb(s)), gsum,
// through the weights (B-spline derivative), the min-max scaling and its min / max.
cudaError_t launch_mi_bwd_x(const float* X, int64_t n, int64_t m, int64_t ldx, int bins, int order, int64_t g0,
                            int64_t g1, const float* gsum, const float* dWq, int64_t lddw, float* dX, int64_t lddx,
                            cudaStream_t stream, int64_t* launches);
// Tensor-core MI (tcgen05).  mode TC_SINGLE: 16-bit weights Whi; TC_SPLIT16: adds
// the 16-bit lo terms from Wlo; TC_F8C: BF16 Whi (x 2^8) plus the interleaved E4M3
// correction plane HL8 (launch_bspline_weights_f8).
// Returns cudaErrorNotSupported when the shape/bins is outside the kernel's tiling.
// Gene range as launch_mi_fp32 (gene0 a multiple of 12).
enum TcMode : int { TC_SINGLE = 0, TC_SPLIT16 = 1, TC_F8C = 2 };
// Limit of every mbarrier wait of the tensor-core MI kernels (the kernel gives up,
// raises *timeout_flag, drains, frees its tensor memory and returns).
constexpr unsigned long long TC_WAIT_NS_DEFAULT = 2000000000ull;
// Test hook of one launch: wait_ns replaces the default limit; starve != 0 makes the
// TMA producers issue no load at all, so the MMA issuer's first wait runs out with
// no load or MMA outstanding (the timeout path, without a GPU fault).
struct TcWaitHook {
    unsigned long long wait_ns = TC_WAIT_NS_DEFAULT;
    int starve = 0;
};
// Row pitch (samples) of the tensor-core weight planes for m samples: a multiple of 64.
int64_t mi_tc_pitch(int64_t m);
cudaError_t launch_mi_tc(const uint16_t* Whi, const uint16_t* Wlo, const uint8_t* HL8, int64_t ldw, const double* H, int64_t n, int64_t m, int bins, int fmt, int mode, float* MI,
                         int64_t ldmi, int* timeout_flag, cudaStream_t stream, int64_t* launches, int64_t gene0 = 0,
                         int64_t gene1 = -1, const TcWaitHook* hook = nullptr, void* work = nullptr);
// Bytes of the work area launch_mi_tc's 2-SM form takes for n genes (its tile
// counters); without it the 1-SM form runs.
int64_t mi_tc_work_bytes(int64_t n, int bins);

// ---------------- gold-standard evaluation (eval.cu) ----------------
enum TruthMode : int {
    TRUTH_LOWER = 0,  // entries (i, j), j < i          select_lower_triangle
    TRUTH_ALL = 1,    // every entry
    TRUTH_TF = 2,     // TF rows: j != g(i), and not (g(i) > j and j is a TF)   select_tfs_from_mat
};
struct TruthRegion {
    const int8_t* labels; int64_t ldl;   // 1 = positive, 0 = negative, anything else unknown
    int64_t rows, cols;
    int mode;
    const int32_t* row_gene;             // TRUTH_TF: global gene index of each row (device)
    const uint8_t* col_tf;               // TRUTH_TF: non-zero where the column gene is a TF (device)
};
struct GatherSrc {                       // up to four matrices gathered at the selected entries
    int n;
    const float* src[4]; int64_t lds[4];
    float* dst[4];
    int8_t* lab_dst;                     // nullable: the entries' labels (for lab < 0)
};
// compute_combo coefficients prepared once per launch: kind 0 = skipped (0),
// 1 = added as is (1), 2 = scaled; hi + lo = the double coefficient to 2^-48.
struct ComboCoef {
    double c[4];
    float hi[4], lo[4];
    int kind[4];
};
inline ComboCoef make_combo_coef(const double* cs) {
    ComboCoef k;
    for (int i = 0; i < 4; ++i) {
        k.c[i] = cs[i];
        k.kind[i] = cs[i] == 0.0 ? 0 : (cs[i] == 1.0 ? 1 : 2);
        k.hi[i] = (float)cs[i];
        k.lo[i] = (float)(cs[i] - (double)k.hi[i]);
    }
    return k;
}
struct ComboSrc {                        // gathered (mi, M1, M2, M3) and the combo coefficients
    const float* g[4];
    int64_t n;
    double cs[4];
    ComboCoef kc;                        // make_combo_coef(cs)
};
// Work items of a region: rows x ceil(cols / 4096) row segments.
int64_t truth_items(const TruthRegion& r);
// Scratch sizes (elements): scan partials for n inputs; radix-sort blocks of n keys;
// curve partials.
int64_t scan_tmp_elems(int64_t n);
int64_t radix_blocks(int64_t n);
int64_t curve_part_elems();
// Per-item counts of positive and negative labels inside the region.
cudaError_t launch_truth_count(const TruthRegion& r, uint32_t* cpos, uint32_t* cneg, cudaStream_t stream,
                               int64_t* launches);
// out[0..n) = exclusive prefix sum of in, out[n] = total (tmp: scan_tmp_elems(n)).
cudaError_t launch_scan_u32(const uint32_t* in, int64_t n, uint64_t* out, uint64_t* tmp, cudaStream_t stream,
                            int64_t* launches);
// Writes, in row-major order, every selected entry labelled `lab` (lab < 0: every
// entry labelled 0 or 1, with its label to g.lab_dst when given) of the g.n
// sources to g.dst at positions off[item] + rank (off: scanned per-item counts).
cudaError_t launch_truth_gather(const TruthRegion& r, int lab, const uint64_t* off, const GatherSrc& g, int* nan_flag,
                                cudaStream_t stream, int64_t* launches);
// out[i] = a[i] + b[i].
cudaError_t launch_add_u32(const uint32_t* a, const uint32_t* b, int64_t n, uint32_t* out, cudaStream_t stream,
                           int64_t* launches);
// Entries perm[a..b) of mask-order entry arrays: the score (vals[e], or with
// combo the compute_combo value of c at e) as an order key into kp (label 1) or
// kn (label 0), compacted in no particular order; cnt[0] / cnt[1] (zeroed by the
// caller) count them.  NaN sets *nan_flag.
cudaError_t launch_split_keys(const uint32_t* perm, int64_t a, int64_t b, const float* vals, const ComboSrc& c,
                              int combo, const int8_t* lab, uint32_t* kp, uint32_t* kn, unsigned long long* cnt,
                              int* nan_flag, cudaStream_t stream, int64_t* launches);
// Order-preserving 32-bit keys of float scores (-0 as +0); NaN sets *nan_flag.
cudaError_t launch_keys_from_floats(const float* v, int64_t n, uint32_t* keys, int* nan_flag, cudaStream_t stream,
                                    int64_t* launches);
cudaError_t launch_combo_keys(const ComboSrc& c, uint32_t* keys, int* nan_flag, cudaStream_t stream,
                              int64_t* launches);
// Ascending LSD radix sort of keys in place (alt: n keys; bh: 256*radix_blocks(n);
// bh_off: 256*radix_blocks(n)+1; tmp: scan_tmp_elems(256*radix_blocks(n))).
cudaError_t launch_radix_sort(uint32_t* keys, uint32_t* alt, int64_t n, uint32_t* bh, uint64_t* bh_off,
                              uint64_t* tmp, cudaStream_t stream, int64_t* launches);
// lt[i] / eq[i] (nX + 1 each, zeroed here) = number of Y keys whose lower_bound
// in the sorted X is i and that are < X[i] / == X[i].  nX in [1, 2^31).
// dir: rank_dir_elems() scratch for the key-prefix directory of X (built here).
int64_t rank_dir_elems();
cudaError_t launch_rank_count_matrix(const uint32_t* X, int64_t nX, const TruthRegion& r, const float* v, int64_t ldv,
                                     int lab, uint64_t* lt, uint64_t* eq, uint32_t* dir, int* nan_flag,
                                     cudaStream_t stream, int64_t* launches);
cudaError_t launch_rank_count_keys(const uint32_t* X, int64_t nX, const uint32_t* Y, int64_t nY, uint64_t* lt,
                                   uint64_t* eq, uint32_t* dir, cudaStream_t stream, int64_t* launches);
cudaError_t launch_rank_count_combo(const uint32_t* X, int64_t nX, const ComboSrc& c, uint64_t* lt, uint64_t* eq,
                                    uint32_t* dir, int* nan_flag, cudaStream_t stream, int64_t* launches);
// out[0] = sum of AUPR terms (X = positives, Y = negatives), out[1] = sum of
// AUROC terms (#Y >= t / |Y|) (run / |X|) over the distinct thresholds t of X.
// work: 2*nX + 1; tmp: scan_tmp_elems(nX); part: curve_part_elems().
cudaError_t launch_curve(const uint32_t* X, int64_t nX, int64_t nY, const uint64_t* lt, const uint64_t* eq,
                         uint64_t* work, uint64_t* tmp, double* part, unsigned* ticket, double* out,
                         cudaStream_t stream, int64_t* launches);

// ---------------- adaptive-partitioning MI (apmi.cu) ----------------
int64_t ap_max_samples();
// Descending ranks of each gene's samples (ties share the lowest rank), after
// adding U[0, noise) to every value when noise > 0 (seeded, counter-based).
// *flag |= 1 on a NaN.
cudaError_t launch_ap_ranks(const float* X, int64_t n, int64_t m, int64_t ldx, float noise, uint64_t seed,
                            int32_t* R, int64_t ldr, int* flag, cudaStream_t stream, int64_t* launches);
// Ranks -> uint16 ranks (n x m), samples ordered by rank (n x m) and cumulative
// histograms (n x ldc, m + 1 used).  *flag |= 1 on a rank outside [0, m).
cudaError_t launch_ap_prep(const int32_t* R, int64_t n, int64_t m, int64_t ldr, uint16_t* xr, uint16_t* order,
                           uint16_t* cH, int64_t ldc, int* flag, cudaStream_t stream, int64_t* launches);
// Symmetric AP MI (float) from the prepared rank tables; next_i: device counter.
// *flag |= 2 if a pair's window walk broke its bounds (the entry is NaN).
cudaError_t launch_ap_mi(const uint16_t* xr, const uint16_t* order, const uint16_t* cH, int64_t ldc, int64_t n,
                         int64_t m, float* MI, int64_t ldmi, unsigned* next_i, int* flag, cudaStream_t stream,
                         int64_t* launches);

// ---------------- Stouffer / CLR (stouffer.cu) ----------------
// mean[i], sd[i] (float, from FP64 two-pass sums) of row i; excl_diag skips A[i][i];
// sd uses the (N - ddof) variance (ddof 1: unbiased, 0: population), 0 when N <= ddof.
cudaError_t launch_row_stats(const float* A, int64_t rows, int64_t cols, int64_t lda, int excl_diag, int ddof,
                             float* mean, float* sd, cudaStream_t stream, int64_t* launches);
// mean[j], sd[j] of column j over the rows (FP64 two-pass, population variance).
cudaError_t launch_col_stats(const float* A, int64_t rows, int64_t cols, int64_t lda, float* mean, float* sd,
                             cudaStream_t stream, int64_t* launches);
// out[i][j] = zscored_stouffer_kernel (clr = 0) or zscored_clr_kernel (clr = 1) of the
// row and column z-scores of A[i][j].
cudaError_t launch_stouffer_tf(const float* A, int64_t rows, int64_t cols, int64_t lda, const float* rmean,
                               const float* rsd, const float* cmean, const float* csd, int clr, float* out,
                               int64_t ldo, cudaStream_t stream, int64_t* launches);
// out[i][j] = stouffer_vector_kernel (clr = 0) or clr_vector_kernel (clr = 1) of A[i][j]
// with row i's and row j's statistics.
cudaError_t launch_transform(const float* A, int64_t n, int64_t lda, const float* mean, const float* sd, int clr,
                             float* out, int64_t ldo, cudaStream_t stream, int64_t* launches);

}  // namespace mcpg
