// Shared device helpers for the mcpgpu kernels (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "internal.h"

namespace mcpg {

// ---- 3-input FP32 max/min (PTX `max.f32 d, a, b, c`, sm_100+) ----
// Both ignore a NaN operand (the result is the max/min of the others), which
// the DPI kernel uses as the neutral element of an empty maximum.
__device__ __forceinline__ float fmax3(float a, float b, float c) {
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}
__device__ __forceinline__ float fmin2(float a, float b) {
    float r;
    asm("min.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ float fmax2(float a, float b) {
    float r;
    asm("max.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
    return r;
}

// ---- cp.async (16-byte, L2-only) with zero fill of the bytes beyond src_bytes ----
__device__ __forceinline__ void cp_async16(void* smem_dst, const void* gmem_src, int src_bytes) {
    uint32_t s = (uint32_t)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gmem_src), "r"(src_bytes));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

__host__ __device__ __forceinline__ int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

// ---- element-wise traversal of a rows x cols matrix ----
// Blocks of EW_TPB threads take (row, EW_SEG-column segment) items grid-stride;
// a thread handles its EW_SEG / EW_TPB columns of the segment (coalesced across
// the block) in one unrolled step, so that, with __restrict__ operands, their
// loads are in flight together.  One 64-bit division per segment instead of one
// per element.  Launch with ew_grid2d(rows, cols) blocks of EW_TPB threads.
constexpr int EW_SEG = 1024, EW_TPB = 256;
template <class F>
__device__ __forceinline__ void for_each_entry(int64_t rows, int64_t cols, F&& f) {
    const int64_t segs = (cols + EW_SEG - 1) / EW_SEG;
    const int64_t items = rows * segs;
    for (int64_t it = blockIdx.x; it < items; it += gridDim.x) {
        const int64_t i = it / segs;
        const int64_t c0 = (it - i * segs) * EW_SEG + threadIdx.x;
        const int64_t c1 = c0 + EW_SEG - threadIdx.x < cols ? c0 + EW_SEG - threadIdx.x : cols;
#pragma unroll
        for (int k = 0; k < EW_SEG / EW_TPB; ++k) {
            const int64_t j = c0 + k * EW_TPB;
            if (j < c1) f(i, j);
        }
    }
}
inline unsigned ew_grid2d(int64_t rows, int64_t cols) {
    int64_t items = rows * ceil_div(cols, EW_SEG);
    if (items > 152 * 16) items = 152 * 16;
    return (unsigned)(items < 1 ? 1 : items);
}

// One entry of compute_combo (apps/pipeline/mcpnet_helper.hpp:507-573): the
// denominator is summed in double in the reference's order, coefficient 1 adds
// the value itself and coefficient 0 skips the term; explicit _rn intrinsics
// keep nvcc from fusing the multiply-adds.  m1..m3 are only read when their
// coefficient is non-zero.
__device__ __forceinline__ float combo_value(float v, float m1, float m2, float m3, double a, double b, double c,
                                             double d) {
    double mm = 0.0;
    if (a == 1.0) mm = __dadd_rn(mm, (double)v); else if (a != 0.0) mm = __dadd_rn(mm, __dmul_rn(a, (double)v));
    if (b == 1.0) mm = __dadd_rn(mm, (double)m1); else if (b != 0.0) mm = __dadd_rn(mm, __dmul_rn(b, (double)m1));
    if (c == 1.0) mm = __dadd_rn(mm, (double)m2); else if (c != 0.0) mm = __dadd_rn(mm, __dmul_rn(c, (double)m2));
    if (d == 1.0) mm = __dadd_rn(mm, (double)m3); else if (d != 0.0) mm = __dadd_rn(mm, __dmul_rn(d, (double)m3));
    return (fabsf(v) < 1.1920928955078125e-07f) ? 0.0f                       // FLT_EPSILON
         : (fabs(mm) < 1.1920928955078125e-07) ? 3.4028234663852886e+38f     // FLT_MAX
         : __double2float_rn(__ddiv_rn((double)v, mm));
}

// ---- compute_combo without the FP64 pipe in the common case ----
// (ComboCoef, prepared once per launch, is declared in internal.h.)

// combo_value, with the same result for every input: the denominator and the
// quotient are first formed in float-float arithmetic (FMA-exact products,
// TwoSum additions, a remainder-corrected division) together with a bound on
// their distance from the reference's double values; when that bound keeps
// the quotient strictly inside one float's rounding interval, that float is
// fl32(fl64(v / mm)) of the reference; otherwise (ties, the FLT_EPSILON guard's
// boundary, heavy cancellation, over/underflow, NaN) the double formula runs.
__device__ __forceinline__ float combo_value_ff(float v, float m1, float m2, float m3, const ComboCoef& k) {
    if (fabsf(v) < 1.1920928955078125e-07f) return 0.0f;  // |mi| < FLT_EPSILON (exact test)
    const float xs[4] = {v, m1, m2, m3};
    float sh = 0.0f, sl = 0.0f, mag = 0.0f;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        if (k.kind[i] == 0) continue;
        float ph = xs[i], pl = 0.0f;
        if (k.kind[i] == 2) {
            ph = __fmul_rn(k.hi[i], xs[i]);
            pl = __fadd_rn(__fmaf_rn(k.hi[i], xs[i], -ph), __fmul_rn(k.lo[i], xs[i]));
        }
        mag = __fadd_rn(mag, fabsf(ph));
        // (sh, sl) += (ph, pl): TwoSum of the heads, tails added, renormalised
        const float s = __fadd_rn(sh, ph);
        const float bb = __fsub_rn(s, sh);
        float e = __fadd_rn(__fsub_rn(sh, __fsub_rn(s, bb)), __fsub_rn(ph, bb));
        e = __fadd_rn(e, __fadd_rn(sl, pl));
        sh = __fadd_rn(s, e);
        sl = __fsub_rn(e, __fsub_rn(sh, s));
    }
    // |(sh + sl) - mm_ref| <= 2^-41 * sum |terms| (float-float rounding, the
    // reference's own double roundings), with slack for the float sum of |terms|
    const float emm = __fmul_rn(mag, 4.6e-13f);
    const float sabs = fabsf(sh);
    if (!(sabs < 3.0e38f) || !(mag < 3.0e38f)) return combo_value(v, m1, m2, m3, k.c[0], k.c[1], k.c[2], k.c[3]);
    const float margin = __fadd_rn(fabsf(sl), emm) * 1.001f;
    if (sabs + margin < 1.1920928955078125e-07f) return 3.4028234663852886e+38f;  // |mm| < FLT_EPSILON
    if (!(sabs - margin > 1.1920928955078125e-07f) || mag > 1024.0f * sabs)   // guard boundary, cancellation
        return combo_value(v, m1, m2, m3, k.c[0], k.c[1], k.c[2], k.c[3]);
    const float qh = __fdiv_rn(v, sh);
    const float aq = fabsf(qh);
    if (!(aq < 1.0e38f) || !(aq > 1.0e-30f)) return combo_value(v, m1, m2, m3, k.c[0], k.c[1], k.c[2], k.c[3]);
    float r = __fmaf_rn(-qh, sh, v);     // v - qh*sh, exact for the correctly rounded qh
    r = __fmaf_rn(-qh, sl, r);
    const float ql = __fdiv_rn(r, sh);
    const float F = __fadd_rn(qh, ql);
    const float d = __fadd_rn(__fsub_rn(qh, F), ql);  // (qh + ql) - F
    const uint32_t fb = __float_as_uint(F) & 0x7fffffffu;
    const float ulp = __uint_as_float(((fb >> 23) - 23u) << 23);  // |F| > 1e-30: biased exponent > 27
    const float gap = (d < 0.0f && (fb & 0x7fffffu) == 0u) ? __fmul_rn(ulp, 0.25f) : __fmul_rn(ulp, 0.5f);
    // relative distance of qh + ql from fl64(v / mm_ref): 2^-44 (division) + emm/|sh| + 2^-52
    const float rel = __fadd_rn(2.0e-13f, __fdiv_rn(emm, sabs)) * 1.01f;
    const float tol = __fadd_rn(__fmul_rn(rel, fabsf(F)), __fmul_rn(fabsf(d), 1.2e-7f));
    if (fabsf(d) + tol < gap) return F;
    return combo_value(v, m1, m2, m3, k.c[0], k.c[1], k.c[2], k.c[3]);
}

}  // namespace mcpg