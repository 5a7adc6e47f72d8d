// Shared device helpers for the mcpgpu kernels (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

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

}  // namespace mcpg
