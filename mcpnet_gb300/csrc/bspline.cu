// Per-gene min-max scaling, B-spline weights and FP64 marginal entropy (K1).
//
// Restates, one CTA per gene:
//   MinMaxScale::operator()            include/mcp/correlation/BSplineMI.hpp:81-115
//   buildKnotVector                     BSplineMI.hpp:35-71   (host, passed in)
//   BSplineWeightsKernel::basisFunction BSplineMI.hpp:130-164 (Cox-de Boor)
//   BSplineWeightsKernel::operator()    BSplineMI.hpp:248-273
//   entropy1d_2                         BSplineMI.hpp:204-224 (here in FP64)
// The basis recursion is evaluated bottom-up (order 1 .. k) with the same float
// operations in the same order as the recursive reference, and with explicit
// round-to-nearest intrinsics so nvcc cannot fuse a multiply and an add into an
// FMA: the weights are bit-identical to the reference compiled without FMA
// contraction.
//
// Output layouts (one kernel, chosen by template):
//   OUT_REF   : W[g*(bins*m+1) + a*m + s] and W[g*(bins*m+1) + bins*m] = (float)H_g
//               -- the reference's own Transform output row.
//   OUT_T32   : Wt[s*ldwt + g*bins + a] (sample-major FP32, CUDA-core MI)
//   OUT_BF16/OUT_FP16 : Whi/Wlo[(g*bins + a)*ldw + s] (gene-bin-major, K = samples
//               contiguous, zero-padded to ldw; tcgen05 MI)
//   OUT_BF16F8 : Whi = bf16(w) * 2^8 (BF16, the layout above), and the E4M3 correction
//               operands H8 = e4m3(bf16(w) * 2^4), L8 = e4m3((w - bf16(w)) * 2^12) in one
//               interleaved plane HL8 of rows of 2 * ldw bytes: for every 64 samples of a
//               row, their 64 H8 bytes then their 64 L8 bytes, so that one 128-byte TMA box
//               row carries both correction operands of a 64-sample slice.
//               The scales multiply to 2^16 in every product (hi*hi, H8*L8, L8*H8), so
//               the three contractions accumulate 2^16 * P into one FP32 accumulator.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_fp8.h>
#include <math.h>

#include <cmath>

#include "common.cuh"
#include "internal.h"

namespace mcpg {
namespace {

constexpr int KMAX_BINS = 32, KMAX_ORDER = 8, KNOTS_MAX = KMAX_BINS + KMAX_ORDER;
constexpr int WTHREADS = 256;

struct Knots {
    float v[KNOTS_MAX];
    // When every nonzero knot span is a power of two (10 bins / order 3: spans
    // of 1/8 and 1/4), n / span == n * (1 / span) exactly, so the recursion's
    // divisions become multiplications by these exact reciprocals without
    // changing a bit.  r1[p][i] = 1 / (t[i+p-1] - t[i]), r2[p][i] = 1 / (t[i+p] - t[i+1]).
    int pow2;
    // The reference's guards compare a float against the double 1e-10.  For a float x,
    // (double)x < 1e-10 exactly when x < eps, eps = the smallest float above 1e-10
    // (1e-10 is not a float), so the guards run on the FP32 pipe with the same outcome.
    float eps;
    float r1[KMAX_ORDER + 1][KNOTS_MAX];
    float r2[KMAX_ORDER + 1][KNOTS_MAX];
};

enum OutKind { OUT_REF = 0, OUT_T32 = 1, OUT_BF16 = 2, OUT_FP16 = 3, OUT_BF16F8 = 4 };

void host_knots(int bins, int order, Knots& k) {
    // buildKnotVector<float> (BSplineMI.hpp:35-71): norm_factor in double,
    // v[i] = (float)((float)(i - order + 1) * norm_factor).
    const int nint = bins - order;
    const double nf = 1.0 / (double)(nint + 1);
    for (int i = 0; i < KNOTS_MAX; ++i) k.v[i] = 0.0f;
    for (int i = 0; i < order; ++i) k.v[i] = 0.0f;
    for (int i = order; i < order + nint; ++i) k.v[i] = (float)((double)(float)(i - order + 1) * nf);
    for (int i = order + nint; i < 2 * order + nint; ++i) k.v[i] = 1.0f;
    k.eps = (float)1e-10;
    if ((double)k.eps < 1e-10) k.eps = std::nextafter(k.eps, INFINITY);
    // exact reciprocals of the knot spans, when they are all powers of two
    k.pow2 = 1;
    for (int p = 0; p <= KMAX_ORDER; ++p)
        for (int i = 0; i < KNOTS_MAX; ++i) k.r1[p][i] = k.r2[p][i] = 0.0f;
    auto pow2_or_zero = [](float d) {
        if (!(d >= 1e-10f)) return true;
        int e = 0;
        return std::frexp(d, &e) == 0.5f;
    };
    for (int p = 2; p <= order; ++p)
        for (int i = 0; i + p < KNOTS_MAX && i < bins + order - p; ++i) {
            const float d1 = k.v[i + p - 1] - k.v[i], d2 = k.v[i + p] - k.v[i + 1];
            if (!pow2_or_zero(d1) || !pow2_or_zero(d2)) k.pow2 = 0;
            k.r1[p][i] = d1 >= 1e-10f ? 1.0f / d1 : 0.0f;
            k.r2[p][i] = d2 >= 1e-10f ? 1.0f / d2 : 0.0f;
        }
}

// n / d for a knot span d: an exact multiplication when the spans are powers of two.
__device__ __forceinline__ float span_div(const Knots& kv, float n, float d, float rinv) {
    return kv.pow2 ? __fmul_rn(n, rinv) : __fdiv_rn(n, d);
}

// All bins' basis values at t, bottom-up.  N[i] holds basis(i, p, t) for the
// current p.  Each value is produced by the same float operations as the
// recursive reference (divide, multiply, add, clamp), so the results agree bit
// for bit.  BT / OT > 0 fix bins / order at compile time (registers only);
// 0 takes them from the arguments.
template <int BT, int OT>
__device__ __forceinline__ void basis_all(const Knots& kv, int bins_rt, int order_rt, float t, float* out,
                                          float* prev = nullptr) {
    const int bins = BT ? BT : bins_rt;
    const int order = OT ? OT : order_rt;
    constexpr int NMAX = (BT && OT) ? BT + OT : KNOTS_MAX;
    float N[NMAX];
    const int n1 = bins + order - 1;  // number of order-1 functions needed
#pragma unroll
    for (int i = 0; i < NMAX - 1; ++i) {
        if (i >= n1) break;
        const float a = kv.v[i], b = kv.v[i + 1];
        const bool in = (t >= a && t < b && a < b) ||
                        (fabsf(__fsub_rn(t, b)) < kv.eps && (i + 1 == bins));
        N[i] = in ? 1.0f : 0.0f;
    }
#pragma unroll
    for (int p = 2; p <= (OT ? OT : KMAX_ORDER); ++p) {
        if (p > order) break;
        if (prev && p == order) {  // keep the order-1 level (bins + 1 values) for the derivative
#pragma unroll
            for (int i = 0; i < (BT ? BT + 1 : KMAX_BINS + 1); ++i)
                if (i <= bins) prev[i] = N[i];
        }
        const int np = bins + order - p;
#pragma unroll
        for (int i = 0; i < NMAX - 1; ++i) {
            if (i >= np) break;
            const float d1 = __fsub_rn(kv.v[i + p - 1], kv.v[i]);
            const float n1v = __fsub_rn(t, kv.v[i]);
            const float d2 = __fsub_rn(kv.v[i + p], kv.v[i + 1]);
            const float n2v = __fsub_rn(kv.v[i + p], t);
            float r;
            if (d1 < kv.eps && d2 < kv.eps) {
                r = 0.0f;
            } else {
                float e1, e2;
                if (d1 < kv.eps) {
                    e1 = 0.0f;
                    e2 = __fmul_rn(span_div(kv, n2v, d2, kv.r2[p][i]), N[i + 1]);
                } else if (d2 < kv.eps) {
                    e2 = 0.0f;
                    e1 = __fmul_rn(span_div(kv, n1v, d1, kv.r1[p][i]), N[i]);
                } else {
                    e1 = __fmul_rn(span_div(kv, n1v, d1, kv.r1[p][i]), N[i]);
                    e2 = __fmul_rn(span_div(kv, n2v, d2, kv.r2[p][i]), N[i + 1]);
                }
                const float s = __fadd_rn(e1, e2);
                r = (s < 0.0f) ? 0.0f : s;
            }
            N[i] = r;  // N[i+1] (still order p-1) is read before it is overwritten
        }
    }
#pragma unroll
    for (int a = 0; a < (BT ? BT : KMAX_BINS); ++a)
        if (a < bins) out[a] = N[a];
}

// Per-thread bin sums in FP32 with Neumaier compensation (sum + carry): the FP64
// pipe of this part is far slower than FP32, and the compensated pair keeps
// the per-thread partial to about 2^-48 relative before the FP64 block reduction.
struct CompSum {
    float s = 0.0f, c = 0.0f;
    __device__ __forceinline__ void add(float v) {
        const float t = __fadd_rn(s, v);
        c = __fadd_rn(c, (fabsf(s) >= fabsf(v)) ? __fadd_rn(__fsub_rn(s, t), v) : __fadd_rn(__fsub_rn(v, t), s));
        s = t;
    }
    __device__ __forceinline__ double value() const { return (double)s + (double)c; }
};

template <typename T>
__device__ __forceinline__ T block_reduce(T v, T (*op)(T, T), T* scratch) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = op(v, __shfl_xor_sync(0xffffffffu, v, o));
    __syncthreads();
    if (lane == 0) scratch[warp] = v;
    __syncthreads();
    T r = scratch[0];
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) r = op(r, scratch[w]);
    return r;
}
__device__ float op_min(float a, float b) { return (b < a) ? b : a; }
__device__ float op_max(float a, float b) { return (a < b) ? b : a; }

template <int OUT, int BT, int OT>
__global__ void __launch_bounds__(WTHREADS) bspline_weights_kernel(const float* __restrict__ X, int64_t n, int64_t m,
                                                                   int64_t ldx, int bins_rt, int order_rt, const Knots kv,
                                                                   void* __restrict__ out0, void* __restrict__ out1,
                                                                   void* __restrict__ out2, int64_t ldo,
                                                                   double* __restrict__ H) {
    __shared__ float fscratch[32];
    __shared__ float sh_scale;
    __shared__ double psum[KMAX_BINS][WTHREADS / 32];
    const int64_t g = blockIdx.x;
    if (g >= n) return;
    const float* x = X + g * ldx;
    const int bins = BT ? BT : bins_rt;
    constexpr int NB = BT ? BT : KMAX_BINS;

    // ---- MinMaxScale (BSplineMI.hpp:86-115) ----
    float mn = INFINITY, mx = -INFINITY;
    for (int64_t s = threadIdx.x; s < m; s += blockDim.x) {
        const float v = x[s];
        mn = (v < mn) ? v : mn;
        mx = (mx < v) ? v : mx;
    }
    mn = block_reduce<float>(mn, op_min, fscratch);
    mx = block_reduce<float>(mx, op_max, fscratch);
    // the reference's 1 / (max - min) in double, once per gene (FP64 is a narrow pipe here)
    if (threadIdx.x == 0) sh_scale = (mx > mn) ? (float)(1.0 / (double)__fsub_rn(mx, mn)) : 1.0f;
    __syncthreads();
    const float scale = sh_scale;
    const float offset = (mx > mn) ? mn : 0.0f;

    CompSum acc[NB];

    float w[NB];
    for (int64_t s = threadIdx.x; s < m; s += blockDim.x) {
        const float t = __fmul_rn(scale, __fsub_rn(x[s], offset));
        basis_all<BT, OT>(kv, bins_rt, order_rt, t, w);
#pragma unroll
        for (int a = 0; a < NB; ++a)
            if (a < bins) acc[a].add(w[a]);
        if (OUT == OUT_REF) {
            float* W = static_cast<float*>(out0) + g * ((int64_t)bins * m + 1);
            for (int a = 0; a < bins; ++a) W[(int64_t)a * m + s] = w[a];
        } else if (OUT == OUT_T32) {
            float* W = static_cast<float*>(out0) + s * ldo + g * bins;
            for (int a = 0; a < bins; ++a) W[a] = w[a];
        } else if (OUT == OUT_BF16F8) {
            const int64_t s8 = (s >> 6) * 128 + (s & 63);  // H8 byte of sample s in an HL8 row; L8 at +64
            for (int a = 0; a < bins; ++a) {
                const int64_t o = (g * bins + a) * ldo + s;
                const __nv_bfloat16 hi = __float2bfloat16_rn(w[a]);
                const float hf = __bfloat162float(hi);
                static_cast<__nv_bfloat16*>(out0)[o] = __float2bfloat16_rn(hf * 256.0f);
                __nv_fp8_storage_t* hl = static_cast<__nv_fp8_storage_t*>(out1) + (g * bins + a) * 2 * ldo + s8;
                hl[0] = __nv_cvt_float_to_fp8(hf * 16.0f, __NV_SATFINITE, __NV_E4M3);
                hl[64] = __nv_cvt_float_to_fp8(__fsub_rn(w[a], hf) * 4096.0f, __NV_SATFINITE, __NV_E4M3);
            }
        } else {
            for (int a = 0; a < bins; ++a) {
                const int64_t o = (g * bins + a) * ldo + s;
                if (OUT == OUT_BF16) {
                    const __nv_bfloat16 hi = __float2bfloat16_rn(w[a]);
                    static_cast<__nv_bfloat16*>(out0)[o] = hi;
                    if (out1) static_cast<__nv_bfloat16*>(out1)[o] = __float2bfloat16_rn(w[a] - __bfloat162float(hi));
                } else {
                    const __half hi = __float2half_rn(w[a]);
                    static_cast<__half*>(out0)[o] = hi;
                    if (out1) static_cast<__half*>(out1)[o] = __float2half_rn(w[a] - __half2float(hi));
                }
            }
        }
    }
    // zero the K padding of the tensor-core layouts
    if (OUT == OUT_BF16F8) {
        for (int64_t s = m + threadIdx.x; s < ldo; s += blockDim.x)
            for (int a = 0; a < bins; ++a) {
                const int64_t o = (g * bins + a) * ldo + s;
                static_cast<uint16_t*>(out0)[o] = 0;
                uint8_t* hl = static_cast<uint8_t*>(out1) + (g * bins + a) * 2 * ldo + (s >> 6) * 128 + (s & 63);
                hl[0] = 0;
                hl[64] = 0;
            }
    }
    if (OUT == OUT_BF16 || OUT == OUT_FP16) {
        for (int64_t s = m + threadIdx.x; s < ldo; s += blockDim.x)
            for (int a = 0; a < bins; ++a) {
                const int64_t o = (g * bins + a) * ldo + s;
                static_cast<uint16_t*>(out0)[o] = 0;
                if (out1) static_cast<uint16_t*>(out1)[o] = 0;
            }
    }

    // ---- marginal entropy in FP64 (entropy1d_2, BSplineMI.hpp:204-224) ----
    // Per-bin sums: each thread's compensated pair is reduced across the warp in
    // float-float (TwoSum, about 2^-44 relative), converted to FP64 once per warp;
    // lanes 0..bins-1 of warp 0 then sum the warps and form p log2 p in FP64.
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int a = 0; a < NB; ++a) {
        if (a >= bins) break;
        float hs = acc[a].s, hc = acc[a].c;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float s2 = __shfl_xor_sync(0xffffffffu, hs, o), c2 = __shfl_xor_sync(0xffffffffu, hc, o);
            const float t = __fadd_rn(hs, s2);
            const float bp = __fsub_rn(t, hs);
            const float e = __fadd_rn(__fsub_rn(hs, __fsub_rn(t, bp)), __fsub_rn(s2, bp));
            hc = __fadd_rn(__fadd_rn(hc, c2), e);
            hs = t;
        }
        if (lane == 0) psum[a][warp] = (double)hs + (double)hc;
    }
    __syncthreads();
    if (warp == 0) {
        double term = 0.0;
        if (lane < bins) {
            double p = 0.0;
            for (int w2 = 0; w2 < (int)(blockDim.x >> 5); ++w2) p += psum[lane][w2];
            p *= 1.0 / (double)m;
            if (p > 0.0) term = p * log2(p);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) term += __shfl_xor_sync(0xffffffffu, term, o);
        if (lane == 0) {
            const double Hg = -term;
            if (H) H[g] = Hg;
            if (OUT == OUT_REF) static_cast<float*>(out0)[g * ((int64_t)bins * m + 1) + (int64_t)bins * m] = (float)Hg;
        }
    }
}

// ---------------- MI adjoint through the weights and the scaling ----------------
// Derivative of the basis, from the order-1 level:
//   N'_{a,p}(t) = (p-1) [ N_{a,p-1}(t)/(t_{a+p-1}-t_a) - N_{a+1,p-1}(t)/(t_{a+p}-t_{a+1}) ]
// (a term is dropped when its knot span is below 1e-10, the basis's own guard).
__device__ __forceinline__ float basis_deriv(const Knots& kv, int order, int a, const float* prev) {
    if (order <= 1) return 0.0f;
    const float d1 = kv.v[a + order - 1] - kv.v[a], d2 = kv.v[a + order] - kv.v[a + 1];
    float r = 0.0f;
    if (!(d1 < 1e-10f)) r += prev[a] / d1;
    if (!(d2 < 1e-10f)) r -= prev[a + 1] / d2;
    return (float)(order - 1) * r;
}

struct ValIdx {
    float v;
    int64_t i;
};

template <int BT, int OT>
__global__ void __launch_bounds__(WTHREADS) mi_bwd_x_kernel(const float* __restrict__ X, int64_t m, int64_t ldx,
                                                            int bins_rt, int order_rt, const Knots kv, int64_t g0,
                                                            const float* __restrict__ gsum,
                                                            const float* __restrict__ dWq, int64_t lddw,
                                                            float* __restrict__ dX, int64_t lddx) {
    __shared__ ValIdx red_min[WTHREADS / 32], red_max[WTHREADS / 32];
    __shared__ double dred[2][WTHREADS / 32];
    __shared__ double psum[KMAX_BINS][WTHREADS / 32];
    __shared__ float hc[KMAX_BINS];
    const int64_t g = g0 + blockIdx.x;
    const float* x = X + g * ldx;
    const int bins = BT ? BT : bins_rt;
    const int order = OT ? OT : order_rt;
    constexpr int NB = BT ? BT : KMAX_BINS;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;

    // first arg-min / arg-max (ties -> lowest sample index)
    ValIdx mn{INFINITY, INT64_MAX}, mx{-INFINITY, INT64_MAX};
    for (int64_t s = threadIdx.x; s < m; s += blockDim.x) {
        const float v = x[s];
        if (v < mn.v || (v == mn.v && s < mn.i)) mn = {v, s};
        if (v > mx.v || (v == mx.v && s < mx.i)) mx = {v, s};
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        ValIdx a{__shfl_xor_sync(0xffffffffu, mn.v, o), __shfl_xor_sync(0xffffffffu, mn.i, o)};
        ValIdx b{__shfl_xor_sync(0xffffffffu, mx.v, o), __shfl_xor_sync(0xffffffffu, mx.i, o)};
        if (a.v < mn.v || (a.v == mn.v && a.i < mn.i)) mn = a;
        if (b.v > mx.v || (b.v == mx.v && b.i < mx.i)) mx = b;
    }
    if (lane == 0) { red_min[warp] = mn; red_max[warp] = mx; }
    __syncthreads();
    mn = red_min[0];
    mx = red_max[0];
    for (int w = 1; w < nw; ++w) {
        const ValIdx a = red_min[w], b = red_max[w];
        if (a.v < mn.v || (a.v == mn.v && a.i < mn.i)) mn = a;
        if (b.v > mx.v || (b.v == mx.v && b.i < mx.i)) mx = b;
    }
    const bool ranged = mx.v > mn.v;
    const float scale = ranged ? (float)(1.0 / (double)__fsub_rn(mx.v, mn.v)) : 1.0f;
    const float offset = ranged ? mn.v : 0.0f;

    // marginals p_a -> log2 p_a + 1/ln 2
    float w[NB], prev[NB + 1];
    CompSum acc[NB];
    for (int64_t s = threadIdx.x; s < m; s += blockDim.x) {
        const float t = __fmul_rn(scale, __fsub_rn(x[s], offset));
        basis_all<BT, OT>(kv, bins_rt, order_rt, t, w);
#pragma unroll
        for (int a = 0; a < NB; ++a)
            if (a < bins) acc[a].add(w[a]);
    }
#pragma unroll
    for (int a = 0; a < NB; ++a) {
        if (a >= bins) break;
        double v = acc[a].value();
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) psum[a][warp] = v;
    }
    __syncthreads();
    if (threadIdx.x < bins) {
        double p = 0.0;
        for (int w2 = 0; w2 < nw; ++w2) p += psum[threadIdx.x][w2];
        p /= (double)m;
        hc[threadIdx.x] = p > 0.0 ? (float)(log2(p) + 1.4426950408889634) : 0.0f;
    }
    __syncthreads();

    // dL/dt_s = (1/m) sum_a (-hc_a gsum + dWq[a][s]) N'_a(t_s), then dL/dx
    const float gs = gsum[g];
    const float inv_m = 1.0f / (float)m;
    double s1 = 0.0, s2 = 0.0;
    const float* dw = dWq + (int64_t)blockIdx.x * bins * lddw;
    for (int64_t s = threadIdx.x; s < m; s += blockDim.x) {
        const float t = __fmul_rn(scale, __fsub_rn(x[s], offset));
        basis_all<BT, OT>(kv, bins_rt, order_rt, t, w, prev);
        float dt = 0.0f;
#pragma unroll
        for (int a = 0; a < NB; ++a) {
            if (a >= bins) break;
            const float gw = dw[(int64_t)a * lddw + s] - hc[a] * gs;
            dt += gw * basis_deriv(kv, order, a, prev);
        }
        dt *= inv_m;
        dX[g * lddx + s] = scale * dt;
        s1 += (double)dt * ((double)t - 1.0);
        s2 += (double)dt * (double)t;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        s1 += __shfl_xor_sync(0xffffffffu, s1, o);
        s2 += __shfl_xor_sync(0xffffffffu, s2, o);
    }
    if (lane == 0) { dred[0][warp] = s1; dred[1][warp] = s2; }
    __syncthreads();
    if (threadIdx.x == 0 && ranged) {
        double a1 = 0.0, a2 = 0.0;
        for (int w2 = 0; w2 < nw; ++w2) { a1 += dred[0][w2]; a2 += dred[1][w2]; }
        dX[g * lddx + mn.i] += (float)((double)scale * a1);   // d t_s / d min = scale (t_s - 1)
        dX[g * lddx + mx.i] -= (float)((double)scale * a2);   // d t_s / d max = -scale t_s
    }
}

__global__ void pair_sums_kernel(const float* __restrict__ G, int64_t ldg, int64_t n, float* __restrict__ gsum) {
    // one warp per gene: row sum + column sum, diagonal excluded
    const int64_t i = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (i >= n) return;
    double s = 0.0;
    for (int64_t j = lane; j < n; j += 32)
        if (j != i) s += (double)G[i * ldg + j] + (double)G[j * ldg + i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) gsum[i] = (float)s;
}

}  // namespace

cudaError_t launch_pair_sums(const float* G, int64_t ldg, int64_t n, float* gsum, cudaStream_t stream,
                             int64_t* launches) {
    if (n <= 0) return cudaSuccess;
    if (launches) ++*launches;
    pair_sums_kernel<<<(unsigned)ceil_div(n, 8), 256, 0, stream>>>(G, ldg, n, gsum);
    return cudaGetLastError();
}

cudaError_t launch_mi_bwd_x(const float* X, int64_t n, int64_t m, int64_t ldx, int bins, int order, int64_t g0,
                            int64_t g1, const float* gsum, const float* dWq, int64_t lddw, float* dX, int64_t lddx,
                            cudaStream_t stream, int64_t* launches) {
    if (g1 <= g0) return cudaSuccess;
    if (g0 < 0 || g1 > n) return cudaErrorInvalidValue;
    Knots kv;
    host_knots(bins, order, kv);
    if (launches) ++*launches;
    if (bins == 10 && order == 3)
        mi_bwd_x_kernel<10, 3><<<(unsigned)(g1 - g0), WTHREADS, 0, stream>>>(X, m, ldx, bins, order, kv, g0, gsum,
                                                                            dWq, lddw, dX, lddx);
    else
        mi_bwd_x_kernel<0, 0><<<(unsigned)(g1 - g0), WTHREADS, 0, stream>>>(X, m, ldx, bins, order, kv, g0, gsum,
                                                                          dWq, lddw, dX, lddx);
    return cudaGetLastError();
}

cudaError_t launch_bspline_weights_ref(const float* X, int64_t n, int64_t m, int64_t ldx, int bins, int order,
                                       float* W, double* H, cudaStream_t stream, int64_t* launches) {
    if (n <= 0) return cudaSuccess;
    Knots kv;
    host_knots(bins, order, kv);
    if (launches) ++*launches;
    if (bins == 10 && order == 3)
        bspline_weights_kernel<OUT_REF, 10, 3><<<(unsigned)n, WTHREADS, 0, stream>>>(X, n, m, ldx, bins, order, kv, W,
                                                                                 nullptr, nullptr, 0, H);
    else
        bspline_weights_kernel<OUT_REF, 0, 0><<<(unsigned)n, WTHREADS, 0, stream>>>(X, n, m, ldx, bins, order, kv, W,
                                                                               nullptr, nullptr, 0, H);
    return cudaGetLastError();
}

cudaError_t launch_bspline_weights_fp32(const float* X, int64_t n, int64_t m, int64_t ldx, int bins, int order,
                                        float* Wt, int64_t ldwt, double* H, cudaStream_t stream, int64_t* launches) {
    if (n <= 0) return cudaSuccess;
    Knots kv;
    host_knots(bins, order, kv);
    if (launches) ++*launches;
    if (bins == 10 && order == 3)
        bspline_weights_kernel<OUT_T32, 10, 3><<<(unsigned)n, WTHREADS, 0, stream>>>(X, n, m, ldx, bins, order, kv, Wt,
                                                                                 nullptr, nullptr, ldwt, H);
    else
        bspline_weights_kernel<OUT_T32, 0, 0><<<(unsigned)n, WTHREADS, 0, stream>>>(X, n, m, ldx, bins, order, kv, Wt,
                                                                               nullptr, nullptr, ldwt, H);
    return cudaGetLastError();
}

cudaError_t launch_bspline_weights_16(const float* X, int64_t n, int64_t m, int64_t ldx, int bins, int order,
                                      int fmt, uint16_t* Whi, uint16_t* Wlo, int64_t ldw, double* H,
                                      cudaStream_t stream, int64_t* launches) {
    if (n <= 0) return cudaSuccess;
    Knots kv;
    host_knots(bins, order, kv);
    if (launches) ++*launches;
    const bool fast = bins == 10 && order == 3;
    if (fmt == 0 && fast)
        bspline_weights_kernel<OUT_BF16, 10, 3><<<(unsigned)n, WTHREADS, 0, stream>>>(X, n, m, ldx, bins, order, kv,
                                                                                  Whi, Wlo, nullptr, ldw, H);
    else if (fmt == 0)
        bspline_weights_kernel<OUT_BF16, 0, 0><<<(unsigned)n, WTHREADS, 0, stream>>>(X, n, m, ldx, bins, order, kv,
                                                                                Whi, Wlo, nullptr, ldw, H);
    else if (fast)
        bspline_weights_kernel<OUT_FP16, 10, 3><<<(unsigned)n, WTHREADS, 0, stream>>>(X, n, m, ldx, bins, order, kv,
                                                                                  Whi, Wlo, nullptr, ldw, H);
    else
        bspline_weights_kernel<OUT_FP16, 0, 0><<<(unsigned)n, WTHREADS, 0, stream>>>(X, n, m, ldx, bins, order, kv,
                                                                                Whi, Wlo, nullptr, ldw, H);
    return cudaGetLastError();
}

cudaError_t launch_bspline_weights_f8(const float* X, int64_t n, int64_t m, int64_t ldx, int bins, int order,
                                      uint16_t* Whi, uint8_t* HL8, int64_t ldw, double* H, cudaStream_t stream,
                                      int64_t* launches) {
    if (n <= 0) return cudaSuccess;
    Knots kv;
    host_knots(bins, order, kv);
    if (launches) ++*launches;
    if (bins == 10 && order == 3)
        bspline_weights_kernel<OUT_BF16F8, 10, 3><<<(unsigned)n, WTHREADS, 0, stream>>>(X, n, m, ldx, bins, order, kv,
                                                                                    Whi, HL8, nullptr, ldw, H);
    else
        bspline_weights_kernel<OUT_BF16F8, 0, 0><<<(unsigned)n, WTHREADS, 0, stream>>>(X, n, m, ldx, bins, order, kv,
                                                                                  Whi, HL8, nullptr, ldw, H);
    return cudaGetLastError();
}

}  // namespace mcpg
