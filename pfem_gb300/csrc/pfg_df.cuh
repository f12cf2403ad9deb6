// Double-float arithmetic: a value is an unevaluated sum hi + lo of two FP32 numbers (~48
// significant bits), combined with error-free transforms (TwoSum, FMA-based TwoProduct; Dekker
// 1971, Knuth TAOCP vol. 2 4.2.2).  GB300 issues FP64 at 1/64 of the FP32 rate, so kernels
// whose FP64 work is the bottleneck run their arithmetic in double-float on the FP32 pipe and
// convert to FP64 only at their inputs and outputs.  The __f*_rn intrinsics keep the compiler
// from contracting or reassociating the transforms.  Header-only device code.
#pragma once

#include <cuda_runtime.h>

namespace pfg {

struct DF {
    float h, l;
};

__device__ __forceinline__ void two_sum_f(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__device__ __forceinline__ void quick_two_sum_f(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    e = __fsub_rn(b, __fsub_rn(s, a));
}

// FP64 -> double-float (FP64 instructions: inputs only)
__device__ __forceinline__ DF df_from(double d) {
    const float h = (float)d;
    return DF{h, (float)(d - (double)h)};
}

// double-float -> FP64 (exact sum of the two parts)
__device__ __forceinline__ double df_to(DF a) { return (double)a.h + (double)a.l; }

__device__ __forceinline__ DF df_add(DF a, DF b) {
    float s, e, t, f;
    two_sum_f(a.h, b.h, s, e);
    two_sum_f(a.l, b.l, t, f);
    e = __fadd_rn(e, t);
    quick_two_sum_f(s, e, s, e);
    e = __fadd_rn(e, f);
    DF r;
    quick_two_sum_f(s, e, r.h, r.l);
    return r;
}

__device__ __forceinline__ DF df_neg(DF a) { return DF{-a.h, -a.l}; }

__device__ __forceinline__ DF df_mul(DF a, DF b) {
    const float p = __fmul_rn(a.h, b.h);
    float e = __fmaf_rn(a.h, b.h, -p);
    e = __fmaf_rn(a.h, b.l, e);
    e = __fmaf_rn(a.l, b.h, e);
    DF r;
    quick_two_sum_f(p, e, r.h, r.l);
    return r;
}

__device__ __forceinline__ DF df_sub(DF a, DF b) { return df_add(a, df_neg(b)); }

// a / b: the FP32 quotient q1 of the high parts, the exact remainder a - q1 b in double-float,
// and one correction term q2 = remainder / b.h (Dekker 1971, division with one correction).
__device__ __forceinline__ DF df_div(DF a, DF b) {
    const float q1 = __fdiv_rn(a.h, b.h);
    const float p = __fmul_rn(q1, b.h);
    const float pe = __fmaf_rn(q1, b.h, -p);  // q1 * b.h = p + pe exactly
    // r = a - q1 b = (a.h - p) - pe + a.l - q1 b.l
    float s, e;
    two_sum_f(a.h, -p, s, e);
    e = __fadd_rn(e, __fsub_rn(__fsub_rn(a.l, pe), __fmul_rn(q1, b.l)));
    const float r = __fadd_rn(s, e);
    const float q2 = __fdiv_rn(r, b.h);
    DF out;
    quick_two_sum_f(q1, q2, out.h, out.l);
    return out;
}

// sqrt(a) for a >= 0: the correctly rounded FP32 root y of the high part and one Newton
// correction (a - y^2) / (2 y) with a - y^2 formed exactly from the FMA residual (Karp and
// Markstein 1997).  sqrt(0) = 0; a < 0 gives NaN like the FP64 root.
__device__ __forceinline__ DF df_sqrt(DF a) {
    if (!(a.h > 0.0f)) return DF{a.h == 0.0f ? 0.0f : __fsqrt_rn(a.h), 0.0f};
    const float y = __fsqrt_rn(a.h);
    const float y2 = __fmul_rn(y, y);
    const float y2e = __fmaf_rn(y, y, -y2);  // y * y = y2 + y2e exactly
    const float r = __fadd_rn(__fsub_rn(__fsub_rn(a.h, y2), y2e), a.l);
    const float c = __fdiv_rn(r, __fadd_rn(y, y));
    DF out;
    quick_two_sum_f(y, c, out.h, out.l);
    return out;
}

}  // namespace pfg
