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

}  // namespace pfg
