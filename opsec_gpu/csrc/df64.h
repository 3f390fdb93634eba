// Double-FP32 arithmetic: a value is the unevaluated sum hi + lo of two floats (|lo| <= half an
// ulp of hi), about 48 significant bits.  On this part FP64 instructions issue at 1/64 of the
// FP32 rate, so a product-accumulate in pairs of floats (about 15 FP32 instructions) is several
// times faster than one FP64 FMA.  The building blocks are the error-free transformations of
// Knuth (two-sum) and Dekker (fast two-sum), with the product error from one FMA (exact, as
// the FMA rounds once).
#pragma once

#include <cuda_runtime.h>

namespace opsec {

struct df {
    float h, l;
};

__device__ __forceinline__ df df_from(double x) {
    const float h = (float)x;
    return {h, (float)(x - (double)h)};
}
__device__ __forceinline__ double df_to(df x) { return (double)x.h + (double)x.l; }
__device__ __forceinline__ float2 df_pack(df x) { return make_float2(x.h, x.l); }
__device__ __forceinline__ df df_unpack(float2 v) { return {v.x, v.y}; }

// s + e = a + b exactly
__device__ __forceinline__ float two_sum(float a, float b, float& e) {
    const float s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
    return s;
}
// s + e = a + b exactly when |a| >= |b| (or a = 0)
__device__ __forceinline__ df fast_two_sum(float a, float b) {
    const float s = a + b;
    return {s, b - (s - a)};
}

// acc + x * y
__device__ __forceinline__ df df_fma(df acc, df x, df y) {
    const float p = x.h * y.h;
    float e = fmaf(x.h, y.h, -p);
    e = fmaf(x.h, y.l, e);
    e = fmaf(x.l, y.h, e);
    float t;
    const float s = two_sum(acc.h, p, t);
    return fast_two_sum(s, t + (acc.l + e));
}
// acc - x * y
__device__ __forceinline__ df df_fms(df acc, df x, df y) { return df_fma(acc, {-x.h, -x.l}, y); }
// x * y
__device__ __forceinline__ df df_mul(df x, df y) {
    const float p = x.h * y.h;
    float e = fmaf(x.h, y.h, -p);
    e = fmaf(x.h, y.l, e);
    e = fmaf(x.l, y.h, e);
    return fast_two_sum(p, e);
}
// x + y
__device__ __forceinline__ df df_add(df x, df y) {
    float t;
    const float s = two_sum(x.h, y.h, t);
    return fast_two_sum(s, t + (x.l + y.l));
}

}  // namespace opsec
