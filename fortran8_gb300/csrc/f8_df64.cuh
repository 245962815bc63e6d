// f8_df64.cuh — double-float ("df64") arithmetic for the mixed-precision path.
//
// A df64 value is an unevaluated sum hi + lo of two FP32 numbers with
// |lo| <= ulp(hi)/2, i.e. a 48-bit significand.  The state fields of the mixed
// path (U, V, W, P and the pressure correction Phi) are held this way so that
// their accumulation and their differences keep FP64-class accuracy while all
// arithmetic runs on the FP32 pipes (the FP64 rate of this part is a small
// fraction of the FP32 rate).
//
// The operations are the error-free transformations of Knuth (two-sum) and
// Dekker (fast two-sum, and the product error via fused multiply-add), as used
// in double-double libraries (Hida, Li and Bailey, "Algorithms for quad-double
// precision floating point arithmetic", 2001), specialised to FP32 pairs.
// Every step uses the _rn intrinsics so that the compiler neither contracts
// nor reassociates them.
#pragma once
#include <cuda_runtime.h>

namespace f8 {

struct df {
    float hi, lo;
};

// s + e = a + b exactly (Knuth)
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// s + e = a + b exactly, for |a| >= |b| or a = 0 (Dekker)
__device__ __forceinline__ void fast_two_sum(float a, float b, float &s, float &e) {
    s = __fadd_rn(a, b);
    e = __fsub_rn(b, __fsub_rn(s, a));
}

__device__ __forceinline__ df df_make(float hi, float lo) { return df{hi, lo}; }

// a + b, b a float
__device__ __forceinline__ df df_add_f(df a, float b) {
    float s, e;
    two_sum(a.hi, b, s, e);
    e = __fadd_rn(e, a.lo);
    df r;
    fast_two_sum(s, e, r.hi, r.lo);
    return r;
}

// a + b with absolute error ~2^-48 (|a| + |b|): the accuracy FP64 gives the
// stencil differences and sums of this path (the "sloppy" double-double add)
__device__ __forceinline__ df df_add(df a, df b) {
    float s, e;
    two_sum(a.hi, b.hi, s, e);
    e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
    df r;
    fast_two_sum(s, e, r.hi, r.lo);
    return r;
}

__device__ __forceinline__ df df_neg(df a) { return df{-a.hi, -a.lo}; }

__device__ __forceinline__ df df_sub(df a, df b) { return df_add(a, df_neg(b)); }

// a - b for two floats, exact
__device__ __forceinline__ df df_diff_ff(float a, float b) {
    df r;
    two_sum(a, -b, r.hi, r.lo);
    return r;
}

// a * b
__device__ __forceinline__ df df_mul(df a, df b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    df r;
    fast_two_sum(p, e, r.hi, r.lo);
    return r;
}

// a * b, b a float
__device__ __forceinline__ df df_mul_f(df a, float b) {
    const float p = __fmul_rn(a.hi, b);
    float e = __fmaf_rn(a.hi, b, -p);
    e = __fmaf_rn(a.lo, b, e);
    df r;
    fast_two_sum(p, e, r.hi, r.lo);
    return r;
}

__device__ __forceinline__ float df_to_f(df a) { return __fadd_rn(a.hi, a.lo); }

// split of a double into a df64 pair (host and device)
__host__ __device__ inline df df_from_d(double x) {
    const float hi = (float)x;
    return df{hi, (float)(x - (double)hi)};
}

}  // namespace f8
