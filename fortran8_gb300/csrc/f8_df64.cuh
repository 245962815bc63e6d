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

// Two independent df64 values in the lanes of FP32x2 registers, for the
// packed FP32 instructions of sm_100 and later.  Each lane performs the
// operations of the scalar routine of the same name in the same order with
// the same rounding (a - b is a + (-b) exactly), so a lane's result is
// bit-identical to the scalar one.
struct df2 {
    float2 hi, lo;
};

__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 add2_rn(float2 a, float2 b) { return __fadd2_rn(a, b); }
// a - b as one packed FMA: b * (-1) is exact, so the result is a - b rounded
// once, as __fsub_rn gives it (the sign of a zero result included)
__device__ __forceinline__ float2 sub2_rn(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.0f, -1.0f), a); }

__device__ __forceinline__ void two_sum2(float2 a, float2 b, float2 &s, float2 &e) {
    s = add2_rn(a, b);
    const float2 bb = sub2_rn(s, a);
    e = add2_rn(sub2_rn(a, sub2_rn(s, bb)), sub2_rn(b, bb));
}

__device__ __forceinline__ void fast_two_sum2(float2 a, float2 b, float2 &s, float2 &e) {
    s = add2_rn(a, b);
    e = sub2_rn(b, sub2_rn(s, a));
}

__device__ __forceinline__ df2 df2_pack(df a, df b) {
    return df2{make_float2(a.hi, b.hi), make_float2(a.lo, b.lo)};
}
__device__ __forceinline__ df df2_x(df2 a) { return df{a.hi.x, a.lo.x}; }
__device__ __forceinline__ df df2_y(df2 a) { return df{a.hi.y, a.lo.y}; }

__device__ __forceinline__ df2 df2_add(df2 a, df2 b) {
    float2 s, e;
    two_sum2(a.hi, b.hi, s, e);
    e = add2_rn(e, add2_rn(a.lo, b.lo));
    df2 r;
    fast_two_sum2(s, e, r.hi, r.lo);
    return r;
}

__device__ __forceinline__ df2 df2_neg(df2 a) { return df2{neg2(a.hi), neg2(a.lo)}; }

// a - b: df2_add(a, -b) with each addition of a negated operand written as
// the subtraction (exactly the same roundings)
__device__ __forceinline__ df2 df2_sub(df2 a, df2 b) {
    const float2 s = sub2_rn(a.hi, b.hi);
    const float2 bb = sub2_rn(s, a.hi);
    float2 e = sub2_rn(sub2_rn(a.hi, sub2_rn(s, bb)), add2_rn(b.hi, bb));
    e = add2_rn(e, sub2_rn(a.lo, b.lo));
    df2 r;
    fast_two_sum2(s, e, r.hi, r.lo);
    return r;
}

// a + b, b a float pair
__device__ __forceinline__ df2 df2_add_f(df2 a, float2 b) {
    float2 s, e;
    two_sum2(a.hi, b, s, e);
    e = add2_rn(e, a.lo);
    df2 r;
    fast_two_sum2(s, e, r.hi, r.lo);
    return r;
}

// a - b for float pairs, exact
__device__ __forceinline__ df2 df2_diff_ff(float2 a, float2 b) {
    // two_sum2(a, -b) with the additions of -b written as subtractions
    df2 r;
    r.hi = sub2_rn(a, b);
    const float2 bb = sub2_rn(r.hi, a);
    r.lo = sub2_rn(sub2_rn(a, sub2_rn(r.hi, bb)), add2_rn(b, bb));
    return r;
}

__device__ __forceinline__ df2 df2_mul(df2 a, df2 b) {
    const float2 p = __fmul2_rn(a.hi, b.hi);
    float2 e = __ffma2_rn(a.hi, b.hi, neg2(p));
    e = __ffma2_rn(a.hi, b.lo, e);
    e = __ffma2_rn(a.lo, b.hi, e);
    df2 r;
    fast_two_sum2(p, e, r.hi, r.lo);
    return r;
}

// split of a double into a df64 pair (host and device)
__host__ __device__ inline df df_from_d(double x) {
    const float hi = (float)x;
    return df{hi, (float)(x - (double)hi)};
}

}  // namespace f8
