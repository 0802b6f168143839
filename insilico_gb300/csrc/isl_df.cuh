// Double-float arithmetic: a value is the unevaluated sum hi + lo of two
// FP32 numbers with |lo| <= ulp(hi) / 2, about 48 significant bits.  GB300
// runs FP32 at about 64 times its FP64 rate, so element kernels that need
// FP64-level accuracy (entries within 1e-12 of an FP64 computation) compute
// in double-float on the FP32 pipe.  The building blocks are the classical
// error-free transformations: Knuth's TwoSum, Dekker's Fast2Sum, and the
// exact product error from a fused multiply-add.
#pragma once

#include <stdint.h>

namespace isl {

struct df {
    float hi, lo;
};

// a + b = s.hi + s.lo exactly (Knuth's TwoSum, no ordering assumption)
__device__ __forceinline__ df df_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return {s, e};
}

// a + b exactly when |a| >= |b| (Dekker's Fast2Sum)
__device__ __forceinline__ df df_fast_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ df df_make(float a) { return {a, 0.0f}; }

// the FP64 value's nearest double-float (two FP64 operations: set-up only)
__host__ __device__ inline df df_from_double(double x) {
    const float h = (float)x;
    return {h, (float)(x - (double)h)};
}

// product: hi*hi exactly split by an FMA, the cross terms added to the error
__device__ __forceinline__ df df_mul(df a, df b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, e));
    return df_fast_two_sum(p, e);
}

// sum with one TwoSum on the high parts (accurate unless a and b cancel
// almost completely; used inside short dot products)
__device__ __forceinline__ df df_add(df a, df b) {
    const df s = df_two_sum(a.hi, b.hi);
    return df_fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}

// sum with TwoSum on both parts (accurate under cancellation; used for
// accumulations across elements)
__device__ __forceinline__ df df_add_acc(df a, df b) {
    df s = df_two_sum(a.hi, b.hi);
    const df t = df_two_sum(a.lo, b.lo);
    s = df_fast_two_sum(s.hi, __fadd_rn(s.lo, t.hi));
    return df_fast_two_sum(s.hi, __fadd_rn(s.lo, t.lo));
}

__device__ __forceinline__ df df_fma(df a, df b, df c) { return df_add(df_mul(a, b), c); }

__device__ __forceinline__ df df_neg(df a) { return {-a.hi, -a.lo}; }

// IEEE binary32 -> binary64 by bit manipulation (exact; FP32 subnormals go
// to a signed zero, infinities and NaNs keep their class), so that the final
// FP64 value of a double-float costs one FP64 addition instead of two
// conversions and an addition on the FP64 pipe
__device__ __forceinline__ double f32_to_f64_bits(float f) {
    const uint32_t u = __float_as_uint(f);
    const uint64_t sign = (uint64_t)(u >> 31) << 63;
    const uint32_t ex = (u >> 23) & 0xFFu;
    const uint64_t man = (uint64_t)(u & 0x7FFFFFu) << 29;
    uint64_t bits;
    if (ex == 0) bits = sign;                                     // zero (and FP32 subnormals)
    else if (ex == 0xFFu) bits = sign | (0x7FFull << 52) | man;   // inf / NaN
    else bits = sign | ((uint64_t)(ex + 896u) << 52) | man;       // 896 = 1023 - 127
    return __longlong_as_double((long long)bits);
}

__device__ __forceinline__ double df_to_double(df a) { return __dadd_rn(f32_to_f64_bits(a.hi), f32_to_f64_bits(a.lo)); }

}  // namespace isl
