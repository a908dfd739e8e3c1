// Double-float arithmetic: a real number as the unevaluated sum hi + lo of
// two FP32 numbers with |lo| <= ulp(hi) / 2, about 48 significant bits, on
// the FP32 pipes.  GB300 issues FP64 at 1/64 of the FP32 rate, so the Wilson
// operator in this form runs at several times its FP64 speed, with a
// rounding error of order 2^-46 of the terms summed (FP64: 2^-53) and FP32's
// exponent range.
//
// Error-free transformations used (published algorithms, written here from
// their definitions): Knuth's TwoSum (s + e = a + b exactly, no ordering
// condition), Dekker's Fast2Sum (the same for |a| >= |b|) and TwoProduct by
// one FMA (p + e = a * b exactly).  Sums and products follow Dekker (1971):
// the low parts are added once, without a second error-free step
// ("sloppy" addition), which bounds the error relative to |a| + |b|.
// The _rn intrinsics keep the compiler from contracting or reordering the
// steps.
#pragma once

#include <cuda_runtime.h>

namespace gbds {

// The constructors are explicit: generic kernel code calls fma() and the
// arithmetic operators unqualified inside namespace gbds, and an implicit
// float -> dfloat conversion could turn FP32 or FP64 calls into double-float
// ones.  ::fma stays visible next to the dfloat overload.
using ::fma;

struct dfloat {
    float hi, lo;
    __host__ __device__ constexpr dfloat() : hi(0.f), lo(0.f) {}
    __host__ __device__ constexpr explicit dfloat(float h) : hi(h), lo(0.f) {}  // T(0), T(2)
    __host__ __device__ constexpr dfloat(float h, float l) : hi(h), lo(l) {}
};

// s + e = a + b exactly (Knuth)
__device__ __forceinline__ dfloat df_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return {s, e};
}

// s + e = a + b exactly when |a| >= |b| or a == 0 (Dekker)
__device__ __forceinline__ dfloat df_fast_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ dfloat operator-(dfloat a) { return {-a.hi, -a.lo}; }

__device__ __forceinline__ dfloat operator+(dfloat a, dfloat b) {
    const dfloat s = df_two_sum(a.hi, b.hi);
    return df_fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}

__device__ __forceinline__ dfloat operator-(dfloat a, dfloat b) { return a + (-b); }

// the low-order cross terms of the product enter the FMA chain of the exact
// high product's error; lo * lo (below 2^-48 of the result) is dropped
__device__ __forceinline__ float df_prod_err(dfloat a, dfloat b, float p) {
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    return __fmaf_rn(a.lo, b.hi, e);
}

__device__ __forceinline__ dfloat operator*(dfloat a, dfloat b) {
    const float p = __fmul_rn(a.hi, b.hi);
    return df_fast_two_sum(p, df_prod_err(a, b, p));
}

// a * b + c with one rounding of the double-float product's parts
__device__ __forceinline__ dfloat fma(dfloat a, dfloat b, dfloat c) {
    const float p = __fmul_rn(a.hi, b.hi);
    const float e = df_prod_err(a, b, p);
    const dfloat s = df_two_sum(p, c.hi);
    return df_fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(e, c.lo)));
}

// FP64 <-> double-float, one complex (double2 <-> float4 re.hi, re.lo, im.hi,
// im.lo): the same 16 bytes, so a field keeps the FP64 layout's size and
// indexing.  d -> hi + lo keeps 48 of d's 53 significant bits; hi + lo -> d
// is exact.
__device__ __forceinline__ float4 df_from_double2(double2 d) {
    const float rh = __double2float_rn(d.x), ih = __double2float_rn(d.y);
    return make_float4(rh, __double2float_rn(d.x - (double)rh), ih, __double2float_rn(d.y - (double)ih));
}

__device__ __forceinline__ double2 df_to_double2(float4 f) {
    return make_double2((double)f.x + (double)f.y, (double)f.z + (double)f.w);
}

}  // namespace gbds
