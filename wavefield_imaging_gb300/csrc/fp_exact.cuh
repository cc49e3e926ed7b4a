// FP32 helpers for the EXACT precision mode.
//
// The reference CPU update (ts_kernel.c:156, :306-307) is
//     u0 = 2.*u1 - u0 + vel*lap      (C: the `2.` literal makes it FP64)
// i.e. one rounding of the three-term sum 2*u1 - u0 + fl(vel*lap) to float.
// FP64 throughput on GB300 is a small fraction of FP32, so the exact path
// computes the correctly rounded sum of three floats in FP32 with the
// algorithm of Boldo & Melquiond ("Emulation of FMA and correctly rounded
// sums: proved algorithms using rounding to odd", IEEE TC 57(4), 2008):
//     (uh, ul) = TwoSum(b, c); (th, tl) = TwoSum(a, uh);
//     v = RO(tl + ul);  result = RN(th + v)
// where RO is rounding to odd, built here from TwoSum's error term.  It
// equals the reference's FP64 evaluation whenever that evaluation is exact
// before its final rounding, i.e. unless the three terms span more than 29
// binary orders of magnitude and the sum then lands within 2^-53 of a float
// rounding boundary.
#pragma once

namespace awe {

__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = __fadd_rn(a, b);
    float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// round-to-odd sum of two floats
__device__ __forceinline__ float add_ro(float a, float b) {
    float s, e;
    two_sum(a, b, s, e);
    unsigned bits = __float_as_uint(s);
    if (e != 0.f && (bits & 1u) == 0u) {
        // the exact sum lies strictly between s and its neighbour toward e;
        // that neighbour is the odd one
        bits += ((e > 0.f) == (s > 0.f)) ? 1u : 0xffffffffu;
    }
    return __uint_as_float(bits);
}

// round-to-nearest-even of a + b + c
__device__ __forceinline__ float sum3_rn(float a, float b, float c) {
    float uh, ul, th, tl;
    two_sum(b, c, uh, ul);
    two_sum(a, uh, th, tl);
    return __fadd_rn(th, add_ro(tl, ul));
}

template <bool EXACT>
__device__ __forceinline__ float fmul(float a, float b) {
    if constexpr (EXACT) return __fmul_rn(a, b);
    else return a * b;
}
template <bool EXACT>
__device__ __forceinline__ float fadd(float a, float b) {
    if constexpr (EXACT) return __fadd_rn(a, b);
    else return a + b;
}
template <bool EXACT>
__device__ __forceinline__ float fsub(float a, float b) {
    if constexpr (EXACT) return __fsub_rn(a, b);
    else return a - b;
}

}  // namespace awe
