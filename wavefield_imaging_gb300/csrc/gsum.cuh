// Gradient / image accumulator of the adjoint kernels: one compensated FP32
// pair per cell (Kahan summation, "Further remarks on reducing truncation
// errors", CACM 8(1), 1965).  .x is the running sum, .y the negated low part
// that the last additions lost; the value is x - y, formed in FP64 only when
// the gradient is folded to the model grid.  Its error is bounded by about
// 2 u32 * sum |terms| whatever the number of time steps, so it stands in for
// an FP64 sum at 8 bytes per cell and without FP64 instructions (GB300 runs
// FP64 at a small fraction of its FP32 rate).
#pragma once

namespace awe {

__device__ __forceinline__ float2 gsum_add(float2 a, float x) {
    const float y = __fsub_rn(x, a.y);
    const float t = __fadd_rn(a.x, y);
    a.y = __fsub_rn(__fsub_rn(t, a.x), y);
    a.x = t;
    return a;
}

// adds u * v exactly: the rounded product and its rounding error (an FMA)
__device__ __forceinline__ float2 gsum_add_prod(float2 a, float u, float v) {
    const float p = __fmul_rn(u, v);
    const float e = __fmaf_rn(u, v, -p);
    return gsum_add(gsum_add(a, p), e);
}

__device__ __forceinline__ double gsum_value(float2 a) { return (double)a.x - (double)a.y; }

}  // namespace awe
