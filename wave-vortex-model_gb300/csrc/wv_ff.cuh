// Paired-FP32 ("float-float") arithmetic for the FP32X2 precision: a value is
// hi + lo, the low word carrying the rounding errors of the high word (a few
// ulp(hi) at most), about 45-48 significand bits, computed on the FP32 pipe
// (GB300 runs FP32 at 64x its FP64 rate).  The error-free
// transformations are the classic ones of Knuth (TAOCP vol. 2, 4.2.2, the
// two-sum) and of Dekker (1971, the exact product, here through a fused
// multiply-add).  Additions use the "sloppy" form (one two-sum on the high
// words, the low words added once): its error is bounded by a few units of
// 2^-48 times |x| + |y|, which is the absolute accuracy an FFT or a dot product
// needs.  Every operation is spelled with round-to-nearest intrinsics so that
// no contraction or reassociation can break an error-free step.
#pragma once

#include <cuda_runtime.h>

namespace wvgpu {
namespace dev {

struct __align__(8) ff {
    float hi, lo;
    ff() = default;
    __host__ __device__ constexpr ff(float h, float l) : hi(h), lo(l) {}
    __host__ __device__ ff(double v) : hi(static_cast<float>(v)), lo(static_cast<float>(v - static_cast<double>(static_cast<float>(v)))) {}
    __host__ __device__ ff(float v) : hi(v), lo(0.0f) {}
    __host__ __device__ ff(int v) : ff(static_cast<double>(v)) {}
    __host__ __device__ explicit operator double() const { return static_cast<double>(hi) + static_cast<double>(lo); }
    __host__ __device__ explicit operator float() const { return hi + lo; }
};

#ifdef __CUDACC__
// Sum and product keep the exact error of the high-word operation in the low
// word without renormalizing the pair: hi + lo stays the represented value,
// only |lo| may grow to a few units of ulp(hi) along a chain of operations,
// which costs a few bits of the ~48 and saves a third of the instructions.
// Nothing here relies on |lo| <= ulp(hi)/2 (no fast two-sum on operands).
__device__ __forceinline__ ff operator+(ff x, ff y) {
    const float s = __fadd_rn(x.hi, y.hi);
    const float bb = __fsub_rn(s, x.hi);
    const float e = __fadd_rn(__fsub_rn(x.hi, __fsub_rn(s, bb)), __fsub_rn(y.hi, bb));  // two-sum error
    return ff(s, __fadd_rn(__fadd_rn(x.lo, y.lo), e));
}
__device__ __forceinline__ ff operator-(ff x) { return ff(-x.hi, -x.lo); }
__device__ __forceinline__ ff operator-(ff x, ff y) { return x + (-y); }
__device__ __forceinline__ ff operator*(ff x, ff y) {
    const float p = __fmul_rn(x.hi, y.hi);
    float e = __fmaf_rn(x.hi, y.hi, -p);  // exact product error
    e = __fmaf_rn(x.hi, y.lo, e);
    e = __fmaf_rn(x.lo, y.hi, e);
    return ff(p, e);
}
__device__ __forceinline__ ff& operator+=(ff& x, ff y) { x = x + y; return x; }
__device__ __forceinline__ ff& operator-=(ff& x, ff y) { x = x - y; return x; }
__device__ __forceinline__ ff& operator*=(ff& x, ff y) { x = x * y; return x; }

struct __align__(16) ff2 {
    ff x, y;
};
#endif

}  // namespace dev
}  // namespace wvgpu
