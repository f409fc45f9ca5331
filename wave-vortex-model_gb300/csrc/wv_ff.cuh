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
    // constexpr so that literals (T(0.5), T(2), ...) fold at compile time instead
    // of running FP64 conversions in device code
    __host__ __device__ constexpr ff(double v)
        : hi(static_cast<float>(v)), lo(static_cast<float>(v - static_cast<double>(static_cast<float>(v)))) {}
    __host__ __device__ constexpr ff(float v) : hi(v), lo(0.0f) {}
    // integers without FP64: hi = v rounded to FP32, lo = the exact remainder
    __host__ __device__ constexpr ff(int v)
        : hi(static_cast<float>(v)),
          lo(static_cast<float>(static_cast<long long>(v) - static_cast<long long>(static_cast<float>(v)))) {}
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

// x 2^e for e in [-252, 254] by two exact multiplications by powers of two.
__device__ __forceinline__ float ff_scale_pow2(float x, int e) {
    const int h = e / 2;
    return __fmul_rn(__fmul_rn(x, __int_as_float((h + 127) << 23)), __int_as_float((e - h + 127) << 23));
}

// A double as an unevaluated pair with integer operations only (GB300 runs
// FP64 conversions at the FP64 rate): hi = the double truncated to 24
// significant bits, lo = the remaining 29 bits rounded to FP32 (pair error
// <= 2^-48 relative).  Zero and values outside the normal FP32 range take the
// FP64 conversion.
__device__ __forceinline__ ff ff_from_double(double v) {
    const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(v));
    const unsigned hw = static_cast<unsigned>(b >> 32), lw = static_cast<unsigned>(b);
    const int ex = static_cast<int>((hw >> 20) & 0x7FFu);
    const int fe = ex - 1023 + 127;
    if (fe <= 24 || fe >= 255) return ff(v);
    const unsigned sign = hw & 0x80000000u;
    const float hi = __uint_as_float(sign | (static_cast<unsigned>(fe) << 23) | ((hw & 0xFFFFFu) << 3) | (lw >> 29));
    const float lo = ff_scale_pow2(__uint2float_rn(lw & 0x1FFFFFFFu), ex - 1075);
    return ff(hi, sign ? -lo : lo);
}

// sin and cos of an FP64 angle as pairs, with six FP64 operations: the
// angle is reduced by the nearest multiple k of pi/2 (Cody and Waite: pi/2 as
// a double plus its remainder, two fused multiply-adds), and the reduced
// |r| <= pi/4 goes through the Taylor series of sin and cos to degree 15 and
// 14 in paired FP32 (truncation below 1e-15; coefficients (-1)^i/(2i+1)! and
// (-1)^i/(2i)! rounded to pairs), then the quadrant k mod 4 swaps and signs.
__device__ __forceinline__ void ff_sincos(double a, ff& s, ff& c) {
    const double k = rint(a * 0.63661977236758134308);
    double r = fma(-k, 1.5707963267948966192, a);
    r = fma(-k, 6.123233995736766036e-17, r);
    const int q = __double2int_rn(k) & 3;
    const ff x = ff_from_double(r);
    const ff z = x * x;
    ff ps = ff(-7.647163609812713e-13f, -1.2200710471178288e-20f);
    ps = ps * z + ff(1.6059044372074283e-10f, -5.352526511562726e-18f);
    ps = ps * z + ff(-2.5052107943679403e-08f, -4.4176230446483665e-16f);
    ps = ps * z + ff(2.7557318844628753e-06f, 3.793571224297229e-14f);
    ps = ps * z + ff(-0.00019841270113829523f, 2.725596874933456e-12f);
    ps = ps * z + ff(0.008333333767950535f, -4.34617203337595e-10f);
    ps = ps * z + ff(-0.1666666716337204f, 4.967053879312289e-09f);
    ps = ps * z + ff(1.0f, 0.0f);
    ff pc = ff(-1.147074536050896e-11f, -2.372207689231238e-19f);
    pc = pc * z + ff(2.0876755879584152e-09f, 1.1082839147459852e-16f);
    pc = pc * z + ff(-2.755731998149713e-07f, 7.575112209051195e-15f);
    pc = pc * z + ff(2.4801587642286904e-05f, -3.40699609366682e-13f);
    pc = pc * z + ff(-0.0013888889225199819f, 3.3631094437103215e-11f);
    pc = pc * z + ff(0.0416666679084301f, -1.2417634698280722e-09f);
    pc = pc * z + ff(-0.5f, 0.0f);
    pc = pc * z + ff(1.0f, 0.0f);
    const ff sn = x * ps;
    const ff cs = pc;
    // a = k pi/2 + r:  q = 0: (sin r, cos r); 1: (cos r, -sin r); 2: (-sin r, -cos r); 3: (-cos r, sin r)
    const ff s0 = (q & 1) ? cs : sn, c0 = (q & 1) ? sn : cs;
    s = (q & 2) ? -s0 : s0;
    c = ((q + 1) & 2) ? -c0 : c0;
}

// Paired FP32 in split form.  A complex paired value (re.hi, re.lo, im.hi,
// im.lo) is held as two float2: its high words (re.hi, im.hi) and its low
// words (re.lo, im.lo).  The real and the imaginary part then run every step
// of the pair arithmetic together on one paired FP32 instruction (FADD2 /
// FMUL2 / FFMA2, sm_100+), half the issue slots of the scalar form: a complex
// sum is 8 paired instructions instead of 16, a product by a twiddle 16 plus
// 4 register moves instead of 32.  Each component sees the scalar form's
// operations in the scalar form's order (sums as operator+, products of a
// value by a twiddle as operator* with the value on the left).

struct ffs {
    float2 h, l;
};
__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ float2 f2_sub(float2 a, float2 b) { return __ffma2_rn(b, f2(-1.0f, -1.0f), a); }
__device__ __forceinline__ ffs to_split(ff2 a) { return {f2(a.x.hi, a.y.hi), f2(a.x.lo, a.y.lo)}; }
__device__ __forceinline__ ff2 from_split(ffs a) {
    ff2 r;
    r.x = ff(a.h.x, a.l.x);
    r.y = ff(a.h.y, a.l.y);
    return r;
}
// x + y per component (operator+: two-sum of the high words, low words added once)
__device__ __forceinline__ ffs s_add(ffs x, ffs y) {
    const float2 s = __fadd2_rn(x.h, y.h);
    const float2 bb = f2_sub(s, x.h);
    const float2 e = __fadd2_rn(f2_sub(x.h, f2_sub(s, bb)), f2_sub(y.h, bb));
    return {s, __fadd2_rn(__fadd2_rn(x.l, y.l), e)};
}
// x - y per component as operator- (x + (-y)), with the negations folded
__device__ __forceinline__ ffs s_sub(ffs x, ffs y) {
    const float2 s = f2_sub(x.h, y.h);
    const float2 bb = f2_sub(s, x.h);
    const float2 e = f2_sub(f2_sub(x.h, f2_sub(s, bb)), __fadd2_rn(y.h, bb));
    return {s, __fadd2_rn(f2_sub(x.l, y.l), e)};
}
// s v + u, s = +1 or -1 (exact sign, then operator+)
__device__ __forceinline__ ffs s_sign_add(float sg, ffs v, ffs u) {
    const float2 g = f2(sg, sg);
    return s_add({__fmul2_rn(g, v.h), __fmul2_rn(g, v.l)}, u);
}
// x * y per component (operator*, x on the left)
__device__ __forceinline__ ffs s_mul(ffs x, ffs y) {
    const float2 p = __fmul2_rn(x.h, y.h);
    float2 e = __ffma2_rn(x.h, y.h, f2(-p.x, -p.y));
    e = __ffma2_rn(x.h, y.l, e);
    e = __ffma2_rn(x.l, y.h, e);
    return {p, e};
}
// A twiddle w ready for products: W = (w.re, w.im), Wp = (-w.im, w.re), split.
struct ffw {
    ffs W, Wp;
};
template <bool INV>
__device__ __forceinline__ ffw s_twiddle(const ff2* tw, int idx) {
    const ff2 w = tw[idx];
    const float si = INV ? -1.0f : 1.0f;  // the inverse transform takes conj(w)
    ffw t;
    t.W = {f2(w.x.hi, si * w.y.hi), f2(w.x.lo, si * w.y.lo)};
    t.Wp = {f2(-si * w.y.hi, w.x.hi), f2(-si * w.y.lo, w.x.lo)};
    return t;
}
__device__ __forceinline__ ffw s_unit() { return {{f2(1.0f, 0.0f), f2(0.0f, 0.0f)}, {f2(0.0f, 1.0f), f2(0.0f, 0.0f)}}; }
// a w as cmul(a, w): re = a.re w.re + (-(a.im w.im)), im = a.re w.im + a.im w.re
__device__ __forceinline__ ffs s_cmul(ffs a, const ffw& t) {
    const ffs re = {f2(a.h.x, a.h.x), f2(a.l.x, a.l.x)};
    const ffs im = {f2(a.h.y, a.h.y), f2(a.l.y, a.l.y)};
    return s_add(s_mul(re, t.W), s_mul(im, t.Wp));
}
// multiply by +i (INV) or -i (forward)
template <bool INV>
__device__ __forceinline__ ffs s_rot90(ffs b) {
    return INV ? ffs{f2(-b.h.y, b.h.x), f2(-b.l.y, b.l.x)} : ffs{f2(b.h.y, -b.h.x), f2(b.l.y, -b.l.x)};
}

// w v as cmul(w, v): the twiddle on the left of each product
__device__ __forceinline__ ffs s_cmul_left(const ffw& t, ffs v) {
    // re = w.re v.re + (-(w.im v.im)), im = w.re v.im + w.im v.re
    const ffs wre = {f2(t.W.h.x, t.W.h.x), f2(t.W.l.x, t.W.l.x)};
    const ffs wim = {f2(t.W.h.y, t.W.h.y), f2(t.W.l.y, t.W.l.y)};
    const ffs vsw = {f2(-v.h.y, v.h.x), f2(-v.l.y, v.l.x)};  // (-v.im, v.re)
    return s_add(s_mul(wre, v), s_mul(wim, vsw));
}

#endif

}  // namespace dev
}  // namespace wvgpu
