// Double-single ("float-float") arithmetic: a value is hi + lo with two
// floats, about 48 significant bits, from FP32 operations only.  Built from
// the error-free transformations of T. J. Dekker, "A floating-point technique
// for extending the available precision" (Numer. Math. 18, 1971) and
// D. E. Knuth's TwoSum (TAOCP vol. 2), with the FMA form of TwoProduct.
//
// The FP32 form keeps the variance in this format: the QE scheme branches on
// Psi = s^2/m^2 < 1.5 (HSimulation.tpp:63), and a path whose float variance
// sits within float rounding of that threshold would take the other branch
// than the FP64 oracle, draw a uniform instead of a normal, and become a
// different path.  With ~48 bits the branch decisions agree with FP64.
// Every operation names its rounding, so results are the same in every
// template instantiation.
#pragma once

namespace hexo {
namespace ds {

struct F2 { float h, l; };

__device__ __forceinline__ F2 two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return {s, e};
}
// |a| >= |b| (or a == 0)
__device__ __forceinline__ F2 fast_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ F2 from(double x) {
    const float h = __double2float_rn(x);
    return {h, __double2float_rn(x - (double)h)};
}
__device__ __forceinline__ F2 add(F2 x, F2 y) {
    const F2 s = two_sum(x.h, y.h);
    return fast_two_sum(s.h, __fadd_rn(s.l, __fadd_rn(x.l, y.l)));
}
__device__ __forceinline__ F2 add_f(F2 x, float f) {
    const F2 s = two_sum(x.h, f);
    return fast_two_sum(s.h, __fadd_rn(s.l, x.l));
}
// |x| >= |y| known: one fast TwoSum instead of a full one
__device__ __forceinline__ F2 add_ordered(F2 x, F2 y) {
    const F2 s = fast_two_sum(x.h, y.h);
    return fast_two_sum(s.h, __fadd_rn(s.l, __fadd_rn(x.l, y.l)));
}
__device__ __forceinline__ F2 add_f_ordered(F2 x, float f) {
    const F2 s = fast_two_sum(x.h, f);
    return fast_two_sum(s.h, __fadd_rn(s.l, x.l));
}
__device__ __forceinline__ F2 neg(F2 x) { return {-x.h, -x.l}; }
__device__ __forceinline__ F2 mul(F2 x, F2 y) {
    const float p = __fmul_rn(x.h, y.h);
    float e = __fmaf_rn(x.h, y.h, -p);
    e = __fmaf_rn(x.h, y.l, e);
    e = __fmaf_rn(x.l, y.h, e);
    return fast_two_sum(p, e);
}
__device__ __forceinline__ F2 mul_f(F2 x, float f) {
    const float p = __fmul_rn(x.h, f);
    float e = __fmaf_rn(x.h, f, -p);
    e = __fmaf_rn(x.l, f, e);
    return fast_two_sum(p, e);
}
__device__ __forceinline__ F2 sqr(F2 x) {
    const float p = __fmul_rn(x.h, x.h);
    float e = __fmaf_rn(x.h, x.h, -p);
    e = __fmaf_rn(__fadd_rn(x.h, x.h), x.l, e);
    return fast_two_sum(p, e);
}
// Approximate MUFU reciprocal and reciprocal square root.  Each is a fixed
// function of its input, so results stay reproducible; the Newton-style
// corrections below bring the double-single results to full precision.
__device__ __forceinline__ float rcp_approx(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float rsqrt_approx(float x) {
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
// x * c + d
__device__ __forceinline__ F2 fma(F2 x, F2 c, F2 d) {
    const float p = __fmul_rn(x.h, c.h);
    float e = __fmaf_rn(x.h, c.h, -p);
    e = __fmaf_rn(x.h, c.l, e);
    e = __fmaf_rn(x.l, c.h, e);
    const F2 s = two_sum(p, d.h);
    return fast_two_sum(s.h, __fadd_rn(s.l, __fadd_rn(e, d.l)));
}
// x / y, y > 0 normal: a float quotient q1 from the approximate reciprocal,
// the remainder x - q1 y (its leading part exact by FMA), one correction.
__device__ __forceinline__ F2 div(F2 x, F2 y) {
    const float r = rcp_approx(y.h);
    const float q1 = __fmul_rn(x.h, r);
    float e = __fmaf_rn(-q1, y.h, x.h);
    e = __fadd_rn(e, x.l);
    e = __fmaf_rn(-q1, y.l, e);
    return fast_two_sum(q1, __fmul_rn(e, r));
}
// sqrt(x), x > 0 normal: a float root from the approximate reciprocal square
// root and one Newton correction with the exact residual x - s^2.
__device__ __forceinline__ F2 sqrt(F2 x) {
    const float rs = rsqrt_approx(x.h);
    const float s = __fmul_rn(x.h, rs);
    float e = __fmaf_rn(-s, s, x.h);
    e = __fadd_rn(e, x.l);
    return fast_two_sum(s, __fmul_rn(e, __fmul_rn(0.5f, rs)));
}
// x < y
__device__ __forceinline__ bool less(F2 x, F2 y) { return x.h < y.h || (x.h == y.h && x.l < y.l); }

} // namespace ds
} // namespace hexo
