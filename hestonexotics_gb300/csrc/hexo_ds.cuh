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
// x / y, y != 0: one float quotient, its remainder in double-single, one correction.
__device__ __forceinline__ F2 div(F2 x, F2 y) {
    const float r = __frcp_rn(y.h);
    const float q1 = __fmul_rn(x.h, r);
    const F2 rem = add(x, neg(mul_f(y, q1)));
    const float q2 = __fmul_rn(rem.h, r);
    return fast_two_sum(q1, q2);
}
// sqrt(x), x > 0: a float root and one Newton correction.
__device__ __forceinline__ F2 sqrt(F2 x) {
    const float rs = rsqrtf(x.h);
    const float s = __fmul_rn(x.h, rs);
    const F2 sq = sqr(F2{s, 0.0f});
    const F2 d = add(x, neg(sq));
    return fast_two_sum(s, __fmul_rn(__fmul_rn(d.h, 0.5f), rs));
}
// x < y
__device__ __forceinline__ bool less(F2 x, F2 y) { return x.h < y.h || (x.h == y.h && x.l < y.l); }

} // namespace ds
} // namespace hexo
