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

#include <stdint.h>

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

// N 2^-64 for an integer 0 < N < 2^64: the top 24 bits (exact) and the next
// 24 (rounded) of N.
__device__ __forceinline__ F2 from_u64_2m64(uint64_t N) {
    const uint32_t lz = (uint32_t)__clzll((long long)N);
    const uint64_t n = N << lz;                           // msb at bit 63
    const float sh = __uint_as_float((103u - lz) << 23);  // 2^(-24 - lz)
    const float sl = __uint_as_float((79u - lz) << 23);   // 2^(-48 - lz)
    const float h = __fmul_rn(__uint2float_rz((uint32_t)(n >> 40)), sh);
    const float l = __fmul_rn(__uint2float_rn((uint32_t)(n >> 16) & 0x00ffffffu), sl);
    return F2{h, l};
}

// Natural logarithm in double-single.  The
// reduction x = 2^k c_j (1 + r) with c_j = 1 + (j + 1/2)/128 from a table of
// 1/c_j and log c_j (double-single, built by log_table_init), |r| <= 2^-8,
// and log(1 + r) = r - r^2/2 + r^3/3 - r^4/4 + r^5/5 (the neglected terms are
// below 2^-50): the square in double-single, the rest in float.  About 2^-46
// absolute error for x near 1, relative beyond; x > 0 normal.
struct LogTab {
    float inv_h, inv_l, log_h, log_l;
};
constexpr uint32_t kLogTab = 128;

__device__ __forceinline__ void log_table_init(LogTab *t, uint32_t tid, uint32_t nthreads) {
    for (uint32_t j = tid; j < kLogTab; j += nthreads) {
        const double c = 1.0 + ((double)j + 0.5) / (double)kLogTab;
        const double ic = 1.0 / c, lc = ::log(c);
        const float ih = __double2float_rn(ic), lh = __double2float_rn(lc);
        t[j] = LogTab{ih, __double2float_rn(ic - (double)ih), lh, __double2float_rn(lc - (double)lh)};
    }
}

__device__ __forceinline__ F2 log(F2 x, const LogTab *t) {
    const uint32_t b = __float_as_uint(x.h);
    const int k = (int)(b >> 23) - 127;
    const uint32_t mb = (b & 0x007fffffu) | 0x3f800000u;
    const float M = __uint_as_float(mb);                                        // x.h 2^-k in [1, 2)
    const float ls = __fmul_rn(x.l, __uint_as_float((uint32_t)(127 - k) << 23));  // x.l 2^-k
    const uint32_t j = (mb >> 16) & (kLogTab - 1u);
    const float c = __uint_as_float(0x3f800000u | (j << 16) | (1u << 15));      // c_j
    const LogTab e = t[j];
    // r = ((M - c_j) + ls) / c_j: M - c_j is exact, ls below 2^-23 of M
    F2 r = mul_f(F2{e.inv_h, e.inv_l}, __fsub_rn(M, c));
    r.l = __fmaf_rn(ls, e.inv_h, r.l);
    const float p2 = __fmul_rn(r.h, r.h);
    const float e2 = __fmaf_rn(__fadd_rn(r.h, r.h), r.l, __fmaf_rn(r.h, r.h, -p2));
    float poly = __fmaf_rn(r.h, 0.2f, -0.25f);
    poly = __fmaf_rn(r.h, poly, 0x1.555556p-2f);
    poly = __fmul_rn(__fmul_rn(p2, r.h), poly);                                 // r^3/3 - r^4/4 + r^5/5
    // r - r^2/2 + poly, with |r^2/2| <= 2^-9 |r|: one ordered sum and the small terms
    const F2 s1 = fast_two_sum(r.h, __fmul_rn(-0.5f, p2));
    const F2 l1 = fast_two_sum(s1.h, __fadd_rn(__fadd_rn(s1.l, r.l), __fmaf_rn(-0.5f, e2, poly)));
    const F2 kl = mul_f(F2{0x1.62e430p-1f, -0x1.05c610p-29f}, (float)k);       // k ln 2
    return add(add(kl, F2{e.log_h, e.log_l}), l1);
}

} // namespace ds
} // namespace hexo
