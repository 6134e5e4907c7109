// Price and standard error from exact limb sums.  Compiled both for the
// host (hexo_finalize_limbs, shard merges) and the device (finaliser
// kernel) with the same unfused IEEE operation sequence, so both produce
// identical bits.
#pragma once
#include <stdint.h>
#include <math.h>

#if defined(__CUDACC__)
#define HEXO_HD __host__ __device__ __forceinline__
#else
#define HEXO_HD inline
#endif

namespace hexo {

#if defined(__CUDA_ARCH__)
HEXO_HD double fadd(double a, double b) { return __dadd_rn(a, b); }
HEXO_HD double fsub(double a, double b) { return __dsub_rn(a, b); }
HEXO_HD double fmul(double a, double b) { return __dmul_rn(a, b); }
HEXO_HD double fdiv(double a, double b) { return __ddiv_rn(a, b); }
HEXO_HD double fsqr(double a) { return __dsqrt_rn(a); }
HEXO_HD double u64d(uint64_t a) { return __ull2double_rn(a); }
HEXO_HD double pow2(int k) { return __longlong_as_double((long long)(k + 1023) << 52); }
#else
HEXO_HD double fadd(double a, double b) { volatile double r = a + b; return r; }
HEXO_HD double fsub(double a, double b) { volatile double r = a - b; return r; }
HEXO_HD double fmul(double a, double b) { volatile double r = a * b; return r; }
HEXO_HD double fdiv(double a, double b) { volatile double r = a / b; return r; }
HEXO_HD double fsqr(double a) { return sqrt(a); }
HEXO_HD double u64d(uint64_t a) { return (double)a; }
HEXO_HD double pow2(int k) { return ldexp(1.0, k); }   // k in [-1022, 1023]: exact
#endif

// sum = l[0] + l[1] 2^25 + l[2] 2^50 (exact, 128-bit) converted to double.
HEXO_HD double limbs_to_double(uint64_t l0, uint64_t l1, uint64_t l2) {
    const unsigned __int128 s = (unsigned __int128)l0 + ((unsigned __int128)l1 << 25) + ((unsigned __int128)l2 << 50);
    const uint64_t hi = (uint64_t)(s >> 64), lo = (uint64_t)s;
    return fadd(fmul(u64d(hi), 18446744073709551616.0), u64d(lo));
}

// An exact 128-bit sum converted to double.
HEXO_HD double u128_to_double(unsigned __int128 s) {
    const uint64_t hi = (uint64_t)(s >> 64), lo = (uint64_t)s;
    return fadd(fmul(u64d(hi), 18446744073709551616.0), u64d(lo));
}

// Mean and (unbiased) variance of the payoffs behind six limb sums, whose
// values are y = pay 2^-E in fixed point (q = round(y 2^47), q2 =
// round(y^2 2^43)); biased sums (the control variate's signed differences)
// carry 2^63 per path in their first sum.  The scalings by powers of two are
// exact, so the result does not depend on where they are applied.
HEXO_HD void moments_limbs6(const uint64_t *l, uint64_t n_paths, bool biased, int E, double *mean, double *var) {
    const double n = u64d(n_paths);
    const unsigned __int128 u = (unsigned __int128)l[0] + ((unsigned __int128)l[1] << 25) + ((unsigned __int128)l[2] << 50);
    double s1;
    if (biased) {
        const __int128 v = (__int128)u - ((__int128)n_paths << 63);
        s1 = v < 0 ? -u128_to_double((unsigned __int128)(-v)) : u128_to_double((unsigned __int128)v);
    } else {
        s1 = u128_to_double(u);
    }
    const double s2 = limbs_to_double(l[3], l[4], l[5]);
    *mean = n_paths ? fdiv(fmul(s1, pow2(E - 47)), n) : 0.0;
    const double m2 = n_paths ? fdiv(fmul(s2, pow2(2 * E - 43)), n) : 0.0;
    double v = 0.0;
    if (n_paths > 1) v = fmul(fsub(m2, fmul(*mean, *mean)), fdiv(n, fsub(n, 1.0)));
    *var = v > 0.0 ? v : 0.0;
}

// The control-variate estimate of an Asian option from the sums of
// a = (A - K)^+, g = (G - K)^+ and d = a - g over the same paths:
// Cov(a, g) = (Var a + Var g - Var d) / 2, beta = Cov / Var g, price
// disc (mean a - beta (mean g - eg)), standard error that of a - beta g.
HEXO_HD void finalize_cv(const uint64_t *la, const uint64_t *lg, const uint64_t *ld, uint64_t n_paths, double disc,
                         int E, double eg, double *price, double *se) {
    double ma, va, mg, vg, md, vd;
    moments_limbs6(la, n_paths, false, E, &ma, &va);
    moments_limbs6(lg, n_paths, false, E, &mg, &vg);
    moments_limbs6(ld, n_paths, true, E, &md, &vd);
    double mean = ma, var = va;
    if (vg > 0.0) {
        const double cov = fmul(fsub(fadd(va, vg), vd), 0.5);
        mean = fsub(ma, fmul(fdiv(cov, vg), fsub(mg, eg)));
        var = fsub(va, fdiv(fmul(cov, cov), vg));
        if (!(var > 0.0)) var = 0.0;
    }
    *price = fmul(disc, mean);
    *se = n_paths ? fmul(disc, fsqr(fdiv(var, u64d(n_paths)))) : 0.0;
}

HEXO_HD void finalize_limbs6(const uint64_t *l, uint64_t n_paths, double disc, int E, double *price, double *se) {
    const double n = u64d(n_paths);
    const double s1 = limbs_to_double(l[0], l[1], l[2]);
    const double s2 = limbs_to_double(l[3], l[4], l[5]);
    const double mean = fdiv(fmul(s1, pow2(E - 47)), n);
    const double m2 = fdiv(fmul(s2, pow2(2 * E - 43)), n);
    double var = 0.0;
    if (n_paths > 1) var = fmul(fsub(m2, fmul(mean, mean)), fdiv(n, fsub(n, 1.0)));
    if (!(var > 0.0)) var = 0.0;
    *price = fmul(disc, mean);
    *se = fmul(disc, fsqr(fdiv(var, n)));
}

} // namespace hexo
