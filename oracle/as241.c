/*
 * ORACLE / TEST INFRASTRUCTURE ONLY.  Nothing in the product links this file.
 *
 * C restatement of the reference's AS241 inverse normal, src/as241.f90:15-119
 * (`PPND16`, bound to C as `double ppnd16(double*, int*)`, declared by the
 * reference at src/RNG.cpp:6).  There is no Fortran compiler in this image, so
 * the Fortran is restated with its exact arithmetic:
 *
 *   - every constant and the locals Q, R are default REAL (as241.f90:20-25),
 *     i.e. IEEE binary32; each PARAMETER is a double literal (…D0) rounded to
 *     float, so the constants below are written `(float)<double literal>`;
 *   - `Q = P - HALF` subtracts in double (P is C_DOUBLE) and rounds to float
 *     on assignment (as241.f90:86);
 *   - `R = ONE - P` likewise subtracts in double and rounds to float (:97);
 *   - every other operation is a separate float multiply / add / divide:
 *     the reference compiles this file with autoconf's default FCFLAGS
 *     (`-g -O2`, no -march, configure.ac:13), so no FMA contraction happens;
 *     this file must be compiled with -ffp-contract=off;
 *   - `SQRT` is IEEE sqrtf; `LOG` of a REAL is a float logarithm.  The
 *     reference gets it from the C library, whose result is not specified to
 *     the bit, so this restatement fixes it to `oracle_logf` below (a
 *     deterministic float logarithm written for this project: Cody & Waite
 *     argument reduction, then log(m) = 2*atanh(s), s = (m-1)/(m+1), summed
 *     as an odd series to s^11 with explicit fmaf).  The GPU evaluates the
 *     same operation sequence, so normals agree bit for bit; the test suite
 *     also measures how far oracle_logf is from the C library's logf.
 *
 * IFAULT=1 with result 0 when R <= 0 (as241.f90:99-102), i.e. P == 0 or
 * P == 1.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

#if defined(__FAST_MATH__)
#error "as241.c must not be compiled with -ffast-math"
#endif

#define F32(x) ((float)(x))

/* as241.f90:26-27 */
static const float SPLIT1 = F32(0.425), SPLIT2 = F32(5.0), CONST1 = F32(0.180625), CONST2 = F32(1.6);
/* as241.f90:31-44 */
static const float A0 = F32(3.3871328727963666080), A1 = F32(1.3314166789178437745e+2),
                   A2 = F32(1.9715909503065514427e+3), A3 = F32(1.3731693765509461125e+4),
                   A4 = F32(4.5921953931549871457e+4), A5 = F32(6.7265770927008700853e+4),
                   A6 = F32(3.3430575583588128105e+4), A7 = F32(2.5090809287301226727e+3),
                   B1 = F32(4.2313330701600911252e+1), B2 = F32(6.8718700749205790830e+2),
                   B3 = F32(5.3941960214247511077e+3), B4 = F32(2.1213794301586595867e+4),
                   B5 = F32(3.9307895800092710610e+4), B6 = F32(2.8729085735721942674e+4),
                   B7 = F32(5.2264952788528545610e+3);
/* as241.f90:49-63 */
static const float C0 = F32(1.42343711074968357734), C1 = F32(4.63033784615654529590),
                   C2 = F32(5.76949722146069140550), C3 = F32(3.64784832476320460504),
                   C4 = F32(1.27045825245236838258), C5 = F32(2.41780725177450611770e-1),
                   C6 = F32(2.27238449892691845833e-2), C7 = F32(7.74545014278341407640e-4),
                   D1 = F32(2.05319162663775882187), D2 = F32(1.67638483018380384940),
                   D3 = F32(6.89767334985100004550e-1), D4 = F32(1.48103976427480074590e-1),
                   D5 = F32(1.51986665636164571966e-2), D6 = F32(5.47593808499534494600e-4),
                   D7 = F32(1.05075007164441684324e-9);
/* as241.f90:68-82 */
static const float E0 = F32(6.65790464350110377720), E1 = F32(5.46378491116411436990),
                   E2 = F32(1.78482653991729133580), E3 = F32(2.96560571828504891230e-1),
                   E4 = F32(2.65321895265761230930e-2), E5 = F32(1.24266094738807843860e-3),
                   E6 = F32(2.71155556874348757815e-5), E7 = F32(2.01033439929228813265e-7),
                   F1 = F32(5.99832206555887937690e-1), F2 = F32(1.36929880922735805310e-1),
                   F3 = F32(1.48753612908506148525e-2), F4 = F32(7.86869131145613259100e-4),
                   F5 = F32(1.84631831751005468180e-5), F6 = F32(1.42151175831644588870e-7),
                   F7 = F32(2.04426310338993978564e-15);

/*
 * Deterministic float logarithm for x > 0 (finite).  Written from the
 * textbook method (W. J. Cody & W. Waite, "Software Manual for the Elementary
 * Functions", 1980): x = 2^k * m with m in [sqrt(1/2), sqrt(2)),
 * log(m) = 2*atanh(s) with s = (m-1)/(m+1), k*ln2 split into an exact high
 * part and a small low part.  Every step is one IEEE float operation or an
 * explicit fmaf, so any IEEE-conforming machine returns the same bits.
 */
float oracle_logf(float x)
{
    const float LN2_HI = 0x1.62e4p-1f;     /* 0x3f317200: 16 trailing zero bits */
    const float LN2_LO = 0x1.7f7d1cp-20f;  /* ln2 - LN2_HI, rounded to float */
    /* 2/3, 2/5, 2/7, 2/9, 2/11 rounded to float */
    const float c3 = 0x1.555556p-1f, c5 = 0x1.99999ap-2f, c7 = 0x1.24924ap-2f, c9 = 0x1.c71c72p-3f,
                c11 = 0x1.745d18p-3f;
    uint32_t bits;
    int k = 0;
    if (x < 1.17549435e-38f) { /* subnormal: scale into the normal range */
        x = x * 8388608.0f;   /* 2^23, exact */
        k = -23;
    }
    memcpy(&bits, &x, 4);
    k += (int)(bits >> 23) - 127;
    bits = (bits & 0x007fffffu) | 0x3f800000u; /* m in [1, 2) */
    if (bits > 0x3fb504f3u) {                  /* m > sqrt(2): halve it */
        bits -= 0x00800000u;
        k += 1;
    }
    float m;
    memcpy(&m, &bits, 4);
    float f = m - 1.0f;          /* exact */
    float s = f / (2.0f + f);
    float z = s * s;
    float p = fmaf(z, c11, c9);
    p = fmaf(z, p, c7);
    p = fmaf(z, p, c5);
    p = fmaf(z, p, c3);
    p = p * z;
    float two_s = s + s;         /* exact */
    float log_m = fmaf(s, p, two_s);
    float kf = (float)k;         /* exact */
    return fmaf(kf, LN2_HI, fmaf(kf, LN2_LO, log_m));
}

/* Float32 AS241 on a double probability; the restated body of PPND16. */
double ppnd16(double *P_in, int *IFAULT)
{
    const double P = *P_in;
    float Q, R, val;
    *IFAULT = 0;
    Q = (float)(P - 0.5);                              /* as241.f90:86 */
    if (fabsf(Q) <= SPLIT1) {                          /* :88 */
        R = CONST1 - Q * Q;                            /* :89 */
        float num = ((((((A7 * R + A6) * R + A5) * R + A4) * R + A3) * R + A2) * R + A1) * R + A0;
        float den = ((((((B7 * R + B6) * R + B5) * R + B4) * R + B3) * R + B2) * R + B1) * R + 1.0f;
        val = (Q * num) / den;                         /* :90-91 */
        return (double)val;
    }
    if (Q < 0.0f) R = (float)P;                        /* :94-98 */
    else R = (float)(1.0 - P);
    if (R <= 0.0f) {                                   /* :99-102 */
        *IFAULT = 1;
        return 0.0;
    }
    R = sqrtf(-oracle_logf(R));                        /* :104 */
    if (R <= SPLIT2) {                                 /* :105-109 */
        R = R - CONST2;
        float num = ((((((C7 * R + C6) * R + C5) * R + C4) * R + C3) * R + C2) * R + C1) * R + C0;
        float den = ((((((D7 * R + D6) * R + D5) * R + D4) * R + D3) * R + D2) * R + D1) * R + 1.0f;
        val = num / den;
    } else {                                           /* :110-114 */
        R = R - SPLIT2;
        float num = ((((((E7 * R + E6) * R + E5) * R + E4) * R + E3) * R + E2) * R + E1) * R + E0;
        float den = ((((((F7 * R + F6) * R + F5) * R + F4) * R + F3) * R + F2) * R + F1) * R + 1.0f;
        val = num / den;
    }
    double out = (double)val;
    if (Q < 0.0f) out = -out;                          /* :116 */
    return out;
}
