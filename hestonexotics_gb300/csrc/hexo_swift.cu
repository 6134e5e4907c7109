// SWIFT European call pricer on the GPU: prices and their gradients in the
// Heston parameters, for batches of option chains.
//
// The reference prices European calls with the SWIFT method (Ortiz-Gracia &
// Oosterlee, SIAM J. Sci. Comput. 38, 2016) in src/SWIFT.cpp:18-118, using the
// characteristic function and gradient of src/HDistribution.cpp:8-113 (the
// form of Cui, del Bano Rollin & Germano, EJOR 263, 2017); its calibration
// evaluates them for every chain at every Levenberg-Marquardt step
// (src/HCalibration.cpp:35-57).  Per expiry, with J frequencies
// u_j = pi (2j+1) 2^m / (2J) and k in [k1, k2]:
//   h_j  = H(upper) - H(max(lower, 0)),  H(y) = -i e^{-i u_j y} (1/u_j - e^y/(i + u_j))
//   V_k  = Re(sum_j h_j w^{k(2j+1)}) sqrt(2^m) / J                 (SWIFT.cpp:54-68)
//   c_j  = sum_k V_k w^{k(2j+1)} sqrt(2^m) / J                      (SWIFT.cpp:69-72)
//   price_i (and gradient) = Re sum_j phi(u_j) c_j disc K_i e^{-i u_j x_i}  (SWIFT.cpp:102-118)
// with w = e^{i pi / (2J)} and x_i = r tau + log(S / K_i).  The reference
// evaluates the two transforms with FFTW; here they are direct sums (the same
// sums), spread one warp per 32 outputs over the whole GPU.  Everything is
// FP64: the work per call is small and the results must match the
// reference's known answers to 1e-9.
#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "hexo_mc.h"
#include "hexo_runtime.h"

namespace hexo {
namespace swift {

// ---------------------------------------------------------------- complex

struct cplx {
    double re, im;
};
__host__ __device__ inline cplx C(double r, double i = 0.0) { return cplx{r, i}; }
__host__ __device__ inline cplx operator+(cplx a, cplx b) { return C(a.re + b.re, a.im + b.im); }
__host__ __device__ inline cplx operator-(cplx a, cplx b) { return C(a.re - b.re, a.im - b.im); }
__host__ __device__ inline cplx operator-(cplx a) { return C(-a.re, -a.im); }
__host__ __device__ inline cplx operator*(cplx a, cplx b) {
    return C(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
__host__ __device__ inline cplx operator*(double s, cplx a) { return C(s * a.re, s * a.im); }
__host__ __device__ inline cplx operator*(cplx a, double s) { return C(s * a.re, s * a.im); }
__host__ __device__ inline cplx operator+(cplx a, double s) { return C(a.re + s, a.im); }
__host__ __device__ inline cplx operator+(double s, cplx a) { return C(a.re + s, a.im); }
__host__ __device__ inline cplx operator-(double s, cplx a) { return C(s - a.re, -a.im); }
__host__ __device__ inline cplx operator-(cplx a, double s) { return C(a.re - s, a.im); }
// a / b by Smith's method (scaled, no overflow for the magnitudes met here)
__host__ __device__ inline cplx operator/(cplx a, cplx b) {
    if (fabs(b.re) >= fabs(b.im)) {
        const double t = b.im / b.re, d = b.re + b.im * t;
        return C((a.re + a.im * t) / d, (a.im - a.re * t) / d);
    }
    const double t = b.re / b.im, d = b.re * t + b.im;
    return C((a.re * t + a.im) / d, (a.im * t - a.re) / d);
}
__host__ __device__ inline cplx operator/(cplx a, double s) { return C(a.re / s, a.im / s); }
__host__ __device__ inline cplx operator/(double s, cplx b) { return C(s) / b; }
__host__ __device__ inline double cabs_(cplx a) { return hypot(a.re, a.im); }
__host__ __device__ inline cplx cexp_(cplx a) {
    const double e = exp(a.re);
    return C(e * cos(a.im), e * sin(a.im));
}
// principal logarithm
__host__ __device__ inline cplx clog_(cplx a) { return C(log(cabs_(a)), atan2(a.im, a.re)); }
// principal square root
__host__ __device__ inline cplx csqrt_(cplx a) {
    const double r = cabs_(a);
    if (r == 0.0) return C(0.0, a.im);
    if (a.re >= 0.0) {
        const double t = sqrt(0.5 * (r + a.re));
        return C(t, a.im / (2.0 * t));
    }
    const double t = sqrt(0.5 * (r - a.re));
    return C(fabs(a.im) / (2.0 * t), copysign(t, a.im));
}
__host__ __device__ inline cplx csinh_(cplx a) { return C(sinh(a.re) * cos(a.im), cosh(a.re) * sin(a.im)); }
__host__ __device__ inline cplx ccosh_(cplx a) { return C(cosh(a.re) * cos(a.im), sinh(a.re) * sin(a.im)); }

// ------------------------------------------------ characteristic function

struct HP {
    double v0, vm, rho, kappa, sigma;
};

// Helper quantities of one frequency (HDistribution.cpp:13-26).
struct Aux {
    cplx xi, d, A1, A2, A, B, D, sh, ch;
    double ekt;
};

__host__ __device__ inline Aux aux(const HP &p, cplx u, double tau) {
    const cplx I = C(0.0, 1.0);
    Aux a;
    a.xi = p.kappa + p.sigma * p.rho * (I * u);
    const cplx f = u * u - I * u;
    a.d = csqrt_(a.xi * a.xi + p.sigma * p.sigma * f);
    a.sh = csinh_(a.d * (tau * 0.5));
    a.ch = ccosh_(a.d * (tau * 0.5));
    a.A1 = f * a.sh;
    a.A2 = a.d / p.v0 * a.ch + a.xi / p.v0 * a.sh;
    a.A = a.A1 / a.A2;
    a.ekt = exp(p.kappa * tau * 0.5);
    a.B = a.d * a.ekt / (p.v0 * a.A2);
    a.D = clog_((2.0 * a.d) / (a.d + a.xi + (a.d - a.xi) * cexp_(-(a.d * tau)))) + (p.kappa - a.d) * (tau * 0.5);
    return a;
}

// phi(u) of the log-return without drift (HDistribution.cpp:31-37)
__host__ __device__ inline cplx chf(const HP &p, double tau, cplx u, const Aux &a) {
    const cplx I = C(0.0, 1.0);
    return cexp_((p.kappa * p.vm * p.rho * tau) * (u * I) / p.sigma - a.A + (2.0 * p.kappa * p.vm) * a.D / (p.sigma * p.sigma));
}

// phi and its partial derivatives in (v0, vm, rho, kappa, sigma) (HDistribution.cpp:48-84)
__host__ __device__ inline void chf_grad(const HP &p, double tau, cplx u, cplx out[6]) {
    const cplx I = C(0.0, 1.0);
    const Aux a = aux(p, u, tau);
    const cplx c = chf(p, tau, u, a);
    const cplx iu = I * u;
    const cplx d_rho = a.xi * p.sigma * iu / a.d;
    const cplx A2_rho = p.sigma * iu * (2.0 + a.xi * tau) / (2.0 * a.d * p.v0) * (a.xi * a.ch + a.d * a.sh);
    const cplx B_rho = a.ekt / p.v0 * (d_rho / a.A2 - a.d / (a.A2 * a.A2) * A2_rho);
    const cplx A1_rho = (iu * (u * u - iu) * tau * a.xi * p.sigma) / (2.0 * a.d) * a.ch;
    const cplx A_rho = A1_rho / a.A2 - a.A / a.A2 * A2_rho;
    const cplx B_kappa = -I / (p.sigma * u) * B_rho + a.B * (tau * 0.5);
    const cplx d_sigma = (p.rho / p.sigma - 1.0 / a.xi) * d_rho + p.sigma * u * u / a.d;
    const cplx A1_sigma = (u * u - iu) * (0.5 * tau) * d_sigma * a.ch;
    const cplx A2_sigma = p.rho / p.sigma * A2_rho + (2.0 + tau * a.xi) / (p.v0 * tau * a.xi * iu) * A1_rho +
                          p.sigma * tau * a.A1 / p.v0 * 0.5;
    const cplx A_sigma = A1_sigma / a.A2 - a.A / a.A2 * A2_sigma;
    const cplx t_iu_vm_s = p.vm * tau * iu / p.sigma;
    const double s2 = p.sigma * p.sigma;
    const double k2 = 2.0 * p.kappa * p.vm / s2;
    const cplx g_v0 = -a.A / p.v0;
    const cplx g_vm = 2.0 * p.kappa / s2 * a.D + p.kappa * p.rho * tau * iu / p.sigma;
    const cplx g_sigma = -A_sigma - 2.0 * k2 / p.sigma * a.D + k2 / a.d * (d_sigma - a.d / a.A2 * A2_sigma) -
                         t_iu_vm_s / p.sigma * p.rho * p.kappa;
    const cplx g_kappa = -A_rho / (p.sigma * iu) + 2.0 * p.vm / s2 * a.D + k2 / a.B * B_kappa + t_iu_vm_s * p.rho;
    const cplx g_rho = -A_rho + k2 / a.d * (d_rho - a.d / a.A2 * A2_rho) + t_iu_vm_s * p.kappa;
    out[0] = c;
    out[1] = c * g_v0;
    out[2] = c * g_vm;
    out[3] = c * g_rho;
    out[4] = c * g_kappa;
    out[5] = c * g_sigma;
}

// ------------------------------------------------ dynamic wavelet parameters

double int_error(const HP &p, double tau, unsigned m) {   // HDistribution.cpp:8-11
    const double e = std::exp2((double)m);
    const cplx u1 = C(e * M_PI), u2 = C(-e * M_PI);
    return cabs_(chf(p, tau, u1, aux(p, u1, tau)) + chf(p, tau, u2, aux(p, u2, tau))) / (4.0 * e * M_PI * M_PI * tau);
}

// Cumulants (HDistribution.cpp:86-113).  The reference binds its parameter
// struct positionally as (v, s2, r, kappa, k) = (v0, vm, rho, kappa, sigma),
// so in these formulas "s2" is vm and "r" is rho.
double cum1(const HP &p, double tau) { return -0.5 * p.vm * tau; }
double cum2(const HP &p, double t) {
    const double s2 = p.vm, r = p.rho, kap = p.kappa, k = p.sigma;
    const double kap2 = kap * kap, kap3 = kap2 * kap, k2 = k * k;
    return s2 / (8 * kap3) *
           (-k2 * std::exp(-2 * kap * t) + 4 * k * std::exp(-kap * t) * (k - 2 * kap * r) +
            2 * kap * t * (4 * kap2 + k2 - 4 * kap * k * r) + k * (8 * kap * r - 3 * k));
}
double cum4(const HP &p, double t) {
    const double s2 = p.vm, r = p.rho, a = p.kappa, k = p.sigma;
    const double a2 = a * a, a3 = a2 * a, a4 = a3 * a, k2 = k * k, k3 = k2 * k, k4 = k3 * k;
    const double t2 = t * t, r2 = r * r, km = k - 2 * a * r;
    return (3 * k2 * s2) / (64 * std::pow(a, 7)) *
           (-3 * k4 * std::exp(-4 * a * t)
            - 8 * k2 * std::exp(-3 * a * t) * (2 * a * k * t * km + 4 * a2 + k2 - 6 * a * k * r)
            - 4 * std::exp(-2 * a * t) *
                  (4 * a2 * k2 * t2 * km * km +
                   2 * a * k * t * (k3 - 16 * a3 * r - 12 * a * k2 * r + 4 * a2 * k * (3 + 4 * r2)) + 8 * a4 -
                   3 * k4 - 32 * a3 * k * r + 8 * a * k3 * r + 16 * a2 * k2 * r2)
            - 8 * std::exp(-a * t) *
                  (-2 * a2 * k * t2 * km * km * km -
                   8 * a * t * (k4 - 7 * a * k3 * r + 4 * a4 * r2 - 8 * a3 * k * r * (1 + r2) + a2 * k2 * (3 + 14 * r2)) -
                   9 * k4 + 70 * a * k3 * r + 32 * a3 * k * r * (4 + 3 * r2) - 16 * a4 * (1 + 4 * r2) -
                   4 * a2 * k2 * (9 + 40 * r2))
            + 4 * a * t *
                  (5 * k4 - 40 * a * k3 * r - 32 * a3 * k * r * (3 + 2 * r2) + 16 * a4 * (1 + 4 * r2) +
                   24 * a2 * k2 * (1 + 4 * r2))
            - 73 * k4 + 544 * a * k3 * r + 128 * a3 * k * r * (7 + 6 * r2) - 32 * a4 * (3 + 16 * r2) -
            64 * a2 * k2 * (4 + 19 * r2));
}

// ------------------------------------------------------------------ kernels

constexpr uint32_t kMaxJ = 1u << 16;

struct Exp {                 // one expiry of one request
    HP p;
    double tau, r, S, sqrt2m, lower, upper, du;   // du = pi 2^m / (2J): u_j = (2j + 1) du
    int32_t k1, k2;
    uint32_t J, n_opt;
    uint64_t tw_off, h_off, v_off, w_off, o_off;  // element offsets into the work buffers
    uint32_t fft, logN;      // the two transforms by FFT of length N = 2J = 2^logN (else direct sums)
    uint64_t f_off;          // its two N-element FFT buffers in the FFT workspace
};

// Expiries with at least this many frequencies use the FFT (automatic method).
constexpr uint32_t kFftMinJ = 1024;

struct Item {                // 32 consecutive outputs of one expiry
    uint32_t e, first;
};

// w^n = e^{i pi n / (2J)} for n < 4J, and the payoff terms h_j.
__global__ void tables_kernel(const Exp *ex, const Item *items, uint32_t n_items, double2 *tw, double2 *h) {
    const uint32_t it = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (it >= n_items) return;
    const Exp E = ex[items[it].e];
    const uint32_t n = items[it].first + (threadIdx.x & 31u);
    if (n >= 4 * E.J) return;
    double s, c;
    sincospi((double)n / (double)(2 * E.J), &s, &c);
    tw[E.tw_off + n] = make_double2(c, s);
    if (n < E.J) {
        const double u = (2.0 * n + 1.0) * E.du;
        auto H = [&](double y, double ey) {     // -i e^{-i u y} (1/u - ey/(i + u))
            double sy, cy;
            sincos(u * y, &sy, &cy);
            const double q = 1.0 + u * u;
            const double A = 1.0 / u - ey * u / q, B = ey / q;
            return C(cy * B - sy * A, -(cy * A + sy * B));
        };
        const double lo = fmax(E.lower, 0.0);
        const cplx v = H(E.upper, exp(E.upper)) - H(lo, exp(lo));
        h[E.h_off + n] = make_double2(v.re, v.im);
    }
}

// ------------------------------------------------------------------- FFT
//
// Both transforms are inverse DFTs of length N = 2J: with w = e^{i pi/(2J)},
// w^{k(2j+1)} = w^k e^{2 pi i k j / N}, so
//   V_k = Re(w^k F[k mod N]) sqrt(2^m)/J,  F = IDFT_N(h_0 .. h_{J-1}, 0 .. 0),
//   c_j = w^{2 k1 j} G[j] sqrt(2^m)/J,     G = IDFT_N(g folded mod N),
//         g_m = V_{k1+m} w^{k1+m},  m in [0, k2 - k1],
// IDFT_N(x)[n] = sum_r x_r e^{2 pi i r n / N}.  The IDFT is the radix-2
// Stockham autosort formulation (Govindaraju et al., "High performance
// discrete Fourier transforms on graphics processors", SC 2008): log2 N
// passes, each a butterfly over elements j and j + N/2 whose results land
// at ((j - k) << 1) + k and that plus Ns, k = j mod Ns, Ns = 2^pass, with
// twiddle e^{i pi k / Ns}; buffers alternate and the output is in natural
// order.  O(N log N) instead of the direct sums' O(J (k2 - k1)).

// buffer 0 of an FFT expiry: h_j for j < J, then zeros
__global__ void fft_load_h_kernel(const Exp *ex, const Item *items, uint32_t n_items, const double2 *h,
                                  double2 *fbuf) {
    const uint32_t it = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (it >= n_items) return;
    const Exp E = ex[items[it].e];
    const uint32_t m = items[it].first + (threadIdx.x & 31u);
    if (m >= 2 * E.J) return;
    fbuf[E.f_off + m] = m < E.J ? h[E.h_off + m] : make_double2(0.0, 0.0);
}

// buffer 0 of an FFT expiry: the terms V_{k1+m} w^{k1+m} folded mod N
__global__ void fft_load_g_kernel(const Exp *ex, const Item *items, uint32_t n_items, const double2 *tw,
                                  const double *V, double2 *fbuf) {
    const uint32_t it = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (it >= n_items) return;
    const Exp E = ex[items[it].e];
    const uint32_t r = items[it].first + (threadIdx.x & 31u), N = 2 * E.J;
    if (r >= N) return;
    const uint32_t mask = 4 * E.J - 1, K = (uint32_t)(E.k2 - E.k1 + 1);
    double re = 0.0, im = 0.0;
    for (uint32_t m = r; m < K; m += N) {   // K <= 4J = 2N: at most two terms
        const double v = V[E.v_off + m];
        const double2 t = tw[E.tw_off + ((uint32_t)(E.k1 + (int32_t)m) & mask)];
        re = fma(v, t.x, re);
        im = fma(v, t.y, im);
    }
    fbuf[E.f_off + r] = make_double2(re, im);
}

// one Stockham pass (Ns = 2^pass) of every FFT expiry with more passes to go
__global__ void fft_pass_kernel(const Exp *ex, const Item *items, uint32_t n_items, uint32_t pass, double2 *fbuf) {
    const uint32_t it = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (it >= n_items) return;
    const Exp E = ex[items[it].e];
    if (pass >= E.logN) return;
    const uint32_t N = 2 * E.J, half = E.J, j = items[it].first + (threadIdx.x & 31u);
    if (j >= half) return;
    const double2 *in = fbuf + E.f_off + (pass & 1u ? N : 0u);
    double2 *out = fbuf + E.f_off + (pass & 1u ? 0u : N);
    const uint32_t Ns = 1u << pass, k = j & (Ns - 1u);
    double s, c;
    sincospi((double)k / (double)Ns, &s, &c);
    const double2 a = in[j], b0 = in[j + half];
    const double2 b = make_double2(b0.x * c - b0.y * s, b0.x * s + b0.y * c);
    const uint32_t o = ((j - k) << 1) + k;
    out[o] = make_double2(a.x + b.x, a.y + b.y);
    out[o + Ns] = make_double2(a.x - b.x, a.y - b.y);
}

// the result of an FFT expiry's transform (after logN passes)
__device__ __forceinline__ const double2 *fft_result(const Exp &E, const double2 *fbuf) {
    return fbuf + E.f_off + (E.logN & 1u ? 2u * E.J : 0u);
}

// V_k, one lane per k
__global__ void payoff_kernel(const Exp *ex, const Item *items, uint32_t n_items, const double2 *tw,
                              const double2 *h, double *V, const double2 *fbuf) {
    const uint32_t it = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (it >= n_items) return;
    const Exp E = ex[items[it].e];
    const int32_t k = E.k1 + (int32_t)(items[it].first + (threadIdx.x & 31u));
    if (k > E.k2) return;
    const uint32_t mask = 4 * E.J - 1;
    const double2 *T = tw + E.tw_off;
    if (E.fft) {   // Re(w^k F[k mod N])
        const double2 f = fft_result(E, fbuf)[(uint32_t)k & (2 * E.J - 1)], t = T[(uint32_t)k & mask];
        V[E.v_off + (uint32_t)(k - E.k1)] = fma(f.x, t.x, -f.y * t.y) * E.sqrt2m / (double)E.J;
        return;
    }
    const double2 *Hh = h + E.h_off;
    double acc = 0.0;
    uint32_t idx = (uint32_t)k & mask, step = ((uint32_t)(2 * k)) & mask;   // k (2j + 1) mod 4J
    for (uint32_t j = 0; j < E.J; ++j) {
        const double2 a = Hh[j], t = T[idx];
        acc = fma(a.x, t.x, fma(-a.y, t.y, acc));
        idx = (idx + step) & mask;
    }
    V[E.v_off + (uint32_t)(k - E.k1)] = acc * E.sqrt2m / (double)E.J;
}

// c_j and phi(u_j) c_j with its gradient, one lane per j
__global__ void density_kernel(const Exp *ex, const Item *items, uint32_t n_items, const double2 *tw,
                               const double *V, double2 *W, const double2 *fbuf) {
    const uint32_t it = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (it >= n_items) return;
    const Exp E = ex[items[it].e];
    const uint32_t j = items[it].first + (threadIdx.x & 31u);
    if (j >= E.J) return;
    const uint32_t mask = 4 * E.J - 1;
    const double2 *T = tw + E.tw_off;
    const uint32_t odd = 2 * j + 1;
    double re = 0.0, im = 0.0;
    if (E.fft) {   // w^{2 k1 j} G[j]
        const double2 g = fft_result(E, fbuf)[j], t = T[((uint32_t)E.k1 * 2u * j) & mask];
        re = fma(g.x, t.x, -g.y * t.y);
        im = fma(g.x, t.y, g.y * t.x);
    } else {
        const double *Vk = V + E.v_off;
        uint32_t idx = ((uint32_t)E.k1 * odd) & mask;
        for (int32_t k = E.k1; k <= E.k2; ++k) {
            const double v = Vk[k - E.k1];
            const double2 t = T[idx];
            re = fma(v, t.x, re);
            im = fma(v, t.y, im);
            idx = (idx + odd) & mask;
        }
    }
    const double sc = E.sqrt2m / (double)E.J;
    const cplx c = C(re * sc, im * sc);
    cplx g[6];
    chf_grad(E.p, E.tau, C((double)odd * E.du), g);
#pragma unroll
    for (int q = 0; q < 6; ++q) {
        const cplx w = g[q] * c;
        W[E.w_off + (uint64_t)q * E.J + j] = make_double2(w.re, w.im);
    }
}

// one warp per option: Re sum_j W_q(j) disc K e^{-i u_j x}
__global__ void price_kernel(const Exp *ex, const Item *items, uint32_t n_items, const double2 *W,
                             const double *strikes, double *price, double *grad) {
    const uint32_t it = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (it >= n_items) return;
    const Exp E = ex[items[it].e];
    const uint32_t i = items[it].first, lane = threadIdx.x & 31u;
    const double K = strikes[E.o_off + i];
    const double x = E.r * E.tau + log(E.S / K);
    double acc[6] = {0, 0, 0, 0, 0, 0};
    for (uint32_t j = lane; j < E.J; j += 32) {
        double s, c;
        sincos((2.0 * j + 1.0) * E.du * x, &s, &c);     // e^{-i u x} = c - i s
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            const double2 w = W[E.w_off + (uint64_t)q * E.J + j];
            acc[q] = fma(w.x, c, fma(w.y, s, acc[q]));
        }
    }
#pragma unroll
    for (int q = 0; q < 6; ++q)
        for (int o = 16; o > 0; o >>= 1) acc[q] += __shfl_xor_sync(0xffffffffu, acc[q], o);
    if (lane == 0) {
        const double f = exp(-E.r * E.tau) * K;
        price[E.o_off + i] = f * acc[0];
        if (grad != nullptr)
#pragma unroll
            for (int q = 0; q < 5; ++q) grad[(E.o_off + i) * 5 + q] = f * acc[q + 1];
    }
}

} // namespace swift
} // namespace hexo

using namespace hexo;
using namespace hexo::swift;

namespace {

hexo_status params_dynamic(const HP &p, double tau, double r, double S, double K_min, double K_max, double prec,
                           hexo_swift_params &out) {
    unsigned m = 0;
    while (int_error(p, tau, m++) > prec)
        if (m > 30) return HEXO_ERR_NUMERIC;
    const double mx = r * tau + std::log(S / K_min), mn = r * tau + std::log(S / K_max);
    const double c = std::fabs(cum1(p, tau)) + 10.0 * std::sqrt(std::fabs(cum2(p, tau)) + std::sqrt(std::fabs(cum4(p, tau))));
    out.m = m;
    out.exp2_m = (uint32_t)std::exp2((double)m);
    out.sqrt_exp2_m = std::sqrt((double)out.exp2_m);
    out.lower = mn - c;
    out.upper = mx + c;
    out.k1 = (int32_t)std::ceil(out.exp2_m * out.lower);
    out.k2 = (int32_t)std::floor(out.exp2_m * out.upper);
    const double iota = std::ceil(std::log2(M_PI * std::abs(out.k1 - out.k2))) - 1;
    out.J = (uint32_t)std::exp2(iota - 1);
    return HEXO_OK;
}

bool valid_params(const hexo_swift_params &sp) {
    const uint32_t J = sp.J;
    return J >= 1 && J <= kMaxJ && (J & (J - 1)) == 0 && sp.k1 <= sp.k2 &&
           (int64_t)sp.k2 - (int64_t)sp.k1 + 1 <= 4 * (int64_t)J && sp.exp2_m >= 1 && std::isfinite(sp.lower) &&
           std::isfinite(sp.upper) && sp.sqrt_exp2_m > 0.0;
}

} // namespace

extern "C" {

hexo_status hexo_swift_params_dynamic(const hexo_params *p, double tau, double S, double K_min, double K_max,
                                      double trunc_precision, hexo_swift_params *out) {
    if (!p || !out || !(tau > 0.0) || !(S > 0.0) || !(K_min > 0.0) || !(K_max >= K_min) || !(trunc_precision > 0.0))
        return HEXO_ERR_INVALID;
    const HP hp{p->v0, p->theta, p->rho, p->kappa, p->sigma};
    if (!(hp.v0 > 0.0) || !(hp.sigma > 0.0) || !(hp.kappa > 0.0)) return HEXO_ERR_INVALID;
    return params_dynamic(hp, tau, p->r, S, K_min, K_max, trunc_precision, *out);
}

hexo_status hexo_swift_price(hexo_ctx *ctx, const hexo_swift_request *reqs, uint32_t n_reqs) {
    if (!ctx || !reqs || n_reqs == 0) return HEXO_ERR_INVALID;
    std::vector<Exp> ex;
    std::vector<double> strikes;
    std::vector<const hexo_swift_chain *> chain_of;
    uint64_t tw = 0, h = 0, v = 0, w = 0, f = 0;
    uint32_t max_log = 0;
    bool any_grad = false;
    for (uint32_t q = 0; q < n_reqs; ++q) {
        const hexo_swift_request &rq = reqs[q];
        const HP hp{rq.params.v0, rq.params.theta, rq.params.rho, rq.params.kappa, rq.params.sigma};
        if (!(hp.v0 > 0.0) || !(hp.sigma > 0.0) || !(hp.kappa > 0.0) || !(rq.S > 0.0) ||
            !std::isfinite(rq.params.r) || (rq.n_chains > 0 && !rq.chains))
            return ctx_fail(ctx, HEXO_ERR_INVALID, "swift request " + std::to_string(q) + ": bad parameters");
        for (uint32_t c = 0; c < rq.n_chains; ++c) {
            const hexo_swift_chain &ch = rq.chains[c];
            if (ch.n == 0) continue;
            if (!ch.strikes || !ch.price_out || !(ch.tau > 0.0))
                return ctx_fail(ctx, HEXO_ERR_INVALID, "swift chain: missing strikes/outputs or tau <= 0");
            double kmin = ch.strikes[0], kmax = ch.strikes[0];
            for (uint32_t i = 0; i < ch.n; ++i) {
                if (!(ch.strikes[i] > 0.0)) return ctx_fail(ctx, HEXO_ERR_INVALID, "swift chain: strike <= 0");
                kmin = std::min(kmin, ch.strikes[i]);
                kmax = std::max(kmax, ch.strikes[i]);
            }
            hexo_swift_params sp;
            if (ch.params) sp = *ch.params;
            else {
                const double prec = ch.trunc_precision > 0.0 ? ch.trunc_precision : 1e-7;
                const hexo_status s = params_dynamic(hp, ch.tau, rq.params.r, rq.S, kmin, kmax, prec, sp);
                if (s != HEXO_OK) return ctx_fail(ctx, s, "swift: the truncation loop did not converge");
            }
            if (!valid_params(sp))
                return ctx_fail(ctx, HEXO_ERR_UNSUPPORTED, "swift: J must be a power of two up to 65536 with k2 - k1 < 4J");
            if (ch.method > HEXO_SWIFT_FFT) return ctx_fail(ctx, HEXO_ERR_INVALID, "swift chain: unknown method");
            Exp e{};
            e.fft = ch.method == HEXO_SWIFT_FFT || (ch.method == HEXO_SWIFT_AUTO && sp.J >= kFftMinJ);
            if (e.fft) {   // two buffers of N = 2J
                while ((1u << e.logN) < 2u * sp.J) ++e.logN;
                e.f_off = f;
                f += 4ull * sp.J;
                max_log = std::max(max_log, e.logN);
            }
            e.p = hp;
            e.tau = ch.tau;
            e.r = rq.params.r;
            e.S = rq.S;
            e.sqrt2m = sp.sqrt_exp2_m;
            e.lower = sp.lower;
            e.upper = sp.upper;
            e.du = M_PI * (double)sp.exp2_m / (2.0 * sp.J);
            e.k1 = sp.k1;
            e.k2 = sp.k2;
            e.J = sp.J;
            e.n_opt = ch.n;
            e.tw_off = tw; tw += 4ull * sp.J;
            e.h_off = h; h += sp.J;
            e.v_off = v; v += (uint64_t)(sp.k2 - sp.k1 + 1);
            e.w_off = w; w += 6ull * sp.J;
            e.o_off = strikes.size();
            strikes.insert(strikes.end(), ch.strikes, ch.strikes + ch.n);
            ex.push_back(e);
            chain_of.push_back(&ch);
            any_grad |= ch.grad_out != nullptr;
        }
    }
    if (ex.empty()) return HEXO_OK;
    std::vector<Item> it_tab, it_pay, it_den, it_pri, it_fn, it_fb;
    for (uint32_t e = 0; e < ex.size(); ++e) {
        for (uint32_t n = 0; n < 4 * ex[e].J; n += 32) it_tab.push_back({e, n});
        for (uint32_t k = 0; k < (uint32_t)(ex[e].k2 - ex[e].k1 + 1); k += 32) it_pay.push_back({e, k});
        for (uint32_t j = 0; j < ex[e].J; j += 32) it_den.push_back({e, j});
        for (uint32_t i = 0; i < ex[e].n_opt; ++i) it_pri.push_back({e, i});
        if (ex[e].fft) {
            for (uint32_t n = 0; n < 2 * ex[e].J; n += 32) it_fn.push_back({e, n});   // N elements
            for (uint32_t j = 0; j < ex[e].J; j += 32) it_fb.push_back({e, j});       // N/2 butterflies
        }
    }
    const size_t n_opt = strikes.size();
    std::lock_guard<std::mutex> lk(ctx->run_mu);
    cudaSetDevice(ctx->device);
    cudaStream_t st = ctx->stream;
    // one allocation: descriptors, items, tables, outputs
    size_t off = 0;
    auto take = [&](size_t bytes) { const size_t o = off; off = (off + bytes + 255) / 256 * 256; return o; };
    const size_t o_ex = take(ex.size() * sizeof(Exp));
    const size_t o_i1 = take(it_tab.size() * sizeof(Item)), o_i2 = take(it_pay.size() * sizeof(Item));
    const size_t o_i3 = take(it_den.size() * sizeof(Item)), o_i4 = take(it_pri.size() * sizeof(Item));
    const size_t o_k = take(n_opt * sizeof(double));
    const size_t o_tw = take(tw * sizeof(double2)), o_h = take(h * sizeof(double2));
    const size_t o_v = take(v * sizeof(double)), o_w = take(w * sizeof(double2));
    const size_t o_p = take(n_opt * sizeof(double)), o_g = take(any_grad ? n_opt * 5 * sizeof(double) : 0);
    const size_t o_i5 = take(it_fn.size() * sizeof(Item)), o_i6 = take(it_fb.size() * sizeof(Item));
    const size_t o_f = take(f * sizeof(double2));
    void *dmem = nullptr;   // the context's arena: no allocation once it is large enough
    cudaError_t err = ctx_scratch(ctx, off, &dmem);
    if (err != cudaSuccess) return cuda_fail(ctx, err, "cudaMalloc swift");
    char *d = static_cast<char *>(dmem);
    auto up = [&](size_t o, const void *src, size_t bytes) {
        return bytes ? cudaMemcpyAsync(d + o, src, bytes, cudaMemcpyHostToDevice, st) : cudaSuccess;
    };
    if ((err = up(o_ex, ex.data(), ex.size() * sizeof(Exp))) != cudaSuccess ||
        (err = up(o_i1, it_tab.data(), it_tab.size() * sizeof(Item))) != cudaSuccess ||
        (err = up(o_i2, it_pay.data(), it_pay.size() * sizeof(Item))) != cudaSuccess ||
        (err = up(o_i3, it_den.data(), it_den.size() * sizeof(Item))) != cudaSuccess ||
        (err = up(o_i4, it_pri.data(), it_pri.size() * sizeof(Item))) != cudaSuccess ||
        (err = up(o_i5, it_fn.data(), it_fn.size() * sizeof(Item))) != cudaSuccess ||
        (err = up(o_i6, it_fb.data(), it_fb.size() * sizeof(Item))) != cudaSuccess ||
        (err = up(o_k, strikes.data(), n_opt * sizeof(double))) != cudaSuccess)
        return cuda_fail(ctx, err, "upload swift");
    const Exp *dex = reinterpret_cast<const Exp *>(d + o_ex);
    double2 *dtw = reinterpret_cast<double2 *>(d + o_tw), *dh = reinterpret_cast<double2 *>(d + o_h);
    double *dv = reinterpret_cast<double *>(d + o_v);
    double2 *dw = reinterpret_cast<double2 *>(d + o_w);
    double *dp = reinterpret_cast<double *>(d + o_p), *dg = any_grad ? reinterpret_cast<double *>(d + o_g) : nullptr;
    double2 *df = reinterpret_cast<double2 *>(d + o_f);
    const uint32_t n1 = (uint32_t)it_tab.size(), n2 = (uint32_t)it_pay.size(), n3 = (uint32_t)it_den.size(),
                   n4 = (uint32_t)it_pri.size(), n5 = (uint32_t)it_fn.size(), n6 = (uint32_t)it_fb.size();
    const Item *ifn = reinterpret_cast<const Item *>(d + o_i5), *ifb = reinterpret_cast<const Item *>(d + o_i6);
    auto fft_passes = [&]() {
        for (uint32_t pass = 0; pass < max_log; ++pass)
            fft_pass_kernel<<<(n6 + 3) / 4, 128, 0, st>>>(dex, ifb, n6, pass, df);
    };
    tables_kernel<<<(n1 + 3) / 4, 128, 0, st>>>(dex, reinterpret_cast<const Item *>(d + o_i1), n1, dtw, dh);
    if (n5) {   // F = IDFT(h) of the FFT expiries
        fft_load_h_kernel<<<(n5 + 3) / 4, 128, 0, st>>>(dex, ifn, n5, dh, df);
        fft_passes();
    }
    payoff_kernel<<<(n2 + 3) / 4, 128, 0, st>>>(dex, reinterpret_cast<const Item *>(d + o_i2), n2, dtw, dh, dv, df);
    if (n5) {   // G = IDFT(folded V w^k)
        fft_load_g_kernel<<<(n5 + 3) / 4, 128, 0, st>>>(dex, ifn, n5, dtw, dv, df);
        fft_passes();
    }
    density_kernel<<<(n3 + 3) / 4, 128, 0, st>>>(dex, reinterpret_cast<const Item *>(d + o_i3), n3, dtw, dv, dw,
                                                 df);
    price_kernel<<<(n4 + 3) / 4, 128, 0, st>>>(dex, reinterpret_cast<const Item *>(d + o_i4), n4, dw,
                                               reinterpret_cast<const double *>(d + o_k), dp, dg);
    if ((err = cudaGetLastError()) != cudaSuccess) return cuda_fail(ctx, err, "swift kernels");
    std::vector<double> hp(n_opt), hg(any_grad ? n_opt * 5 : 0);
    if ((err = cudaMemcpyAsync(hp.data(), dp, n_opt * sizeof(double), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (any_grad && (err = cudaMemcpyAsync(hg.data(), dg, n_opt * 5 * sizeof(double), cudaMemcpyDeviceToHost, st)) !=
                         cudaSuccess) ||
        (err = cudaStreamSynchronize(st)) != cudaSuccess)
        return cuda_fail(ctx, err, "swift results");
    for (size_t e = 0; e < ex.size(); ++e) {
        const hexo_swift_chain &ch = *chain_of[e];
        std::memcpy(ch.price_out, hp.data() + ex[e].o_off, ch.n * sizeof(double));
        if (ch.grad_out) std::memcpy(ch.grad_out, hg.data() + ex[e].o_off * 5, ch.n * 5 * sizeof(double));
    }
    return HEXO_OK;
}

// ------------------------------------------------ calibration callbacks

// The reference's calibration data (adata_s, src/inc/HCalibration.h:13-30):
// the spot and every chain's expiry and strikes.  prices / jacobian are the
// objective and Jacobian that its Levenberg-Marquardt call evaluates
// (get_prices_for_levmar / get_jacobian_for_levmar, HCalibration.cpp:35-57):
// for a parameter vector p = (v0, vm, rho, kappa, sigma) the wavelet
// parameters of every chain are chosen for p (update_adata,
// HCalibration.cpp:11-33), then all chains are priced in one call.  The last
// p's prices and Jacobian are kept, so the pair of calls levmar makes per
// step prices once.
struct hexo_calib {
    hexo_ctx *ctx = nullptr;
    double S = 0.0, r = 0.0, trunc = 1e-7;
    std::vector<double> taus, strikes;
    std::vector<uint32_t> counts;
    bool have = false;
    double last_p[5] = {0, 0, 0, 0, 0};
    std::vector<double> prices, jac;
};

namespace {
hexo_status calib_eval(hexo_calib *c, const double *p) {
    if (c->have && std::memcmp(p, c->last_p, sizeof c->last_p) == 0) return HEXO_OK;
    const size_t n = c->strikes.size();
    c->prices.assign(n, 0.0);
    c->jac.assign(n * 5, 0.0);
    std::vector<hexo_swift_chain> chains(c->taus.size());
    size_t off = 0;
    for (size_t k = 0; k < chains.size(); ++k) {
        hexo_swift_chain &ch = chains[k];
        std::memset(&ch, 0, sizeof ch);
        ch.tau = c->taus[k];
        ch.strikes = c->strikes.data() + off;
        ch.n = c->counts[k];
        ch.params = nullptr;
        ch.trunc_precision = c->trunc;
        ch.price_out = c->prices.data() + off;
        ch.grad_out = c->jac.data() + off * 5;
        off += c->counts[k];
    }
    hexo_swift_request rq;
    std::memset(&rq, 0, sizeof rq);
    rq.params = hexo_params{p[0], p[1], p[2], p[3], p[4], c->r, 0.0};
    rq.S = c->S;
    rq.chains = chains.data();
    rq.n_chains = (uint32_t)chains.size();
    const hexo_status s = hexo_swift_price(c->ctx, &rq, 1);
    c->have = s == HEXO_OK;
    if (c->have) std::memcpy(c->last_p, p, sizeof c->last_p);
    return s;
}
} // namespace

hexo_status hexo_calib_create(hexo_ctx *ctx, double S, double r, const double *taus, const uint32_t *counts,
                              const double *strikes, uint32_t n_chains, double trunc_precision, hexo_calib **out) {
    if (!ctx || !out || !taus || !counts || !strikes || n_chains == 0 || !(S > 0.0) || !std::isfinite(r))
        return HEXO_ERR_INVALID;
    *out = nullptr;
    hexo_calib *c = new (std::nothrow) hexo_calib();
    if (!c) return HEXO_ERR_NOMEM;
    c->ctx = ctx;
    c->S = S;
    c->r = r;
    c->trunc = trunc_precision > 0.0 ? trunc_precision : 1e-7;
    size_t n = 0;
    for (uint32_t k = 0; k < n_chains; ++k) {
        if (!(taus[k] > 0.0) || counts[k] == 0) { delete c; return HEXO_ERR_INVALID; }
        c->taus.push_back(taus[k]);
        c->counts.push_back(counts[k]);
        n += counts[k];
    }
    c->strikes.assign(strikes, strikes + n);
    *out = c;
    return HEXO_OK;
}

uint32_t hexo_calib_observations(const hexo_calib *c) { return c ? (uint32_t)c->strikes.size() : 0u; }

hexo_status hexo_calib_prices(hexo_calib *c, const double *p, double *x) {
    if (!c || !p || !x) return HEXO_ERR_INVALID;
    const hexo_status s = calib_eval(c, p);
    if (s == HEXO_OK) std::memcpy(x, c->prices.data(), c->prices.size() * sizeof(double));
    return s;
}

hexo_status hexo_calib_jacobian(hexo_calib *c, const double *p, double *jac) {
    if (!c || !p || !jac) return HEXO_ERR_INVALID;
    const hexo_status s = calib_eval(c, p);
    if (s == HEXO_OK) std::memcpy(jac, c->jac.data(), c->jac.size() * sizeof(double));
    return s;
}

hexo_status hexo_calib_destroy(hexo_calib *c) {
    if (!c) return HEXO_ERR_INVALID;
    delete c;
    return HEXO_OK;
}

} // extern "C"
