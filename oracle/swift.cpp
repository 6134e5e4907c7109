// ORACLE / TEST INFRASTRUCTURE ONLY.
//
// CPU restatement of the reference's SWIFT European pricer and the Heston
// characteristic function it uses, as the check for European Monte Carlo
// prices.  The reference computes these with FFTW and Eigen, neither of which
// is available here, so both transforms are written as direct sums (the same
// sums the FFTs evaluate) and the final matrix product as plain loops.
// Pinned by the reference's own golden vectors: the 40 prices of
// pricing_test (src/UnitTest.cpp:219-274) and the 200 gradient entries of
// gradient_test (src/UnitTest.cpp:276-321), both at the predefined wavelet
// parameters of src/UnitTest.cpp:174-181.
//
// Method: L. Ortiz-Gracia and C. W. Oosterlee, "A highly efficient Shannon
// wavelet inverse Fourier technique for pricing European options", SIAM J.
// Sci. Comput. 38 (2016); characteristic-function form and gradient of
// Y. Cui, S. del Bano Rollin and G. Germano, "Full and fast calibration of the
// Heston stochastic volatility model", EJOR 263 (2017).
#include <cmath>
#include <complex>
#include <cstdint>
#include <vector>

namespace {

using cd = std::complex<double>;
const cd I(0.0, 1.0);

struct HP { double v0, vm, rho, kappa, sigma; };

// Per-frequency helper quantities (HDistribution.cpp:13-26).
struct Aux {
    cd xi, d, A1, A2, A, B, D, sh, ch;
    double ekt;
};

Aux aux(const HP &p, cd u, double tau) {
    Aux a;
    a.xi = p.kappa + p.sigma * p.rho * I * u;
    const cd f = u * u - I * u;
    a.d = std::sqrt(a.xi * a.xi + p.sigma * p.sigma * f);
    a.sh = std::sinh(a.d * tau * 0.5);
    a.ch = std::cosh(a.d * tau * 0.5);
    a.A1 = f * a.sh;
    a.A2 = a.d / p.v0 * a.ch + a.xi / p.v0 * a.sh;
    a.A = a.A1 / a.A2;
    a.ekt = std::exp(p.kappa * tau * 0.5);
    a.B = a.d * a.ekt / (p.v0 * a.A2);
    a.D = std::log((2.0 * a.d) / (a.d + a.xi + (a.d - a.xi) * std::exp(-a.d * tau))) + (p.kappa - a.d) * tau * 0.5;
    return a;
}

// Characteristic function of the log-return without drift (HDistribution.cpp:31-37).
cd chf(const HP &p, double tau, cd u, const Aux &a) {
    return std::exp((p.kappa * p.vm * p.rho * tau * u * I) / p.sigma - a.A + (2.0 * a.D * p.kappa * p.vm) / (p.sigma * p.sigma));
}

// chf and its five partial derivatives in HParams order (HDistribution.cpp:48-84).
void chf_grad(const HP &p, double tau, cd u, cd out[6]) {
    const Aux a = aux(p, u, tau);
    const cd c = chf(p, tau, u, a);
    const cd iu = I * u;
    const cd d_rho = a.xi * p.sigma * iu / a.d;
    const cd A2_rho = p.sigma * iu * (2.0 + a.xi * tau) / (2.0 * a.d * p.v0) * (a.xi * a.ch + a.d * a.sh);
    const cd B_rho = a.ekt / p.v0 * (d_rho / a.A2 - a.d / (a.A2 * a.A2) * A2_rho);
    const cd A1_rho = (iu * (u * u - iu) * tau * a.xi * p.sigma) / (2.0 * a.d) * a.ch;
    const cd A_rho = A1_rho / a.A2 - a.A / a.A2 * A2_rho;
    const cd B_kappa = -I / (p.sigma * u) * B_rho + a.B * tau * 0.5;
    const cd d_sigma = (p.rho / p.sigma - 1.0 / a.xi) * d_rho + p.sigma * u * u / a.d;
    const cd A1_sigma = (u * u - iu) * 0.5 * tau * d_sigma * a.ch;
    const cd A2_sigma = p.rho / p.sigma * A2_rho + (2.0 + tau * a.xi) / (p.v0 * tau * a.xi * iu) * A1_rho +
                        p.sigma * tau * a.A1 / p.v0 * 0.5;
    const cd A_sigma = A1_sigma / a.A2 - a.A / a.A2 * A2_sigma;
    const cd t_iu_vm_s = p.vm * tau * iu / p.sigma;
    const double s2 = p.sigma * p.sigma;
    const double k_vm_2_s2 = 2.0 * p.kappa * p.vm / s2;
    const cd g_v0 = -a.A / p.v0;
    const cd g_vm = 2.0 * p.kappa / s2 * a.D + p.kappa * p.rho * tau * iu / p.sigma;
    const cd g_sigma = -A_sigma - 2.0 * k_vm_2_s2 / p.sigma * a.D + k_vm_2_s2 / a.d * (d_sigma - a.d / a.A2 * A2_sigma) -
                       t_iu_vm_s / p.sigma * p.rho * p.kappa;
    const cd g_kappa = -A_rho / (p.sigma * iu) + 2.0 * p.vm / s2 * a.D + k_vm_2_s2 / a.B * B_kappa + t_iu_vm_s * p.rho;
    const cd g_rho = -A_rho + k_vm_2_s2 / a.d * (d_rho - a.d / a.A2 * A2_rho) + t_iu_vm_s * p.kappa;
    out[0] = c;
    out[1] = c * g_v0;
    out[2] = c * g_vm;
    out[3] = c * g_rho;
    out[4] = c * g_kappa;
    out[5] = c * g_sigma;
}

// Truncation error of wavelet scale m (HDistribution.cpp:8-11).
double int_error(const HP &p, double tau, unsigned m) {
    const double e = std::exp2((double)m);
    const cd u1(e * M_PI, 0.0), u2(-e * M_PI, 0.0);
    return std::abs(chf(p, tau, u1, aux(p, u1, tau)) + chf(p, tau, u2, aux(p, u2, tau))) / (4.0 * e * M_PI * M_PI * tau);
}

// Cumulants (HDistribution.cpp:86-113).  The reference binds the parameter
// struct positionally as (v, s2, r, kappa, k) = (v0, vm, rho, kappa, sigma),
// so "s2" is vm and "r" is rho in these formulas.
double cum1(const HP &p, double tau) { return -0.5 * p.vm * tau; }

double cum2(const HP &p, double t) {
    const double s2 = p.vm, r = p.rho, kappa = p.kappa, k = p.sigma;
    const double kappa2 = kappa * kappa, kappa3 = kappa2 * kappa, k2 = k * k;
    return s2 / (8 * kappa3) *
           (-k2 * std::exp(-2 * kappa * t) + 4 * k * std::exp(-kappa * t) * (k - 2 * kappa * r) +
            2 * kappa * t * (4 * kappa2 + k2 - 4 * kappa * k * r) + k * (8 * kappa * r - 3 * k));
}

double cum4(const HP &p, double t) {
    const double s2 = p.vm, r = p.rho, a = p.kappa, k = p.sigma;
    const double a2 = a * a, a3 = a2 * a, a4 = a3 * a;
    const double k2 = k * k, k3 = k2 * k, k4 = k3 * k;
    const double t2 = t * t, r2 = r * r;
    const double km = k - 2 * a * r;
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

// exp(i * pi * n / den) with n reduced modulo 2 den first, so the angle stays small.
cd cis_pi(int64_t n, int64_t den) {
    const int64_t per = 2 * den;
    int64_t r = n % per;
    if (r < 0) r += per;
    const double ang = M_PI * (double)r / (double)den;
    return cd(std::cos(ang), std::sin(ang));
}

struct Params {
    unsigned m, exp2_m;
    double sqrt_exp2_m, lower, upper;
    int k1, k2;
    unsigned J;
    double u(unsigned j) const { return M_PI * (2.0 * j + 1.0) / (2.0 * J) * (double)exp2_m; }
};

// Density coefficients (SWIFT.cpp:37-79), transforms as direct sums.
std::vector<cd> density_coeffs(const Params &sp) {
    const unsigned J = sp.J;
    const double ue = std::exp(sp.upper), le = std::exp(std::max(sp.lower, 0.0));
    const double lo = std::max(sp.lower, 0.0);
    std::vector<cd> h(J);
    for (unsigned j = 0; j < J; ++j) {
        const double uj = sp.u(j);
        auto H = [&](double y, double ey) { return -I * std::exp(-I * uj * y) * (1.0 / uj - ey / (I + uj)); };
        h[j] = H(sp.upper, ue) - H(lo, le);
    }
    // V_k = Re(e^{i pi k / 2J} * sum_j h_j e^{2 pi i j k / 2J}) * sqrt(2^m) / J
    //     = Re(sum_j h_j e^{i pi k (2j+1) / 2J}) * sqrt(2^m) / J
    const int nk = sp.k2 - sp.k1 + 1;
    std::vector<double> V(nk > 0 ? nk : 0);
    for (int k = sp.k1; k <= sp.k2; ++k) {
        cd s = 0.0;
        for (unsigned j = 0; j < J; ++j) s += h[j] * cis_pi((int64_t)k * (2 * j + 1), 2 * (int64_t)J);
        V[k - sp.k1] = s.real() * sp.sqrt_exp2_m / (double)J;
    }
    // c_j = conj(sum_k V_k e^{-2 pi i k (2j+1) / 4J}) * sqrt(2^m) / J
    std::vector<cd> c(J);
    for (unsigned j = 0; j < J; ++j) {
        cd s = 0.0;
        for (int k = sp.k1; k <= sp.k2; ++k) s += V[k - sp.k1] * cis_pi((int64_t)k * (2 * j + 1), 2 * (int64_t)J);
        c[j] = s * sp.sqrt_exp2_m / (double)J;
    }
    return c;
}

} // namespace

extern "C" {

// Dynamic wavelet parameters (SWIFT.cpp:21-35); out8 = {m, exp2_m,
// sqrt_exp2_m, lower, upper, k1, k2, J}.  trunc_precision is 1e-10 in the
// reference's default build, 1e-7 with FASTMATH (SWIFT.cpp:12-16).
int oracle_swift_params(const double *p5, double tau, double r, double S, double K_min, double K_max,
                        double trunc_precision, double *out8) {
    const HP p{p5[0], p5[1], p5[2], p5[3], p5[4]};
    unsigned m = 0;
    while (int_error(p, tau, m++) > trunc_precision)
        if (m > 40) return 1;
    const double mx = r * tau + std::log(S / K_min);
    const double mn = r * tau + std::log(S / K_max);
    const double c = std::abs(cum1(p, tau)) + 10.0 * std::sqrt(std::fabs(cum2(p, tau)) + std::sqrt(std::abs(cum4(p, tau))));
    const unsigned e = (unsigned)std::exp2((double)m);
    const double lower = mn - c, upper = mx + c;
    const int k1 = (int)std::ceil(e * lower), k2 = (int)std::floor(e * upper);
    const double iota = std::ceil(std::log2(M_PI * std::abs(k1 - k2))) - 1;
    const unsigned J = (unsigned)std::exp2(iota - 1);
    out8[0] = m;
    out8[1] = e;
    out8[2] = std::sqrt((double)e);
    out8[3] = lower;
    out8[4] = upper;
    out8[5] = k1;
    out8[6] = k2;
    out8[7] = J;
    return 0;
}

// European call prices (and, if grad_out != NULL, their gradients, five per
// option in HParams order) of one expiry (SWIFT.cpp:102-118).
int oracle_swift_price(const double *p5, double tau, double r, double S, const double *strikes, uint32_t n,
                       const double *sp8, double *price_out, double *grad_out) {
    const HP p{p5[0], p5[1], p5[2], p5[3], p5[4]};
    Params sp{(unsigned)sp8[0], (unsigned)sp8[1], sp8[2], sp8[3], sp8[4], (int)sp8[5], (int)sp8[6], (unsigned)sp8[7]};
    if (sp.J == 0) return 1;
    const std::vector<cd> c = density_coeffs(sp);
    std::vector<cd> w(6 * (size_t)sp.J);
    for (unsigned j = 0; j < sp.J; ++j) {
        cd g[6];
        chf_grad(p, tau, cd(sp.u(j), 0.0), g);
        for (int q = 0; q < 6; ++q) w[6 * j + q] = g[q] * c[j];
    }
    const double disc = std::exp(-r * tau);
    for (uint32_t i = 0; i < n; ++i) {
        const double x = r * tau + std::log(S / strikes[i]);
        cd acc[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
        for (unsigned j = 0; j < sp.J; ++j) {
            const cd e = disc * strikes[i] * std::exp(-I * sp.u(j) * x);
            for (int q = 0; q < 6; ++q) acc[q] += w[6 * j + q] * e;
        }
        price_out[i] = acc[0].real();
        if (grad_out)
            for (int q = 0; q < 5; ++q) grad_out[5 * i + q] = acc[q + 1].real();
    }
    return 0;
}

// chf and gradient at a complex frequency: out12 = re/im of 6 values.
void oracle_heston_chf_grad(const double *p5, double tau, double u_re, double u_im, double *out12) {
    const HP p{p5[0], p5[1], p5[2], p5[3], p5[4]};
    cd g[6];
    chf_grad(p, tau, cd(u_re, u_im), g);
    for (int q = 0; q < 6; ++q) {
        out12[2 * q] = g[q].real();
        out12[2 * q + 1] = g[q].imag();
    }
}

} // extern "C"
