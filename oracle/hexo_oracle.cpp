/*
 * ORACLE / TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement ("port") of the reference's Monte Carlo pricing path, used
 * as the oracle of the GPU engine's parity tests and as the timed CPU baseline.
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
 * it; the product never links or calls it.
 *
 * What it restates (reference file:line):
 *   OracleRNG        RNG wrapper, src/inc/RNG.h:17-52 + src/RNG.cpp:8-47:
 *                    one SHISHUA stream seeded {seed,0,0,0} (the engine's
 *                    per-request stream number goes to seed word 1, which
 *                    the reference's four-word seed, RNG.h:24, leaves 0)
 *                    feeds a uniform
 *                    buffer (filled first) and a normal buffer (filled next);
 *                    each refills from the same stream when it runs dry;
 *                    u = (double)w / (double)UINT64_MAX (RNG.cpp:31); normals
 *                    are ppnd16(u) (RNG.cpp:34-43).
 *   qe_step          HQEAnderson::operator++, src/HSimulation.tpp:52-86, with
 *                    an optional (r-q)*delta drift folded into K_0 (zero drift
 *                    leaves every operation bit-identical).
 *   run_path         the per-path body of HSimulation::price,
 *                    src/HSimulation.tpp:30-46, with the Asian contract
 *                    (src/inc/AsianContract.h:25-47) and the European contract
 *                    (src/inc/VanillaContract.h:28-39) tracked on one path.
 *   reference partition driver: price()'s thread partition
 *                    (HSimulation.tpp:23-29: n/threads paths per thread, one
 *                    RNG(RAND_BUF_SIZE=2^20, 1<<tid) per thread, the trailing
 *                    step after the last maturity) with the per-option
 *                    accumulation `prices[i] += payoff/n` (tpp:40) kept in
 *                    path order but race-free (per-thread arrays).
 *   per-path driver: the stream partition the GPU engine uses: path k of a
 *                    request draws from its own RNG(block_words, seed+k),
 *                    seeded {seed+k, stream, 0, 0};
 *                    oracle_branch_counts walks the same paths and counts
 *                    the QE steps on the quadratic branch (tpp:63-68).
 *
 * Built twice by oracle/Makefile: liboracle.so (-O2 -ffp-contract=off, the
 * parity tests' oracle) and liboracle_fast.so (the reference's release flags minus
 * -march=native, the timed CPU baseline).  as241.c is always compiled
 * without fast-math, as the reference compiles as241.f90.
 */
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#include <numeric>
#include <complex>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "shishua.h"

extern "C" double ppnd16(double *, int *);
extern "C" float oracle_logf(float);

namespace {

/* RNG.h:17-52, RNG.cpp:8-47 */
class OracleRNG {
    std::vector<double> u_, g_;
    size_t cu_, cg_, size_;
    prng_state s_;
    void fill_uniform(std::vector<double> &buf) {
        prng_gen(&s_, reinterpret_cast<uint8_t *>(buf.data()), size_ * sizeof(double));
        for (double &x : buf) {
            uint64_t w;
            std::memcpy(&w, &x, 8);
            x = static_cast<double>(w) / static_cast<double>(UINT64_MAX);
        }
    }
    void fill_normal() {
        fill_uniform(g_);
        for (double &x : g_) {
            int ifault = 0;
            x = ppnd16(&x, &ifault);
        }
    }

public:
    OracleRNG(size_t size, uint64_t seed0, uint64_t seed1 = 0) : u_(size), g_(size), cu_(0), cg_(0), size_(size) {
        uint64_t seed[4] = {seed0, seed1, 0, 0};
        prng_init(&s_, seed);
        fill_uniform(u_);
        fill_normal();
    }
    double grand() {
        if (cg_ == size_) { fill_normal(); cg_ = 0; }
        return g_[cg_++];
    }
    double urand() {
        if (cu_ == size_) { fill_uniform(u_); cu_ = 0; }
        return u_[cu_++];
    }
};

struct Params { double v0, theta, rho, kappa, sigma, r, q; };

struct PathState { double Xc, Xp, vc, vp, t, tp, logX; };

/* HSimulation.tpp:52-86 (+ drift in K_0); returns whether the step took the
 * quadratic branch (Psi < 1.5, tpp:63). */
inline bool qe_step(PathState &st, const Params &p, double delta, OracleRNG &rng) {
    const double v_0 = p.v0, theta = p.theta, rho = p.rho, kappa = p.kappa, eps = p.sigma;
    (void)v_0;
    const double gamma_1 = .5, gamma_2 = .5;
    double discount = std::exp(-kappa * delta);
    double m = theta + (st.vc - theta) * discount;
    double sp2 = std::fabs(st.vc * eps * eps * discount / kappa * (1 - discount) +
                           theta * eps * eps / (2 * kappa) * (1. - discount) * (1. - discount));
    double Psi = sp2 / (m * m);
    st.vp = st.vc;
    const bool quad = Psi < 1.5;
    if (quad) {
        double bp2 = 2 / Psi - 1 + std::sqrt(2 / Psi * (2 / Psi - 1));
        double b = std::sqrt(bp2);
        double a = m / (1 + bp2);
        double Z_V = rng.grand();
        st.vc = a * (b + Z_V) * (b + Z_V);
    } else {
        double pp = (Psi - 1) / (Psi + 1);
        double beta = 2 / (m * (Psi + 1));
        double U_V = rng.urand();
        st.vc = pp < U_V ? std::log((1 - pp) / (1 - U_V)) / beta : 0.;
    }
    double K_0 = -rho * kappa * theta / eps * delta + (p.r - p.q) * delta;
    double K_1 = gamma_1 * delta * (kappa * rho / eps - .5) - rho / eps;
    double K_2 = gamma_2 * delta * (kappa * rho / eps - .5) + rho / eps;
    double K_3 = gamma_1 * delta * (1 - rho * rho);
    double K_4 = gamma_2 * delta * (1 - rho * rho);
    st.logX = st.logX + K_0 + K_1 * st.vp + K_2 * st.vc + std::sqrt(K_3 * st.vp + K_4 * st.vc) * rng.grand();
    st.Xp = st.Xc;
    st.Xc = std::exp(st.logX);
    st.tp = st.t;
    st.t += delta;
    return quad;
}

/* Maturity-grouped view of one pricing request. */
struct Problem {
    Params p;
    double S0;
    std::vector<double> T;           // distinct maturities, ascending
    std::vector<uint32_t> steps;     // steps per maturity (the reference's `steps` argument)
    std::vector<std::vector<uint32_t>> opts; // option indices per maturity
    const double *strike;
    const uint8_t *kind;             // 0 = arithmetic Asian call, 1 = European call
    const uint64_t *n_paths;         // per option
    uint32_t n_opts;
};

/* Per-path body of HSimulation.tpp:30-46.  `visit(j, asian_final, euro_final)`
 * is called at each maturity j in increasing order; it returns false once the
 * path is no longer needed.  `trailing` runs the extra step the reference's
 * for-increment takes after the last pricing (tpp:35), which matters only
 * when the stream is shared with the next path. */
template <class Visit>
inline void run_path(const Problem &pr, OracleRNG &rng, bool trailing, Visit &&visit, uint64_t *counts = nullptr) {
    PathState st{pr.S0, pr.S0, pr.p.v0, pr.p.v0, 0., 0., std::log(pr.S0)};
    const double logS0 = st.logX;
    const size_t m = pr.T.size();
    size_t j = 0;
    uint64_t n_quad = 0, n_steps = 0;   // optional branch counts (counts[0], counts[1])
    double dt = pr.T[0] / pr.steps[0];  // update_earliest, AsianContract.h:35-38
    double acc = 0.;                    // reset, AsianContract.h:39-42
    // the control variate's geometric counterpart of the Asian average: the
    // same weights on y = log(X / S0) instead of X
    double yc = 0., yp = 0., accg = 0.;
    n_quad += qe_step(st, pr.p, dt, rng);   // ++(heston_sde = initial_state), tpp:35
    ++n_steps;
    yp = yc; yc = st.logX - logS0;
    for (;;) {
        bool more = true;
        while (j < m && st.t >= pr.T[j]) {                              // tpp:36
            double T = pr.T[j];
            double interp = (st.Xc - st.Xp) * (T - st.tp) / dt;
            double asian = (acc + interp) / T;                          // AsianContract.h:29-34
            double euro = st.Xp + (st.Xc - st.Xp) * (T - st.tp) / dt;   // VanillaContract.h:28-31
            double geo = pr.S0 * std::exp((accg + (yc - yp) * (T - st.tp) / dt) / T);
            more = visit(j, asian, euro, geo);
            ++j;
            if (j < m) dt = pr.T[j] / pr.steps[j];                      // tpp:41-42
            if (!more) break;
        }
        if (j >= m || !more) {
            if (trailing) qe_step(st, pr.p, dt, rng);                   // tpp:35 for-increment
            if (counts) { counts[0] += n_quad; counts[1] += n_steps; }
            return;
        }
        acc += dt * .5 * (st.Xc + st.Xp);                               // AsianContract.h:25-28
        accg += dt * .5 * (yc + yp);
        n_quad += qe_step(st, pr.p, dt, rng);
        ++n_steps;
        yp = yc; yc = st.logX - logS0;
    }
}

inline double payoff_of(const Problem &pr, uint32_t o, double asian, double euro) {
    double fv = pr.kind[o] == 0 ? asian : euro;
    return std::max(0., fv - pr.strike[o]);                             // AsianContract.h:43-47
}

/* The binary exponent E of a spot, 2^(E-1) <= S0 < 2^E: payoffs are summed
 * in units of 2^E. */
inline int pay_exponent(double S0) {
    int e = 0;
    (void)std::frexp(S0, &e);
    return e;
}

/* Exact fixed-point accumulation in the engine's format: with y = pay 2^-E,
 * q = round(y*2^47) and q2 = round(y^2*2^43) (y^2 rounded to double, ties to
 * even), each split into three 25-bit limbs; limb sums are exact, so the
 * order of paths does not matter. */
struct ExactSums {
    std::vector<uint64_t> l;   // [o*6 + limb]
    int E;
    ExactSums(size_t n, int E_) : l(6 * n, 0), E(E_) {}
    void add(uint32_t o, double pay) {
        const double y = std::ldexp(pay, -E);
        const unsigned __int128 q = (unsigned __int128)std::nearbyint(y * 0x1p47);
        const unsigned __int128 q2 = (unsigned __int128)std::nearbyint(y * y * 0x1p43);
        const uint64_t M = (1ull << 25) - 1;
        uint64_t *d = &l[6 * (size_t)o];
        d[0] += (uint64_t)(q & M); d[1] += (uint64_t)((q >> 25) & M); d[2] += (uint64_t)(q >> 50);
        d[3] += (uint64_t)(q2 & M); d[4] += (uint64_t)((q2 >> 25) & M); d[5] += (uint64_t)(q2 >> 50);
    }
    void merge(const ExactSums &o) {
        for (size_t i = 0; i < l.size(); ++i) l[i] += o.l[i];
    }
    static unsigned __int128 value(const uint64_t *d) {
        return (unsigned __int128)d[0] + ((unsigned __int128)d[1] << 25) + ((unsigned __int128)d[2] << 50);
    }
};

int build_problem(Problem &pr, const double *params7, double S0, uint32_t n_opts, const double *strike,
                  const double *T, const uint8_t *kind, const uint64_t *n_paths, uint32_t step_mode,
                  uint32_t steps, double steps_per_year) {
    if (n_opts == 0) return 1;
    pr.p = Params{params7[0], params7[1], params7[2], params7[3], params7[4], params7[5], params7[6]};
    pr.S0 = S0;
    pr.strike = strike;
    pr.kind = kind;
    pr.n_paths = n_paths;
    pr.n_opts = n_opts;
    std::vector<uint32_t> idx(n_opts);
    std::iota(idx.begin(), idx.end(), 0u);
    std::stable_sort(idx.begin(), idx.end(), [&](uint32_t a, uint32_t b) { return T[a] < T[b]; });
    for (uint32_t i : idx) {
        if (!(T[i] > 0.)) return 2;
        if (pr.T.empty() || pr.T.back() != T[i]) {
            pr.T.push_back(T[i]);
            uint32_t n = steps;
            if (step_mode == 1) {
                double g = std::nearbyint(steps_per_year * T[i]);
                n = static_cast<uint32_t>(std::max(5.0, g));
            }
            if (n == 0) return 3;
            pr.steps.push_back(n);
            pr.opts.emplace_back();
        }
        pr.opts.back().push_back(i);
    }
    return 0;
}


/* ---------------------------------------------------------------------
 * Geometric-average control variate (the future idea of HSimulation.h:51).
 *
 * Per path, L = (sum_k h_k (y_k + y_{k-1}) + (y_n - y_{n-1}) w) / T on
 * y = log(X / S0): the Asian contract's weights (AsianContract.h:25-34,
 * the spot-difference term included) on the log-spot, and G = S0 exp(L).
 * E[(G - K)^+] under the Heston model itself (continuous time, the same
 * time grid) comes from the characteristic function of L, a backward
 * recursion of the affine solution over the grid steps, and Lewis's single
 * integral; the estimator is mean((A - K)^+ - (G - K)^+) + E[(G - K)^+].
 * ------------------------------------------------------------------- */

/* The grid steps up to maturity jt and the weights c_k of y_1..y_n in L,
 * walking the time grid exactly as run_path does. */
void cv_schedule(const Problem &pr, size_t jt, std::vector<double> &dts, std::vector<double> &c) {
    const size_t m = pr.T.size();
    double t = 0., tp = 0., dt = pr.T[0] / pr.steps[0];
    size_t j = 0;
    std::vector<double> h;   // h[k-1] weighs y_k + y_{k-1}
    dts.clear();
    tp = t; t += dt; dts.push_back(dt);
    for (;;) {
        while (j < m && t >= pr.T[j]) {
            if (j == jt) {
                const double T = pr.T[j], w = (T - tp) / dt;
                const size_t n = dts.size();
                c.assign(n, 0.);
                for (size_t k = 1; k < n; ++k) {
                    c[k - 1] += h[k - 1];
                    if (k >= 2) c[k - 2] += h[k - 1];
                }
                if (n >= 2) c[n - 2] -= w;
                c[n - 1] += w;
                for (double &x : c) x /= T;
                return;
            }
            ++j;
            if (j < m) dt = pr.T[j] / pr.steps[j];
        }
        h.push_back(dt * .5);
        tp = t; t += dt; dts.push_back(dt);
    }
}

typedef std::complex<double> cplx;

/* E_t[exp(a (y_T - y_t) + b v_T)] = exp(A + B v_t) over tau = T - t:
 * the Heston affine solution with terminal b (the "little trap" form). */
inline void heston_affine(cplx a, cplx b, double tau, const Params &p, cplx &A, cplx &B) {
    const double s2 = p.sigma * p.sigma, mu = p.r - p.q;
    const cplx beta = p.kappa - p.rho * p.sigma * a;
    cplx D = std::sqrt(beta * beta - s2 * a * (a - 1.));
    if (D.real() < 0.) D = -D;
    const cplx g = (beta - D - s2 * b) / (beta + D - s2 * b);
    const cplx e = std::exp(-D * tau);
    B = ((beta - D) - (beta + D) * g * e) / (s2 * (1. - g * e));
    A = a * mu * tau + p.kappa * p.theta / s2 * ((beta - D) * tau - 2. * std::log((1. - g * e) / (1. - g)));
}

/* E[exp(z L)] for complex z. */
inline cplx cf_L(cplx z, const std::vector<double> &dts, const std::vector<double> &c, const Params &p) {
    cplx Asum = 0., b = 0., Th = 0.;
    for (size_t k = dts.size(); k-- > 0;) {
        Th += z * c[k];                        // weight of the increment of step k+1
        cplx A, B;
        heston_affine(Th, b, dts[k], p, A, B);
        Asum += A;
        b = B;
    }
    return std::exp(Asum + b * p.v0);
}

/* Gauss-Legendre nodes and weights on [-1, 1] (Newton on P_N). */
void gauss_legendre(int N, std::vector<double> &x, std::vector<double> &w) {
    x.assign(N, 0.); w.assign(N, 0.);
    for (int i = 0; i < (N + 1) / 2; ++i) {
        double z = std::cos(M_PI * (i + 0.75) / (N + 0.5)), pp = 0.;
        for (int it = 0; it < 100; ++it) {
            double p1 = 1., p2 = 0.;
            for (int k = 1; k <= N; ++k) { const double p3 = p2; p2 = p1; p1 = ((2. * k - 1.) * z * p2 - (k - 1.) * p3) / k; }
            pp = N * (z * p1 - p2) / (z * z - 1.);
            const double dz = p1 / pp;
            z -= dz;
            if (std::fabs(dz) < 1e-16) break;
        }
        x[i] = -z; x[N - 1 - i] = z;
        w[i] = w[N - 1 - i] = 2. / ((1. - z * z) * pp * pp);
    }
}

constexpr int kCvNodesNear = 256, kCvNodesTail = 128;   // [0, U] and [U, inf) by u = U / s
constexpr double kCvRange = 40.;                        // U = 40 standard deviations of L

/* E[G] and E[(G - K_i)^+] for the strikes of one maturity (undiscounted). */
void cv_geo_calls(const Params &p, double S0, const std::vector<double> &dts, const std::vector<double> &c,
                  const double *K, size_t nk, double *out, double *F_out) {
    const double F = S0 * cf_L(1., dts, c, p).real();
    // the scale of L from its variance with the variance's mean path
    double var = 0., t = 0., Cw = 0.;
    std::vector<double> Cws(dts.size());
    for (size_t k = dts.size(); k-- > 0;) { Cw += c[k]; Cws[k] = Cw; }
    for (size_t k = 0; k < dts.size(); ++k) {
        const double Ev = p.theta + (p.v0 - p.theta) * std::exp(-p.kappa * t);
        var += Cws[k] * Cws[k] * Ev * dts[k];
        t += dts[k];
    }
    const double U = kCvRange / std::sqrt(std::max(var, 1e-12));
    std::vector<double> x1, w1, x2, w2;
    gauss_legendre(kCvNodesNear, x1, w1);
    gauss_legendre(kCvNodesTail, x2, w2);
    std::vector<double> u, w;
    for (int i = 0; i < kCvNodesNear; ++i) { u.push_back(.5 * U * (x1[i] + 1.)); w.push_back(.5 * U * w1[i]); }
    for (int i = 0; i < kCvNodesTail; ++i) { const double s = .5 * (x2[i] + 1.); u.push_back(U / s); w.push_back(.5 * w2[i] * U / (s * s)); }
    const double lf = std::log(F / S0);
    std::vector<cplx> psi(u.size());
    for (size_t i = 0; i < u.size(); ++i) {
        const cplx z(.5, u[i]);
        psi[i] = cf_L(z, dts, c, p) * std::exp(-z * lf);
    }
    for (size_t q = 0; q < nk; ++q) {
        const double k = std::log(F / K[q]);
        double sum = 0.;
        for (size_t i = 0; i < u.size(); ++i)
            sum += w[i] * (std::exp(cplx(0., u[i] * k)) * psi[i]).real() / (u[i] * u[i] + .25);
        out[q] = F - std::sqrt(F * K[q]) / M_PI * sum;
    }
    if (F_out) *F_out = F;
}

/* Signed fixed-point sums of the control variate's differences, with
 * y = d 2^-E: q + 2^63 (q = round(y 2^47)) and q2 = round(y^2 2^43), three
 * 25-bit limbs each. */
struct SignedSums {
    std::vector<uint64_t> l;
    int E;
    SignedSums(size_t n, int E_) : l(6 * n, 0), E(E_) {}
    void add(uint32_t o, double d) {
        const double y = std::ldexp(d, -E);
        const __int128 q = (__int128)std::nearbyint(y * 0x1p47);
        const unsigned __int128 qu = (unsigned __int128)(q + ((__int128)1 << 63));
        const unsigned __int128 q2 = (unsigned __int128)std::nearbyint(y * y * 0x1p43);
        const uint64_t M = (1ull << 25) - 1;
        uint64_t *dd = &l[6 * (size_t)o];
        dd[0] += (uint64_t)(qu & M); dd[1] += (uint64_t)((qu >> 25) & M); dd[2] += (uint64_t)(qu >> 50);
        dd[3] += (uint64_t)(q2 & M); dd[4] += (uint64_t)((q2 >> 25) & M); dd[5] += (uint64_t)(q2 >> 50);
    }
};

} // namespace

extern "C" {

/* Raw SHISHUA words of the stream seeded {seed4}. */
void oracle_shishua_words(const uint64_t seed4[4], uint64_t n_words, uint64_t *out) {
    prng_state s;
    uint64_t seed[4] = {seed4[0], seed4[1], seed4[2], seed4[3]};
    prng_init(&s, seed);
    std::vector<uint8_t> blk(128);
    for (uint64_t w = 0; w < n_words; w += 16) {
        prng_gen(&s, blk.data(), 128);
        for (uint64_t k = 0; k < 16 && w + k < n_words; ++k) std::memcpy(&out[w + k], &blk[8 * k], 8);
    }
}

/* Draws of RNG(block_words, seed) on the stream seeded {seed, stream, 0, 0}:
 * kinds[i] = 0 -> get_grand, 1 -> get_urand. */
void oracle_rng_draws(uint32_t seed, uint32_t stream, uint32_t block_words, const uint8_t *kinds, uint64_t n,
                      double *out) {
    OracleRNG rng(block_words, seed, stream);
    for (uint64_t i = 0; i < n; ++i) out[i] = kinds[i] ? rng.urand() : rng.grand();
}

double oracle_ppnd16(double p, int *ifault) { return ppnd16(&p, ifault); }

/* ppnd16 of u = (double)w / (double)UINT64_MAX for each word (RNG.cpp:31-41). */
void oracle_normals(const uint64_t *words, uint64_t n, double *out) {
    for (uint64_t i = 0; i < n; ++i) {
        double u = static_cast<double>(words[i]) / static_cast<double>(UINT64_MAX);
        int ifault = 0;
        out[i] = ppnd16(&u, &ifault);
    }
}
float oracle_logf_c(float x) { return oracle_logf(x); }

/*
 * Per-path stream partition (the GPU engine's): path k uses
 * RNG(block_words, (uint32)(seed + k)) on the stream seeded
 * {seed + k, stream, 0, 0}; option o is priced on paths k < n_paths[o].
 * Outputs per option, over paths [path_lo, path_hi): discounted price, its
 * standard error, and six limb sums (the engine's format: 25-bit limbs of
 * round(y*2^47) and round(y^2*2^43), y = pay 2^-E, 2^(E-1) <= S0 < 2^E).
 * params7 = {v0, theta(v_m), rho, kappa, sigma, r, q}; HParams order,
 * src/inc/HDistribution.h:9-24.  step_mode 0 = the reference's T_i/steps
 * stepping; 1 = max(5, round(steps_per_year*T_i)) steps per maturity.
 */
int oracle_price_paths(const double *params7, double S0, uint32_t n_opts, const double *strike, const double *T,
                       const uint8_t *kind, const uint64_t *n_paths, uint32_t step_mode, uint32_t steps,
                       double steps_per_year, uint32_t seed, uint32_t stream, uint32_t block_words, uint64_t path_lo,
                       uint64_t path_hi, int n_threads, double *price, double *stderr_out, uint64_t *limbs_out) {
    Problem pr;
    int rc = build_problem(pr, params7, S0, n_opts, strike, T, kind, n_paths, step_mode, steps, steps_per_year);
    if (rc) return rc;
    if (block_words == 0 || (block_words * 8) % 128 != 0) return 4;  // RNG.cpp:10
    // last maturity index each path needs
    std::vector<uint64_t> mat_paths(pr.T.size(), 0);
    for (size_t j = 0; j < pr.T.size(); ++j)
        for (uint32_t o : pr.opts[j]) mat_paths[j] = std::max(mat_paths[j], n_paths[o]);
    uint64_t n_max = *std::max_element(mat_paths.begin(), mat_paths.end());
    path_hi = std::min(path_hi, n_max);
    int nt = n_threads > 0 ? n_threads : 1;
    const int E = pay_exponent(S0);
    std::vector<ExactSums> part(nt, ExactSums(n_opts, E));
#pragma omp parallel for num_threads(nt) schedule(dynamic, 64)
    for (int64_t k = (int64_t)path_lo; k < (int64_t)path_hi; ++k) {
#ifdef _OPENMP
        ExactSums &acc = part[omp_get_thread_num()];
#else
        ExactSums &acc = part[0];
#endif
        size_t last = 0;
        for (size_t j = 0; j < pr.T.size(); ++j)
            if (mat_paths[j] > (uint64_t)k) last = j;
        OracleRNG rng(block_words, static_cast<uint32_t>(seed + (uint64_t)k), stream);
        run_path(pr, rng, false, [&](size_t j, double asian, double euro, double) {
            for (uint32_t o : pr.opts[j])
                if ((uint64_t)k < n_paths[o]) acc.add(o, payoff_of(pr, o, asian, euro));
            return j < last;
        });
    }
    for (int t = 1; t < nt; ++t) part[0].merge(part[t]);
    for (uint32_t o = 0; o < n_opts; ++o) {
        const uint64_t *d = &part[0].l[6 * (size_t)o];
        if (limbs_out) std::memcpy(&limbs_out[6 * (size_t)o], d, 6 * sizeof(uint64_t));
        const unsigned __int128 s1 = ExactSums::value(d), s2 = ExactSums::value(d + 3);
        const uint64_t hi = std::min<uint64_t>(n_paths[o], path_hi);
        const double n = hi > path_lo ? (double)(hi - path_lo) : 0.0;
        const long double mean = n > 0 ? std::ldexp((long double)s1, E - 47) / n : 0.L;
        const long double m2 = n > 0 ? std::ldexp((long double)s2, 2 * E - 43) / n : 0.L;
        long double var = n > 1 ? (m2 - mean * mean) * n / (n - 1) : 0.L;
        if (var < 0) var = 0;
        const double disc = std::exp(-pr.p.r * T[o]);
        if (price) price[o] = disc * (double)mean;
        if (stderr_out) stderr_out[o] = n > 0 ? disc * std::sqrt((double)(var / n)) : 0.0;
    }
    return 0;
}

/*
 * Branch counts of the per-path partition: over paths [path_lo, path_hi),
 * each walked to its last needed maturity as oracle_price_paths walks it,
 * counts[0] = QE steps on the quadratic branch (HSimulation.tpp:63-68),
 * counts[1] = all QE steps.  The GPU kernels report the same two numbers
 * (the executed path-steps of a launch and its quadratic-branch steps).
 */
int oracle_branch_counts(const double *params7, double S0, uint32_t n_opts, const double *strike, const double *T,
                         const uint8_t *kind, const uint64_t *n_paths, uint32_t step_mode, uint32_t steps,
                         double steps_per_year, uint32_t seed, uint32_t stream, uint32_t block_words,
                         uint64_t path_lo, uint64_t path_hi, int n_threads, uint64_t *counts) {
    Problem pr;
    int rc = build_problem(pr, params7, S0, n_opts, strike, T, kind, n_paths, step_mode, steps, steps_per_year);
    if (rc) return rc;
    if (block_words == 0 || (block_words * 8) % 128 != 0) return 4;  // RNG.cpp:10
    std::vector<uint64_t> mat_paths(pr.T.size(), 0);
    for (size_t j = 0; j < pr.T.size(); ++j)
        for (uint32_t o : pr.opts[j]) mat_paths[j] = std::max(mat_paths[j], n_paths[o]);
    const uint64_t n_max = *std::max_element(mat_paths.begin(), mat_paths.end());
    path_hi = std::min(path_hi, n_max);
    const int nt = n_threads > 0 ? n_threads : 1;
    std::vector<uint64_t> part(2 * (size_t)nt, 0);
#pragma omp parallel for num_threads(nt) schedule(dynamic, 64)
    for (int64_t k = (int64_t)path_lo; k < (int64_t)path_hi; ++k) {
#ifdef _OPENMP
        uint64_t *c = &part[2 * (size_t)omp_get_thread_num()];
#else
        uint64_t *c = &part[0];
#endif
        size_t last = 0;
        for (size_t j = 0; j < pr.T.size(); ++j)
            if (mat_paths[j] > (uint64_t)k) last = j;
        OracleRNG rng(block_words, static_cast<uint32_t>(seed + (uint64_t)k), stream);
        run_path(pr, rng, false, [&](size_t j, double, double, double) { return j < last; }, c);
    }
    counts[0] = counts[1] = 0;
    for (int t = 0; t < nt; ++t) { counts[0] += part[2 * (size_t)t]; counts[1] += part[2 * (size_t)t + 1]; }
    return 0;
}

/*
 * Final values per path (debug / localisation): for each path k in
 * [path_lo, path_hi) and each distinct maturity j, the Asian average and
 * the interpolated terminal spot, NaN where the path stops earlier.
 * out arrays are [(k - path_lo) * n_mats + j]; n_mats_out receives the count.
 */
int oracle_path_finals(const double *params7, double S0, uint32_t n_opts, const double *strike, const double *T,
                       const uint8_t *kind, const uint64_t *n_paths, uint32_t step_mode, uint32_t steps,
                       double steps_per_year, uint32_t seed, uint32_t stream, uint32_t block_words, uint64_t path_lo,
                       uint64_t path_hi, double *asian_out, double *euro_out, uint32_t *n_mats_out) {
    Problem pr;
    int rc = build_problem(pr, params7, S0, n_opts, strike, T, kind, n_paths, step_mode, steps, steps_per_year);
    if (rc) return rc;
    const size_t m = pr.T.size();
    if (n_mats_out) *n_mats_out = (uint32_t)m;
    std::vector<uint64_t> mat_paths(m, 0);
    for (size_t j = 0; j < m; ++j)
        for (uint32_t o : pr.opts[j]) mat_paths[j] = std::max(mat_paths[j], n_paths[o]);
    for (uint64_t k = path_lo; k < path_hi; ++k) {
        size_t last = 0;
        bool any = false;
        for (size_t j = 0; j < m; ++j)
            if (mat_paths[j] > k) { last = j; any = true; }
        for (size_t j = 0; j < m; ++j) {
            asian_out[(k - path_lo) * m + j] = NAN;
            euro_out[(k - path_lo) * m + j] = NAN;
        }
        if (!any) continue;
        OracleRNG rng(block_words, static_cast<uint32_t>(seed + k), stream);
        run_path(pr, rng, false, [&](size_t j, double asian, double euro, double) {
            asian_out[(k - path_lo) * m + j] = asian;
            euro_out[(k - path_lo) * m + j] = euro;
            return j < last;
        });
    }
    return 0;
}

/*
 * The reference's own partition (HSimulation.tpp:23-49): n_threads "threads",
 * each with RNG(buf_words, 1<<tid) and n/n_threads consecutive paths sharing
 * that stream, the trailing step included, every path pricing every option,
 * prices[o] = sum over paths of payoff/n in path order (undiscounted, as the
 * reference returns).  With n_threads == 1 and buf_words == 2^20 this equals
 * the untouched HSimulation::price<> on one OpenMP thread.  `omp_threads`
 * runs the partition's threads concurrently (each into its own array,
 * merged in thread order).  Returns the number of paths simulated.
 */
int64_t oracle_price_reference_partition(const double *params7, double S0, uint32_t n_opts, const double *strike,
                                         const double *T, const uint8_t *kind, uint32_t steps, uint32_t n_sims,
                                         int n_threads, uint32_t buf_words, int omp_threads, double *prices) {
    std::vector<uint64_t> all(n_opts, n_sims);
    Problem pr;
    if (build_problem(pr, params7, S0, n_opts, strike, T, kind, all.data(), 0, steps, 252.)) return -1;
    const int nt = n_threads > 0 ? n_threads : 1;
    const uint32_t local_sims = n_sims / (uint32_t)nt;                  // tpp:27
    std::vector<std::vector<double>> local(nt, std::vector<double>(n_opts, 0.));
#pragma omp parallel for num_threads(omp_threads > 0 ? omp_threads : 1) schedule(static, 1)
    for (int t = 0; t < nt; ++t) {
        OracleRNG rng(buf_words, 1u << t);                              // tpp:28
        std::vector<double> &pr_t = local[t];
        for (uint32_t i = 0; i < local_sims; ++i)
            run_path(pr, rng, true, [&](size_t j, double asian, double euro, double) {
                for (uint32_t o : pr.opts[j]) pr_t[o] += payoff_of(pr, o, asian, euro) / n_sims;  // tpp:40
                return true;
            });
    }
    for (uint32_t o = 0; o < n_opts; ++o) {
        double s = 0.;
        for (int t = 0; t < nt; ++t) s += local[t][o];
        prices[o] = s;
    }
    return (int64_t)local_sims * nt;
}


/*
 * E[(G - K)^+] of the control variate for every Asian option (kind 0), the
 * other options 0; undiscounted.  The same step modes as oracle_price_paths.
 */
int oracle_geo_calls(const double *params7, double S0, uint32_t n_opts, const double *strike, const double *T,
                     const uint8_t *kind, uint32_t step_mode, uint32_t steps, double steps_per_year, double *out) {
    Problem pr;
    std::vector<uint64_t> np(n_opts, 1);
    int rc = build_problem(pr, params7, S0, n_opts, strike, T, kind, np.data(), step_mode, steps, steps_per_year);
    if (rc) return rc;
    std::vector<double> dts, c;
    for (size_t j = 0; j < pr.T.size(); ++j) {
        std::vector<double> K;
        for (uint32_t o : pr.opts[j]) K.push_back(strike[o]);
        std::vector<double> res(K.size());
        cv_schedule(pr, j, dts, c);
        cv_geo_calls(pr.p, S0, dts, c, K.data(), K.size(), res.data(), nullptr);
        for (size_t i = 0; i < K.size(); ++i) out[pr.opts[j][i]] = kind[pr.opts[j][i]] == 0 ? res[i] : 0.;
    }
    return 0;
}

/*
 * oracle_price_paths with the geometric control variate on the Asian
 * options.  Per Asian option the paths give the sums of a = (A - K)^+,
 * g = (G - K)^+ and d = a - g; Cov(a, g) = (Var a + Var g - Var d) / 2,
 * beta = Cov / Var g, and the price is exp(-r T) (mean a - beta (mean g -
 * E[g])) with the standard error of a - beta g.  Europeans as before.
 */
int oracle_price_paths_cv(const double *params7, double S0, uint32_t n_opts, const double *strike, const double *T,
                          const uint8_t *kind, const uint64_t *n_paths, uint32_t step_mode, uint32_t steps,
                          double steps_per_year, uint32_t seed, uint32_t stream, uint32_t block_words,
                          uint64_t path_lo, uint64_t path_hi, int n_threads, double *price, double *stderr_out) {
    Problem pr;
    int rc = build_problem(pr, params7, S0, n_opts, strike, T, kind, n_paths, step_mode, steps, steps_per_year);
    if (rc) return rc;
    if (block_words == 0 || (block_words * 8) % 128 != 0) return 4;
    std::vector<double> eg(n_opts, 0.);
    rc = oracle_geo_calls(params7, S0, n_opts, strike, T, kind, step_mode, steps, steps_per_year, eg.data());
    if (rc) return rc;
    std::vector<uint64_t> mat_paths(pr.T.size(), 0);
    for (size_t j = 0; j < pr.T.size(); ++j)
        for (uint32_t o : pr.opts[j]) mat_paths[j] = std::max(mat_paths[j], n_paths[o]);
    const uint64_t n_max = *std::max_element(mat_paths.begin(), mat_paths.end());
    path_hi = std::min(path_hi, n_max);
    const int nt = n_threads > 0 ? n_threads : 1;
    // per thread: a sums (ExactSums [o]), g sums (ExactSums [o]), d sums (SignedSums [o])
    const int E = pay_exponent(S0);
    std::vector<ExactSums> pa(nt, ExactSums(n_opts, E)), pg(nt, ExactSums(n_opts, E));
    std::vector<SignedSums> pd(nt, SignedSums(n_opts, E));
#pragma omp parallel for num_threads(nt) schedule(dynamic, 64)
    for (int64_t k = (int64_t)path_lo; k < (int64_t)path_hi; ++k) {
#ifdef _OPENMP
        const int tn = omp_get_thread_num();
#else
        const int tn = 0;
#endif
        size_t last = 0;
        for (size_t j = 0; j < pr.T.size(); ++j)
            if (mat_paths[j] > (uint64_t)k) last = j;
        OracleRNG rng(block_words, static_cast<uint32_t>(seed + (uint64_t)k), stream);
        run_path(pr, rng, false, [&](size_t j, double asian, double euro, double geo) {
            for (uint32_t o : pr.opts[j]) {
                if ((uint64_t)k >= n_paths[o]) continue;
                const double a = payoff_of(pr, o, asian, euro);
                pa[tn].add(o, a);
                if (pr.kind[o] == 0) {
                    const double g = std::max(0., geo - pr.strike[o]);
                    pg[tn].add(o, g);
                    pd[tn].add(o, a - g);
                }
            }
            return j < last;
        });
    }
    for (int t = 1; t < nt; ++t) {
        pa[0].merge(pa[t]);
        pg[0].merge(pg[t]);
        for (size_t i = 0; i < pd[0].l.size(); ++i) pd[0].l[i] += pd[t].l[i];
    }
    for (uint32_t o = 0; o < n_opts; ++o) {
        const uint64_t hi = std::min<uint64_t>(n_paths[o], path_hi);
        const uint64_t cnt = hi > path_lo ? hi - path_lo : 0;
        const long double n = (long double)cnt;
        const double disc = std::exp(-pr.p.r * T[o]);
        auto moments = [&](const uint64_t *d, bool biased, long double &mean, long double &var) {
            __int128 s1 = (__int128)ExactSums::value(d);
            if (biased) s1 -= (__int128)cnt << 63;
            mean = cnt ? std::ldexp((long double)s1, E - 47) / n : 0.L;
            const long double m2 = cnt ? std::ldexp((long double)ExactSums::value(d + 3), 2 * E - 43) / n : 0.L;
            var = cnt > 1 ? (m2 - mean * mean) * n / (n - 1) : 0.L;
            if (var < 0) var = 0;
        };
        long double ma, va;
        moments(&pa[0].l[6 * (size_t)o], false, ma, va);
        long double mean = ma, var = va;
        if (pr.kind[o] == 0) {
            long double mg, vg, md, vd;
            moments(&pg[0].l[6 * (size_t)o], false, mg, vg);
            moments(&pd[0].l[6 * (size_t)o], true, md, vd);
            const long double cov = (va + vg - vd) / 2;
            const long double beta = vg > 0 ? cov / vg : 0.L;
            mean = ma - beta * (mg - (long double)eg[o]);
            var = vg > 0 ? va - cov * cov / vg : va;
            if (var < 0) var = 0;
        }
        price[o] = disc * (double)mean;
        if (stderr_out) stderr_out[o] = cnt ? disc * std::sqrt((double)(var / n)) : 0.0;
    }
    return 0;
}

} // extern "C"
