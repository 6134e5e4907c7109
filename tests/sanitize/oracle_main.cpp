// TEST INFRASTRUCTURE: drives the CPU oracle under AddressSanitizer and
// UndefinedBehaviorSanitizer (tests/test_host_sanitizers.py builds it).  Each
// entry point runs on a small problem with ragged path counts, several
// maturities, both payoffs and both step modes; the exit code is non-zero
// when a result is not finite.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <vector>

extern "C" {
int oracle_price_paths(const double *params7, double S0, uint32_t n_opts, const double *strike, const double *T,
                       const uint8_t *kind, const uint64_t *n_paths, uint32_t step_mode, uint32_t steps,
                       double steps_per_year, uint32_t seed, uint32_t stream, uint32_t block_words, uint64_t path_lo,
                       uint64_t path_hi, int n_threads, double *price, double *stderr_out, uint64_t *limbs_out);
int oracle_branch_counts(const double *params7, double S0, uint32_t n_opts, const double *strike, const double *T,
                         const uint8_t *kind, const uint64_t *n_paths, uint32_t step_mode, uint32_t steps,
                         double steps_per_year, uint32_t seed, uint32_t stream, uint32_t block_words,
                         uint64_t path_lo, uint64_t path_hi, int n_threads, uint64_t *counts);
int64_t oracle_price_reference_partition(const double *params7, double S0, uint32_t n_opts, const double *strike,
                                         const double *T, const uint8_t *kind, uint32_t steps, uint32_t n_sims,
                                         int n_threads, uint32_t buf_words, int omp_threads, double *prices);
int oracle_price_paths_cv(const double *params7, double S0, uint32_t n_opts, const double *strike, const double *T,
                          const uint8_t *kind, const uint64_t *n_paths, uint32_t step_mode, uint32_t steps,
                          double steps_per_year, uint32_t seed, uint32_t stream, uint32_t block_words,
                          uint64_t path_lo, uint64_t path_hi, int n_threads, double *price, double *stderr_out);
int oracle_swift_params(const double *p5, double tau, double r, double S, double K_min, double K_max,
                        double trunc_precision, double *out8);
int oracle_swift_price(const double *p5, double tau, double r, double S, const double *strikes, uint32_t n,
                       const double *sp8, double *price_out, double *grad_out);
}

static int bad = 0;
static void check(const std::vector<double> &v, const char *what) {
    for (double x : v)
        if (!std::isfinite(x)) { std::fprintf(stderr, "%s: not finite\n", what); bad = 1; return; }
}

int main() {
    const double p7[7] = {0.05, 0.03, -0.6, 2.0, 0.8, 0.02, 0.01};
    const double K[6] = {80.0, 100.0, 120.0, 90.0, 110.0, 100.0};
    const double T[6] = {0.1, 0.1, 0.5, 0.5, 1.3, 1.3};
    const uint8_t kind[6] = {0, 1, 0, 1, 0, 1};
    const uint64_t np[6] = {1, 37, 300, 513, 64, 1000};
    for (uint32_t mode = 0; mode < 2; ++mode) {
        std::vector<double> price(6), se(6);
        std::vector<uint64_t> limbs(36);
        if (oracle_price_paths(p7, 100.0, 6, K, T, kind, np, mode, 20, 252.0, 7, 3, 16, 0, 1000, 2, price.data(),
                               se.data(), limbs.data()) != 0) return 2;
        check(price, "price_paths");
        check(se, "price_paths se");
        uint64_t counts[2] = {0, 0};
        if (oracle_branch_counts(p7, 100.0, 6, K, T, kind, np, mode, 20, 252.0, 7, 3, 16, 100, 700, 2, counts) != 0)
            return 3;
        if (counts[1] == 0 || counts[0] > counts[1]) return 4;
        std::vector<double> pc(6), sc(6);
        if (oracle_price_paths_cv(p7, 100.0, 6, K, T, kind, np, mode, 20, 252.0, 7, 0, 16, 0, 1000, 2, pc.data(),
                                  sc.data()) != 0) return 5;
        check(pc, "price_paths_cv");
    }
    std::vector<double> ref(6);
    if (oracle_price_reference_partition(p7, 100.0, 6, K, T, kind, 20, 999, 4, 64, 2, ref.data()) < 0) return 6;
    check(ref, "reference partition");
    const double p5[5] = {0.04, 0.05, -0.6, 1.5, 0.5};
    double sp8[8];
    if (oracle_swift_params(p5, 0.5, 0.01, 100.0, 80.0, 120.0, 1e-7, sp8) != 0) return 7;
    std::vector<double> sp(6), sg(30);
    if (oracle_swift_price(p5, 0.5, 0.01, 100.0, K, 6, sp8, sp.data(), sg.data()) != 0) return 8;
    check(sp, "swift price");
    check(sg, "swift gradient");
    return bad;
}
