// The reference's call through the drop-in shim (include/hexo/reference_compat.h):
// builds option chains as src/Main.cpp does and prices them with
// HSimulation::price<hexo::GpuQE<Contract>>, printing the prices as hex floats.
// Built with -DHEXO_COMPAT_STANDALONE_TYPES, or against the reference's own
// headers (src/inc) where they exist.
#include <cstdio>
#include <cstdlib>
#include <list>
#include <vector>
#ifndef HEXO_COMPAT_STANDALONE_TYPES
#include "HSimulation.h"
#include "AsianContract.h"
#include "VanillaContract.h"
#endif
#include "hexo/reference_compat.h"

int main(int argc, char **argv) {
    const HParams p{0.04, 0.04, -0.7, 1.5, 0.5};
    const double T[3] = {0.25, 0.5, 1.0};
    const double K[3][2] = {{95.0, 105.0}, {100.0, 110.0}, {90.0, 100.0}};
    unsigned n_opts = 0;
    // chains in the given order of maturities, as WebAPI.cpp builds them (options_chain is move-only)
    auto make = [&](const int *order, std::list<options_chain> &out) {
        for (int i = 0; i < 3; ++i) {
            const int c = order[i];
            out.emplace_back((unsigned)(T[c] * 252.0), T[c]);
            for (int k = 0; k < 2; ++k) {
                option o{};
                o.strike = K[c][k];
                out.back().options.push_back(o);
            }
        }
    };
    const int inc[3] = {0, 1, 2}, dec[3] = {2, 1, 0};
    std::list<options_chain> chains, bad;
    make(inc, chains);
    make(dec, bad);
    n_opts = 6;
    const unsigned n_sims = argc > 1 ? (unsigned)std::atoi(argv[1]) : 20000u, steps = 63;
    try {
        const std::vector<ffloat> a = HSimulation::price<hexo::GpuQE<AAsianCallNonAdaptive>>(p, 100.0, chains, n_sims, n_opts, steps);
        const std::vector<ffloat> e = HSimulation::price<hexo::GpuQE<EuropeanCallNonAdaptive>>(p, 100.0, chains, n_sims, n_opts, steps);
        for (double x : a) std::printf("asian %a\n", x);
        for (double x : e) std::printf("euro %a\n", x);
        // a chain list out of maturity order is refused with std::runtime_error
        try {
            HSimulation::price<hexo::GpuQE<AAsianCallNonAdaptive>>(p, 100.0, bad, n_sims, n_opts, steps);
            std::printf("unordered accepted\n");
        } catch (const std::runtime_error &) {
            std::printf("unordered refused\n");
        }
    } catch (const std::exception &ex) {
        std::printf("error %s\n", ex.what());
        return 1;
    }
    return 0;
}
