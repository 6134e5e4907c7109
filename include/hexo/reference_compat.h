/*
 * reference_compat.h: the GB300 engine behind the reference's own C++ entry
 * point.
 *
 * The reference prices through
 *
 *   template<class Scheme> std::vector<ffloat> HSimulation::price(
 *       const HParams& p, const ffloat S, const std::list<options_chain>& all_chains,
 *       unsigned int n_simulations, unsigned int n_opts, unsigned int steps);
 *                                   (src/inc/HSimulation.h:61-63, src/HSimulation.tpp:10-51)
 *
 * with Scheme = HQEAnderson<ffloat, AAsianCallNonAdaptive> or
 * HQEAnderson<ffloat, EuropeanCallNonAdaptive> (src/inc/AsianContract.h:49,
 * src/inc/VanillaContract.h:41), called from src/Main.cpp:88.  Including this
 * header after the reference's HSimulation.h adds the scheme
 * hexo::GpuQE<Contract>; the call site changes only its template argument:
 *
 *   auto prices = HSimulation::price<hexo::GpuQE<AAsianCallNonAdaptive>>(p, S, chains, 100000, n, 1000);
 *
 * Semantics kept: the reference's step schedule (maturity i reached with
 * width T_i/steps, time accumulated in double), its QE scheme, contracts and
 * AS241; undiscounted mean payoffs in flattened chain order (no rate, as the
 * reference has none); chains must be in increasing maturity order
 * (checked, as HSimulation.tpp:14-21 does in debug builds); a failure throws
 * std::runtime_error, as AsianContract.h:30 does.  What differs: every path
 * k draws from its own RNG(16, seed + k) stream instead of one stream per
 * OpenMP thread, so results are deterministic (the reference's threads race
 * on the shared result vector, HSimulation.tpp:22,40), and all n_simulations
 * paths are simulated (the reference drops n mod threads, tpp:27).
 * hexo::compat_seed() sets the seed (default 1, the reference's first
 * thread seed 1<<0).
 *
 * Define HEXO_COMPAT_STANDALONE_TYPES to use this header without the
 * reference's headers (it then declares minimal HParams / option /
 * options_chain / ffloat with the reference's layouts).
 */
#ifndef HEXO_REFERENCE_COMPAT_H
#define HEXO_REFERENCE_COMPAT_H

#include <cstdint>
#include <list>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "../hexo_mc.h"

#ifdef HEXO_COMPAT_STANDALONE_TYPES
typedef double ffloat;
typedef struct HP { ffloat v_0, v_m, rho, kappa, sigma; } HParams;
typedef struct { ffloat price, bid, strike; int64_t volume; } option;
typedef struct OptionsChain {
    std::vector<option> options;
    unsigned int days_to_expiry;
    ffloat time_to_expiry, max_strike, min_strike;
    OptionsChain(unsigned int days_until, ffloat time_until)
        : days_to_expiry(days_until), time_to_expiry(time_until), max_strike(-1.7976931348623157e308),
          min_strike(1.7976931348623157e308) {}
    OptionsChain(OptionsChain &&) = default;
} options_chain;
class AAsianCallNonAdaptive;
class EuropeanCallNonAdaptive;
namespace HSimulation {
template <class Scheme>
std::vector<ffloat> price(const HParams &p, const ffloat S, const std::list<options_chain> &all_chains,
                          unsigned int n_simulations, unsigned int n_opts, unsigned int steps);
}
#endif

namespace hexo {

template <class Contract> struct GpuQE {};

template <class Contract> struct payoff_of;
template <> struct payoff_of<AAsianCallNonAdaptive> { static constexpr uint32_t value = HEXO_ASIAN_CALL; };
template <> struct payoff_of<EuropeanCallNonAdaptive> { static constexpr uint32_t value = HEXO_EUROPEAN_CALL; };

inline uint32_t &compat_seed() {
    static uint32_t seed = 1u;
    return seed;
}

// One engine context per process, created on first use on the current device.
inline hexo_ctx *compat_context() {
    static std::once_flag once;
    static hexo_ctx *ctx = nullptr;
    static hexo_status st = HEXO_OK;
    if (hexo_abi_version() != HEXO_ABI_VERSION)
        throw std::runtime_error("hexo: libhexo_mc.so was built for another version of hexo_mc.h");
    std::call_once(once, [] { st = hexo_ctx_create(&ctx, nullptr); });
    if (st != HEXO_OK || ctx == nullptr)
        throw std::runtime_error(std::string("hexo: cannot create engine context: ") + hexo_status_string(st));
    return ctx;
}

template <class Contract>
std::vector<ffloat> compat_price(const HParams &p, const ffloat S, const std::list<options_chain> &all_chains,
                                 unsigned int n_simulations, unsigned int n_opts, unsigned int steps) {
    std::vector<hexo_option> opts;
    opts.reserve(n_opts);
    double prev = -1.0;
    for (const options_chain &ch : all_chains) {
        if (!(ch.time_to_expiry > prev)) throw std::runtime_error("hexo: chains must have increasing expiries");
        prev = ch.time_to_expiry;
        for (const option &o : ch.options) {
            if (opts.size() == n_opts) break;
            hexo_option h{};
            h.strike = o.strike;
            h.T = ch.time_to_expiry;
            h.payoff = payoff_of<Contract>::value;
            h.n_paths = 0;
            opts.push_back(h);
        }
    }
    hexo_params hp{p.v_0, p.v_m, p.rho, p.kappa, p.sigma, 0.0, 0.0};
    hexo_mc_cfg cfg;
    hexo_mc_cfg_default(&cfg);
    cfg.n_paths = n_simulations;
    cfg.step_mode = HEXO_STEP_REFERENCE;
    cfg.steps = steps;
    cfg.seed = compat_seed();
    cfg.precision = HEXO_FP64;
    std::vector<double> out(opts.size(), 0.0);
    hexo_ctx *ctx = compat_context();
    const hexo_status st = hexo_price(ctx, &hp, S, opts.data(), (uint32_t)opts.size(), &cfg, out.data(), nullptr);
    if (st != HEXO_OK) {
        char msg[256] = {0};
        hexo_ctx_last_error(ctx, msg, sizeof msg);
        throw std::runtime_error(std::string("hexo: ") + hexo_status_string(st) + ": " + msg);
    }
    std::vector<ffloat> prices(n_opts, 0.0);
    for (size_t i = 0; i < out.size(); ++i) prices[i] = out[i];
    return prices;
}

} // namespace hexo

namespace HSimulation {
template <>
inline std::vector<ffloat> price<hexo::GpuQE<AAsianCallNonAdaptive>>(
    const HParams &p, const ffloat S, const std::list<options_chain> &all_chains, unsigned int n_simulations,
    unsigned int n_opts, unsigned int steps) {
    return hexo::compat_price<AAsianCallNonAdaptive>(p, S, all_chains, n_simulations, n_opts, steps);
}
template <>
inline std::vector<ffloat> price<hexo::GpuQE<EuropeanCallNonAdaptive>>(
    const HParams &p, const ffloat S, const std::list<options_chain> &all_chains, unsigned int n_simulations,
    unsigned int n_opts, unsigned int steps) {
    return hexo::compat_price<EuropeanCallNonAdaptive>(p, S, all_chains, n_simulations, n_opts, steps);
}
} // namespace HSimulation

#endif
