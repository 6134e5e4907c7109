/*
 * ORACLE / TEST INFRASTRUCTURE ONLY.
 *
 * Thin C entry points over the reference's own, unmodified sources, compiled
 * by oracle/Makefile from the reference checkout (src/RNG.cpp and the header
 * templates src/inc/HSimulation.h + src/HSimulation.tpp,
 * src/inc/AsianContract.h, src/inc/VanillaContract.h) together with the
 * project's SHISHUA (oracle/shishua.h) and AS241 restatement (oracle/as241.c),
 * which replace the two pieces the reference does not ship in compilable form.
 * The result, oracle/_ref/libhexo_ref.so, exists only where the reference
 * checkout exists; it pins the oracle port and generates tests/golden/.
 *
 *   ref_price          HSimulation::price<HQEAnderson<ffloat, Contract>>
 *                      (src/inc/HSimulation.h:61-63), untouched.
 *   ref_rng_draws      the reference RNG class (src/inc/RNG.h:17-52).
 *   ref_paths          per-path streams driven through the reference's own
 *                      HQEAnderson/contract classes: the loop body of
 *                      HSimulation.tpp:30-46 for one path, with
 *                      RNG(block_words, seed + k) per path.
 */
#include <list>
#include <vector>
#include <cstdint>
#include <cmath>
#include "HSimulation.h"
#include "AsianContract.h"
#include "VanillaContract.h"

using namespace HSimulation;

namespace {
std::list<options_chain> make_chains(uint32_t n_chains, const double *T, const uint32_t *opts_per_chain,
                                     const double *strikes) {
    std::list<options_chain> chains;
    uint32_t o = 0;
    for (uint32_t c = 0; c < n_chains; ++c) {
        options_chain ch(0u, T[c]);
        for (uint32_t i = 0; i < opts_per_chain[c]; ++i) {
            option op{};
            op.strike = strikes[o++];
            op.volume = 1;
            ch.options.push_back(op);
            ch.min_strike = std::min(ch.min_strike, op.strike);
            ch.max_strike = std::max(ch.max_strike, op.strike);
        }
        chains.push_back(std::move(ch));
    }
    return chains;
}

template <class Scheme>
void one_path(const HParams &p, double S, const std::list<options_chain> &chains, RNG &rng, uint32_t steps,
              uint32_t n_opts, std::vector<double> &payoff_out) {
    const SDE_state<2> initial_state = {{S, p.v_0}, {S, p.v_0}, .0, .0};
    Scheme heston_sde(p, chains.begin()->time_to_expiry / steps, &rng, initial_state);
    unsigned int opts_priced = 0;
    auto earliest_unpriced = chains.begin();
    heston_sde.update_earliest(earliest_unpriced->time_to_expiry, steps);
    heston_sde.reset();
    for (++(heston_sde = initial_state); opts_priced < n_opts; ++heston_sde) {
        while (heston_sde >= earliest_unpriced->time_to_expiry && opts_priced < n_opts) {
            unsigned int opt_index = 0;
            heston_sde.accumulate_final_value(heston_sde.state);
            for (const auto &opt : earliest_unpriced->options)
                payoff_out[opts_priced + (opt_index++)] = heston_sde.final_payoff(opt.strike);
            if ((opts_priced = opts_priced + earliest_unpriced->options.size()) < n_opts)
                heston_sde.update_earliest((++earliest_unpriced)->time_to_expiry, steps);
        }
        if (opts_priced >= n_opts) break;  // the trailing step only advances this path's own stream
        heston_sde.accumulate_value(heston_sde.state);
    }
}
} // namespace

extern "C" {

/* kind 0 = Asian (AAsianCallNonAdaptive), 1 = European (EuropeanCallNonAdaptive). */
int ref_price(int kind, const double *params5, double S, uint32_t n_chains, const double *T,
              const uint32_t *opts_per_chain, const double *strikes, uint32_t n_sims, uint32_t steps,
              double *out) {
    HParams p{params5[0], params5[1], params5[2], params5[3], params5[4]};
    auto chains = make_chains(n_chains, T, opts_per_chain, strikes);
    uint32_t n_opts = 0;
    for (uint32_t c = 0; c < n_chains; ++c) n_opts += opts_per_chain[c];
    std::vector<ffloat> r = kind == 0
        ? price<HQEAnderson<ffloat, AAsianCallNonAdaptive>>(p, S, chains, n_sims, n_opts, steps)
        : price<HQEAnderson<ffloat, EuropeanCallNonAdaptive>>(p, S, chains, n_sims, n_opts, steps);
    for (uint32_t i = 0; i < n_opts; ++i) out[i] = r[i];
    return 0;
}

void ref_rng_draws(uint32_t seed, uint32_t size, const uint8_t *kinds, uint64_t n, double *out) {
    RNG rng(size, seed);
    for (uint64_t i = 0; i < n; ++i) out[i] = kinds[i] ? rng.get_urand() : rng.get_grand();
}

/* Per-path payoffs (undiscounted) for paths [path_lo, path_hi), path k on
 * RNG(block_words, seed + k); out is [(k - path_lo) * n_opts + o]. */
int ref_paths(int kind, const double *params5, double S, uint32_t n_chains, const double *T,
              const uint32_t *opts_per_chain, const double *strikes, uint32_t steps, uint32_t seed,
              uint32_t block_words, uint64_t path_lo, uint64_t path_hi, double *out) {
    HParams p{params5[0], params5[1], params5[2], params5[3], params5[4]};
    auto chains = make_chains(n_chains, T, opts_per_chain, strikes);
    uint32_t n_opts = 0;
    for (uint32_t c = 0; c < n_chains; ++c) n_opts += opts_per_chain[c];
    std::vector<double> pay(n_opts);
    for (uint64_t k = path_lo; k < path_hi; ++k) {
        RNG rng(block_words, static_cast<unsigned int>(seed + k));
        if (kind == 0)
            one_path<HQEAnderson<ffloat, AAsianCallNonAdaptive>>(p, S, chains, rng, steps, n_opts, pay);
        else
            one_path<HQEAnderson<ffloat, EuropeanCallNonAdaptive>>(p, S, chains, rng, steps, n_opts, pay);
        for (uint32_t o = 0; o < n_opts; ++o) out[(k - path_lo) * n_opts + o] = pay[o];
    }
    return 0;
}

} // extern "C"
