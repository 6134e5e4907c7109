// TEST INFRASTRUCTURE: drives the engine's host planner (csrc/hexo_plan.cpp)
// and host finaliser under AddressSanitizer and UndefinedBehaviorSanitizer
// (tests/test_host_sanitizers.py builds it; no CUDA is involved).  Seeded
// random requests shaped like the uneven batch, in both step modes, with and
// without the control variate, whole and as path-range shards, are planned
// into one batch, and the tile list is checked to cover every path exactly
// once; malformed requests must be refused with an error status.  Exit code
// 0 when every check holds.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <random>
#include <string>
#include <vector>

#include "hexo_plan.h"

using namespace hexo;

static int fails = 0;
#define EXPECT(c)                                                         \
    do {                                                                  \
        if (!(c)) { std::fprintf(stderr, "check failed: %s (line %d)\n", #c, __LINE__); ++fails; } \
    } while (0)

int main() {
    std::mt19937_64 rng(2);
    std::uniform_real_distribution<double> U(0.0, 1.0);
    for (uint32_t round = 0; round < 4; ++round) {
        hexo_mc_cfg cfg{};
        cfg.n_paths = 1000;
        cfg.step_mode = round % 2 ? HEXO_STEP_REFERENCE : HEXO_STEP_GRID;
        cfg.steps = 37;
        cfg.steps_per_year = 252.0;
        cfg.rng_block_words = 16;
        cfg.precision = round / 2;
        cfg.control_variate = round == 3 ? 1u : 0u;
        BatchPlan bp;
        std::vector<SetPlan> plans;
        std::vector<std::vector<hexo_option>> store;
        const uint32_t n_sets = 12;
        uint32_t n_user = 0, n_cv = 0;
        std::vector<uint32_t> n_opts(n_sets);
        for (uint32_t s = 0; s < n_sets; ++s) n_opts[s] = 1 + (uint32_t)(U(rng) * 150);
        for (uint32_t s = 0; s < n_sets; ++s) n_user += n_opts[s];
        uint32_t out_base = 0, cv_base = n_user;
        for (uint32_t s = 0; s < n_sets; ++s) {
            std::vector<hexo_option> o(n_opts[s]);
            for (auto &x : o) {
                x.strike = 100.0 * std::exp(std::log(0.6) + U(rng) * std::log(1.6 / 0.6));
                x.T = std::max(5.0, std::nearbyint(252.0 * (0.02 + 4.98 * U(rng)))) / 252.0;
                x.payoff = U(rng) < 0.75 ? HEXO_ASIAN_CALL : HEXO_EUROPEAN_CALL;
                x.n_paths = (uint64_t)std::exp2(6.0 + 8.0 * U(rng));
            }
            store.push_back(o);
            hexo_params p{0.01 + 0.08 * U(rng), 0.01 + 0.08 * U(rng), -0.9 + 0.8 * U(rng), 0.5 + 4.5 * U(rng),
                          0.1 + 0.9 * U(rng), 0.05 * U(rng), 0.0};
            SetPlan sp;
            std::string err;
            // every third set as the middle shard of three
            const uint64_t lo = s % 3 == 0 ? 100 : 0, hi = s % 3 == 0 ? 5000 : ~0ull;
            const hexo_status st = plan_set(p, 100.0 * (1.0 + s), store.back().data(), n_opts[s], cfg,
                                            (uint32_t)rng(), s, lo, hi, sp, err);
            EXPECT(st == HEXO_OK);
            if (st != HEXO_OK) continue;
            plans.push_back(sp);
            batch_add(bp, plans.back(), out_base, cv_base);
            out_base += n_opts[s];
            cv_base += 2 * sp.n_cv;
            n_cv += sp.n_cv;
        }
        bp.shape = LaunchShape{128 + 64 * round, 1 + round % 2, 1};
        batch_tiles(bp, plans);
        EXPECT(bp.n_out == n_user + 2 * n_cv);
        // the tiles cover every simulated path of every set exactly once
        std::vector<uint64_t> covered(plans.size(), 0);
        const uint32_t P = bp.shape.paths_per_tile();
        for (const TileDesc &t : bp.tiles) {
            EXPECT(t.set < plans.size());
            if (t.set >= plans.size()) continue;
            const SetPlan &sp = plans[t.set];
            EXPECT(t.path_begin >= sp.path_lo && t.path_begin < sp.path_hi);
            EXPECT(t.seg_count >= 1 && t.seg_count <= sp.segs.size());
            covered[t.set] += std::min<uint64_t>(P, sp.path_hi - t.path_begin);
        }
        for (size_t s = 0; s < plans.size(); ++s) EXPECT(covered[s] == plans[s].path_hi - plans[s].path_lo);
        // the host finaliser at every spot exponent
        for (int E = -59; E <= 60; E += 7) {
            const uint64_t l[6] = {rng() >> 40, rng() >> 40, rng() >> 52, rng() >> 40, rng() >> 40, rng() >> 40};
            double price = 0.0, se = 0.0;
            finalize_one(l, 1 + (rng() >> 44), 0.97, E, &price, &se);
            EXPECT(std::isfinite(price) && std::isfinite(se) && price >= 0.0 && se >= 0.0);
        }
    }
    // malformed requests are refused, not planned
    hexo_mc_cfg cfg{};
    cfg.n_paths = 100;
    cfg.steps = 10;
    const hexo_params ok{0.04, 0.04, -0.7, 1.5, 0.5, 0.0, 0.0};
    hexo_option o{100.0, 1.0, HEXO_ASIAN_CALL, 0, 0};
    SetPlan sp;
    std::string err;
    EXPECT(plan_set(ok, 100.0, &o, 1, cfg, 1, 0, 0, ~0ull, sp, err) == HEXO_OK);
    hexo_params nan_p = ok;
    nan_p.sigma = NAN;
    EXPECT(plan_set(nan_p, 100.0, &o, 1, cfg, 1, 0, 0, ~0ull, sp, err) != HEXO_OK);
    EXPECT(plan_set(ok, 0x1p60, &o, 1, cfg, 1, 0, 0, ~0ull, sp, err) != HEXO_OK);
    EXPECT(plan_set(ok, -1.0, &o, 1, cfg, 1, 0, 0, ~0ull, sp, err) != HEXO_OK);
    EXPECT(plan_set(ok, 100.0, &o, 0, cfg, 1, 0, 0, ~0ull, sp, err) != HEXO_OK);
    hexo_option bad = o;
    bad.T = -1.0;
    EXPECT(plan_set(ok, 100.0, &bad, 1, cfg, 1, 0, 0, ~0ull, sp, err) != HEXO_OK);
    bad = o;
    bad.payoff = 9;
    EXPECT(plan_set(ok, 100.0, &bad, 1, cfg, 1, 0, 0, ~0ull, sp, err) != HEXO_OK);
    bad = o;
    bad.n_paths = 1ull << 40;
    EXPECT(plan_set(ok, 100.0, &bad, 1, cfg, 1, 0, 0, ~0ull, sp, err) != HEXO_OK);
    hexo_mc_cfg long_cfg = cfg;
    long_cfg.steps = 1u << 25;   // a schedule beyond the per-set step limit
    EXPECT(plan_set(ok, 100.0, &o, 1, long_cfg, 1, 0, 0, ~0ull, sp, err) != HEXO_OK);
    std::printf("%d failed checks\n", fails);
    return fails == 0 ? 0 : 1;
}
