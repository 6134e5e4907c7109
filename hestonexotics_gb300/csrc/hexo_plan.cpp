// Host-side planning of pricing requests (no CUDA).
#include "hexo_plan.h"
#include "hexo_final.h"
#include <algorithm>
#include <cmath>
#include <numeric>
#include <sstream>

namespace hexo {

namespace {
bool finite(double x) { return std::isfinite(x); }
constexpr uint64_t kMaxStepsPerSet = 1ull << 24;
constexpr uint64_t kMaxPaths = 0xFFFFFFFFull;  // stream seeds are seed + k modulo 2^32
}

hexo_status plan_set(const hexo_params &p, double S0, const hexo_option *opts, uint32_t n_opts,
                     const hexo_mc_cfg &cfg, uint32_t seed, uint32_t stream, uint64_t path_lo, uint64_t path_hi,
                     SetPlan &out, std::string &err) {
    out = SetPlan();
    if (n_opts == 0 || opts == nullptr) { err = "request has no options"; return HEXO_ERR_INVALID; }
    const double pv[7] = {p.v0, p.theta, p.rho, p.kappa, p.sigma, p.r, p.q};
    for (double x : pv)
        if (!finite(x)) { err = "non-finite Heston parameter"; return HEXO_ERR_INVALID; }
    if (!(p.v0 >= 0.0) || !(p.theta > 0.0) || !(p.kappa > 0.0) || !(p.sigma > 0.0) || !(std::fabs(p.rho) <= 1.0)) {
        err = "Heston parameters out of range (need v0 >= 0, theta > 0, kappa > 0, sigma > 0, |rho| <= 1)";
        return HEXO_ERR_INVALID;
    }
    if (!finite(S0) || !(S0 >= 0x1p-60) || !(S0 < 0x1p60)) { err = "S0 must be in [2^-60, 2^60)"; return HEXO_ERR_INVALID; }
    const uint32_t block_words = cfg.rng_block_words ? cfg.rng_block_words : 16u;
    if (block_words != 16u) {
        err = "rng_block_words other than 16 is not supported by the GPU engine";
        return HEXO_ERR_UNSUPPORTED;
    }
    const double spy = cfg.steps_per_year > 0.0 ? cfg.steps_per_year : 252.0;
    if (cfg.step_mode > 1u) { err = "unknown step mode"; return HEXO_ERR_INVALID; }
    if (cfg.step_mode == HEXO_STEP_REFERENCE && cfg.steps == 0) { err = "steps must be positive"; return HEXO_ERR_INVALID; }
    if (cfg.precision > 1u) { err = "unknown precision"; return HEXO_ERR_INVALID; }
    if (cfg.control_variate > 1u) { err = "unknown control variate"; return HEXO_ERR_INVALID; }

    // Group options by distinct maturity, ascending; stable within a maturity.
    std::vector<uint32_t> idx(n_opts);
    std::iota(idx.begin(), idx.end(), 0u);
    for (uint32_t i = 0; i < n_opts; ++i) {
        const hexo_option &o = opts[i];
        if (!finite(o.T) || !(o.T > 0.0)) { err = "option maturity must be positive and finite"; return HEXO_ERR_INVALID; }
        if (!finite(o.strike)) { err = "option strike must be finite"; return HEXO_ERR_INVALID; }
        if (o.payoff > 1u) { err = "unknown payoff type"; return HEXO_ERR_INVALID; }
        const uint64_t np = o.n_paths ? o.n_paths : cfg.n_paths;
        if (np == 0 || np > kMaxPaths) { err = "paths per option must be in [1, 2^32)"; return HEXO_ERR_INVALID; }
    }
    std::stable_sort(idx.begin(), idx.end(), [&](uint32_t a, uint32_t b) { return opts[a].T < opts[b].T; });
    std::vector<double> T;
    for (uint32_t i : idx) {
        if (T.empty() || T.back() != opts[i].T) {
            T.push_back(opts[i].T);
            uint32_t n = cfg.steps;
            if (cfg.step_mode == HEXO_STEP_GRID) {
                const double g = std::nearbyint(spy * opts[i].T);
                if (!(g < 4.0e9)) { err = "grid step count too large"; return HEXO_ERR_INVALID; }
                n = (uint32_t)std::max(5.0, g);
            }
            out.mat_steps.push_back(n);
            MatDesc md{};
            md.T = opts[i].T;
            md.opt_begin = (uint32_t)out.opts.size();
            out.mats.push_back(md);
            out.mat_paths.push_back(0);
        }
        OptDesc od{};
        od.strike = opts[i].strike;
        od.f_strike = (float)opts[i].strike;
        od.kind = opts[i].payoff;
        od.n_paths = opts[i].n_paths ? opts[i].n_paths : cfg.n_paths;
        od.out_index = i;
        out.opts.push_back(od);
        out.opt_disc.push_back(std::exp(-p.r * opts[i].T));
        if (cfg.control_variate && od.kind == HEXO_ASIAN_CALL) {
            // the geometric call and the difference follow their Asian option, in
            // request-local slots n_opts + 2 c and n_opts + 2 c + 1
            for (uint32_t x = 0; x < 2; ++x) {
                OptDesc cv = od;
                cv.kind = 2u + x;
                cv.out_index = n_opts + 2u * out.n_cv + x;
                out.opts.push_back(cv);
                out.opt_disc.push_back(out.opt_disc.back());
            }
            ++out.n_cv;
        }
        out.mats.back().opt_end = (uint32_t)out.opts.size();
        out.mat_paths.back() = std::max(out.mat_paths.back(), od.n_paths);
    }
    out.n_user = n_opts;
    out.params = p;
    const size_t m = T.size();

    // Walk the reference's time grid once (HSimulation.tpp:29-46,
    // AsianContract.h:35-38): width T_j/steps_j while maturity j is the
    // earliest unpriced one, t += width in double, price every maturity the
    // step reaches, then continue with the next maturity's width.
    out.seg_of_mat.assign(m, 0);
    out.steps_to_mat.assign(m, 0);
    const double sig2 = p.sigma * p.sigma;
    auto make_seg = [&](double dt) {
        SegDesc s{};
        s.dt = dt;
        s.disc = std::exp(-p.kappa * dt);
        s.cA = sig2 * s.disc / p.kappa * (1.0 - s.disc);
        s.cB = p.theta * sig2 / (2.0 * p.kappa) * (1.0 - s.disc) * (1.0 - s.disc);
        s.K0 = -p.rho * p.kappa * p.theta / p.sigma * dt + (p.r - p.q) * dt;
        s.K1 = 0.5 * dt * (p.kappa * p.rho / p.sigma - 0.5) - p.rho / p.sigma;
        s.K2 = 0.5 * dt * (p.kappa * p.rho / p.sigma - 0.5) + p.rho / p.sigma;
        s.K3 = 0.5 * dt * (1.0 - p.rho * p.rho);
        s.K4 = 0.5 * dt * (1.0 - p.rho * p.rho);
        s.hdt = dt * 0.5;
        s.f_disc = (float)s.disc; s.f_cA = (float)s.cA; s.f_cB = (float)s.cB;
        s.f_K0 = (float)s.K0; s.f_K1 = (float)s.K1; s.f_K2 = (float)s.K2;
        s.f_K3 = (float)s.K3; s.f_K4 = (float)s.K4; s.f_hdt = (float)s.hdt;
        s.f_c = (float)(0.5 * dt * (p.kappa * p.rho / p.sigma - 0.5));
        ds_split(s.disc, s.ds_disc);
        ds_split(p.theta * (1.0 - s.disc), s.ds_m0);
        ds_split(s.cA, s.ds_cA);
        ds_split(s.cB, s.ds_cB);
        return s;
    };
    double t = 0.0;
    size_t j = 0;
    double dt = T[0] / out.mat_steps[0];
    SegDesc seg = make_seg(dt);
    uint64_t steps_total = 0;
    for (;;) {
        const double tp = t;
        t += dt;
        ++seg.n_steps;
        ++steps_total;
        if (steps_total > kMaxStepsPerSet) { err = "step schedule too long"; return HEXO_ERR_INVALID; }
        if (t >= T[j]) {
            seg.mat_begin = (uint32_t)j;
            while (j < m && t >= T[j]) {
                MatDesc &md = out.mats[j];
                md.tmtp = T[j] - tp;
                md.dt = T[j] / out.mat_steps[j];
                md.f_w = (float)(md.tmtp / md.dt);
                md.f_invT = (float)(1.0 / T[j]);
                out.seg_of_mat[j] = (uint32_t)out.segs.size();
                out.steps_to_mat[j] = steps_total;
                ++j;
            }
            seg.mat_end = (uint32_t)j;
            const double dt_next = j < m ? T[j] / out.mat_steps[j] : dt;
            seg.hdt_after = dt_next * 0.5;
            seg.f_hdt_after = (float)seg.hdt_after;
            out.segs.push_back(seg);
            if (j == m) break;
            dt = dt_next;
            seg = make_seg(dt);
        }
    }

    // Paths that reach each maturity.
    out.thr.assign(m + 1, 0);
    for (size_t q = m; q-- > 0;) out.thr[q] = std::max(out.thr[q + 1], out.mat_paths[q]);
    const uint64_t n_max = out.thr[0];
    out.path_lo = std::min(path_lo, n_max);
    out.path_hi = std::min(path_hi, n_max);
    if (out.path_hi < out.path_lo) out.path_hi = out.path_lo;

    SetDesc &sd = out.set;
    sd.S0 = S0;
    sd.logS0 = std::log(S0);
    sd.v0 = p.v0;
    sd.theta = p.theta;
    sd.f_S0 = (float)S0;
    sd.f_v0 = (float)p.v0;
    sd.f_theta = (float)p.theta;
    sd.f_r = (float)(p.rho / p.sigma);
    ds_split(p.v0, sd.ds_v0);
    sd.seed = seed;
    sd.stream = stream;
    sd.pay_exp = pay_exponent(S0);
    sd.seg_count = (uint32_t)out.segs.size();
    sd.mat_count = (uint32_t)m;
    sd.opt_count = (uint32_t)out.opts.size();
    sd.n_paths = out.path_hi;
    return HEXO_OK;
}

int last_maturity(const SetPlan &sp, uint64_t k) {
    // thr is non-increasing, so the maturities path k reaches are a prefix
    const auto end = sp.thr.begin() + (long)sp.mats.size();
    return (int)(std::partition_point(sp.thr.begin(), end, [k](uint64_t t) { return t > k; }) - sp.thr.begin()) - 1;
}

void plan_work(const SetPlan &sp, uint64_t &nominal, uint64_t &executed, uint32_t paths_per_tile) {
    nominal = 0;
    executed = 0;
    const size_t m = sp.mats.size();
    // paths in [lo, hi) whose last maturity is j: those with thr[j+1] <= k < thr[j]
    for (size_t j = 0; j < m; ++j) {
        const uint64_t a = std::max(sp.thr[j + 1], sp.path_lo), b = std::min(sp.thr[j], sp.path_hi);
        if (b > a) nominal += (b - a) * sp.mat_steps[j];
    }
    if (paths_per_tile == 0) return;
    for (uint64_t k0 = sp.path_lo; k0 < sp.path_hi; k0 += paths_per_tile) {
        const int jl = last_maturity(sp, k0);
        if (jl < 0) continue;
        executed += sp.steps_to_mat[jl] * (std::min<uint64_t>(k0 + paths_per_tile, sp.path_hi) - k0);
    }
}

void batch_add(BatchPlan &b, const SetPlan &sp, uint32_t out_base, uint32_t cv_base) {
    // request-local slots: the user's options, then the control variate's
    // internal pairs, which go to the batch's internal range at cv_base
    auto global = [&](uint32_t local) { return local < sp.n_user ? out_base + local : cv_base + (local - sp.n_user); };
    SetDesc sd = sp.set;
    sd.seg_begin = (uint32_t)b.segs.size();
    sd.mat_begin = (uint32_t)b.mats.size();
    sd.opt_begin = (uint32_t)b.opts.size();
    b.sets.push_back(sd);
    b.segs.insert(b.segs.end(), sp.segs.begin(), sp.segs.end());
    b.mats.insert(b.mats.end(), sp.mats.begin(), sp.mats.end());
    for (size_t i = 0; i < sp.opts.size(); ++i) {
        OptDesc od = sp.opts[i];
        od.out_index = global(sp.opts[i].out_index);
        b.opts.push_back(od);
    }
    uint32_t n_out_end = out_base + sp.n_user;
    if (sp.n_cv) n_out_end = std::max(n_out_end, cv_base + 2u * sp.n_cv);
    if (b.n_out < n_out_end) {
        b.n_out = n_out_end;
        b.opt_paths.resize(n_out_end, 0);
        b.opt_disc.resize(n_out_end, 1.0);
        b.opt_pexp.resize(n_out_end, 0);
        b.opt_carry.resize(n_out_end, ~0ull);
    }
    for (size_t i = 0; i < sp.opts.size(); ++i) {
        const uint32_t o = global(sp.opts[i].out_index);
        // paths that price this option within the plan's range
        const uint64_t hi = std::min<uint64_t>(sp.opts[i].n_paths, sp.path_hi);
        b.opt_paths[o] = hi > sp.path_lo ? hi - sp.path_lo : 0;
        b.opt_disc[o] = sp.opt_disc[i];
        b.opt_pexp[o] = sp.set.pay_exp;
    }
    b.max_mats = std::max<uint32_t>(b.max_mats, (uint32_t)sp.mats.size());
    b.set_params.push_back(sp.params);
    for (uint32_t j = 0; j < (uint32_t)sp.mats.size(); ++j)
        for (uint32_t i = sp.mats[j].opt_begin; i < sp.mats[j].opt_end; ++i)
            if (sp.opts[i].kind == 2u)   // the geometric slot, right after its Asian option
                b.cv.push_back(BatchPlan::CvLeader{global(sp.opts[i - 1].out_index), global(sp.opts[i].out_index),
                                                   (uint32_t)b.sets.size() - 1u, j, sp.opts[i].strike});
}

void batch_tiles(BatchPlan &b, const std::vector<SetPlan> &plans) {
    struct Costed { TileDesc t; uint64_t cost; uint64_t order; };
    std::vector<Costed> all;
    const uint32_t P = b.shape.paths_per_tile();
    size_t n_tiles = 0;
    for (const SetPlan &sp : plans) n_tiles += (size_t)((sp.path_hi - sp.path_lo + P - 1) / P);
    all.reserve(n_tiles);
    b.nominal_path_steps = 0;
    b.executed_path_steps = 0;
    b.n_paths = 0;
    for (size_t s = 0; s < plans.size(); ++s) {
        const SetPlan &sp = plans[s];
        uint64_t nom = 0, exe = 0;
        plan_work(sp, nom, exe, P);
        b.nominal_path_steps += nom;
        b.executed_path_steps += exe;
        b.n_paths += sp.path_hi - sp.path_lo;
        for (uint64_t k0 = sp.path_lo; k0 < sp.path_hi; k0 += P) {
            const int jl = last_maturity(sp, k0);
            if (jl < 0) continue;
            Costed c;
            c.t.path_begin = k0;
            c.t.set = (uint32_t)s;
            c.t.seg_count = sp.seg_of_mat[jl] + 1;
            c.cost = sp.steps_to_mat[jl] * (std::min<uint64_t>(k0 + P, sp.path_hi) - k0) +
                     (uint64_t)(sp.mats.size() + sp.opts.size());
            c.order = all.size();
            all.push_back(c);
        }
    }
    // longest first; ties keep their planning order
    std::sort(all.begin(), all.end(), [](const Costed &x, const Costed &y) {
        return x.cost != y.cost ? x.cost > y.cost : x.order < y.order;
    });
    b.tiles.clear();
    b.tiles.reserve(all.size());
    for (const Costed &c : all) b.tiles.push_back(c.t);
}

void finalize_one(const uint64_t *limbs, uint64_t n_paths, double disc, int pay_exp, double *price, double *se) {
    finalize_limbs6(limbs, n_paths, disc, pay_exp, price, se);
}

} // namespace hexo
