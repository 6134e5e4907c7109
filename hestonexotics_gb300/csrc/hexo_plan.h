// Host-side planning: turns requests into the descriptors of hexo_types.h.
// Pure C++ (no CUDA), so the planner also runs and is tested without a GPU.
#pragma once
#include <stdint.h>
#include <string>
#include <vector>
#include "hexo_mc.h"
#include "hexo_types.h"

namespace hexo {

struct LaunchShape {
    uint32_t block = 256, ppt = 1, unroll = 1;
    bool cv = false;   // the geometric control variate's kernel (one path per thread, no unroll)
    uint32_t paths_per_tile() const { return block * ppt; }
};

// One parameter set planned: maturities, step schedule, options sorted by
// maturity, and the path-count profile that decides how far each path runs.
struct SetPlan {
    SetDesc set{};                      // set-local offsets (0-based)
    std::vector<SegDesc> segs;
    std::vector<MatDesc> mats;
    std::vector<OptDesc> opts;          // sorted by maturity; out_index = request-local option index
    std::vector<double> opt_disc;       // exp(-r T) per sorted option
    std::vector<uint32_t> mat_steps;    // nominal steps per maturity
    std::vector<uint64_t> mat_paths;    // max paths over the maturity's options
    std::vector<uint64_t> thr;          // thr[j] = max_{j' >= j} mat_paths[j'] (paths that reach maturity j)
    std::vector<uint32_t> seg_of_mat;   // segment whose last step prices maturity j
    std::vector<uint64_t> steps_to_mat; // executed steps up to and including the pricing step of j
    uint64_t path_lo = 0, path_hi = 0;  // simulated path range
    uint32_t n_user = 0;                // the request's options (request-local slots [0, n_user))
    uint32_t n_cv = 0;                  // Asian options with the control variate (2 internal slots each)
    hexo_params params{};
};

// Validates and plans one request.  Returns HEXO_OK or an error with a message.
hexo_status plan_set(const hexo_params &p, double S0, const hexo_option *opts, uint32_t n_opts,
                     const hexo_mc_cfg &cfg, uint32_t seed, uint32_t stream, uint64_t path_lo, uint64_t path_hi,
                     SetPlan &out, std::string &err);

// Last maturity index a path k needs, or -1 when no option uses path k.
int last_maturity(const SetPlan &sp, uint64_t k);

// Nominal path-steps (grid steps to each path's last maturity) and executed
// steps, over the plan's path range.
void plan_work(const SetPlan &sp, uint64_t &nominal, uint64_t &executed_if_blocked, uint32_t paths_per_tile);

// A whole batch: concatenated descriptors plus a cost-sorted tile list.
struct BatchPlan {
    std::vector<SetDesc> sets;
    std::vector<SegDesc> segs;
    std::vector<MatDesc> mats;
    std::vector<OptDesc> opts;
    std::vector<TileDesc> tiles;
    std::vector<uint64_t> opt_paths;    // per output slot: paths that price it
    std::vector<double> opt_disc;       // per output slot: exp(-r T)
    std::vector<int32_t> opt_pexp;      // per output slot: E, payoffs summed in units of 2^E
    std::vector<uint64_t> opt_carry;    // per output slot: (row << 1) | last block of a request whose sums
                                        // are carried across launches (the serving loop); ~0 = none
    uint32_t n_out = 0;                 // output slots: the requests' options, then the control variate's
    std::vector<hexo_params> set_params;
    struct CvLeader {                   // an Asian option priced with the geometric control variate
        uint32_t leader, gslot;         // its output slot; the geometric call's (the difference's is gslot + 1)
        uint32_t set, mat;              // set and set-local maturity
        double strike;
    };
    std::vector<CvLeader> cv;
    uint32_t max_mats = 0;
    uint64_t nominal_path_steps = 0, executed_path_steps = 0, n_paths = 0;
    LaunchShape shape;
};

// Appends a planned set whose outputs start at out_base; its control-variate
// slots (if any) start at cv_base, after every request's outputs.
void batch_add(BatchPlan &b, const SetPlan &sp, uint32_t out_base, uint32_t cv_base = 0);
// Builds the tile list for the batch's launch shape, longest tiles first.
void batch_tiles(BatchPlan &b, const std::vector<SetPlan> &plans);

// Finaliser arithmetic shared bit for bit with the device finaliser:
// price and standard error from six limb sums.
void finalize_one(const uint64_t *limbs, uint64_t n_paths, double disc, int pay_exp, double *price, double *se);

} // namespace hexo
