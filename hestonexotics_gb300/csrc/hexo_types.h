// Plain descriptors shared by the host planner and the device kernels.
//
// A batch is a set of parameter sets ("sets"), each with its options grouped
// by distinct maturity ("mats") and a step schedule ("segs").  The schedule
// is the reference's own time stepping (HSimulation.tpp:29-46 with
// AsianContract.h:35-38): maturity i is approached with width T_i/steps_i,
// time accumulates as t += width in double, a maturity is priced after the
// first step whose time reaches it.  Because that time grid does not depend on
// the path, the host walks it once per set; a segment is a run of equal-width
// steps whose last step prices one or more maturities.  Tiles are
// (set, path block) work items for the persistent kernel.
#pragma once
#include <stdint.h>
#include <math.h>

namespace hexo {

// Fixed-point payoff sums.  A request's payoffs are measured in units of
// 2^E, E the binary exponent of its spot (2^(E-1) <= S0 < 2^E): y = pay 2^-E
// is of order one whatever the spot, so the sums keep the same relative
// precision at S0 = 1e-3 as at 1e8.  Per path q = round(y 2^47) and
// q2 = round(y^2 2^43) (ties to even), y < 2^16, so q < 2^63 and q2 < 2^75,
// each cut into three 25-bit limbs.
constexpr int kLimbs = 6;            // 3 x 25-bit limbs of sum(q), 3 of sum(q2)
constexpr int kLimbBits = 25;        // a warp adds up to 128 limb values in 32 bits
constexpr uint32_t kLimbMask = (1u << kLimbBits) - 1u;
constexpr int kPayFrac = 47;         // q = round(y 2^47)
constexpr int kSqFrac = 43;          // q2 = round(y^2 2^43)
constexpr int kPayExpMin = -59, kPayExpMax = 60;   // spots in [2^-60, 2^60)

// E of a spot (the exponent frexp returns); callers check the range.
inline int pay_exponent(double S0) {
    int e = 0;
    (void)frexp(S0, &e);
    return e;
}
constexpr int kRngWords = 16;        // words per RNG buffer (one SHISHUA block)
constexpr uint32_t kConvQueue = 96;                    // per warp: queued conversion items
constexpr uint32_t kWarpScratchBytes = kConvQueue * 2; // per warp: the queue
// per launch control block: tile queue head (u32), error flags (u32), exponential-branch steps (u64),
// the first failed bounds check (u32, checked builds), padding (u32)
constexpr size_t kCtlBytes = 24;
constexpr int kRingSlots = 3;        // per path: normal buffer, uniform buffer, one look-ahead block
// Private copies of a launch's payoff sums: CTA b adds into copy b % kSumSlots,
// so few CTAs share an address while the copies' memory and traffic stay
// small (n_options * 48 bytes each)
constexpr uint32_t kSumSlots = 16;

struct SegDesc {
    // FP64 constants of one step width dt (HSimulation.tpp:55-79, hoisted)
    double dt;      // step width
    double disc;    // exp(-kappa dt)
    double cA;      // sigma^2 disc / kappa (1 - disc)
    double cB;      // theta sigma^2 / (2 kappa) (1 - disc)^2
    double K0, K1, K2, K3, K4;  // K0 includes (r - q) dt
    double hdt;       // 0.5 dt: trapezoid weight after a non-pricing step
    double hdt_after; // 0.5 dt of the next segment: trapezoid weight after the pricing step
    // FP32 copies
    float f_disc, f_cA, f_cB, f_K0, f_K1, f_K2, f_K3, f_K4, f_hdt, f_hdt_after;
    float f_c;      // 0.5 dt (kappa rho / sigma - 0.5): K1 = c - rho/sigma, K2 = c + rho/sigma
    float f_pad0;
    // double-single (hi, lo) copies for the FP32 form's variance: m = v disc + m0, s^2 = v cA + cB
    float ds_disc[2], ds_m0[2], ds_cA[2], ds_cB[2];
    uint32_t n_steps;   // steps in this segment, the last one prices
    uint32_t mat_begin; // maturities priced after the last step: [mat_begin, mat_end) (set-local)
    uint32_t mat_end;
    uint32_t pad;
};

struct MatDesc {
    double T;       // maturity
    double tmtp;    // T - t_prev of the pricing step (AsianContract.h:30-31)
    double dt;      // T / steps at pricing time (the contract's init_step_size)
    float f_w;      // tmtp / dt
    float f_invT;   // 1 / T
    uint32_t opt_begin, opt_end;   // set-local option range (options sorted by maturity)
};

struct OptDesc {
    double strike;
    float f_strike;
    uint32_t kind;       // 0 Asian, 1 European; with the control variate: 2 geometric-average call
                         // (G - K)^+, 3 the signed difference (A - K)^+ - (G - K)^+
    uint64_t n_paths;    // paths k < n_paths price this option
    uint32_t out_index;  // position in the batch's result arrays
    uint32_t pad;
};

struct SetDesc {
    double S0, logS0, v0, theta;
    float f_S0, f_v0, f_theta, f_r;   // f_r = rho / sigma
    float ds_v0[2];                   // v0 in double-single (FP32 form)
    uint32_t stream;                  // seed word 1 of every path's SHISHUA stream
    int32_t pay_exp;                  // E: payoffs are summed in units of 2^E
    uint32_t seed;
    uint32_t seg_begin, seg_count;
    uint32_t mat_begin, mat_count;
    uint32_t opt_begin, opt_count;
    uint32_t pad;
    uint64_t n_paths;    // max over options
};

struct TileDesc {
    uint64_t path_begin; // first path of the block
    uint32_t set;        // set index
    uint32_t seg_count;  // segments this block must run (to its last maturity)
};

// hi + lo float pair of a double (host side; the double-single constants)
inline void ds_split(double x, float out[2]) {
    out[0] = (float)x;
    out[1] = (float)(x - (double)out[0]);
}

struct KernelArgs {
    const SetDesc *sets;
    const SegDesc *segs;     // global arrays; set-local indices are offset by SetDesc
    const MatDesc *mats;
    const OptDesc *opts;
    const TileDesc *tiles;
    uint32_t n_tiles;
    uint32_t n_slots;        // private copies of the sums: CTA b adds into copy b % n_slots
    unsigned long long *acc; // [slot * acc_slot_stride + out_index * kLimbs + limb]
    uint64_t acc_slot_stride;
    unsigned int *queue;     // [0] tile queue head
    int *error;              // [0] error flags (bit 0: non-finite payoff, bit 1: fixed-point range)
    unsigned long long *exp_steps;  // [0] QE steps of active paths on the exponential branch, or null
    double *dbg_asian;       // optional per-path final values (debug): [(k - dbg_lo) * dbg_mats + j]
    double *dbg_euro;
    uint64_t dbg_lo;
    uint32_t dbg_mats;
    uint32_t n_out;          // output slots: out_index < n_out
    uint32_t n_sets, n_segs, n_mats, n_opts;   // descriptor counts, for the bounds-checked build
    unsigned int *check;     // bounds-checked build: the first failed check, (code << 24) | detail, or null
};

// Bounds checks of the HEXO_CHECKS build (compiled out otherwise): a failed
// check sets error bit 2 and records its code and a detail (the offending
// index, cut to 24 bits) in *check, and the kernel skips the access.
enum CheckCode : uint32_t {
    kCheckSet = 1,        // a tile's set index >= n_sets
    kCheckSegs = 2,       // a set's segment range beyond n_segs
    kCheckMat = 3,        // a maturity index >= n_mats
    kCheckOpt = 4,        // an option index >= n_opts or beyond its set
    kCheckOut = 5,        // an option's out_index >= n_out
    kCheckWindow = 6,     // a payoff-window offset >= kWindow
    kCheckQueue = 7,      // a conversion-queue index >= kConvQueue
    kCheckRing = 8,       // a ring slot other than 0 or 1
};
constexpr uint32_t kErrCheck = 4u;   // error bit of a failed bounds check

} // namespace hexo
