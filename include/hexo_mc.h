/*
 * hexo_mc.h: C ABI of the GB300 Monte Carlo engine for hexo's Heston pricer.
 *
 * This is the drop-in boundary for the reference's simulation and pricing
 * entry point
 *
 *   template<class Scheme> std::vector<ffloat> HSimulation::price(
 *       const HParams& p, const ffloat S, const std::list<options_chain>& all_chains,
 *       unsigned n_simulations, unsigned n_opts, unsigned steps);
 *                                         (reference src/inc/HSimulation.h:61-63,
 *                                          body src/HSimulation.tpp:10-51)
 *
 * Everything crosses as plain pointers and sizes.  Buffers are owned by the
 * caller; no call keeps a pointer after it returns, except the serving
 * requests, whose output arrays must stay valid until the request
 * completes.  Errors are status codes, never exceptions; a
 * message for the last failure of a context is available from
 * hexo_ctx_last_error().  include/hexo/reference_compat.h wraps this ABI
 * in the reference's own C++ signature.
 *
 * Random numbers.  Path k (0-based) of a request draws from its own SHISHUA
 * stream seeded {(uint32_t)(seed + k), stream, 0, 0}, used exactly as the
 * reference RNG class uses its stream (src/inc/RNG.h:17-52,
 * src/RNG.cpp:8-47): a uniform buffer filled first and a normal buffer next,
 * each refilled from the same stream when it runs dry;
 * u = (double)word / (double)UINT64_MAX; normals are the float32 AS241
 * (reference src/as241.f90).  With stream = 0 this is the reference class
 * RNG(rng_block_words, seed + k) itself; the second seed word (the
 * reference's seed is four words, RNG.h:24) separates requests, so requests
 * with different stream numbers never share a path's stream even when their
 * seed ranges [seed, seed + n_paths) overlap.  Results do not depend on
 * block size, paths per thread, batching, sharding or which other requests
 * share a launch.
 *
 * Payoff sums.  Prices and standard errors come from exact integer sums, so
 * they are bit for bit the same however paths are split across CTAs,
 * launches or devices.  A request's payoffs are summed in units of 2^E, E the
 * binary exponent of its spot (2^(E-1) <= S0 < 2^E): per path
 * q = round(y 2^47) and q2 = round(y^2 2^43) with y = pay 2^-E, so prices and
 * standard errors keep the same relative precision at every spot level.
 * Spots must lie in [2^-60, 2^60); a payoff at or above 2^16 2^E (65,536
 * times the spot or more) returns HEXO_ERR_NUMERIC.
 */
#ifndef HEXO_MC_H
#define HEXO_MC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Raised whenever a struct's layout or a function's signature changes.
 * 2: hexo_batch_info.quad_steps; hexo_debug_pipe_peaks fills five rates;
 *    hexo_debug_payoff_limbs.
 * 3: hexo_mc_cfg.control_variate.
 * 4: the stream seed word (hexo_mc_cfg.stream, hexo_request.stream); limb
 *    sums in units of the spot's power of two (hexo_finalize_limbs and
 *    hexo_debug_payoff_limbs take S0); the debug RNG calls take the stream. */
#define HEXO_ABI_VERSION 4u

typedef enum hexo_status {
    HEXO_OK = 0,
    HEXO_ERR_INVALID = 1,      /* bad argument (NaN parameter, T <= 0, zero paths, ...) */
    HEXO_ERR_CUDA = 2,         /* a CUDA runtime call failed */
    HEXO_ERR_NOMEM = 3,        /* device or host allocation failed */
    HEXO_ERR_UNSUPPORTED = 4,  /* valid but not supported by the library (e.g. rng_block_words != 16) */
    HEXO_ERR_TIMEOUT = 5,      /* a bounded wait ran out */
    HEXO_ERR_NUMERIC = 6,      /* a payoff was not finite or exceeded the fixed-point range */
    HEXO_ERR_NOT_FOUND = 7,    /* unknown ticket */
    HEXO_ERR_ADMISSION = 8,    /* request can never fit the device-memory cap */
    HEXO_ERR_SHUTDOWN = 9,     /* server is shutting down */
    HEXO_ERR_TOO_LARGE = 10,   /* request exceeds the fixed limits of hexo_price_noalloc */
    HEXO_ERR_CHECK = 11        /* a bounds check of the checked build (libhexo_mc_checks.so) failed */
} hexo_status;

const char *hexo_status_string(hexo_status s);
uint32_t hexo_abi_version(void);

/* ---------------------------------------------------------------- context */

typedef struct hexo_ctx hexo_ctx;

typedef struct hexo_ctx_opts {
    int device;                 /* CUDA device ordinal */
    uint64_t mem_cap_bytes;     /* device-memory cap for admission; 0 = 32 GiB */
    const char *autotune_cache; /* file to read/write tuned launch shapes; NULL = none */
    uint32_t flags;             /* reserved, 0 */
} hexo_ctx_opts;

/* A context keeps the device and pinned host memory of its largest one-shot
 * call (hexo_price, hexo_price_batch, hexo_price_partial,
 * hexo_price_batch_partial) for the next one, so repeated calls allocate
 * nothing, up to 256 MiB of each: a call that needs more frees its memory
 * when it returns.  hexo_ctx_trim and hexo_ctx_destroy free what is kept.
 * This memory is the context's own; a server's memory cap does not count it. */
hexo_status hexo_ctx_create(hexo_ctx **out, const hexo_ctx_opts *opts /* NULL = defaults */);
/* Waits for the context's work and frees it.  Batches, servers and
 * calibration handles made on the context must be destroyed first. */
hexo_status hexo_ctx_destroy(hexo_ctx *ctx);
/* Waits for the context's one-shot calls and frees the device and pinned
 * host memory it keeps for the next one (the next call allocates again). */
hexo_status hexo_ctx_trim(hexo_ctx *ctx);
/* Copies the message of the last failure on this context into buf. */
hexo_status hexo_ctx_last_error(hexo_ctx *ctx, char *buf, size_t buf_len);
/* The cudaStream_t (as void*) on which this context launches its kernels. */
void *hexo_ctx_stream(hexo_ctx *ctx);

/* --------------------------------------------------------------- problem */

/* HParams (reference src/inc/HDistribution.h:9-24, same order) plus the
 * risk-free rate r and dividend yield q.  r = q = 0 reproduces the
 * reference, which has neither drift nor discounting. */
typedef struct hexo_params {
    double v0, theta, rho, kappa, sigma; /* v_0, v_m, rho, kappa, sigma */
    double r, q;
} hexo_params;

typedef enum hexo_payoff {
    HEXO_ASIAN_CALL = 0,    /* AAsianCallNonAdaptive, src/inc/AsianContract.h:14-48 */
    HEXO_EUROPEAN_CALL = 1  /* EuropeanCallNonAdaptive, src/inc/VanillaContract.h:14-40 */
} hexo_payoff;

/* One option: the strike of a reference `option` (src/inc/Types.h:26-33)
 * plus the time_to_expiry of its `options_chain` (Types.h:37-58). */
typedef struct hexo_option {
    double strike;
    double T;          /* years, > 0 */
    uint32_t payoff;   /* hexo_payoff */
    uint32_t reserved; /* 0 */
    uint64_t n_paths;  /* paths for this option; 0 = hexo_mc_cfg.n_paths */
} hexo_option;

typedef enum hexo_step_mode {
    /* the reference's stepping: maturity i is reached with width T_i/steps,
     * time accumulated as t += width in double (HSimulation.tpp:29,42,84) */
    HEXO_STEP_REFERENCE = 0,
    /* the same stepping with steps_i = max(5, round(steps_per_year * T_i)) */
    HEXO_STEP_GRID = 1
} hexo_step_mode;

typedef enum hexo_precision {
    HEXO_FP64 = 0, /* plain form: paths in FP64 */
    HEXO_FP32 = 1  /* paths in FP32; AS241 float32 as in the reference; FP64 finalisation */
} hexo_precision;

typedef struct hexo_mc_cfg {
    uint64_t n_paths;         /* default paths per option (n_simulations) */
    uint32_t step_mode;       /* hexo_step_mode */
    uint32_t steps;           /* REFERENCE mode: steps per maturity */
    double steps_per_year;    /* GRID mode; 0 = 252 */
    uint32_t seed;            /* default seed for hexo_price */
    uint32_t rng_block_words; /* RNG buffer size in 64-bit words; 0 = 16; the GPU supports 16 */
    uint32_t precision;       /* hexo_precision */
    uint32_t block;           /* launch shape override: threads per CTA, 0 = tuned/default */
    uint32_t paths_per_thread;/* 0 = tuned/default */
    uint32_t unroll;          /* 0 = tuned/default */
    uint32_t control_variate; /* 0: the reference's estimator (default).  1: Asian options are priced
                                 with the geometric-average control variate (the future idea of
                                 HSimulation.h:51): the same weights on log X give G, E[(G - K)^+]
                                 comes from the Heston characteristic function, and beta is
                                 estimated from the paths; Europeans unchanged.  Not with
                                 hexo_price_partial or hexo_price_noalloc. */
    uint32_t stream;          /* seed word 1 of every path's stream for hexo_price, hexo_price_partial,
                                 hexo_price_noalloc; 0 = the reference's RNG(16, seed + k) */
} hexo_mc_cfg;

/* Fills cfg with the defaults: 65,536 paths, REFERENCE stepping with 252
 * steps, seed 42, stream 0, 16-word RNG buffers, FP64, tuned launch shape. */
void hexo_mc_cfg_default(hexo_mc_cfg *cfg);

/* ------------------------------------------------------- plain pricing */

/* Prices n_opts options on one parameter set; blocks until done.
 * price_out[i]  = exp(-r T_i) * mean payoff of option i
 * stderr_out[i] = standard error of price_out[i] (may be NULL). */
hexo_status hexo_price(hexo_ctx *ctx, const hexo_params *p, double S0, const hexo_option *opts,
                       uint32_t n_opts, const hexo_mc_cfg *cfg, double *price_out, double *stderr_out);

/* ------------------------------------------------------ batched pricing */

typedef struct hexo_request {
    hexo_params params;
    double S0;
    const hexo_option *opts;
    uint32_t n_opts;
    uint32_t seed;
    double *price_out;   /* n_opts */
    double *stderr_out;  /* n_opts, may be NULL */
    uint32_t stream;     /* seed word 1 of this request's paths; give the requests of one batch or one
                            server different numbers so that none shares a path's stream */
    uint32_t reserved;   /* 0 */
} hexo_request;

/* Prices many parameter sets in one persistent launch. */
hexo_status hexo_price_batch(hexo_ctx *ctx, const hexo_request *reqs, uint32_t n_reqs, const hexo_mc_cfg *cfg);

/* A batch planned and uploaded once, launchable many times (a captured CUDA
 * graph); used for repeated pricing of the same shapes and for timing. */
typedef struct hexo_batch hexo_batch;

typedef struct hexo_batch_info {
    uint64_t nominal_path_steps;  /* sum over paths of the grid steps to the path's last maturity */
    uint64_t executed_path_steps; /* QE steps actually executed (includes the reference's extra steps) */
    uint64_t n_paths;             /* simulated paths */
    uint32_t n_tiles, n_sets, n_options, block, paths_per_thread, unroll, grid;
    uint64_t device_bytes;        /* device memory the batch holds */
    uint64_t h2d_bytes;           /* bytes uploaded when the batch is planned (descriptors) */
    uint64_t d2h_bytes;           /* bytes copied back per run (prices, standard errors, status) */
    double last_kernel_ms;        /* path-kernel time of the last collected run (CUDA events) */
    uint64_t quad_steps;          /* of the last collected run: QE steps that took the quadratic branch
                                     (HSimulation.tpp:63-68); quad_steps / executed_path_steps is the
                                     branch mix p_Q */
} hexo_batch_info;

hexo_status hexo_batch_prepare(hexo_ctx *ctx, const hexo_request *reqs, uint32_t n_reqs, const hexo_mc_cfg *cfg,
                               hexo_batch **out);
/* Enqueues one run on the context stream (graph launch); returns at once. */
hexo_status hexo_batch_launch(hexo_batch *b);
/* Waits for the last launch and copies prices / standard errors into the
 * requests' output arrays. */
hexo_status hexo_batch_collect(hexo_batch *b);
hexo_status hexo_batch_info_get(hexo_batch *b, hexo_batch_info *info);
hexo_status hexo_batch_destroy(hexo_batch *b);

/* -------------------------------------------------------------- serving */

/* A continuous-batching pricing server on one context.  No counterpart in
 * the reference (whose only pricing call is the blocking HSimulation::price,
 * src/inc/HSimulation.h:44-96); it exists so that a calibration or quoting
 * service can keep many small requests in flight at once.
 *
 * A request runs as one or more blocks of consecutive paths, each in a
 * persistent launch shared with the blocks of other requests; its exact
 * payoff sums stay in a device pool between launches, and the launch with its
 * last block finalises it.  Each launch takes one block from each admitted
 * request without a block in flight, those that have had the fewest blocks
 * first, sized so that the launch holds about launch_path_steps of work: a
 * large request no longer holds the device while small ones wait.  Requests
 * are admitted first come, first served while their running sums fit the
 * pool (a quarter of the cap, at most 64 MiB), and one that does not fit yet
 * lets later ones pass for at most 50 ms; launches run while the device
 * memory of those in flight stays under mem_cap_bytes, up to max_inflight at
 * once, each on its own stream.  Path k of a request always draws from the
 * stream seeded {seed + k, stream, 0, 0} and sums are exact integers, so a
 * request's prices equal those of hexo_price_batch for the request alone,
 * bit for bit, whatever it was batched with and however it was split.  With
 * the geometric control variate a request runs as one block. */
typedef struct hexo_server hexo_server;

typedef struct hexo_server_opts {
    hexo_mc_cfg cfg;               /* paths-per-option default, stepping, precision, ... */
    uint64_t mem_cap_bytes;        /* device memory of launches in flight; 0 = the context's cap */
    uint32_t max_batch_requests;   /* requests per launch; 0 = 64 */
    uint32_t max_inflight;         /* launches in flight (streams); 0 = 2, at most 16 */
    uint64_t launch_path_steps;    /* work of one launch, in path-steps; blocks are cut to it; 0 = 2^30
                                      (about 25 ms on a GB300); UINT64_MAX = never split a request */
} hexo_server_opts;

typedef struct hexo_server_stats {
    uint64_t submitted, admitted, completed, failed;
    uint64_t batches;              /* launches made */
    uint64_t chunks;               /* request blocks launched (a request split in k blocks counts k) */
    uint64_t queued_now, queued_max, inflight_now;
    uint64_t mem_in_use, mem_peak; /* device bytes: the pool of running sums and the launches in flight */
    uint64_t nominal_path_steps;   /* of completed requests */
    double busy_seconds;           /* wall time with at least one launch in flight */
    double p50_ms, p99_ms, mean_ms;/* submit-to-completion latency of completed requests */
} hexo_server_stats;

hexo_status hexo_server_create(hexo_ctx *ctx, const hexo_server_opts *opts, hexo_server **out);
/* Queues a request and returns at once with its ticket.  The options are
 * copied; price_out / stderr_out must stay valid until the request is done. */
hexo_status hexo_server_submit(hexo_server *s, const hexo_request *req, uint64_t *ticket);
/* done = 1 once the request finished; the return value is then its status.
 * A finished request is reported once (by poll or wait) and then forgotten:
 * later calls with its ticket return HEXO_ERR_NOT_FOUND. */
hexo_status hexo_server_poll(hexo_server *s, uint64_t ticket, int *done);
/* Waits up to timeout_ms for the request; HEXO_ERR_TIMEOUT if still running. */
hexo_status hexo_server_wait(hexo_server *s, uint64_t ticket, uint32_t timeout_ms);
hexo_status hexo_server_stats_get(hexo_server *s, hexo_server_stats *out);
/* Finishes every queued and running request, then stops; later submits
 * from other threads get HEXO_ERR_SHUTDOWN. */
hexo_status hexo_server_destroy(hexo_server *s);

/* ------------------------------------------------------ SWIFT Europeans */

/* European calls by the SWIFT wavelet method with their gradients in
 * (v0, theta, rho, kappa, sigma): the reference's SWIFT::price_opts and
 * price_opts_grad (src/SWIFT.cpp:87-118, src/inc/SWIFT.h:150-164) with the
 * characteristic function of src/HDistribution.cpp, batched on the GPU in
 * FP64.  It is the reference's calibration objective and the check for the
 * Monte Carlo European prices. */

/* The reference's SwiftParameters (src/inc/SWIFT.h:27-76), same fields. */
typedef struct hexo_swift_params {
    uint32_t m, exp2_m;       /* wavelet scale m and 2^m */
    double sqrt_exp2_m;
    double lower, upper;      /* integration range of the log-price */
    int32_t k1, k2;           /* sum range */
    uint32_t J, reserved;     /* frequencies (a power of two, at most 65536); reserved = 0 */
} hexo_swift_params;

/* Host-only: the reference's dynamic choice of the parameters for one expiry
 * (SwiftParameters(distr, S, chain), src/SWIFT.cpp:21-35): the smallest m
 * whose truncation error is below trunc_precision, plus one (the reference's
 * loop), and the range from the first, second and fourth cumulants.
 * trunc_precision: 1e-7 in the reference's release build (FASTMATH), 1e-10
 * otherwise (SWIFT.cpp:12-16).  Uses p->r as the risk-free rate. */
hexo_status hexo_swift_params_dynamic(const hexo_params *p, double tau, double S, double K_min, double K_max,
                                      double trunc_precision, hexo_swift_params *out);

/* How the two transforms of a chain are evaluated (the reference uses FFTW,
 * SWIFT.cpp:51-52): direct sums cost O(J (k2 - k1)), the FFT O(J log J);
 * both give the same prices to rounding. */
typedef enum hexo_swift_method {
    HEXO_SWIFT_AUTO = 0,    /* the FFT from J = 1024 frequencies on, direct sums below */
    HEXO_SWIFT_DIRECT = 1,  /* direct sums */
    HEXO_SWIFT_FFT = 2      /* radix-2 FFT of length 2J */
} hexo_swift_method;

typedef struct hexo_swift_chain {
    double tau;                        /* years to expiry */
    const double *strikes;             /* n strikes */
    uint32_t n;
    uint32_t method;                   /* hexo_swift_method */
    const hexo_swift_params *params;   /* NULL: chosen as hexo_swift_params_dynamic does */
    double trunc_precision;            /* for params == NULL; 0 = 1e-7 */
    double *price_out;                 /* n discounted call prices */
    double *grad_out;                  /* n x 5 (v0, theta, rho, kappa, sigma), row per option; may be NULL */
} hexo_swift_chain;

typedef struct hexo_swift_request {
    hexo_params params;                /* r is the risk-free rate; q must be 0 */
    double S;
    const hexo_swift_chain *chains;
    uint32_t n_chains, reserved;
} hexo_swift_request;

/* Prices every chain of every request in one sequence of launches; blocks. */
hexo_status hexo_swift_price(hexo_ctx *ctx, const hexo_swift_request *reqs, uint32_t n_reqs);

/* Calibration callbacks.  The reference calibrates by Levenberg-Marquardt
 * (levmar's dlevmar_der) over the SWIFT prices of every chain of an
 * underlying, with the objective and Jacobian callbacks
 *   void get_prices_for_levmar(double *p, double *x, int m, int n, void *adata);
 *   void get_jacobian_for_levmar(double *p, double *jac, int m, int n, void *adata);
 * (src/HCalibration.cpp:35-57).  hexo_calib holds the same data (spot, rate,
 * each chain's expiry and strikes); hexo_calib_prices / _jacobian compute x
 * (n observations, chains in order) and jac (n x 5, row per observation,
 * columns v0, vm, rho, kappa, sigma) for p = {v0, vm, rho, kappa, sigma} on the
 * GPU, choosing every chain's wavelet parameters for p as update_adata does
 * (HCalibration.cpp:11-33).  One evaluation serves both calls for the same p. */
typedef struct hexo_calib hexo_calib;
hexo_status hexo_calib_create(hexo_ctx *ctx, double S, double r, const double *taus, const uint32_t *counts,
                              const double *strikes, uint32_t n_chains, double trunc_precision, hexo_calib **out);
uint32_t hexo_calib_observations(const hexo_calib *c);
hexo_status hexo_calib_prices(hexo_calib *c, const double *p /* 5 */, double *x);
hexo_status hexo_calib_jacobian(hexo_calib *c, const double *p /* 5 */, double *jac);
hexo_status hexo_calib_destroy(hexo_calib *c);

/* --------------------------------------------------------------- shards */

/* Exact partial sums over paths [path_lo, path_hi) of one request: for each
 * option six uint64 limbs, the sums of q = round(y 2^47) and of
 * q2 = round(y^2 2^43) with y = pay 2^-E (2^(E-1) <= S0 < 2^E), each split
 * into three 25-bit limb sums.  Limb sums of disjoint path ranges add
 * exactly, so any split across shards or devices merges to the bit-identical
 * result of one launch. */
#define HEXO_LIMBS 6
hexo_status hexo_price_partial(hexo_ctx *ctx, const hexo_params *p, double S0, const hexo_option *opts,
                               uint32_t n_opts, const hexo_mc_cfg *cfg, uint64_t path_lo, uint64_t path_hi,
                               uint64_t *limbs_out /* n_opts * HEXO_LIMBS */);
/* Shard `shard` of n_shards of a whole batch, in one persistent launch:
 * every request's paths [0, n) (n its largest path count) are cut into
 * n_shards contiguous ranges of sizes differing by at most one, and this
 * shard simulates range `shard` of every request.  limbs_out receives six
 * uint64 limbs per option, the requests' options in order (sum of n_opts
 * rows), as hexo_price_partial gives them.  Adding the limbs of all shards
 * (one SUM all-reduce) and finalising each request with hexo_finalize_limbs
 * gives the prices of hexo_price_batch bit for bit.  The reference's
 * counterpart is the path partition over threads of HSimulation::price
 * (src/HSimulation.tpp:23-28).  Not with the control variate. */
hexo_status hexo_price_batch_partial(hexo_ctx *ctx, const hexo_request *reqs, uint32_t n_reqs, const hexo_mc_cfg *cfg,
                                     uint32_t shard, uint32_t n_shards, uint64_t *limbs_out);
/* The same shard planned and uploaded once as a captured CUDA graph (launch
 * and collect as any batch); hexo_batch_collect_limbs then copies the last
 * run's limbs out.  hexo_batch_collect leaves the requests' price arrays
 * alone for such a batch: its prices exist only after the merge. */
hexo_status hexo_batch_prepare_partial(hexo_ctx *ctx, const hexo_request *reqs, uint32_t n_reqs,
                                       const hexo_mc_cfg *cfg, uint32_t shard, uint32_t n_shards, hexo_batch **out);
/* Waits for the last launch of a batch and copies its limb sums (six per
 * option, requests in order) into limbs_out. */
hexo_status hexo_batch_collect_limbs(hexo_batch *b, uint64_t *limbs_out);

/* Host-only: prices and standard errors from (merged) limb sums; the same
 * operation sequence as the device finaliser, so results match it bit for bit. */
hexo_status hexo_finalize_limbs(const hexo_params *p, double S0, const hexo_option *opts, uint32_t n_opts,
                                const hexo_mc_cfg *cfg, const uint64_t *limbs, double *price_out,
                                double *stderr_out);

/* ------------------------------------------------- pricing without allocation */

/* No counterpart in the reference: this entry point exists for callers that
 * cannot let a library allocate GPU memory, such as a process whose framework
 * or serving stack has reserved nearly all device memory through its own
 * pool (an allocation behind its back would fail or fragment that pool), or a
 * latency-critical loop where cudaMalloc/cudaFree would add device-wide
 * synchronisation.  It prices one request like hexo_price, with the same
 * results bit for bit, and allocates nothing: no device memory and no host
 * heap.  Its device-side working memory is one array of
 * HEXO_NOALLOC_SCRATCH_BYTES compiled into the library, which every GPU that
 * loads the library holds until the process exits.  Limits: at most
 * HEXO_NOALLOC_MAX_OPTIONS options and HEXO_NOALLOC_MAX_PATHS paths per
 * option; beyond them it returns HEXO_ERR_TOO_LARGE before touching the GPU.
 * The launch shape is fixed (256 threads, one path each).  It runs on the
 * current device and on `stream` (a cudaStream_t; NULL = the default stream)
 * and blocks until the results are in price_out / stderr_out (host arrays of
 * n_opts; stderr_out may be NULL).  The first call on each device looks up
 * the array's device address, so make that first call before any stream
 * capture.  All calls share the one array: calls that overlap on the GPU
 * (from several threads or streams) race and must be serialised. */
#define HEXO_NOALLOC_MAX_OPTIONS 128u
#define HEXO_NOALLOC_MAX_PATHS (1u << 20)
#define HEXO_NOALLOC_SCRATCH_BYTES (128u << 10)
hexo_status hexo_price_noalloc(const hexo_params *p, double S0, const hexo_option *opts, uint32_t n_opts,
                               const hexo_mc_cfg *cfg, double *price_out, double *stderr_out, void *stream);

/* ------------------------------------------------------------- planning */

/* Host-only (no GPU needed): the work a batch represents. */
typedef struct hexo_plan_stats {
    uint64_t nominal_path_steps;  /* grid steps to each path's last maturity, summed over paths */
    uint64_t executed_path_steps; /* QE steps the kernel executes for active paths */
    uint64_t n_paths;             /* simulated paths */
    uint32_t n_maturities, n_segments, n_tiles, n_options;
} hexo_plan_stats;
hexo_status hexo_plan_stats_get(const hexo_request *reqs, uint32_t n_reqs, const hexo_mc_cfg *cfg,
                                hexo_plan_stats *out);

/* Host-only: the step schedule of one request.  For each distinct maturity j
 * (ascending): steps executed up to and including the step that prices it,
 * and T_j - t_prev of that step.  Returns the number of maturities in
 * *n_mats; arrays must hold `cap` entries. */
hexo_status hexo_plan_schedule(const hexo_params *p, double S0, const hexo_option *opts, uint32_t n_opts,
                               const hexo_mc_cfg *cfg, uint32_t cap, uint64_t *steps_to_mat, double *tmtp,
                               double *maturity, uint32_t *n_mats);

/* ------------------------------------------------------------- autotune */

typedef struct hexo_tune_result {
    uint32_t block, paths_per_thread, unroll, n_tried;
    double best_ms;
} hexo_tune_result;

typedef struct hexo_tune_entry {
    uint32_t block, paths_per_thread, unroll;
    float ms;
} hexo_tune_entry;

/* Sweeps threads per CTA {128,192,256,384,512} x paths per thread {1,2,4} x step
 * unroll {1,2,4} (shapes that do not fit an SM are skipped) on the given
 * requests, times one launch of each, and makes the fastest the context's
 * shape for cfg->precision (saved to the context's autotune cache file when
 * one was given).  entries (may be NULL) receives up to max_entries timings. */
hexo_status hexo_autotune(hexo_ctx *ctx, const hexo_request *reqs, uint32_t n_reqs, const hexo_mc_cfg *cfg,
                          hexo_tune_result *result, hexo_tune_entry *entries, uint32_t max_entries);

/* ---------------------------------------------------------------- debug */

/* Raw SHISHUA words of the streams seeded {seed + k, stream, 0, 0}, k in
 * [0, n_streams): out[k*n_words + i]. */
hexo_status hexo_debug_rng_words(hexo_ctx *ctx, uint32_t seed, uint32_t stream, uint32_t n_streams,
                                 uint32_t n_words, uint64_t *out);
/* Draws of the two-buffer RNG on the streams seeded {seed + k, stream, 0, 0}
 * (stream 0: RNG(16, seed + k)) for n_streams streams following one shared
 * kinds[] sequence (0 = normal, 1 = uniform); out[k*n + i]. */
hexo_status hexo_debug_rng_draws(hexo_ctx *ctx, uint32_t seed, uint32_t stream, uint32_t n_streams,
                                 const uint8_t *kinds, uint32_t n, double *out);
/* AS241 of u = (double)w / (double)UINT64_MAX for each word: out[i]. */
hexo_status hexo_debug_normals(hexo_ctx *ctx, const uint64_t *words, uint64_t n, double *out);
/* Checks the path kernels' shortcuts inside AS241 on a range of inputs,
 * b in [bits_lo, bits_hi) with bits_hi <= 2^32.  Branches 0 and 1: the
 * division and square root (a reciprocal estimate with Newton and Markstein
 * corrections, in place of the IEEE intrinsics); every float bit pattern b
 * goes through the central branch (branch 0, Q = b) or the tail (branch 1,
 * R = b) once each way.  Branch 2: the 32-bit input stage; for every high
 * word b of a raw word, with low words 0x800, 2^32 - 0x801, 2^31 and a hash
 * of b, a Q the 32-bit stage certifies must equal the exact stage's.
 * out2[0] receives how many b disagree and out2[1] the smallest such b
 * (UINT64_MAX when none).  No reference counterpart: it pins the kernels'
 * arithmetic to the reference's float AS241 on the double uniform
 * (src/as241.f90:86-116, src/RNG.cpp:34-43). */
hexo_status hexo_debug_as241_check(hexo_ctx *ctx, uint32_t branch, uint64_t bits_lo, uint64_t bits_hi,
                                   uint64_t *out2);
/* The fixed-point split of payoffs as the path kernels fold them for a
 * request with spot S0: for each pay[i] (converted to float first when
 * precision is HEXO_FP32) the six 25-bit limbs out[6*i .. 6*i+5] of
 * q = round(y 2^47) and q2 = round(y^2 2^43), y = pay 2^-E,
 * 2^(E-1) <= S0 < 2^E, ties to even (y^2 rounded to double in the FP64 form,
 * exact in the FP32 form); all six are 0xFFFFFFFF for a payoff the kernels
 * reject (not finite, negative or y >= 2^16). */
hexo_status hexo_debug_payoff_limbs(hexo_ctx *ctx, const double *pay, uint64_t n, uint32_t precision, double S0,
                                    uint32_t *out);
/* Measured lane-operation rates (per second) of this GPU's pipes, from
 * throughput probes: out5 = {FP32 FMA, FP64 FMA, MUFU ex2, INT32 IMAD,
 * INT32 ALU (shift and logic)}. */
hexo_status hexo_debug_pipe_peaks(hexo_ctx *ctx, double *out5);
/* Per-path final values (Asian average, interpolated terminal spot) at every
 * distinct maturity for paths [path_lo, path_hi); NaN after a path's last
 * maturity.  Arrays are [(k - path_lo) * n_mats + j]; n_mats_out receives
 * the number of distinct maturities. */
hexo_status hexo_debug_path_finals(hexo_ctx *ctx, const hexo_params *p, double S0, const hexo_option *opts,
                                   uint32_t n_opts, const hexo_mc_cfg *cfg, uint64_t path_lo, uint64_t path_hi,
                                   double *asian_out, double *euro_out, uint32_t *n_mats_out);

#ifdef __cplusplus
}
#endif
#endif
