// hexo_price_noalloc: pricing of one request with no memory allocation.
//
// Who needs it: a caller that cannot let a library call cudaMalloc.  Typical
// cases are a process whose framework (a deep-learning runtime or a serving
// stack with its own caching pool) has reserved nearly all of the GPU's
// memory, so that an allocation behind its back fails or fragments the pool,
// and latency-critical loops, where cudaMalloc/cudaFree would add
// device-wide synchronisation.  This entry point therefore allocates nothing:
// no device memory, no pinned or pageable host heap.  It plans on the stack,
// keeps every device-side buffer (descriptors, the per-option limb sums, the
// tile queue and the device copy of the results) in one file-scope
// __device__ array of HEXO_NOALLOC_SCRATCH_BYTES, and runs the same path
// kernel and finaliser as hexo_price with the same launch shape, so its
// results are bit-identical to hexo_price's.
//
// The array exists once per device that loads this library, for the life of
// the process.  Host code reaches it only through the address returned by
// cudaGetSymbolAddress (the array's name on the host is a stand-in, not a
// device address); that lookup happens on the first call on each device,
// with the device current, so the first call on a device should come before
// any stream capture.  A call blocks until its results are on the host, so
// it refuses a stream that is being captured (HEXO_ERR_UNSUPPORTED) before
// it enqueues anything.  Every call shares the array and the call clears
// what must start at zero; calls whose work overlaps on the GPU (from several
// threads or streams) race on it and must be serialised by the caller.
//
// The path kernels' dynamic shared-memory limit is a per-kernel attribute
// that every entry point of the library sets; all of them set it to the
// same value, the device's opt-in maximum less the kernel's static shared
// memory (paths_smem_limit), so no caller can lower it under another's
// launch.
#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>

#include "hexo_mc.h"
#include "hexo_launch.h"
#include "hexo_types.h"

namespace hexo {
namespace {

constexpr uint32_t kNaMaxOptions = HEXO_NOALLOC_MAX_OPTIONS;
constexpr uint64_t kNaMaxPaths = HEXO_NOALLOC_MAX_PATHS;
constexpr uint32_t kNaBlock = 256;                            // threads per CTA (one path each)
constexpr uint32_t kNaMaxTiles = (uint32_t)(kNaMaxPaths / kNaBlock);
constexpr uint32_t kNaTileChunk = 256;                        // tiles staged on the stack per upload
constexpr uint64_t kNaMaxStepsPerSet = 1ull << 24;
constexpr int kNaMaxDevices = 64;

constexpr size_t na_align(size_t x) { return (x + 255) / 256 * 256; }
constexpr size_t kOffSet = 0;
constexpr size_t kOffSegs = kOffSet + na_align(sizeof(SetDesc));
constexpr size_t kOffMats = kOffSegs + na_align(kNaMaxOptions * sizeof(SegDesc));
constexpr size_t kOffOpts = kOffMats + na_align(kNaMaxOptions * sizeof(MatDesc));
constexpr size_t kOffTiles = kOffOpts + na_align(kNaMaxOptions * sizeof(OptDesc));
constexpr size_t kOffPaths = kOffTiles + na_align(kNaMaxTiles * sizeof(TileDesc));
constexpr size_t kOffDisc = kOffPaths + na_align(kNaMaxOptions * sizeof(uint64_t));
constexpr size_t kOffPexp = kOffDisc + na_align(kNaMaxOptions * sizeof(double));
constexpr size_t kOffAcc = kOffPexp + na_align(kNaMaxOptions * sizeof(int32_t));
constexpr size_t kOffPrice = kOffAcc + na_align(kNaMaxOptions * kLimbs * sizeof(unsigned long long));
constexpr size_t kOffSe = kOffPrice + na_align(kNaMaxOptions * sizeof(double));
constexpr size_t kOffCtl = kOffSe + na_align(kNaMaxOptions * sizeof(double));
constexpr size_t kNaUsed = kOffCtl + na_align(3 * sizeof(uint32_t));   // tile queue head, error flags, check
static_assert(kNaUsed <= HEXO_NOALLOC_SCRATCH_BYTES, "no-allocation scratch layout exceeds its array");

} // namespace
} // namespace hexo

// The scratch itself: one array per device, alive until the process exits.
static __device__ __align__(256) unsigned char g_hexo_noalloc_scratch[HEXO_NOALLOC_SCRATCH_BYTES];

namespace hexo {
namespace {

std::mutex g_na_setup_mutex;
unsigned char *g_na_scratch[kNaMaxDevices] = {};
uint32_t g_na_sm_count[kNaMaxDevices] = {};
uint32_t g_na_ctas[2][kNaMaxDevices] = {};

// Per-device set-up on the first call: the scratch's device address, the
// SM count and the path kernels' shared-memory limit and occupancy.
hexo_status na_setup(int dev, bool f32, unsigned char **scratch, uint32_t *grid_slots) {
    if (dev < 0 || dev >= kNaMaxDevices) return HEXO_ERR_UNSUPPORTED;
    std::lock_guard<std::mutex> lk(g_na_setup_mutex);
    if (g_na_scratch[dev] == nullptr) {
        void *ptr = nullptr;
        if (cudaGetSymbolAddress(&ptr, g_hexo_noalloc_scratch) != cudaSuccess || ptr == nullptr)
            return HEXO_ERR_CUDA;
        int sms = 0;
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
            return HEXO_ERR_CUDA;
        const size_t smem = paths_smem_bytes(kNaBlock, 1);
        for (int k = 0; k < 2; ++k) {
            const void *fn = paths_kernel_ptr(k == 1, 1, 1);
            int nb = 0;
            if (paths_smem_limit(fn, dev) != cudaSuccess ||
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, (int)kNaBlock, smem) != cudaSuccess || nb <= 0)
                return HEXO_ERR_CUDA;
            g_na_ctas[k][dev] = (uint32_t)nb;
        }
        g_na_sm_count[dev] = (uint32_t)sms;
        g_na_scratch[dev] = static_cast<unsigned char *>(ptr);
    }
    *scratch = g_na_scratch[dev];
    *grid_slots = g_na_sm_count[dev] * g_na_ctas[f32 ? 1 : 0][dev];
    return HEXO_OK;
}

// QE constants of one step width, the same expressions as the batch planner.
SegDesc na_segment(const hexo_params &p, double dt) {
    const double sig2 = p.sigma * p.sigma;
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
}

} // namespace
} // namespace hexo

using namespace hexo;

extern "C" hexo_status hexo_price_noalloc(const hexo_params *pp, double S0, const hexo_option *opts, uint32_t n_opts,
                                          const hexo_mc_cfg *cfg, double *price_out, double *stderr_out,
                                          void *stream) {
    if (!pp || !opts || !cfg || !price_out) return HEXO_ERR_INVALID;
    if (n_opts == 0) return HEXO_ERR_INVALID;
    if (n_opts > kNaMaxOptions) return HEXO_ERR_TOO_LARGE;
    if (cfg->control_variate) return HEXO_ERR_UNSUPPORTED;
    const hexo_params p = *pp;
    const double pv[7] = {p.v0, p.theta, p.rho, p.kappa, p.sigma, p.r, p.q};
    for (double x : pv)
        if (!std::isfinite(x)) return HEXO_ERR_INVALID;
    if (!(p.v0 >= 0.0) || !(p.theta > 0.0) || !(p.kappa > 0.0) || !(p.sigma > 0.0) || !(std::fabs(p.rho) <= 1.0))
        return HEXO_ERR_INVALID;
    if (!std::isfinite(S0) || !(S0 >= 0x1p-60) || !(S0 < 0x1p60)) return HEXO_ERR_INVALID;
    if ((cfg->rng_block_words ? cfg->rng_block_words : 16u) != 16u) return HEXO_ERR_UNSUPPORTED;
    if (cfg->step_mode > 1u || cfg->precision > 1u) return HEXO_ERR_INVALID;
    if (cfg->step_mode == HEXO_STEP_REFERENCE && cfg->steps == 0) return HEXO_ERR_INVALID;
    const double spy = cfg->steps_per_year > 0.0 ? cfg->steps_per_year : 252.0;
    const bool f32 = cfg->precision == HEXO_FP32;

    // ---- plan on the stack: options sorted by maturity (stable), grouped
    uint32_t order[kNaMaxOptions];
    for (uint32_t i = 0; i < n_opts; ++i) {
        const hexo_option &o = opts[i];
        if (!std::isfinite(o.T) || !(o.T > 0.0) || !std::isfinite(o.strike) || o.payoff > 1u) return HEXO_ERR_INVALID;
        const uint64_t np = o.n_paths ? o.n_paths : cfg->n_paths;
        if (np == 0) return HEXO_ERR_INVALID;
        if (np > kNaMaxPaths) return HEXO_ERR_TOO_LARGE;
        uint32_t j = i;
        while (j > 0 && opts[order[j - 1]].T > o.T) { order[j] = order[j - 1]; --j; }
        order[j] = i;
    }
    SetDesc sd{};
    SegDesc segs[kNaMaxOptions];
    MatDesc mats[kNaMaxOptions];
    OptDesc od[kNaMaxOptions];
    uint64_t opt_paths[kNaMaxOptions];
    double opt_disc[kNaMaxOptions];
    int32_t opt_pexp[kNaMaxOptions];
    const int32_t E = pay_exponent(S0);
    uint32_t mat_steps[kNaMaxOptions];
    uint64_t mat_paths[kNaMaxOptions];
    uint32_t seg_of_mat[kNaMaxOptions];
    uint64_t thr[kNaMaxOptions + 1];
    uint32_t m = 0;
    for (uint32_t r = 0; r < n_opts; ++r) {
        const uint32_t i = order[r];
        if (m == 0 || mats[m - 1].T != opts[i].T) {
            uint32_t n = cfg->steps;
            if (cfg->step_mode == HEXO_STEP_GRID) {
                const double g = std::nearbyint(spy * opts[i].T);
                if (!(g < 4.0e9)) return HEXO_ERR_INVALID;
                n = (uint32_t)std::max(5.0, g);
            }
            mats[m] = MatDesc{};
            mats[m].T = opts[i].T;
            mats[m].opt_begin = r;
            mat_steps[m] = n;
            mat_paths[m] = 0;
            ++m;
        }
        od[r] = OptDesc{};
        od[r].strike = opts[i].strike;
        od[r].f_strike = (float)opts[i].strike;
        od[r].kind = opts[i].payoff;
        od[r].n_paths = opts[i].n_paths ? opts[i].n_paths : cfg->n_paths;
        od[r].out_index = i;
        opt_paths[i] = od[r].n_paths;
        opt_disc[i] = std::exp(-p.r * opts[i].T);
        opt_pexp[i] = E;
        mats[m - 1].opt_end = r + 1;
        mat_paths[m - 1] = std::max(mat_paths[m - 1], od[r].n_paths);
    }

    // ---- the reference's time walk (HSimulation.tpp:29-46), one segment per pricing step
    uint32_t n_segs = 0;
    {
        double t = 0.0, dt = mats[0].T / mat_steps[0];
        uint32_t j = 0;
        uint64_t steps_total = 0;
        SegDesc seg = na_segment(p, dt);
        for (;;) {
            const double tp = t;
            t += dt;
            ++seg.n_steps;
            if (++steps_total > kNaMaxStepsPerSet) return HEXO_ERR_TOO_LARGE;
            if (t >= mats[j].T) {
                seg.mat_begin = j;
                while (j < m && t >= mats[j].T) {
                    MatDesc &md = mats[j];
                    md.tmtp = md.T - tp;
                    md.dt = md.T / mat_steps[j];
                    md.f_w = (float)(md.tmtp / md.dt);
                    md.f_invT = (float)(1.0 / md.T);
                    seg_of_mat[j] = n_segs;
                    ++j;
                }
                seg.mat_end = j;
                const double dt_next = j < m ? mats[j].T / mat_steps[j] : dt;
                seg.hdt_after = dt_next * 0.5;
                seg.f_hdt_after = (float)seg.hdt_after;
                segs[n_segs++] = seg;
                if (j == m) break;
                dt = dt_next;
                seg = na_segment(p, dt);
            }
        }
    }
    thr[m] = 0;
    for (uint32_t q = m; q-- > 0;) thr[q] = std::max(thr[q + 1], mat_paths[q]);
    const uint64_t n_max = thr[0];
    sd.S0 = S0;
    sd.logS0 = std::log(S0);
    sd.v0 = p.v0;
    sd.theta = p.theta;
    sd.f_S0 = (float)S0;
    sd.f_v0 = (float)p.v0;
    sd.f_theta = (float)p.theta;
    sd.f_r = (float)(p.rho / p.sigma);
    ds_split(p.v0, sd.ds_v0);
    sd.seed = cfg->seed;
    sd.stream = cfg->stream;
    sd.pay_exp = E;
    sd.seg_count = n_segs;
    sd.mat_count = m;
    sd.opt_count = n_opts;
    sd.n_paths = n_max;
    const uint32_t n_tiles = (uint32_t)((n_max + kNaBlock - 1) / kNaBlock);

    // ---- device side: everything lives in the static scratch array
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return HEXO_ERR_CUDA;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cap) != cudaSuccess) return HEXO_ERR_CUDA;
    if (cap != cudaStreamCaptureStatusNone) return HEXO_ERR_UNSUPPORTED;   // the call waits for its results
    unsigned char *base = nullptr;
    uint32_t slots = 0;
    hexo_status st = na_setup(dev, f32, &base, &slots);
    if (st != HEXO_OK) return st;
    cudaError_t e = cudaSuccess;
    auto up = [&](size_t off, const void *src, size_t bytes) {
        if (e == cudaSuccess && bytes) e = cudaMemcpyAsync(base + off, src, bytes, cudaMemcpyHostToDevice, s);
    };
    up(kOffSet, &sd, sizeof sd);
    up(kOffSegs, segs, n_segs * sizeof(SegDesc));
    up(kOffMats, mats, m * sizeof(MatDesc));
    up(kOffOpts, od, n_opts * sizeof(OptDesc));
    up(kOffPaths, opt_paths, n_opts * sizeof(uint64_t));
    up(kOffDisc, opt_disc, n_opts * sizeof(double));
    up(kOffPexp, opt_pexp, n_opts * sizeof(int32_t));
    TileDesc chunk[kNaTileChunk];
    for (uint32_t t0 = 0; t0 < n_tiles && e == cudaSuccess; t0 += kNaTileChunk) {
        const uint32_t cnt = std::min(kNaTileChunk, n_tiles - t0);
        for (uint32_t q = 0; q < cnt; ++q) {
            const uint64_t k0 = (uint64_t)(t0 + q) * kNaBlock;
            uint32_t jl = 0;
            for (uint32_t j = 0; j < m; ++j)
                if (thr[j] > k0) jl = j;
            chunk[q].path_begin = k0;
            chunk[q].set = 0;
            chunk[q].seg_count = seg_of_mat[jl] + 1;
        }
        up(kOffTiles + (size_t)t0 * sizeof(TileDesc), chunk, cnt * sizeof(TileDesc));
    }
    // sums, queue head and error flags start at zero on every call
    if (e == cudaSuccess) e = cudaMemsetAsync(base + kOffAcc, 0, (size_t)n_opts * kLimbs * sizeof(unsigned long long), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(base + kOffCtl, 0, 3 * sizeof(uint32_t), s);
    KernelArgs a;
    std::memset(&a, 0, sizeof a);
    a.sets = reinterpret_cast<const SetDesc *>(base + kOffSet);
    a.segs = reinterpret_cast<const SegDesc *>(base + kOffSegs);
    a.mats = reinterpret_cast<const MatDesc *>(base + kOffMats);
    a.opts = reinterpret_cast<const OptDesc *>(base + kOffOpts);
    a.tiles = reinterpret_cast<const TileDesc *>(base + kOffTiles);
    a.n_tiles = n_tiles;
    a.acc = reinterpret_cast<unsigned long long *>(base + kOffAcc);
    a.n_slots = 1;
    a.acc_slot_stride = (uint64_t)n_opts * kLimbs;
    a.queue = reinterpret_cast<unsigned int *>(base + kOffCtl);
    a.error = reinterpret_cast<int *>(base + kOffCtl + sizeof(uint32_t));
    a.check = reinterpret_cast<unsigned int *>(base + kOffCtl + 2 * sizeof(uint32_t));
    a.n_out = n_opts;
    a.n_sets = 1;
    a.n_segs = n_segs;
    a.n_mats = m;
    a.n_opts = n_opts;
    const LaunchShape sh{kNaBlock, 1, 1};
    const uint32_t grid = std::max<uint32_t>(1, std::min(slots, n_tiles));
    if (e == cudaSuccess && n_tiles > 0) e = launch_paths(f32, sh, grid, paths_smem_bytes(kNaBlock, 1), s, a);
    double *d_price = reinterpret_cast<double *>(base + kOffPrice);
    double *d_se = reinterpret_cast<double *>(base + kOffSe);
    if (e == cudaSuccess) {
        FinalizeArgs fa;
        fa.acc = a.acc;
        fa.n_slots = 1;
        fa.slot_stride = a.acc_slot_stride;
        fa.n_paths = reinterpret_cast<const uint64_t *>(base + kOffPaths);
        fa.disc = reinterpret_cast<const double *>(base + kOffDisc);
        fa.pay_exp = reinterpret_cast<const int32_t *>(base + kOffPexp);
        fa.n = n_opts;
        fa.price = d_price;
        fa.se = d_se;
        e = launch_finalize(fa, s);
    }
    uint32_t ctl[2] = {0, 0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(price_out, d_price, n_opts * sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && stderr_out)
        e = cudaMemcpyAsync(stderr_out, d_se, n_opts * sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(ctl, base + kOffCtl, sizeof ctl, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return HEXO_ERR_CUDA;
    if (ctl[1] & kErrCheck) return HEXO_ERR_CHECK;
    return ctl[1] != 0u ? HEXO_ERR_NUMERIC : HEXO_OK;
}
