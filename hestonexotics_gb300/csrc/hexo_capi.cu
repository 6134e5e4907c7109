// C ABI of the engine (include/hexo_mc.h): contexts, planning + upload of
// batches, launches (direct or through a captured CUDA graph), shards and
// debug entry points.
#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "hexo_mc.h"
#include "hexo_launch.h"
#include "hexo_plan.h"
#include "hexo_runtime.h"

using namespace hexo;

// ------------------------------------------------------------------ context

namespace hexo {

hexo_status ctx_fail(hexo_ctx *ctx, hexo_status s, const std::string &msg) {
    if (ctx) {
        std::lock_guard<std::mutex> g(ctx->err_mu);
        ctx->last_error = msg;
    }
    return s;
}

hexo_status cuda_fail(hexo_ctx *ctx, cudaError_t e, const char *what) {
    return ctx_fail(ctx, e == cudaErrorMemoryAllocation ? HEXO_ERR_NOMEM : HEXO_ERR_CUDA,
                    std::string(what) + ": " + cudaGetErrorString(e));
}

LaunchShape ctx_shape(hexo_ctx *ctx, const hexo_mc_cfg &cfg) {
    LaunchShape sh = cfg.precision == HEXO_FP32 ? ctx->shape_f32 : ctx->shape_f64;
    if (cfg.block) sh.block = cfg.block;
    if (cfg.paths_per_thread) sh.ppt = cfg.paths_per_thread;
    if (cfg.unroll) sh.unroll = cfg.unroll;
    if (cfg.control_variate) {   // its kernels run one path per thread, no unroll
        sh.cv = true;
        if (!cfg.paths_per_thread) sh.ppt = 1;
        if (!cfg.unroll) sh.unroll = 1;
    }
    return sh;
}

// A batch with fewer paths than the default shape's CTA slots (2 per SM of
// 256 threads, one path each) would leave SMs with one CTA and others with
// two; with narrower CTAs (a multiple of 32 threads, at least 128) the same
// paths spread over every slot, so the most loaded SM runs fewer warps.
// Only the default shape is changed (not an explicit or tuned one); the
// launch shape does not change results.
void fit_small_batch(hexo_ctx *ctx, const hexo_mc_cfg &cfg, LaunchShape &sh, const std::vector<SetPlan> &plans) {
    const LaunchShape def{256, 1, 1};
    const LaunchShape &tuned = cfg.precision == HEXO_FP32 ? ctx->shape_f32 : ctx->shape_f64;
    if (cfg.block || cfg.paths_per_thread || cfg.unroll || sh.block != def.block || sh.ppt != def.ppt ||
        tuned.block != def.block || tuned.ppt != def.ppt || tuned.unroll != def.unroll)
        return;
    uint64_t paths = 0;
    for (const SetPlan &sp : plans) paths += sp.path_hi - sp.path_lo;
    const uint64_t slots = (uint64_t)ctx->sm_count * 2;
    if (paths == 0 || paths >= slots * def.block) return;
    const uint64_t per = (paths + slots - 1) / slots;
    sh.block = (uint32_t)std::max<uint64_t>(128, (per + 31) / 32 * 32);
}

hexo_status shape_check(hexo_ctx *ctx, bool f32, const LaunchShape &sh, size_t &smem, uint32_t &ctas_per_sm) {
    const void *fn = paths_kernel_ptr(f32, sh.ppt, sh.unroll, sh.cv);
    if (fn == nullptr || sh.block == 0 || sh.block % 32 != 0 || sh.block > 512)
        return ctx_fail(ctx, HEXO_ERR_INVALID, "unsupported launch shape (block multiple of 32 up to 512, ppt/unroll in {1,2,4})");
    smem = paths_smem_bytes(sh.block, sh.ppt);
    size_t smem_static = 0;
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, fn) == cudaSuccess) smem_static = fa.sharedSizeBytes;
    if (smem + smem_static > ctx->smem_optin)
        return ctx_fail(ctx, HEXO_ERR_INVALID, "launch shape needs more shared memory than a CTA can have");
    cudaError_t e = paths_smem_limit(fn, ctx->device);   // the same value for every caller
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaFuncSetAttribute");
    int nb = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, (int)sh.block, smem);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
    if (nb <= 0) return ctx_fail(ctx, HEXO_ERR_INVALID, "launch shape does not fit on an SM");
    ctas_per_sm = (uint32_t)nb;
    return HEXO_OK;
}

// ------------------------------------------------------------ device batch

DeviceBatch::~DeviceBatch() {
    if (graph_exec) cudaGraphExecDestroy(graph_exec);
    if (ev_k0) cudaEventDestroy(ev_k0);
    if (ev_k1) cudaEventDestroy(ev_k1);
    if (dmem && own_d) cudaFree(dmem);
    if (hmem && own_h) cudaFreeHost(hmem);
}

namespace {
size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }
}

hexo_status batch_upload(hexo_ctx *ctx, BatchPlan &&plan, bool f32, DeviceBatch &db) {
    db.ctx = ctx;
    if (db.stream == nullptr) db.stream = ctx->stream;
    db.f32 = f32;
    db.plan = std::move(plan);
    BatchPlan &bp = db.plan;
    hexo_status s = shape_check(ctx, f32, bp.shape, db.smem, db.ctas_per_sm);
    if (s != HEXO_OK) return s;
    const uint32_t n_out = bp.n_out;
    db.grid = std::max<uint32_t>(1, std::min<uint32_t>(ctx->sm_count * db.ctas_per_sm, (uint32_t)bp.tiles.size()));
    db.n_slots = std::max<uint32_t>(1, std::min<uint32_t>(db.grid, kSumSlots));   // private copies of the sums
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off = align_up(off + bytes, 256); return o; };
    const size_t o_sets = take(bp.sets.size() * sizeof(SetDesc));
    const size_t o_segs = take(bp.segs.size() * sizeof(SegDesc));
    const size_t o_mats = take(bp.mats.size() * sizeof(MatDesc));
    const size_t o_opts = take(bp.opts.size() * sizeof(OptDesc));
    const size_t o_tiles = take(std::max<size_t>(1, bp.tiles.size()) * sizeof(TileDesc));
    const size_t o_paths = take(n_out * sizeof(uint64_t));
    const size_t o_disc = take(n_out * sizeof(double));
    const size_t o_pexp = take(n_out * sizeof(int32_t));
    const bool carried = db.carry != nullptr;   // the serving loop's split requests
    const size_t o_carry = take(carried ? n_out * sizeof(uint64_t) : 0);
    const size_t o_acc = take((size_t)db.n_slots * n_out * kLimbs * sizeof(unsigned long long));
    const size_t o_acc_sum = take((size_t)n_out * kLimbs * sizeof(unsigned long long));
    const size_t o_price = take(n_out * sizeof(double));
    const size_t o_se = take(n_out * sizeof(double));
    const size_t o_ctl = take(kCtlBytes);   // queue head, error flags, exponential-branch steps
    CvPlan cvp;                              // the control variate's analytic part (host vectors until the sync)
    if (!bp.cv.empty()) cv_plan(bp, cvp);
    const size_t o_cv = take(cvp.bytes);
    db.bytes = off;
    cudaError_t e = cudaSuccess;
    if (db.dmem == nullptr || db.dcap < db.bytes) {
        db.dmem = nullptr;
        db.own_d = true;
        e = cudaMalloc(&db.dmem, db.bytes);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMalloc batch");
        db.dcap = db.bytes;
    }
    // pinned host mirror of outputs: price, se, acc, ctl
    size_t hoff = 0;
    const size_t h_price = hoff; hoff = align_up(hoff + n_out * sizeof(double), 64);
    const size_t h_se = hoff; hoff = align_up(hoff + n_out * sizeof(double), 64);
    const size_t h_acc = hoff; hoff = align_up(hoff + (size_t)n_out * kLimbs * sizeof(unsigned long long), 64);
    const size_t h_ctl = hoff; hoff = align_up(hoff + kCtlBytes, 64);
    if (db.hmem == nullptr || db.hcap < hoff) {
        db.hmem = nullptr;
        db.own_h = true;
        e = cudaMallocHost(&db.hmem, hoff);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMallocHost batch");
        db.hcap = hoff;
    }
    char *d = static_cast<char *>(db.dmem);
    char *h = static_cast<char *>(db.hmem);
    db.h_price = reinterpret_cast<double *>(h + h_price);
    db.h_se = reinterpret_cast<double *>(h + h_se);
    db.h_acc = reinterpret_cast<unsigned long long *>(h + h_acc);
    db.h_ctl = reinterpret_cast<uint32_t *>(h + h_ctl);

    KernelArgs &a = db.args;
    std::memset(&a, 0, sizeof(a));
    a.sets = reinterpret_cast<const SetDesc *>(d + o_sets);
    a.segs = reinterpret_cast<const SegDesc *>(d + o_segs);
    a.mats = reinterpret_cast<const MatDesc *>(d + o_mats);
    a.opts = reinterpret_cast<const OptDesc *>(d + o_opts);
    a.tiles = reinterpret_cast<const TileDesc *>(d + o_tiles);
    a.n_tiles = (uint32_t)bp.tiles.size();
    a.acc = reinterpret_cast<unsigned long long *>(d + o_acc);
    a.n_slots = db.n_slots;
    a.acc_slot_stride = (uint64_t)n_out * kLimbs;
    db.d_acc_sum = reinterpret_cast<unsigned long long *>(d + o_acc_sum);
    a.queue = reinterpret_cast<unsigned int *>(d + o_ctl);
    a.error = reinterpret_cast<int *>(d + o_ctl + sizeof(uint32_t));
    a.exp_steps = reinterpret_cast<unsigned long long *>(d + o_ctl + 2 * sizeof(uint32_t));
    a.check = reinterpret_cast<unsigned int *>(d + o_ctl + 4 * sizeof(uint32_t));
    a.n_out = n_out;
    a.n_sets = (uint32_t)bp.sets.size();
    a.n_segs = (uint32_t)bp.segs.size();
    a.n_mats = (uint32_t)bp.mats.size();
    a.n_opts = (uint32_t)bp.opts.size();
    db.d_paths = reinterpret_cast<uint64_t *>(d + o_paths);
    db.d_disc = reinterpret_cast<double *>(d + o_disc);
    db.d_pexp = reinterpret_cast<int32_t *>(d + o_pexp);
    db.d_carry_row = carried ? reinterpret_cast<uint64_t *>(d + o_carry) : nullptr;
    db.d_price = reinterpret_cast<double *>(d + o_price);
    db.d_se = reinterpret_cast<double *>(d + o_se);

    cudaStream_t st = db.stream;
    auto up = [&](size_t o, const void *src, size_t bytes) -> cudaError_t {
        if (bytes == 0) return cudaSuccess;
        return cudaMemcpyAsync(d + o, src, bytes, cudaMemcpyHostToDevice, st);
    };
    if ((e = up(o_sets, bp.sets.data(), bp.sets.size() * sizeof(SetDesc))) != cudaSuccess ||
        (e = up(o_segs, bp.segs.data(), bp.segs.size() * sizeof(SegDesc))) != cudaSuccess ||
        (e = up(o_mats, bp.mats.data(), bp.mats.size() * sizeof(MatDesc))) != cudaSuccess ||
        (e = up(o_opts, bp.opts.data(), bp.opts.size() * sizeof(OptDesc))) != cudaSuccess ||
        (e = up(o_tiles, bp.tiles.data(), bp.tiles.size() * sizeof(TileDesc))) != cudaSuccess ||
        (e = up(o_paths, bp.opt_paths.data(), n_out * sizeof(uint64_t))) != cudaSuccess ||
        (e = up(o_disc, bp.opt_disc.data(), n_out * sizeof(double))) != cudaSuccess ||
        (e = up(o_pexp, bp.opt_pexp.data(), n_out * sizeof(int32_t))) != cudaSuccess ||
        (carried && (e = up(o_carry, bp.opt_carry.data(), n_out * sizeof(uint64_t))) != cudaSuccess))
        return cuda_fail(ctx, e, "upload batch");
    db.d_cv_eg = nullptr;
    db.d_cv_partner = nullptr;
    if (!bp.cv.empty() && (e = cv_run(cvp, d + o_cv, st, &db.d_cv_eg, &db.d_cv_partner)) != cudaSuccess)
        return cuda_fail(ctx, e, "control variate");
    e = cudaStreamSynchronize(st);   // the host vectors are pageable: finish before they can change
    if (e != cudaSuccess) return cuda_fail(ctx, e, "upload batch");
    db.h2d_bytes = bp.sets.size() * sizeof(SetDesc) + bp.segs.size() * sizeof(SegDesc) +
                   bp.mats.size() * sizeof(MatDesc) + bp.opts.size() * sizeof(OptDesc) +
                   bp.tiles.size() * sizeof(TileDesc) + n_out * (sizeof(uint64_t) + sizeof(double) + sizeof(int32_t));
    if ((e = cudaEventCreate(&db.ev_k0)) != cudaSuccess || (e = cudaEventCreate(&db.ev_k1)) != cudaSuccess)
        return cuda_fail(ctx, e, "cudaEventCreate");
    return HEXO_OK;
}

// Enqueues one run: clear sums and queue, path kernel, finaliser, copies back.
cudaError_t batch_enqueue(DeviceBatch &db, cudaStream_t st, bool copy_acc) {
    const uint32_t n_out = db.plan.n_out;
    cudaError_t e;
    if ((e = cudaMemsetAsync(db.args.acc, 0, (size_t)db.n_slots * n_out * kLimbs * sizeof(unsigned long long), st)) !=
        cudaSuccess)
        return e;
    if ((e = cudaMemsetAsync(db.args.queue, 0, kCtlBytes, st)) != cudaSuccess) return e;
    // inside a stream capture the timing events become event-record nodes of the graph
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if ((e = cudaStreamIsCapturing(st, &cap)) != cudaSuccess) return e;
    const unsigned rec_flags = cap == cudaStreamCaptureStatusActive ? cudaEventRecordExternal : cudaEventRecordDefault;
    if ((e = cudaEventRecordWithFlags(db.ev_k0, st, rec_flags)) != cudaSuccess) return e;
    if (db.args.n_tiles > 0)
        if ((e = launch_paths(db.f32, db.plan.shape, db.grid, db.smem, st, db.args)) != cudaSuccess) return e;
    if ((e = cudaEventRecordWithFlags(db.ev_k1, st, rec_flags)) != cudaSuccess) return e;
    FinalizeArgs fa;
    fa.acc = db.args.acc;
    fa.n_slots = db.n_slots;
    fa.slot_stride = db.args.acc_slot_stride;
    fa.n_paths = db.d_paths;
    fa.disc = db.d_disc;
    fa.pay_exp = db.d_pexp;
    fa.n = n_out;
    fa.price = db.d_price;
    fa.se = db.d_se;
    fa.acc_sum = db.d_acc_sum;
    fa.cv_eg = db.d_cv_eg;
    fa.cv_partner = db.d_cv_partner;
    fa.carry = db.carry;
    fa.carry_row = db.d_carry_row;
    if ((e = launch_finalize(fa, st)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(db.h_price, db.d_price, n_out * sizeof(double), cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(db.h_se, db.d_se, n_out * sizeof(double), cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
    if (copy_acc)
        if ((e = cudaMemcpyAsync(db.h_acc, db.d_acc_sum, (size_t)n_out * kLimbs * sizeof(unsigned long long),
                                 cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
    return cudaMemcpyAsync(db.h_ctl, db.args.queue, kCtlBytes, cudaMemcpyDeviceToHost, st);
}

hexo_status batch_wait(DeviceBatch &db) {
    cudaError_t e = cudaStreamSynchronize(db.stream);
    if (e != cudaSuccess) return cuda_fail(db.ctx, e, "batch run");
    if (db.h_ctl[1] & kErrCheck)
        return ctx_fail(db.ctx, HEXO_ERR_CHECK,
                        "a bounds check of the path kernel failed: code " + std::to_string(db.h_ctl[4] >> 24) +
                            ", detail " + std::to_string(db.h_ctl[4] & 0xffffffu));
    if (db.h_ctl[1] != 0u)
        return ctx_fail(db.ctx, HEXO_ERR_NUMERIC,
                        "a payoff was not finite or outside the fixed-point range [0, 2^16 * 2^E), 2^(E-1) <= S0 < 2^E");
    return HEXO_OK;
}

hexo_status plan_requests(hexo_ctx *ctx, const hexo_request *reqs, uint32_t n_reqs, const hexo_mc_cfg &cfg,
                          uint64_t path_lo, uint64_t path_hi, BatchPlan &bp, std::vector<SetPlan> &plans,
                          uint32_t shard, uint32_t n_shards) {
    if (reqs == nullptr || n_reqs == 0) return ctx_fail(ctx, HEXO_ERR_INVALID, "no requests");
    plans.resize(n_reqs);
    uint32_t out_base = 0, cv_base = 0;
    for (uint32_t r = 0; r < n_reqs; ++r) cv_base += reqs[r].n_opts;   // internal slots after all outputs
    for (uint32_t r = 0; r < n_reqs; ++r) {
        std::string err;
        hexo_status s = plan_set(reqs[r].params, reqs[r].S0, reqs[r].opts, reqs[r].n_opts, cfg, reqs[r].seed,
                                 reqs[r].stream, path_lo, path_hi, plans[r], err);
        if (s != HEXO_OK) return ctx_fail(ctx, s, "request " + std::to_string(r) + ": " + err);
        if (n_shards > 1) {   // this shard's contiguous range of the request's paths
            SetPlan &sp = plans[r];
            const uint64_t n = sp.path_hi, base = n / n_shards, extra = n % n_shards;
            sp.path_lo = shard * base + std::min<uint64_t>(shard, extra);
            sp.path_hi = sp.path_lo + base + (shard < extra ? 1 : 0);
            sp.set.n_paths = sp.path_hi;
        }
        batch_add(bp, plans[r], out_base, cv_base);
        out_base += reqs[r].n_opts;
        cv_base += 2u * plans[r].n_cv;
    }
    bp.shape = ctx_shape(ctx, cfg);
    fit_small_batch(ctx, cfg, bp.shape, plans);
    batch_tiles(bp, plans);
    return HEXO_OK;
}

void scatter_outputs(const DeviceBatch &db, const hexo_request *reqs, uint32_t n_reqs) {
    uint32_t base = 0;
    for (uint32_t r = 0; r < n_reqs; ++r) {
        for (uint32_t i = 0; i < reqs[r].n_opts; ++i) {
            if (reqs[r].price_out) reqs[r].price_out[i] = db.h_price[base + i];
            if (reqs[r].stderr_out) reqs[r].stderr_out[i] = db.h_se[base + i];
        }
        base += reqs[r].n_opts;
    }
}

} // namespace hexo

// ----------------------------------------------------------------- C ABI

extern "C" {

const char *hexo_status_string(hexo_status s) {
    switch (s) {
    case HEXO_OK: return "ok";
    case HEXO_ERR_INVALID: return "invalid argument";
    case HEXO_ERR_CUDA: return "CUDA error";
    case HEXO_ERR_NOMEM: return "out of memory";
    case HEXO_ERR_UNSUPPORTED: return "unsupported";
    case HEXO_ERR_TIMEOUT: return "timeout";
    case HEXO_ERR_NUMERIC: return "numeric range error";
    case HEXO_ERR_NOT_FOUND: return "not found";
    case HEXO_ERR_ADMISSION: return "request exceeds the device-memory cap";
    case HEXO_ERR_SHUTDOWN: return "server shut down";
    case HEXO_ERR_TOO_LARGE: return "request exceeds the no-allocation entry point's limits";
    case HEXO_ERR_CHECK: return "a bounds check of the checked build failed";
    }
    return "unknown status";
}

uint32_t hexo_abi_version(void) { return HEXO_ABI_VERSION; }

void hexo_mc_cfg_default(hexo_mc_cfg *cfg) {
    if (!cfg) return;
    std::memset(cfg, 0, sizeof(*cfg));
    cfg->n_paths = 65536;
    cfg->step_mode = HEXO_STEP_REFERENCE;
    cfg->steps = 252;
    cfg->steps_per_year = 252.0;
    cfg->seed = 42;
    cfg->rng_block_words = 16;
    cfg->precision = HEXO_FP64;
}

hexo_status hexo_ctx_create(hexo_ctx **out, const hexo_ctx_opts *opts) {
    if (out == nullptr) return HEXO_ERR_INVALID;
    *out = nullptr;
    hexo_ctx *ctx = new (std::nothrow) hexo_ctx();
    if (!ctx) return HEXO_ERR_NOMEM;
    ctx->device = opts ? opts->device : 0;
    ctx->mem_cap = (opts && opts->mem_cap_bytes) ? opts->mem_cap_bytes : (32ull << 30);
    if (opts && opts->autotune_cache) ctx->tune_cache = opts->autotune_cache;
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    int v = 0;
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, ctx->device);
    ctx->sm_count = (uint32_t)v;
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device);
    ctx->smem_optin = (size_t)v;
    if (e != cudaSuccess) {
        delete ctx;
        return e == cudaErrorMemoryAllocation ? HEXO_ERR_NOMEM : HEXO_ERR_CUDA;
    }
    tune_load(ctx);
    *out = ctx;
    return HEXO_OK;
}

hexo_status hexo_ctx_destroy(hexo_ctx *ctx) {
    if (!ctx) return HEXO_ERR_INVALID;
    cudaSetDevice(ctx->device);
    if (ctx->stream) {
        cudaStreamSynchronize(ctx->stream);
        cudaStreamDestroy(ctx->stream);
    }
    if (ctx->arena_d) cudaFree(ctx->arena_d);
    if (ctx->arena_h) cudaFreeHost(ctx->arena_h);
    delete ctx;
    return HEXO_OK;
}

hexo_status hexo_ctx_trim(hexo_ctx *ctx) {
    if (!ctx) return HEXO_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->run_mu);
    cudaSetDevice(ctx->device);
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "hexo_ctx_trim");
    if (ctx->arena_d) cudaFree(ctx->arena_d);
    if (ctx->arena_h) cudaFreeHost(ctx->arena_h);
    ctx->arena_d = ctx->arena_h = nullptr;
    ctx->arena_dcap = ctx->arena_hcap = 0;
    return HEXO_OK;
}

hexo_status hexo_ctx_last_error(hexo_ctx *ctx, char *buf, size_t buf_len) {
    if (!ctx || !buf || buf_len == 0) return HEXO_ERR_INVALID;
    std::lock_guard<std::mutex> g(ctx->err_mu);
    std::strncpy(buf, ctx->last_error.c_str(), buf_len - 1);
    buf[buf_len - 1] = '\0';
    return HEXO_OK;
}

void *hexo_ctx_stream(hexo_ctx *ctx) { return ctx ? (void *)ctx->stream : nullptr; }

hexo_status hexo_price_batch(hexo_ctx *ctx, const hexo_request *reqs, uint32_t n_reqs, const hexo_mc_cfg *cfg) {
    if (!ctx || !cfg) return HEXO_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->run_mu);
    cudaSetDevice(ctx->device);
    NvtxRange call("hexo_price_batch");
    BatchPlan bp;
    std::vector<SetPlan> plans;
    hexo_status s;
    {
        NvtxRange r("plan");
        s = plan_requests(ctx, reqs, n_reqs, *cfg, 0, ~0ull, bp, plans);
    }
    if (s != HEXO_OK) return s;
    DeviceBatch db;
    ArenaLoan loan(ctx, db);
    {
        NvtxRange r("upload");
        s = batch_upload(ctx, std::move(bp), cfg->precision == HEXO_FP32, db);
    }
    if (s != HEXO_OK) return s;
    NvtxRange r("run");
    cudaError_t e = batch_enqueue(db, ctx->stream, false);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "batch launch");
    if ((s = batch_wait(db)) != HEXO_OK) return s;
    scatter_outputs(db, reqs, n_reqs);
    return HEXO_OK;
}

hexo_status hexo_price(hexo_ctx *ctx, const hexo_params *p, double S0, const hexo_option *opts, uint32_t n_opts,
                       const hexo_mc_cfg *cfg, double *price_out, double *stderr_out) {
    if (!ctx || !p || !cfg || !price_out) return HEXO_ERR_INVALID;
    hexo_request r;
    r.params = *p;
    r.S0 = S0;
    r.opts = opts;
    r.n_opts = n_opts;
    r.seed = cfg->seed;
    r.stream = cfg->stream;
    r.reserved = 0;
    r.price_out = price_out;
    r.stderr_out = stderr_out;
    return hexo_price_batch(ctx, &r, 1, cfg);
}

hexo_status hexo_batch_prepare(hexo_ctx *ctx, const hexo_request *reqs, uint32_t n_reqs, const hexo_mc_cfg *cfg,
                               hexo_batch **out) {
    if (!ctx || !cfg || !out) return HEXO_ERR_INVALID;
    *out = nullptr;
    return batch_prepare(ctx, reqs, n_reqs, cfg, 0, 1, out);
}

} // extern "C"

namespace hexo {

hexo_status batch_prepare(hexo_ctx *ctx, const hexo_request *reqs, uint32_t n_reqs, const hexo_mc_cfg *cfg,
                          uint32_t shard, uint32_t n_shards, hexo_batch **out) {
    std::lock_guard<std::mutex> lk(ctx->run_mu);
    cudaSetDevice(ctx->device);
    hexo_batch *b = new (std::nothrow) hexo_batch();
    if (!b) return HEXO_ERR_NOMEM;
    BatchPlan bp;
    std::vector<SetPlan> plans;
    hexo_status s = plan_requests(ctx, reqs, n_reqs, *cfg, 0, ~0ull, bp, plans, shard, n_shards);
    if (s == HEXO_OK) s = batch_upload(ctx, std::move(bp), cfg->precision == HEXO_FP32, b->db);
    if (s != HEXO_OK) { delete b; return s; }
    b->reqs.assign(reqs, reqs + n_reqs);
    b->partial = n_shards > 1;
    // capture one run in a graph
    cudaStream_t st = ctx->stream;
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        cudaError_t e2 = batch_enqueue(b->db, st, b->partial);
        e = cudaStreamEndCapture(st, &graph);
        if (e2 != cudaSuccess) e = e2;
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&b->db.graph_exec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
        delete b;
        return cuda_fail(ctx, e, "graph capture");
    }
    *out = b;
    return HEXO_OK;
}

} // namespace hexo

extern "C" {

hexo_status hexo_batch_launch(hexo_batch *b) {
    if (!b) return HEXO_ERR_INVALID;
    hexo_ctx *ctx = b->db.ctx;
    cudaSetDevice(ctx->device);
    NvtxRange r("hexo_batch_launch");
    cudaError_t e = cudaGraphLaunch(b->db.graph_exec, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaGraphLaunch");
    return HEXO_OK;
}

hexo_status hexo_batch_collect(hexo_batch *b) {
    if (!b) return HEXO_ERR_INVALID;
    cudaSetDevice(b->db.ctx->device);
    NvtxRange r("hexo_batch_collect");
    hexo_status s = batch_wait(b->db);
    if (s != HEXO_OK) return s;
    if (!b->partial) scatter_outputs(b->db, b->reqs.data(), (uint32_t)b->reqs.size());
    return HEXO_OK;
}

hexo_status hexo_batch_info_get(hexo_batch *b, hexo_batch_info *info) {
    if (!b || !info) return HEXO_ERR_INVALID;
    const BatchPlan &bp = b->db.plan;
    info->nominal_path_steps = bp.nominal_path_steps;
    info->executed_path_steps = bp.executed_path_steps;
    info->n_paths = bp.n_paths;
    info->n_tiles = (uint32_t)bp.tiles.size();
    info->n_sets = (uint32_t)bp.sets.size();
    info->n_options = bp.n_out - 2u * (uint32_t)bp.cv.size();   // without the control variate's internal slots
    info->block = bp.shape.block;
    info->paths_per_thread = bp.shape.ppt;
    info->unroll = bp.shape.unroll;
    info->grid = b->db.grid;
    info->device_bytes = b->db.bytes;
    info->h2d_bytes = b->db.h2d_bytes;
    info->d2h_bytes = (uint64_t)bp.n_out * 2 * sizeof(double) + kCtlBytes;
    float ms = 0.0f;
    info->last_kernel_ms = cudaEventElapsedTime(&ms, b->db.ev_k0, b->db.ev_k1) == cudaSuccess ? (double)ms : -1.0;
    uint64_t exp_steps = 0;   // counted by the kernels; every other executed step took the quadratic branch
    std::memcpy(&exp_steps, b->db.h_ctl + 2, sizeof(uint64_t));
    info->quad_steps = bp.executed_path_steps - std::min(exp_steps, bp.executed_path_steps);
    return HEXO_OK;
}

hexo_status hexo_batch_destroy(hexo_batch *b) {
    if (!b) return HEXO_ERR_INVALID;
    cudaSetDevice(b->db.ctx->device);
    cudaStreamSynchronize(b->db.ctx->stream);
    delete b;
    return HEXO_OK;
}

hexo_status hexo_price_partial(hexo_ctx *ctx, const hexo_params *p, double S0, const hexo_option *opts,
                               uint32_t n_opts, const hexo_mc_cfg *cfg, uint64_t path_lo, uint64_t path_hi,
                               uint64_t *limbs_out) {
    if (!ctx || !p || !cfg || !limbs_out) return HEXO_ERR_INVALID;
    if (path_hi < path_lo) return ctx_fail(ctx, HEXO_ERR_INVALID, "path_hi < path_lo");
    if (cfg->control_variate)
        return ctx_fail(ctx, HEXO_ERR_UNSUPPORTED, "the control variate is not supported by partial sums");
    std::lock_guard<std::mutex> lk(ctx->run_mu);
    cudaSetDevice(ctx->device);
    hexo_request r;
    std::memset(&r, 0, sizeof(r));
    r.params = *p;
    r.S0 = S0;
    r.opts = opts;
    r.n_opts = n_opts;
    r.seed = cfg->seed;
    r.stream = cfg->stream;
    BatchPlan bp;
    std::vector<SetPlan> plans;
    hexo_status s = plan_requests(ctx, &r, 1, *cfg, path_lo, path_hi, bp, plans);
    if (s != HEXO_OK) return s;
    DeviceBatch db;
    ArenaLoan loan(ctx, db);
    if ((s = batch_upload(ctx, std::move(bp), cfg->precision == HEXO_FP32, db)) != HEXO_OK) return s;
    cudaError_t e = batch_enqueue(db, ctx->stream, true);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "partial launch");
    if ((s = batch_wait(db)) != HEXO_OK) return s;
    std::memcpy(limbs_out, db.h_acc, (size_t)n_opts * kLimbs * sizeof(uint64_t));
    return HEXO_OK;
}

hexo_status hexo_price_batch_partial(hexo_ctx *ctx, const hexo_request *reqs, uint32_t n_reqs, const hexo_mc_cfg *cfg,
                                     uint32_t shard, uint32_t n_shards, uint64_t *limbs_out) {
    if (!ctx || !cfg || !limbs_out || n_shards == 0) return HEXO_ERR_INVALID;
    if (shard >= n_shards) return ctx_fail(ctx, HEXO_ERR_INVALID, "shard must be below n_shards");
    if (cfg->control_variate)
        return ctx_fail(ctx, HEXO_ERR_UNSUPPORTED, "the control variate is not supported by partial sums");
    std::lock_guard<std::mutex> lk(ctx->run_mu);
    cudaSetDevice(ctx->device);
    NvtxRange call("hexo_price_batch_partial");
    BatchPlan bp;
    std::vector<SetPlan> plans;
    hexo_status s = plan_requests(ctx, reqs, n_reqs, *cfg, 0, ~0ull, bp, plans, shard, n_shards);
    if (s != HEXO_OK) return s;
    const uint32_t n_out = bp.n_out;
    DeviceBatch db;
    ArenaLoan loan(ctx, db);
    if ((s = batch_upload(ctx, std::move(bp), cfg->precision == HEXO_FP32, db)) != HEXO_OK) return s;
    cudaError_t e = batch_enqueue(db, ctx->stream, true);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "partial launch");
    if ((s = batch_wait(db)) != HEXO_OK) return s;
    std::memcpy(limbs_out, db.h_acc, (size_t)n_out * kLimbs * sizeof(uint64_t));
    return HEXO_OK;
}

hexo_status hexo_batch_prepare_partial(hexo_ctx *ctx, const hexo_request *reqs, uint32_t n_reqs,
                                       const hexo_mc_cfg *cfg, uint32_t shard, uint32_t n_shards, hexo_batch **out) {
    if (!ctx || !cfg || !out || n_shards == 0) return HEXO_ERR_INVALID;
    *out = nullptr;
    if (shard >= n_shards) return ctx_fail(ctx, HEXO_ERR_INVALID, "shard must be below n_shards");
    if (cfg->control_variate)
        return ctx_fail(ctx, HEXO_ERR_UNSUPPORTED, "the control variate is not supported by partial sums");
    return batch_prepare(ctx, reqs, n_reqs, cfg, shard, n_shards, out);
}

hexo_status hexo_batch_collect_limbs(hexo_batch *b, uint64_t *limbs_out) {
    if (!b || !limbs_out) return HEXO_ERR_INVALID;
    cudaSetDevice(b->db.ctx->device);
    hexo_status s = batch_wait(b->db);
    if (s != HEXO_OK) return s;
    std::memcpy(limbs_out, b->db.h_acc, (size_t)b->db.plan.n_out * kLimbs * sizeof(uint64_t));
    return HEXO_OK;
}

hexo_status hexo_finalize_limbs(const hexo_params *p, double S0, const hexo_option *opts, uint32_t n_opts,
                                const hexo_mc_cfg *cfg, const uint64_t *limbs, double *price_out, double *stderr_out) {
    if (!p || !opts || !cfg || !limbs || !price_out) return HEXO_ERR_INVALID;
    if (!std::isfinite(S0) || !(S0 >= 0x1p-60) || !(S0 < 0x1p60)) return HEXO_ERR_INVALID;
    const int E = pay_exponent(S0);
    for (uint32_t i = 0; i < n_opts; ++i) {
        const uint64_t n = opts[i].n_paths ? opts[i].n_paths : cfg->n_paths;
        if (n == 0) return HEXO_ERR_INVALID;
        double pr, se;
        finalize_one(limbs + (size_t)i * kLimbs, n, std::exp(-p->r * opts[i].T), E, &pr, &se);
        price_out[i] = pr;
        if (stderr_out) stderr_out[i] = se;
    }
    return HEXO_OK;
}

// -------------------------------------------------------------- planning

hexo_status hexo_plan_stats_get(const hexo_request *reqs, uint32_t n_reqs, const hexo_mc_cfg *cfg,
                                hexo_plan_stats *out) {
    if (!reqs || n_reqs == 0 || !cfg || !out) return HEXO_ERR_INVALID;
    BatchPlan bp;
    std::vector<SetPlan> plans(n_reqs);
    uint32_t base = 0, n_mats = 0, n_segs = 0, cv_base = 0;
    for (uint32_t r = 0; r < n_reqs; ++r) cv_base += reqs[r].n_opts;
    for (uint32_t r = 0; r < n_reqs; ++r) {
        std::string err;
        hexo_status s = plan_set(reqs[r].params, reqs[r].S0, reqs[r].opts, reqs[r].n_opts, *cfg, reqs[r].seed,
                                 reqs[r].stream, 0, ~0ull, plans[r], err);
        if (s != HEXO_OK) return s;
        batch_add(bp, plans[r], base, cv_base);
        base += reqs[r].n_opts;
        cv_base += 2u * plans[r].n_cv;
        n_mats += (uint32_t)plans[r].mats.size();
        n_segs += (uint32_t)plans[r].segs.size();
    }
    bp.shape.block = cfg->block ? cfg->block : 256;
    bp.shape.ppt = cfg->paths_per_thread ? cfg->paths_per_thread : 1;
    batch_tiles(bp, plans);
    out->nominal_path_steps = bp.nominal_path_steps;
    out->executed_path_steps = bp.executed_path_steps;
    out->n_paths = bp.n_paths;
    out->n_maturities = n_mats;
    out->n_segments = n_segs;
    out->n_tiles = (uint32_t)bp.tiles.size();
    out->n_options = base;   // the requests' options (not the control variate's internal slots)
    return HEXO_OK;
}

hexo_status hexo_plan_schedule(const hexo_params *p, double S0, const hexo_option *opts, uint32_t n_opts,
                               const hexo_mc_cfg *cfg, uint32_t cap, uint64_t *steps_to_mat, double *tmtp,
                               double *maturity, uint32_t *n_mats) {
    if (!p || !cfg || !n_mats) return HEXO_ERR_INVALID;
    SetPlan sp;
    std::string err;
    hexo_status s = plan_set(*p, S0, opts, n_opts, *cfg, cfg->seed, cfg->stream, 0, ~0ull, sp, err);
    if (s != HEXO_OK) return s;
    *n_mats = (uint32_t)sp.mats.size();
    for (uint32_t j = 0; j < *n_mats && j < cap; ++j) {
        if (steps_to_mat) steps_to_mat[j] = sp.steps_to_mat[j];
        if (tmtp) tmtp[j] = sp.mats[j].tmtp;
        if (maturity) maturity[j] = sp.mats[j].T;
    }
    return HEXO_OK;
}

// ----------------------------------------------------------------- debug

hexo_status hexo_debug_rng_words(hexo_ctx *ctx, uint32_t seed, uint32_t stream, uint32_t n_streams, uint32_t n_words,
                                 uint64_t *out) {
    if (!ctx || !out || n_streams == 0 || n_words == 0) return HEXO_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->run_mu);
    cudaSetDevice(ctx->device);
    DevBuf d;
    const size_t bytes = (size_t)n_streams * n_words * sizeof(uint64_t);
    cudaError_t e = d.alloc(bytes);
    if (e == cudaSuccess) e = launch_dbg_words(seed, stream, n_streams, n_words, (uint64_t *)d.p, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, d.p, bytes, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    return e == cudaSuccess ? HEXO_OK : cuda_fail(ctx, e, "debug rng words");
}

hexo_status hexo_debug_rng_draws(hexo_ctx *ctx, uint32_t seed, uint32_t stream, uint32_t n_streams,
                                 const uint8_t *kinds, uint32_t n, double *out) {
    if (!ctx || !out || !kinds || n_streams == 0 || n == 0) return HEXO_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->run_mu);
    cudaSetDevice(ctx->device);
    DevBuf dk, dout;
    const size_t bytes = (size_t)n_streams * n * sizeof(double);
    cudaError_t e = dk.alloc(n);
    if (e == cudaSuccess) e = dout.alloc(bytes);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dk.p, kinds, n, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess)
        e = launch_dbg_draws(seed, stream, n_streams, (const uint8_t *)dk.p, n, (double *)dout.p, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, dout.p, bytes, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    return e == cudaSuccess ? HEXO_OK : cuda_fail(ctx, e, "debug rng draws");
}

hexo_status hexo_debug_normals(hexo_ctx *ctx, const uint64_t *words, uint64_t n, double *out) {
    if (!ctx || !words || !out || n == 0) return HEXO_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->run_mu);
    cudaSetDevice(ctx->device);
    DevBuf dw, dout;
    cudaError_t e = dw.alloc(n * sizeof(uint64_t));
    if (e == cudaSuccess) e = dout.alloc(n * sizeof(double));
    if (e == cudaSuccess) e = cudaMemcpyAsync(dw.p, words, n * sizeof(uint64_t), cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = launch_dbg_normals((const uint64_t *)dw.p, n, (double *)dout.p, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, dout.p, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    return e == cudaSuccess ? HEXO_OK : cuda_fail(ctx, e, "debug normals");
}

hexo_status hexo_debug_as241_check(hexo_ctx *ctx, uint32_t branch, uint64_t bits_lo, uint64_t bits_hi,
                                   uint64_t *out2) {
    if (!ctx || !out2 || branch > 2u || bits_hi > (1ull << 32) || bits_lo > bits_hi) return HEXO_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->run_mu);
    cudaSetDevice(ctx->device);
    DevBuf dout;
    const unsigned long long init[2] = {0ull, ~0ull};
    cudaError_t e = dout.alloc(sizeof(init));
    if (e == cudaSuccess) e = cudaMemcpyAsync(dout.p, init, sizeof(init), cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess)
        e = launch_dbg_as241_check(branch, bits_lo, bits_hi, (unsigned long long *)dout.p, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out2, dout.p, sizeof(init), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    return e == cudaSuccess ? HEXO_OK : cuda_fail(ctx, e, "debug AS241 check");
}

hexo_status hexo_debug_payoff_limbs(hexo_ctx *ctx, const double *pay, uint64_t n, uint32_t precision, double S0,
                                    uint32_t *out) {
    if (!ctx || !pay || !out || n == 0) return HEXO_ERR_INVALID;
    if (precision != HEXO_FP64 && precision != HEXO_FP32) return ctx_fail(ctx, HEXO_ERR_INVALID, "unknown precision");
    if (!std::isfinite(S0) || !(S0 >= 0x1p-60) || !(S0 < 0x1p60))
        return ctx_fail(ctx, HEXO_ERR_INVALID, "S0 must be in [2^-60, 2^60)");
    std::lock_guard<std::mutex> lk(ctx->run_mu);
    cudaSetDevice(ctx->device);
    DevBuf dp, dout;
    cudaError_t e = dp.alloc(n * sizeof(double));
    if (e == cudaSuccess) e = dout.alloc(n * kLimbs * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemcpyAsync(dp.p, pay, n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess)
        e = launch_dbg_limbs((const double *)dp.p, n, precision == HEXO_FP32, pay_exponent(S0), (uint32_t *)dout.p,
                             ctx->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(out, dout.p, n * kLimbs * sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    return e == cudaSuccess ? HEXO_OK : cuda_fail(ctx, e, "debug payoff limbs");
}

hexo_status hexo_debug_pipe_peaks(hexo_ctx *ctx, double *out5) {
    if (!ctx || !out5) return HEXO_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->run_mu);
    cudaSetDevice(ctx->device);
    cudaError_t e = measure_pipe_peaks((int)ctx->sm_count, ctx->stream, out5);
    return e == cudaSuccess ? HEXO_OK : cuda_fail(ctx, e, "pipe peaks");
}

hexo_status hexo_debug_path_finals(hexo_ctx *ctx, const hexo_params *p, double S0, const hexo_option *opts,
                                   uint32_t n_opts, const hexo_mc_cfg *cfg, uint64_t path_lo, uint64_t path_hi,
                                   double *asian_out, double *euro_out, uint32_t *n_mats_out) {
    if (!ctx || !p || !cfg || !asian_out || !euro_out) return HEXO_ERR_INVALID;
    if (path_hi <= path_lo) return ctx_fail(ctx, HEXO_ERR_INVALID, "empty path range");
    std::lock_guard<std::mutex> lk(ctx->run_mu);
    cudaSetDevice(ctx->device);
    hexo_request r;
    std::memset(&r, 0, sizeof(r));
    r.params = *p;
    r.S0 = S0;
    r.opts = opts;
    r.n_opts = n_opts;
    r.seed = cfg->seed;
    r.stream = cfg->stream;
    BatchPlan bp;
    std::vector<SetPlan> plans;
    hexo_status s = plan_requests(ctx, &r, 1, *cfg, path_lo, path_hi, bp, plans);
    if (s != HEXO_OK) return s;
    const uint32_t m = (uint32_t)plans[0].mats.size();
    if (n_mats_out) *n_mats_out = m;
    const uint64_t n = path_hi - path_lo;
    DeviceBatch db;
    if ((s = batch_upload(ctx, std::move(bp), cfg->precision == HEXO_FP32, db)) != HEXO_OK) return s;
    DevBuf da, de;
    const size_t bytes = (size_t)n * m * sizeof(double);
    cudaError_t e = da.alloc(bytes);
    if (e == cudaSuccess) e = de.alloc(bytes);
    // NaN everywhere a path does not reach
    if (e == cudaSuccess) e = cudaMemsetAsync(da.p, 0xff, bytes, ctx->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(de.p, 0xff, bytes, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "debug finals alloc");
    db.args.dbg_asian = (double *)da.p;
    db.args.dbg_euro = (double *)de.p;
    db.args.dbg_lo = path_lo;
    db.args.dbg_mats = m;
    e = batch_enqueue(db, ctx->stream, false);
    if (e == cudaSuccess) e = cudaMemcpyAsync(asian_out, da.p, bytes, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(euro_out, de.p, bytes, cudaMemcpyDeviceToHost, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "debug finals launch");
    return batch_wait(db);
}

} // extern "C"
