// Runtime objects behind the opaque handles of hexo_mc.h.
#pragma once
#include <cuda_runtime.h>
#include <mutex>
#include <string>
#include <vector>
#include "hexo_mc.h"
#include "hexo_plan.h"

// NVTX ranges (header-only; a profiler that injects NVTX shows them, and
// without one they cost a null check): planning, upload, the run and result
// collection of each host call, the server's admission and launches.
#include <nvtx3/nvToolsExt.h>

namespace hexo {

struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};

// A device allocation freed on scope exit.
struct DevBuf {
    void *p = nullptr;
    cudaError_t alloc(size_t bytes) { return cudaMalloc(&p, bytes ? bytes : 1); }
    ~DevBuf() { if (p) cudaFree(p); }
};

// Planned batch resident on the device, with pinned host mirrors of its outputs.
struct DeviceBatch {
    hexo_ctx *ctx = nullptr;
    cudaStream_t stream = nullptr;   // the context's stream unless set before upload
    BatchPlan plan;
    bool f32 = false;
    size_t smem = 0;
    uint32_t ctas_per_sm = 0, grid = 0, n_slots = 1;
    unsigned long long *d_acc_sum = nullptr;   // totals of the private sum copies
    void *dmem = nullptr;
    size_t bytes = 0;
    void *hmem = nullptr;
    // Memory handed in before upload is reused when large enough (own_* false:
    // the batch does not free it); otherwise the upload allocates its own.
    size_t dcap = 0, hcap = 0;
    bool own_d = true, own_h = true;
    KernelArgs args{};
    uint64_t *d_paths = nullptr;
    double *d_disc = nullptr, *d_price = nullptr, *d_se = nullptr;
    int32_t *d_pexp = nullptr;       // per output slot: E, payoffs summed in units of 2^E
    unsigned long long *carry = nullptr;   // running sums of split requests (the server's pool), or null
    uint64_t *d_carry_row = nullptr;       // per output slot: (row << 1) | last block, ~0 = not carried
    double *h_price = nullptr, *h_se = nullptr;
    unsigned long long *h_acc = nullptr;
    double *d_cv_eg = nullptr;         // control variate (in dmem): E[(G - K)^+] per output slot (NaN elsewhere)
    uint32_t *d_cv_partner = nullptr;  // control variate (in dmem): the slot of the geometric sums (~0 elsewhere)
    uint32_t *h_ctl = nullptr;   // control block of the last run (kCtlBytes): queue head, error flags, quad steps
    cudaGraphExec_t graph_exec = nullptr;
    cudaEvent_t ev_k0 = nullptr, ev_k1 = nullptr;   // around the path kernel
    uint64_t h2d_bytes = 0;
    DeviceBatch() = default;
    DeviceBatch(const DeviceBatch &) = delete;
    DeviceBatch &operator=(const DeviceBatch &) = delete;
    ~DeviceBatch();
};

} // namespace hexo

struct hexo_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    uint32_t sm_count = 0;
    size_t smem_optin = 0;
    uint64_t mem_cap = 0;
    std::string tune_cache;
    hexo::LaunchShape shape_f64, shape_f32;   // tuned or default launch shapes
    std::mutex run_mu;                        // one launch sequence at a time on the stream
    std::mutex err_mu;
    std::string last_error;
    // device and pinned host memory of the last one-shot call, reused by the
    // next (guarded by run_mu; freed by hexo_ctx_destroy): no allocation, and
    // so no device synchronisation, per call once the largest batch was seen
    void *arena_d = nullptr, *arena_h = nullptr;
    size_t arena_dcap = 0, arena_hcap = 0;
};

struct hexo_batch {
    hexo::DeviceBatch db;
    std::vector<hexo_request> reqs;
    bool partial = false;   // a shard of a batch: limbs only, prices after the merge
};

namespace hexo {
// One-shot memory larger than this is freed at the end of its call instead of
// being kept for the next one (hexo_ctx_trim frees what is kept).
constexpr size_t kArenaKeepBytes = 256ull << 20;

// Lends the context's arena to a one-shot batch and keeps whatever larger
// memory the batch allocated instead, up to kArenaKeepBytes (declare after
// the DeviceBatch; the DeviceBatch frees what is not kept).
struct ArenaLoan {
    hexo_ctx *ctx;
    DeviceBatch &db;
    ArenaLoan(hexo_ctx *c, DeviceBatch &d) : ctx(c), db(d) {
        db.dmem = ctx->arena_d; db.dcap = ctx->arena_dcap;
        db.hmem = ctx->arena_h; db.hcap = ctx->arena_hcap;
        db.own_d = db.own_h = false;
    }
    ~ArenaLoan() {
        if (db.own_d && db.dmem && db.dcap <= kArenaKeepBytes) {
            if (ctx->arena_d) cudaFree(ctx->arena_d);
            ctx->arena_d = db.dmem;
            ctx->arena_dcap = db.dcap;
            db.own_d = false;
        }
        if (db.own_h && db.hmem && db.hcap <= kArenaKeepBytes) {
            if (ctx->arena_h) cudaFreeHost(ctx->arena_h);
            ctx->arena_h = db.hmem;
            ctx->arena_hcap = db.hcap;
            db.own_h = false;
        }
    }
    ArenaLoan(const ArenaLoan &) = delete;
    ArenaLoan &operator=(const ArenaLoan &) = delete;
};

// The context's device arena as scratch of at least `bytes` (grown when
// smaller); valid until the next call on the context (hold run_mu).
inline cudaError_t ctx_scratch(hexo_ctx *ctx, size_t bytes, void **p) {
    if (ctx->arena_d == nullptr || ctx->arena_dcap < bytes) {
        if (ctx->arena_d) cudaFree(ctx->arena_d);
        ctx->arena_d = nullptr;
        ctx->arena_dcap = 0;
        const cudaError_t e = cudaMalloc(&ctx->arena_d, bytes ? bytes : 1);
        if (e != cudaSuccess) { ctx->arena_d = nullptr; return e; }
        ctx->arena_dcap = bytes;
    }
    *p = ctx->arena_d;
    return cudaSuccess;
}

hexo_status ctx_fail(hexo_ctx *ctx, hexo_status s, const std::string &msg);
hexo_status cuda_fail(hexo_ctx *ctx, cudaError_t e, const char *what);
LaunchShape ctx_shape(hexo_ctx *ctx, const hexo_mc_cfg &cfg);
// Narrows the default launch shape of a batch too small to fill the GPU's CTA slots.
void fit_small_batch(hexo_ctx *ctx, const hexo_mc_cfg &cfg, LaunchShape &sh, const std::vector<SetPlan> &plans);
hexo_status shape_check(hexo_ctx *ctx, bool f32, const LaunchShape &sh, size_t &smem, uint32_t &ctas_per_sm);
hexo_status batch_upload(hexo_ctx *ctx, BatchPlan &&plan, bool f32, DeviceBatch &db);
cudaError_t batch_enqueue(DeviceBatch &db, cudaStream_t st, bool copy_acc);
hexo_status batch_wait(DeviceBatch &db);
hexo_status plan_requests(hexo_ctx *ctx, const hexo_request *reqs, uint32_t n_reqs, const hexo_mc_cfg &cfg,
                          uint64_t path_lo, uint64_t path_hi, BatchPlan &bp, std::vector<SetPlan> &plans,
                          uint32_t shard = 0, uint32_t n_shards = 1);
void scatter_outputs(const DeviceBatch &db, const hexo_request *reqs, uint32_t n_reqs);
// Plans, uploads and captures a batch (shard `shard` of n_shards of every
// request's paths when n_shards > 1) as a graph.
hexo_status batch_prepare(hexo_ctx *ctx, const hexo_request *reqs, uint32_t n_reqs, const hexo_mc_cfg *cfg,
                          uint32_t shard, uint32_t n_shards, hexo_batch **out);
// Autotune cache: reads ctx->tune_cache (if any) into the context's shapes.
void tune_load(hexo_ctx *ctx);
} // namespace hexo
