// Launch-shape autotuner: sweeps threads per CTA x paths per thread x step
// unroll on a caller-supplied batch, timing one graph launch of each shape
// with CUDA events, and keeps the fastest per precision.  Results depend
// only on the launch shape's speed, never on its numbers: every shape gives
// bit-identical prices (per-path streams, exact integer sums).
#include <cuda_runtime.h>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>

#include "hexo_mc.h"
#include "hexo_launch.h"
#include "hexo_runtime.h"

namespace hexo {

void tune_load(hexo_ctx *ctx) {
    // defaults: the sweep's fastest shape for both forms on the uneven 64-set batch (256 threads, one
    // path each, no unrolling; two CTAs per SM, which registers and shared memory both allow)
    ctx->shape_f64 = LaunchShape{256, 1, 1};
    ctx->shape_f32 = LaunchShape{256, 1, 1};
    if (ctx->tune_cache.empty()) return;
    std::ifstream in(ctx->tune_cache);
    std::string prec;
    uint32_t b, p, u;
    while (in >> prec >> b >> p >> u) {
        const LaunchShape sh{b, p, u};
        if (paths_kernel_ptr(false, p, u) == nullptr || b == 0 || b % 32 || b > 512) continue;
        if (prec == "fp64") ctx->shape_f64 = sh;
        else if (prec == "fp32") ctx->shape_f32 = sh;
    }
}

static void tune_save(hexo_ctx *ctx) {
    if (ctx->tune_cache.empty()) return;
    std::ofstream out(ctx->tune_cache, std::ios::trunc);
    out << "fp64 " << ctx->shape_f64.block << ' ' << ctx->shape_f64.ppt << ' ' << ctx->shape_f64.unroll << '\n';
    out << "fp32 " << ctx->shape_f32.block << ' ' << ctx->shape_f32.ppt << ' ' << ctx->shape_f32.unroll << '\n';
}

} // namespace hexo

using namespace hexo;

extern "C" hexo_status hexo_autotune(hexo_ctx *ctx, const hexo_request *reqs, uint32_t n_reqs,
                                     const hexo_mc_cfg *cfg, hexo_tune_result *result,
                                     hexo_tune_entry *entries, uint32_t max_entries) {
    if (!ctx || !cfg || !reqs || n_reqs == 0) return HEXO_ERR_INVALID;
    const bool f32 = cfg->precision == HEXO_FP32;
    const uint32_t blocks[5] = {128, 192, 256, 384, 512}, ppts[3] = {1, 2, 4}, unrolls[3] = {1, 2, 4};
    std::lock_guard<std::mutex> lk(ctx->run_mu);
    cudaSetDevice(ctx->device);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = -1.0f;
    LaunchShape best_sh;
    uint32_t tried = 0;
    hexo_status status = HEXO_OK;
    for (uint32_t b : blocks)
        for (uint32_t p : ppts)
            for (uint32_t u : unrolls) {
                hexo_mc_cfg c = *cfg;
                c.block = b;
                c.paths_per_thread = p;
                c.unroll = u;
                size_t smem;
                uint32_t ctas;
                const LaunchShape sh{b, p, u};
                if (paths_smem_bytes(b, p) > ctx->smem_optin) continue;
                if (shape_check(ctx, f32, sh, smem, ctas) != HEXO_OK) continue;
                BatchPlan bp;
                std::vector<SetPlan> plans;
                hexo_status s = plan_requests(ctx, reqs, n_reqs, c, 0, ~0ull, bp, plans);
                if (s != HEXO_OK) { status = s; goto done; }
                {
                    DeviceBatch db;
                    if ((s = batch_upload(ctx, std::move(bp), f32, db)) != HEXO_OK) continue;
                    // warm-up, then one timed run
                    if (batch_enqueue(db, ctx->stream, false) != cudaSuccess || batch_wait(db) != HEXO_OK) continue;
                    cudaEventRecord(e0, ctx->stream);
                    cudaError_t ce = batch_enqueue(db, ctx->stream, false);
                    cudaEventRecord(e1, ctx->stream);
                    if (ce != cudaSuccess || batch_wait(db) != HEXO_OK) continue;
                    float ms = 0.0f;
                    cudaEventElapsedTime(&ms, e0, e1);
                    if (entries && tried < max_entries) {
                        entries[tried].block = b;
                        entries[tried].paths_per_thread = p;
                        entries[tried].unroll = u;
                        entries[tried].ms = ms;
                    }
                    ++tried;
                    if (best < 0.0f || ms < best) { best = ms; best_sh = sh; }
                }
            }
done:
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (status != HEXO_OK) return status;
    if (best < 0.0f) return ctx_fail(ctx, HEXO_ERR_UNSUPPORTED, "no launch shape could run this batch");
    if (f32) ctx->shape_f32 = best_sh;
    else ctx->shape_f64 = best_sh;
    tune_save(ctx);
    if (result) {
        result->block = best_sh.block;
        result->paths_per_thread = best_sh.ppt;
        result->unroll = best_sh.unroll;
        result->best_ms = best;
        result->n_tried = tried;
    }
    return HEXO_OK;
}
