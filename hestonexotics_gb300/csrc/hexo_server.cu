// Serving loop: continuous batching of pricing requests.
//
// Requests are submitted from any thread into a FIFO.  One scheduler thread
//  * admits queued requests, in arrival order, while the device memory their
//    launch needs fits under the cap together with the launches in flight;
//  * folds every admitted request (up to max_batch_requests) into the next
//    persistent launch, on one of max_inflight streams, so requests that
//    arrive while others run join the next launch and the launches overlap
//    on the device;
//  * retires finished launches, scatters prices to the requests' own output
//    arrays and records each request's submit-to-completion latency.
// A request's result does not depend on what it was batched with: path k of
// a request always draws from RNG(16, seed + k) and sums are exact integers,
// so a request alone and in any mix gives the same bits.
#include <cuda_runtime.h>
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "hexo_mc.h"
#include "hexo_launch.h"
#include "hexo_plan.h"
#include "hexo_runtime.h"

using namespace hexo;

namespace {

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct SrvReq {
    uint64_t ticket = 0;
    hexo_request req{};
    std::vector<hexo_option> opts;
    double t_submit = 0.0;
    hexo_status status = HEXO_OK;
    bool done = false;
    SetPlan plan;
    bool planned = false;
    uint64_t bytes = 0;      // device memory estimate of this request within a launch
    uint64_t nominal = 0;
};

// Device and pinned host memory of one stream slot, reused by its launches.
struct Arena {
    void *d = nullptr, *h = nullptr;
    size_t dcap = 0, hcap = 0;
};

struct Inflight {
    std::unique_ptr<DeviceBatch> db;
    std::vector<SrvReq *> reqs;
    cudaEvent_t done = nullptr;
    uint64_t bytes = 0;
    int stream_index = -1;
};

} // namespace

struct hexo_server {
    hexo_ctx *ctx = nullptr;
    hexo_server_opts opts{};
    uint64_t cap = 0;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<SrvReq *> pending;
    std::unordered_map<uint64_t, std::unique_ptr<SrvReq>> all;
    uint64_t next_ticket = 1;
    bool stop = false;
    std::thread th;
    std::vector<cudaStream_t> streams;
    std::vector<bool> stream_busy;
    std::vector<Arena> arenas;
    uint32_t grid_max = 1, tile_paths = 256;
    std::vector<Inflight> inflight;
    hexo_server_stats st{};
    std::vector<double> lat_ms;
    double busy_since = -1.0;
};

namespace {

// Device bytes one request adds to a launch: its descriptors and tiles plus
// its outputs and the CTA-private copies of its sums.
uint64_t request_bytes(hexo_server *s, const SetPlan &sp) {
    const uint64_t n_out = sp.opts.size();
    const uint64_t P = s->tile_paths;
    const uint64_t tiles = (sp.path_hi - sp.path_lo + P - 1) / P;
    return sizeof(SetDesc) + sp.segs.size() * sizeof(SegDesc) + sp.mats.size() * sizeof(MatDesc) +
           n_out * sizeof(OptDesc) + tiles * sizeof(TileDesc) +
           n_out * (kLimbs * 8ull * (s->grid_max + 1) + 32ull) + 4096;
}

void finish(hexo_server *s, SrvReq *r, hexo_status status, double t) {
    r->status = status;
    r->done = true;
    if (status == HEXO_OK) {
        ++s->st.completed;
        s->st.nominal_path_steps += r->nominal;
        s->lat_ms.push_back((t - r->t_submit) * 1e3);
    } else {
        ++s->st.failed;
    }
}

void retire(hexo_server *s, std::unique_lock<std::mutex> &lk) {
    for (size_t i = 0; i < s->inflight.size();) {
        Inflight &f = s->inflight[i];
        const cudaError_t q = cudaEventQuery(f.done);
        if (q == cudaErrorNotReady) { ++i; continue; }
        hexo_status status = q == cudaSuccess ? batch_wait(*f.db) : HEXO_ERR_CUDA;
        const double t = now_s();
        if (status == HEXO_OK) {
            uint32_t base = 0;
            for (SrvReq *r : f.reqs) {
                for (uint32_t k = 0; k < r->req.n_opts; ++k) {
                    if (r->req.price_out) r->req.price_out[k] = f.db->h_price[base + k];
                    if (r->req.stderr_out) r->req.stderr_out[k] = f.db->h_se[base + k];
                }
                base += r->req.n_opts;
            }
        }
        for (SrvReq *r : f.reqs) finish(s, r, status, t);
        // keep the launch's memory for the next launch on this stream
        Arena &ar = s->arenas[f.stream_index];
        if (f.db->own_d && f.db->dmem) {
            if (ar.d) cudaFree(ar.d);
            ar.d = f.db->dmem;
            ar.dcap = f.db->dcap;
        }
        if (f.db->own_h && f.db->hmem) {
            if (ar.h) cudaFreeHost(ar.h);
            ar.h = f.db->hmem;
            ar.hcap = f.db->hcap;
        }
        f.db->own_d = f.db->own_h = false;
        s->st.mem_in_use -= f.bytes;
        s->stream_busy[f.stream_index] = false;
        cudaEventDestroy(f.done);
        s->inflight.erase(s->inflight.begin() + (long)i);
        s->cv_done.notify_all();
    }
    s->st.inflight_now = s->inflight.size();
    if (s->inflight.empty() && s->busy_since >= 0.0) {
        s->st.busy_seconds += now_s() - s->busy_since;
        s->busy_since = -1.0;
    }
    (void)lk;
}

// Takes admitted requests off the queue (FIFO) and launches them together.
bool launch_next(hexo_server *s, std::unique_lock<std::mutex> &lk) {
    if (s->pending.empty() || s->inflight.size() >= s->opts.max_inflight) return false;
    int si = -1;
    for (size_t k = 0; k < s->streams.size(); ++k)
        if (!s->stream_busy[k]) { si = (int)k; break; }
    if (si < 0) return false;
    std::vector<SrvReq *> batch;
    uint64_t bytes = 0;
    while (!s->pending.empty() && batch.size() < s->opts.max_batch_requests) {
        SrvReq *r = s->pending.front();
        if (!r->planned) {
            std::string err;
            r->status = plan_set(r->req.params, r->req.S0, r->req.opts, r->req.n_opts, s->opts.cfg, r->req.seed,
                                 r->req.stream, 0, ~0ull, r->plan, err);
            r->planned = true;
            if (r->status != HEXO_OK) {
                s->pending.pop_front();
                finish(s, r, r->status, now_s());
                s->cv_done.notify_all();
                continue;
            }
            r->bytes = request_bytes(s, r->plan);
            uint64_t exe = 0;
            plan_work(r->plan, r->nominal, exe, s->tile_paths);
        }
        if (r->bytes > s->cap) {                               // can never fit
            s->pending.pop_front();
            finish(s, r, HEXO_ERR_ADMISSION, now_s());
            s->cv_done.notify_all();
            continue;
        }
        if (s->st.mem_in_use + bytes + r->bytes > s->cap) break;   // wait for memory to free up
        bytes += r->bytes;
        batch.push_back(r);
        s->pending.pop_front();
    }
    if (batch.empty()) return false;
    s->st.admitted += batch.size();
    s->st.queued_now = s->pending.size();
    s->st.mem_in_use += bytes;
    s->st.mem_peak = std::max(s->st.mem_peak, s->st.mem_in_use);
    s->stream_busy[si] = true;

    lk.unlock();   // planning the launch and uploading do not need the queue
    NvtxRange nvtx("hexo_server launch");
    BatchPlan bp;
    std::vector<SetPlan> plans;
    plans.reserve(batch.size());
    uint32_t base = 0, cv_base = 0;
    for (SrvReq *r : batch) cv_base += r->req.n_opts;   // control-variate slots after all outputs
    for (SrvReq *r : batch) {
        plans.push_back(r->plan);
        batch_add(bp, plans.back(), base, cv_base);
        base += r->req.n_opts;
        cv_base += 2u * r->plan.n_cv;
    }
    bp.shape = ctx_shape(s->ctx, s->opts.cfg);
    batch_tiles(bp, plans);
    Inflight f;
    f.db.reset(new DeviceBatch());
    f.db->stream = s->streams[si];
    {
        const Arena &ar = s->arenas[si];
        f.db->dmem = ar.d;
        f.db->dcap = ar.dcap;
        f.db->hmem = ar.h;
        f.db->hcap = ar.hcap;
        f.db->own_d = f.db->own_h = false;
    }
    f.reqs = batch;
    f.bytes = bytes;
    f.stream_index = si;
    hexo_status st = batch_upload(s->ctx, std::move(bp), s->opts.cfg.precision == HEXO_FP32, *f.db);
    cudaError_t e = cudaSuccess;
    if (st == HEXO_OK) e = batch_enqueue(*f.db, f.db->stream, false);
    if (st == HEXO_OK && e == cudaSuccess) e = cudaEventCreateWithFlags(&f.done, cudaEventDisableTiming);
    if (st == HEXO_OK && e == cudaSuccess) e = cudaEventRecord(f.done, f.db->stream);
    lk.lock();
    if (st != HEXO_OK || e != cudaSuccess) {
        const hexo_status fail = st != HEXO_OK ? st : HEXO_ERR_CUDA;
        for (SrvReq *r : batch) finish(s, r, fail, now_s());
        Arena &ar = s->arenas[si];
        if (f.db->own_d && f.db->dmem) { if (ar.d) cudaFree(ar.d); ar.d = f.db->dmem; ar.dcap = f.db->dcap; }
        if (f.db->own_h && f.db->hmem) { if (ar.h) cudaFreeHost(ar.h); ar.h = f.db->hmem; ar.hcap = f.db->hcap; }
        f.db->own_d = f.db->own_h = false;
        s->st.mem_in_use -= bytes;
        s->stream_busy[si] = false;
        if (f.done) cudaEventDestroy(f.done);
        s->cv_done.notify_all();
        return true;
    }
    ++s->st.batches;
    if (s->busy_since < 0.0) s->busy_since = now_s();
    s->inflight.push_back(std::move(f));
    s->st.inflight_now = s->inflight.size();
    return true;
}

void loop(hexo_server *s) {
    cudaSetDevice(s->ctx->device);
    std::unique_lock<std::mutex> lk(s->mu);
    for (;;) {
        retire(s, lk);
        bool launched = false;
        while (launch_next(s, lk)) launched = true;
        if (s->stop && s->pending.empty() && s->inflight.empty()) break;
        if (launched) continue;
        if (!s->inflight.empty()) s->cv_work.wait_for(lk, std::chrono::microseconds(50));
        else s->cv_work.wait_for(lk, std::chrono::milliseconds(20));
    }
}

} // namespace

extern "C" {

hexo_status hexo_server_create(hexo_ctx *ctx, const hexo_server_opts *opts, hexo_server **out) {
    if (!ctx || !opts || !out) return HEXO_ERR_INVALID;
    *out = nullptr;
    std::unique_ptr<hexo_server> s(new (std::nothrow) hexo_server());
    if (!s) return HEXO_ERR_NOMEM;
    s->ctx = ctx;
    s->opts = *opts;
    if (s->opts.max_batch_requests == 0) s->opts.max_batch_requests = 64;
    if (s->opts.max_inflight == 0) s->opts.max_inflight = 2;
    if (s->opts.max_inflight > 16) s->opts.max_inflight = 16;
    s->cap = opts->mem_cap_bytes ? opts->mem_cap_bytes : ctx->mem_cap;
    cudaSetDevice(ctx->device);
    {
        size_t smem = 0;
        uint32_t cps = 0;
        const LaunchShape sh = ctx_shape(ctx, s->opts.cfg);
        const hexo_status st = shape_check(ctx, s->opts.cfg.precision == HEXO_FP32, sh, smem, cps);
        if (st != HEXO_OK) return st;
        s->grid_max = ctx->sm_count * cps;
        s->tile_paths = sh.paths_per_tile();
    }
    for (uint32_t k = 0; k < s->opts.max_inflight; ++k) {
        cudaStream_t st;
        if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) {
            for (cudaStream_t x : s->streams) cudaStreamDestroy(x);
            return HEXO_ERR_CUDA;
        }
        s->streams.push_back(st);
        s->stream_busy.push_back(false);
        s->arenas.push_back(Arena{});
    }
    hexo_server *raw = s.get();
    s->th = std::thread(loop, raw);
    *out = s.release();
    return HEXO_OK;
}

hexo_status hexo_server_submit(hexo_server *s, const hexo_request *req, uint64_t *ticket) {
    if (!s || !req || !ticket || !req->opts || req->n_opts == 0 || !req->price_out) return HEXO_ERR_INVALID;
    std::unique_ptr<SrvReq> r(new (std::nothrow) SrvReq());
    if (!r) return HEXO_ERR_NOMEM;
    r->req = *req;
    r->opts.assign(req->opts, req->opts + req->n_opts);
    r->req.opts = r->opts.data();
    r->t_submit = now_s();
    std::lock_guard<std::mutex> g(s->mu);
    if (s->stop) return HEXO_ERR_SHUTDOWN;
    r->ticket = s->next_ticket++;
    *ticket = r->ticket;
    s->pending.push_back(r.get());
    s->all[r->ticket] = std::move(r);
    ++s->st.submitted;
    s->st.queued_now = s->pending.size();
    s->st.queued_max = std::max<uint64_t>(s->st.queued_max, s->pending.size());
    s->cv_work.notify_one();
    return HEXO_OK;
}

hexo_status hexo_server_poll(hexo_server *s, uint64_t ticket, int *done) {
    if (!s || !done) return HEXO_ERR_INVALID;
    std::lock_guard<std::mutex> g(s->mu);
    auto it = s->all.find(ticket);
    if (it == s->all.end()) return HEXO_ERR_NOT_FOUND;
    *done = it->second->done ? 1 : 0;
    if (!it->second->done) return HEXO_OK;
    const hexo_status st = it->second->status;
    s->all.erase(it);   // reported once, then forgotten
    return st;
}

hexo_status hexo_server_wait(hexo_server *s, uint64_t ticket, uint32_t timeout_ms) {
    if (!s) return HEXO_ERR_INVALID;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->all.find(ticket);
    if (it == s->all.end()) return HEXO_ERR_NOT_FOUND;
    SrvReq *r = it->second.get();
    const bool ok = s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), [&] { return r->done; });
    if (!ok) return HEXO_ERR_TIMEOUT;
    const hexo_status st = r->status;
    s->all.erase(it);   // reported once, then forgotten
    return st;
}

hexo_status hexo_server_stats_get(hexo_server *s, hexo_server_stats *out) {
    if (!s || !out) return HEXO_ERR_INVALID;
    std::lock_guard<std::mutex> g(s->mu);
    *out = s->st;
    out->queued_now = s->pending.size();
    if (s->busy_since >= 0.0) out->busy_seconds += now_s() - s->busy_since;
    if (!s->lat_ms.empty()) {
        std::vector<double> v = s->lat_ms;
        std::sort(v.begin(), v.end());
        auto pct = [&](double q) {
            const double x = q * (double)(v.size() - 1);
            const size_t i = (size_t)x;
            const double f = x - (double)i;
            return i + 1 < v.size() ? v[i] * (1.0 - f) + v[i + 1] * f : v[i];
        };
        out->p50_ms = pct(0.50);
        out->p99_ms = pct(0.99);
        double sum = 0.0;
        for (double x : v) sum += x;
        out->mean_ms = sum / (double)v.size();
    }
    return HEXO_OK;
}

hexo_status hexo_server_destroy(hexo_server *s) {
    if (!s) return HEXO_ERR_INVALID;
    {
        std::lock_guard<std::mutex> g(s->mu);
        s->stop = true;
        s->cv_work.notify_all();
    }
    if (s->th.joinable()) s->th.join();
    cudaSetDevice(s->ctx->device);
    for (cudaStream_t x : s->streams) cudaStreamDestroy(x);
    for (Arena &ar : s->arenas) {
        if (ar.d) cudaFree(ar.d);
        if (ar.h) cudaFreeHost(ar.h);
    }
    delete s;
    return HEXO_OK;
}

} // extern "C"
