// Serving loop: continuous batching of pricing requests, split into path
// blocks that continue across persistent launches.
//
// Requests are submitted from any thread into a queue.  One scheduler thread
//  * admits queued requests while their running sums fit the server's device
//    pool; a request that does not fit yet lets later ones that fit go ahead
//    (first come, first served otherwise), until it has waited
//    kStarveSeconds, after which nothing is admitted past it;
//  * builds each persistent launch from the admitted requests that have no
//    block in flight, those that have had the fewest blocks first, one block
//    of consecutive paths per request, sized so that a launch holds about
//    launch_path_steps of work; the launch runs on one of max_inflight
//    streams while the next is planned and uploaded, as long as the device
//    memory of the launches in flight stays under the cap;
//  * after each launch, the finaliser adds every block's exact limb sums into
//    its request's running sums, which stay in the device pool between
//    launches; the launch that carries a request's last block finalises it
//    from those sums, and the scheduler scatters the prices to the
//    request's own output arrays and records its submit-to-completion
//    latency.
// Path k of a request always draws from the stream seeded
// {seed + k, stream, 0, 0}, and the sums are exact integers, so what the
// request carries from one launch to the next is its next path index and its
// running sums: a request alone, in any mix, in one block or in many gives
// the same bits.  Requests with the geometric control variate run as one
// block (their estimator needs all three sums of a path set at once).
#include <cuda_runtime.h>
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
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

constexpr double kStarveSeconds = 0.05;              // longest a request lets later ones pass it
constexpr uint64_t kDefaultLaunchPathSteps = 1ull << 30;
constexpr uint64_t kRowBytes = kLimbs * sizeof(unsigned long long);
constexpr uint64_t kMaxPoolBytes = 64ull << 20;

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
    SetPlan plan;             // the whole request, paths [0, n_max)
    bool planned = false;
    bool admitted = false;
    bool in_flight = false;
    bool whole = false;       // one block (control variate)
    uint64_t seq = 0;         // admission order
    uint64_t n_max = 0;       // paths the request simulates
    uint64_t next_path = 0;   // first path of its next block
    uint64_t deep_steps = 1;  // steps its longest path executes
    uint64_t blocks = 0;      // blocks launched so far
    uint64_t row = 0, n_rows = 0;   // its running sums: pool rows [row, row + n_rows)
    uint64_t fixed_bytes = 0; // device bytes a launch needs for it, whatever the block size
    uint64_t nominal = 0;
};

// Device and pinned host memory of one stream slot, reused by its launches.
struct Arena {
    void *d = nullptr, *h = nullptr;
    size_t dcap = 0, hcap = 0;
};

// First-fit allocator of 48-byte rows in the device pool of running sums.
struct RowPool {
    unsigned long long *base = nullptr;
    uint64_t rows = 0;
    std::map<uint64_t, uint64_t> free_;   // first row -> rows
    void reset(uint64_t n) { rows = n; free_.clear(); if (n) free_[0] = n; }
    bool alloc(uint64_t n, uint64_t &at) {
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < n) continue;
            at = it->first;
            const uint64_t rest = it->second - n;
            free_.erase(it);
            if (rest) free_[at + n] = rest;
            return true;
        }
        return false;
    }
    void release(uint64_t at, uint64_t n) {
        if (n == 0) return;
        auto next = free_.lower_bound(at);
        if (next != free_.end() && at + n == next->first) { n += next->second; next = free_.erase(next); }
        if (next != free_.begin()) {
            auto prev = std::prev(next);
            if (prev->first + prev->second == at) { prev->second += n; return; }
        }
        free_[at] = n;
    }
};

struct Block {
    SrvReq *r;
    uint64_t lo, hi;
    bool last;
};

struct Inflight {
    std::unique_ptr<DeviceBatch> db;
    std::vector<Block> blocks;
    cudaEvent_t done = nullptr;
    uint64_t bytes = 0;
    int stream_index = -1;
};

} // namespace

struct hexo_server {
    hexo_ctx *ctx = nullptr;
    hexo_server_opts opts{};
    uint64_t cap = 0;
    uint64_t launch_budget = kDefaultLaunchPathSteps;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<SrvReq *> pending;   // submitted, not yet admitted
    std::vector<SrvReq *> active;   // admitted, not finished
    std::unordered_map<uint64_t, std::unique_ptr<SrvReq>> all;
    uint64_t next_ticket = 1, next_seq = 0;
    bool stop = false;
    std::thread th;
    std::vector<cudaStream_t> streams;
    std::vector<bool> stream_busy;
    std::vector<Arena> arenas;
    RowPool pool;
    uint64_t pool_bytes = 0;
    uint32_t tile_paths = 256;
    std::vector<Inflight> inflight;
    hexo_server_stats st{};
    std::vector<double> lat_ms;
    double busy_since = -1.0;
};

namespace {

// Device bytes one block of a request adds to a launch: the request's
// descriptors, its outputs with their private sum copies, and the block's tiles.
uint64_t block_bytes(hexo_server *s, const SrvReq &r, uint64_t paths) {
    return r.fixed_bytes + (paths + s->tile_paths - 1) / s->tile_paths * sizeof(TileDesc);
}

void finish(hexo_server *s, SrvReq *r, hexo_status status, double t) {
    r->status = status;
    r->done = true;
    if (r->n_rows) {
        s->pool.release(r->row, r->n_rows);
        r->n_rows = 0;
    }
    if (status == HEXO_OK) {
        ++s->st.completed;
        s->st.nominal_path_steps += r->nominal;
        s->lat_ms.push_back((t - r->t_submit) * 1e3);
    } else {
        ++s->st.failed;
    }
}

void drop_active(hexo_server *s) {
    s->active.erase(std::remove_if(s->active.begin(), s->active.end(), [](SrvReq *r) { return r->done; }),
                    s->active.end());
}

void keep_arena(hexo_server *s, Inflight &f) {
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
}

void retire(hexo_server *s) {
    for (size_t i = 0; i < s->inflight.size();) {
        Inflight &f = s->inflight[i];
        const cudaError_t q = cudaEventQuery(f.done);
        if (q == cudaErrorNotReady) { ++i; continue; }
        const hexo_status status = q == cudaSuccess ? batch_wait(*f.db) : HEXO_ERR_CUDA;
        const double t = now_s();
        uint32_t base = 0;
        for (const Block &b : f.blocks) {
            SrvReq *r = b.r;
            r->in_flight = false;
            if (status != HEXO_OK) {
                if (!r->done) finish(s, r, status, t);
            } else if (b.last) {
                for (uint32_t k = 0; k < r->req.n_opts; ++k) {
                    if (r->req.price_out) r->req.price_out[k] = f.db->h_price[base + k];
                    if (r->req.stderr_out) r->req.stderr_out[k] = f.db->h_se[base + k];
                }
                finish(s, r, HEXO_OK, t);
            }
            base += r->req.n_opts;
        }
        drop_active(s);
        keep_arena(s, f);   // the launch's memory serves the next launch on this stream
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
}

// Plans queued requests and admits those whose running sums fit the pool:
// first come, first served, except that a request that does not fit lets
// later ones pass until it has waited kStarveSeconds.
void admit(hexo_server *s) {
    const double t = now_s();
    for (auto it = s->pending.begin(); it != s->pending.end();) {
        SrvReq *r = *it;
        if (!r->planned) {
            std::string err;
            r->status = plan_set(r->req.params, r->req.S0, r->req.opts, r->req.n_opts, s->opts.cfg, r->req.seed,
                                 r->req.stream, 0, ~0ull, r->plan, err);
            r->planned = true;
            if (r->status == HEXO_OK) {
                uint64_t exe = 0;
                plan_work(r->plan, r->nominal, exe, s->tile_paths);
                const SetPlan &sp = r->plan;
                r->n_max = sp.path_hi;
                r->deep_steps = std::max<uint64_t>(1, sp.steps_to_mat.empty() ? 1 : sp.steps_to_mat.back());
                r->whole = sp.n_cv > 0;
                const uint64_t n_out = sp.opts.size();
                r->fixed_bytes = sizeof(SetDesc) + sp.segs.size() * sizeof(SegDesc) +
                                 sp.mats.size() * sizeof(MatDesc) + n_out * sizeof(OptDesc) +
                                 n_out * (kRowBytes * (kSumSlots + 1) + 48ull) + 4096;
                // the control variate's region of the launch's arena, bounded with one maturity per
                // option: per maturity its characteristic function at 385 nodes and its grid steps
                if (sp.n_cv > 0)
                    r->fixed_bytes += (uint64_t)sp.n_cv * (385ull * 16ull + r->deep_steps * 16ull + 64ull) +
                                      n_out * 12ull + 384ull * 16ull + 7ull * 256ull;
                // its smallest block (one tile; all of it with the control variate) beside the pool
                if (block_bytes(s, *r, r->whole ? r->n_max : s->tile_paths) + s->pool_bytes > s->cap ||
                    (!r->whole && r->plan.n_user > s->pool.rows))
                    r->status = HEXO_ERR_ADMISSION;   // can never fit
            }
            if (r->status != HEXO_OK) {
                it = s->pending.erase(it);
                finish(s, r, r->status, t);
                s->cv_done.notify_all();
                continue;
            }
        }
        bool fits = true;
        if (!r->whole) fits = s->pool.alloc(r->plan.n_user, r->row);
        if (fits) {
            r->n_rows = r->whole ? 0 : r->plan.n_user;
            r->admitted = true;
            r->seq = s->next_seq++;
            r->next_path = 0;
            s->active.push_back(r);
            ++s->st.admitted;
            it = s->pending.erase(it);
            continue;
        }
        if (t - r->t_submit > kStarveSeconds) break;   // nothing passes a request that has waited long
        ++it;
    }
    s->st.queued_now = s->pending.size();
}

// Builds and enqueues the next launch from the admitted requests without a
// block in flight; false when there is nothing to launch now.
bool launch_next(hexo_server *s, std::unique_lock<std::mutex> &lk) {
    if (s->inflight.size() >= s->opts.max_inflight) return false;
    int si = -1;
    for (size_t k = 0; k < s->streams.size(); ++k)
        if (!s->stream_busy[k]) { si = (int)k; break; }
    if (si < 0) return false;
    admit(s);
    std::vector<SrvReq *> cand;
    for (SrvReq *r : s->active)
        if (!r->in_flight && !r->done && r->next_path < r->n_max) cand.push_back(r);
    if (cand.empty()) return false;
    // least attained service: requests with the fewest blocks so far first
    std::sort(cand.begin(), cand.end(), [](const SrvReq *a, const SrvReq *b) {
        return a->blocks != b->blocks ? a->blocks < b->blocks : a->seq < b->seq;
    });
    if (cand.size() > s->opts.max_batch_requests) cand.resize(s->opts.max_batch_requests);
    const uint64_t share = std::max<uint64_t>(1, s->launch_budget / cand.size());
    std::vector<Block> blocks;
    uint64_t bytes = 0, work = 0;
    for (SrvReq *r : cand) {
        if (work >= s->launch_budget && !blocks.empty()) break;
        uint64_t n = r->n_max - r->next_path;
        if (!r->whole) {   // about `share` path-steps, whole tiles, at least 8 tiles
            const uint64_t P = s->tile_paths;
            uint64_t want = std::max<uint64_t>(8 * P, share / r->deep_steps / P * P);
            n = std::min(n, want);
        }
        uint64_t b = block_bytes(s, *r, n);
        const uint64_t room = s->cap - std::min(s->cap, s->st.mem_in_use + bytes);
        if (b > room) {   // a smaller block, or wait for a launch to finish
            if (r->whole || room < block_bytes(s, *r, s->tile_paths)) continue;
            n = std::min(n, (room - r->fixed_bytes) / sizeof(TileDesc) * s->tile_paths);
            b = block_bytes(s, *r, n);
        }
        blocks.push_back(Block{r, r->next_path, r->next_path + n, r->next_path + n == r->n_max});
        bytes += b;
        work += n * r->deep_steps;
    }
    if (blocks.empty()) return false;
    for (Block &b : blocks) {
        b.r->in_flight = true;
        b.r->next_path = b.hi;
        ++b.r->blocks;
    }
    s->st.chunks += blocks.size();
    s->st.mem_in_use += bytes;
    s->st.mem_peak = std::max(s->st.mem_peak, s->st.mem_in_use);
    s->stream_busy[si] = true;

    lk.unlock();   // planning the launch and uploading do not need the queue
    NvtxRange nvtx("hexo_server launch");
    BatchPlan bp;
    std::vector<SetPlan> plans;
    plans.reserve(blocks.size());
    uint32_t base = 0, cv_base = 0;
    for (const Block &b : blocks) cv_base += b.r->req.n_opts;   // control-variate slots after all outputs
    for (const Block &b : blocks) {
        SetPlan sp = b.r->plan;   // the request's schedule, restricted to the block's paths
        sp.path_lo = b.lo;
        sp.path_hi = b.hi;
        sp.set.n_paths = b.hi;
        plans.push_back(std::move(sp));
        batch_add(bp, plans.back(), base, cv_base);
        if (!b.r->whole)
            for (uint32_t k = 0; k < b.r->req.n_opts; ++k) {   // carried: finalised from the running sums
                const hexo_option &o = b.r->opts[k];
                bp.opt_paths[base + k] = o.n_paths ? o.n_paths : s->opts.cfg.n_paths;
                bp.opt_carry[base + k] = ((b.r->row + k) << 1) | (b.last ? 1ull : 0ull);
            }
        base += b.r->req.n_opts;
        cv_base += 2u * b.r->plan.n_cv;
    }
    bp.shape = ctx_shape(s->ctx, s->opts.cfg);
    fit_small_batch(s->ctx, s->opts.cfg, bp.shape, plans);
    batch_tiles(bp, plans);
    Inflight f;
    f.db.reset(new DeviceBatch());
    f.db->stream = s->streams[si];
    f.db->carry = s->pool.base;
    {
        const Arena &ar = s->arenas[si];
        f.db->dmem = ar.d;
        f.db->dcap = ar.dcap;
        f.db->hmem = ar.h;
        f.db->hcap = ar.hcap;
        f.db->own_d = f.db->own_h = false;
    }
    f.blocks = blocks;
    f.bytes = bytes;
    f.stream_index = si;
    hexo_status st = batch_upload(s->ctx, std::move(bp), s->opts.cfg.precision == HEXO_FP32, *f.db);
    cudaError_t e = cudaSuccess;
    // a request's first block clears its running sums, in stream order before the launch
    for (const Block &b : blocks)
        if (st == HEXO_OK && e == cudaSuccess && b.lo == 0 && b.r->n_rows)
            e = cudaMemsetAsync(s->pool.base + b.r->row * kLimbs, 0, b.r->n_rows * kRowBytes, f.db->stream);
    if (st == HEXO_OK && e == cudaSuccess) e = batch_enqueue(*f.db, f.db->stream, false);
    if (st == HEXO_OK && e == cudaSuccess) e = cudaEventCreateWithFlags(&f.done, cudaEventDisableTiming);
    if (st == HEXO_OK && e == cudaSuccess) e = cudaEventRecord(f.done, f.db->stream);
    lk.lock();
    if (st != HEXO_OK || e != cudaSuccess) {
        const hexo_status fail = st != HEXO_OK ? st : HEXO_ERR_CUDA;
        for (const Block &b : blocks) {
            b.r->in_flight = false;
            if (!b.r->done) finish(s, b.r, fail, now_s());
        }
        drop_active(s);
        keep_arena(s, f);
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
        retire(s);
        bool launched = false;
        while (launch_next(s, lk)) launched = true;
        if (!launched) admit(s);   // also fails requests that can never fit while launches run
        if (s->stop && s->pending.empty() && s->active.empty() && s->inflight.empty()) break;
        if (launched) continue;
        if (!s->inflight.empty()) s->cv_work.wait_for(lk, std::chrono::microseconds(50));
        else s->cv_work.wait_for(lk, std::chrono::milliseconds(5));
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
    if (s->opts.launch_path_steps) s->launch_budget = s->opts.launch_path_steps;
    s->cap = opts->mem_cap_bytes ? opts->mem_cap_bytes : ctx->mem_cap;
    cudaSetDevice(ctx->device);
    {
        size_t smem = 0;
        uint32_t cps = 0;
        const LaunchShape sh = ctx_shape(ctx, s->opts.cfg);
        const hexo_status st = shape_check(ctx, s->opts.cfg.precision == HEXO_FP32, sh, smem, cps);
        if (st != HEXO_OK) return st;
        s->tile_paths = sh.paths_per_tile();
    }
    // the pool of running sums: a quarter of the cap, at most 64 MiB
    const uint64_t rows = std::min<uint64_t>(s->cap / 4, kMaxPoolBytes) / kRowBytes;
    if (rows == 0) return HEXO_ERR_INVALID;
    if (cudaMalloc(&s->pool.base, rows * kRowBytes) != cudaSuccess) return HEXO_ERR_NOMEM;
    s->pool.reset(rows);
    s->pool_bytes = rows * kRowBytes;
    s->st.mem_in_use = s->st.mem_peak = s->pool_bytes;
    for (uint32_t k = 0; k < s->opts.max_inflight; ++k) {
        cudaStream_t st;
        if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) {
            for (cudaStream_t x : s->streams) cudaStreamDestroy(x);
            cudaFree(s->pool.base);
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
    if (s->pool.base) cudaFree(s->pool.base);
    delete s;
    return HEXO_OK;
}

} // extern "C"
