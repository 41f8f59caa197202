// tc_server.cpp -- continuous-batching request loop for triangle counts.
//
// Requests carry an edge list (or only the key of a graph already resident).
// They are split by size into two lanes, small and large, each driven by two
// host threads on their own contexts (streams) of one device:
//
//   prep thread   takes its lane's queued requests in arrival order, admits
//                 each when its footprint fits the HBM budget shared by both
//                 lanes (evicting least-recently-used idle resident graphs when
//                 needed), and builds the oriented CSR on the device (clean-up +
//                 orientation on the lane's prep stream); the graph stays
//                 resident under its key for later requests.
//   count thread  takes every ready request of its lane (up to max_batch),
//                 counts all their graphs with one batched persistent launch on
//                 the lane's count stream, and completes the requests.
//
// So requests arriving while a batch is counting are admitted, uploaded and
// oriented on the device concurrently with it and join their lane's next
// batch, and a small request never queues behind a large one: not for its
// build (the small lane's own prep thread) and not for its count (the small
// lane's own count stream).  On the device, the small lane's streams have the
// higher priority, and the large lane's persistent count kernel runs with
// reserve_blocks fewer blocks per SM than fit, so the block scheduler has
// room for the small lane's kernels while a large batch is running.  No
// kernel waits on another: the only waits are host-side and bounded (the
// batch watchdog, batch_timeout_ms); a batch that does not finish fails its
// requests with TC_E_TIMEOUT and stops the server from admitting more work.
// Submitted edge lists are copied (on up to 8 threads) into a pinned host
// staging area when it has room, so the build uploads them at the link's rate.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "tc_internal.h"

namespace {

using Clock = std::chrono::steady_clock;
using tc::set_error;

enum ReqState { kQueued, kPreparing, kReady, kCounting, kDone, kFailed };

constexpr int kSmall = 0, kLarge = 1, kLanes = 2;

struct Request {
    uint64_t id = 0, key = 0;
    int lane = kLarge;
    std::vector<int64_t> src, dst;  // the edges, when they did not fit the pinned staging area
    int64_t *h_src = nullptr, *h_dst = nullptr;  // the edges in the pinned staging area
    size_t stage_off = 0, stage_len = 0;         // their byte range there (stage_len 0: not staged)
    int64_t n_edges = 0;
    int64_t n_nodes = 0;
    Clock::time_point t_submit;
    double latency_ms = 0;
    ReqState state = kQueued;
    int status = TC_OK;
    std::string error;
    uint64_t count = 0;
    tc_graph *g = nullptr;
    bool owns_graph = false;  // graph without a key: freed after the count
};

struct Resident {
    tc_graph *g = nullptr;
    size_t bytes = 0;
    uint64_t last_use = 0;
    int in_use = 0;
    int lane = kLarge;  // the graph is bound to this lane's count context
};

}  // namespace

// One size class of requests: its queues, contexts and threads.
struct Lane {
    tc_ctx *count_ctx = nullptr, *prep_ctx = nullptr;
    cudaStream_t own_streams[2] = {nullptr, nullptr};  // prioritised streams (small lane), destroyed last
    std::deque<Request *> queued, ready;
    std::thread prep_thr, count_thr;
};

// First-fit allocator over one pinned host area (byte ranges), so that
// submitted edge lists are uploaded from page-locked memory at the link's
// rate instead of being staged through the driver.  Caller holds the mutex.
struct PinnedArena {
    unsigned char *base = nullptr;
    size_t size = 0;
    std::map<size_t, size_t> free_;  // offset -> length, coalesced
    void init(unsigned char *b, size_t n) {
        base = b;
        size = n;
        free_.clear();
        if (n) free_[0] = n;
    }
    bool take(size_t n, size_t *off) {
        n = (n + 255) & ~(size_t)255;
        for (auto it = free_.begin(); it != free_.end(); ++it)
            if (it->second >= n) {
                *off = it->first;
                const size_t rest = it->second - n, at = it->first + n;
                free_.erase(it);
                if (rest) free_[at] = rest;
                return true;
            }
        return false;
    }
    void give(size_t off, size_t n) {
        n = (n + 255) & ~(size_t)255;
        auto it = free_.emplace(off, n).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free_.erase(nx);
        }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_.erase(it);
            }
        }
    }
};

struct tc_server {
    Lane lane[2];  // kSmall, kLarge
    PinnedArena arena;
    tc_server_config cfg{};
    int64_t small_edges = 0;  // requests with at most this many edges take the small lane (< 0: none)
    size_t budget = 0, used = 0;
    std::mutex mu;
    std::condition_variable cv;
    std::unordered_map<uint64_t, Request *> reqs;
    std::unordered_map<uint64_t, Resident> cache;
    uint64_t next_id = 1, tick = 0;
    bool stopping = false;
    int fault = TC_OK;  // set when a batch failed; no more admissions
    tc_server_stats stats{};
};

namespace {

// Device bytes while building the oriented CSR from n edges: two 64-bit key
// buffers of 2n, flags, positions and the CSR arrays.
size_t prep_bytes(int64_t n) { return (size_t)n * 16 * 2 + (size_t)n * 2 * (1 + 4 + 8) + ((size_t)1 << 20); }

void release_edges(tc_server *s, Request *r);

void finish(tc_server *s, Request *r, int status, const char *err) {
    release_edges(s, r);
    r->status = status;
    r->state = status == TC_OK ? kDone : kFailed;
    if (err) r->error = err;
    r->latency_ms = std::chrono::duration<double, std::milli>(Clock::now() - r->t_submit).count();
    if (status == TC_OK) s->stats.completed++;
    else s->stats.failed++;
}

// Evicts LRU idle resident graphs until `need` more bytes fit.  Caller holds mu.
bool make_room(tc_server *s, size_t need) {
    while (s->used + need > s->budget) {
        auto victim = s->cache.end();
        for (auto it = s->cache.begin(); it != s->cache.end(); ++it)
            if (it->second.in_use == 0 && (victim == s->cache.end() || it->second.last_use < victim->second.last_use))
                victim = it;
        if (victim == s->cache.end()) return false;
        s->used -= victim->second.bytes;
        tc_graph_destroy(victim->second.g);
        s->cache.erase(victim);
        s->stats.evictions++;
    }
    return true;
}

// memcpy of n bytes on up to 8 threads (a large edge list is copied at the
// host's memory bandwidth rather than one core's).
void copy_parallel(void *dst, const void *src, size_t n) {
    const size_t kPer = (size_t)32 << 20;
    const int T = (int)std::min<size_t>(8, (n + kPer - 1) / kPer);
    if (T <= 1) {
        memcpy(dst, src, n);
        return;
    }
    std::vector<std::thread> th;
    const size_t step = (n + T - 1) / T;
    for (int t = 0; t < T; ++t) {
        const size_t a = std::min(n, (size_t)t * step), b = std::min(n, a + step);
        th.emplace_back([=] { memcpy((unsigned char *)dst + a, (const unsigned char *)src + a, b - a); });
    }
    for (auto &x : th) x.join();
}

// Drops a request's edge lists (staging range or vectors).  Caller holds mu.
void release_edges(tc_server *s, Request *r) {
    if (r->stage_len) s->arena.give(r->stage_off, r->stage_len);
    r->stage_len = 0;
    r->h_src = r->h_dst = nullptr;
    std::vector<int64_t>().swap(r->src);
    std::vector<int64_t>().swap(r->dst);
}

int lane_of(const tc_server *s, int64_t edges) { return s->small_edges >= 0 && edges <= s->small_edges ? kSmall : kLarge; }

void prep_loop(tc_server *s, int li) {
    Lane &L = s->lane[li];
    std::unique_lock<std::mutex> lk(s->mu);
    for (;;) {
        s->cv.wait(lk, [&] { return s->stopping || !L.queued.empty(); });
        if (s->stopping) return;
        Request *r = L.queued.front();
        if (s->fault != TC_OK) {
            L.queued.pop_front();
            finish(s, r, TC_E_STATE, "server stopped admitting after a failed batch");
            s->cv.notify_all();
            continue;
        }
        if (r->key) {
            auto it = s->cache.find(r->key);
            if (it != s->cache.end()) {  // resident: no preprocessing
                L.queued.pop_front();
                release_edges(s, r);
                it->second.in_use++;
                it->second.last_use = ++s->tick;
                r->g = it->second.g;
                r->state = kReady;
                s->stats.cache_hits++;
                s->lane[it->second.lane].ready.push_back(r);
                s->cv.notify_all();
                continue;
            }
        }
        if (r->n_edges == 0 && r->key) {
            L.queued.pop_front();
            finish(s, r, TC_E_STATE, "graph key is not resident and no edges were given");
            s->cv.notify_all();
            continue;
        }
        const int64_t n = r->n_edges;
        const size_t need = prep_bytes(n);
        if (need > s->budget) {
            L.queued.pop_front();
            finish(s, r, TC_E_NOMEM, "request needs more device memory than the whole budget");
            s->cv.notify_all();
            continue;
        }
        if (!make_room(s, need)) {  // wait for batches to release resident graphs
            s->cv.wait_for(lk, std::chrono::milliseconds(5));
            continue;
        }
        L.queued.pop_front();
        s->used += need;
        r->state = kPreparing;
        lk.unlock();
        tc_graph *g = nullptr;
        const int64_t *es = r->stage_len ? r->h_src : r->src.data();
        const int64_t *ed = r->stage_len ? r->h_dst : r->dst.data();
        int st = tc_graph_from_edges(L.prep_ctx, es, ed, n, r->n_nodes, s->cfg.tie, &g);
        std::string err = st == TC_OK ? std::string() : std::string(tc_last_error());
        if (st == TC_OK) st = tc::graph_rebind(g, L.count_ctx);
        lk.lock();
        s->used -= need;
        release_edges(s, r);  // the build has read them (its upload finished before it returned)
        if (st != TC_OK) {
            if (g) tc_graph_destroy(g);
            finish(s, r, st, err.c_str());
            s->cv.notify_all();
            continue;
        }
        const size_t bytes = tc::graph_device_bytes(g);
        s->used += bytes;
        r->g = g;
        // a key already made resident meanwhile (the other lane built it for a
        // request of another size) keeps its graph; this one is the request's own
        if (r->key && s->cache.count(r->key) == 0) {
            Resident &res = s->cache[r->key];
            res.g = g;
            res.bytes = bytes;
            res.in_use = 1;
            res.last_use = ++s->tick;
            res.lane = li;
        } else {
            r->owns_graph = true;
        }
        r->state = kReady;
        L.ready.push_back(r);
        s->cv.notify_all();
    }
}

void count_loop(tc_server *s, int li) {
    Lane &L = s->lane[li];
    std::unique_lock<std::mutex> lk(s->mu);
    for (;;) {
        s->cv.wait(lk, [&] { return s->stopping || !L.ready.empty(); });
        if (s->stopping && L.ready.empty()) return;
        std::vector<Request *> batch;
        int64_t pooled = 0;  // a launch's pooled edges stay below 2^31 - 1 (int32 in-list offsets)
        while (!L.ready.empty() && (int)batch.size() < s->cfg.max_batch &&
               (batch.empty() || pooled + L.ready.front()->g->nnz < (int64_t)INT32_MAX)) {
            pooled += L.ready.front()->g->nnz;
            batch.push_back(L.ready.front());
            L.ready.pop_front();
            batch.back()->state = kCounting;
        }
        // a batch is counted in the stats when it is taken (so a caller can
        // see that one is in flight)
        s->stats.batches++;
        if (li == kSmall) s->stats.small_batches++;
        else s->stats.large_batches++;
        s->stats.max_batch_seen = std::max<int64_t>(s->stats.max_batch_seen, (int64_t)batch.size());
        lk.unlock();
        std::vector<tc_graph *> gs(batch.size());
        for (size_t i = 0; i < batch.size(); ++i) gs[i] = batch[i]->g;
        std::vector<uint64_t> outs(batch.size());
        float kms = 0;
        int st = tc::count_graphs_direct(L.count_ctx, gs.data(), (int)gs.size(), outs.data(),
                                         s->cfg.batch_timeout_ms, &kms);
        std::string err = st == TC_OK ? std::string() : std::string(tc_last_error());
        lk.lock();
        if (st == TC_E_TIMEOUT) s->fault = st;
        for (size_t i = 0; i < batch.size(); ++i) {
            Request *r = batch[i];
            r->count = outs[i];
            finish(s, r, st, st == TC_OK ? nullptr : err.c_str());
            if (r->owns_graph) {
                s->used -= tc::graph_device_bytes(r->g);
                if (st != TC_E_TIMEOUT) tc_graph_destroy(r->g);
            } else if (r->key) {
                auto it = s->cache.find(r->key);
                if (it != s->cache.end()) {
                    it->second.in_use--;
                    it->second.last_use = ++s->tick;
                }
            }
            r->g = nullptr;
        }
        s->cv.notify_all();
    }
}

// Waits (bounded) until the stream has no work left; false if it still has
// work after timeout_ms or reports an error.
bool stream_drained(cudaStream_t st, int64_t timeout_ms) {
    const auto t0 = Clock::now();
    for (;;) {
        const cudaError_t q = cudaStreamQuery(st);
        if (q == cudaSuccess) return true;
        if (q != cudaErrorNotReady) return false;
        if (Clock::now() - t0 > std::chrono::milliseconds(timeout_ms)) return false;
        std::this_thread::sleep_for(std::chrono::milliseconds(1));
    }
}

int take_result(tc_server *s, Request *r, uint64_t *count, double *latency_ms) {
    if (count) *count = r->count;
    if (latency_ms) *latency_ms = r->latency_ms;
    const int st = r->status;
    if (st != TC_OK) set_error(st, "request %llu failed: %s", (unsigned long long)r->id, r->error.c_str());
    s->reqs.erase(r->id);
    delete r;
    return st;
}

}  // namespace

extern "C" {

int tc_server_create(tc_ctx *ctx, const tc_server_config *cfg, tc_server **out) {
    if (!ctx || !out) return set_error(TC_E_INVALID, "null argument");
    *out = nullptr;
    tc_server *s = new tc_server();
    if (cfg) s->cfg = *cfg;
    if (s->cfg.max_batch <= 0) s->cfg.max_batch = 256;
    if (s->cfg.batch_timeout_ms <= 0) s->cfg.batch_timeout_ms = 60000;
    if (s->cfg.tie != TC_TIE_ID_ASC) s->cfg.tie = TC_TIE_REFERENCE;
    s->small_edges = s->cfg.small_edges == 0 ? ((int64_t)1 << 20) : s->cfg.small_edges;
    const int reserve = s->cfg.reserve_blocks == 0 ? 1 : std::max(0, (int)s->cfg.reserve_blocks);
    const int dev = ctx->device;
    int st = cudaSetDevice(dev) == cudaSuccess ? TC_OK : set_error(TC_E_CUDA, "cudaSetDevice(%d) failed", dev);
    int prio_lo = 0, prio_hi = 0;
    if (st == TC_OK && cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi) != cudaSuccess)
        st = set_error(TC_E_CUDA, "stream priority query failed");
    tc_tuning base;
    if (st == TC_OK) st = tc_ctx_get_tuning(ctx, &base);
    for (int li = 0; li < kLanes && st == TC_OK; ++li) {
        Lane &L = s->lane[li];
        st = tc_ctx_create(dev, &L.count_ctx);
        if (st == TC_OK) st = tc_ctx_create(dev, &L.prep_ctx);
        if (st == TC_OK && li == kSmall) {
            // the small lane's streams at the highest priority: its blocks are
            // scheduled first whenever a large batch frees an SM slot
            for (int q = 0; q < 2 && st == TC_OK; ++q)
                if (cudaStreamCreateWithPriority(&L.own_streams[q], cudaStreamNonBlocking, prio_hi) != cudaSuccess)
                    st = set_error(TC_E_CUDA, "prioritised stream creation failed");
            if (st == TC_OK) st = tc_ctx_set_stream(L.count_ctx, L.own_streams[0]);
            if (st == TC_OK) st = tc_ctx_set_stream(L.prep_ctx, L.own_streams[1]);
        }
        if (st == TC_OK) {
            tc_tuning t = base;
            t.blocks_per_sm = -1;
            st = tc_ctx_set_tuning(L.count_ctx, &t);
            if (st == TC_OK && li == kLarge && reserve > 0 && s->small_edges >= 0) {
                // leave `reserve` block slots per SM to the small lane
                tc_tuning now;
                st = tc_ctx_get_tuning(L.count_ctx, &now);
                if (st == TC_OK && now.blocks_per_sm > reserve) {
                    t.blocks_per_sm = now.blocks_per_sm - reserve;
                    st = tc_ctx_set_tuning(L.count_ctx, &t);
                }
            }
        }
    }
    size_t total = 0;
    if (st == TC_OK) st = tc_ctx_device_info(ctx, nullptr, nullptr, &total);
    if (st != TC_OK) {
        const std::string why = tc_last_error();
        for (Lane &L : s->lane) {
            tc_ctx_destroy(L.count_ctx);
            tc_ctx_destroy(L.prep_ctx);
            for (cudaStream_t q : L.own_streams)
                if (q) cudaStreamDestroy(q);
        }
        delete s;
        return set_error(st, "server creation failed: %s", why.c_str());
    }
    const int64_t stage = s->cfg.staging_bytes == 0 ? ((int64_t)1 << 30) : s->cfg.staging_bytes;
    if (stage > 0) {
        void *h = nullptr;
        if (cudaMallocHost(&h, (size_t)stage) == cudaSuccess) s->arena.init((unsigned char *)h, (size_t)stage);
        else cudaGetLastError();  // no staging area: edges are kept in pageable memory
    }
    const double frac = s->cfg.hbm_budget_frac > 0 ? s->cfg.hbm_budget_frac : 0.8;
    s->budget = s->cfg.hbm_budget_bytes > 0 ? (size_t)s->cfg.hbm_budget_bytes : (size_t)(frac * (double)total);
    s->stats.budget_bytes = (int64_t)s->budget;
    for (int li = 0; li < kLanes; ++li) {
        s->lane[li].prep_thr = std::thread(prep_loop, s, li);
        s->lane[li].count_thr = std::thread(count_loop, s, li);
    }
    *out = s;
    return TC_OK;
}

int tc_server_submit(tc_server *s, uint64_t graph_key, const int64_t *src, const int64_t *dst, int64_t n_edges,
                     int64_t n_nodes, uint64_t *request_id) {
    if (!s || !request_id || n_edges < 0 || (n_edges > 0 && (!src || !dst)))
        return set_error(TC_E_INVALID, "bad request arguments");
    Request *r = new Request();
    r->key = graph_key;
    r->n_nodes = n_nodes;
    r->t_submit = Clock::now();
    r->lane = lane_of(s, n_edges);
    {
        // resident key: pin the graph and go straight to the count thread of
        // the lane that holds it, without copying the edges
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->stopping) {
            delete r;
            return set_error(TC_E_STATE, "server is shutting down");
        }
        auto it = graph_key ? s->cache.find(graph_key) : s->cache.end();
        if (it != s->cache.end() && s->fault == TC_OK) {
            it->second.in_use++;
            it->second.last_use = ++s->tick;
            r->g = it->second.g;
            r->lane = it->second.lane;
            r->state = kReady;
            r->id = s->next_id++;
            s->reqs[r->id] = r;
            s->lane[r->lane].ready.push_back(r);
            s->stats.submitted++;
            s->stats.cache_hits++;
            *request_id = r->id;
            s->cv.notify_all();
            return TC_OK;
        }
    }
    r->n_edges = n_edges;
    if (n_edges > 0) {
        // into the pinned staging area when it has room, else into vectors
        const size_t half = ((size_t)n_edges * sizeof(int64_t) + 255) & ~(size_t)255;
        size_t off = 0;
        bool staged;
        {
            std::lock_guard<std::mutex> lk(s->mu);
            staged = s->arena.size && s->arena.take(2 * half, &off);
        }
        if (staged) {
            r->stage_off = off;
            r->stage_len = 2 * half;
            r->h_src = (int64_t *)(s->arena.base + off);
            r->h_dst = (int64_t *)(s->arena.base + off + half);
            copy_parallel(r->h_src, src, (size_t)n_edges * sizeof(int64_t));
            copy_parallel(r->h_dst, dst, (size_t)n_edges * sizeof(int64_t));
        } else {
            r->src.assign(src, src + n_edges);
            r->dst.assign(dst, dst + n_edges);
        }
    }
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stopping) {
        release_edges(s, r);
        delete r;
        return set_error(TC_E_STATE, "server is shutting down");
    }
    r->id = s->next_id++;
    s->reqs[r->id] = r;
    s->lane[r->lane].queued.push_back(r);
    s->stats.submitted++;
    *request_id = r->id;
    s->cv.notify_all();
    return TC_OK;
}

int tc_server_poll(tc_server *s, uint64_t request_id, uint64_t *count, double *latency_ms) {
    if (!s) return set_error(TC_E_INVALID, "null server");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(request_id);
    if (it == s->reqs.end()) return set_error(TC_E_INVALID, "unknown request %llu", (unsigned long long)request_id);
    Request *r = it->second;
    if (r->state != kDone && r->state != kFailed) return TC_E_NOT_READY;
    return take_result(s, r, count, latency_ms);
}

int tc_server_wait(tc_server *s, uint64_t request_id, int64_t timeout_ms, uint64_t *count, double *latency_ms) {
    if (!s) return set_error(TC_E_INVALID, "null server");
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(request_id);
    if (it == s->reqs.end()) return set_error(TC_E_INVALID, "unknown request %llu", (unsigned long long)request_id);
    Request *r = it->second;
    const auto done = [&] { return r->state == kDone || r->state == kFailed; };
    if (timeout_ms < 0) s->cv.wait(lk, done);
    else if (!s->cv.wait_for(lk, std::chrono::milliseconds(timeout_ms), done))
        return set_error(TC_E_TIMEOUT, "request %llu not done after %lld ms", (unsigned long long)request_id,
                         (long long)timeout_ms);
    return take_result(s, r, count, latency_ms);
}

int tc_server_get_stats(tc_server *s, tc_server_stats *out) {
    if (!s || !out) return set_error(TC_E_INVALID, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    *out = s->stats;
    out->resident_graphs = (int64_t)s->cache.size();
    out->used_bytes = (int64_t)s->used;
    out->queued = (int64_t)(s->lane[kSmall].queued.size() + s->lane[kLarge].queued.size());
    return TC_OK;
}

int tc_server_destroy(tc_server *s) {
    if (!s) return TC_OK;
    {
        std::unique_lock<std::mutex> lk(s->mu);
        // drain: let admitted and ready work finish, fail what is still queued
        for (Lane &L : s->lane)
            while (!L.queued.empty()) {
                Request *r = L.queued.front();
                L.queued.pop_front();
                finish(s, r, TC_E_STATE, "server shut down before the request was admitted");
            }
        s->cv.wait_for(lk, std::chrono::milliseconds(s->cfg.batch_timeout_ms), [&] {
            for (Lane &L : s->lane)
                if (!L.ready.empty()) return false;
            for (auto &kv : s->reqs)
                if (kv.second->state == kPreparing || kv.second->state == kCounting) return false;
            return true;
        });
        s->stopping = true;
        s->cv.notify_all();
    }
    for (Lane &L : s->lane) {
        L.prep_thr.join();
        L.count_thr.join();
    }
    // A batch that overran its watchdog may still be running on a count
    // stream: its graphs must not be freed under it.  Wait for it (bounded);
    // if it is still running, leave the device memory allocated.
    bool drained = true;
    if (s->fault != TC_OK)
        for (Lane &L : s->lane)
            drained = drained &&
                      stream_drained(L.count_ctx->stream, std::max<int64_t>(s->cfg.batch_timeout_ms, 5000));
    for (auto &kv : s->reqs) {
        if (drained && kv.second->owns_graph && kv.second->g) tc_graph_destroy(kv.second->g);
        delete kv.second;
    }
    if (!drained) {
        if (s->arena.base) cudaFreeHost(s->arena.base);  // the builds that read it have returned
        delete s;
        return set_error(TC_E_TIMEOUT, "a timed-out batch is still running; its device memory was left allocated");
    }
    for (auto &kv : s->cache) tc_graph_destroy(kv.second.g);
    for (Lane &L : s->lane) {
        // a context's stream is synchronised when its last object goes
        tc_ctx_destroy(L.count_ctx);
        tc_ctx_destroy(L.prep_ctx);
    }
    for (Lane &L : s->lane)
        for (cudaStream_t q : L.own_streams)
            if (q) {
                cudaStreamSynchronize(q);
                cudaStreamDestroy(q);
            }
    if (s->arena.base) cudaFreeHost(s->arena.base);
    delete s;
    return TC_OK;
}

}  // extern "C"
