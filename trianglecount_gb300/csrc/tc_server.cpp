// tc_server.cpp -- continuous-batching request loop for triangle counts.
//
// Requests carry an edge list (or only the key of a graph already resident).
// Two host threads drive one device through two contexts (two streams):
//
//   prep thread   takes queued requests in arrival order, admits each when its
//                 footprint fits the HBM budget (evicting least-recently-used
//                 idle resident graphs when needed), and builds the oriented CSR
//                 on the device (clean-up + orientation on the prep stream);
//                 the graph stays resident under its key for later requests.
//   count thread  takes every ready request (up to max_batch), counts all their
//                 graphs with one batched persistent launch on the count stream,
//                 and completes the requests.
//
// So requests arriving while a batch is counting are admitted, uploaded and
// oriented on the device concurrently with it and join the next batch.  No
// kernel waits on another: the only waits are host-side and bounded (the
// batch watchdog, batch_timeout_ms); a batch that does not finish fails its
// requests with TC_E_TIMEOUT and stops the server from admitting more work.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "tc_internal.h"

namespace {

using Clock = std::chrono::steady_clock;
using tc::set_error;

enum ReqState { kQueued, kPreparing, kReady, kCounting, kDone, kFailed };

struct Request {
    uint64_t id = 0, key = 0;
    std::vector<int64_t> src, dst;
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
};

}  // namespace

struct tc_server {
    tc_ctx *count_ctx = nullptr, *prep_ctx = nullptr;
    tc_server_config cfg{};
    size_t budget = 0, used = 0;
    std::mutex mu;
    std::condition_variable cv;
    std::deque<Request *> queued, ready;
    std::unordered_map<uint64_t, Request *> reqs;
    std::unordered_map<uint64_t, Resident> cache;
    uint64_t next_id = 1, tick = 0;
    bool stopping = false;
    int fault = TC_OK;  // set when a batch failed; no more admissions
    tc_server_stats stats{};
    std::thread prep_thr, count_thr;
};

namespace {

// Device bytes while building the oriented CSR from n edges: two 64-bit key
// buffers of 2n, flags, positions and the CSR arrays.
size_t prep_bytes(int64_t n) { return (size_t)n * 16 * 2 + (size_t)n * 2 * (1 + 4 + 8) + ((size_t)1 << 20); }

void finish(tc_server *s, Request *r, int status, const char *err) {
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

void prep_loop(tc_server *s) {
    std::unique_lock<std::mutex> lk(s->mu);
    for (;;) {
        s->cv.wait(lk, [&] { return s->stopping || !s->queued.empty(); });
        if (s->stopping) return;
        Request *r = s->queued.front();
        if (s->fault != TC_OK) {
            s->queued.pop_front();
            finish(s, r, TC_E_STATE, "server stopped admitting after a failed batch");
            s->cv.notify_all();
            continue;
        }
        if (r->key) {
            auto it = s->cache.find(r->key);
            if (it != s->cache.end()) {  // resident: no preprocessing
                s->queued.pop_front();
                it->second.in_use++;
                it->second.last_use = ++s->tick;
                r->g = it->second.g;
                r->state = kReady;
                s->stats.cache_hits++;
                s->ready.push_back(r);
                s->cv.notify_all();
                continue;
            }
        }
        if (r->src.empty() && r->dst.empty() && r->key) {
            s->queued.pop_front();
            finish(s, r, TC_E_STATE, "graph key is not resident and no edges were given");
            s->cv.notify_all();
            continue;
        }
        const int64_t n = (int64_t)r->src.size();
        const size_t need = prep_bytes(n);
        if (need > s->budget) {
            s->queued.pop_front();
            finish(s, r, TC_E_NOMEM, "request needs more device memory than the whole budget");
            s->cv.notify_all();
            continue;
        }
        if (!make_room(s, need)) {  // wait for batches to release resident graphs
            s->cv.wait_for(lk, std::chrono::milliseconds(5));
            continue;
        }
        s->queued.pop_front();
        s->used += need;
        r->state = kPreparing;
        lk.unlock();
        tc_graph *g = nullptr;
        int st = tc_graph_from_edges(s->prep_ctx, r->src.data(), r->dst.data(), n, r->n_nodes, s->cfg.tie, &g);
        std::string err = st == TC_OK ? std::string() : std::string(tc_last_error());
        if (st == TC_OK) st = tc::graph_rebind(g, s->count_ctx);
        lk.lock();
        s->used -= need;
        std::vector<int64_t>().swap(r->src);
        std::vector<int64_t>().swap(r->dst);
        if (st != TC_OK) {
            if (g) tc_graph_destroy(g);
            finish(s, r, st, err.c_str());
            s->cv.notify_all();
            continue;
        }
        const size_t bytes = tc::graph_device_bytes(g);
        s->used += bytes;
        r->g = g;
        if (r->key) {
            Resident &res = s->cache[r->key];
            res.g = g;
            res.bytes = bytes;
            res.in_use = 1;
            res.last_use = ++s->tick;
        } else {
            r->owns_graph = true;
        }
        r->state = kReady;
        s->ready.push_back(r);
        s->cv.notify_all();
    }
}

void count_loop(tc_server *s) {
    std::unique_lock<std::mutex> lk(s->mu);
    for (;;) {
        s->cv.wait(lk, [&] { return s->stopping || !s->ready.empty(); });
        if (s->stopping && s->ready.empty()) return;
        std::vector<Request *> batch;
        while (!s->ready.empty() && (int)batch.size() < s->cfg.max_batch) {
            batch.push_back(s->ready.front());
            s->ready.pop_front();
            batch.back()->state = kCounting;
        }
        lk.unlock();
        std::vector<tc_graph *> gs(batch.size());
        for (size_t i = 0; i < batch.size(); ++i) gs[i] = batch[i]->g;
        std::vector<uint64_t> outs(batch.size());
        float kms = 0;
        int st = tc::count_graphs_direct(s->count_ctx, gs.data(), (int)gs.size(), outs.data(),
                                         s->cfg.batch_timeout_ms, &kms);
        std::string err = st == TC_OK ? std::string() : std::string(tc_last_error());
        lk.lock();
        s->stats.batches++;
        s->stats.max_batch_seen = std::max<int64_t>(s->stats.max_batch_seen, (int64_t)batch.size());
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
    int dev = ctx->device;
    int st = tc_ctx_create(dev, &s->count_ctx);
    if (st == TC_OK) st = tc_ctx_create(dev, &s->prep_ctx);
    if (st == TC_OK) {
        tc_tuning t;
        tc_ctx_get_tuning(ctx, &t);
        t.blocks_per_sm = -1;
        st = tc_ctx_set_tuning(s->count_ctx, &t);
    }
    size_t total = 0;
    if (st == TC_OK) st = tc_ctx_device_info(ctx, nullptr, nullptr, &total);
    if (st != TC_OK) {
        tc_ctx_destroy(s->count_ctx);
        tc_ctx_destroy(s->prep_ctx);
        delete s;
        return st;
    }
    const double frac = s->cfg.hbm_budget_frac > 0 ? s->cfg.hbm_budget_frac : 0.8;
    s->budget = s->cfg.hbm_budget_bytes > 0 ? (size_t)s->cfg.hbm_budget_bytes : (size_t)(frac * (double)total);
    s->stats.budget_bytes = (int64_t)s->budget;
    s->prep_thr = std::thread(prep_loop, s);
    s->count_thr = std::thread(count_loop, s);
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
    {
        // resident key: pin the graph and go straight to the count thread,
        // without copying the edges
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
            r->state = kReady;
            r->id = s->next_id++;
            s->reqs[r->id] = r;
            s->ready.push_back(r);
            s->stats.submitted++;
            s->stats.cache_hits++;
            *request_id = r->id;
            s->cv.notify_all();
            return TC_OK;
        }
    }
    if (n_edges > 0) {
        r->src.assign(src, src + n_edges);
        r->dst.assign(dst, dst + n_edges);
    }
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stopping) {
        delete r;
        return set_error(TC_E_STATE, "server is shutting down");
    }
    r->id = s->next_id++;
    s->reqs[r->id] = r;
    s->queued.push_back(r);
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
    out->queued = (int64_t)s->queued.size();
    return TC_OK;
}

int tc_server_destroy(tc_server *s) {
    if (!s) return TC_OK;
    {
        std::unique_lock<std::mutex> lk(s->mu);
        // drain: let admitted and ready work finish, fail what is still queued
        while (!s->queued.empty()) {
            Request *r = s->queued.front();
            s->queued.pop_front();
            finish(s, r, TC_E_STATE, "server shut down before the request was admitted");
        }
        s->cv.wait_for(lk, std::chrono::milliseconds(s->cfg.batch_timeout_ms), [&] {
            if (!s->ready.empty()) return false;
            for (auto &kv : s->reqs)
                if (kv.second->state == kPreparing || kv.second->state == kCounting) return false;
            return true;
        });
        s->stopping = true;
        s->cv.notify_all();
    }
    s->prep_thr.join();
    s->count_thr.join();
    // A batch that overran its watchdog may still be running on the count
    // stream: its graphs must not be freed under it.  Wait for it (bounded);
    // if it is still running, leave the device memory allocated.
    const bool drained = s->fault == TC_OK ||
                         stream_drained(s->count_ctx->stream, std::max<int64_t>(s->cfg.batch_timeout_ms, 5000));
    for (auto &kv : s->reqs) {
        if (drained && kv.second->owns_graph && kv.second->g) tc_graph_destroy(kv.second->g);
        delete kv.second;
    }
    if (!drained) {
        delete s;
        return set_error(TC_E_TIMEOUT, "a timed-out batch is still running; its device memory was left allocated");
    }
    for (auto &kv : s->cache) tc_graph_destroy(kv.second.g);
    tc_ctx_destroy(s->count_ctx);
    tc_ctx_destroy(s->prep_ctx);
    delete s;
    return TC_OK;
}

}  // extern "C"
