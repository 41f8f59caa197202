// tc_api.cu -- C ABI: contexts, oriented graphs, plain and batched counting.
#include <algorithm>
#include <chrono>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <memory>
#include <thread>
#include <vector>

#include "tc_internal.h"

namespace tc {

namespace {
thread_local std::string g_last_error;

constexpr int kVersion = 10000;  // 1.0.0

// ---- CSR validation (rows strictly ascending, ids in range) ----
struct ValidateErr {
    int code;     // 0 ok, 1 row_ptr, 2 id range, 3 order
    int first;    // smallest offending row / entry index
    int max_deg;  // longest row
};

__global__ void mark_rows_kernel(const int32_t *rp, int64_t n_rows, int64_t nnz, uint8_t *start, ValidateErr *err) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    int longest = 0;
    for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < n_rows; u += stride) {
        const int64_t a = rp[u], b = rp[u + 1];
        const bool bad = a > b || a < 0 || b > nnz || (u == 0 && a != 0) || (u == n_rows - 1 && b != nnz);
        if (bad) {
            atomicMax(&err->code, 1);
            atomicMin(&err->first, (int)u);
        } else if (a < b) {
            start[a] = 1;
            longest = max(longest, (int)(b - a));
        }
    }
    longest = __reduce_max_sync(0xffffffffu, longest);
    if ((threadIdx.x & 31) == 0 && longest) atomicMax(&err->max_deg, longest);
}

// Longest row of a CSR (the out-degree bound that selects the flat count).
__global__ void max_row_kernel(const int32_t *rp, int64_t n_rows, int *out) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    int longest = 0;
    for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < n_rows; u += stride)
        longest = max(longest, rp[u + 1] - rp[u]);
    longest = __reduce_max_sync(0xffffffffu, longest);
    if ((threadIdx.x & 31) == 0 && longest) atomicMax(out, longest);
}

// Four entries per thread: one 16-byte load of col[j..j+4), the next entry
// and the four row-start marks after them (col is 256-byte aligned).
__global__ void check_cols_kernel(const int32_t *col, int64_t nnz, int64_t n_rows, const uint8_t *start,
                                  ValidateErr *err) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t groups = (nnz + 3) / 4;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < groups; q += stride) {
        const int64_t j0 = 4 * q;
        int x[5];
        if (j0 + 4 <= nnz) {
            const int4 v = __ldg(reinterpret_cast<const int4 *>(col) + q);
            x[0] = v.x, x[1] = v.y, x[2] = v.z, x[3] = v.w;
        } else {
            for (int i = 0; i < 4; ++i) x[i] = j0 + i < nnz ? __ldg(col + j0 + i) : 0;
        }
        x[4] = j0 + 4 < nnz ? __ldg(col + j0 + 4) : 0;
        for (int i = 0; i < 4; ++i) {
            const int64_t j = j0 + i;
            if (j >= nnz) break;
            int code = 0;
            if (x[i] < 0 || x[i] >= n_rows) code = 2;
            else if (j + 1 < nnz && !__ldg(start + j + 1) && x[i + 1] <= x[i]) code = 3;
            if (code) {
                atomicMax(&err->code, code);
                atomicMin(&err->first, (int)j);
            }
        }
    }
}

__global__ void narrow_u64_kernel(const uint64_t *in, int32_t *out, int64_t n, uint64_t limit, int *overflow) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const uint64_t v = in[i];
        if (v > limit) *overflow = 1;
        out[i] = (int32_t)v;
    }
}

__global__ void set_validate_err_kernel(ValidateErr *dst, ValidateErr v) { *dst = v; }

int grid_for(int64_t n, int sm) {
    const int64_t b = (n + 255) / 256;
    return (int)std::max<int64_t>(1, std::min<int64_t>(b, (int64_t)sm * 32));
}

int validate_csr_impl(tc_ctx *ctx, const int32_t *rp, const int32_t *col, int64_t n_rows, int64_t nnz,
                      int32_t *max_deg = nullptr) {
    cudaStream_t s = ctx->stream;
    DBuf<uint8_t> start;
    DBuf<ValidateErr> err;
    TC_TRY(start.alloc((size_t)nnz + 1, s));
    TC_TRY(err.alloc(1, s));
    TC_CUDA(cudaMemsetAsync(start.p, 0, (size_t)nnz + 1, s));
    ValidateErr init{0, 0x7fffffff, 0};
    TC_CUDA(cudaMemcpyAsync(err.p, &init, sizeof(init), cudaMemcpyHostToDevice, s));
    if (n_rows > 0) {
        mark_rows_kernel<<<grid_for(n_rows, ctx->sm_count), 256, 0, s>>>(rp, n_rows, nnz, start.p, err.p);
        TC_CUDA(cudaGetLastError());
    }
    if (nnz > 0) {
        check_cols_kernel<<<grid_for(nnz, ctx->sm_count), 256, 0, s>>>(col, nnz, n_rows, start.p, err.p);
        TC_CUDA(cudaGetLastError());
    }
    ValidateErr h;
    TC_CUDA(cudaMemcpyAsync(&h, err.p, sizeof(h), cudaMemcpyDeviceToHost, s));
    TC_CUDA(cudaStreamSynchronize(s));
    if (n_rows == 0 && nnz != 0) return set_error(TC_E_FORMAT, "CSR has 0 rows but %lld entries", (long long)nnz);
    switch (h.code) {
    case 1: return set_error(TC_E_FORMAT, "row_ptr is not a valid offset array at row %d", h.first);
    case 2: return set_error(TC_E_FORMAT, "column id out of range [0, %lld) at entry %d", (long long)n_rows, h.first);
    case 3: return set_error(TC_E_FORMAT, "row not strictly ascending at entry %d", h.first);
    default:
        if (max_deg) *max_deg = h.max_deg;
        return TC_OK;
    }
}

// validate_csr_impl's kernels enqueued on stream s, the verdict written to
// the device word d_err (initialised here); start must hold nnz + 1 bytes.
int validate_csr_enqueue(tc_ctx *ctx, cudaStream_t s, const int32_t *rp, const int32_t *col, int64_t n_rows,
                         int64_t nnz, uint8_t *start, ValidateErr *d_err) {
    TC_CUDA(cudaMemsetAsync(start, 0, (size_t)nnz + 1, s));
    const ValidateErr init{0, 0x7fffffff, 0};
    // a parameter of a one-thread kernel, not a copy from this stack frame
    set_validate_err_kernel<<<1, 1, 0, s>>>(d_err, init);
    TC_CUDA(cudaGetLastError());
    if (n_rows > 0) {
        mark_rows_kernel<<<grid_for(n_rows, ctx->sm_count), 256, 0, s>>>(rp, n_rows, nnz, start, d_err);
        TC_CUDA(cudaGetLastError());
    }
    if (nnz > 0) {
        check_cols_kernel<<<grid_for(nnz, ctx->sm_count), 256, 0, s>>>(col, nnz, n_rows, start, d_err);
        TC_CUDA(cudaGetLastError());
    }
    return TC_OK;
}

// The verdict of validate_csr_enqueue as a status (max_deg: the longest row).
int validate_verdict(const ValidateErr &h, int64_t n_rows, int64_t nnz, int32_t *max_deg) {
    if (n_rows == 0 && nnz != 0) return set_error(TC_E_FORMAT, "CSR has 0 rows but %lld entries", (long long)nnz);
    switch (h.code) {
    case 1: return set_error(TC_E_FORMAT, "row_ptr is not a valid offset array at row %d", h.first);
    case 2: return set_error(TC_E_FORMAT, "column id out of range [0, %lld) at entry %d", (long long)n_rows, h.first);
    case 3: return set_error(TC_E_FORMAT, "row not strictly ascending at entry %d", h.first);
    default:
        if (max_deg) *max_deg = h.max_deg;
        return TC_OK;
    }
}

int check_graph(const tc_graph *g) {
    if (!g || !g->ctx) return set_error(TC_E_INVALID, "null graph");
    return TC_OK;
}

// Count scratch of a graph: descriptor, work words + result, CountScratch.
int ensure_count_scratch(tc_graph *g) {
    tc_ctx *ctx = g->ctx;
    if (!g->d_work) {
        void *p = nullptr;
        TC_TRY(dalloc(&p, sizeof(CountWork) + sizeof(unsigned long long), ctx->stream));
        g->d_work = (CountWork *)p;
        g->d_result = (unsigned long long *)(g->d_work + 1);
    }
    if (!g->d_desc) {  // the flat count needs only the work words
        TC_TRY(dalloc((void **)&g->d_desc, sizeof(GraphDesc), ctx->stream));
        TC_TRY(scratch_alloc(&g->sc, g->n_rows + 1, g->nnz,
                             std::min(g->n_rows, g->nnz) + 1, ctx->stream));
    }
    return TC_OK;
}

__global__ void set_desc_kernel(GraphDesc *dst, GraphDesc d) { *dst = d; }

// Up to eight descriptors as one kernel parameter (512 bytes): a table is
// written in stream order with no host copy (a copy from pageable memory
// would first wait for the stream to drain).
struct DescBlock {
    GraphDesc d[8];
};
__global__ void set_descs_kernel(GraphDesc *dst, DescBlock b, int n) {
    if ((int)threadIdx.x < n) dst[threadIdx.x] = b.d[threadIdx.x];
}

// The count kernels' error word (CountWork::error) as text.
const char *count_error_text(int code) {
    return code == 2 ? "a bulk-copy staging wait of the count kernel gave up" : "heavy-unit list overflow";
}

// A stream the library may capture: not a default stream (those cannot be
// captured) and not one the caller is capturing (the chain's launches then
// belong to the caller's graph).
bool capturable(cudaStream_t s) {
    if (s == nullptr || s == cudaStreamLegacy || s == cudaStreamPerThread) return false;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cs) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return cs == cudaStreamCaptureStatusNone;
}

// Captures g's count chain (results into res) on the context's stream, which
// must be capturable, as a CUDA graph in g->exec.  Leaves g->exec null, and
// the stream usable, when the capture fails.
void capture_count(tc_graph *g, unsigned long long *res) {
    tc_ctx *ctx = g->ctx;
    cudaStream_t s = ctx->stream;
    if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        cudaGetLastError();
        return;
    }
    int nl = 0;
    const int st = launch_count(g->d_desc, 1, (g->n_rows + 31) / 32, g->n_rows + 1, g->n_rows, g->sc, g->d_work, res,
                                false, ctx->tuned, s, &nl, ctx->kev, g->n_roots < g->n_rows);
    cudaGraph_t graph = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(s, &graph);
    cudaGraphExec_t exec = nullptr;
    if (st == TC_OK && ce == cudaSuccess && graph && cudaGraphInstantiate(&exec, graph, 0) == cudaSuccess) {
        g->exec = exec;
        g->exec_results = res;
        g->exec_epoch = ctx->tuning_epoch;
        g->exec_launches = nl;
    }
    if (graph) cudaGraphDestroy(graph);
    cudaGetLastError();  // a failed capture falls back to direct launches
}

bool flat_count(const tc_graph *g) { return g->max_deg >= 0 && g->max_deg <= g->ctx->tuned.flat_max_deg; }

// Everything a count of g needs before its launches: the work words, the
// scratch and the descriptor, and -- from the graph's second chain count on
// -- the captured chain.  Callers that time a count run this before their
// start event, so neither allocations nor a capture land in the timed span.
int prepare_graph_count(tc_graph *g, unsigned long long *per_root, unsigned long long *results) {
    tc_ctx *ctx = g->ctx;
    if (flat_count(g)) {  // every list fits a lane's registers: one kernel, no transpose or hash tables
        if (!g->d_work) {
            void *p = nullptr;
            TC_TRY(dalloc(&p, sizeof(CountWork) + sizeof(unsigned long long), ctx->stream));
            g->d_work = (CountWork *)p;
            g->d_result = (unsigned long long *)(g->d_work + 1);
        }
        return TC_OK;
    }
    TC_TRY(ensure_count_scratch(g));
    GraphDesc d;
    memset(&d, 0, sizeof d);
    d.rp = g->rp;
    d.col = g->col;
    d.n_rows = g->n_rows;
    d.n_roots = g->n_roots;
    d.chunk_base = 0;
    d.vbase = 0;
    d.per_root = per_root;
    if (!g->desc_valid || memcmp(&d, &g->desc_on_device, sizeof(d)) != 0) {
        // a one-thread kernel with the descriptor as its parameter, not a copy
        // from this stack frame: a caller capturing the stream keeps the value
        set_desc_kernel<<<1, 1, 0, ctx->stream>>>(g->d_desc, d);
        TC_CUDA(cudaGetLastError());
        g->desc_on_device = d;
        g->desc_valid = true;
    }
    unsigned long long *res = results ? results : g->d_result;
    if (!per_root && g->n_rows > 0 && capturable(ctx->stream)) {
        if (g->exec && g->exec_epoch != ctx->tuning_epoch) {
            cudaGraphExecDestroy(g->exec);
            g->exec = nullptr;
        }
        // (re)capture for a results pointer that the previous count used too;
        // a pointer seen once is counted with direct launches
        const bool stable = g->chain_counts >= 1 && res == g->last_results;
        if (stable && g->exec && g->exec_results != res) {
            cudaGraphExecDestroy(g->exec);
            g->exec = nullptr;
        }
        if (stable && !g->exec) capture_count(g, res);  // on failure: direct launches
    }
    return TC_OK;
}

int enqueue_graph_count(tc_graph *g, unsigned long long *per_root, unsigned long long *results, int *launches) {
    tc_ctx *ctx = g->ctx;
    TC_TRY(prepare_graph_count(g, per_root, results));
    unsigned long long *res = results ? results : g->d_result;
    if (flat_count(g)) {
        ctx->kev_recorded = true;
        return launch_flat(g->rp, g->col, g->n_roots, g->max_deg, g->d_work, res, per_root, ctx->tuned, ctx->stream,
                           launches, ctx->kev);
    }
    const int64_t chunks = (g->n_rows + 31) / 32;
    ctx->kev_recorded = chunks > 0;
    ++g->chain_counts;
    if (!per_root) g->last_results = res;
    if (!per_root && g->exec && g->exec_results == res && g->exec_epoch == ctx->tuning_epoch &&
        capturable(ctx->stream)) {
        TC_CUDA(cudaGraphLaunch(g->exec, ctx->stream));
        if (launches) *launches = g->exec_launches;
        return TC_OK;
    }
    return launch_count(g->d_desc, 1, chunks, g->n_rows + 1, g->n_rows, g->sc, g->d_work, res, per_root != nullptr,
                        ctx->tuned, ctx->stream, launches, ctx->kev, g->n_roots < g->n_rows);
}

int new_graph(tc_ctx *ctx, int64_t n_rows, int64_t nnz, int64_t n_roots, tc_graph **out) {
    if (!ctx || !out) return set_error(TC_E_INVALID, "null context or output");
    if (n_rows < 0 || nnz < 0 || n_roots < 0 || n_roots > n_rows)
        return set_error(TC_E_INVALID, "bad sizes: n_rows=%lld nnz=%lld n_roots=%lld", (long long)n_rows,
                         (long long)nnz, (long long)n_roots);
    if (n_rows >= INT32_MAX || nnz >= INT32_MAX)
        return set_error(TC_E_RANGE, "graph too large for int32 indices: n_rows=%lld nnz=%lld", (long long)n_rows,
                         (long long)nnz);
    tc_graph *g = new tc_graph();
    g->ctx = ctx;
    ctx_retain(ctx);
    g->n_rows = n_rows;
    g->nnz = nnz;
    g->n_roots = n_roots;
    *out = g;
    return TC_OK;
}

}  // namespace

int validate_csr(tc_ctx *ctx, const int32_t *rp, const int32_t *col, int64_t n_rows, int64_t nnz) {
    return validate_csr_impl(ctx, rp, col, n_rows, nnz);
}

int set_error(int status, const char *fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return status;
}

int cuda_error(cudaError_t e, const char *what, const char *file, int line) {
    const char *base = strrchr(file, '/');
    set_error(e == cudaErrorMemoryAllocation ? TC_E_NOMEM : TC_E_CUDA, "%s failed: %s (%s:%d)", what,
              cudaGetErrorString(e), base ? base + 1 : file, line);
    return e == cudaErrorMemoryAllocation ? TC_E_NOMEM : TC_E_CUDA;
}

int dalloc(void **p, size_t bytes, cudaStream_t s) {
    cudaError_t e = cudaMallocAsync(p, bytes, s);
    if (e != cudaSuccess) {
        *p = nullptr;
        return cuda_error(e, "cudaMallocAsync", __FILE__, __LINE__);
    }
    return TC_OK;
}

void dfree(void *p, cudaStream_t s) {
    if (p) cudaFreeAsync(p, s);
}

void ctx_retain(tc_ctx *c) {
    if (c) c->refs.fetch_add(1);
}

void ctx_release(tc_ctx *c) {
    if (!c || c->refs.fetch_sub(1) != 1) return;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (auto &e : c->ev)
        if (e) cudaEventDestroy(e);
    for (auto &e : c->kev)
        if (e) cudaEventDestroy(e);
    if (c->h_pinned) cudaFreeHost(c->h_pinned);
    for (auto &q : c->aux)
        if (q) {
            cudaStreamSynchronize(q);
            cudaStreamDestroy(q);
        }
    if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

int scratch_alloc(CountScratch *sc, int64_t V, int64_t E, int64_t heavy_cap, cudaStream_t s) {
    // in-list offsets and slots are int32 over the launch's pooled edges
    if (E >= INT32_MAX)
        return set_error(TC_E_RANGE,
                         "one count launch holds fewer than 2^31 - 1 oriented edges in total, got %lld: split the "
                         "batch",
                         (long long)E);
    sc->heavy_cap = heavy_cap;
    TC_TRY(dalloc((void **)&sc->heavy, sizeof(HeavyEntry) * (size_t)std::max<int64_t>(heavy_cap, 1), s));
    TC_TRY(dalloc((void **)&sc->light_list, sizeof(uint32_t) * (size_t)std::max<int64_t>(V, 1), s));
    TC_TRY(dalloc((void **)&sc->in_cnt, sizeof(int32_t) * (size_t)std::max<int64_t>(V, 1), s));
    TC_TRY(dalloc((void **)&sc->in_off, sizeof(int32_t) * (size_t)(V + 1), s));
    TC_TRY(dalloc((void **)&sc->in_work, sizeof(unsigned long long) * (size_t)std::max<int64_t>(V, 1), s));
    TC_TRY(dalloc((void **)&sc->out_work, sizeof(unsigned long long) * (size_t)std::max<int64_t>(V, 1), s));
    TC_TRY(dalloc((void **)&sc->in_list, sizeof(int32_t) * (size_t)std::max<int64_t>(E, 1), s));
    TC_TRY(dalloc((void **)&sc->mid, (size_t)std::max<int64_t>(E, 1), s));
    return TC_OK;
}

void scratch_free(CountScratch *sc, cudaStream_t s) {
    dfree(sc->heavy, s);
    dfree(sc->light_list, s);
    dfree(sc->in_cnt, s);
    dfree(sc->in_off, s);
    dfree(sc->in_work, s);
    dfree(sc->out_work, s);
    dfree(sc->in_list, s);
    dfree(sc->mid, s);
    *sc = CountScratch();
}

int graph_rebind(tc_graph *g, tc_ctx *ctx) {
    if (!g || !ctx) return set_error(TC_E_INVALID, "null argument");
    if (g->ctx == ctx) return TC_OK;
    if (g->ctx->device != ctx->device) return set_error(TC_E_INVALID, "graphs move only between contexts of one device");
    TC_CUDA(cudaStreamSynchronize(g->ctx->stream));
    ctx_retain(ctx);
    tc_ctx *old = g->ctx;
    g->ctx = ctx;
    g->desc_valid = false;
    if (g->exec) {  // the captured chain records the old context's events
        cudaGraphExecDestroy(g->exec);
        g->exec = nullptr;
    }
    ctx_release(old);
    return TC_OK;
}

size_t graph_device_bytes(const tc_graph *g) {
    const size_t csr = sizeof(int32_t) * (size_t)(g->n_rows + 1 + g->nnz);
    const size_t scratch = (size_t)(g->n_rows + 1) * (4 + 4 + 8 + 8 + 4 + 16) + (size_t)g->nnz * 5 + 1024;
    return csr + scratch;
}

int count_graphs_direct(tc_ctx *ctx, tc_graph *const *graphs, int n, uint64_t *outs, int64_t timeout_ms,
                        float *kernel_ms) {
    if (!ctx || n <= 0 || !graphs || !outs) return set_error(TC_E_INVALID, "bad batch arguments");
    cudaStream_t s = ctx->stream;
    std::vector<GraphDesc> desc((size_t)n);
    int64_t chunks = 0, cap = 0, vtot = 0, etot = 0, max_rows = 0;
    bool halo_parts = false;
    for (int i = 0; i < n; ++i) {
        const tc_graph *g = graphs[i];
        if (g) max_rows = std::max(max_rows, g->n_rows);
        if (g) halo_parts = halo_parts || g->n_roots < g->n_rows;
        if (!g || g->ctx->device != ctx->device) return set_error(TC_E_INVALID, "graph %d is null or on another device", i);
        memset(&desc[(size_t)i], 0, sizeof(GraphDesc));
        desc[(size_t)i].rp = g->rp;
        desc[(size_t)i].col = g->col;
        desc[(size_t)i].n_rows = g->n_rows;
        desc[(size_t)i].n_roots = g->n_roots;
        desc[(size_t)i].chunk_base = chunks;
        desc[(size_t)i].vbase = vtot;
        desc[(size_t)i].ebase = etot;
        chunks += (g->n_rows + 31) / 32;
        vtot += g->n_rows + 1;
        etot += g->nnz;
        cap += std::min(g->n_rows, g->nnz) + 1;
    }
    CountScratch sc;
    DBuf<GraphDesc> d_desc;
    DBuf<unsigned char> d_work;
    const size_t out_bytes = sizeof(CountWork) + sizeof(unsigned long long) * (size_t)n;
    // the read-back must go to page-locked memory: a copy into pageable memory
    // blocks the host until the launch finishes, which would defeat the bounded wait
    unsigned char *h_out = (unsigned char *)ctx->h_pinned;
    unsigned char *h_own = nullptr;
    if (out_bytes > 4096) {
        if (cudaMallocHost(&h_own, out_bytes) != cudaSuccess) return set_error(TC_E_NOMEM, "pinned result buffer");
        h_out = h_own;
    }
    int st = d_desc.alloc((size_t)n, s);
    if (st == TC_OK) st = d_work.alloc(out_bytes, s);
    if (st == TC_OK) st = scratch_alloc(&sc, vtot, etot, cap, s);
    if (st == TC_OK && cudaMemcpyAsync(d_desc.p, desc.data(), sizeof(GraphDesc) * (size_t)n, cudaMemcpyHostToDevice,
                                       s) != cudaSuccess)
        st = set_error(TC_E_CUDA, "descriptor upload failed");
    if (st == TC_OK && cudaEventRecord(ctx->ev[0], s) != cudaSuccess) st = set_error(TC_E_CUDA, "event record failed");
    if (st == TC_OK)
        st = launch_count(d_desc.p, n, chunks, vtot, max_rows, sc, (CountWork *)d_work.p,
                          (unsigned long long *)(d_work.p + sizeof(CountWork)), false, ctx->tuned, s, nullptr, nullptr,
                          halo_parts);
    if (st == TC_OK && cudaEventRecord(ctx->ev[1], s) != cudaSuccess) st = set_error(TC_E_CUDA, "event record failed");
    if (st == TC_OK && cudaMemcpyAsync(h_out, d_work.p, out_bytes, cudaMemcpyDeviceToHost, s) != cudaSuccess)
        st = set_error(TC_E_CUDA, "result read-back failed");
    if (st == TC_OK && cudaEventRecord(ctx->ev[2], s) != cudaSuccess) st = set_error(TC_E_CUDA, "event record failed");
    if (st == TC_OK) {
        // bounded host wait on the launch: poll the event, give up after timeout_ms
        const auto t0 = std::chrono::steady_clock::now();
        for (;;) {
            const cudaError_t q = cudaEventQuery(ctx->ev[2]);
            if (q == cudaSuccess) break;
            if (q != cudaErrorNotReady) {
                st = cuda_error(q, "batched count", __FILE__, __LINE__);
                break;
            }
            if (timeout_ms > 0 && std::chrono::steady_clock::now() - t0 > std::chrono::milliseconds(timeout_ms)) {
                // the buffers must outlive the launch still in flight: leak them
                d_desc.release();
                d_work.release();
                sc = CountScratch();
                // h_own too (the read-back may still land in it); the context's
                // own pinned area is freed only after its stream has drained
                return set_error(TC_E_TIMEOUT, "batched count of %d graphs did not finish in %lld ms", n,
                                 (long long)timeout_ms);
            }
            std::this_thread::sleep_for(std::chrono::microseconds(50));
        }
    }
    if (st == TC_OK) {
        const CountWork *w = (const CountWork *)h_out;
        if (w->error) st = set_error(TC_E_STATE, "%s", count_error_text(w->error));
        else memcpy(outs, h_out + sizeof(CountWork), sizeof(uint64_t) * (size_t)n);
        if (kernel_ms) cudaEventElapsedTime(kernel_ms, ctx->ev[0], ctx->ev[1]);
    }
    scratch_free(&sc, s);
    if (h_own) cudaFreeHost(h_own);
    return st;
}

int device_sm_count(int device) {
    int sm = 0;
    cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, device);
    return sm;
}

int graph_adopt_device(tc_ctx *ctx, int32_t *rp, int32_t *col, int64_t n_rows, int64_t nnz, int64_t n_roots,
                       tc_graph **out) {
    tc_graph *g = nullptr;
    TC_TRY(new_graph(ctx, n_rows, nnz, n_roots, &g));
    g->rp = rp;
    g->col = col;
    g->owns = true;
    if (n_rows > 0) {  // the longest row, for the flat count
        cudaStream_t s = ctx->stream;
        DBuf<int> d;
        int h = 0;
        int st = d.alloc(1, s);
        if (st == TC_OK && cudaMemsetAsync(d.p, 0, sizeof(int), s) != cudaSuccess) st = TC_E_CUDA;
        if (st == TC_OK) {
            max_row_kernel<<<grid_for(n_rows, ctx->sm_count), 256, 0, s>>>(rp, n_rows, d.p);
            if (cudaGetLastError() != cudaSuccess || cudaMemcpyAsync(&h, d.p, sizeof(int), cudaMemcpyDeviceToHost, s) !=
                                                         cudaSuccess ||
                cudaStreamSynchronize(s) != cudaSuccess)
                st = set_error(TC_E_CUDA, "row length scan failed");
        }
        if (st != TC_OK) {
            g->owns = false;  // the caller still owns rp / col on failure
            tc_graph_destroy(g);
            return st;
        }
        g->max_deg = h;
    } else {
        g->max_deg = 0;
    }
    *out = g;
    return TC_OK;
}

}  // namespace tc

using namespace tc;

// ============================== C ABI ===========================================
extern "C" {

const char *tc_last_error(void) { return g_last_error.c_str(); }

const char *tc_status_string(int s) {
    switch (s) {
    case TC_OK: return "ok";
    case TC_E_INVALID: return "invalid argument";
    case TC_E_CUDA: return "CUDA error";
    case TC_E_NOMEM: return "out of memory";
    case TC_E_RANGE: return "value out of range";
    case TC_E_FORMAT: return "malformed input";
    case TC_E_IO: return "I/O error";
    case TC_E_NOT_READY: return "not ready";
    case TC_E_TIMEOUT: return "timed out";
    case TC_E_NO_DEVICE: return "no CUDA device";
    case TC_E_STATE: return "wrong state";
    default: return "unknown status";
    }
}

int tc_version(void) { return kVersion; }

int tc_host_alloc_pinned(size_t bytes, void **out) {
    if (!out) return set_error(TC_E_INVALID, "null output");
    *out = nullptr;
    TC_CUDA(cudaMallocHost(out, bytes ? bytes : 1));
    return TC_OK;
}

int tc_host_free_pinned(void *p) {
    if (p) TC_CUDA(cudaFreeHost(p));
    return TC_OK;
}

int tc_ctx_create(int device, tc_ctx **out) {
    if (!out) return set_error(TC_E_INVALID, "null output");
    g_last_error.clear();
    *out = nullptr;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) return set_error(TC_E_NO_DEVICE, "no CUDA device available");
    if (device < 0 || device >= n) return set_error(TC_E_NO_DEVICE, "device %d out of range [0, %d)", device, n);
    TC_CUDA(cudaSetDevice(device));
    cudaMemPool_t pool;
    TC_CUDA(cudaDeviceGetDefaultMemPool(&pool, device));
    uint64_t thr = UINT64_MAX;
    TC_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr));
    tc_ctx *c = new tc_ctx();
    c->device = device;
    c->sm_count = device_sm_count(device);
    c->tuning.warp_max_deg = 256;
    c->tuning.light_max_work = 8192;
    c->tuning.unit_work = 1048576;
    c->tuning.long_list = 32;
    c->tuning.probe_kicks = 32;
    c->tuning.heavy_bitmap = 0;  // an autotuner candidate: one 32-warp block per SM rarely pays off
    c->tuning.blocks_per_sm = 0;
    c->tuning.hash_pairs = 0;
    c->tuning.flat_max_deg = 8;
    c->tuning.intersect = 0;
    int st = TC_OK;
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) st = TC_E_CUDA;
    c->own_stream = true;
    for (int i = 0; i < 4 && st == TC_OK; ++i)
        if (cudaEventCreate(&c->ev[i]) != cudaSuccess) st = TC_E_CUDA;
    for (int i = 0; i < 2 && st == TC_OK; ++i)
        if (cudaEventCreate(&c->kev[i]) != cudaSuccess) st = TC_E_CUDA;
    if (st == TC_OK && cudaMallocHost(&c->h_pinned, 4096) != cudaSuccess) st = TC_E_CUDA;
    if (st == TC_OK) st = resolve_tuning(c->tuning, c->sm_count, &c->tuned);
    if (st != TC_OK) {
        const std::string why = tc_last_error();
        set_error(st, "context creation failed on device %d: %s", device, why.empty() ? "CUDA error" : why.c_str());
        tc_ctx_destroy(c);
        return st;
    }
    *out = c;
    return TC_OK;
}

int tc_ctx_destroy(tc_ctx *c) {
    ctx_release(c);  // freed now, or when its last graph / batch is destroyed
    return TC_OK;
}

int tc_ctx_set_stream(tc_ctx *c, void *stream) {
    if (!c) return set_error(TC_E_INVALID, "null context");
    TC_CUDA(cudaStreamSynchronize(c->stream));
    if (c->own_stream) cudaStreamDestroy(c->stream);
    c->stream = (cudaStream_t)stream;
    c->own_stream = false;
    return TC_OK;
}

void *tc_ctx_get_stream(tc_ctx *c) { return c ? (void *)c->stream : nullptr; }

int tc_ctx_last_count_kernel_ms(tc_ctx *c, float *ms) {
    if (!c || !ms) return set_error(TC_E_INVALID, "null argument");
    if (!c->kev_recorded) return set_error(TC_E_STATE, "no count kernel launched on this context yet");
    TC_CUDA(cudaEventSynchronize(c->kev[1]));
    TC_CUDA(cudaEventElapsedTime(ms, c->kev[0], c->kev[1]));
    return TC_OK;
}

int tc_ctx_synchronize(tc_ctx *c) {
    if (!c) return set_error(TC_E_INVALID, "null context");
    TC_CUDA(cudaStreamSynchronize(c->stream));
    return TC_OK;
}

int tc_ctx_device_info(tc_ctx *c, int *sm_count, size_t *free_bytes, size_t *total_bytes) {
    if (!c) return set_error(TC_E_INVALID, "null context");
    TC_CUDA(cudaSetDevice(c->device));
    size_t f = 0, t = 0;
    TC_CUDA(cudaMemGetInfo(&f, &t));
    if (sm_count) *sm_count = c->sm_count;
    if (free_bytes) *free_bytes = f;
    if (total_bytes) *total_bytes = t;
    return TC_OK;
}

int tc_ctx_get_tuning(tc_ctx *c, tc_tuning *out) {
    if (!c || !out) return set_error(TC_E_INVALID, "null argument");
    *out = c->tuning;
    out->blocks_per_sm = c->tuned.blocks / std::max(1, c->sm_count);
    return TC_OK;
}

int tc_ctx_set_tuning(tc_ctx *c, const tc_tuning *in) {
    if (!c || !in) return set_error(TC_E_INVALID, "null argument");
    tc_tuning t = c->tuning;
    if (in->warp_max_deg > 0) t.warp_max_deg = in->warp_max_deg;
    if (in->light_max_work > 0) t.light_max_work = in->light_max_work;
    if (in->unit_work > 0) t.unit_work = in->unit_work;
    if (in->long_list >= 0) t.long_list = in->long_list;
    if (in->probe_kicks >= 0) t.probe_kicks = in->probe_kicks;
    if (in->heavy_bitmap >= 0) t.heavy_bitmap = in->heavy_bitmap;
    if (in->blocks_per_sm >= 0) t.blocks_per_sm = in->blocks_per_sm;
    if (in->hash_pairs >= 0) t.hash_pairs = in->hash_pairs;
    if (in->flat_max_deg >= 0) t.flat_max_deg = in->flat_max_deg;
    if (in->intersect >= 0) t.intersect = in->intersect;
    Tuned r;
    TC_TRY(resolve_tuning(t, c->sm_count, &r));
    c->tuning = t;
    c->tuned = r;
    ++c->tuning_epoch;
    return TC_OK;
}

int tc_graph_upload_i32(tc_ctx *ctx, const int32_t *row_ptr, const int32_t *col, int64_t n_rows, int64_t nnz,
                        int64_t n_roots, tc_graph **out) {
    if (!ctx || !row_ptr || (nnz > 0 && !col) || !out) return set_error(TC_E_INVALID, "null argument");
    *out = nullptr;
    tc_graph *g = nullptr;
    TC_TRY(new_graph(ctx, n_rows, nnz, n_roots, &g));
    cudaStream_t s = ctx->stream;
    int st = dalloc((void **)&g->rp, sizeof(int32_t) * (size_t)(n_rows + 1), s);
    if (st == TC_OK) st = dalloc((void **)&g->col, sizeof(int32_t) * (size_t)std::max<int64_t>(nnz, 1), s);
    if (st == TC_OK && cudaMemcpyAsync(g->rp, row_ptr, sizeof(int32_t) * (size_t)(n_rows + 1), cudaMemcpyHostToDevice,
                                       s) != cudaSuccess)
        st = set_error(TC_E_CUDA, "row_ptr upload failed");
    if (st == TC_OK && nnz > 0 &&
        cudaMemcpyAsync(g->col, col, sizeof(int32_t) * (size_t)nnz, cudaMemcpyHostToDevice, s) != cudaSuccess)
        st = set_error(TC_E_CUDA, "col upload failed");
    if (st == TC_OK) st = validate_csr_impl(ctx, g->rp, g->col, n_rows, nnz, &g->max_deg);
    if (st != TC_OK) {
        tc_graph_destroy(g);
        return st;
    }
    *out = g;
    return TC_OK;
}

int tc_graph_upload_u64(tc_ctx *ctx, const uint64_t *row_ptr, const uint64_t *col, int64_t n_rows, int64_t nnz,
                        int64_t n_roots, tc_graph **out) {
    if (!ctx || !row_ptr || (nnz > 0 && !col) || !out) return set_error(TC_E_INVALID, "null argument");
    *out = nullptr;
    tc_graph *g = nullptr;
    TC_TRY(new_graph(ctx, n_rows, nnz, n_roots, &g));
    cudaStream_t s = ctx->stream;
    DBuf<uint64_t> stage;
    DBuf<int> ovf;
    int st = dalloc((void **)&g->rp, sizeof(int32_t) * (size_t)(n_rows + 1), s);
    if (st == TC_OK) st = dalloc((void **)&g->col, sizeof(int32_t) * (size_t)std::max<int64_t>(nnz, 1), s);
    if (st == TC_OK) st = stage.alloc((size_t)std::max(n_rows + 1, nnz), s);
    if (st == TC_OK) st = ovf.alloc(1, s);
    if (st == TC_OK && cudaMemsetAsync(ovf.p, 0, sizeof(int), s) != cudaSuccess) st = TC_E_CUDA;
    const uint64_t *srcs[2] = {row_ptr, col};
    int32_t *dsts[2] = {g->rp, g->col};
    const int64_t ns[2] = {n_rows + 1, nnz};
    for (int k = 0; k < 2 && st == TC_OK; ++k) {
        if (ns[k] == 0) continue;
        if (cudaMemcpyAsync(stage.p, srcs[k], sizeof(uint64_t) * (size_t)ns[k], cudaMemcpyHostToDevice, s) !=
            cudaSuccess) {
            st = set_error(TC_E_CUDA, "u64 upload failed");
            break;
        }
        narrow_u64_kernel<<<grid_for(ns[k], ctx->sm_count), 256, 0, s>>>(stage.p, dsts[k], ns[k], INT32_MAX - 1,
                                                                          ovf.p);
        if (cudaGetLastError() != cudaSuccess) st = set_error(TC_E_CUDA, "narrow kernel launch failed");
    }
    int h_ovf = 0;
    if (st == TC_OK && (cudaMemcpyAsync(&h_ovf, ovf.p, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
                        cudaStreamSynchronize(s) != cudaSuccess))
        st = set_error(TC_E_CUDA, "u64 narrowing failed");
    if (st == TC_OK && h_ovf) st = set_error(TC_E_RANGE, "u64 CSR value does not fit int32");
    if (st == TC_OK) st = validate_csr_impl(ctx, g->rp, g->col, n_rows, nnz, &g->max_deg);
    if (st != TC_OK) {
        tc_graph_destroy(g);
        return st;
    }
    *out = g;
    return TC_OK;
}

int tc_graph_wrap_device_i32(tc_ctx *ctx, const int32_t *d_row_ptr, const int32_t *d_col, int64_t n_rows, int64_t nnz,
                             int64_t n_roots, tc_graph **out) {
    if (!ctx || !d_row_ptr || !out) return set_error(TC_E_INVALID, "null argument");
    tc_graph *g = nullptr;
    TC_TRY(new_graph(ctx, n_rows, nnz, n_roots, &g));
    g->rp = const_cast<int32_t *>(d_row_ptr);
    g->col = const_cast<int32_t *>(d_col);
    g->owns = false;
    *out = g;
    return TC_OK;
}

int tc_graph_info(const tc_graph *g, int64_t *n_rows, int64_t *nnz, int64_t *n_roots) {
    TC_TRY(check_graph(g));
    if (n_rows) *n_rows = g->n_rows;
    if (nnz) *nnz = g->nnz;
    if (n_roots) *n_roots = g->n_roots;
    return TC_OK;
}

int tc_graph_download_i32(tc_ctx *ctx, const tc_graph *g, int32_t *row_ptr, int32_t *col) {
    TC_TRY(check_graph(g));
    if (!ctx) ctx = g->ctx;
    if (row_ptr)
        TC_CUDA(cudaMemcpyAsync(row_ptr, g->rp, sizeof(int32_t) * (size_t)(g->n_rows + 1), cudaMemcpyDeviceToHost,
                                ctx->stream));
    if (col && g->nnz)
        TC_CUDA(cudaMemcpyAsync(col, g->col, sizeof(int32_t) * (size_t)g->nnz, cudaMemcpyDeviceToHost, ctx->stream));
    TC_CUDA(cudaStreamSynchronize(ctx->stream));
    return TC_OK;
}

int tc_graph_destroy(tc_graph *g) {
    if (!g) return TC_OK;
    cudaStream_t s = g->ctx ? g->ctx->stream : nullptr;
    if (g->owns) {
        dfree(g->rp, s);
        dfree(g->col, s);
    }
    if (g->exec) cudaGraphExecDestroy(g->exec);
    dfree(g->d_desc, s);
    dfree(g->d_work, s);
    scratch_free(&g->sc, s);
    tc_ctx *ctx = g->ctx;
    delete g;
    ctx_release(ctx);
    return TC_OK;
}

int tc_count(tc_ctx *ctx, tc_graph *g, uint64_t *out, tc_count_stats *stats) {
    TC_TRY(check_graph(g));
    if (!out) return set_error(TC_E_INVALID, "null output");
    if (!ctx) ctx = g->ctx;
    if (g->ctx != ctx) return set_error(TC_E_INVALID, "graph belongs to another context");
    cudaStream_t s = ctx->stream;
    int launches = 0;
    TC_TRY(prepare_graph_count(g, nullptr, nullptr));  // setup and any capture stay out of count_ms
    TC_CUDA(cudaEventRecord(ctx->ev[0], s));
    TC_TRY(enqueue_graph_count(g, nullptr, nullptr, &launches));
    TC_CUDA(cudaEventRecord(ctx->ev[1], s));
    TC_CUDA(cudaMemcpyAsync(ctx->h_pinned, g->d_work, sizeof(CountWork) + sizeof(unsigned long long),
                            cudaMemcpyDeviceToHost, s));
    TC_CUDA(cudaEventRecord(ctx->ev[2], s));
    TC_CUDA(cudaStreamSynchronize(s));
    const CountWork *w = (const CountWork *)ctx->h_pinned;
    if (w->error) return set_error(TC_E_STATE, "%s", count_error_text(w->error));
    *out = *(const unsigned long long *)(w + 1);
    if (stats) {
        TC_CUDA(cudaEventElapsedTime(&stats->count_ms, ctx->ev[0], ctx->ev[1]));
        TC_CUDA(cudaEventElapsedTime(&stats->finalize_ms, ctx->ev[1], ctx->ev[2]));
        stats->launches = launches;
        stats->heavy_units = (int32_t)(w->heavy_packed & 0xffffffffull);
    }
    return TC_OK;
}

int tc_count_async(tc_ctx *ctx, tc_graph *g, uint64_t *d_out) {
    TC_TRY(check_graph(g));
    if (!d_out) return set_error(TC_E_INVALID, "null output");
    if (!ctx) ctx = g->ctx;
    return enqueue_graph_count(g, nullptr, (unsigned long long *)d_out, nullptr);
}

int tc_count_per_root(tc_ctx *ctx, tc_graph *g, uint64_t *per_root, uint64_t *total) {
    TC_TRY(check_graph(g));
    if (!per_root) return set_error(TC_E_INVALID, "null output");
    if (!ctx) ctx = g->ctx;
    cudaStream_t s = ctx->stream;
    DBuf<unsigned long long> pr;
    TC_TRY(pr.alloc((size_t)std::max<int64_t>(g->n_roots, 1), s));
    TC_CUDA(cudaMemsetAsync(pr.p, 0, sizeof(unsigned long long) * (size_t)std::max<int64_t>(g->n_roots, 1), s));
    TC_TRY(enqueue_graph_count(g, pr.p, nullptr, nullptr));
    if (g->n_roots)
        TC_CUDA(cudaMemcpyAsync(per_root, pr.p, sizeof(unsigned long long) * (size_t)g->n_roots,
                                cudaMemcpyDeviceToHost, s));
    TC_CUDA(cudaMemcpyAsync(ctx->h_pinned, g->d_work, sizeof(CountWork), cudaMemcpyDeviceToHost, s));
    TC_CUDA(cudaStreamSynchronize(s));
    if (((const CountWork *)ctx->h_pinned)->error)
        return set_error(TC_E_STATE, "%s", count_error_text(((const CountWork *)ctx->h_pinned)->error));
    if (total) {
        uint64_t t = 0;
        for (int64_t u = 0; u < g->n_roots; ++u) t += per_root[u];
        *total = t;
    }
    return TC_OK;
}

int tc_count_csr_i32(tc_ctx *ctx, const int32_t *row_ptr, const int32_t *col, int64_t n_rows, int64_t nnz,
                     uint64_t *out) {
    tc_graph *g = nullptr;
    TC_TRY(tc_graph_upload_i32(ctx, row_ptr, col, n_rows, nnz, n_rows, &g));
    int st = tc_count(ctx, g, out, nullptr);
    tc_graph_destroy(g);
    return st;
}

int tc_count_each(tc_ctx *ctx, tc_graph *const *graphs, int n, uint64_t *outs) {
    if (!ctx || (n > 0 && (!graphs || !outs))) return set_error(TC_E_INVALID, "null argument");
    for (int i = 0; i < n; ++i) TC_TRY(tc_count(ctx, graphs[i], outs + i, nullptr));
    return TC_OK;
}

}  // extern "C"

// ============================== batches =========================================
struct tc_batch {
    tc_ctx *ctx = nullptr;
    int n = 0;
    std::vector<tc_graph *> graphs;
    GraphDesc *d_desc = nullptr;
    CountScratch sc{};
    CountWork *d_work = nullptr;  // followed by n results
    unsigned long long *h_out = nullptr;  // pinned: CountWork + n results
    int64_t total_chunks = 0;
    int64_t total_vertices = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t kev[2] = {nullptr, nullptr};  // around the counting kernels, recorded by every replay
    int launches = 0;                         // kernels per replay
    bool ran = false;
};

extern "C" {

int tc_batch_destroy(tc_batch *b) {
    if (!b) return TC_OK;
    cudaStream_t s = b->ctx ? b->ctx->stream : nullptr;
    if (s) cudaStreamSynchronize(s);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    for (auto &e : b->kev)
        if (e) cudaEventDestroy(e);
    dfree(b->d_desc, s);
    scratch_free(&b->sc, s);
    dfree(b->d_work, s);
    if (b->h_out) cudaFreeHost(b->h_out);
    tc_ctx *ctx = b->ctx;
    delete b;
    ctx_release(ctx);
    return TC_OK;
}

int tc_batch_create(tc_ctx *ctx, tc_graph *const *graphs, int n, tc_batch **out) {
    if (!ctx || !out || n <= 0 || !graphs) return set_error(TC_E_INVALID, "bad batch arguments");
    *out = nullptr;
    tc_batch *b = new tc_batch();
    b->ctx = ctx;
    ctx_retain(ctx);
    b->n = n;
    cudaStream_t s = ctx->stream;
    std::vector<GraphDesc> desc((size_t)n);
    int64_t chunks = 0, cap = 0, vtot = 0, etot = 0, max_rows = 0;
    bool halo_parts = false;
    for (int i = 0; i < n; ++i) {
        tc_graph *g = graphs[i];
        if (g) max_rows = std::max(max_rows, g->n_rows);
        if (g) halo_parts = halo_parts || g->n_roots < g->n_rows;
        if (!g || g->ctx != ctx) {
            tc_batch_destroy(b);
            return set_error(TC_E_INVALID, "graph %d is null or belongs to another context", i);
        }
        b->graphs.push_back(g);
        memset(&desc[i], 0, sizeof(GraphDesc));
        desc[i].rp = g->rp;
        desc[i].col = g->col;
        desc[i].n_rows = g->n_rows;
        desc[i].n_roots = g->n_roots;
        desc[i].chunk_base = chunks;
        desc[i].vbase = vtot;
        desc[i].ebase = etot;
        desc[i].per_root = nullptr;
        chunks += (g->n_rows + 31) / 32;
        vtot += g->n_rows + 1;
        etot += g->nnz;
        cap += std::min(g->n_rows, g->nnz) + 1;
    }
    b->total_chunks = chunks;
    b->total_vertices = vtot;
    int st = dalloc((void **)&b->d_desc, sizeof(GraphDesc) * (size_t)n, s);
    if (st == TC_OK) st = scratch_alloc(&b->sc, vtot, etot, cap, s);
    if (st == TC_OK) st = dalloc((void **)&b->d_work, sizeof(CountWork) + sizeof(unsigned long long) * (size_t)n, s);
    if (st == TC_OK && cudaMallocHost(&b->h_out, sizeof(CountWork) + sizeof(unsigned long long) * (size_t)n) != cudaSuccess)
        st = set_error(TC_E_NOMEM, "pinned result buffer");
    if (st == TC_OK && cudaMemcpyAsync(b->d_desc, desc.data(), sizeof(GraphDesc) * (size_t)n, cudaMemcpyHostToDevice,
                                       s) != cudaSuccess)
        st = set_error(TC_E_CUDA, "descriptor upload failed");
    if (st == TC_OK && cudaStreamSynchronize(s) != cudaSuccess) st = set_error(TC_E_CUDA, "batch setup sync failed");
    for (int i = 0; i < 2 && st == TC_OK; ++i)
        if (cudaEventCreate(&b->kev[i]) != cudaSuccess) st = set_error(TC_E_CUDA, "event creation failed");
    // capture [memset -> classify -> count] once; tc_batch_run replays it
    if (st == TC_OK && cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
        st = set_error(TC_E_CUDA, "stream capture could not start");
    if (st == TC_OK) {
        int ls = launch_count(b->d_desc, n, chunks, vtot, max_rows, b->sc, b->d_work,
                              (unsigned long long *)(b->d_work + 1), false, ctx->tuned, s, &b->launches, b->kev,
                              halo_parts);
        cudaError_t e = cudaStreamEndCapture(s, &b->graph);
        if (ls != TC_OK) st = ls;
        else if (e != cudaSuccess) st = cuda_error(e, "cudaStreamEndCapture", __FILE__, __LINE__);
    }
    if (st == TC_OK) {
        cudaError_t e = cudaGraphInstantiate(&b->exec, b->graph, 0);
        if (e != cudaSuccess) st = cuda_error(e, "cudaGraphInstantiate", __FILE__, __LINE__);
    }
    if (st != TC_OK) {
        tc_batch_destroy(b);
        return st;
    }
    *out = b;
    return TC_OK;
}

int tc_batch_run_async(tc_batch *b) {
    if (!b) return set_error(TC_E_INVALID, "null batch");
    TC_CUDA(cudaGraphLaunch(b->exec, b->ctx->stream));
    b->ran = b->total_chunks > 0;
    return TC_OK;
}

int tc_batch_stats(tc_batch *b, tc_count_stats *stats) {
    if (!b || !stats) return set_error(TC_E_INVALID, "null argument");
    memset(stats, 0, sizeof *stats);
    stats->launches = b->launches;
    if (!b->ran) return TC_OK;
    TC_CUDA(cudaEventSynchronize(b->kev[1]));
    TC_CUDA(cudaEventElapsedTime(&stats->count_ms, b->kev[0], b->kev[1]));
    CountWork w;
    TC_CUDA(cudaMemcpy(&w, b->d_work, sizeof w, cudaMemcpyDeviceToHost));
    stats->heavy_units = (int32_t)(w.heavy_packed & 0xffffffffull);
    return TC_OK;
}

}  // extern "C"

namespace {

// One pooled count launch over a group of parts, enqueued on the context's
// stream with its results in d_res[0..n); the launch's descriptor table,
// work words and scratch are freed in stream order when the group goes.
struct PartGroup {
    DBuf<GraphDesc> desc;
    DBuf<CountWork> work;
    CountScratch sc;
    cudaStream_t s = nullptr;
    ~PartGroup() {
        if (s) scratch_free(&sc, s);
    }
};

int enqueue_group_count(tc_ctx *ctx, tc_graph *const *gs, int n, unsigned long long *d_res, PartGroup *grp) {
    cudaStream_t s = ctx->stream;
    std::vector<GraphDesc> desc((size_t)n);
    int64_t chunks = 0, cap = 0, vtot = 0, etot = 0, max_rows = 0;
    bool halo_parts = false;
    for (int i = 0; i < n; ++i) {
        const tc_graph *g = gs[i];
        max_rows = std::max(max_rows, g->n_rows);
        halo_parts = halo_parts || g->n_roots < g->n_rows;
        GraphDesc &d = desc[(size_t)i];
        memset(&d, 0, sizeof d);
        d.rp = g->rp;
        d.col = g->col;
        d.n_rows = g->n_rows;
        d.n_roots = g->n_roots;
        d.chunk_base = chunks;
        d.vbase = vtot;
        d.ebase = etot;
        chunks += (g->n_rows + 31) / 32;
        vtot += g->n_rows + 1;
        etot += g->nnz;
        cap += std::min(g->n_rows, g->nnz) + 1;
    }
    grp->s = s;
    TC_TRY(grp->desc.alloc((size_t)n, s));
    TC_TRY(grp->work.alloc(1, s));
    TC_TRY(scratch_alloc(&grp->sc, vtot, etot, cap, s));
    for (int i0 = 0; i0 < n; i0 += 8) {
        DescBlock blk;
        const int m = std::min(8, n - i0);
        memcpy(blk.d, desc.data() + i0, sizeof(GraphDesc) * (size_t)m);
        set_descs_kernel<<<1, 8, 0, s>>>(grp->desc.p + i0, blk, m);
        TC_CUDA(cudaGetLastError());
    }
    return launch_count(grp->desc.p, n, chunks, vtot, max_rows, grp->sc, grp->work.p, d_res, false, ctx->tuned, s,
                        nullptr, nullptr, halo_parts);
}

}  // namespace

extern "C" {

int tc_count_parts_csr_i32(tc_ctx *ctx, int n_parts, const int32_t *const *row_ptrs, const int32_t *const *cols,
                           const int64_t *n_rows, const int64_t *nnz, const int64_t *n_roots, uint64_t *outs,
                           uint64_t *total) {
    if (!ctx || n_parts <= 0 || !row_ptrs || !cols || !n_rows || !nnz || !n_roots || !outs)
        return set_error(TC_E_INVALID, "null argument or no parts");
    for (int p = 0; p < n_parts; ++p)
        if (!row_ptrs[p] || (nnz[p] > 0 && !cols[p])) return set_error(TC_E_INVALID, "part %d: null array", p);
    // Three streams: every part's upload goes out on the copy stream at once;
    // part p is validated on the (high-priority) validation stream as soon as
    // its upload lands.  A few large parts (at most 64, 4 M entries each on
    // average; the parts of one graph) are then counted on the context's
    // stream while the later parts are still being uploaded -- the copy
    // engine and the SMs work at the same time (R-MAT 23's eight parts: 3.3 GB
    // of uploads in 16 ms under 41 ms of counts) -- in groups of 1, 2, 4, ...
    // parts, one pooled launch per group (the last group takes the rest once
    // fewer than half the next group's size would be left): part 0 starts as
    // soon as it is in, and the later groups pay one launch tail and one
    // validation gap each instead of one per part.  Many small graphs are
    // counted together in one batched launch once all are in (one launch each
    // would cost more than the copies).  The host waits only for verdicts.
    if (!ctx->aux[0]) {
        int lo = 0, hi = 0;
        TC_CUDA(cudaDeviceGetStreamPriorityRange(&lo, &hi));
        TC_CUDA(cudaStreamCreateWithFlags(&ctx->aux[0], cudaStreamNonBlocking));
        TC_CUDA(cudaStreamCreateWithPriority(&ctx->aux[1], cudaStreamNonBlocking, hi));
    }
    // (one copy stream already runs the link at its rate, 211 GB/s here, and
    // lands the parts in order; four streams did not speed up even the
    // 256-graph batch's 512 small copies)
    cudaStream_t S = ctx->stream, Cs = ctx->aux[0], Vs = ctx->aux[1];
    std::vector<tc_graph *> gs((size_t)n_parts, nullptr);
    std::vector<cudaEvent_t> copied((size_t)n_parts, nullptr);
    DBuf<unsigned long long> d_res;
    DBuf<ValidateErr> d_err;
    DBuf<uint8_t> start;
    int64_t max_nnz = 0, sum_nnz = 0;
    for (int p = 0; p < n_parts; ++p) {
        max_nnz = std::max(max_nnz, nnz[p]);
        sum_nnz += nnz[p];
    }
    const bool overlap = n_parts <= 64 && sum_nnz / n_parts >= ((int64_t)1 << 22);
    std::vector<int> group_end;  // exclusive ends of the overlapped groups
    for (int a = 0, sz = 1; overlap && a < n_parts; a = group_end.back(), sz *= 2) {
        int b = std::min(n_parts, a + sz);
        if (n_parts - b < sz) b = n_parts;
        group_end.push_back(b);
    }
    std::vector<std::unique_ptr<PartGroup>> groups;
    size_t next_group = 0;
    int group_start = 0;
    int st = d_res.alloc((size_t)n_parts, S);
    if (st == TC_OK && cudaMemsetAsync(d_res.p, 0, sizeof(unsigned long long) * (size_t)n_parts, S) != cudaSuccess)
        st = set_error(TC_E_CUDA, "result memset failed");
    if (st == TC_OK) st = d_err.alloc(overlap ? 1 : (size_t)n_parts, Vs);
    if (st == TC_OK) st = start.alloc((size_t)max_nnz + 1, Vs);
    for (int p = 0; p < n_parts && st == TC_OK; ++p) {  // every upload, back to back
        tc_graph *g = nullptr;
        st = new_graph(ctx, n_rows[p], nnz[p], n_roots[p], &g);
        if (st != TC_OK) break;
        gs[(size_t)p] = g;
        st = dalloc((void **)&g->rp, sizeof(int32_t) * (size_t)(n_rows[p] + 1), Cs);
        if (st == TC_OK) st = dalloc((void **)&g->col, sizeof(int32_t) * (size_t)std::max<int64_t>(nnz[p], 1), Cs);
        if (st == TC_OK && cudaMemcpyAsync(g->rp, row_ptrs[p], sizeof(int32_t) * (size_t)(n_rows[p] + 1),
                                           cudaMemcpyHostToDevice, Cs) != cudaSuccess)
            st = set_error(TC_E_CUDA, "part %d: row_ptr upload failed", p);
        if (st == TC_OK && nnz[p] > 0 &&
            cudaMemcpyAsync(g->col, cols[p], sizeof(int32_t) * (size_t)nnz[p], cudaMemcpyHostToDevice, Cs) !=
                cudaSuccess)
            st = set_error(TC_E_CUDA, "part %d: col upload failed", p);
        if (st == TC_OK && (cudaEventCreateWithFlags(&copied[(size_t)p], cudaEventDisableTiming) != cudaSuccess ||
                            cudaEventRecord(copied[(size_t)p], Cs) != cudaSuccess))
            st = set_error(TC_E_CUDA, "part %d: event failed", p);
    }
    if (st == TC_OK && !overlap) {
        // many small graphs: every validation enqueued back to back, each
        // verdict in its own word, then one read-back of all verdicts (a host
        // sync per graph cost the 256-graph batch ~10 ms)
        for (int p = 0; p < n_parts && st == TC_OK; ++p) {
            tc_graph *g = gs[(size_t)p];
            if (cudaStreamWaitEvent(Vs, copied[(size_t)p], 0) != cudaSuccess)
                st = set_error(TC_E_CUDA, "event wait failed");
            if (st == TC_OK)
                st = validate_csr_enqueue(ctx, Vs, g->rp, g->col, n_rows[p], nnz[p], start.p, d_err.p + p);
        }
        std::vector<ValidateErr> hv((size_t)n_parts);
        if (st == TC_OK && (cudaMemcpyAsync(hv.data(), d_err.p, sizeof(ValidateErr) * (size_t)n_parts,
                                            cudaMemcpyDeviceToHost, Vs) != cudaSuccess ||
                            cudaStreamSynchronize(Vs) != cudaSuccess))
            st = set_error(TC_E_CUDA, "validation failed to run");
        for (int p = 0; p < n_parts && st == TC_OK; ++p) {
            st = validate_verdict(hv[(size_t)p], n_rows[p], nnz[p], &gs[(size_t)p]->max_deg);
            if (st != TC_OK) set_error(st, "part %d: %s", p, std::string(tc_last_error()).c_str());
            else if (cudaStreamWaitEvent(S, copied[(size_t)p], 0) != cudaSuccess)
                st = set_error(TC_E_CUDA, "event wait failed");
        }
    }
    for (int p = 0; p < n_parts && st == TC_OK && overlap; ++p) {  // validate, then count, part by part
        tc_graph *g = gs[(size_t)p];
        ValidateErr h;
        if (cudaStreamWaitEvent(Vs, copied[(size_t)p], 0) != cudaSuccess) st = set_error(TC_E_CUDA, "event wait failed");
        if (st == TC_OK) st = validate_csr_enqueue(ctx, Vs, g->rp, g->col, n_rows[p], nnz[p], start.p, d_err.p);
        if (st == TC_OK && (cudaMemcpyAsync(&h, d_err.p, sizeof h, cudaMemcpyDeviceToHost, Vs) != cudaSuccess ||
                            cudaStreamSynchronize(Vs) != cudaSuccess))
            st = set_error(TC_E_CUDA, "part %d: validation failed to run", p);
        if (st == TC_OK) st = validate_verdict(h, n_rows[p], nnz[p], &g->max_deg);
        if (st != TC_OK) {
            set_error(st, "part %d: %s", p, std::string(tc_last_error()).c_str());
            break;
        }
        if (cudaStreamWaitEvent(S, copied[(size_t)p], 0) != cudaSuccess) st = set_error(TC_E_CUDA, "event wait failed");
        if (st == TC_OK && p + 1 == group_end[next_group]) {  // the group is in and valid
            if (p == group_start) {
                st = enqueue_graph_count(g, nullptr, d_res.p + p, nullptr);
            } else {
                groups.push_back(std::make_unique<PartGroup>());
                st = enqueue_group_count(ctx, gs.data() + group_start, p + 1 - group_start, d_res.p + group_start,
                                         groups.back().get());
            }
            group_start = p + 1;
            ++next_group;
        }
    }
    std::vector<unsigned long long> h_res((size_t)n_parts, 0);
    int bad = 0;
    if (st == TC_OK && !overlap) {  // all uploaded and valid: one batched launch
        std::vector<uint64_t> o((size_t)n_parts);
        st = count_graphs_direct(ctx, gs.data(), n_parts, o.data(), 0, nullptr);
        for (int p = 0; p < n_parts && st == TC_OK; ++p) h_res[(size_t)p] = o[(size_t)p];
    } else if (st == TC_OK) {
        if (cudaMemcpyAsync(h_res.data(), d_res.p, sizeof(unsigned long long) * (size_t)n_parts,
                            cudaMemcpyDeviceToHost, S) != cudaSuccess)
            st = set_error(TC_E_CUDA, "result read-back failed");
    }
    // every stream drained before the parts' memory goes back to the pool
    cudaStreamSynchronize(Cs);
    cudaStreamSynchronize(Vs);
    if (cudaStreamSynchronize(S) != cudaSuccess && st == TC_OK) st = set_error(TC_E_CUDA, "parts count failed");
    for (int p = 0; p < n_parts && st == TC_OK && overlap; ++p) {  // parts counted on their own
        tc_graph *g = gs[(size_t)p];
        if (g->d_work) {
            CountWork w;
            if (cudaMemcpy(&w, g->d_work, sizeof w, cudaMemcpyDeviceToHost) != cudaSuccess) bad = -1;
            else if (w.error) bad = w.error;
        }
    }
    for (size_t i = 0; i < groups.size() && st == TC_OK; ++i) {  // the pooled launches
        CountWork w;
        if (cudaMemcpy(&w, groups[i]->work.p, sizeof w, cudaMemcpyDeviceToHost) != cudaSuccess) bad = -1;
        else if (w.error) bad = w.error;
    }
    groups.clear();
    if (st == TC_OK && bad > 0) st = set_error(TC_E_STATE, "%s", count_error_text(bad));
    if (st == TC_OK && bad < 0) st = set_error(TC_E_CUDA, "work word read-back failed");
    for (auto &e : copied)
        if (e) cudaEventDestroy(e);
    for (tc_graph *g : gs) tc_graph_destroy(g);
    if (st != TC_OK) return st;
    uint64_t t = 0;
    for (int p = 0; p < n_parts; ++p) {
        outs[p] = h_res[(size_t)p];
        t += outs[p];
    }
    if (total) *total = t;
    return TC_OK;
}

int tc_batch_results(tc_batch *b, uint64_t *outs) {
    if (!b || !outs) return set_error(TC_E_INVALID, "null argument");
    cudaStream_t s = b->ctx->stream;
    TC_CUDA(cudaMemcpyAsync(b->h_out, b->d_work, sizeof(CountWork) + sizeof(unsigned long long) * (size_t)b->n,
                            cudaMemcpyDeviceToHost, s));
    TC_CUDA(cudaStreamSynchronize(s));
    const CountWork *w = (const CountWork *)b->h_out;
    if (w->error) return set_error(TC_E_STATE, "%s", count_error_text(w->error));
    memcpy(outs, (const void *)(w + 1), sizeof(uint64_t) * (size_t)b->n);
    return TC_OK;
}

int tc_batch_run(tc_batch *b, uint64_t *outs) {
    TC_TRY(tc_batch_run_async(b));
    return tc_batch_results(b, outs);
}

}  // extern "C"
