// tc_internal.h -- shared declarations of libtc's translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <string>

#include "tc.h"

namespace tc {

// ---- errors ------------------------------------------------------------------
// Records a message for tc_last_error() on the calling thread; returns status.
int set_error(int status, const char *fmt, ...) __attribute__((format(printf, 2, 3)));
int cuda_error(cudaError_t e, const char *what, const char *file, int line);

#define TC_CUDA(call)                                                                 \
    do {                                                                              \
        cudaError_t tc_e_ = (call);                                                   \
        if (tc_e_ != cudaSuccess) return ::tc::cuda_error(tc_e_, #call, __FILE__, __LINE__); \
    } while (0)

#define TC_TRY(call)                    \
    do {                                \
        int tc_s_ = (call);             \
        if (tc_s_ != TC_OK) return tc_s_; \
    } while (0)

// ---- device scratch ------------------------------------------------------------
// Stream-ordered allocation from the device's default memory pool (its release
// threshold is raised at context creation, so freed blocks stay cached and a
// steady-state call does not reach the driver allocator).
int dalloc(void **p, size_t bytes, cudaStream_t s);
void dfree(void *p, cudaStream_t s);

template <class T>
struct DBuf {
    T *p = nullptr;
    size_t n = 0;
    cudaStream_t s = nullptr;
    DBuf() = default;
    DBuf(const DBuf &) = delete;
    DBuf &operator=(const DBuf &) = delete;
    ~DBuf() { reset(); }
    int alloc(size_t count, cudaStream_t stream) {
        reset();
        s = stream;
        n = count;
        return dalloc((void **)&p, (count ? count : 1) * sizeof(T), stream);
    }
    void reset() {
        if (p) dfree(p, s);
        p = nullptr;
        n = 0;
    }
    T *release() {
        T *q = p;
        p = nullptr;
        n = 0;
        return q;
    }
};

// ---- counting kernels (tc_count.cu) ----------------------------------------------
struct GraphDesc {
    const int32_t *rp;
    const int32_t *col;
    int64_t n_rows;
    int64_t n_roots;
    int64_t chunk_base;           // exclusive prefix of 32-row chunks over graphs
    int64_t vbase;                // exclusive prefix of (n_rows + 1) over graphs
    int64_t ebase;                // exclusive prefix of nnz over graphs
    unsigned long long *per_root; // optional g_sum output (zeroed by the caller)
};

struct HeavyEntry {
    int32_t g, u, unit_base, n_slices;  // units = ceil(d+(u) / tile) * n_slices
};

// Device arrays of one count launch, sized for its graphs (pooled over a batch):
// V = sum (n_rows + 1), C = sum ceil(n_rows / 32), E = sum nnz.
struct CountScratch {
    HeavyEntry *heavy = nullptr;  // heavy_cap entries
    int64_t heavy_cap = 0;
    uint32_t *light_list = nullptr;         // V: light tasks from entry 0 up, micro tasks from entry V - 1
                                            // down, as global rows chunk * 32 + lane
    int32_t *in_cnt = nullptr;              // V
    int32_t *in_off = nullptr;              // V + 1
    unsigned long long *in_work = nullptr;  // V
    unsigned long long *out_work = nullptr; // V
    int32_t *in_list = nullptr;             // E
    uint8_t *mid = nullptr;                 // E: edge done middle-centric
};
int scratch_alloc(CountScratch *sc, int64_t V, int64_t E, int64_t heavy_cap, cudaStream_t s);
void scratch_free(CountScratch *sc, cudaStream_t s);

// Per-launch device words, zeroed by one memset before each count.
struct CountWork {
    unsigned long long heavy_packed; // (entries << 32) | units, from the classifier
    unsigned int heavy_cursor;
    unsigned int small_cursor;       // light-task cursor
    unsigned int aux_cursor[2];      // chunk cursors of in_count, transpose/classify
    int error;                       // 1: heavy-unit list overflow; 2: a bulk-copy staging wait gave up
    unsigned long long total_work;   // sum over oriented edges of the cheaper side's length
    unsigned long long n_tasks;      // tasks listed by the classifier, one atomic per chunk for both
                                     // lists: light (low half, task list from the bottom) and micro
                                     // (high half, from the top)
};

struct Tuned {  // resolved tc_tuning with derived table geometry
    int warp_max;        // power of two
    int log_warp_slots;
    int light_max_work;
    int unit_work;
    int long_list;
    int probe_kicks;     // 0: linear-probing hash; > 0: cuckoo hash with this kick bound
    int heavy_bitmap;    // 1: heavy units on direct-address bitmaps when the ids fit
    int hash_pairs;      // 1: bucketed-pair hash tables (one 8-byte load per probe)
    int flat_max_deg;    // graphs whose rows are all this short count with flat_kernel (0: never)
    int intersect;       // 0: hash tables; 1: bulk-staged sorted lists; 2: per light task by its work
    int bitmap_bytes;    // shared memory the bitmap kernel may use (ids < 8 x this)
    int sm_count;
    int tile;            // block table entries per tile (a quarter of its slots)
    int log_block_slots;
    int threads;         // per block
    int blocks;          // persistent grid
    int aux_blocks;      // resident grid of the per-chunk auxiliary kernels
    size_t smem;         // dynamic shared memory bytes
};

int resolve_tuning(const tc_tuning &t, int sm_count, Tuned *out);

// launch_count for callers that cannot allocate: the in-edge scan keeps its
// tile sums in scan_tmp (scan_tmp_cap values); nothing is allocated.
int launch_count_noalloc(const GraphDesc *d_desc, int64_t total_chunks, int64_t total_vertices,
                         const CountScratch &sc, int32_t *scan_tmp, int64_t scan_tmp_cap, CountWork *work,
                         unsigned long long *results, const Tuned &tn, cudaStream_t s);

// One-kernel count of a graph whose rows are all at most max_deg <= 8 long
// (one lane per root, lists in registers); fills the work words and result
// like launch_count.
int launch_flat(const int32_t *rp, const int32_t *col, int64_t n_roots, int max_deg, CountWork *work,
                unsigned long long *result, unsigned long long *per_root, const Tuned &tn, cudaStream_t s,
                int *launches, cudaEvent_t *kev);

// Enqueues [degree -> in_count -> scan -> transpose/classify -> micro ->
// count] for n_graphs descriptors on stream s; results[n_graphs] receives the
// per-graph totals (zeroed here); total_vertices = sum (n_rows + 1), max_rows
// = the largest n_rows.  kev (optional, two events) is recorded around the
// counting kernels (heavy bitmap + persistent count).  halo_parts: some graph
// of the launch is a halo part (n_roots < n_rows); its heavy units then run
// the count kernel's instance for small units.
int launch_count(const GraphDesc *d_desc, int n_graphs, int64_t total_chunks, int64_t total_vertices,
                 int64_t max_rows, const CountScratch &sc, CountWork *work, unsigned long long *results, bool per_root,
                 const Tuned &tn, cudaStream_t s, int *launches, cudaEvent_t *kev = nullptr,
                 bool halo_parts = false);

// ---- scans and sort (tc_scan.cu, tc_sort.cu) ----------------------------------------
// Exclusive scan of n values into out[0..n] (out[n] = total).  out may alias in.
int scan_exclusive_i32(const int32_t *in, int32_t *out, int64_t n, cudaStream_t s);
int scan_exclusive_i64(const int64_t *in, int64_t *out, int64_t n, cudaStream_t s);
// Exclusive scan of 0/1 byte flags into int32 positions out[0..n].
int scan_flags_u8(const uint8_t *flags, int32_t *out, int64_t n, cudaStream_t s);
// scan_exclusive_i32 with its tile sums in caller memory (no allocation).
int scan_exclusive_i32_tmp(const int32_t *in, int32_t *out, int64_t n, int32_t *tmp, int64_t tmp_cap,
                           cudaStream_t s);
// The count's in-list offsets: in_off[0..n] = exclusive scan of the in-edge
// counts held in the high halves of in_work[0..n), and each in_work[i]'s high
// half becomes in_off[i] + count, the end of vertex i's in-list.  The tile
// sums go to tmp (tmp_cap values), or to a stream-ordered allocation when tmp
// is null.
int scan_in_slots(unsigned long long *in_work, int32_t *in_off, int64_t n, int32_t *tmp, int64_t tmp_cap,
                  cudaStream_t s);
// LSD radix sort of n 64-bit keys on bits [0, bits).  Result in *keys (the
// two buffers may be swapped).  tmp must hold n keys.
int radix_sort_u64(uint64_t **keys, uint64_t **tmp, int64_t n, int bits, cudaStream_t s);

int device_sm_count(int device);

// Counts n graphs (same device) with one batched launch on ctx's stream and
// waits up to timeout_ms for the results (TC_E_TIMEOUT after that; the
// launch is then still in flight).  Scratch comes from the stream-ordered pool.
int count_graphs_direct(tc_ctx *ctx, tc_graph *const *graphs, int n, uint64_t *outs, int64_t timeout_ms,
                        float *kernel_ms);
// Moves a graph to another context of the same device (reference counts follow).
int graph_rebind(tc_graph *g, tc_ctx *ctx);
// Device bytes held by a graph (CSR + count scratch once sized).
size_t graph_device_bytes(const tc_graph *g);

// Context lifetime: every graph, ugraph and batch holds a reference to its
// context, so tc_ctx_destroy only drops the caller's reference and the
// context is freed when its last object is destroyed.
void ctx_retain(tc_ctx *c);
void ctx_release(tc_ctx *c);

}  // namespace tc

// ---- library object layouts ----------------------------------------------------------
struct tc_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int sm_count = 0;
    tc_tuning tuning{};
    tc::Tuned tuned{};
    unsigned long long tuning_epoch = 0;  // bumped by every tuning change (cached count graphs go stale)
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    cudaEvent_t kev[2] = {nullptr, nullptr};  // around the last count kernel launch
    bool kev_recorded = false;
    unsigned long long *h_pinned = nullptr;  // small pinned read-back area
    // created on first use by tc_count_parts_csr_i32: a copy stream and a
    // high-priority validation stream, so uploads overlap the counts
    cudaStream_t aux[2] = {nullptr, nullptr};
    std::atomic<int> refs{1};                // the handle + one per live object
};

struct tc_graph {
    tc_ctx *ctx = nullptr;
    int32_t *rp = nullptr;
    int32_t *col = nullptr;
    int64_t n_rows = 0, nnz = 0, n_roots = 0;
    int32_t max_deg = -1;  // longest row, when known (uploads and device-built graphs)
    bool owns = true;
    // per-graph count scratch, sized on first use
    tc::GraphDesc *d_desc = nullptr;
    tc::CountWork *d_work = nullptr;
    unsigned long long *d_result = nullptr;
    tc::CountScratch sc{};
    tc::GraphDesc desc_on_device{};  // what d_desc holds (skip re-uploads)
    bool desc_valid = false;
    // The count chain captured as a CUDA graph on the graph's second count and
    // replayed after that (one launch instead of ~10 stream operations), while
    // the results pointer and the context's tuning stay the same; a results
    // pointer is captured once two counts in a row used it.
    cudaGraphExec_t exec = nullptr;
    unsigned long long *exec_results = nullptr;
    unsigned long long *last_results = nullptr;  // results pointer of the previous chain count
    unsigned long long exec_epoch = 0;
    int exec_launches = 0;
    int chain_counts = 0;  // chain counts enqueued so far
};

struct tc_ugraph {
    tc_ctx *ctx = nullptr;
    int32_t *rp = nullptr;
    int32_t *col = nullptr;
    int32_t *deg = nullptr;    // degree used for orientation
    int32_t *rowid = nullptr;  // row of each entry (nnz)
    int64_t n_rows = 0, nnz = 0;
};
