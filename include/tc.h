/*
 * tc.h -- C ABI of libtc, the GB300 (sm_103a) exact triangle-counting engine.
 *
 * The reference (KishantLab/TriangleCount) has no library API: its boundary is
 * the command line and the whitespace-separated text formats of TC_128,
 * wo_sort_tc_256 and round_clean_sg.  libtc keeps that contract in its CLIs
 * and exposes the stages below as plain C entry points (plain pointers and
 * sizes, no C++ or torch types) so that a cgo / JNI / ctypes binding can call
 * them directly.  Each declaration names the reference code it replaces.
 *
 * Conventions
 *  - Every function returns an int status: TC_OK (0) or a negative TC_E_*.
 *    tc_last_error() gives a message for the calling thread's last failure.
 *  - Host pointers are read during the call only; the caller keeps ownership.
 *  - Library objects (contexts, graphs, batches, servers) are opaque handles
 *    created and destroyed through this API.
 *  - Device work of one context is ordered on that context's stream.  Calls
 *    on distinct contexts may run from distinct host threads.
 *  - Counts are exact unsigned 64-bit integers.
 */
#ifndef TC_H
#define TC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define TC_API __attribute__((visibility("default")))
#else
#define TC_API
#endif

/* ---- status codes --------------------------------------------------------- */
#define TC_OK 0
#define TC_E_INVALID (-1)   /* bad argument or handle */
#define TC_E_CUDA (-2)      /* CUDA runtime error */
#define TC_E_NOMEM (-3)     /* host/device allocation failed or over budget */
#define TC_E_RANGE (-4)     /* value does not fit the device index type */
#define TC_E_FORMAT (-5)    /* malformed file or CSR (unsorted row, bad id) */
#define TC_E_IO (-6)        /* file cannot be opened, read or written */
#define TC_E_NOT_READY (-7) /* asynchronous result not available yet */
#define TC_E_TIMEOUT (-8)   /* bounded wait expired */
#define TC_E_NO_DEVICE (-9) /* no CUDA device / device index out of range */
#define TC_E_STATE (-10)    /* object is in the wrong state for the call */

/* Orientation tie-break for vertices of equal degree.
 * TC_TIE_REFERENCE keeps u->w iff deg u < deg w, or deg u == deg w and w < u
 *   (Med_dataset/without_part_preprocess.py:37-50, round_clean_subgraph.cu:180-201).
 * TC_TIE_ID_ASC keeps u->w iff (deg u, u) < (deg w, w).
 * Both orient every edge once; counts are identical, files differ. */
#define TC_TIE_REFERENCE 0
#define TC_TIE_ID_ASC 1

typedef struct tc_ctx tc_ctx;       /* device + stream + scratch pool */
typedef struct tc_graph tc_graph;   /* device-resident oriented CSR, int32 */
typedef struct tc_ugraph tc_ugraph; /* device-resident undirected CSR, int32 */
typedef struct tc_batch tc_batch;   /* many graphs, one persistent launch */
typedef struct tc_server tc_server; /* continuous-batching request loop */

/* ---- errors, version ------------------------------------------------------ */
/* Replaces the reference's printf + exit(0) on failure
 * (ShareKernelTCV62_update_v1.cu:200-203, without_sorting_tc.cu:234-238). */
TC_API const char *tc_last_error(void);
TC_API const char *tc_status_string(int status);
TC_API int tc_version(void); /* major*10000 + minor*100 + patch */

/* ---- context -------------------------------------------------------------- */
/* Replaces cudaSetDevice(0) and the default stream of the reference drivers
 * (without_sorting_tc.cu:226).  The context owns a non-blocking stream and a
 * device scratch pool reused across calls (the reference cudaMallocs inside
 * its timed loop, ShareKernelTCV62_update_v1.cu:254-261, 271-275). */
TC_API int tc_ctx_create(int device, tc_ctx **out);
TC_API int tc_ctx_destroy(tc_ctx *ctx);
/* Use an external cudaStream_t (passed as void*) instead of the own stream. */
TC_API int tc_ctx_set_stream(tc_ctx *ctx, void *cuda_stream);
TC_API void *tc_ctx_get_stream(tc_ctx *ctx);
TC_API int tc_ctx_synchronize(tc_ctx *ctx);
/* Device time of the count kernel alone (the persistent counting launch, not
 * the classification passes) of the last single-graph count on this context;
 * waits for it to finish. */
TC_API int tc_ctx_last_count_kernel_ms(tc_ctx *ctx, float *ms);
TC_API int tc_ctx_device_info(tc_ctx *ctx, int *sm_count, size_t *free_bytes, size_t *total_bytes);

/* Strategy thresholds of the counting kernel (picked by the autotuner).
 * The classifier computes, per vertex task x, d+(x) and its work (the probes
 * of its partners' lists).  Micro tasks (d+(x) <= 8, work <= 128) run on one
 * lane with N+(x) in registers.  Light tasks (d+(x) <= warp_max_deg and work
 * <= light_max_work) run on one warp with a per-warp shared-memory hash of
 * N+(x); heavy ones are split into block units of about unit_work probes over
 * a shared hash of one tile of N+(x).  light_max_work and unit_work are upper
 * bounds: on a small job both are lowered so that every warp / block gets
 * about four tasks / units (a large one would be the kernel's tail).  Per partner, lists with length >=
 * long_list are streamed by the whole warp; shorter lists are flattened
 * across the lanes.  probe_kicks > 0 selects a cuckoo hash (two fixed probe
 * slots per lookup, at most probe_kicks displacements per insertion, falling
 * back to linear probing for a task whose insertion gives up); 0 selects
 * linear probing.  heavy_bitmap = 1 runs heavy tasks on a direct-address
 * shared-memory bitmap of N+(x) (one load per probe) whenever the graphs'
 * vertex ids fit in one block's shared memory (about 1.85 M rows).
 * hash_pairs = 1 selects bucketed-pair tables instead (two slots per 8-byte
 * bucket, one hash, overflow flagged into the next bucket: nearly always one
 * shared load per lookup; never gives up).  flat_max_deg (default 8): a
 * graph none of whose rows is longer (known for uploaded and device-built
 * graphs, not for wrapped ones) is counted by one kernel, one lane per root
 * with N+(u) and each N+(v) in registers -- no transpose, no hash tables
 * (road networks and other bounded-degree graphs).  intersect selects how a
 * task's list N+(x) is probed: 0 (default) through the hash tables above;
 * 1 as the sorted list itself, copied into shared memory as it lies by one
 * bulk copy (cp.async.bulk, no table to clear or fill) and probed by binary
 * search (the reference's probe, ShareKernelTCV62_update_v1.cu:12-42), for
 * light tasks and heavy tiles alike; 2 per light task: the sorted list when
 * the task's work (probes) is below its list length, so building a table
 * would cost more than probing it, the hash otherwise (heavy tiles keep the
 * hash).  hash_pairs = 1 ignores intersect.  In
 * tc_ctx_set_tuning, fields <= 0 (long_list, probe_kicks, heavy_bitmap,
 * blocks_per_sm, hash_pairs, flat_max_deg, intersect: < 0) keep the current value. */
typedef struct tc_tuning {
    int32_t warp_max_deg;   /* 32..512, power of two */
    int32_t light_max_work; /* wedge probes a light task may have */
    int32_t unit_work;      /* target wedge probes per heavy block unit (default 2^20) */
    int32_t long_list;      /* 0..4096 */
    int32_t probe_kicks;    /* 0..1024 */
    int32_t heavy_bitmap;   /* 0 or 1 */
    int32_t blocks_per_sm;  /* persistent grid = SMs * this (0: occupancy) */
    int32_t hash_pairs;     /* 0 or 1: bucketed-pair hash tables instead of cuckoo / linear */
    int32_t flat_max_deg;   /* 0..8: a graph with no row longer than this counts in one kernel */
    int32_t intersect;      /* 0: hash tables; 1: sorted lists, bulk-staged; 2: per light task (see above) */
} tc_tuning;
TC_API int tc_ctx_get_tuning(tc_ctx *ctx, tc_tuning *out);
TC_API int tc_ctx_set_tuning(tc_ctx *ctx, const tc_tuning *in);
/* Autotuner: times the count of g under candidate thresholds (coordinate
 * descent from the current tuning over warp_max_deg, light_max_work,
 * unit_work, long_list, probe_kicks, heavy_bitmap, hash_pairs,
 * flat_max_deg and intersect; each candidate the median of `reps` counts; a change is kept
 * only if it is at least 2% faster) and sets the fastest on ctx.  best / best_ms may be NULL.  At most max_trials
 * candidates are timed. */
TC_API int tc_autotune(tc_ctx *ctx, tc_graph *g, int max_trials, int reps, tc_tuning *best, float *best_ms);
/* tc_autotune that also reports the number of candidates timed (the starting
 * tuning included; at most max_trials) in *trials (may be NULL). */
TC_API int tc_autotune_ex(tc_ctx *ctx, tc_graph *g, int max_trials, int reps, tc_tuning *best, float *best_ms,
                          int *trials);

/* ---- oriented graphs ------------------------------------------------------ */
/* Upload an oriented CSR: n_rows rows, row_ptr[n_rows+1], col[nnz], rows
 * strictly ascending, ids in [0, n_rows).  Roots are rows [0, n_roots); the
 * unpartitioned file has n_roots == n_rows, a halo part has n_roots = t_ver.
 * Replaces the fscanf + cudaMemcpy of ShareKernelTCV62_update_v1.cu:207-239
 * (int32) and without_sorting_tc.cu:250-329 (u64, narrowed to int32 here;
 * TC_E_RANGE when nnz or an id does not fit).  The rows are validated on the
 * device; an unsorted or out-of-range row gives TC_E_FORMAT. */
TC_API int tc_graph_upload_i32(tc_ctx *ctx, const int32_t *row_ptr, const int32_t *col, int64_t n_rows,
                               int64_t nnz, int64_t n_roots, tc_graph **out);
TC_API int tc_graph_upload_u64(tc_ctx *ctx, const uint64_t *row_ptr, const uint64_t *col, int64_t n_rows,
                               int64_t nnz, int64_t n_roots, tc_graph **out);
/* Wrap caller-owned device arrays without copying (no validation). */
TC_API int tc_graph_wrap_device_i32(tc_ctx *ctx, const int32_t *d_row_ptr, const int32_t *d_col, int64_t n_rows,
                                    int64_t nnz, int64_t n_roots, tc_graph **out);
TC_API int tc_graph_info(const tc_graph *g, int64_t *n_rows, int64_t *nnz, int64_t *n_roots);
TC_API int tc_graph_download_i32(tc_ctx *ctx, const tc_graph *g, int32_t *row_ptr, int32_t *col);
TC_API int tc_graph_destroy(tc_graph *g);

/* ---- counting: one graph per launch (the drop-in path) -------------------- */
typedef struct tc_count_stats {
    float count_ms;     /* device time of the counting kernels ("Search") */
    float finalize_ms;  /* device time of the result read-back ("Sum_result") */
    int32_t launches;   /* kernels launched by this call */
    int32_t heavy_units;/* block units produced by the classifier */
} tc_count_stats;

/* Exact triangle count of g: sum over roots u of
 * sum_{v in N+(u)} |N+(u) n N+(v)|.  Replaces Find_Triangle<<<V,128>>> +
 * cub::DeviceReduce::Sum (ShareKernelTCV62_update_v1.cu:43-191, 263-282) and
 * the u64 twin (without_sorting_tc.cu:57-219, 399-434).  Blocks until the
 * result is on the host.  stats may be NULL. */
TC_API int tc_count(tc_ctx *ctx, tc_graph *g, uint64_t *out, tc_count_stats *stats);
/* Enqueue the count of g on the context stream; the result lands in the
 * 8-byte device word d_out (overwritten).  Returns without synchronising.
 * From a graph's second count on (tc_count or tc_count_async), its launch
 * chain is captured once as a CUDA graph and replayed: one launch per count.
 * It is re-captured when the context's tuning changes, and for a new d_out
 * once two counts in a row used it (a d_out that changes every call gets
 * the plain launches).  A stream that the caller is capturing, or a default
 * stream, gets the plain launches. */
TC_API int tc_count_async(tc_ctx *ctx, tc_graph *g, uint64_t *d_out);
/* Per-root counts, the reference's g_sum[u] (ShareKernelTCV62_update_v1.cu:175-186):
 * per_root[u] for u in [0, n_roots), host array. */
TC_API int tc_count_per_root(tc_ctx *ctx, tc_graph *g, uint64_t *per_root, uint64_t *total);
/* End-to-end: host CSR in, count out (upload + validate + count + read-back). */
TC_API int tc_count_csr_i32(tc_ctx *ctx, const int32_t *row_ptr, const int32_t *col, int64_t n_rows, int64_t nnz,
                            uint64_t *out);

/* Count without allocating: for callers that may not allocate GPU memory
 * themselves (an application that owns the device heap and forbids library
 * cudaMalloc calls, a real-time loop, a sandboxed plugin).  No counterpart in
 * the reference.  d_row_ptr / d_col are device arrays of an oriented CSR in
 * the form tc_graph_upload_i32 accepts: row_ptr non-decreasing from 0 to nnz,
 * ids in [0, n_rows), rows strictly ascending.  This entry point does NOT
 * check them (checking needs scratch and a host round trip), and a CSR that
 * breaks them makes the kernels read outside the caller's buffers: pass only
 * a CSR that already passed validation (for example one uploaded once with
 * tc_graph_upload_i32 and read back, or produced by tc_orient).  Roots are
 * rows [0, n_roots); the count is written to the device word d_out in stream
 * order on `stream` (a cudaStream_t, NULL for the default stream); d_out
 * receives UINT64_MAX instead if the classifier's heavy-unit list overflowed
 * (impossible within the limits below, reported all the same).  Scratch is
 * one fixed ~22 MB device array inside libtc: at most 262,144 rows and
 * 2,097,152 oriented edges (TC_E_RANGE beyond).  Calls share that array, so
 * calls that overlap on the GPU race; the first call on a device sets up that
 * device and should come before any stream capture. */
TC_API int tc_count_noalloc_i32(const int32_t *d_row_ptr, const int32_t *d_col, int64_t n_rows, int64_t nnz,
                                int64_t n_roots, uint64_t *d_out, void *stream);

/* ---- batched counting: many graphs or parts, one persistent launch --------- */
/* Replaces the sequential per-part loop of without_sorting_tc.cu:244-465 (one
 * launch + host sync per part).  A batch holds the descriptor table of its
 * graphs and a CUDA graph of [classify -> persistent count]; tc_batch_run
 * replays it and writes outs[i] for graphs[i].  Graphs must outlive the batch. */
TC_API int tc_batch_create(tc_ctx *ctx, tc_graph *const *graphs, int n_graphs, tc_batch **out);
TC_API int tc_batch_run(tc_batch *b, uint64_t *outs);
TC_API int tc_batch_run_async(tc_batch *b);             /* enqueue only */
TC_API int tc_batch_results(tc_batch *b, uint64_t *outs); /* sync + read back */
TC_API int tc_batch_destroy(tc_batch *b);
/* Of the last replay: count_ms = device time of the counting kernels alone
 * (the persistent count launch, not the classification passes), launches =
 * kernels per replay, heavy_units as in tc_count_stats (finalize_ms = 0).
 * Waits for that replay.  Before the first replay only launches is set. */
TC_API int tc_batch_stats(tc_batch *b, tc_count_stats *stats);
/* The partitioned drop-in from host memory: the parts of one graph (the
 * u64 blocks that wo_sort_tc_256 reads, narrowed to int32 by the caller, or
 * int32 parts from tc_halo_extract / the .tcsr cache) are uploaded and
 * validated, counted, and outs[p] (and *total, may be NULL) returned.  All
 * uploads go out at once on a copy stream; a few large parts (at most 64,
 * 4 M entries each on average) are counted one launch each as soon as each is
 * uploaded and validated, overlapping the remaining uploads; many small
 * graphs are counted together in one batched launch.  Host arrays should be
 * page-locked (tc_host_alloc_pinned) for the copies to overlap.  Replaces the
 * per-part cudaMalloc / copy / launch / read-back loop of
 * without_sorting_tc.cu:244-465. */
TC_API int tc_count_parts_csr_i32(tc_ctx *ctx, int n_parts, const int32_t *const *row_ptrs,
                                  const int32_t *const *cols, const int64_t *n_rows, const int64_t *nnz,
                                  const int64_t *n_roots, uint64_t *outs, uint64_t *total);
/* Per-graph launches of the same kernels with a sync after each graph: the
 * plain path the batch is compared against. */
TC_API int tc_count_each(tc_ctx *ctx, tc_graph *const *graphs, int n_graphs, uint64_t *outs);

/* ---- device preprocessing ---------------------------------------------------- */
/* Edge list -> simple undirected CSR on the device: drop self-loops,
 * symmetrise, dedupe (64-bit key radix sort + unique), drop isolated vertices
 * with an order-preserving relabel, rows ascending.  Replaces dgl
 * remove_self_loop / to_bidirected / remove_nodes / adj_tensors
 * (Med_dataset/without_part_preprocess.py:193-228).  n_nodes: vertex count
 * hint (max id + 1 is used when larger).  Ids must be < 2^31. */
TC_API int tc_ugraph_from_edges(tc_ctx *ctx, const int64_t *src, const int64_t *dst, int64_t n_edges,
                                int64_t n_nodes, tc_ugraph **out);
/* Upload an undirected CSR (e.g. a _part.csr file, Halo_creation_preprocess.py:259-278):
 * rows ascending, every edge listed in both rows, no self-loop (TC_E_FORMAT /
 * TC_E_INVALID otherwise).  deg may be NULL (row lengths are used); otherwise
 * it is the file's degree column used by the halo orientation
 * (round_clean_subgraph.cu:172, 178). */
TC_API int tc_ugraph_upload_i64(tc_ctx *ctx, const int64_t *row_ptr, const int64_t *col, const int64_t *deg,
                                int64_t n_rows, int64_t nnz, tc_ugraph **out);
TC_API int tc_ugraph_info(const tc_ugraph *g, int64_t *n_rows, int64_t *nnz);
TC_API int tc_ugraph_download(tc_ctx *ctx, const tc_ugraph *g, int64_t *row_ptr, int64_t *col, int64_t *deg);
TC_API int tc_ugraph_destroy(tc_ugraph *g);
/* Degree orientation on the device: count -> scan -> stable scatter.
 * Replaces Find_size / cp.cumsum / Convert (without_part_preprocess.py:19-111, 253-270). */
TC_API int tc_orient(tc_ctx *ctx, const tc_ugraph *ug, int tie, tc_graph **out);
/* Edge list straight to an oriented graph (tc_ugraph_from_edges + tc_orient). */
TC_API int tc_graph_from_edges(tc_ctx *ctx, const int64_t *src, const int64_t *dst, int64_t n_edges, int64_t n_nodes,
                               int tie, tc_graph **out);

/* ---- halo partitions ---------------------------------------------------------- */
/* Per-part halo subgraphs on the device.  For each part p in [0, k): part
 * vertices (ascending) then their 1-hop halo (ascending) get local ids; the
 * oriented edges among them are kept with rows ascending; halo vertices with
 * zero in-degree are pruned until none is left.  parts_out[p] is an oriented
 * graph with n_roots = t_ver.  part[] is a host array of n_rows non-negative
 * ints; a vertex with part >= k belongs to no extracted part (it can still be
 * in a part's halo), as in the reference's loop over parts 0..k-1.
 * Replaces create_subgraph_with_halo (round_clean_subgraph.cu:357-902) with
 * the prune of Halo_creation_preprocess.py:566-589. */
TC_API int tc_halo_extract(tc_ctx *ctx, const tc_ugraph *ug, const int32_t *part, int k, int tie,
                           tc_graph **parts_out);
/* Halo modes of tc_halo_extract_ex.
 * TC_HALO_REFERENCE: the parts tc_halo_extract writes (1-hop halo, zero
 *   in-degree halo vertices peeled), the round_clean_sg file contract.
 * TC_HALO_COUNT: only the halo vertices with an oriented in-edge from a part
 *   vertex, and the oriented edges among the kept vertices.  A triangle
 *   u -> v -> w rooted at a part vertex u has v and w in N+(u), so both are
 *   kept and every part still counts exactly the triangles rooted in it (the
 *   parts sum to the whole graph's count); the parts are smaller, so their
 *   counts are cheaper.  Not a file format of the reference. */
#define TC_HALO_REFERENCE 0
#define TC_HALO_COUNT 1
/* tc_halo_extract with a halo mode (TC_HALO_*); same part ids and layout. */
TC_API int tc_halo_extract_ex(tc_ctx *ctx, const tc_ugraph *ug, const int32_t *part, int k, int tie, int mode,
                              tc_graph **parts_out);

/* ---- serving: continuous batching over resident graphs ----------------------- */
/* No counterpart in the reference (which runs one file per process).  A
 * server runs two lanes on ctx's device, split by request size (edges given,
 * or the resident graph's oriented edges): a small lane and a large lane,
 * each with a prep thread and a count thread on their own two streams (four
 * contexts).  A prep thread admits its lane's queued requests in arrival
 * order by device-memory footprint (evicting least-recently-used idle
 * resident graphs, across both lanes, to stay within the budget) and builds
 * their oriented CSRs; a count thread counts every ready request of its lane
 * in one batched launch.  So a large build or a large batch holds up neither
 * the small requests' builds nor their counts: the small lane's streams have
 * the higher priority, and the large lane's persistent count kernel leaves
 * reserve_blocks block slots per SM free for them, so small work runs on
 * the device beside a large batch.  Requests arriving during a count are
 * preprocessed concurrently and join their lane's next batch.  Waits are
 * host-side and bounded by batch_timeout_ms; a batch that exceeds it fails
 * with TC_E_TIMEOUT and the server stops admitting. */
typedef struct tc_server_config {
    double hbm_budget_frac;   /* budget = this x device memory (0: 0.8) */
    int64_t hbm_budget_bytes; /* > 0: explicit budget in bytes */
    int32_t max_batch;        /* graphs per batched launch (0: 256) */
    int32_t tie;              /* orientation tie-break of admitted edge lists */
    int32_t batch_timeout_ms; /* watchdog on one batched launch (0: 60000) */
    int32_t reserve_blocks;   /* count-kernel block slots per SM the large lane leaves free (0: 1; < 0: none) */
    int64_t small_edges;      /* requests with at most this many edges take the small lane (0: 2^20; < 0: one
                                 lane for all) */
    int64_t staging_bytes;    /* page-locked host area that submitted edge lists are copied into, so builds
                                 upload them at the link's rate (0: 1 GiB; < 0: none, pageable copies) */
} tc_server_config;

typedef struct tc_server_stats {
    int64_t submitted, completed, failed, batches, cache_hits, evictions, max_batch_seen;
    int64_t budget_bytes, used_bytes, resident_graphs, queued;
    int64_t small_batches, large_batches; /* batches taken by each lane's count thread (counted when taken,
                                              so a batch in flight is already in them and in `batches`) */
} tc_server_stats;

TC_API int tc_server_create(tc_ctx *ctx, const tc_server_config *cfg, tc_server **out);
/* Queue a count.  graph_key != 0 keeps the oriented graph resident under that
 * key; a later request with the same key is counted without preprocessing (it
 * may then pass no edges).  A key names one graph: requests that give edges
 * under a key must give the same graph (repeated edges are dropped, so a
 * longer list of the same edges is the same graph).  If both lanes build one
 * key at once, the first build becomes the resident graph and the other
 * serves only its own request.  The edge arrays are copied before returning (into
 * the pinned staging area when it has room). */
TC_API int tc_server_submit(tc_server *s, uint64_t graph_key, const int64_t *src, const int64_t *dst, int64_t n_edges,
                            int64_t n_nodes, uint64_t *request_id);
/* TC_OK with the count and the latency (submit -> result) once done; the
 * request's own error status if it failed; TC_E_NOT_READY before.  A result
 * is handed out once. */
TC_API int tc_server_poll(tc_server *s, uint64_t request_id, uint64_t *count, double *latency_ms);
/* As poll, blocking up to timeout_ms (< 0: no limit); TC_E_TIMEOUT after it. */
TC_API int tc_server_wait(tc_server *s, uint64_t request_id, int64_t timeout_ms, uint64_t *count, double *latency_ms);
TC_API int tc_server_get_stats(tc_server *s, tc_server_stats *out);
/* Finishes admitted work, fails requests still queued, frees everything.
 * After a batch overran batch_timeout_ms, first waits (up to that long again,
 * at least 5 s) for its kernels; if they are still running, the server's device memory is
 * left allocated and TC_E_TIMEOUT is returned (the handle is gone either way). */
TC_API int tc_server_destroy(tc_server *s);

/* ---- host utilities: text files (the reference's on-disk contract) -------- */
/* Parse a whitespace-separated file of unsigned integers into a flat array,
 * in file order, as the reference's fscanf loops read it
 * (ShareKernelTCV62_update_v1.cu:207-230, without_sorting_tc.cu:242-286,
 * round_clean_subgraph.cu:924-968).  Multi-threaded.  *data is malloc'd by
 * the library; release it with tc_host_free. */
TC_API int tc_text_read_u64(const char *path, uint64_t **data, int64_t *n);
TC_API void tc_host_free(void *p);
/* Append one line of n signed values of elem_bytes (4: int32, 8: int64) to the
 * file; mode 'w' truncates first.  trailing_space != 0 writes "v0 v1 ... vn-1 \n"
 * (every value followed by a space, as without_part_preprocess.py:306-311 and
 * round_clean_subgraph.cu:850-865 write arrays); 0 writes "v0 v1 ... vn-1\n"
 * (round_clean_subgraph.cu:371 header lines). */
TC_API int tc_text_write_line(const char *path, const void *values, int64_t n, int elem_bytes, char mode,
                              int trailing_space);
/* Page-locked host memory for fast transfers (cudaMallocHost). */
TC_API int tc_host_alloc_pinned(size_t bytes, void **out);
TC_API int tc_host_free_pinned(void *p);
/* Edge list of a graph file in the formats the reference's preprocessing
 * reads (Med_dataset/without_part_preprocess.py:126-177): .tsv (Graph
 * Challenge "src dst weight"), .txt (SNAP, '#' comment lines), .mtx / .mmio
 * (Matrix Market coordinate, 1-based, '%' comments, size line skipped); any
 * other extension: two ids per line.  Extra columns are ignored.  *src/*dst
 * are malloc'd by the library (release with tc_host_free). */
TC_API int tc_read_edges(const char *path, int64_t **src, int64_t **dst, int64_t *n_edges);
/* Binary CSR cache (.tcsr): header + int64 row_ptr + int32 col. */
TC_API int tc_tcsr_write(const char *path, const int64_t *row_ptr, const int32_t *col, int64_t n_rows,
                         int64_t nnz, int64_t n_roots, int64_t aux);
TC_API int tc_tcsr_read_header(const char *path, int64_t *n_rows, int64_t *nnz, int64_t *n_roots, int64_t *aux);
TC_API int tc_tcsr_read(const char *path, int64_t *row_ptr, int32_t *col);

/* ---- host utilities: seeded synthetic graphs -------------------------------- */
/* R-MAT: n = edge_factor << scale sampled edges, quadrant probabilities
 * (a, b, c, 1-a-b-c), then a seeded vertex permutation when permute != 0. */
TC_API int tc_gen_rmat(int scale, int edge_factor, double a, double b, double c, uint64_t seed, int permute,
                       int64_t *src, int64_t *dst);
/* Road-like planar graph on a width x height grid: 4-neighbour edges each
 * deleted with probability p_delete, plus one random diagonal per cell with
 * probability diag_rate.  Returns the edge count via *n_edges; buffers must
 * hold 3*width*height edges. */
TC_API int tc_gen_road(int64_t width, int64_t height, double p_delete, double diag_rate, uint64_t seed,
                       int64_t *src, int64_t *dst, int64_t *n_edges);
/* Erdos-Renyi with mean degree p*(n-1): M = round(p*n*(n-1)/2) uniform vertex
 * pairs (G(n, M); repeats and self-loops go in clean-up).  *n_edges: buffer
 * capacity in, M out. */
TC_API int tc_gen_er(int64_t n, double p, uint64_t seed, int64_t *src, int64_t *dst, int64_t *n_edges);
/* Chung-Lu: expected degrees w_i ~ (i+1)^(-1/(gamma-1)) scaled to mean
 * avg_deg and capped at sqrt(n*avg_deg) (= sqrt(2E)); n*avg_deg/2 edges with
 * endpoints drawn proportional to w. */
TC_API int tc_gen_chung_lu(int64_t n, double gamma, double avg_deg, uint64_t seed, int64_t *src, int64_t *dst,
                           int64_t n_edges);
/* Seeded uniform part assignment in [0, k) (replaces the unseeded
 * np.random.randint, Halo_creation_preprocess.py:288, 325, 362). */
TC_API int tc_gen_parts_random(int64_t n, int k, uint64_t seed, int32_t *part);
/* Contiguous assignment exactly as Halo_creation_preprocess.py:293-299:
 * l = n / k, vertices [i*l, (i+1)*l) -> part i, the last n mod k -> part 0. */
TC_API int tc_gen_parts_contig(int64_t n, int k, int32_t *part);
/* Balanced label-propagation parts of ug's vertices on the device, the
 * stand-in for the reference's METIS assignment
 * (dgl.metis_partition_assignment(G, k), Halo_creation_preprocess.py:304,
 * 341, 378): parts of at most ceil(1.03 n / k) vertices (up to sampling
 * noise) with few cut edges, so halos stay small.  Starts from balanced
 * contiguous ranges; each of at most `iterations` synchronous rounds moves
 * vertices to their neighbours' most common label, with room-limited
 * migration.  Integer-only and seeded: the same seed gives the same parts on
 * any GPU.  1 <= k <= 64; part is a host array of n_rows ints. */
TC_API int tc_gen_parts_lp(tc_ctx *ctx, const tc_ugraph *ug, int k, uint64_t seed, int iterations, int32_t *part);

#ifdef __cplusplus
}
#endif
#endif /* TC_H */
