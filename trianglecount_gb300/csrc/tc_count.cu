// tc_count.cu -- exact triangle counting on a degree-oriented int32 CSR.
//
// Quantity: for each root u, sum over v in N+(u) of |N+(u) n N+(v)| -- the
// reference's per-block g_sum[u] (src/WithoutPartition/ShareKernelTCV62_update_v1.cu:43-191,
// src/WithPartition/without_sorting_tc.cu:57-219), summed over roots as the
// reference's cub::DeviceReduce::Sum does (ShareKernelTCV62_update_v1.cu:271-277).
// Every triangle u -> v -> w (u -> w) is found once, at its oriented edge u -> v
// as the hit w of the intersection N+(u) n N+(v).
//
// The reference runs one 128-thread block per root and binary-searches each x
// of N+(v) against 128-entry shared tiles of N+(u).  Here the intersection of
// each oriented edge u -> v is done from its cheaper side:
//
//   root-centric   (d+(v) <= d+(u)): stream N+(v) through a hash of N+(u);
//   middle-centric (d+(u) <  d+(v)): stream N+(u) through a hash of N+(v).
//
// so the probes total sum_{u->v} min(d+(u), d+(v)) instead of the reference's
// sum d+(v) (0.43x on R-MAT scale 21).  Each vertex x gets one task: a hash of
// N+(x) and a list of partners whose lists are streamed through it -- its
// out-neighbours v with d+(v) <= d+(x) (when x is a root) and its in-neighbours
// u with d+(u) < d+(x) (u a root).  The in-neighbour lists are a transpose of
// the middle-centric edges built on the device for every count.
//
// A graph with no row longer than flat_max_deg (8) is counted instead by one
// flat kernel: N+(u) and every N+(v) in registers, one lane per root
// (flat_kernel, rows of up to 8) or a lane pipelining several roots
// (flat4_kernel, rows of up to 4).
//
// Launch sequence (one CUDA-graph-capturable chain, plain or batched):
//   degree     d+(x) of every row into a per-vertex array (in_cnt's storage)
//   in_count   one warp per 32 rows: per root u, per v in N+(u), mark the edge
//              middle-centric or not, count the middle-centric in-edges of v
//              and their work (one packed atomic), the root-centric work of u,
//              and the total
//   scan       in-edge offsets, read from the packed words' high halves; each
//              word's high half becomes the end of the vertex's in-list
//   transpose  per root u, scatter the middle-centric edges into the in-lists
//              (one atomic decrement of the packed word gives the slot);
//              classify each vertex x by d+(x) and its work w(x): micro tasks
//              (d+(x) <= 8, w(x) <= 128) are listed from the top of the task
//              list, light tasks (d+(x) <= warp_max, w(x) <= the light bound)
//              from its bottom, heavy ones become (#tiles x #slices)
//              block units, appended with one packed 64-bit atomic so entries
//              stay sorted by unit
//   micro      one lane per listed micro task (a warp takes 32), N+(x) in
//              registers
//   count      persistent grid (SMs x occupancy blocks):
//                phase A -- blocks pull heavy units from a global cursor; a
//                  unit hashes one tile of N+(x) (load factor <= 1/4) in shared
//                  memory and its warps pull 16-partner chunks of the unit's
//                  slice from a shared cursor;
//                phase B -- warps take light tasks four at a time from the
//                  list and run each with a per-warp shared hash.
//              A launch with halo parts runs the two phases as two kernels
//              (each with its own register allocation).
//              Streaming a chunk of partners: lists with length >= long_list are
//              read by the whole warp, four coalesced loads in flight per lane;
//              shorter lists are flattened across the lanes (warp scan of the
//              lengths, one probe per lane per step).
//   totals     per-lane u64 accumulators, warp-reduced, one atomic per warp per
//              graph change; integer addition is associative, so the count is
//              exact and independent of the schedule.
//
// The same kernels serve the plain path (one graph per launch) and the batched
// path (a descriptor table of many graphs or halo parts, one launch each).
#include <algorithm>
#include <cstdio>

#include "tc_internal.h"

namespace tc {
namespace {

constexpr int kWarp = 32;
constexpr unsigned kFull = 0xffffffffu;
constexpr int kEmpty = -1;
constexpr int kThreads = 256;
constexpr int kWarpsPerBlock = kThreads / kWarp;
constexpr int kHeavyChunk = 16; // partners per warp grab inside a heavy unit (4: R-MAT 21 kernel 6.49 ms, 16: 6.04)
constexpr int kLaneRowDeg = 16; // auxiliary passes: rows with d+ <= this are walked one per lane
constexpr int kMicroDeg = 8;    // micro tasks: d+(x) <= this (N+(x) held in registers) ...
constexpr int kMicroWork = 128; // ... and at most this many probes (one lane runs the task serially)
constexpr int kAuxGrab = 2;     // 32-row chunks an auxiliary-kernel warp takes per cursor grab (4 -> 2:
                                // R-MAT 23's eight parts 40.65 -> 40.50 ms, R-MAT 21's 8.43 -> 8.26 ms, the
                                // 256-graph batch unchanged; 1 costs that batch 3 %, 8 costs the parts 2.5 %)
// One middle-centric in-edge in a packed in_work word.  Both halves stay below
// 2^31: a vertex has fewer than nnz in-edges, and its in-partners' d+(u) sum to
// at most nnz < 2^31 (each u counted once), so one 64-bit atomic adds both.
// After the in-list scan the high half holds in_off + in-edges (at most the
// launch's pooled nnz, also < 2^31), and the transpose counts it back down.
constexpr unsigned long long kInEdge = 1ull << 32;
constexpr int kLightGrab = 4;   // light tasks a count-kernel warp takes per cursor grab (8 in halo parts:
                                // they hold ~4x the light tasks; R-MAT 23's eight parts 38.14 -> 38.00 ms)
constexpr int kMinUnit = 8192;  // smallest heavy block unit (probes)
constexpr int kMinLight = 1024; // smallest light-task bound (probes)
#ifndef TC_COUNT_MIN_BLOCKS
// Resident blocks per SM the count kernel's registers must allow: 6 caps it
// at 40 registers (a few spilled bytes) for 48 warps per SM, ~10% faster on
// R-MAT than the unconstrained 48 registers / 40 warps.
#define TC_COUNT_MIN_BLOCKS 6
#endif

__device__ __forceinline__ uint32_t hash_slot(int x, int shift) { return ((uint32_t)x * 0x9E3779B1u) >> shift; }

__device__ __forceinline__ int ilog2_ceil(int x) { return x <= 1 ? 0 : 32 - __clz(x - 1); }

// Open addressing, linear probing, at most a quarter of the slots used, so a
// miss usually ends at the first slot.  The iteration bound only guards
// against a corrupt table.
__device__ __forceinline__ void table_insert(int *tab, uint32_t mask, int shift, int x) {
    uint32_t h = hash_slot(x, shift);
    for (uint32_t it = 0; it <= mask; ++it) {
        const int old = atomicCAS(&tab[h], kEmpty, x);
        if (old == kEmpty || old == x) return;
        h = (h + 1) & mask;
    }
}

__device__ __forceinline__ uint32_t table_probe(const int *tab, uint32_t mask, int shift, int x) {
    uint32_t h = hash_slot(x, shift);
    int y = tab[h];
    for (uint32_t it = 0; y != x && y != kEmpty && it < mask; ++it) {
        h = (h + 1) & mask;
        y = tab[h];
    }
    return (uint32_t)(y == x);
}

// Cuckoo hashing (two slots per key, Pagh & Rodler; parallel insertion by
// atomicExch as in Alcantara et al., "Real-time parallel hashing on the GPU",
// 2009): a lookup reads exactly the two candidate slots -- two independent
// shared loads, no loop, so the lanes of a warp never diverge on collisions.
// Insertion moves a displaced key to its other slot, at most `kicks` times;
// every key is always either in the table or in one thread's hand, so when no
// insertion gives up, all keys are in.  A give-up switches the task to linear
// probing (rebuilt), decided warp- or block-uniformly.
__device__ __forceinline__ uint32_t hash_slot2(int x, int shift) { return ((uint32_t)x * 0x85EBCA77u) >> shift; }

__device__ __forceinline__ bool cuckoo_insert(int *tab, int shift, int x, int kicks) {
    int cur = x;
    uint32_t pos = hash_slot(cur, shift);
    for (int it = 0; it < kicks; ++it) {
        const int old = atomicExch(&tab[pos], cur);
        if (old == kEmpty) return true;
        cur = old;
        const uint32_t p1 = hash_slot(cur, shift), p2 = hash_slot2(cur, shift);
        pos = pos == p1 ? p2 : p1;
    }
    return false;
}

__device__ __forceinline__ uint32_t cuckoo_probe(const int *tab, int shift, int x) {
    const int a = tab[hash_slot(x, shift)];
    const int b = tab[hash_slot2(x, shift)];
    return (uint32_t)((a == x) | (b == x));
}

// Bucketed pairs: slots 2b and 2b+1 form bucket b and are read together by
// one 8-byte shared load; one hash picks a key's home bucket.  A key goes to
// the first bucket from its home with a free slot, and every full bucket it
// passes is flagged (bit 31 of the bucket's first slot, which is occupied), so
// a lookup reads past a bucket only when that bucket is flagged.  At a load of
// at most 1/4 (half a key per bucket on average) about 1.4% of the buckets
// hold more than two home keys, so nearly every probe is one shared load
// against two for the cuckoo hash.  Measured slower than the cuckoo hash all
// the same (the wider loads and the rare flagged chains cost more than the
// second load saves), so it is an autotuner candidate only.  Keys are vertex
// ids <= 2^31 - 2, so a flagged slot (key | 2^31, negative, not -1) never
// reads as empty or as a key.
constexpr int kFlagBit = (int)0x80000000u;
constexpr int kKeyBits = 0x7fffffff;

__device__ __forceinline__ void pair_insert(int *tab, uint32_t bmask, int shift, int x) {
    uint32_t b = hash_slot(x, shift + 1);
    for (uint32_t it = 0; it <= bmask; ++it) {
        if (atomicCAS(&tab[2 * b], kEmpty, x) == kEmpty) return;
        if (atomicCAS(&tab[2 * b + 1], kEmpty, x) == kEmpty) return;
        atomicOr(&tab[2 * b], kFlagBit);
        b = (b + 1) & bmask;
    }
}

__device__ __forceinline__ uint32_t pair_hit(int2 v, int x) { return (uint32_t)(((v.x & kKeyBits) == x) | (v.y == x)); }

// The rest of a pair lookup after its home bucket v (read at b) missed and was
// flagged.  The bound only guards against a corrupt table.
__device__ __forceinline__ uint32_t pair_probe_rest(const int *tab, uint32_t bmask, uint32_t b, int x) {
    const int2 *tv = reinterpret_cast<const int2 *>(tab);
    for (uint32_t it = 0; it < bmask; ++it) {
        b = (b + 1) & bmask;
        const int2 v = tv[b];
        if (pair_hit(v, x)) return 1u;
        if (v.x >= kEmpty) return 0u;  // not flagged: the chain ends here
    }
    return 0u;
}

__device__ __forceinline__ uint32_t pair_probe(const int *tab, uint32_t bmask, int shift, int x) {
    const uint32_t b = hash_slot(x, shift + 1);
    const int2 v = reinterpret_cast<const int2 *>(tab)[b];
    uint32_t h = pair_hit(v, x);
    if (!h && v.x < kEmpty) h = pair_probe_rest(tab, bmask, b, x);
    return h;
}

// Membership of x in a direct-address bitmap of vertex ids (bit x of word
// x/32).  A negative x (a padding lane) reads word 0 and reports no hit, so
// the load stays inside the bitmap.
__device__ __forceinline__ uint32_t bitmap_probe(const int *bm, int x) {
    const int y = x < 0 ? 0 : x;
    return ((uint32_t)bm[(unsigned)y >> 5] >> (y & 31)) & (uint32_t)(x >= 0);
}

// Table modes, chosen per table (warp- or block-uniform).  kSorted is not a
// hash: the task's list itself, staged in shared memory as it lies (sorted),
// probed by binary search.
constexpr int kLinear = 0, kCuckoo = 1, kPairs = 2, kSorted = 3;

// ---- bulk staging of a sorted list into shared memory ------------------------
// A list col[s, s + n) is copied into a 16-byte-aligned shared buffer by one
// cp.async.bulk (the Blackwell/Hopper bulk-copy engine, no registers or
// load instructions per element), completing on an mbarrier.  The copy covers
// the 16-byte-aligned span [s & ~3, ceil4(s + n)) of col, clamped below
// floor4(nnz) so it never reads past the array; the few elements past the
// clamp (only at the end of col) are loaded by plain loads.  Element i of the
// list is then buf[o + i], o = s - (s & ~3).  A col that is not 16-byte
// aligned (a wrapped caller array) is staged by plain loads only.
__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long *bar, int count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

// Orders this thread's earlier generic-proxy shared accesses before later
// async-proxy (bulk copy) writes to the same addresses.
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void bulk_load(void *dst, const void *src, uint32_t bytes, unsigned long long *bar) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return done != 0;
}

// Waits for the barrier's phase `parity` to complete, at most kWaitRounds
// try_wait calls (each suspends for a bounded, hardware-chosen time); false
// when it gave up.  A bulk copy of a few KB completes in microseconds, so a
// give-up means a broken invariant, which the caller reports as an error.
constexpr int kWaitRounds = 1 << 22;
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, uint32_t parity) {
    for (int it = 0; it < kWaitRounds; ++it)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// Bytes the bulk part of staging col[s, s + n) copies (0: none); every
// thread of the staging group computes it, one issues the copy.
__device__ __forceinline__ uint32_t stage_bytes(const int32_t *col, int64_t lim4, int s, int n) {
    if (((uintptr_t)col & 15u) != 0) return 0;
    const int64_t a0 = s & ~3;
    int64_t a1 = ((int64_t)s + n + 3) & ~(int64_t)3;
    if (a1 > lim4) a1 = lim4;
    return a1 > a0 ? (uint32_t)(a1 - a0) * 4u : 0u;
}

// Issues the staging of col[s, s + n) into buf (16-byte aligned) by one
// thread (the caller's elected thread) and returns the bulk part's byte
// count (0: nothing issued, no barrier phase used).  lim4 = floor4(nnz).
__device__ __forceinline__ uint32_t stage_issue(const int32_t *col, int64_t lim4, int s, int n, int *buf,
                                                unsigned long long *bar) {
    if (((uintptr_t)col & 15u) != 0) return 0;
    const int64_t a0 = s & ~3;
    int64_t a1 = ((int64_t)s + n + 3) & ~(int64_t)3;
    if (a1 > lim4) a1 = lim4;
    if (a1 <= a0) return 0;
    const uint32_t bytes = (uint32_t)(a1 - a0) * 4u;
    bulk_load(buf, col + a0, bytes, bar);
    return bytes;
}

// The elements of col[s, s + n) that the bulk part does not cover, by plain
// loads; threads tid, tid + nthreads, ...
// Returns whether any element was written this way (the same on every thread).
__device__ __forceinline__ bool stage_rest(const int32_t *col, int64_t lim4, int s, int n, int *buf, int tid,
                                           int nthreads) {
    int64_t first = s;  // the first element the bulk part does not cover
    if (((uintptr_t)col & 15u) == 0) {
        int64_t a1 = ((int64_t)s + n + 3) & ~(int64_t)3;
        if (a1 > lim4) a1 = lim4;
        if (a1 > (int64_t)(s & ~3) && a1 > first) first = a1;
    }
    const int o = s & 3;
    for (int64_t j = first + tid; j < (int64_t)s + n; j += nthreads) buf[o + (int)(j - s)] = __ldg(col + j);
    return first < (int64_t)s + n;
}

// Membership of x in the sorted list a[0, n) (n >= 1) by a branch-free binary
// search: ceil(log2 n) dependent shared loads, the same count on every lane
// of a warp probing one list (the reference's Search on a shared tile,
// ShareKernelTCV62_update_v1.cu:12-42, on the whole list instead of 128-entry
// tiles).
__device__ __forceinline__ uint32_t sorted_probe(const int *a, int n, int x) {
    int lo = 0;
    for (int len = n; len > 1;) {
        const int half = len >> 1;
        lo = a[lo + half] <= x ? lo + half : lo;
        len -= half;
    }
    return (uint32_t)(a[lo] == x);
}

// Membership of x >= 0 in the table, by the table's mode (kPairsOnly: the
// kernel instance that builds pair tables only).
template <bool kPairsOnly, bool kSortedOk = false>
__device__ __forceinline__ uint32_t probe_any(const int *tab, uint32_t mask, int shift, int x, int mode) {
    if (kPairsOnly) return pair_probe(tab, mask >> 1, shift, x);
    if (kSortedOk && mode == kSorted) return sorted_probe(tab, (int)mask, x);  // mask = the list's length
    return mode == kCuckoo ? cuckoo_probe(tab, shift, x) : table_probe(tab, mask, shift, x);
}

// Fills an emptied table with the keys keys[i], i in [tid, n) step nthreads, in
// the preferred mode and returns that mode; *ok turns false when a cuckoo
// insertion gave up (the caller then empties the table and inserts linearly).
template <bool kPairsOnly>
__device__ __forceinline__ int table_fill(int *tab, uint32_t mask, int shift, const int32_t *__restrict__ keys, int n,
                                          int tid, int nthreads, int pref, int kicks, bool *ok) {
    if (kPairsOnly) {
        for (int i = tid; i < n; i += nthreads) pair_insert(tab, mask >> 1, shift, __ldg(keys + i));
    } else if (pref == kCuckoo) {
        for (int i = tid; i < n; i += nthreads) *ok &= cuckoo_insert(tab, shift, __ldg(keys + i), kicks);
    } else {
        for (int i = tid; i < n; i += nthreads) table_insert(tab, mask, shift, __ldg(keys + i));
    }
    return pref;
}

// Table geometry for n keys: slots = max(32, next_pow2(4 n)).
__device__ __forceinline__ int table_log_slots(int n) { return max(5, ilog2_ceil(4 * n)); }

// Empties a table of (mask + 1) slots with `nthreads` threads numbered `tid`;
// the caller synchronises before inserting.
__device__ __forceinline__ void table_clear(int *tab, uint32_t mask, int tid, int nthreads) {
    for (int i = tid; i <= (int)mask; i += nthreads) tab[i] = kEmpty;
}

__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long v) {
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
    return v;
}

__device__ __forceinline__ int find_graph(const GraphDesc *gd, int n_graphs, int64_t chunk) {
    int lo = 0, hi = n_graphs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (gd[mid].chunk_base <= chunk) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

struct KParams {
    const GraphDesc *gd;
    int n_graphs;
    int64_t total_chunks;
    const HeavyEntry *heavy;
    int64_t heavy_cap;
    CountWork *work;
    unsigned long long *results;
    uint32_t *light_list;  // tasks as global rows chunk * 32 + lane: light tasks from entry 0 up,
                           // micro tasks from entry list_cap - 1 down (counts in work->n_tasks)
    int64_t list_cap;      // entries of light_list (the launch's rows: a row is at most one task)
    int32_t *in_cnt;       // per vertex (pooled): d+, for in_count's gathers
    int32_t *in_off;       // per vertex (pooled) + 1: exclusive scan of the middle-centric in-edge counts
    unsigned long long *in_work;   // per vertex: (in-edges << 32) | sum of d+(u) over its in-partners u; the scan
                                   // adds in_off to the high half, and the transpose counts it back down to in_off
    unsigned long long *out_work;  // per vertex: sum of d+(v) over its out-partners v
    int32_t *in_list;      // in-partner lists, in_off-indexed
    uint8_t *mid;          // per oriented edge (pooled by ebase): 1 = middle-centric
    int warp_max;
    int log_warp_slots;
    int light_max_work;
    int unit_work;
    int tile;
    int long_list;
    int probe_kicks;  // 0: linear probing; > 0: cuckoo with this many kicks
    int table_mode;   // preferred table mode: kPairs, kCuckoo (probe_kicks > 0) or kLinear
    int heavy_done;   // heavy units belong to heavy_bitmap_kernel: count_kernel skips phase A
    int intersect;    // 0: hash tables; 1: every task on its bulk-staged sorted list (binary search);
                      // 2: per light task, the sorted list when its work is below its list length
    int aux_dynamic;  // auxiliary kernels walk chunks from cursors (batches) instead of grid-stride
    int count_blocks; // persistent grid of count_kernel
};

// Where the partner p_j of task x lives and whose root it credits.
struct Task {
    const int32_t *out_nbr;  // col + rp[x]
    const int32_t *in_nbr;   // in_list + in_off[x]
    int n_out;               // d+(x) if x is a root, else 0
    int dx;                  // d+(x)
    int x;
};

// Streams the lists of partners [j0, j1) of task T (at most 32 partners)
// through the hash of N+(x) (or of a tile of it).  Partners j < n_out are
// out-neighbours v of x, skipped unless d+(v) <= d+(x); the others are
// in-neighbours u.  Returns this lane's hit count; with per_root set, hits are
// also credited to their root (x for out-partners, u for in-partners).
template <bool kPerRoot, bool kBitmap = false, bool kPairsOnly = false, bool kSortedOk = false>
__device__ __forceinline__ uint32_t probe_partners(const int32_t *__restrict__ rp, const int32_t *__restrict__ col,
                                                   const Task &T, int j0, int j1, const int *tab, uint32_t mask,
                                                   int shift, int mode, int long_list, int lane,
                                                   unsigned long long *__restrict__ per_root) {
    uint32_t hits = 0;
    const int j = j0 + lane;
    int s2 = 0, len = 0, owner = T.x;
    if (j < j1) {
        int p;
        if (j < T.n_out) {
            p = __ldg(T.out_nbr + j);
        } else {
            p = __ldg(T.in_nbr + (j - T.n_out));
            owner = p;
        }
        s2 = __ldg(rp + p);
        len = __ldg(rp + p + 1) - s2;
        if (j < T.n_out && len > T.dx) len = 0;  // middle-centric edge: done from p's side
    }
    // long lists: the whole warp streams one list, four loads in flight per lane
    unsigned longm = __ballot_sync(kFull, len >= long_list && len > 0);
    while (longm) {
        const int k = __ffs(longm) - 1;
        longm &= longm - 1u;
        const int ls = __shfl_sync(kFull, s2, k);
        const int ll = __shfl_sync(kFull, len, k);
        const int32_t *__restrict__ p = col + ls;
        uint32_t h = 0;
        for (int base = 0; base < ll; base += 4 * kWarp) {
            int x[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int t = base + i * kWarp + lane;
                x[i] = t < ll ? __ldg(p + t) : -1;
            }
            if (kBitmap) {
#pragma unroll
                for (int i = 0; i < 4; ++i) h += (uint32_t)(x[i] >= 0) & bitmap_probe(tab, x[i]);
            } else if (kPairsOnly) {
                // the four home buckets first (independent loads), then the rare flagged chains
                const uint32_t bmask = mask >> 1;
                int2 v[4];
                uint32_t b[4];
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    b[i] = hash_slot(x[i], shift + 1);
                    v[i] = reinterpret_cast<const int2 *>(tab)[b[i]];
                }
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    uint32_t hi = pair_hit(v[i], x[i]);
                    if (!hi && v[i].x < kEmpty && x[i] >= 0) hi = pair_probe_rest(tab, bmask, b[i], x[i]);
                    h += (uint32_t)(x[i] >= 0) & hi;
                }
            } else if (mode == kCuckoo) {
#pragma unroll
                for (int i = 0; i < 4; ++i) h += (uint32_t)(x[i] >= 0) & cuckoo_probe(tab, shift, x[i]);
            } else if (kSortedOk && mode == kSorted) {  // four independent searches in flight
#pragma unroll
                for (int i = 0; i < 4; ++i) h += (uint32_t)(x[i] >= 0) & sorted_probe(tab, (int)mask, x[i]);
            } else {
#pragma unroll
                for (int i = 0; i < 4; ++i)
                    if (x[i] >= 0) h += table_probe(tab, mask, shift, x[i]);
            }
        }
        hits += h;
        if (kPerRoot) {
            const unsigned long long s = warp_sum_u64(h);
            const int ow = __shfl_sync(kFull, owner, k);
            if (lane == 0 && s) atomicAdd(per_root + ow, s);
        }
    }
    // short lists: flattened across the lanes
    if (len >= long_list) len = 0;
    int incl = len;
#pragma unroll
    for (int o = 1; o < kWarp; o <<= 1) {
        const int t = __shfl_up_sync(kFull, incl, o);
        if (lane >= o) incl += t;
    }
    const int excl = incl - len;
    const int total = __shfl_sync(kFull, incl, kWarp - 1);
    for (int base = 0; base < total; base += kWarp) {
        const int t = base + lane;
        // largest lane k with excl_k <= t (excl is non-decreasing)
        int seg = 0;
#pragma unroll
        for (int step = 16; step >= 1; step >>= 1) {
            const int ex = __shfl_sync(kFull, excl, seg + step);
            if (ex <= t) seg += step;
        }
        const int ex_seg = __shfl_sync(kFull, excl, seg);
        const int s_seg = __shfl_sync(kFull, s2, seg);
        const int own = kPerRoot ? __shfl_sync(kFull, owner, seg) : 0;
        if (t < total) {
            const int y = __ldg(col + s_seg + (t - ex_seg));
            const uint32_t h =
                kBitmap ? bitmap_probe(tab, y) : probe_any<kPairsOnly, kSortedOk>(tab, mask, shift, y, mode);
            hits += h;
            if (kPerRoot && h) atomicAdd(per_root + own, 1ull);
        }
    }
    return hits;
}

// Chunk walk of the auxiliary kernels.  One graph: a static grid-stride walk
// over a grid larger than what is resident (the block scheduler balances it).
// A batch (aux_dynamic): the resident grid grabs kAuxGrab chunks at a time
// from a cursor, so the chunks in flight form one window moving through the
// graphs in order (each graph's in-lists and hub lists stay hot in L2 while
// it is walked, and heavy entries come out graph-ordered).  [c, c_end) is the
// next range; c >= c_end means done.
__device__ __forceinline__ void aux_next(const KParams &P, int k, int lane, bool first, int64_t &c, int64_t &c_end) {
    if (P.aux_dynamic) {
        unsigned cg = 0;
        if (lane == 0) cg = atomicAdd(&P.work->aux_cursor[k], (unsigned)kAuxGrab);
        cg = __shfl_sync(kFull, cg, 0);
        c = (int64_t)cg;
        c_end = min(c + kAuxGrab, P.total_chunks);
    } else {
        const int64_t gwarp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / kWarp;
        const int64_t nwarps = (int64_t)gridDim.x * blockDim.x / kWarp;
        c = first ? gwarp : c_end - 1 + nwarps;
        c_end = min(c + 1, P.total_chunks);
    }
}

// in_count: per root u of a 32-row chunk, per v in N+(u): middle-centric edges
// (d+(u) < d+(v)) add one in-edge and d+(u) of work to v; the others add d+(v)
// to u's root-centric work.  Both in_count and transpose_classify are held to
// 40 registers, 6 resident blocks (R-MAT 23's count 36.92 -> 36.87 ms against
// 48 registers and 5 blocks).
__global__ void __launch_bounds__(kThreads, 6) in_count_kernel(KParams P) {
    const int lane = threadIdx.x & (kWarp - 1);
    unsigned long long probes = 0;  // this lane's share of sum_{u->v} min(d+(u), d+(v))
    int64_t c, c_end;
    aux_next(P, 0, lane, true, c, c_end);
    for (; c < c_end; aux_next(P, 0, lane, false, c, c_end)) {
        for (; c < c_end; ++c) {
            const int g = find_graph(P.gd, P.n_graphs, c);
            const GraphDesc &G = P.gd[g];
            const int32_t *__restrict__ rp = G.rp;
            const int32_t *__restrict__ col = G.col;
            const int64_t x0 = (c - G.chunk_base) * kWarp;
            int rs = 0, d = 0;
            if (x0 + lane < G.n_roots) {
                rs = __ldg(rp + x0 + lane);
                d = __ldg(rp + x0 + lane + 1) - rs;
            }
            // short rows: one per lane, four edges' loads in flight at a time
            if (d >= 1 && d <= kLaneRowDeg) {
                unsigned long long ow = 0;
                for (int i0 = 0; i0 < d; i0 += 4) {
                    int v[4], dv[4];
#pragma unroll
                    for (int q = 0; q < 4; ++q) v[q] = i0 + q < d ? __ldg(col + rs + i0 + q) : -1;
#pragma unroll
                    for (int q = 0; q < 4; ++q) dv[q] = v[q] >= 0 ? __ldg(P.in_cnt + G.vbase + v[q]) : 0;
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        if (v[q] < 0) continue;
                        const bool m = d < dv[q];
                        P.mid[G.ebase + rs + i0 + q] = (uint8_t)m;
                        if (m) {
                            atomicAdd(P.in_work + G.vbase + v[q], kInEdge | (unsigned long long)d);
                            probes += (unsigned long long)d;
                        } else {
                            ow += (unsigned long long)dv[q];
                        }
                    }
                }
                P.out_work[G.vbase + x0 + lane] = ow;
                probes += ow;
            }
            // long rows: the whole warp
            unsigned todo = __ballot_sync(kFull, d > kLaneRowDeg);
            while (todo) {
                const int k = __ffs(todo) - 1;
                todo &= todo - 1u;
                const int rrs = __shfl_sync(kFull, rs, k);
                const int rd = __shfl_sync(kFull, d, k);
                unsigned long long ow = 0;
                for (int i0 = lane; i0 < rd; i0 += 4 * kWarp) {  // four edges' loads in flight
                    int v[4], dv[4];
#pragma unroll
                    for (int q = 0; q < 4; ++q) v[q] = i0 + q * kWarp < rd ? __ldg(col + rrs + i0 + q * kWarp) : -1;
#pragma unroll
                    for (int q = 0; q < 4; ++q) dv[q] = v[q] >= 0 ? __ldg(P.in_cnt + G.vbase + v[q]) : 0;
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        if (v[q] < 0) continue;
                        const bool m = rd < dv[q];
                        P.mid[G.ebase + rrs + i0 + q * kWarp] = (uint8_t)m;
                        if (m) {
                            atomicAdd(P.in_work + G.vbase + v[q], kInEdge | (unsigned long long)rd);
                            probes += (unsigned long long)rd;
                        } else {
                            ow += (unsigned long long)dv[q];
                        }
                    }
                }
                probes += ow;
                ow = warp_sum_u64(ow);
                if (lane == 0) P.out_work[G.vbase + x0 + k] = ow;
            }
        }
    }
    // every edge's probes (the cheaper side) once, for the classifier's unit size
    probes = warp_sum_u64(probes);
    if (lane == 0 && probes) atomicAdd(&P.work->total_work, probes);
}

// in_cnt[vbase + x] = d+(x) for every row, for in_count's gathers (one load
// per edge instead of a row_ptr pair).
__global__ void __launch_bounds__(kThreads) degree_kernel(KParams P) {
    const int lane = threadIdx.x & (kWarp - 1);
    const int64_t gwarp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / kWarp;
    const int64_t nwarps = (int64_t)gridDim.x * blockDim.x / kWarp;
    for (int64_t c = gwarp; c < P.total_chunks; c += nwarps) {
        const GraphDesc &G = P.gd[find_graph(P.gd, P.n_graphs, c)];
        const int64_t x = (c - G.chunk_base) * kWarp + lane;
        if (x < G.n_rows) P.in_cnt[G.vbase + x] = __ldg(G.rp + x + 1) - __ldg(G.rp + x);
    }
}

// The transpose's scatter of up to four middle-centric edges i0 + q * step
// (q < 4, i < d) of root u's row.  The in-list scan left the end of v's
// in-list in in_work[v]'s high half, so one atomic decrement per edge returns
// its slot (no in_off gather); the four are issued together, so a lane waits
// on one L2 round trip per four edges, not one chain per edge.
__device__ __forceinline__ void scatter4(const KParams &P, const GraphDesc &G, const int32_t *__restrict__ row,
                                         int64_t e0, int i0, int step, int d, int32_t u) {
    int v[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int i = i0 + q * step;
        v[q] = i < d && P.mid[e0 + i] ? __ldg(row + i) : -1;
    }
    int slot[4];
#pragma unroll
    for (int q = 0; q < 4; ++q)
        slot[q] = v[q] >= 0 ? (int)(atomicAdd(P.in_work + G.vbase + v[q], 0ull - kInEdge) >> 32) - 1 : 0;
#pragma unroll
    for (int q = 0; q < 4; ++q)
        if (v[q] >= 0) P.in_list[slot[q]] = u;
}

// transpose + classify: scatter the chunk's middle-centric edges into the
// in-lists, then classify each row of the chunk as a micro task (task list,
// from the top), a light task (task list, from the bottom), a heavy task
// (block units) or no work.
__global__ void __launch_bounds__(kThreads, 6) transpose_classify_kernel(KParams P, HeavyEntry *heavy) {
    const int lane = threadIdx.x & (kWarp - 1);
    // Block-unit size: unit_work, or less on a small job so that every count
    // block gets about four units; the light-task bound likewise, so that a
    // warp's largest light task is at most a quarter of a fair share (one unit
    // is one block's work, one light task one warp's: on a small graph, a
    // large one would be the whole kernel's tail).
    const unsigned long long total = P.work->total_work;
    const unsigned long long unit =
        min((unsigned long long)P.unit_work, max((unsigned long long)kMinUnit, total / (4ull * P.count_blocks)));
    const unsigned long long light_max =
        min((unsigned long long)P.light_max_work,
            max((unsigned long long)kMinLight, total / (4ull * P.count_blocks * kWarpsPerBlock)));
    // the micro / light masks of the chunks of one grab; their task-list slots
    // are reserved with one atomic per grab (one hot word for the whole launch)
    __shared__ uint32_t s_mask[kWarpsPerBlock][2 * kAuxGrab];
    uint32_t *wmask = s_mask[threadIdx.x / kWarp];
    int64_t c, c_end;
    aux_next(P, 1, lane, true, c, c_end);
    for (; c < c_end; aux_next(P, 1, lane, false, c, c_end)) {
        const int64_t c0 = c;
        for (; c < c_end; ++c) {
            const int g = find_graph(P.gd, P.n_graphs, c);
            const GraphDesc &G = P.gd[g];
            const int32_t *__restrict__ rp = G.rp;
            const int32_t *__restrict__ col = G.col;
            const int64_t x0 = (c - G.chunk_base) * kWarp;
            const int64_t x = x0 + lane;
            int rs = 0, d = 0, nin = 0;
            unsigned long long w = 0;
            if (x < G.n_rows) {
                rs = __ldg(rp + x);
                d = __ldg(rp + x + 1) - rs;
                nin = P.in_off[G.vbase + x + 1] - P.in_off[G.vbase + x];
                w = P.out_work[G.vbase + x] + (P.in_work[G.vbase + x] & 0xffffffffull);
            }
            // scatter the middle-centric out-edges of the chunk's roots (marked by
            // in_count): short rows one per lane ...
            if (d >= 1 && d <= kLaneRowDeg && x < G.n_roots) {
                for (int i0 = 0; i0 < d; i0 += 4)
                    scatter4(P, G, col + rs, G.ebase + rs, i0, 1, d, (int32_t)x);
            }
            // ... long rows by the whole warp
            unsigned todo = __ballot_sync(kFull, d > kLaneRowDeg && x < G.n_roots);
            while (todo) {
                const int k = __ffs(todo) - 1;
                todo &= todo - 1u;
                const int rrs = __shfl_sync(kFull, rs, k);
                const int rd = __shfl_sync(kFull, d, k);
                for (int i0 = lane; i0 < rd; i0 += 4 * kWarp)
                    scatter4(P, G, col + rrs, G.ebase + rrs, i0, kWarp, rd, (int32_t)(x0 + k));
            }
            // classify
            const bool has = w > 0 && d >= 1;
            const bool micro = has && d <= kMicroDeg && w <= (unsigned long long)kMicroWork;
            const bool light = has && !micro && d <= P.warp_max && w <= light_max;
            const bool hv = has && !micro && !light;
            const uint32_t mm = __ballot_sync(kFull, micro);
            const uint32_t lm = __ballot_sync(kFull, light);
            if (lane == 0) {
                wmask[2 * (c - c0)] = mm;
                wmask[2 * (c - c0) + 1] = lm;
            }
            // the chunk's heavy tasks in one append: a warp scan of their
            // units and one packed 64-bit atomic for the chunk, so entries stay
            // contiguous and sorted by unit.  (One atomic per heavy task on the
            // one hot word serialised the pass when a batch of halo parts holds
            // hundreds of thousands of heavy tasks.)
            const unsigned hm = __ballot_sync(kFull, hv);
            if (hm) {
                unsigned units = 0;
                int ns = 0;
                if (hv) {
                    const int n_part = (x < G.n_roots ? d : 0) + nin;
                    const int max_slices = max(1, (n_part + kHeavyChunk - 1) / kHeavyChunk);
                    ns = (int)min((w + unit - 1) / unit, (unsigned long long)max_slices);
                    ns = max(ns, 1);
                    units = (unsigned)((d + P.tile - 1) / P.tile) * (unsigned)ns;
                }
                unsigned incl = units;
#pragma unroll
                for (int o = 1; o < kWarp; o <<= 1) {
                    const unsigned t = __shfl_up_sync(kFull, incl, o);
                    if (lane >= o) incl += t;
                }
                const unsigned chunk_units = __shfl_sync(kFull, incl, kWarp - 1);
                unsigned long long base = 0;
                if (lane == 0)
                    base = atomicAdd(&P.work->heavy_packed, ((unsigned long long)__popc(hm) << 32) | chunk_units);
                base = __shfl_sync(kFull, base, 0);
                if (hv) {
                    const unsigned long long idx = (base >> 32) + (unsigned)__popc(hm & ((1u << lane) - 1u));
                    if ((int64_t)idx < P.heavy_cap) {
                        HeavyEntry e;
                        e.g = g;
                        e.u = (int32_t)x;
                        e.unit_base = (int32_t)((unsigned)base + (incl - units));
                        e.n_slices = ns;
                        heavy[idx] = e;
                    } else {
                        atomicExch(&P.work->error, 1);
                    }
                }
            }
        }
        // list the grab's micro tasks (from the top) and light tasks (from the
        // bottom): one atomic reserves both lists' slots
        __syncwarp();
        const int nc = (int)(c_end - c0);
        unsigned tm = 0, tl = 0;
        for (int k = 0; k < nc; ++k) {
            tm += __popc(wmask[2 * k]);
            tl += __popc(wmask[2 * k + 1]);
        }
        if (tm | tl) {
            unsigned long long base = 0;
            if (lane == 0) base = atomicAdd(&P.work->n_tasks, (unsigned long long)tl | ((unsigned long long)tm << 32));
            base = __shfl_sync(kFull, base, 0);
            unsigned bm = (unsigned)(base >> 32), bl = (unsigned)base;
            const uint32_t below = (1u << lane) - 1u;
            for (int k = 0; k < nc; ++k) {
                const uint32_t mm = wmask[2 * k], lm = wmask[2 * k + 1];
                const uint32_t row = (uint32_t)((c0 + k) * kWarp + lane);
                if ((mm >> lane) & 1u) P.light_list[P.list_cap - 1 - (int64_t)(bm + __popc(mm & below))] = row;
                if ((lm >> lane) & 1u) P.light_list[bl + __popc(lm & below)] = row;
                bm += __popc(mm);
                bl += __popc(lm);
            }
        }
        __syncwarp();  // wmask is rewritten by the next grab
    }
}

// A micro task compares lists of at most D ids (each loaded in one burst, two
// lists in flight) with its d <= D register ids r; compares stop at the real
// lengths (both sets are duplicate-free).
template <int D>
__device__ __forceinline__ void micro_load(const int32_t *__restrict__ lst, int len, int (&y)[D]) {
#pragma unroll
    for (int t = 0; t < D; ++t) y[t] = t < len ? __ldg(lst + t) : -2;
}

template <int D>
__device__ __forceinline__ uint32_t micro_hits(const int (&y)[D], int len, const int (&r)[D], int d) {
    uint32_t h = 0;
#pragma unroll
    for (int t = 0; t < D; ++t) {
        if (t >= len) break;
#pragma unroll
        for (int q = 0; q < D; ++q) {
            if (q >= d) break;
            h += (uint32_t)(r[q] == y[t]);
        }
    }
    return h;
}

// One micro task x (d+(x) = d <= D) on one lane; returns its hits (credited
// per root when per_root is set).
template <bool kPerRoot, int D>
__device__ __forceinline__ uint32_t micro_task(const KParams &P, const GraphDesc &G, int x, int rs, int d) {
    const int32_t *__restrict__ rp = G.rp;
    const int32_t *__restrict__ col = G.col;
    int r[D];
#pragma unroll
    for (int i = 0; i < D; ++i) r[i] = i < d ? __ldg(col + rs + i) : -1;
    uint32_t own = 0;  // hits credited to x (root-centric partners)
    if (x < G.n_roots) {
        // every out-partner's row bounds at once, then each short list in one burst
        int ps[D], pe[D];
#pragma unroll
        for (int i = 0; i < D; ++i) {
            ps[i] = r[i] >= 0 ? __ldg(rp + r[i]) : 0;
            pe[i] = r[i] >= 0 ? __ldg(rp + r[i] + 1) : 0;
        }
#pragma unroll
        for (int i = 0; i < D; i += 2) {
            if (i >= d) break;
            // a list longer than d is middle-centric: done from p's side
            const int la = pe[i] - ps[i] <= d ? pe[i] - ps[i] : 0;
            const int lb = pe[i + 1] - ps[i + 1] <= d ? pe[i + 1] - ps[i + 1] : 0;
            int ya[D], yb[D];
            micro_load<D>(col + ps[i], la, ya);
            micro_load<D>(col + ps[i + 1], lb, yb);
            own += micro_hits<D>(ya, la, r, d) + micro_hits<D>(yb, lb, r, d);
        }
    }
    uint32_t in_hits = 0;
    const int i0 = P.in_off[G.vbase + x], i1 = P.in_off[G.vbase + x + 1];
    for (int k = i0; k < i1; k += 2) {  // in-partners (d+(u) < d+(x)), two at a time
        const int pa = P.in_list[k];
        const int pb = k + 1 < i1 ? P.in_list[k + 1] : -1;
        const int sa = __ldg(rp + pa), la = __ldg(rp + pa + 1) - sa;
        const int sb = pb >= 0 ? __ldg(rp + pb) : 0, lb = pb >= 0 ? __ldg(rp + pb + 1) - sb : 0;
        int ya[D], yb[D];
        micro_load<D>(col + sa, la, ya);
        micro_load<D>(col + sb, lb, yb);
        const uint32_t ha = micro_hits<D>(ya, la, r, d), hb = micro_hits<D>(yb, lb, r, d);
        in_hits += ha + hb;
        if (kPerRoot && ha) atomicAdd(G.per_root + pa, (unsigned long long)ha);
        if (kPerRoot && hb) atomicAdd(G.per_root + pb, (unsigned long long)hb);
    }
    if (kPerRoot && own) atomicAdd(G.per_root + x, (unsigned long long)own);
    return own + in_hits;
}

// micro tasks: one lane runs a whole task x (d+(x) <= kMicroDeg, work <=
// kMicroWork) with N+(x) in registers; every streamed partner list is then at
// most kMicroDeg long (the cheaper side), and membership is predicated
// compares -- no hash table, no shared memory.  Tasks with d+(x) <= 4 (most
// of a road network's) take a 4-wide path: a quarter of the compares.  Warps
// take 32 consecutive tasks from the top of the task list, so every lane has
// one (a chunk of 32 rows holds only a few micro tasks on most graphs).
template <bool kPerRoot>
__global__ void __launch_bounds__(kThreads) micro_kernel(KParams P) {
    const int lane = threadIdx.x & (kWarp - 1);
    const int64_t n = (int64_t)(P.work->n_tasks >> 32);
    const int64_t gwarp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / kWarp;
    const int64_t nwarps = (int64_t)gridDim.x * blockDim.x / kWarp;
    unsigned long long acc = 0;  // this lane's hits for graph cur_g
    int cur_g = -1;
    for (int64_t b = gwarp * kWarp; b < n; b += nwarps * kWarp) {
        const int64_t t = b + lane;
        if (t >= n) break;
        const uint32_t gi = P.light_list[P.list_cap - 1 - t];
        const int64_t c = (int64_t)(gi / kWarp);
        const int g = find_graph(P.gd, P.n_graphs, c);
        const GraphDesc &G = P.gd[g];
        const int x = (int)((c - G.chunk_base) * kWarp + (int64_t)(gi % kWarp));
        const int rs = __ldg(G.rp + x);
        const int d = __ldg(G.rp + x + 1) - rs;
        const uint32_t h = d <= 4 ? micro_task<kPerRoot, 4>(P, G, x, rs, d)
                                  : micro_task<kPerRoot, kMicroDeg>(P, G, x, rs, d);
        if (!kPerRoot) {
            if (g != cur_g) {  // a batch's next graph: this lane's hits so far go out
                if (cur_g >= 0 && acc) atomicAdd(P.results + cur_g, acc);
                acc = 0;
                cur_g = g;
            }
            acc += h;
        }
    }
    if (!kPerRoot) {  // one atomic per warp when its lanes ended on one graph
        const int g0 = __reduce_max_sync(kFull, cur_g);
        if (__all_sync(kFull, cur_g < 0 || cur_g == g0)) {
            const unsigned long long s = warp_sum_u64(acc);
            if (lane == 0 && g0 >= 0 && s) atomicAdd(P.results + g0, s);
        } else if (cur_g >= 0 && acc) {
            atomicAdd(P.results + cur_g, acc);
        }
    }
}

// flat count: for graphs whose every row has at most D entries, one lane per
// root u holds N+(u) in registers and compares every N+(v), v in N+(u),
// against it -- the reference's per-edge intersection, with no transpose, no
// classification and no hash tables.  Row bounds of all v are loaded at once
// and two lists are in flight, as in the micro tasks.  The lanes wait on four
// dependent loads per root, so residency is what hides it.  This is the
// 8-wide count (rows of 5..8 entries); flat4_kernel below counts graphs whose
// rows have at most 4.
template <bool kPerRoot, int D>
__global__ void __launch_bounds__(kThreads) flat_kernel(const int32_t *__restrict__ rp, const int32_t *__restrict__ col,
                                                        int64_t n_roots, unsigned long long *result,
                                                        unsigned long long *per_root) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    unsigned long long acc = 0;
    for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < n_roots; u += stride) {
        const int rs = __ldg(rp + u);
        const int d = __ldg(rp + u + 1) - rs;
        int r[D];
#pragma unroll
        for (int i = 0; i < D; ++i) r[i] = i < d ? __ldg(col + rs + i) : -1;
        int ps[D], pe[D];
#pragma unroll
        for (int i = 0; i < D; ++i) {
            ps[i] = r[i] >= 0 ? __ldg(rp + r[i]) : 0;
            pe[i] = r[i] >= 0 ? __ldg(rp + r[i] + 1) : 0;
        }
        uint32_t h = 0;
#pragma unroll
        for (int i = 0; i < D; i += 2) {
            if (i >= d) break;
            const int la = pe[i] - ps[i], lb = pe[i + 1] - ps[i + 1];
            int ya[D], yb[D];
            micro_load<D>(col + ps[i], la, ya);
            micro_load<D>(col + ps[i + 1], lb, yb);
            h += micro_hits<D>(ya, la, r, d) + micro_hits<D>(yb, lb, r, d);
        }
        if (kPerRoot) per_root[u] = h;
        acc += h;
    }
    acc = warp_sum_u64(acc);
    if ((threadIdx.x & (kWarp - 1)) == 0 && acc) atomicAdd(result, acc);
}

// The 4-wide flat count with each lane pipelining its roots: the next root's
// row loads (bounds, then list) go out beside this root's neighbour loads, so
// a root costs two dependent load rounds instead of four.  It runs one
// resident wave (6 blocks per SM at 40 registers: the extra registers of the
// pipeline spill at 32); road networks count ~30% faster than with a lane
// per root.  The 8-wide count keeps the plain form: at 80 registers the
// pipelined one loses the residency it needs.
template <bool kPerRoot>
__global__ void __launch_bounds__(kThreads, kPerRoot ? 1 : 6) flat4_kernel(const int32_t *__restrict__ rp,
                                                                          const int32_t *__restrict__ col,
                                                                          int64_t n_roots, unsigned long long *result,
                                                                          unsigned long long *per_root) {
    constexpr int D = 4;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    unsigned long long acc = 0;
    int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int d = 0, r[D];  // this root's row, loaded ahead
    {
        int rs = 0;
        if (u < n_roots) {
            rs = __ldg(rp + u);
            d = __ldg(rp + u + 1) - rs;
        }
#pragma unroll
        for (int i = 0; i < D; ++i) r[i] = i < d ? __ldg(col + rs + i) : -1;
    }
    for (; u < n_roots; u += stride) {
        const int64_t un = u + stride;
        int rsn = 0, dn = 0;
        if (un < n_roots) {
            rsn = __ldg(rp + un);
            dn = __ldg(rp + un + 1) - rsn;
        }
        int ps[D], pe[D];
#pragma unroll
        for (int i = 0; i < D; ++i) {
            ps[i] = r[i] >= 0 ? __ldg(rp + r[i]) : 0;
            pe[i] = r[i] >= 0 ? __ldg(rp + r[i] + 1) : 0;
        }
        int rn[D];
#pragma unroll
        for (int i = 0; i < D; ++i) rn[i] = i < dn ? __ldg(col + rsn + i) : -1;
        uint32_t h = 0;
#pragma unroll
        for (int i = 0; i < D; i += 2) {
            if (i >= d) break;
            const int la = pe[i] - ps[i], lb = pe[i + 1] - ps[i + 1];
            int ya[D], yb[D];
            micro_load<D>(col + ps[i], la, ya);
            micro_load<D>(col + ps[i + 1], lb, yb);
            h += micro_hits<D>(ya, la, r, d) + micro_hits<D>(yb, lb, r, d);
        }
        if (kPerRoot) per_root[u] = h;
        acc += h;
        d = dn;
#pragma unroll
        for (int i = 0; i < D; ++i) r[i] = rn[i];
    }
    acc = warp_sum_u64(acc);
    if ((threadIdx.x & (kWarp - 1)) == 0 && acc) atomicAdd(result, acc);
}

// Heavy units with a direct-address bitmap of N+(x) over all vertex ids in
// shared memory (graphs of at most bitmap_words * 32 rows): one shared load per
// probe instead of the two of the cuckoo hash, and no tiling of N+(x).  One
// kBigThreads block per SM drains the heavy-unit cursor before count_kernel
// runs (which then finds no heavy units left).  Bits are set for the unit's
// N+(x) and cleared again (their words zeroed) when the next unit needs
// another set.
constexpr int kBigThreads = 1024;

template <bool kPerRoot>
__global__ void __launch_bounds__(kBigThreads, 1) heavy_bitmap_kernel(KParams P, int bitmap_words) {
    extern __shared__ int bm[];
    __shared__ unsigned s_unit;
    __shared__ int s_entry;
    __shared__ int s_chunk;
    const int lane = threadIdx.x & (kWarp - 1);
    const int warp = threadIdx.x / kWarp;
    if (P.work->error) return;
    const unsigned long long packed = P.work->heavy_packed;
    const unsigned n_entries = (unsigned)min((unsigned long long)(packed >> 32), (unsigned long long)P.heavy_cap);
    const unsigned n_units = (unsigned)(packed & 0xffffffffull);
    if (n_units == 0) return;
    for (int i = threadIdx.x; i < bitmap_words; i += kBigThreads) bm[i] = 0;
    unsigned long long acc = 0;
    int cur_g = -1;
    int set_entry = -1;  // entry whose N+(x) bits are set
    const int32_t *set_list = nullptr;
    int set_len = 0;
    for (;;) {
        if (warp == 0) {
            unsigned unit = 0;
            if (lane == 0) unit = atomicAdd(&P.work->heavy_cursor, 1u);
            unit = __shfl_sync(kFull, unit, 0);
            int e = -1;
            if (unit < n_units && n_entries > 0) {
                int lo = 0, hi = (int)n_entries;
                while (hi - lo > kWarp) {
                    const int step = (hi - lo + kWarp - 1) / kWarp;
                    const int idx = lo + lane * step;
                    const bool le = idx < hi && (unsigned)P.heavy[idx].unit_base <= unit;
                    const unsigned m = __ballot_sync(kFull, le);
                    lo += (31 - __clz(m)) * step;
                    hi = min(hi, lo + step);
                }
                const bool le = lo + lane < hi && (unsigned)P.heavy[lo + lane].unit_base <= unit;
                e = lo + 31 - __clz(__ballot_sync(kFull, le));
            }
            if (lane == 0) {
                s_unit = unit;
                s_entry = e;
                s_chunk = 0;
            }
        }
        __syncthreads();
        const unsigned unit = s_unit;
        const int ei = s_entry;
        if (ei < 0) break;
        const HeavyEntry e = P.heavy[ei];
        const GraphDesc &G = P.gd[e.g];
        const int32_t *__restrict__ rp = G.rp;
        const int32_t *__restrict__ col = G.col;
        Task T;
        const int rs = __ldg(rp + e.u);
        T.dx = __ldg(rp + e.u + 1) - rs;
        T.x = e.u;
        T.n_out = e.u < G.n_roots ? T.dx : 0;
        T.out_nbr = col + rs;
        const int in0 = P.in_off[G.vbase + e.u];
        T.in_nbr = P.in_list + in0;
        const int n_part = T.n_out + (P.in_off[G.vbase + e.u + 1] - in0);
        if (ei != set_entry) {
            for (int i = threadIdx.x; i < set_len; i += kBigThreads) bm[(unsigned)__ldg(set_list + i) >> 5] = 0;
            __syncthreads();
            for (int i = threadIdx.x; i < T.dx; i += kBigThreads) {
                const int y = __ldg(col + rs + i);
                atomicOr(&bm[(unsigned)y >> 5], 1 << (y & 31));
            }
            set_entry = ei;
            set_list = col + rs;
            set_len = T.dx;
        }
        __syncthreads();
        const int ns = e.n_slices;
        const int si = (int)(unit - (unsigned)e.unit_base);
        const int per = (n_part + ns - 1) / ns;
        const int j0 = si * per, j1 = min(n_part, j0 + per);
        uint32_t hits = 0;
        for (;;) {
            int c = 0;
            if (lane == 0) c = atomicAdd(&s_chunk, 1);
            c = __shfl_sync(kFull, c, 0);
            const int jb = j0 + c * kHeavyChunk;
            if (jb >= j1) break;
            hits += probe_partners<kPerRoot, true>(rp, col, T, jb, min(jb + kHeavyChunk, j1), bm, 0, 0, kLinear,
                                                   P.long_list, lane, G.per_root);
        }
        if (!kPerRoot) {
            if (e.g != cur_g) {
                const unsigned long long s = warp_sum_u64(acc);
                if (lane == 0 && cur_g >= 0 && s) atomicAdd(P.results + cur_g, s);
                acc = 0;
                cur_g = e.g;
            }
            acc += hits;
        }
        __syncthreads();
    }
    if (!kPerRoot) {
        const unsigned long long s = warp_sum_u64(acc);
        if (lane == 0 && cur_g >= 0 && s) atomicAdd(P.results + cur_g, s);
    }
}

// kParts: the launch holds halo parts (roots a prefix of the rows): heavy
// units grab fewer partners when they have few, and warp 0 takes the next
// unit while the other warps finish the current one (below).  Whole graphs
// get the instance without either: the same rules cost them 2-3 % (R-MAT 21
// 6.03 -> 6.21 ms, R-MAT 23 33.8 -> 34.6 ms) even where they never fire.
// kPhases: 3 = both phases in one kernel, 1 = phase A only (heavy units),
// 2 = phase B only (light tasks).  Launches with halo parts run the two
// phases as two kernels, each with its own register allocation: in one
// kernel, phase B's live values made the halo-part instance spill 108 bytes
// at 40 registers and its phase A ran ~2 ms slower on R-MAT 23's eight parts
// (per-block %globaltimer stamps: phase A ended at 33.9 ms with phase B in
// the kernel, 31.8 ms without); split, those parts count in 38.09 instead of
// 40.47 ms and R-MAT 21's in 7.89 instead of 8.26.  Whole graphs keep one
// kernel: there the blocks that finish phase A early fill its tail with light
// tasks, which two kernels cannot (R-MAT 21 6.65 -> 7.08 ms split).  Light
// tasks do not depend on heavy units (the totals are atomic adds), so only
// the schedule differs.
template <bool kPerRoot, bool kPairsOnly, bool kStage = false, bool kParts = false, int kPhases = 3>
__global__ void __launch_bounds__(kThreads, TC_COUNT_MIN_BLOCKS) count_kernel(KParams P) {
    extern __shared__ __align__(16) int smem[];
    __shared__ unsigned s_unit;
    __shared__ int s_entry;
    __shared__ int s_chunk;
    __shared__ __align__(8) unsigned long long s_bar[kWarpsPerBlock + 1];  // bulk-copy barriers: per warp, block
    const int lane = threadIdx.x & (kWarp - 1);
    const int warp = threadIdx.x / kWarp;

    unsigned long long acc = 0;  // this lane's partial for graph cur_g
    int cur_g = -1;
    auto flush = [&](int next_g) {
        const unsigned long long s = warp_sum_u64(acc);
        if (lane == 0 && cur_g >= 0 && s) atomicAdd(P.results + cur_g, s);
        acc = 0;
        cur_g = next_g;
    };

    if (P.work->error) return;
    const unsigned long long packed = P.work->heavy_packed;
    const unsigned n_entries = (unsigned)min((unsigned long long)(packed >> 32), (unsigned long long)P.heavy_cap);
    const unsigned n_units = (unsigned)(packed & 0xffffffffull);
    // sorted-list tasks stage their list with bulk copies (uniform: a kernel parameter)
    const bool staging = kStage && !kPairsOnly && P.intersect != 0;
    uint32_t bphase = 0, wphase = 0;  // parity of the block's and this warp's barrier
    bool stage_ok = true;
    // The block's (warp's) shared region was last written by generic stores
    // (a hash table, or the plain-load part of a staged list): a bulk copy over
    // it must first be ordered after them by a proxy fence.
    bool block_dirty = false, warp_dirty = false;
    if (staging) {
        if (threadIdx.x <= kWarpsPerBlock) mbar_init(&s_bar[threadIdx.x], 1);
        mbar_fence_init();
        __syncthreads();
    }

    // ---- phase A: heavy units, one block each ----
    int cached_entry = -1, cached_tile = -1;
    int cached_mode = kLinear;
    const int *cached_tab = smem;
    // Warp 0 takes a unit: its number and heavy entry (-1 when none is left).
    // With kParts it takes the next unit as soon as it has no partners of the
    // current one left to probe, so the grab's atomic and the dependent loads
    // of its 32-ary search overlap the other warps' last probes instead of
    // idling the whole block after the unit (a halo part's units are many and
    // small); otherwise at the top of each unit.
    auto grab_next = [&]() {
        unsigned unit = 0;
        if (lane == 0) unit = atomicAdd(&P.work->heavy_cursor, 1u);
        unit = __shfl_sync(kFull, unit, 0);
        unsigned ne = n_entries, nu = n_units;
        if (kParts) {  // re-read here rather than kept live across the probes
            const unsigned long long pk = __ldg(&P.work->heavy_packed);
            ne = (unsigned)min((unsigned long long)(pk >> 32), (unsigned long long)P.heavy_cap);
            nu = (unsigned)(pk & 0xffffffffull);
        }
        int e = -1;
        if (unit < nu && ne > 0) {
            // last entry with unit_base <= unit (entries ascend; entry 0 starts at unit 0):
            // 32-ary search, one dependent load per round
            int lo = 0, hi = (int)ne;
            while (hi - lo > kWarp) {
                const int step = (hi - lo + kWarp - 1) / kWarp;
                const int idx = lo + lane * step;
                const bool le = idx < hi && (unsigned)P.heavy[idx].unit_base <= unit;
                const unsigned m = __ballot_sync(kFull, le);
                lo += (31 - __clz(m)) * step;
                hi = min(hi, lo + step);
            }
            const bool le = lo + lane < hi && (unsigned)P.heavy[lo + lane].unit_base <= unit;
            e = lo + 31 - __clz(__ballot_sync(kFull, le));
        }
        if (lane == 0) {
            s_unit = unit;
            s_entry = e;
            if (!kParts) s_chunk = 0;
        }
    };
    if (kParts && (kPhases & 1) && !P.heavy_done && warp == 0) grab_next();
    for (; (kPhases & 1) && !P.heavy_done;) {
        if (!kParts && warp == 0) grab_next();
        __syncthreads();  // this unit's s_unit / s_entry are set (and the last unit's probes are done)
        const unsigned unit = s_unit;
        const int ei = s_entry;
        if (ei < 0) break;
        if (kParts && threadIdx.x == 0) s_chunk = 0;
        const HeavyEntry e = P.heavy[ei];
        const GraphDesc &G = P.gd[e.g];
        const int32_t *__restrict__ rp = G.rp;
        const int32_t *__restrict__ col = G.col;
        Task T;
        const int rs = __ldg(rp + e.u);
        T.dx = __ldg(rp + e.u + 1) - rs;
        T.x = e.u;
        T.n_out = e.u < G.n_roots ? T.dx : 0;
        T.out_nbr = col + rs;
        const int in0 = P.in_off[G.vbase + e.u];
        T.in_nbr = P.in_list + in0;
        const int n_part = T.n_out + (P.in_off[G.vbase + e.u + 1] - in0);
        const int ns = e.n_slices;
        const int k = (int)(unit - (unsigned)e.unit_base);
        const int ti = k / ns, si = k - ti * ns;
        const int t0 = ti * P.tile;
        const int tl = min(T.dx - t0, P.tile);
        const int lg = table_log_slots(tl);
        const uint32_t mask = (1u << lg) - 1u;
        const int shift = 32 - lg;
        if (ei != cached_entry || ti != cached_tile) {
            if (staging && P.intersect == 1) {
                // the tile as it lies (sorted) by one bulk copy: no clear, no inserts
                const int64_t lim4 = (int64_t)__ldg(rp + G.n_rows) & ~(int64_t)3;
                const uint32_t bytes = stage_bytes(col, lim4, rs + t0, tl);
                if (bytes && block_dirty) {
                    fence_proxy_async();
                    __syncthreads();
                }
                if (threadIdx.x == 0 && bytes) stage_issue(col, lim4, rs + t0, tl, smem, &s_bar[kWarpsPerBlock]);
                block_dirty = stage_rest(col, lim4, rs + t0, tl, smem, threadIdx.x, kThreads);
                if (bytes) {
                    if (!mbar_wait(&s_bar[kWarpsPerBlock], bphase)) {
                        stage_ok = false;
                        mbar_wait(&s_bar[kWarpsPerBlock], bphase);  // the copy in flight, bounded again
                    }
                    bphase ^= 1u;
                }
                cached_mode = kSorted;
                cached_tab = smem + ((rs + t0) & 3);
            } else {
                table_clear(smem, mask, threadIdx.x, kThreads);
                __syncthreads();
                bool ok = true;
                cached_mode = table_fill<kPairsOnly>(smem, mask, shift, col + rs + t0, tl, threadIdx.x, kThreads,
                                                     P.table_mode, P.probe_kicks, &ok);
                if (__syncthreads_or(!ok)) {  // a cuckoo give-up: linear probing instead
                    table_clear(smem, mask, threadIdx.x, kThreads);
                    __syncthreads();
                    cached_mode = table_fill<false>(smem, mask, shift, col + rs + t0, tl, threadIdx.x, kThreads,
                                                    kLinear, 0, &ok);
                }
                cached_tab = smem;
                block_dirty = true;
            }
            cached_entry = ei;
            cached_tile = ti;
        }
        if (staging && __syncthreads_or(!stage_ok)) {  // a staging wait gave up: report, stop
            if (threadIdx.x == 0) atomicExch(&P.work->error, 2);
            return;
        }
        __syncthreads();
        const int per = (n_part + ns - 1) / ns;
        const int j0 = si * per, j1 = min(n_part, j0 + per);
        const uint32_t pmask = cached_mode == kSorted ? (uint32_t)tl : mask;
        // partners per grab: kHeavyChunk; in halo parts (kParts) fewer when the
        // unit has fewer than kHeavyChunk partners per warp, so that every warp
        // gets a grab.  A hub's unit in a halo part
        // holds only that part's in-partners: at 16 per grab several warps
        // waited at the barrier below (barrier stalls 5.4 per issue on R-MAT
        // 21's eight parts; R-MAT 23's eight parts 41.0 -> 39.1 ms).  Whole
        // graphs keep 16: smaller grabs there cost 2-3% (fewer short lists per
        // grab to flatten across the lanes).
        const int chunk = kParts ? max(1, min(kHeavyChunk, (j1 - j0 + kWarpsPerBlock - 1) / kWarpsPerBlock))
                                 : kHeavyChunk;
        uint32_t hits = 0;
        for (;;) {
            int c = 0;
            if (lane == 0) c = atomicAdd(&s_chunk, 1);
            c = __shfl_sync(kFull, c, 0);
            const int jb = j0 + c * chunk;
            if (jb >= j1) break;
            hits += probe_partners<kPerRoot, false, kPairsOnly, kStage>(rp, col, T, jb, min(jb + chunk, j1), cached_tab,
                                                                pmask, shift, cached_mode, P.long_list, lane,
                                                                G.per_root);
        }
        if (!kPerRoot) {
            if (e.g != cur_g) flush(e.g);
            acc += hits;
        }
        if (kParts) {
            if (warp == 0) grab_next();  // while the other warps finish their grabs
        } else {
            __syncthreads();
        }
    }
    warp_dirty = block_dirty;  // the warp regions lie in the block's region

    // ---- phase B: light tasks, one warp each ----
    // Warps take kLightGrab tasks at a time from the classifier's list, so the
    // last tasks of the kernel are single tasks, not whole 32-row chunks.
    int *wtab = smem + warp * (1 << P.log_warp_slots);
    const unsigned n_light = (unsigned)P.work->n_tasks;
    for (; kPhases & 2;) {
        unsigned t0 = 0;
        if (lane == 0) t0 = atomicAdd(&P.work->small_cursor, (unsigned)(kParts ? 8 : kLightGrab));
        t0 = __shfl_sync(kFull, t0, 0);
        if (t0 >= n_light) break;
        const int nt = (int)min((unsigned)(kParts ? 8 : kLightGrab), n_light - t0);
        // the grabbed tasks' rows, one lane each
        int rs = 0, d = 0, i0 = 0, i1 = 0, tg = 0, tx = 0;
        unsigned long long tw = 0;  // the task's work (probes), for the per-task switch
        if (lane < nt) {
            const uint32_t gi = P.light_list[t0 + lane];
            const int64_t c = (int64_t)(gi / kWarp);
            tg = find_graph(P.gd, P.n_graphs, c);
            const GraphDesc &Gl = P.gd[tg];
            tx = (int)((c - Gl.chunk_base) * kWarp + (int64_t)(gi % kWarp));
            rs = __ldg(Gl.rp + tx);
            d = __ldg(Gl.rp + tx + 1) - rs;
            i0 = P.in_off[Gl.vbase + tx];
            i1 = P.in_off[Gl.vbase + tx + 1];
            if (staging && P.intersect == 2)
                tw = P.out_work[Gl.vbase + tx] + (P.in_work[Gl.vbase + tx] & 0xffffffffull);
        }
        for (int k = 0; k < nt; ++k) {
            const int g = __shfl_sync(kFull, tg, k);
            const GraphDesc &G = P.gd[g];
            const int32_t *__restrict__ rp = G.rp;
            const int32_t *__restrict__ col = G.col;
            if (!kPerRoot && g != cur_g) flush(g);
            Task T;
            const int rrs = __shfl_sync(kFull, rs, k);
            T.dx = __shfl_sync(kFull, d, k);
            T.x = __shfl_sync(kFull, tx, k);
            T.n_out = T.x < G.n_roots ? T.dx : 0;
            T.out_nbr = col + rrs;
            const int ri0 = __shfl_sync(kFull, i0, k);
            T.in_nbr = P.in_list + ri0;
            const int n_part = T.n_out + (__shfl_sync(kFull, i1, k) - ri0);
            const int lg = table_log_slots(T.dx);
            uint32_t mask = (1u << lg) - 1u;
            const int shift = 32 - lg;
            int mode;
            const int *tab = wtab;
            const unsigned long long task_w = __shfl_sync(kFull, tw, k);
            if (staging && (P.intersect == 1 || task_w < (unsigned long long)T.dx)) {
                // few probes for the list's length (or every task): the list as it
                // lies, bulk-copied, instead of a table built for it
                const int64_t lim4 = (int64_t)__ldg(rp + G.n_rows) & ~(int64_t)3;
                const uint32_t bytes = stage_bytes(col, lim4, rrs, T.dx);
                if (bytes && warp_dirty) {
                    fence_proxy_async();
                    __syncwarp();
                }
                if (lane == 0 && bytes) stage_issue(col, lim4, rrs, T.dx, wtab, &s_bar[warp]);
                warp_dirty = stage_rest(col, lim4, rrs, T.dx, wtab, lane, kWarp);
                if (bytes) {
                    if (!mbar_wait(&s_bar[warp], wphase)) {
                        stage_ok = false;
                        mbar_wait(&s_bar[warp], wphase);  // the copy in flight, bounded again
                    }
                    wphase ^= 1u;
                }
                mode = kSorted;
                tab = wtab + (rrs & 3);
                mask = (uint32_t)T.dx;
            } else {
                table_clear(wtab, mask, lane, kWarp);
                __syncwarp();
                bool ok = true;
                mode = table_fill<kPairsOnly>(wtab, mask, shift, col + rrs, T.dx, lane, kWarp, P.table_mode,
                                              P.probe_kicks, &ok);
                if (!__all_sync(kFull, ok)) {  // a cuckoo give-up: linear probing instead
                    __syncwarp();
                    table_clear(wtab, mask, lane, kWarp);
                    __syncwarp();
                    mode = table_fill<false>(wtab, mask, shift, col + rrs, T.dx, lane, kWarp, kLinear, 0, &ok);
                }
                warp_dirty = true;
            }
            if (staging && __any_sync(kFull, !stage_ok)) {  // a staging wait gave up: report, stop
                if (lane == 0) atomicExch(&P.work->error, 2);
                return;
            }
            __syncwarp();
            uint32_t hits = 0;
            for (int jb = 0; jb < n_part; jb += kWarp)
                hits += probe_partners<kPerRoot, false, kPairsOnly, kStage>(rp, col, T, jb, min(jb + kWarp, n_part), tab, mask,
                                                                    shift, mode, P.long_list, lane, G.per_root);
            __syncwarp();
            if (!kPerRoot) acc += hits;
        }
    }
    if (!kPerRoot) flush(-1);
}

// Dynamic shared memory of the kernels launch_phases runs for one instance.
template <bool kPerRoot, bool kPairsOnly, bool kStage = false, bool kParts = false>
int set_count_smem(size_t smem) {
    if constexpr (!kParts) {
        TC_CUDA(cudaFuncSetAttribute(count_kernel<kPerRoot, kPairsOnly, kStage, kParts, 3>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    } else {
        TC_CUDA(cudaFuncSetAttribute(count_kernel<kPerRoot, kPairsOnly, kStage, kParts, 1>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        TC_CUDA(cudaFuncSetAttribute(count_kernel<kPerRoot, kPairsOnly, kStage, kParts, 2>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    }
    return TC_OK;
}

// The count of one instance on s: one kernel for both phases, or (halo
// parts) phase A's kernel -- unless the bitmap kernel took the heavy units --
// and then phase B's; returns the launches.
template <bool kPerRoot, bool kPairsOnly, bool kStage = false, bool kParts = false>
int launch_phases(const KParams &P, const Tuned &tn, cudaStream_t s) {
    if constexpr (!kParts) {
        count_kernel<kPerRoot, kPairsOnly, kStage, kParts, 3><<<tn.blocks, kThreads, tn.smem, s>>>(P);
        return 1;
    } else {
        int n = 0;
        if (!P.heavy_done) {
            count_kernel<kPerRoot, kPairsOnly, kStage, kParts, 1><<<tn.blocks, kThreads, tn.smem, s>>>(P);
            ++n;
        }
        count_kernel<kPerRoot, kPairsOnly, kStage, kParts, 2><<<tn.blocks, kThreads, tn.smem, s>>>(P);
        return n + 1;
    }
}

int pow2_floor_log(int x) {
    int l = 0;
    while ((2 << l) <= x) ++l;
    return l;
}

}  // namespace

int resolve_tuning(const tc_tuning &t, int sm_count, Tuned *out) {
    Tuned r;
    const int wm = t.warp_max_deg > 0 ? t.warp_max_deg : 256;
    if (wm < 32 || wm > 512 || (wm & (wm - 1)))
        return set_error(TC_E_INVALID, "warp_max_deg must be a power of two in [32, 512], got %d", wm);
    r.warp_max = wm;
    r.log_warp_slots = pow2_floor_log(4 * wm);
    const int warp_slots_total = kWarpsPerBlock * (1 << r.log_warp_slots);
    const int block_slots = std::max(8192, warp_slots_total);
    r.log_block_slots = pow2_floor_log(block_slots);
    r.tile = block_slots / 4;
    r.light_max_work = t.light_max_work > 0 ? t.light_max_work : 8192;
    // 2^20 probes per heavy unit: against 2^18, R-MAT 23 36.85 -> 36.10 ms whole and
    // 40.97 -> 40.65 ms in eight halo parts, R-MAT 21 6.70 -> 6.65 ms (fewer table
    // builds per hub; the persistent grid's dynamic grabs keep the blocks balanced)
    r.unit_work = t.unit_work > 0 ? t.unit_work : 1048576;
    r.long_list = t.long_list >= 0 ? t.long_list : 32;
    r.probe_kicks = t.probe_kicks >= 0 ? t.probe_kicks : 32;
    r.heavy_bitmap = t.heavy_bitmap >= 0 ? t.heavy_bitmap : 0;
    r.hash_pairs = t.hash_pairs >= 0 ? t.hash_pairs : 0;
    if (r.hash_pairs > 1) return set_error(TC_E_INVALID, "hash_pairs must be 0 or 1, got %d", r.hash_pairs);
    r.flat_max_deg = t.flat_max_deg >= 0 ? t.flat_max_deg : 8;
    r.intersect = t.intersect >= 0 ? t.intersect : 0;
    if (r.intersect > 2) return set_error(TC_E_INVALID, "intersect must be 0, 1 or 2, got %d", r.intersect);
    if (r.flat_max_deg > kMicroDeg)
        return set_error(TC_E_INVALID, "flat_max_deg must be in [0, %d], got %d", kMicroDeg, r.flat_max_deg);
    r.sm_count = sm_count;
    {
        // the bitmap takes what one block may opt into, minus the kernel's static shared memory
        int dev = 0, optin = 0;
        TC_CUDA(cudaGetDevice(&dev));
        TC_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
        cudaFuncAttributes fa;
        TC_CUDA(cudaFuncGetAttributes(&fa, heavy_bitmap_kernel<true>));
        r.bitmap_bytes = std::max(0, (optin - (int)fa.sharedSizeBytes - 256) & ~255);
        TC_CUDA(cudaFuncSetAttribute(heavy_bitmap_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     r.bitmap_bytes));
        TC_CUDA(cudaFuncSetAttribute(heavy_bitmap_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     r.bitmap_bytes));
    }
    if (r.probe_kicks > 1024) return set_error(TC_E_INVALID, "probe_kicks must be <= 1024, got %d", r.probe_kicks);
    if (r.long_list > 4096) return set_error(TC_E_INVALID, "long_list must be <= 4096, got %d", r.long_list);
    r.threads = kThreads;
    r.smem = (size_t)block_slots * sizeof(int);
    TC_TRY((set_count_smem<false, false>(r.smem)));
    TC_TRY((set_count_smem<true, false>(r.smem)));
    TC_TRY((set_count_smem<false, true>(r.smem)));
    TC_TRY((set_count_smem<true, true>(r.smem)));
    TC_TRY((set_count_smem<false, false, true>(r.smem)));
    TC_TRY((set_count_smem<true, false, true>(r.smem)));
    TC_TRY((set_count_smem<false, false, false, true>(r.smem)));
    TC_TRY((set_count_smem<true, false, false, true>(r.smem)));
    int occ = 0;
    TC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, count_kernel<false, false>, kThreads, r.smem));
    if (occ < 1) return set_error(TC_E_INVALID, "count kernel does not fit on an SM with %zu B shared memory", r.smem);
    const int bps = t.blocks_per_sm > 0 ? std::min(t.blocks_per_sm, occ) : occ;
    r.blocks = sm_count * bps;
    // The auxiliary kernels walk the 32-row chunks grid-stride.  With no more
    // blocks than fit on the GPU at once, the chunks in flight form one moving
    // window, so a batch touches its graphs (and their in-lists) one after the
    // other instead of all at once, and heavy entries come out graph-ordered.
    int aux_occ = 0, o = 0;
    TC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, in_count_kernel, kThreads, 0));
    aux_occ = o;
    TC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, transpose_classify_kernel, kThreads, 0));
    aux_occ = std::min(aux_occ, o);
    TC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, micro_kernel<false>, kThreads, 0));
    aux_occ = std::min(aux_occ, o);
    TC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, micro_kernel<true>, kThreads, 0));
    aux_occ = std::min(aux_occ, o);
    r.aux_blocks = sm_count * std::max(1, aux_occ);
    *out = r;
    return TC_OK;
}

// Launches of one scan of n values: one tile, or reduce + the tile sums' scan + scan.
static int scan_launches(int64_t n) {
    constexpr int64_t kScanTile = 4096;
    return n <= kScanTile ? 1 : 2 + scan_launches((n + kScanTile - 1) / kScanTile);
}

// Records a kernel-timing event on s; inside a stream capture (the plain
// count's cached graph) as an external event node, so that every replay of
// the captured chain records it too.
static int record_kernel_event(cudaEvent_t ev, cudaStream_t s) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    TC_CUDA(cudaStreamIsCapturing(s, &cs));
    if (cs == cudaStreamCaptureStatusActive) TC_CUDA(cudaEventRecordWithFlags(ev, s, cudaEventRecordExternal));
    else TC_CUDA(cudaEventRecord(ev, s));
    return TC_OK;
}

int launch_count(const GraphDesc *d_desc, int n_graphs, int64_t total_chunks, int64_t total_vertices,
                 int64_t max_rows, const CountScratch &sc, CountWork *work, unsigned long long *results, bool per_root,
                 const Tuned &tn, cudaStream_t s, int *launches, cudaEvent_t *kev, bool halo_parts) {
    KParams P;
    P.gd = d_desc;
    P.n_graphs = n_graphs;
    P.total_chunks = total_chunks;
    P.heavy = sc.heavy;
    P.heavy_cap = sc.heavy_cap;
    P.work = work;
    P.results = results;
    P.light_list = sc.light_list;
    P.list_cap = total_vertices;
    P.in_cnt = sc.in_cnt;
    P.in_off = sc.in_off;
    P.in_work = sc.in_work;
    P.out_work = sc.out_work;
    P.in_list = sc.in_list;
    P.mid = sc.mid;
    P.warp_max = tn.warp_max;
    P.log_warp_slots = tn.log_warp_slots;
    P.light_max_work = tn.light_max_work;
    P.unit_work = tn.unit_work;
    P.tile = tn.tile;
    P.long_list = tn.long_list;
    P.probe_kicks = tn.probe_kicks;
    P.table_mode = tn.hash_pairs ? kPairs : tn.probe_kicks > 0 ? kCuckoo : kLinear;
    P.count_blocks = tn.blocks;
    P.intersect = tn.hash_pairs ? 0 : tn.intersect;  // the pair-table instance has no sorted mode
    // heavy units on direct-address bitmaps when every graph's ids fit in shared memory
    const int64_t bitmap_words = (max_rows + 31) / 32;
    const bool bitmap = tn.heavy_bitmap && bitmap_words > 0 && bitmap_words * 4 <= (int64_t)tn.bitmap_bytes;
    P.heavy_done = bitmap ? 1 : 0;
    if (bitmap) P.tile = INT32_MAX / 2;  // one tile: the bitmap has no capacity limit
    // light tasks are listed as 32-bit global row indices
    if (total_chunks * kWarp >= ((int64_t)1 << 32))
        return set_error(TC_E_RANGE, "a count of more than 2^32 rows in one launch is not supported");
    TC_CUDA(cudaMemsetAsync(work, 0, sizeof(CountWork), s));
    TC_CUDA(cudaMemsetAsync(results, 0, sizeof(unsigned long long) * (size_t)n_graphs, s));
    int nl = 0;
    if (total_chunks > 0) {
        TC_CUDA(cudaMemsetAsync(sc.in_work, 0, sizeof(unsigned long long) * (size_t)total_vertices, s));
        TC_CUDA(cudaMemsetAsync(sc.out_work, 0, sizeof(unsigned long long) * (size_t)total_vertices, s));
        const int64_t want = (total_chunks + kWarpsPerBlock - 1) / kWarpsPerBlock;
        P.aux_dynamic = n_graphs > 1 ? 1 : 0;
        const int64_t cap = P.aux_dynamic ? (int64_t)tn.aux_blocks : (int64_t)tn.blocks * 4;
        const int aux_blocks = (int)std::max<int64_t>(1, std::min<int64_t>(want, cap));
        degree_kernel<<<aux_blocks, kThreads, 0, s>>>(P);
        TC_CUDA(cudaGetLastError());
        in_count_kernel<<<aux_blocks, kThreads, 0, s>>>(P);
        TC_CUDA(cudaGetLastError());
        TC_TRY(scan_in_slots(sc.in_work, sc.in_off, total_vertices, nullptr, 0, s));
        transpose_classify_kernel<<<aux_blocks, kThreads, 0, s>>>(P, sc.heavy);
        TC_CUDA(cudaGetLastError());
        if (per_root) micro_kernel<true><<<aux_blocks, kThreads, 0, s>>>(P);
        else micro_kernel<false><<<aux_blocks, kThreads, 0, s>>>(P);
        if (kev) TC_TRY(record_kernel_event(kev[0], s));
        if (bitmap) {
            const size_t bytes = (size_t)bitmap_words * 4;
            if (per_root) heavy_bitmap_kernel<true><<<tn.sm_count, kBigThreads, bytes, s>>>(P, (int)bitmap_words);
            else heavy_bitmap_kernel<false><<<tn.sm_count, kBigThreads, bytes, s>>>(P, (int)bitmap_words);
            TC_CUDA(cudaGetLastError());
            ++nl;
        }
        if (per_root) {
            if (tn.hash_pairs) nl += launch_phases<true, true>(P, tn, s);
            else if (P.intersect) nl += launch_phases<true, false, true>(P, tn, s);
            else if (halo_parts) nl += launch_phases<true, false, false, true>(P, tn, s);
            else nl += launch_phases<true, false>(P, tn, s);
        } else {
            if (tn.hash_pairs) nl += launch_phases<false, true>(P, tn, s);
            else if (P.intersect) nl += launch_phases<false, false, true>(P, tn, s);
            else if (halo_parts) nl += launch_phases<false, false, false, true>(P, tn, s);
            else nl += launch_phases<false, false>(P, tn, s);
        }
        if (kev) TC_TRY(record_kernel_event(kev[1], s));
        TC_CUDA(cudaGetLastError());
        nl += 4 + scan_launches(total_vertices);
    }
    if (launches) *launches = nl;
    return TC_OK;
}

int launch_flat(const int32_t *rp, const int32_t *col, int64_t n_roots, int max_deg, CountWork *work,
                unsigned long long *result, unsigned long long *per_root, const Tuned &tn, cudaStream_t s,
                int *launches, cudaEvent_t *kev) {
    if (max_deg > kMicroDeg) return set_error(TC_E_INVALID, "flat count needs rows of at most %d entries", kMicroDeg);
    TC_CUDA(cudaMemsetAsync(work, 0, sizeof(CountWork), s));
    TC_CUDA(cudaMemsetAsync(result, 0, sizeof(unsigned long long), s));
    if (kev) TC_TRY(record_kernel_event(kev[0], s));
    if (n_roots > 0) {
        const int64_t want = (n_roots + kThreads - 1) / kThreads;
        if (max_deg <= 4) {  // one resident wave, several roots per lane
            int occ = 1;
            TC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                &occ, per_root ? flat4_kernel<true> : flat4_kernel<false>, kThreads, 0));
            const int blocks =
                (int)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)tn.sm_count * std::max(occ, 1)));
            if (per_root) flat4_kernel<true><<<blocks, kThreads, 0, s>>>(rp, col, n_roots, result, per_root);
            else flat4_kernel<false><<<blocks, kThreads, 0, s>>>(rp, col, n_roots, result, per_root);
        } else {
            const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)tn.blocks * 8));
            if (per_root) flat_kernel<true, kMicroDeg><<<blocks, kThreads, 0, s>>>(rp, col, n_roots, result, per_root);
            else flat_kernel<false, kMicroDeg><<<blocks, kThreads, 0, s>>>(rp, col, n_roots, result, per_root);
        }
        TC_CUDA(cudaGetLastError());
    }
    if (kev) TC_TRY(record_kernel_event(kev[1], s));
    if (launches) *launches = n_roots > 0 ? 1 : 0;
    return TC_OK;
}

int launch_count_noalloc(const GraphDesc *d_desc, int64_t total_chunks, int64_t total_vertices,
                         const CountScratch &sc, int32_t *scan_tmp, int64_t scan_tmp_cap, CountWork *work,
                         unsigned long long *results, const Tuned &tn, cudaStream_t s) {
    KParams P;
    P.gd = d_desc;
    P.n_graphs = 1;
    P.total_chunks = total_chunks;
    P.heavy = sc.heavy;
    P.heavy_cap = sc.heavy_cap;
    P.work = work;
    P.results = results;
    P.light_list = sc.light_list;
    P.list_cap = total_vertices;
    P.in_cnt = sc.in_cnt;
    P.in_off = sc.in_off;
    P.in_work = sc.in_work;
    P.out_work = sc.out_work;
    P.in_list = sc.in_list;
    P.mid = sc.mid;
    P.warp_max = tn.warp_max;
    P.log_warp_slots = tn.log_warp_slots;
    P.light_max_work = tn.light_max_work;
    P.unit_work = tn.unit_work;
    P.tile = tn.tile;
    P.long_list = tn.long_list;
    P.probe_kicks = tn.probe_kicks;
    P.table_mode = tn.hash_pairs ? kPairs : tn.probe_kicks > 0 ? kCuckoo : kLinear;
    P.count_blocks = tn.blocks;
    P.heavy_done = 0;
    P.intersect = 0;
    TC_CUDA(cudaMemsetAsync(work, 0, sizeof(CountWork), s));
    TC_CUDA(cudaMemsetAsync(results, 0, sizeof(unsigned long long), s));
    if (total_chunks > 0) {
        TC_CUDA(cudaMemsetAsync(sc.in_work, 0, sizeof(unsigned long long) * (size_t)total_vertices, s));
        TC_CUDA(cudaMemsetAsync(sc.out_work, 0, sizeof(unsigned long long) * (size_t)total_vertices, s));
        const int64_t want = (total_chunks + kWarpsPerBlock - 1) / kWarpsPerBlock;
        P.aux_dynamic = 0;
        const int aux_blocks = (int)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)tn.blocks * 4));
        degree_kernel<<<aux_blocks, kThreads, 0, s>>>(P);
        TC_CUDA(cudaGetLastError());
        in_count_kernel<<<aux_blocks, kThreads, 0, s>>>(P);
        TC_CUDA(cudaGetLastError());
        TC_TRY(scan_in_slots(sc.in_work, sc.in_off, total_vertices, scan_tmp, scan_tmp_cap, s));
        transpose_classify_kernel<<<aux_blocks, kThreads, 0, s>>>(P, sc.heavy);
        TC_CUDA(cudaGetLastError());
        micro_kernel<false><<<aux_blocks, kThreads, 0, s>>>(P);
        launch_phases<false, false>(P, tn, s);
        TC_CUDA(cudaGetLastError());
    }
    return TC_OK;
}

}  // namespace tc
