// tc_count.cu -- exact triangle counting on a degree-oriented int32 CSR.
//
// Quantity: for each root u, sum over v in N+(u) of |N+(u) n N+(v)| -- the
// reference's per-block g_sum[u] (src/WithoutPartition/ShareKernelTCV62_update_v1.cu:43-191,
// src/WithPartition/without_sorting_tc.cu:57-219), summed over roots as the
// reference's cub::DeviceReduce::Sum does (ShareKernelTCV62_update_v1.cu:271-277).
//
// The reference runs one 128-thread block per root, stages N+(u) in 128-entry
// shared tiles and binary-searches every x in N+(v) against each tile, one
// v at a time, so most threads idle on the short lists of a power-law graph.
// Here the same set of probes (one per oriented wedge u->v->x) is organised
// for the GB300 as follows:
//
//  * classify (one warp per 32 roots): the warp computes, per root, d+(u) and
//    the work w(u) = sum_{v in N+(u)} d+(v).  Light roots (d+(u) <= warp_max
//    and w(u) <= light_max_work) are marked in a 32-bit mask per chunk; heavy
//    roots become (#tiles x #slices) block units, #slices ~ w(u) / unit_work,
//    appended with one packed 64-bit atomic so entries stay sorted by unit.
//  * count (persistent grid, SMs x occupancy blocks):
//      phase A -- blocks pull heavy units from a global cursor.  A unit builds
//        an open-addressing hash (load factor <= 1/4) of one tile of N+(u) in
//        shared memory; the block's warps pull 32-neighbour chunks of the
//        unit's slice from a shared cursor and probe their wedges;
//      phase B -- each warp pulls 32-root chunks and counts the light roots
//        of the chunk with a per-warp shared hash of N+(u).
//    Probing a chunk of 32 out-neighbours: lists N+(v) with d+(v) >= long_list
//    are streamed by the whole warp, four coalesced loads in flight per lane;
//    the shorter lists are flattened across the lanes (warp scan of d+(v),
//    one probe per lane per step), so lanes stay busy on short lists too.
//  * totals: per-lane u64 accumulators, warp-reduced and added with one
//    atomic per warp per graph change.  Integer addition is associative, so
//    the count is exact and independent of the schedule.
//
// The same two kernels serve the plain path (one graph per launch) and the
// batched path (a descriptor table of many graphs or halo parts, one launch).
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

// Table geometry for n keys: slots = max(32, next_pow2(4 n)).
__device__ __forceinline__ int table_log_slots(int n) { return max(5, ilog2_ceil(4 * n)); }

// Empties a table of (mask + 1) slots with `nthreads` threads numbered `tid`;
// the caller synchronises before inserting.
__device__ __forceinline__ void table_clear(int *tab, uint32_t mask, int tid, int nthreads) {
    for (int i = tid; i <= (int)mask; i += nthreads) tab[i] = kEmpty;
}

// Probes every wedge u->v->x for v = nbr[j], j in [j0, j1) (at most 32
// neighbours), x in N+(v), against the hash of N+(u) (or of a tile of it).
// Returns this lane's hit count.
__device__ __forceinline__ uint32_t probe_chunk(const int32_t *__restrict__ rp, const int32_t *__restrict__ col,
                                                const int32_t *__restrict__ nbr, int j0, int j1, const int *tab,
                                                uint32_t mask, int shift, int long_list, int lane) {
    uint32_t hits = 0;
    const int j = j0 + lane;
    int s2 = 0, len = 0;
    if (j < j1) {
        const int v = __ldg(nbr + j);
        s2 = __ldg(rp + v);
        len = __ldg(rp + v + 1) - s2;
    }
    // long lists: the whole warp streams one list, four loads in flight per lane
    unsigned longm = __ballot_sync(kFull, len >= long_list);
    while (longm) {
        const int k = __ffs(longm) - 1;
        longm &= longm - 1u;
        const int ls = __shfl_sync(kFull, s2, k);
        const int ll = __shfl_sync(kFull, len, k);
        const int32_t *__restrict__ p = col + ls;
        for (int base = 0; base < ll; base += 4 * kWarp) {
            int x[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int t = base + i * kWarp + lane;
                x[i] = t < ll ? __ldg(p + t) : -1;
            }
#pragma unroll
            for (int i = 0; i < 4; ++i)
                if (x[i] >= 0) hits += table_probe(tab, mask, shift, x[i]);
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
        if (t < total) hits += table_probe(tab, mask, shift, __ldg(col + s_seg + (t - ex_seg)));
    }
    return hits;
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
    uint32_t *light_mask;  // one word per 32-root chunk
    int warp_max;
    int log_warp_slots;
    int light_max_work;
    int unit_work;
    int tile;
    int long_list;
};

__global__ void __launch_bounds__(kThreads) classify_kernel(KParams P, HeavyEntry *heavy) {
    const int lane = threadIdx.x & (kWarp - 1);
    const int64_t gwarp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / kWarp;
    const int64_t nwarps = (int64_t)gridDim.x * blockDim.x / kWarp;
    for (int64_t c = gwarp; c < P.total_chunks; c += nwarps) {
        const int g = find_graph(P.gd, P.n_graphs, c);
        const int32_t *__restrict__ rp = P.gd[g].rp;
        const int32_t *__restrict__ col = P.gd[g].col;
        const int64_t u0 = (c - P.gd[g].chunk_base) * kWarp;
        int rs = 0, d = 0;
        if (u0 + lane < P.gd[g].n_roots) {
            rs = __ldg(rp + u0 + lane);
            d = __ldg(rp + u0 + lane + 1) - rs;
        }
        uint32_t light = 0;
        unsigned todo = __ballot_sync(kFull, d >= 2);
        while (todo) {
            const int k = __ffs(todo) - 1;
            todo &= todo - 1u;
            const int rrs = __shfl_sync(kFull, rs, k);
            const int rd = __shfl_sync(kFull, d, k);
            unsigned long long w = 0;
            for (int i = lane; i < rd; i += kWarp) {
                const int v = __ldg(col + rrs + i);
                w += (unsigned long long)(__ldg(rp + v + 1) - __ldg(rp + v));
            }
            w = warp_sum_u64(w);
            if (w == 0) continue;
            if (rd <= P.warp_max && w <= (unsigned long long)P.light_max_work) {
                light |= 1u << k;
                continue;
            }
            if (lane == 0) {
                const int max_slices = (rd + kWarp - 1) / kWarp;
                int ns = (int)min((w + (unsigned long long)P.unit_work - 1) / (unsigned long long)P.unit_work,
                                  (unsigned long long)max_slices);
                ns = max(ns, 1);
                const unsigned units = (unsigned)((rd + P.tile - 1) / P.tile) * (unsigned)ns;
                const unsigned long long base = atomicAdd(&P.work->heavy_packed, (1ull << 32) | units);
                const unsigned long long idx = base >> 32;
                if ((int64_t)idx < P.heavy_cap) {
                    HeavyEntry e;
                    e.g = g;
                    e.u = (int32_t)(u0 + k);
                    e.unit_base = (int32_t)(unsigned)base;
                    e.n_slices = ns;
                    heavy[idx] = e;
                } else {
                    atomicExch(&P.work->error, 1);
                }
            }
        }
        if (lane == 0) P.light_mask[c] = light;
    }
}

__global__ void __launch_bounds__(kThreads) count_kernel(KParams P) {
    extern __shared__ int smem[];
    __shared__ unsigned s_unit;
    __shared__ int s_chunk;
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

    // ---- phase A: heavy units, one block each ----
    int cached_entry = -1, cached_tile = -1;
    for (;;) {
        if (threadIdx.x == 0) {
            s_unit = atomicAdd(&P.work->heavy_cursor, 1u);
            s_chunk = 0;
        }
        __syncthreads();
        const unsigned unit = s_unit;
        if (unit >= n_units || n_entries == 0) break;
        int lo = 0, hi = (int)n_entries - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if ((unsigned)P.heavy[mid].unit_base <= unit) lo = mid;
            else hi = mid - 1;
        }
        const HeavyEntry e = P.heavy[lo];
        const GraphDesc &G = P.gd[e.g];
        const int32_t *__restrict__ rp = G.rp;
        const int32_t *__restrict__ col = G.col;
        const int rs = __ldg(rp + e.u);
        const int d = __ldg(rp + e.u + 1) - rs;
        const int ns = e.n_slices;
        const int k = (int)(unit - (unsigned)e.unit_base);
        const int ti = k / ns, si = k - ti * ns;
        const int t0 = ti * P.tile;
        const int tl = min(d - t0, P.tile);
        const int lg = table_log_slots(tl);
        const uint32_t mask = (1u << lg) - 1u;
        const int shift = 32 - lg;
        if (lo != cached_entry || ti != cached_tile) {
            table_clear(smem, mask, threadIdx.x, kThreads);
            __syncthreads();
            for (int i = threadIdx.x; i < tl; i += kThreads) table_insert(smem, mask, shift, __ldg(col + rs + t0 + i));
            cached_entry = lo;
            cached_tile = ti;
        }
        __syncthreads();
        const int per = (d + ns - 1) / ns;
        const int j0 = si * per, j1 = min(d, j0 + per);
        uint32_t hits = 0;
        for (;;) {
            int c = 0;
            if (lane == 0) c = atomicAdd(&s_chunk, 1);
            c = __shfl_sync(kFull, c, 0);
            const int jb = j0 + c * kWarp;
            if (jb >= j1) break;
            hits += probe_chunk(rp, col, col + rs, jb, min(jb + kWarp, j1), smem, mask, shift, P.long_list, lane);
        }
        if (G.per_root) {
            const unsigned long long s = warp_sum_u64(hits);
            if (lane == 0 && s) atomicAdd(G.per_root + e.u, s);
        } else {
            if (e.g != cur_g) flush(e.g);
            acc += hits;
        }
        __syncthreads();
    }

    // ---- phase B: light roots, one warp each ----
    int *wtab = smem + warp * (1 << P.log_warp_slots);
    for (;;) {
        unsigned c = 0;
        if (lane == 0) c = atomicAdd(&P.work->small_cursor, 1u);
        c = __shfl_sync(kFull, c, 0);
        if ((int64_t)c >= P.total_chunks) break;
        unsigned todo = P.light_mask[c];
        if (!todo) continue;
        const int g = find_graph(P.gd, P.n_graphs, c);
        const GraphDesc &G = P.gd[g];
        const int32_t *__restrict__ rp = G.rp;
        const int32_t *__restrict__ col = G.col;
        if (g != cur_g && !G.per_root) flush(g);
        const int64_t u0 = ((int64_t)c - G.chunk_base) * kWarp;
        int rs = 0, d = 0;
        if ((todo >> lane) & 1u) {
            rs = __ldg(rp + u0 + lane);
            d = __ldg(rp + u0 + lane + 1) - rs;
        }
        while (todo) {
            const int k = __ffs(todo) - 1;
            todo &= todo - 1u;
            const int rrs = __shfl_sync(kFull, rs, k);
            const int rd = __shfl_sync(kFull, d, k);
            const int lg = table_log_slots(rd);
            const uint32_t mask = (1u << lg) - 1u;
            const int shift = 32 - lg;
            table_clear(wtab, mask, lane, kWarp);
            __syncwarp();
            for (int i = lane; i < rd; i += kWarp) table_insert(wtab, mask, shift, __ldg(col + rrs + i));
            __syncwarp();
            uint32_t hits = 0;
            for (int jb = 0; jb < rd; jb += kWarp)
                hits += probe_chunk(rp, col, col + rrs, jb, min(jb + kWarp, rd), wtab, mask, shift, P.long_list, lane);
            __syncwarp();
            if (G.per_root) {
                const unsigned long long s = warp_sum_u64(hits);
                if (lane == 0) G.per_root[u0 + k] = s;
            } else {
                acc += hits;
            }
        }
    }
    flush(-1);
}

int pow2_floor_log(int x) {
    int l = 0;
    while ((2 << l) <= x) ++l;
    return l;
}

}  // namespace

int resolve_tuning(const tc_tuning &t, int sm_count, Tuned *out) {
    Tuned r;
    const int wm = t.warp_max_deg > 0 ? t.warp_max_deg : 128;
    if (wm < 32 || wm > 512 || (wm & (wm - 1)))
        return set_error(TC_E_INVALID, "warp_max_deg must be a power of two in [32, 512], got %d", wm);
    r.warp_max = wm;
    r.log_warp_slots = pow2_floor_log(4 * wm);
    const int warp_slots_total = kWarpsPerBlock * (1 << r.log_warp_slots);
    const int block_slots = std::max(8192, warp_slots_total);
    r.log_block_slots = pow2_floor_log(block_slots);
    r.tile = block_slots / 4;
    r.light_max_work = t.light_max_work > 0 ? t.light_max_work : 32768;
    r.unit_work = t.unit_work > 0 ? t.unit_work : 65536;
    r.long_list = t.long_list >= 0 ? t.long_list : 16;
    if (r.long_list > 4096) return set_error(TC_E_INVALID, "long_list must be <= 4096, got %d", r.long_list);
    r.threads = kThreads;
    r.smem = (size_t)block_slots * sizeof(int);
    TC_CUDA(cudaFuncSetAttribute(count_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)r.smem));
    int occ = 0;
    TC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, count_kernel, kThreads, r.smem));
    if (occ < 1) return set_error(TC_E_INVALID, "count kernel does not fit on an SM with %zu B shared memory", r.smem);
    const int bps = t.blocks_per_sm > 0 ? std::min(t.blocks_per_sm, occ) : occ;
    r.blocks = sm_count * bps;
    *out = r;
    return TC_OK;
}

int launch_count(const GraphDesc *d_desc, int n_graphs, int64_t total_chunks, HeavyEntry *heavy, int64_t heavy_cap,
                 uint32_t *light_mask, CountWork *work, unsigned long long *results, const Tuned &tn, cudaStream_t s,
                 int *launches) {
    KParams P;
    P.gd = d_desc;
    P.n_graphs = n_graphs;
    P.total_chunks = total_chunks;
    P.heavy = heavy;
    P.heavy_cap = heavy_cap;
    P.work = work;
    P.results = results;
    P.light_mask = light_mask;
    P.warp_max = tn.warp_max;
    P.log_warp_slots = tn.log_warp_slots;
    P.light_max_work = tn.light_max_work;
    P.unit_work = tn.unit_work;
    P.tile = tn.tile;
    P.long_list = tn.long_list;
    TC_CUDA(cudaMemsetAsync(work, 0, sizeof(CountWork), s));
    TC_CUDA(cudaMemsetAsync(results, 0, sizeof(unsigned long long) * (size_t)n_graphs, s));
    int nl = 0;
    if (total_chunks > 0) {
        const int64_t want = (total_chunks + kWarpsPerBlock - 1) / kWarpsPerBlock;
        const int cls_blocks = (int)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)tn.blocks * 4));
        classify_kernel<<<cls_blocks, kThreads, 0, s>>>(P, heavy);
        TC_CUDA(cudaGetLastError());
        count_kernel<<<tn.blocks, kThreads, tn.smem, s>>>(P);
        TC_CUDA(cudaGetLastError());
        nl = 2;
    }
    if (launches) *launches = nl;
    return TC_OK;
}

}  // namespace tc
