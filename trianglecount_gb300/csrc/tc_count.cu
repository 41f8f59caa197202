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
//  * classify (one warp per 32 roots): roots with d+(u) > warp_max are heavy;
//    each becomes (#tiles x #slices) block units, appended with one packed
//    64-bit atomic per warp so entries stay sorted by their first unit.
//  * count (persistent grid, SMs x occupancy blocks):
//      phase A -- blocks pull heavy units from a global cursor.  A unit builds
//        an open-addressing hash of one tile of N+(u) in shared memory and
//        its warps probe the wedges of one slice of N+(u) against it;
//      phase B -- each warp pulls 32-root chunks from a second cursor and
//        counts every light root (2 <= d+ <= warp_max) with a per-warp shared
//        hash of N+(u), or, for d+ <= tiny_max, a register-broadcast compare.
//    In both phases the wedges of 32 consecutive out-neighbours are
//    flattened across the warp (warp scan of d+(v), one probe per lane per
//    step), so lanes stay busy however short the lists N+(v) are.
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

// Open addressing, linear probing.  The table always has at least half of its
// slots empty, so both loops end after a few steps; the iteration bound only
// guards against a corrupt table.
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
    for (uint32_t it = 0; it <= mask; ++it) {
        const int y = tab[h];
        if (y == x) return 1u;
        if (y == kEmpty) return 0u;
        h = (h + 1) & mask;
    }
    return 0u;
}

// Probes every wedge u->v->x for v = nbr[j], j in [j0, j1), x in N+(v).
// Membership in N+(u) (or a tile of it) is tested against the shared hash
// table (kBcast = false) or against up to 32 values held one per lane in bval
// (kBcast = true, bcnt of them).  Returns this lane's hit count.
template <bool kBcast>
__device__ __forceinline__ uint32_t probe_range(const int32_t *__restrict__ rp, const int32_t *__restrict__ col,
                                                const int32_t *__restrict__ nbr, int j0, int j1, const int *tab,
                                                uint32_t mask, int shift, int bval, int bcnt, int lane) {
    uint32_t hits = 0;
    for (int jb = j0; jb < j1; jb += kWarp) {
        const int j = jb + lane;
        int s2 = 0, len = 0;
        if (j < j1) {
            const int v = __ldg(nbr + j);
            s2 = __ldg(rp + v);
            len = __ldg(rp + v + 1) - s2;
        }
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
            if (kBcast) {
                const int x = (t < total) ? __ldg(col + s_seg + (t - ex_seg)) : -2;
                uint32_t hit = 0;
                for (int k = 0; k < bcnt; ++k) hit |= (uint32_t)(__shfl_sync(kFull, bval, k) == x);
                hits += hit;
            } else if (t < total) {
                hits += table_probe(tab, mask, shift, __ldg(col + s_seg + (t - ex_seg)));
            }
        }
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
    int warp_max;
    int log_warp_slots;
    int slice;
    int tile;
    int tiny_max;
};

__global__ void __launch_bounds__(kThreads) classify_kernel(KParams P, HeavyEntry *heavy) {
    const int lane = threadIdx.x & (kWarp - 1);
    const int64_t gwarp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / kWarp;
    const int64_t nwarps = (int64_t)gridDim.x * blockDim.x / kWarp;
    for (int64_t c = gwarp; c < P.total_chunks; c += nwarps) {
        const int g = find_graph(P.gd, P.n_graphs, c);
        const int32_t *rp = P.gd[g].rp;
        const int64_t u = (c - P.gd[g].chunk_base) * kWarp + lane;
        int d = 0;
        if (u < P.gd[g].n_roots) d = __ldg(rp + u + 1) - __ldg(rp + u);
        const bool hv = d > P.warp_max;
        const unsigned m = __ballot_sync(kFull, hv);
        if (m == 0) continue;
        unsigned units = 0;
        if (hv) units = (unsigned)((d + P.tile - 1) / P.tile) * (unsigned)((d + P.slice - 1) / P.slice);
        unsigned incl = units;
#pragma unroll
        for (int o = 1; o < kWarp; o <<= 1) {
            const unsigned t = __shfl_up_sync(kFull, incl, o);
            if (lane >= o) incl += t;
        }
        const unsigned tot = __shfl_sync(kFull, incl, kWarp - 1);
        const int leader = __ffs(m) - 1;
        unsigned long long base = 0;
        if (lane == leader)
            base = atomicAdd(&P.work->heavy_packed, ((unsigned long long)__popc(m) << 32) | (unsigned long long)tot);
        base = __shfl_sync(kFull, base, leader);
        if (hv) {
            const unsigned long long idx = (base >> 32) + __popc(m & ((1u << lane) - 1u));
            if ((int64_t)idx < P.heavy_cap) {
                HeavyEntry e;
                e.g = g;
                e.u = (int32_t)u;
                e.unit_base = (int32_t)((unsigned)base + incl - units);
                e.n_units = (int32_t)units;
                heavy[idx] = e;
            } else {
                atomicExch(&P.work->error, 1);
            }
        }
    }
}

__global__ void __launch_bounds__(kThreads) count_kernel(KParams P) {
    extern __shared__ int smem[];
    __shared__ unsigned s_unit;
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
        if (threadIdx.x == 0) s_unit = atomicAdd(&P.work->heavy_cursor, 1u);
        __syncthreads();
        const unsigned unit = s_unit;
        __syncthreads();
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
        const int ns = (d + P.slice - 1) / P.slice;
        const int k = (int)(unit - (unsigned)e.unit_base);
        const int ti = k / ns, si = k - (k / ns) * ns;
        const int t0 = ti * P.tile;
        const int tl = min(d - t0, P.tile);
        const int lg = max(5, ilog2_ceil(2 * tl));
        const uint32_t mask = (1u << lg) - 1u;
        const int shift = 32 - lg;
        if (lo != cached_entry || ti != cached_tile) {
            for (int i = threadIdx.x; i <= (int)mask; i += kThreads) smem[i] = kEmpty;
            __syncthreads();
            for (int i = threadIdx.x; i < tl; i += kThreads) table_insert(smem, mask, shift, __ldg(col + rs + t0 + i));
            __syncthreads();
            cached_entry = lo;
            cached_tile = ti;
        }
        const int j0 = si * P.slice, j1 = min(d, j0 + P.slice);
        uint32_t hits = 0;
        for (int jb = j0 + warp * kWarp; jb < j1; jb += kThreads)
            hits += probe_range<false>(rp, col, col + rs, jb, min(jb + kWarp, j1), smem, mask, shift, 0, 0, lane);
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
        const int g = find_graph(P.gd, P.n_graphs, c);
        const GraphDesc &G = P.gd[g];
        const int32_t *__restrict__ rp = G.rp;
        const int32_t *__restrict__ col = G.col;
        if (g != cur_g && !G.per_root) flush(g);
        const int64_t u0 = ((int64_t)c - G.chunk_base) * kWarp;
        int rs = 0, d = 0;
        if (u0 + lane < G.n_roots) {
            rs = __ldg(rp + u0 + lane);
            d = __ldg(rp + u0 + lane + 1) - rs;
        }
        unsigned todo = __ballot_sync(kFull, d >= 2 && d <= P.warp_max);
        while (todo) {
            const int k = __ffs(todo) - 1;
            todo &= todo - 1u;
            const int rrs = __shfl_sync(kFull, rs, k);
            const int rd = __shfl_sync(kFull, d, k);
            uint32_t hits;
            if (rd <= P.tiny_max) {
                const int bval = lane < rd ? __ldg(col + rrs + lane) : -1;
                hits = probe_range<true>(rp, col, col + rrs, 0, rd, nullptr, 0, 0, bval, rd, lane);
            } else {
                const int lg = max(5, ilog2_ceil(2 * rd));
                const uint32_t mask = (1u << lg) - 1u;
                const int shift = 32 - lg;
                for (int i = lane; i <= (int)mask; i += kWarp) wtab[i] = kEmpty;
                __syncwarp();
                for (int i = lane; i < rd; i += kWarp) table_insert(wtab, mask, shift, __ldg(col + rrs + i));
                __syncwarp();
                hits = probe_range<false>(rp, col, col + rrs, 0, rd, wtab, mask, shift, 0, 0, lane);
                __syncwarp();
            }
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
    int wm = t.warp_max_deg > 0 ? t.warp_max_deg : 128;
    if (wm < 32 || wm > 1024 || (wm & (wm - 1)))
        return set_error(TC_E_INVALID, "warp_max_deg must be a power of two in [32, 1024], got %d", wm);
    r.warp_max = wm;
    r.log_warp_slots = pow2_floor_log(2 * wm);
    const int warp_slots_total = kWarpsPerBlock * (1 << r.log_warp_slots);
    const int block_slots = std::max(8192, warp_slots_total);
    r.log_block_slots = pow2_floor_log(block_slots);
    r.tile = block_slots / 2;
    r.slice = t.block_slice > 0 ? t.block_slice : 512;
    if (r.slice % kWarp) return set_error(TC_E_INVALID, "block_slice must be a multiple of 32, got %d", r.slice);
    r.tiny_max = t.tiny_max_deg >= 0 ? t.tiny_max_deg : 0;
    if (r.tiny_max > 32) return set_error(TC_E_INVALID, "tiny_max_deg must be <= 32, got %d", r.tiny_max);
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
                 CountWork *work, unsigned long long *results, const Tuned &tn, cudaStream_t s, int *launches) {
    KParams P;
    P.gd = d_desc;
    P.n_graphs = n_graphs;
    P.total_chunks = total_chunks;
    P.heavy = heavy;
    P.heavy_cap = heavy_cap;
    P.work = work;
    P.results = results;
    P.warp_max = tn.warp_max;
    P.log_warp_slots = tn.log_warp_slots;
    P.slice = tn.slice;
    P.tile = tn.tile;
    P.tiny_max = tn.tiny_max;
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
