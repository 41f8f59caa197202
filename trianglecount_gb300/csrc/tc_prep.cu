// tc_prep.cu -- device preprocessing: edge list -> simple undirected CSR ->
// degree-oriented CSR, and per-part halo subgraphs.
//
// Clean-up restates the DGL pipeline of Med_dataset/without_part_preprocess.py:193-228
// (remove_self_loop, to_bidirected, remove isolated nodes, adj_tensors('csr')):
//   keys (u<<B|v) and (v<<B|u) per non-loop edge -> LSD radix sort -> unique
//   -> per-vertex counts -> order-preserving relabel of non-isolated vertices.
// Orientation restates Find_size / cp.cumsum / Convert (:19-111, :253-270)
// (count the kept entries, scan, write them in order), over 4096-entry tiles:
//   keep bits + tile counts -> scan of the tile counts -> ordered write of the
//   kept entries and the new row starts, so rows stay ascending.
// Halo extraction restates create_subgraph_with_halo
// (preprocess_GPU/Halo_cleanned_preprocess/round_clean_subgraph.cu:357-902) with the
// intended prune loop of Halo_creation_preprocess.py:566-589: the halo sets of
// all parts from one pass (k <= 32); per part, local ids (part vertices, then
// halo, each ascending) -> P/H/R class bits, tile counts and row-start ranks
// over the orientation's tiles -> scan -> local row lengths and halo in-degrees
// -> scan -> ordered write of every local edge; then halo vertices with zero
// in-degree are peeled until none is left.
#include <algorithm>
#include <vector>

#include "tc_internal.h"

namespace tc {

int validate_csr(tc_ctx *ctx, const int32_t *rp, const int32_t *col, int64_t n_rows, int64_t nnz);
int graph_adopt_device(tc_ctx *ctx, int32_t *rp, int32_t *col, int64_t n_rows, int64_t nnz, int64_t n_roots,
                       tc_graph **out);

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr uint64_t kSentinel = ~0ull;

#define GRID_STRIDE(i, n) \
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < (n); i += (int64_t)gridDim.x * blockDim.x)

int grid(int64_t n, const tc_ctx *ctx) {
    const int64_t b = (n + 255) / 256;
    return (int)std::max<int64_t>(1, std::min<int64_t>(b, (int64_t)ctx->sm_count * 32));
}

__device__ __forceinline__ bool keep_edge(int du, int dw, int u, int w, int tie) {
    if (du != dw) return du < dw;
    return tie == TC_TIE_REFERENCE ? (w < u) : (u < w);
}

// Adds 1 to cnt[key] for a warp of (mostly sorted) keys with one atomic per
// distinct key in the warp.
__device__ __forceinline__ void warp_count(int32_t *cnt, int key, bool valid) {
    const unsigned act = __ballot_sync(kFull, valid);
    if (!valid) return;
    const unsigned peers = __match_any_sync(act, key);
    const int lane = threadIdx.x & 31;
    if ((peers & ((1u << lane) - 1u)) == 0) atomicAdd(&cnt[key], __popc(peers));
}

__global__ void max_id_kernel(const int64_t *a, const int64_t *b, int64_t n, unsigned long long *mx, int *neg) {
    unsigned long long m = 0;
    bool bad = false;
    GRID_STRIDE(i, n) {
        const int64_t x = a[i], y = b[i];
        bad |= (x < 0) | (y < 0);
        m = max(m, (unsigned long long)max(x, y));
    }
    if (bad) *neg = 1;
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) m = max(m, __shfl_xor_sync(kFull, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(mx, m);
}

__global__ void make_keys_kernel(const int64_t *src, const int64_t *dst, int64_t n, int B, uint64_t *keys) {
    GRID_STRIDE(i, n) {
        const uint64_t u = (uint64_t)src[i], v = (uint64_t)dst[i];
        if (u == v) {
            keys[2 * i] = kSentinel;
            keys[2 * i + 1] = kSentinel;
        } else {
            keys[2 * i] = (u << B) | v;
            keys[2 * i + 1] = (v << B) | u;
        }
    }
}

__global__ void unique_flags_kernel(const uint64_t *keys, int64_t n, uint8_t *flags) {
    GRID_STRIDE(i, n) {
        const uint64_t k = keys[i];
        flags[i] = (uint8_t)(k != kSentinel && (i == 0 || keys[i - 1] != k));
    }
}

__global__ void unique_scatter_kernel(const uint64_t *keys, int64_t n, const uint8_t *flags, const int32_t *pos, int B,
                                      int32_t *col, int32_t *rowid, int32_t *cnt) {
    const uint64_t mask = (1ull << B) - 1ull;
    // every thread of a warp runs the same number of iterations (warp_count needs them all)
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t start = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t rounds = (n + stride - 1) / stride;
    for (int64_t r = 0; r < rounds; ++r) {
        const int64_t i = start + r * stride;
        const bool f = i < n && flags[i];
        int u = 0;
        if (f) {
            const uint64_t k = keys[i];
            u = (int)(k >> B);
            const int32_t p = pos[i];
            col[p] = (int32_t)(k & mask);
            rowid[p] = u;
        }
        warp_count(cnt, u, f);
    }
}

__global__ void keep_nonisolated_kernel(const int32_t *cnt, int64_t n, uint8_t *keep) {
    GRID_STRIDE(v, n) keep[v] = (uint8_t)(cnt[v] > 0);
}

__global__ void relabel_rows_kernel(const uint8_t *keep, const int32_t *newid, const int32_t *rs_old, int64_t n0,
                                    int32_t *rp) {
    GRID_STRIDE(v, n0) {
        if (keep[v]) rp[newid[v]] = rs_old[v];
    }
}

__global__ void remap_kernel(int32_t *a, int64_t n, const int32_t *map) {
    GRID_STRIDE(i, n) a[i] = map[a[i]];
}

__global__ void degree_kernel(const int32_t *rp, int64_t n, int32_t *deg) {
    GRID_STRIDE(v, n) deg[v] = rp[v + 1] - rp[v];
}

// An undirected CSR lists every edge in both rows and has no self-loop: entry
// (u, w) needs u in row w (rows ascending: a binary search).  *bad is set on
// the first violation.
__global__ void check_symmetric_kernel(const int32_t *__restrict__ rp, const int32_t *__restrict__ col,
                                       const int32_t *__restrict__ rowid, int64_t nnz, int *bad) {
    GRID_STRIDE(j, nnz) {
        const int u = rowid[j], w = col[j];
        int lo = rp[w], hi = rp[w + 1];
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (col[mid] < u) lo = mid + 1;
            else hi = mid;
        }
        if (u == w || lo == rp[w + 1] || col[lo] != u) *bad = 1;
    }
}

// rowid[j] = u for j in row u (one warp per row)
__global__ void rowid_kernel(const int32_t *rp, int64_t n_rows, int32_t *rowid) {
    const int lane = threadIdx.x & 31;
    const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t u = w0; u < n_rows; u += nw)
        for (int64_t j = rp[u] + lane; j < rp[u + 1]; j += 32) rowid[j] = (int32_t)u;
}

__global__ void narrow_i64_kernel(const int64_t *in, int32_t *out, int64_t n, int64_t limit, int *bad) {
    GRID_STRIDE(i, n) {
        const int64_t v = in[i];
        if (v < 0 || v > limit) *bad = 1;
        out[i] = (int32_t)v;
    }
}

// Orientation in two balanced passes over tiles of 4096 undirected entries
// (no per-entry flags or positions kept): pass 1 decides every entry (16 keep
// bits per thread, kept for pass 2) and counts each tile's kept entries; after
// a scan of the tile counts, pass 2 ranks the bits with one block scan and
// writes the kept entries in order, plus every row's start (the rows that
// begin at an entry are those between its predecessor's row and its own).
//
// A tile's 256 threads cover its entries in one of two layouts; warp q owns
// the 512 entries [tile + 512 q, + 512) in both.  Strided: lane l takes
// entries + 32 i + l (i = 0..15), so each load and store instruction of a warp
// covers 32 consecutive entries.  Runs: lane l takes entries + 16 l + [0, 16),
// loaded with four 16-byte loads, few instructions per entry.  Measured per
// pass on R-MAT 21 (63.5 M entries), runs / strided: orientation keep pass
// 244 / 216 us, orientation write 159 / 264 us, halo class pass 306 / 436 us,
// halo write 342 / 222 us.  So the orientation decides strided and writes in
// runs, the halo classifies in runs and writes strided, and each second pass
// regroups the first pass's bits with warp ballots or shuffles.
constexpr int kOT = 256, kOI = 16, kOTile = kOT * kOI, kOWarpSpan = 32 * kOI;

// Index of the thread's entry 0 (its entry i is this + 32 i).
__device__ __forceinline__ int64_t strided_first() {
    return (int64_t)blockIdx.x * kOTile + (int64_t)(threadIdx.x >> 5) * kOWarpSpan + (threadIdx.x & 31);
}

// Exclusive scan over the 8 warps of a 256-thread block of a warp-uniform
// value; *total gets the block's sum.
template <class T>
__device__ __forceinline__ T warp_offsets_256(T wv, T *total) {
    __shared__ T ws[kOT / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) ws[warp] = wv;
    __syncthreads();
    T excl = 0, tot = 0;
#pragma unroll
    for (int q = 0; q < kOT / 32; ++q) {
        const T x = ws[q];
        if (q < warp) excl += x;
        tot += x;
    }
    *total = tot;
    return excl;
}

// Exclusive scan of one value per thread over a 256-thread block; *total gets
// the block's sum.
__device__ __forceinline__ int block_scan_256(int v, int *total) {
    __shared__ int wsum[kOT / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(kFull, x, o);
        if (lane >= o) x += t;
    }
    if (lane == 31) wsum[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int w = lane < kOT / 32 ? wsum[lane] : 0;
#pragma unroll
        for (int o = 1; o < kOT / 32; o <<= 1) {
            const int t = __shfl_up_sync(kFull, w, o);
            if (lane >= o) w += t;
        }
        if (lane < kOT / 32) wsum[lane] = w;
    }
    __syncthreads();
    const int excl = x - v + (warp ? wsum[warp - 1] : 0);
    *total = wsum[kOT / 32 - 1];
    __syncthreads();  // wsum is reused by the next call
    return excl;
}

// The thread's 16 contiguous entries [j0, j0 + 16): rows u[] and ids w[] (0 past nnz).
__device__ __forceinline__ void load16(const int32_t *__restrict__ rowid, const int32_t *__restrict__ col, int64_t j0,
                                       int64_t nnz, int (&u)[kOI], int (&w)[kOI]) {
    if (j0 + kOI <= nnz) {  // 64-byte aligned: four 16-byte loads per array
#pragma unroll
        for (int q = 0; q < kOI / 4; ++q) {
            const int4 a = __ldg(reinterpret_cast<const int4 *>(rowid + j0) + q);
            const int4 b = __ldg(reinterpret_cast<const int4 *>(col + j0) + q);
            u[4 * q] = a.x, u[4 * q + 1] = a.y, u[4 * q + 2] = a.z, u[4 * q + 3] = a.w;
            w[4 * q] = b.x, w[4 * q + 1] = b.y, w[4 * q + 2] = b.z, w[4 * q + 3] = b.w;
        }
    } else {
#pragma unroll
        for (int i = 0; i < kOI; ++i) {
            const bool in = j0 + i < nnz;
            u[i] = in ? __ldg(rowid + j0 + i) : 0;
            w[i] = in ? __ldg(col + j0 + i) : 0;
        }
    }
}

__global__ void __launch_bounds__(kOT) orient_tile_count_kernel(const int32_t *__restrict__ rowid,
                                                                 const int32_t *__restrict__ col,
                                                                 const int32_t *__restrict__ deg, int64_t nnz,
                                                                 int tie, int32_t *tile_cnt, uint16_t *keep) {
    const int64_t j0 = strided_first();
    unsigned bits = 0;
#pragma unroll
    for (int i = 0; i < kOI; ++i) {
        const int64_t j = j0 + 32 * i;
        if (j < nnz) {
            const int u = __ldg(rowid + j), w = __ldg(col + j);
            if (keep_edge(__ldg(deg + u), __ldg(deg + w), u, w, tie)) bits |= 1u << i;
        }
    }
    keep[(int64_t)blockIdx.x * kOT + threadIdx.x] = (uint16_t)bits;  // pass 2 reads the bits back
    int total = 0;
    warp_offsets_256(__reduce_add_sync(kFull, __popc(bits)), &total);
    if (threadIdx.x == 0) tile_cnt[blockIdx.x] = total;
}

// The orientation's write pass runs on runs.  Its bits come from pass 1's
// strided layout: the run of lane l is entries 32 (l / 2) + 16 (l % 2) +
// [0, 16) of the warp's 512, i.e. bit l / 2 of 16 lanes, one ballot per i.
__device__ __forceinline__ unsigned strided_to_runs(unsigned sw) {
    const int lane = threadIdx.x & 31;
    unsigned bits = 0;
#pragma unroll
    for (int i = 0; i < kOI; ++i) {
        const unsigned b = __ballot_sync(kFull, (sw >> i) & 1u);
        if ((lane >> 1) == i) bits = (b >> ((lane & 1) * 16)) & 0xffffu;
    }
    return bits;
}

__global__ void __launch_bounds__(kOT) orient_tile_write_kernel(const int32_t *__restrict__ rowid,
                                                                 const int32_t *__restrict__ col, const uint16_t *keep,
                                                                 int64_t nnz, int64_t V, const int32_t *tile_off,
                                                                 int32_t *out_rp, int32_t *out_col) {
    int u[kOI], w[kOI];
    const int64_t j0 = (int64_t)blockIdx.x * kOTile + (int64_t)threadIdx.x * kOI;
    const unsigned bits = strided_to_runs(keep[(int64_t)blockIdx.x * kOT + threadIdx.x]);
    load16(rowid, col, j0, nnz, u, w);
    int total = 0;
    int o = tile_off[blockIdx.x] + block_scan_256(__popc(bits), &total);
    if (j0 >= nnz) return;
    int prev = j0 == 0 ? -1 : __ldg(rowid + j0 - 1);
#pragma unroll
    for (int i = 0; i < kOI; ++i) {
        if (j0 + i >= nnz) break;
        for (int r = prev + 1; r <= u[i]; ++r) out_rp[r] = o;  // rows that start at this entry
        prev = u[i];
        if ((bits >> i) & 1u) out_col[o++] = w[i];
    }
    if (j0 + kOI >= nnz)  // the last entry's thread: the rows after it (and out_rp[V]) start at the end
        for (int64_t r = (int64_t)prev + 1; r <= V; ++r) out_rp[r] = o;
}

// ---- halo ----------------------------------------------------------------------
// Halo sets of all parts (k <= 32) in one pass: mask[v] gets bit q for every
// neighbour of v in part q, so v is in part p's halo when bit p is set and
// part[v] != p (the undirected CSR is symmetric: v has a neighbour in p iff
// some vertex of p has v as a neighbour).  One atomicOr per row run of a
// thread's 16 entries.  With `in_only` (the counting halo) a neighbour w in
// part q sets bit q only when w -> v is the oriented direction, so the halo
// of part p is the set of vertices with an oriented in-edge from p.
__global__ void __launch_bounds__(kOT) halo_mask_kernel(const int32_t *__restrict__ rowid,
                                                         const int32_t *__restrict__ col,
                                                         const int32_t *__restrict__ part,
                                                         const int32_t *__restrict__ deg, int64_t nnz, int in_only,
                                                         int tie, unsigned *__restrict__ mask) {
    int u[kOI], w[kOI];
    const int64_t j0 = (int64_t)blockIdx.x * kOTile + (int64_t)threadIdx.x * kOI;
    if (j0 >= nnz) return;
    load16(rowid, col, j0, nnz, u, w);
    int cur = u[0];
    int dcur = in_only ? __ldg(deg + cur) : 0;
    unsigned m = 0;
#pragma unroll
    for (int i = 0; i < kOI; ++i) {
        if (j0 + i >= nnz) break;
        if (u[i] != cur) {
            if (m) atomicOr(mask + cur, m);
            cur = u[i];
            if (in_only) dcur = __ldg(deg + cur);
            m = 0;
        }
        const unsigned q = (unsigned)__ldg(part + w[i]);
        if (q < 32u && (!in_only || keep_edge(__ldg(deg + w[i]), dcur, w[i], cur, tie))) m |= 1u << q;
    }
    if (m) atomicOr(mask + cur, m);
}

__global__ void part_halo_flags_kernel(const int32_t *part, const unsigned *mask, int64_t n, int p, uint8_t *inP,
                                       uint8_t *inH) {
    GRID_STRIDE(v, n) {
        const bool in = part[v] == p;
        inP[v] = (uint8_t)in;
        inH[v] = (uint8_t)(!in && ((mask[v] >> p) & 1u));
    }
}

// More than 32 parts: part p's flags, and its halo by one pass over the entries.
__global__ void part_flags_kernel(const int32_t *part, int64_t n, int p, uint8_t *inP) {
    GRID_STRIDE(v, n) inP[v] = (uint8_t)(part[v] == p);
}

__global__ void halo_flags_kernel(const int32_t *rowid, const int32_t *col, int64_t nnz, const int32_t *part,
                                  const int32_t *deg, int p, int in_only, int tie, uint8_t *inH) {
    GRID_STRIDE(j, nnz) {
        const int s = rowid[j], d = col[j];
        if (part[s] == p && part[d] != p && (!in_only || keep_edge(deg[s], deg[d], s, d, tie))) inH[d] = 1;
    }
}

// ld[v] = (local id or -1, degree): the tile passes gather both with one load.
__global__ void local_ids_kernel(const uint8_t *inP, const uint8_t *inH, const int32_t *lidP, const int32_t *lidH,
                                 const int32_t *deg, int64_t n, int t_ver, int2 *ld) {
    GRID_STRIDE(v, n) ld[v] = make_int2(inP[v] ? lidP[v] : (inH[v] ? t_ver + lidH[v] : -1), deg[v]);
}

// Exclusive scan of one 64-bit value per thread over a 256-thread block.
__device__ __forceinline__ unsigned long long block_scan_256_u64(unsigned long long v, unsigned long long *total) {
    __shared__ unsigned long long wsum[kOT / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned long long x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long t = __shfl_up_sync(kFull, x, o);
        if (lane >= o) x += t;
    }
    if (lane == 31) wsum[warp] = x;
    __syncthreads();
    if (warp == 0) {
        unsigned long long w = lane < kOT / 32 ? wsum[lane] : 0;
#pragma unroll
        for (int o = 1; o < kOT / 32; o <<= 1) {
            const unsigned long long t = __shfl_up_sync(kFull, w, o);
            if (lane >= o) w += t;
        }
        if (lane < kOT / 32) wsum[lane] = w;
    }
    __syncthreads();
    const unsigned long long excl = x - v + (warp ? wsum[warp - 1] : 0);
    *total = wsum[kOT / 32 - 1];
    __syncthreads();
    return excl;
}

// Local edges over the orientation's 4096-entry tiles.  Entry j (row s, id d)
// is a local edge of the part when both ends have a local id and s -> d is the
// oriented direction: a P entry when d is a part vertex (local id < t_ver),
// else an H entry.  A local row lists its P entries, then its H entries, each
// in the undirected row's (ascending) order, so an entry's offset in its local
// row is its rank among the row's entries of its class (plus the row's P count
// for an H entry).  Ranks come from the tiles' P and H counts, scanned, and one
// block scan per tile, as in the orientation; no per-entry flag or position
// array is written.  A third class, R, counts the halo in-degrees without
// atomics: entry j of a halo row s is an R entry when d has a local id and
// d -> s is the oriented direction, so s's in-degree is its row's R count.
//
// Pass 1 (runs) stores the P and H bits of each thread's 16 entries (P in the
// low half, H in the high half), the tile's P, H and R counts (tile_cnt[c *
// tiles + t]) and every row's P, H and R ranks within the tile of its start (16
// bits each, packed: a tile holds 4096 entries).
constexpr int kRankBits = 16;
constexpr unsigned long long kRankMask = (1ull << kRankBits) - 1ull;

__global__ void __launch_bounds__(kOT) halo_tile_count_kernel(const int32_t *__restrict__ rowid,
                                                               const int32_t *__restrict__ col,
                                                               const int2 *__restrict__ ld, int64_t nnz, int64_t V,
                                                               int64_t tiles, int t_ver, int tie,
                                                               uint32_t *__restrict__ bits,
                                                               int32_t *__restrict__ tile_cnt,
                                                               unsigned long long *__restrict__ row_rank) {
    int u[kOI], w[kOI];
    const int64_t j0 = (int64_t)blockIdx.x * kOTile + (int64_t)threadIdx.x * kOI;
    load16(rowid, col, j0, nnz, u, w);
    unsigned pb = 0, hb = 0, rb = 0;
    int cs = -1;
    int2 cx = make_int2(-1, 0);  // the current row: local id, degree
#pragma unroll
    for (int i = 0; i < kOI; ++i) {
        if (j0 + i >= nnz) break;
        if (u[i] != cs) {
            cs = u[i];
            cx = __ldg(ld + cs);
        }
        if (cx.x < 0) continue;
        const int2 wx = __ldg(ld + w[i]);
        if (wx.x < 0) continue;
        if (keep_edge(cx.y, wx.y, cs, w[i], tie)) {
            if (wx.x < t_ver) pb |= 1u << i;
            else hb |= 1u << i;
        } else if (cx.x >= t_ver) {
            rb |= 1u << i;
        }
    }
    bits[(int64_t)blockIdx.x * kOT + threadIdx.x] = pb | (hb << 16);
    auto pack = [](unsigned a, unsigned b, unsigned c) {
        return (unsigned long long)a | ((unsigned long long)b << kRankBits) | ((unsigned long long)c << (2 * kRankBits));
    };
    unsigned long long total = 0;
    const unsigned long long excl = block_scan_256_u64(pack(__popc(pb), __popc(hb), __popc(rb)), &total);
    if (threadIdx.x == 0) {
        tile_cnt[blockIdx.x] = (int)(total & kRankMask);
        tile_cnt[tiles + blockIdx.x] = (int)((total >> kRankBits) & kRankMask);
        tile_cnt[2 * tiles + blockIdx.x] = (int)(total >> (2 * kRankBits));
    }
    if (j0 >= nnz) return;
    int prev = j0 == 0 ? -1 : __ldg(rowid + j0 - 1);
#pragma unroll
    for (int i = 0; i < kOI; ++i) {
        if (j0 + i >= nnz) break;
        if (u[i] == prev) continue;
        const unsigned below = (1u << i) - 1u;
        const unsigned long long rk = excl + pack(__popc(pb & below), __popc(hb & below), __popc(rb & below));
        for (int r = prev + 1; r <= u[i]; ++r) row_rank[r] = rk;  // rows that start at this entry
        prev = u[i];
    }
    if (j0 + kOI >= nnz) {  // the last entry's thread: the rows after it (and row V) start at the end
        const unsigned long long rk = excl + pack(__popc(pb), __popc(hb), __popc(rb));
        for (int64_t r = (int64_t)prev + 1; r <= V; ++r) row_rank[r] = rk;
    }
}

// Global rank of class c (0 = P, 1 = H, 2 = R) at entry index a, whose row-start
// rank (within the tile of a; the last tile for a = nnz) is rk.  off[] is the
// exclusive scan of the 3 * tiles tile counts.
__device__ __forceinline__ int halo_rank(int a, unsigned long long rk, const int32_t *off, int64_t tiles, int c) {
    const int64_t t = min((int64_t)(a / kOTile), tiles - 1);
    return off[c * tiles + t] - off[c * tiles] + (int)((rk >> (c * kRankBits)) & kRankMask);
}

// Per vertex of the part's combined set: its P and H entry counts (from the
// ranks at its row's start and at the next row's start) -> cnt[local id], the
// bases that turn an entry's global rank into its local-row offset, and the
// in-degree of a halo vertex (its row's R count; 0 for a part vertex).
__global__ void halo_rows_kernel(const int32_t *__restrict__ rp, const int2 *__restrict__ ld,
                                 const unsigned long long *__restrict__ row_rank, const int32_t *__restrict__ off,
                                 int64_t V, int64_t tiles, int t_ver, int32_t *__restrict__ cnt,
                                 int32_t *__restrict__ base_p, int32_t *__restrict__ base_h,
                                 int32_t *__restrict__ indeg) {
    GRID_STRIDE(v, V) {
        const int l = ld[v].x;
        if (l < 0) continue;
        const int a = rp[v], b = rp[v + 1];
        const unsigned long long ra = row_rank[v], rb = row_rank[v + 1];
        const int pa = halo_rank(a, ra, off, tiles, 0), np = halo_rank(b, rb, off, tiles, 0) - pa;
        const int ha = halo_rank(a, ra, off, tiles, 1), nh = halo_rank(b, rb, off, tiles, 1) - ha;
        cnt[l] = np + nh;
        base_p[v] = pa;       // P entry of rank x: local offset x - pa
        base_h[v] = ha - np;  // H entry of rank x: local offset np + (x - ha)
        indeg[l] = l >= t_ver ? halo_rank(b, rb, off, tiles, 2) - halo_rank(a, ra, off, tiles, 2) : 0;
    }
}

// Pass 2 (strided): ranks each tile's P and H entries again from the stored
// bits with warp ballots and writes every local edge at lrp[local row] + its
// offset (lcol = the local id of the target); consecutive lanes write
// consecutive positions.
__global__ void __launch_bounds__(kOT) halo_tile_write_kernel(const int32_t *__restrict__ rowid,
                                                               const int32_t *__restrict__ col,
                                                               const int2 *__restrict__ ld,
                                                               const uint32_t *__restrict__ bits, int64_t nnz,
                                                               int64_t tiles, const int32_t *__restrict__ off,
                                                               const int32_t *__restrict__ lrp,
                                                               const int32_t *__restrict__ base_p,
                                                               const int32_t *__restrict__ base_h,
                                                               int32_t *__restrict__ lcol) {
    const int64_t j0 = strided_first();
    const int lane = threadIdx.x & 31;
    const uint32_t cw = bits[(int64_t)blockIdx.x * kOT + threadIdx.x];  // pass 1's run of this lane
    const unsigned lt = (1u << lane) - 1u;
    const unsigned wsum = (unsigned)__reduce_add_sync(kFull, __popc(cw & 0xffffu)) |
                          ((unsigned)__reduce_add_sync(kFull, __popc(cw >> 16)) << 16);
    unsigned total = 0;
    const unsigned wo = warp_offsets_256(wsum, &total);
    int pr = off[blockIdx.x] + (int)(wo & 0xffffu);                // P rank of the warp's next P entry
    int hr = off[tiles + blockIdx.x] - off[tiles] + (int)(wo >> 16);  // H rank likewise
#pragma unroll
    for (int i = 0; i < kOI; ++i) {
        const int64_t j = j0 + 32 * i;
        if (j - lane >= nnz) break;  // warp-uniform
        // entry 32 i + lane of the warp's 512 is bit lane % 16 of lane 2 i + lane / 16's run
        const uint32_t rw = __shfl_sync(kFull, cw, 2 * i + (lane >> 4)) >> (lane & 15);
        const bool kp = rw & 1u, kh = (rw >> 16) & 1u;
        const unsigned bp = __ballot_sync(kFull, kp), bh = __ballot_sync(kFull, kh);
        if (kp || kh) {
            const int s = __ldg(rowid + j);
            const int ls = __ldg(ld + s).x;
            const int lr = __ldg(lrp + ls);
            const int o = kp ? lr - __ldg(base_p + s) + pr + __popc(bp & lt) : lr - __ldg(base_h + s) + hr + __popc(bh & lt);
            lcol[o] = __ldg(ld + __ldg(col + j)).x;
        }
        pr += __popc(bp);
        hr += __popc(bh);
    }
}

__global__ void frontier_init_kernel(const int32_t *indeg, int64_t n, int t_ver, uint8_t *removed, int32_t *front,
                                     int32_t *front_n) {
    GRID_STRIDE(i, n) {
        if (i >= t_ver && indeg[i] == 0) {
            removed[i] = 1;
            front[atomicAdd(front_n, 1)] = (int32_t)i;
        }
    }
}

// Peel round r, one warp per frontier vertex: drop its out-edges; halo targets
// reaching in-degree 0 join the next frontier (exactly once: the 1 -> 0
// transition).  Frontier sizes stay on the device so that several rounds go
// out per host check: fn[r % 3] is round r's frontier size (front_a for even r,
// front_b for odd r), fn[(r + 1) % 3] (zeroed by round r - 1, or before round 0)
// counts the next frontier, and fn[(r + 2) % 3], which no block of round r
// reads, is zeroed for round r + 1.  fn[3] totals the frontier sizes.  A round
// whose frontier is empty does nothing.
__global__ void peel_round_kernel(int32_t *front_a, int32_t *front_b, int32_t *fn, int r, const int32_t *lrp,
                                  const int32_t *lcol, int t_ver, int32_t *indeg, uint8_t *removed) {
    const int32_t *front = (r & 1) ? front_b : front_a;
    int32_t *next = (r & 1) ? front_a : front_b;
    const int n_front = fn[r % 3];
    int32_t *next_n = fn + (r + 1) % 3;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        fn[(r + 2) % 3] = 0;
        fn[3] += n_front;
    }
    const int lane = threadIdx.x & 31;
    const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t f = w0; f < n_front; f += nw) {
        const int x = front[f];
        for (int j = lrp[x] + lane; j < lrp[x + 1]; j += 32) {
            const int d = lcol[j];
            if (atomicSub(&indeg[d], 1) == 1 && d >= t_ver) {
                removed[d] = 1;
                next[atomicAdd(next_n, 1)] = d;
            }
        }
    }
}

__global__ void alive_kernel(const uint8_t *removed, const int32_t *lrp, int64_t n, uint8_t *alive, int32_t *len) {
    GRID_STRIDE(i, n) {
        const bool a = !removed[i];
        alive[i] = (uint8_t)a;
        len[i] = a ? lrp[i + 1] - lrp[i] : 0;
    }
}

__global__ void prune_rows_kernel(const uint8_t *alive, const int32_t *nid, const int32_t *newpos, int64_t n,
                                  int32_t *rp2) {
    GRID_STRIDE(i, n) {
        if (alive[i]) rp2[nid[i]] = newpos[i];
    }
}

// One warp per surviving local row: its entries, renumbered, at the row's new
// start (consecutive lanes write consecutive positions).
__global__ void prune_cols_kernel(const int32_t *__restrict__ lcol, const int32_t *__restrict__ lrp, int64_t n,
                                  const uint8_t *__restrict__ alive, const int32_t *__restrict__ nid,
                                  const int32_t *__restrict__ newpos, int32_t *__restrict__ col2) {
    const int lane = threadIdx.x & 31;
    const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t i = w0; i < n; i += nw) {
        if (!alive[i]) continue;
        const int a = lrp[i], b = lrp[i + 1], o = newpos[i] - a;
        for (int e = a + lane; e < b; e += 32) col2[o + e] = nid[lcol[e]];
    }
}

template <class T>
int d2h_scalar(T *h, const T *d, cudaStream_t s) {
    TC_CUDA(cudaMemcpyAsync(h, d, sizeof(T), cudaMemcpyDeviceToHost, s));
    TC_CUDA(cudaStreamSynchronize(s));
    return TC_OK;
}

int finish_ugraph(tc_ctx *ctx, int32_t *rp, int32_t *col, int32_t *deg, int32_t *rowid, int64_t n_rows, int64_t nnz,
                  tc_ugraph **out) {
    tc_ugraph *g = new tc_ugraph();
    g->ctx = ctx;
    ctx_retain(ctx);
    g->rp = rp;
    g->col = col;
    g->deg = deg;
    g->rowid = rowid;
    g->n_rows = n_rows;
    g->nnz = nnz;
    *out = g;
    return TC_OK;
}

}  // namespace

}  // namespace tc

using namespace tc;

extern "C" {

int tc_ugraph_from_edges(tc_ctx *ctx, const int64_t *src, const int64_t *dst, int64_t n_edges, int64_t n_nodes,
                         tc_ugraph **out) {
    if (!ctx || !out || n_edges < 0 || (n_edges > 0 && (!src || !dst)))
        return set_error(TC_E_INVALID, "bad edge-list arguments");
    *out = nullptr;
    if (2 * n_edges >= INT32_MAX) return set_error(TC_E_RANGE, "%lld edges exceed the int32 entry limit", (long long)n_edges);
    cudaStream_t s = ctx->stream;
    DBuf<int64_t> dsrc, ddst;
    DBuf<unsigned long long> dmax;
    DBuf<int> dneg;
    TC_TRY(dsrc.alloc((size_t)n_edges, s));
    TC_TRY(ddst.alloc((size_t)n_edges, s));
    TC_TRY(dmax.alloc(1, s));
    TC_TRY(dneg.alloc(1, s));
    TC_CUDA(cudaMemsetAsync(dmax.p, 0, sizeof(unsigned long long), s));
    TC_CUDA(cudaMemsetAsync(dneg.p, 0, sizeof(int), s));
    if (n_edges) {
        TC_CUDA(cudaMemcpyAsync(dsrc.p, src, sizeof(int64_t) * (size_t)n_edges, cudaMemcpyHostToDevice, s));
        TC_CUDA(cudaMemcpyAsync(ddst.p, dst, sizeof(int64_t) * (size_t)n_edges, cudaMemcpyHostToDevice, s));
        max_id_kernel<<<grid(n_edges, ctx), 256, 0, s>>>(dsrc.p, ddst.p, n_edges, dmax.p, dneg.p);
        TC_CUDA(cudaGetLastError());
    }
    unsigned long long mx = 0;
    int neg = 0;
    TC_TRY(d2h_scalar(&mx, dmax.p, s));
    TC_TRY(d2h_scalar(&neg, dneg.p, s));
    if (neg) return set_error(TC_E_RANGE, "negative vertex id in edge list");
    const int64_t n0 = std::max<int64_t>(n_nodes, n_edges ? (int64_t)mx + 1 : 0);
    if (n0 >= INT32_MAX) return set_error(TC_E_RANGE, "vertex id %lld does not fit int32", (long long)n0 - 1);
    int B = 1;
    while (B < 31 && ((int64_t)1 << B) < n0) ++B;
    const int64_t n2 = 2 * n_edges;
    DBuf<uint64_t> ka, kb;
    TC_TRY(ka.alloc((size_t)n2, s));
    TC_TRY(kb.alloc((size_t)n2, s));
    if (n_edges) {
        make_keys_kernel<<<grid(n_edges, ctx), 256, 0, s>>>(dsrc.p, ddst.p, n_edges, B, ka.p);
        TC_CUDA(cudaGetLastError());
    }
    dsrc.reset();
    ddst.reset();
    uint64_t *keys = ka.p, *tmp = kb.p;
    TC_TRY(radix_sort_u64(&keys, &tmp, n2, 2 * B, s));
    DBuf<uint8_t> flags;
    DBuf<int32_t> pos;
    TC_TRY(flags.alloc((size_t)n2, s));
    TC_TRY(pos.alloc((size_t)n2 + 1, s));
    if (n2) {
        unique_flags_kernel<<<grid(n2, ctx), 256, 0, s>>>(keys, n2, flags.p);
        TC_CUDA(cudaGetLastError());
    }
    TC_TRY(scan_flags_u8(flags.p, pos.p, n2, s));
    int32_t nnz32 = 0;
    TC_TRY(d2h_scalar(&nnz32, pos.p + n2, s));
    const int64_t nnz = nnz32;
    DBuf<int32_t> col, rowid, cnt;
    TC_TRY(col.alloc((size_t)nnz, s));
    TC_TRY(rowid.alloc((size_t)nnz, s));
    TC_TRY(cnt.alloc((size_t)n0 + 1, s));
    TC_CUDA(cudaMemsetAsync(cnt.p, 0, sizeof(int32_t) * ((size_t)n0 + 1), s));
    if (n2) {
        unique_scatter_kernel<<<grid(n2, ctx), 256, 0, s>>>(keys, n2, flags.p, pos.p, B, col.p, rowid.p, cnt.p);
        TC_CUDA(cudaGetLastError());
    }
    ka.reset();
    kb.reset();
    pos.reset();
    // order-preserving relabel of the non-isolated vertices
    DBuf<uint8_t> keep;
    DBuf<int32_t> newid, rs_old;
    TC_TRY(keep.alloc((size_t)n0, s));
    TC_TRY(newid.alloc((size_t)n0 + 1, s));
    TC_TRY(rs_old.alloc((size_t)n0 + 1, s));
    if (n0) {
        keep_nonisolated_kernel<<<grid(n0, ctx), 256, 0, s>>>(cnt.p, n0, keep.p);
        TC_CUDA(cudaGetLastError());
    }
    TC_TRY(scan_flags_u8(keep.p, newid.p, n0, s));
    TC_TRY(scan_exclusive_i32(cnt.p, rs_old.p, n0, s));
    int32_t V32 = 0;
    TC_TRY(d2h_scalar(&V32, newid.p + n0, s));
    const int64_t V = V32;
    DBuf<int32_t> rp, deg;
    TC_TRY(rp.alloc((size_t)V + 1, s));
    TC_TRY(deg.alloc((size_t)std::max<int64_t>(V, 1), s));
    if (n0) {
        relabel_rows_kernel<<<grid(n0, ctx), 256, 0, s>>>(keep.p, newid.p, rs_old.p, n0, rp.p);
        TC_CUDA(cudaGetLastError());
    }
    TC_CUDA(cudaMemcpyAsync(rp.p + V, &nnz32, sizeof(int32_t), cudaMemcpyHostToDevice, s));
    if (nnz) {
        remap_kernel<<<grid(nnz, ctx), 256, 0, s>>>(col.p, nnz, newid.p);
        remap_kernel<<<grid(nnz, ctx), 256, 0, s>>>(rowid.p, nnz, newid.p);
        TC_CUDA(cudaGetLastError());
    }
    if (V) {
        degree_kernel<<<grid(V, ctx), 256, 0, s>>>(rp.p, V, deg.p);
        TC_CUDA(cudaGetLastError());
    }
    TC_CUDA(cudaStreamSynchronize(s));
    return finish_ugraph(ctx, rp.release(), col.release(), deg.release(), rowid.release(), V, nnz, out);
}

int tc_ugraph_upload_i64(tc_ctx *ctx, const int64_t *row_ptr, const int64_t *col, const int64_t *deg, int64_t n_rows,
                         int64_t nnz, tc_ugraph **out) {
    if (!ctx || !out || !row_ptr || n_rows < 0 || nnz < 0 || (nnz > 0 && !col))
        return set_error(TC_E_INVALID, "bad undirected CSR arguments");
    *out = nullptr;
    if (n_rows >= INT32_MAX || nnz >= INT32_MAX)
        return set_error(TC_E_RANGE, "undirected CSR too large for int32 indices");
    cudaStream_t s = ctx->stream;
    DBuf<int64_t> stage;
    DBuf<int> bad;
    DBuf<int32_t> rp, cl, dg, rowid;
    TC_TRY(stage.alloc((size_t)std::max(n_rows + 1, nnz), s));
    TC_TRY(bad.alloc(1, s));
    TC_TRY(rp.alloc((size_t)n_rows + 1, s));
    TC_TRY(cl.alloc((size_t)nnz, s));
    TC_TRY(dg.alloc((size_t)std::max<int64_t>(n_rows, 1), s));
    TC_TRY(rowid.alloc((size_t)nnz, s));
    TC_CUDA(cudaMemsetAsync(bad.p, 0, sizeof(int), s));
    const int64_t *srcs[3] = {row_ptr, col, deg};
    int32_t *dsts[3] = {rp.p, cl.p, dg.p};
    const int64_t ns[3] = {n_rows + 1, nnz, deg ? n_rows : 0};
    for (int k = 0; k < 3; ++k) {
        if (ns[k] == 0) continue;
        TC_CUDA(cudaMemcpyAsync(stage.p, srcs[k], sizeof(int64_t) * (size_t)ns[k], cudaMemcpyHostToDevice, s));
        narrow_i64_kernel<<<grid(ns[k], ctx), 256, 0, s>>>(stage.p, dsts[k], ns[k], INT32_MAX - 1, bad.p);
        TC_CUDA(cudaGetLastError());
    }
    int hbad = 0;
    TC_TRY(d2h_scalar(&hbad, bad.p, s));
    if (hbad) return set_error(TC_E_RANGE, "undirected CSR value is negative or does not fit int32");
    stage.reset();
    TC_TRY(validate_csr(ctx, rp.p, cl.p, n_rows, nnz));
    if (!deg && n_rows) {
        degree_kernel<<<grid(n_rows, ctx), 256, 0, s>>>(rp.p, n_rows, dg.p);
        TC_CUDA(cudaGetLastError());
    }
    if (n_rows) {
        rowid_kernel<<<grid(n_rows * 32, ctx), 256, 0, s>>>(rp.p, n_rows, rowid.p);
        TC_CUDA(cudaGetLastError());
    }
    if (nnz) {  // the halo extraction reads each edge from either end
        check_symmetric_kernel<<<grid(nnz, ctx), 256, 0, s>>>(rp.p, cl.p, rowid.p, nnz, bad.p);
        TC_CUDA(cudaGetLastError());
        TC_TRY(d2h_scalar(&hbad, bad.p, s));
        if (hbad) return set_error(TC_E_INVALID, "undirected CSR has a self-loop or an edge missing from one of its rows");
    }
    TC_CUDA(cudaStreamSynchronize(s));
    return finish_ugraph(ctx, rp.release(), cl.release(), dg.release(), rowid.release(), n_rows, nnz, out);
}

int tc_ugraph_info(const tc_ugraph *g, int64_t *n_rows, int64_t *nnz) {
    if (!g) return set_error(TC_E_INVALID, "null graph");
    if (n_rows) *n_rows = g->n_rows;
    if (nnz) *nnz = g->nnz;
    return TC_OK;
}

int tc_ugraph_download(tc_ctx *ctx, const tc_ugraph *g, int64_t *row_ptr, int64_t *col, int64_t *deg) {
    if (!g) return set_error(TC_E_INVALID, "null graph");
    if (!ctx) ctx = g->ctx;
    cudaStream_t s = ctx->stream;
    std::vector<int32_t> tmp;
    const int32_t *srcs[3] = {g->rp, g->col, g->deg};
    int64_t *dsts[3] = {row_ptr, col, deg};
    const int64_t ns[3] = {g->n_rows + 1, g->nnz, g->n_rows};
    for (int k = 0; k < 3; ++k) {
        if (!dsts[k] || ns[k] == 0) continue;
        tmp.resize((size_t)ns[k]);
        TC_CUDA(cudaMemcpyAsync(tmp.data(), srcs[k], sizeof(int32_t) * (size_t)ns[k], cudaMemcpyDeviceToHost, s));
        TC_CUDA(cudaStreamSynchronize(s));
        for (int64_t i = 0; i < ns[k]; ++i) dsts[k][i] = tmp[(size_t)i];
    }
    return TC_OK;
}

int tc_ugraph_destroy(tc_ugraph *g) {
    if (!g) return TC_OK;
    cudaStream_t s = g->ctx ? g->ctx->stream : nullptr;
    dfree(g->rp, s);
    dfree(g->col, s);
    dfree(g->deg, s);
    dfree(g->rowid, s);
    tc_ctx *ctx = g->ctx;
    delete g;
    ctx_release(ctx);
    return TC_OK;
}

int tc_orient(tc_ctx *ctx, const tc_ugraph *ug, int tie, tc_graph **out) {
    if (!ug || !out || (tie != TC_TIE_REFERENCE && tie != TC_TIE_ID_ASC))
        return set_error(TC_E_INVALID, "bad orientation arguments");
    if (!ctx) ctx = ug->ctx;
    *out = nullptr;
    cudaStream_t s = ctx->stream;
    const int64_t V = ug->n_rows, nnz = ug->nnz;
    const int64_t tiles = (nnz + kOTile - 1) / kOTile;
    DBuf<int32_t> tile_cnt, tile_off, orp, ocol;
    DBuf<uint16_t> keep;
    TC_TRY(keep.alloc((size_t)std::max<int64_t>(tiles, 1) * kOT, s));
    TC_TRY(tile_cnt.alloc((size_t)std::max<int64_t>(tiles, 1), s));
    TC_TRY(tile_off.alloc((size_t)tiles + 1, s));
    TC_TRY(orp.alloc((size_t)V + 1, s));
    int32_t m32 = 0;
    if (tiles) {
        orient_tile_count_kernel<<<(unsigned)tiles, kOT, 0, s>>>(ug->rowid, ug->col, ug->deg, nnz, tie, tile_cnt.p,
                                                                  keep.p);
        TC_CUDA(cudaGetLastError());
        TC_TRY(scan_exclusive_i32(tile_cnt.p, tile_off.p, tiles, s));  // tile_off[tiles] = the kept total
        TC_TRY(d2h_scalar(&m32, tile_off.p + tiles, s));
    }
    TC_TRY(ocol.alloc((size_t)std::max<int32_t>(m32, 1), s));
    if (tiles) {
        orient_tile_write_kernel<<<(unsigned)tiles, kOT, 0, s>>>(ug->rowid, ug->col, keep.p, nnz, V, tile_off.p,
                                                                  orp.p, ocol.p);
        TC_CUDA(cudaGetLastError());
    } else {
        TC_CUDA(cudaMemsetAsync(orp.p, 0, sizeof(int32_t) * (size_t)(V + 1), s));
    }
    TC_CUDA(cudaStreamSynchronize(s));
    tc_graph *g = nullptr;
    TC_TRY(graph_adopt_device(ctx, orp.p, ocol.p, V, m32, V, &g));
    orp.release();
    ocol.release();
    *out = g;
    return TC_OK;
}

int tc_graph_from_edges(tc_ctx *ctx, const int64_t *src, const int64_t *dst, int64_t n_edges, int64_t n_nodes, int tie,
                        tc_graph **out) {
    tc_ugraph *ug = nullptr;
    TC_TRY(tc_ugraph_from_edges(ctx, src, dst, n_edges, n_nodes, &ug));
    const int st = tc_orient(ctx, ug, tie, out);
    tc_ugraph_destroy(ug);
    return st;
}

int tc_halo_extract(tc_ctx *ctx, const tc_ugraph *ug, const int32_t *part, int k, int tie, tc_graph **parts_out) {
    return tc_halo_extract_ex(ctx, ug, part, k, tie, TC_HALO_REFERENCE, parts_out);
}

int tc_halo_extract_ex(tc_ctx *ctx, const tc_ugraph *ug, const int32_t *part, int k, int tie, int mode,
                       tc_graph **parts_out) {
    if (!ug || !part || k < 1 || !parts_out || (tie != TC_TIE_REFERENCE && tie != TC_TIE_ID_ASC))
        return set_error(TC_E_INVALID, "bad halo arguments");
    if (mode != TC_HALO_REFERENCE && mode != TC_HALO_COUNT) return set_error(TC_E_INVALID, "bad halo mode %d", mode);
    const int in_only = mode == TC_HALO_COUNT;
    if (!ctx) ctx = ug->ctx;
    for (int p = 0; p < k; ++p) parts_out[p] = nullptr;
    cudaStream_t s = ctx->stream;
    const int64_t V = ug->n_rows, nnz = ug->nnz;
    for (int64_t v = 0; v < V; ++v)
        if (part[v] < 0) return set_error(TC_E_RANGE, "part[%lld] = %d is negative", (long long)v, part[v]);
    const int64_t tiles = (nnz + kOTile - 1) / kOTile;
    DBuf<int32_t> dpart, lidP, lidH, cnt, lrp, tile_cnt, tile_off, base_p, base_h;
    DBuf<int2> ld;
    DBuf<uint32_t> bits, mask;
    DBuf<unsigned long long> row_rank;
    DBuf<uint8_t> inP, inH;
    TC_TRY(dpart.alloc((size_t)std::max<int64_t>(V, 1), s));
    if (V) TC_CUDA(cudaMemcpyAsync(dpart.p, part, sizeof(int32_t) * (size_t)V, cudaMemcpyHostToDevice, s));
    TC_TRY(inP.alloc((size_t)V, s));
    TC_TRY(inH.alloc((size_t)V, s));
    TC_TRY(lidP.alloc((size_t)V + 1, s));
    TC_TRY(lidH.alloc((size_t)V + 1, s));
    TC_TRY(ld.alloc((size_t)std::max<int64_t>(V, 1), s));
    TC_TRY(cnt.alloc((size_t)V + 1, s));
    TC_TRY(lrp.alloc((size_t)V + 1, s));
    TC_TRY(base_p.alloc((size_t)std::max<int64_t>(V, 1), s));
    TC_TRY(base_h.alloc((size_t)std::max<int64_t>(V, 1), s));
    TC_TRY(row_rank.alloc((size_t)V + 1, s));
    TC_TRY(bits.alloc((size_t)std::max<int64_t>(tiles, 1) * kOT, s));
    TC_TRY(tile_cnt.alloc((size_t)std::max<int64_t>(3 * tiles, 1), s));
    TC_TRY(tile_off.alloc((size_t)3 * tiles + 1, s));
    const int gV = grid(V, ctx), gE = grid(nnz, ctx);
    const bool masks = k <= 32;  // every part's halo from one pass
    if (masks) {
        TC_TRY(mask.alloc((size_t)std::max<int64_t>(V, 1), s));
        TC_CUDA(cudaMemsetAsync(mask.p, 0, sizeof(uint32_t) * (size_t)std::max<int64_t>(V, 1), s));
        if (tiles)
            halo_mask_kernel<<<(unsigned)tiles, kOT, 0, s>>>(ug->rowid, ug->col, dpart.p, ug->deg, nnz, in_only, tie,
                                                              mask.p);
        TC_CUDA(cudaGetLastError());
    }
    // one part; any failure returns its status (the caller frees all parts)
    auto one_part = [&](int p) -> int {
        if (masks) {
            if (V) part_halo_flags_kernel<<<gV, 256, 0, s>>>(dpart.p, mask.p, V, p, inP.p, inH.p);
        } else {
            if (V) part_flags_kernel<<<gV, 256, 0, s>>>(dpart.p, V, p, inP.p);
            TC_CUDA(cudaMemsetAsync(inH.p, 0, (size_t)V, s));
            if (nnz)
                halo_flags_kernel<<<gE, 256, 0, s>>>(ug->rowid, ug->col, nnz, dpart.p, ug->deg, p, in_only, tie, inH.p);
        }
        TC_CUDA(cudaGetLastError());
        TC_TRY(scan_flags_u8(inP.p, lidP.p, V, s));
        TC_TRY(scan_flags_u8(inH.p, lidH.p, V, s));
        int32_t t_ver = 0, n_halo = 0;
        TC_CUDA(cudaMemcpyAsync(&t_ver, lidP.p + V, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        TC_CUDA(cudaMemcpyAsync(&n_halo, lidH.p + V, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        TC_CUDA(cudaStreamSynchronize(s));
        const int64_t n_comb = (int64_t)t_ver + n_halo;
        if (V) local_ids_kernel<<<gV, 256, 0, s>>>(inP.p, inH.p, lidP.p, lidH.p, ug->deg, V, t_ver, ld.p);
        DBuf<int32_t> indeg;
        TC_TRY(indeg.alloc((size_t)std::max<int64_t>(n_comb, 1), s));
        if (tiles) {
            halo_tile_count_kernel<<<(unsigned)tiles, kOT, 0, s>>>(ug->rowid, ug->col, ld.p, nnz, V, tiles, t_ver, tie,
                                                                    bits.p, tile_cnt.p, row_rank.p);
            TC_CUDA(cudaGetLastError());
            TC_TRY(scan_exclusive_i32(tile_cnt.p, tile_off.p, 3 * tiles, s));
            if (V)
                halo_rows_kernel<<<gV, 256, 0, s>>>(ug->rp, ld.p, row_rank.p, tile_off.p, V, tiles, t_ver, cnt.p,
                                                    base_p.p, base_h.p, indeg.p);
            TC_CUDA(cudaGetLastError());
        } else {
            TC_CUDA(cudaMemsetAsync(cnt.p, 0, sizeof(int32_t) * ((size_t)n_comb + 1), s));
            TC_CUDA(cudaMemsetAsync(indeg.p, 0, sizeof(int32_t) * (size_t)std::max<int64_t>(n_comb, 1), s));
        }
        TC_TRY(scan_exclusive_i32(cnt.p, lrp.p, n_comb, s));
        int32_t lnnz = 0;
        TC_TRY(d2h_scalar(&lnnz, lrp.p + n_comb, s));
        DBuf<int32_t> lcol, front, next, fn;
        DBuf<uint8_t> removed;
        TC_TRY(lcol.alloc((size_t)lnnz, s));
        if (tiles && lnnz)
            halo_tile_write_kernel<<<(unsigned)tiles, kOT, 0, s>>>(ug->rowid, ug->col, ld.p, bits.p, nnz, tiles,
                                                                    tile_off.p, lrp.p, base_p.p, base_h.p, lcol.p);
        TC_CUDA(cudaGetLastError());
        // prune: peel halo vertices of zero in-degree until none is left
        TC_TRY(removed.alloc((size_t)std::max<int64_t>(n_comb, 1), s));
        TC_TRY(front.alloc((size_t)std::max<int32_t>(n_halo, 1), s));
        TC_TRY(next.alloc((size_t)std::max<int32_t>(n_halo, 1), s));
        TC_TRY(fn.alloc(4, s));
        TC_CUDA(cudaMemsetAsync(removed.p, 0, (size_t)std::max<int64_t>(n_comb, 1), s));
        TC_CUDA(cudaMemsetAsync(fn.p, 0, 4 * sizeof(int32_t), s));
        if (n_comb) frontier_init_kernel<<<grid(n_comb, ctx), 256, 0, s>>>(indeg.p, n_comb, t_ver, removed.p, front.p, fn.p);
        TC_CUDA(cudaGetLastError());
        // kPeelBatch rounds per host check; each non-empty round removes at
        // least one halo vertex, so at most n_halo of them are non-empty
        constexpr int kPeelBatch = 4;
        const int peel_grid = std::min(grid((int64_t)std::max<int32_t>(n_halo, 1) * 32, ctx), ctx->sm_count * 4);
        int32_t hfn[4] = {0, 0, 0, 0};
        int round = 0;
        while (round <= n_halo) {
            for (int q = 0; q < kPeelBatch; ++q, ++round)
                peel_round_kernel<<<peel_grid, 256, 0, s>>>(front.p, next.p, fn.p, round, lrp.p, lcol.p, t_ver, indeg.p,
                                                            removed.p);
            TC_CUDA(cudaGetLastError());
            TC_CUDA(cudaMemcpyAsync(hfn, fn.p, sizeof(hfn), cudaMemcpyDeviceToHost, s));
            TC_CUDA(cudaStreamSynchronize(s));
            if (hfn[round % 3] == 0) break;  // the next round's frontier is empty
        }
        const int64_t n_removed = (int64_t)hfn[3] + hfn[round % 3];
        int32_t *out_rp = nullptr, *out_col = nullptr;
        int64_t n_local = n_comb, out_nnz = lnnz;
        if (n_removed == 0) {
            DBuf<int32_t> rp_copy;
            TC_TRY(rp_copy.alloc((size_t)n_comb + 1, s));
            TC_CUDA(cudaMemcpyAsync(rp_copy.p, lrp.p, sizeof(int32_t) * ((size_t)n_comb + 1), cudaMemcpyDeviceToDevice, s));
            out_rp = rp_copy.release();
            out_col = lcol.release();
        } else {
            DBuf<uint8_t> alive;
            DBuf<int32_t> len, nid, newpos, rp2, col2;
            TC_TRY(alive.alloc((size_t)n_comb, s));
            TC_TRY(len.alloc((size_t)n_comb, s));
            TC_TRY(nid.alloc((size_t)n_comb + 1, s));
            TC_TRY(newpos.alloc((size_t)n_comb + 1, s));
            alive_kernel<<<grid(n_comb, ctx), 256, 0, s>>>(removed.p, lrp.p, n_comb, alive.p, len.p);
            TC_CUDA(cudaGetLastError());
            TC_TRY(scan_flags_u8(alive.p, nid.p, n_comb, s));
            TC_TRY(scan_exclusive_i32(len.p, newpos.p, n_comb, s));
            int32_t nl = 0, nn = 0;
            TC_CUDA(cudaMemcpyAsync(&nl, nid.p + n_comb, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
            TC_CUDA(cudaMemcpyAsync(&nn, newpos.p + n_comb, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
            TC_CUDA(cudaStreamSynchronize(s));
            n_local = nl;
            out_nnz = nn;
            TC_TRY(rp2.alloc((size_t)nl + 1, s));
            TC_TRY(col2.alloc((size_t)std::max(nn, 1), s));
            prune_rows_kernel<<<grid(n_comb, ctx), 256, 0, s>>>(alive.p, nid.p, newpos.p, n_comb, rp2.p);
            TC_CUDA(cudaMemcpyAsync(rp2.p + nl, &nn, sizeof(int32_t), cudaMemcpyHostToDevice, s));
            if (lnnz)
                prune_cols_kernel<<<grid(n_comb * 32, ctx), 256, 0, s>>>(lcol.p, lrp.p, n_comb, alive.p, nid.p,
                                                                         newpos.p, col2.p);
            TC_CUDA(cudaGetLastError());
            TC_CUDA(cudaStreamSynchronize(s));
            out_rp = rp2.release();
            out_col = col2.release();
        }
        TC_CUDA(cudaStreamSynchronize(s));
        const int ast = graph_adopt_device(ctx, out_rp, out_col, n_local, out_nnz, t_ver, &parts_out[p]);
        if (ast != TC_OK) {
            dfree(out_rp, s);
            dfree(out_col, s);
        }
        return ast;
    };
    int st = TC_OK;
    for (int p = 0; p < k && st == TC_OK; ++p) st = one_part(p);
    if (st != TC_OK)
        for (int p = 0; p < k; ++p) {
            tc_graph_destroy(parts_out[p]);
            parts_out[p] = nullptr;
        }
    return st;
}

}  // extern "C"
