// tc_scan.cu -- device-wide exclusive scans and the LSD radix sort used by the
// preprocessing and halo stages (the reference uses cp.cumsum,
// cub::DeviceScan::InclusiveSum, cub::DeviceMergeSort and cub::DeviceSelect
// for these steps: without_part_preprocess.py:256, round_clean_subgraph.cu:468-495, 561-567).
//
// Scan: reduce-then-scan over tiles of 4096 values (256 threads x 16, each
// warp scanning runs of 32 consecutive values, so every access is
// coalesced), the tile sums scanned recursively.  Radix sort: 8-bit digits, per pass
// (1) per-tile digit histograms, (2) one exclusive scan over the
// digit-major histogram table, (3) a stable scatter in which each warp ranks
// its contiguous 512-key segment with __match_any_sync and the block stages
// the tile in shared memory so that global writes are runs of equal digits.
#include <algorithm>

#include "tc_internal.h"

namespace tc {
namespace {

constexpr int kT = 256;           // threads per block
constexpr int kItems = 16;        // values per thread
constexpr int kTile = kT * kItems;
constexpr unsigned kFull = 0xffffffffu;

// Scan input: the high halves of packed 64-bit words (the count kernel's
// in-edge counts in its in_work words).
struct HighHalf {
    const unsigned long long *p;
    __device__ __forceinline__ int32_t operator[](int64_t i) const { return (int32_t)(p[i] >> 32); }
};

template <class T>
__device__ __forceinline__ T warp_incl_scan(T v, int lane) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const T t = __shfl_up_sync(kFull, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

// Block-wide exclusive scan of one value per thread; returns the block total
// through *total.
template <class T>
__device__ __forceinline__ T block_excl_scan(T v, T *total) {
    __shared__ T warp_tot[kT / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const T incl = warp_incl_scan(v, lane);
    if (lane == 31) warp_tot[w] = incl;
    __syncthreads();
    if (w == 0) {
        T x = lane < kT / 32 ? warp_tot[lane] : T(0);
        x = warp_incl_scan(x, lane);
        if (lane < kT / 32) warp_tot[lane] = x;
    }
    __syncthreads();
    const T before = w ? warp_tot[w - 1] : T(0);
    *total = warp_tot[kT / 32 - 1];
    __syncthreads();
    return before + incl - v;
}

// The scans read their input through In: a plain pointer, or HighHalf below.
template <class In, class Out>
__global__ void __launch_bounds__(kT) tile_reduce_kernel(In in, int64_t n, Out *tile_sums) {
    const int64_t base = (int64_t)blockIdx.x * kTile;
    Out s = 0;
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
        const int64_t i = base + (int64_t)k * kT + threadIdx.x;
        if (i < n) s += (Out)in[i];
    }
    Out tot;
    block_excl_scan<Out>(s, &tot);
    if (threadIdx.x == 0) tile_sums[blockIdx.x] = tot;
}

// Exclusive scan of one tile [base, base + kTile) in a warp-striped layout:
// warp w owns kItems runs of 32 consecutive values, so every load and store
// of a warp is one coalesced 32-value access.  Values are held in registers
// between the warp totals' block scan and the per-run warp scans, so out may
// alias in.  out[i] = off + the tile's exclusive prefix; with slots set,
// slots[i] also gets out[i] added to its high half.  Returns the tile total.
template <class In, class Out>
__device__ __forceinline__ Out scan_tile_striped(In in, int64_t n, int64_t base, Out off, Out *out,
                                                 unsigned long long *slots) {
    __shared__ Out warp_tot[kT / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t wb = base + (int64_t)w * (kItems * 32);
    Out v[kItems];
    Out s = 0;
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
        const int64_t i = wb + k * 32 + lane;
        v[k] = i < n ? (Out)in[i] : Out(0);
        s += v[k];
    }
    s = __shfl_sync(kFull, warp_incl_scan(s, lane), 31);
    if (lane == 0) warp_tot[w] = s;
    __syncthreads();
    Out run = off, tot = 0;
#pragma unroll
    for (int j = 0; j < kT / 32; ++j) {
        const Out t = warp_tot[j];
        run += j < w ? t : Out(0);
        tot += t;
    }
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
        const Out incl = warp_incl_scan(v[k], lane);
        const int64_t i = wb + k * 32 + lane;
        if (i < n) {
            const Out x = run + incl - v[k];
            out[i] = x;
            if (slots) slots[i] += (unsigned long long)x << 32;
        }
        run += __shfl_sync(kFull, incl, 31);
    }
    return tot;
}

// Exclusive scan of each tile plus the tile's offset; out[n] gets the total
// when the last tile is processed (tile_off has n_tiles + 1 entries).
template <class In, class Out>
__global__ void __launch_bounds__(kT) tile_scan_kernel(In in, int64_t n, const Out *tile_off, Out *out,
                                                       unsigned long long *slots) {
    scan_tile_striped<In, Out>(in, n, (int64_t)blockIdx.x * kTile, tile_off[blockIdx.x], out, slots);
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) out[n] = tile_off[gridDim.x];
}

// One-tile scan (n <= kTile): out[0..n) exclusive, out[n] = total.
template <class In, class Out>
__global__ void __launch_bounds__(kT) single_tile_scan_kernel(In in, int64_t n, Out *out, unsigned long long *slots) {
    const Out tot = scan_tile_striped<In, Out>(in, n, 0, Out(0), out, slots);
    if (threadIdx.x == 0) out[n] = tot;
}

template <class In, class Out>
int scan_impl(In in, Out *out, int64_t n, cudaStream_t s, unsigned long long *slots = nullptr) {
    if (n <= 0) {
        TC_CUDA(cudaMemsetAsync(out, 0, sizeof(Out), s));
        return TC_OK;
    }
    const int64_t tiles = (n + kTile - 1) / kTile;
    if (tiles == 1) {
        single_tile_scan_kernel<In, Out><<<1, kT, 0, s>>>(in, n, out, slots);
        TC_CUDA(cudaGetLastError());
        return TC_OK;
    }
    DBuf<Out> sums;
    TC_TRY(sums.alloc((size_t)tiles + 1, s));
    tile_reduce_kernel<In, Out><<<(unsigned)tiles, kT, 0, s>>>(in, n, sums.p);
    TC_CUDA(cudaGetLastError());
    // exclusive scan of the tile sums in place (recursion ends at one tile)
    TC_TRY((scan_impl<const Out *, Out>(sums.p, sums.p, tiles, s)));
    tile_scan_kernel<In, Out><<<(unsigned)tiles, kT, 0, s>>>(in, n, sums.p, out, slots);
    TC_CUDA(cudaGetLastError());
    return TC_OK;
}

// ---- radix sort ---------------------------------------------------------------------
constexpr int kRadixBits = 8;
constexpr int kBins = 1 << kRadixBits;
constexpr int kWarps = kT / 32;
constexpr int kSeg = kTile / kWarps;  // keys per warp segment (512)

__global__ void __launch_bounds__(kT) radix_hist_kernel(const uint64_t *keys, int64_t n, int shift, int n_tiles,
                                                       int32_t *hist) {
    __shared__ int32_t h[kBins];
    h[threadIdx.x] = 0;
    __syncthreads();
    const int64_t base = (int64_t)blockIdx.x * kTile;
#pragma unroll 4
    for (int k = 0; k < kItems; ++k) {
        const int64_t i = base + (int64_t)k * kT + threadIdx.x;
        if (i < n) atomicAdd(&h[(keys[i] >> shift) & (kBins - 1)], 1);
    }
    __syncthreads();
    hist[(int64_t)threadIdx.x * n_tiles + blockIdx.x] = h[threadIdx.x];  // digit-major
}

__global__ void __launch_bounds__(kT) radix_scatter_kernel(const uint64_t *keys, uint64_t *out, int64_t n, int shift,
                                                          int n_tiles, const int32_t *offs) {
    __shared__ int32_t wh[kWarps][kBins];  // per-warp digit counts -> warp offsets
    __shared__ int32_t tile_start[kBins];   // digit start inside the tile
    __shared__ int32_t glob[kBins];         // digit start in the output
    __shared__ uint64_t stage[kTile];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < kWarps * kBins; i += kT) (&wh[0][0])[i] = 0;
    glob[threadIdx.x] = offs[(int64_t)threadIdx.x * n_tiles + blockIdx.x];
    __syncthreads();
    const int64_t seg_base = (int64_t)blockIdx.x * kTile + (int64_t)w * kSeg;
    uint64_t key[kItems];
    int rank[kItems];
    const unsigned lt = (1u << lane) - 1u;
#pragma unroll
    for (int r = 0; r < kItems; ++r) {
        const int64_t i = seg_base + r * 32 + lane;
        const bool valid = i < n;
        key[r] = valid ? keys[i] : ~0ull;
        const int d = valid ? (int)((key[r] >> shift) & (kBins - 1)) : kBins;  // kBins: padding
        const unsigned peers = __match_any_sync(kFull, d);
        int prior = 0;
        if (valid) prior = wh[w][d];
        __syncwarp();
        rank[r] = prior + __popc(peers & lt);
        if (valid && (peers & lt) == 0) wh[w][d] = prior + __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    // exclusive scan over warps for each digit, then over digits for the tile
    {
        const int d = threadIdx.x;
        int run = 0;
#pragma unroll
        for (int ww = 0; ww < kWarps; ++ww) {
            const int c = wh[ww][d];
            wh[ww][d] = run;
            run += c;
        }
        int tot;
        const int start = block_excl_scan<int>(run, &tot);
        tile_start[d] = start;
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kItems; ++r) {
        const int64_t i = seg_base + r * 32 + lane;
        if (i < n) {
            const int d = (int)((key[r] >> shift) & (kBins - 1));
            stage[tile_start[d] + wh[w][d] + rank[r]] = key[r];
        }
    }
    __syncthreads();
    const int64_t rem = n - (int64_t)blockIdx.x * kTile;
    const int tile_n = rem < kTile ? (int)rem : kTile;
    for (int i = threadIdx.x; i < tile_n; i += kT) {
        const uint64_t k = stage[i];
        const int d = (int)((k >> shift) & (kBins - 1));
        out[glob[d] + (i - tile_start[d])] = k;
    }
}

// Same scan with the tile sums of every recursion level in tmp (tmp_cap values).
template <class In, class Out>
int scan_tmp_impl(In in, Out *out, int64_t n, Out *tmp, int64_t tmp_cap, cudaStream_t s,
                  unsigned long long *slots = nullptr) {
    if (n <= 0) {
        TC_CUDA(cudaMemsetAsync(out, 0, sizeof(Out), s));
        return TC_OK;
    }
    const int64_t tiles = (n + kTile - 1) / kTile;
    if (tiles == 1) {
        single_tile_scan_kernel<In, Out><<<1, kT, 0, s>>>(in, n, out, slots);
        TC_CUDA(cudaGetLastError());
        return TC_OK;
    }
    if (tiles + 1 > tmp_cap) return set_error(TC_E_RANGE, "scan temp of %lld values is too small", (long long)tmp_cap);
    tile_reduce_kernel<In, Out><<<(unsigned)tiles, kT, 0, s>>>(in, n, tmp);
    TC_CUDA(cudaGetLastError());
    TC_TRY((scan_tmp_impl<const Out *, Out>(tmp, tmp, tiles, tmp + tiles + 1, tmp_cap - (tiles + 1), s)));
    tile_scan_kernel<In, Out><<<(unsigned)tiles, kT, 0, s>>>(in, n, tmp, out, slots);
    TC_CUDA(cudaGetLastError());
    return TC_OK;
}

}  // namespace

int scan_exclusive_i32_tmp(const int32_t *in, int32_t *out, int64_t n, int32_t *tmp, int64_t tmp_cap,
                           cudaStream_t s) {
    return scan_tmp_impl<const int32_t *, int32_t>(in, out, n, tmp, tmp_cap, s);
}

int scan_exclusive_i32(const int32_t *in, int32_t *out, int64_t n, cudaStream_t s) {
    return scan_impl<const int32_t *, int32_t>(in, out, n, s);
}
int scan_exclusive_i64(const int64_t *in, int64_t *out, int64_t n, cudaStream_t s) {
    return scan_impl<const int64_t *, int64_t>(in, out, n, s);
}
int scan_flags_u8(const uint8_t *flags, int32_t *out, int64_t n, cudaStream_t s) {
    return scan_impl<const uint8_t *, int32_t>(flags, out, n, s);
}
int scan_in_slots(unsigned long long *in_work, int32_t *in_off, int64_t n, int32_t *tmp, int64_t tmp_cap,
                  cudaStream_t s) {
    const HighHalf in{in_work};
    if (tmp) return scan_tmp_impl<HighHalf, int32_t>(in, in_off, n, tmp, tmp_cap, s, in_work);
    return scan_impl<HighHalf, int32_t>(in, in_off, n, s, in_work);
}

int radix_sort_u64(uint64_t **keys, uint64_t **tmp, int64_t n, int bits, cudaStream_t s) {
    if (n <= 1 || bits <= 0) return TC_OK;
    const int64_t tiles64 = (n + kTile - 1) / kTile;
    if (tiles64 * kBins >= INT32_MAX) return set_error(TC_E_RANGE, "radix sort of %lld keys is too large", (long long)n);
    const int n_tiles = (int)tiles64;
    DBuf<int32_t> hist;
    TC_TRY(hist.alloc((size_t)n_tiles * kBins + 1, s));
    for (int shift = 0; shift < bits; shift += kRadixBits) {
        radix_hist_kernel<<<n_tiles, kT, 0, s>>>(*keys, n, shift, n_tiles, hist.p);
        TC_CUDA(cudaGetLastError());
        TC_TRY(scan_exclusive_i32(hist.p, hist.p, (int64_t)n_tiles * kBins, s));
        radix_scatter_kernel<<<n_tiles, kT, 0, s>>>(*keys, *tmp, n, shift, n_tiles, hist.p);
        TC_CUDA(cudaGetLastError());
        std::swap(*keys, *tmp);
    }
    return TC_OK;
}

}  // namespace tc
