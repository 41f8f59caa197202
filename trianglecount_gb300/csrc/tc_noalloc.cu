// tc_noalloc.cu -- triangle count that allocates no memory.
//
// Some callers cannot allocate GPU memory on their own: an application that
// owns the device heap through its own allocator and forbids libraries from
// calling cudaMalloc, a real-time loop where an allocation (and the
// synchronisation it may imply) is not acceptable, or a sandboxed plugin whose
// host denies allocations.  tc_count_noalloc_i32 serves them: the caller hands
// in device pointers to the oriented CSR and to the 8-byte result, and every
// scratch array the count needs lives in one file-scope device array of fixed
// size (kScratchBytes below, about 22 MB), which each GPU that loads libtc
// keeps until the process exits.
//
// Limits: n_rows <= kMaxRows (262,144) and nnz <= kMaxNnz (2,097,152); larger
// graphs are rejected with TC_E_RANGE.  All calls share the one array, so two
// calls whose work overlaps on the GPU (different streams, or different host
// threads) race and give wrong counts; order them on one stream.  The first
// call on a device looks up the array's device address and the kernel
// configuration for that device (cudaGetSymbolAddress, occupancy query); make
// that first call before any stream capture.
//
// Every device-side step of a call is a kernel launch or a device-to-device
// memset in stream order: the graph descriptor travels as a kernel parameter
// (no copy from host memory), and the result is written by a one-thread
// kernel, which stores all ones (UINT64_MAX) in place of the count if the
// classifier's heavy-unit list overflowed (it cannot for a CSR within the
// limits: each row gives at most one heavy entry and the list has a slot per
// row).
#include <algorithm>
#include <cstring>
#include <mutex>

#include "tc_internal.h"

namespace tc {
namespace {

constexpr int64_t kMaxRows = 1 << 18;
constexpr int64_t kMaxNnz = 1 << 21;
constexpr int64_t kScanTmp = 4096;  // tile sums of the in-edge scan (needs 66 for kMaxRows)

constexpr size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Byte offsets of the scratch sections (each 256-byte aligned).
constexpr size_t kOffWork = 0;  // CountWork + 8-byte result
constexpr size_t kOffDesc = align256(kOffWork + sizeof(CountWork) + 8);
constexpr size_t kOffTasks = align256(kOffDesc + sizeof(GraphDesc));
constexpr size_t kOffHeavy = align256(kOffTasks + sizeof(uint32_t) * (kMaxRows + 1));
constexpr size_t kOffInCnt = align256(kOffHeavy + sizeof(HeavyEntry) * (kMaxRows + 1));
constexpr size_t kOffInOff = align256(kOffInCnt + sizeof(int32_t) * (kMaxRows + 1));
constexpr size_t kOffInWork = align256(kOffInOff + sizeof(int32_t) * (kMaxRows + 2));
constexpr size_t kOffOutWork = align256(kOffInWork + sizeof(unsigned long long) * (kMaxRows + 1));
constexpr size_t kOffInList = align256(kOffOutWork + sizeof(unsigned long long) * (kMaxRows + 1));
constexpr size_t kOffMid = align256(kOffInList + sizeof(int32_t) * kMaxNnz);
constexpr size_t kOffScan = align256(kOffMid + kMaxNnz);
constexpr size_t kScratchBytes = align256(kOffScan + sizeof(int32_t) * kScanTmp);

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

struct DeviceSetup {
    bool ready = false;
    unsigned char *scratch = nullptr;  // device address of g_noalloc_scratch
    Tuned tuned{};
};

// The descriptor of one call, written in stream order from a kernel
// parameter (a host-to-device copy from the caller's stack would stage
// through pageable memory).
__global__ void noalloc_set_desc_kernel(GraphDesc *dst, GraphDesc d) { *dst = d; }

// d_out = the count, or all ones when the heavy-unit list overflowed.
__global__ void noalloc_finish_kernel(const CountWork *work, const unsigned long long *result,
                                      unsigned long long *d_out) {
    *d_out = work->error ? ~0ull : *result;
}

std::mutex g_setup_mu;
DeviceSetup g_setup[64];

// Once per device, with that device current: the array's device address and
// the default kernel configuration.  The array's name is only a host-side
// stand-in in host code, so kernels are given the looked-up address.
int setup_device(int dev, DeviceSetup **out) {
    if (dev < 0 || dev >= 64) return set_error(TC_E_NO_DEVICE, "device %d out of range", dev);
    std::lock_guard<std::mutex> lock(g_setup_mu);
    DeviceSetup &d = g_setup[dev];
    if (!d.ready) {
        void *p = nullptr;
        TC_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        tc_tuning t{};
        t.warp_max_deg = 256;
        t.light_max_work = 8192;
        t.unit_work = 1048576;
        t.long_list = 32;
        t.probe_kicks = 32;
        t.heavy_bitmap = 0;  // the allocation-free variant keeps the fixed heavy path
        t.blocks_per_sm = 0;
        t.hash_pairs = 0;
        t.flat_max_deg = 0;  // the flat count is not used here
        t.intersect = 0;
        TC_TRY(resolve_tuning(t, device_sm_count(dev), &d.tuned));
        d.scratch = (unsigned char *)p;
        d.ready = true;
    }
    *out = &d;
    return TC_OK;
}

}  // namespace
}  // namespace tc

using namespace tc;

extern "C" int tc_count_noalloc_i32(const int32_t *d_row_ptr, const int32_t *d_col, int64_t n_rows, int64_t nnz,
                                    int64_t n_roots, uint64_t *d_out, void *stream) {
    if (!d_row_ptr || (nnz > 0 && !d_col) || !d_out) return set_error(TC_E_INVALID, "null device pointer");
    if (n_rows < 0 || nnz < 0 || n_roots < 0 || n_roots > n_rows)
        return set_error(TC_E_INVALID, "bad sizes: n_rows=%lld nnz=%lld n_roots=%lld", (long long)n_rows,
                         (long long)nnz, (long long)n_roots);
    if (n_rows > kMaxRows || nnz > kMaxNnz)
        return set_error(TC_E_RANGE,
                         "tc_count_noalloc_i32 handles at most %lld rows and %lld oriented edges (got %lld, %lld); "
                         "use tc_count for larger graphs",
                         (long long)kMaxRows, (long long)kMaxNnz, (long long)n_rows, (long long)nnz);
    int dev = 0;
    TC_CUDA(cudaGetDevice(&dev));
    DeviceSetup *ds = nullptr;
    TC_TRY(setup_device(dev, &ds));
    cudaStream_t s = (cudaStream_t)stream;
    unsigned char *base = ds->scratch;
    CountWork *work = (CountWork *)(base + kOffWork);
    unsigned long long *result = (unsigned long long *)(work + 1);
    GraphDesc *desc = (GraphDesc *)(base + kOffDesc);
    CountScratch sc;
    sc.heavy = (HeavyEntry *)(base + kOffHeavy);
    sc.heavy_cap = std::min(n_rows, nnz) + 1;
    sc.light_list = (uint32_t *)(base + kOffTasks);
    sc.in_cnt = (int32_t *)(base + kOffInCnt);
    sc.in_off = (int32_t *)(base + kOffInOff);
    sc.in_work = (unsigned long long *)(base + kOffInWork);
    sc.out_work = (unsigned long long *)(base + kOffOutWork);
    sc.in_list = (int32_t *)(base + kOffInList);
    sc.mid = (uint8_t *)(base + kOffMid);
    GraphDesc d;
    memset(&d, 0, sizeof d);
    d.rp = d_row_ptr;
    d.col = d_col;
    d.n_rows = n_rows;
    d.n_roots = n_roots;
    noalloc_set_desc_kernel<<<1, 1, 0, s>>>(desc, d);
    TC_CUDA(cudaGetLastError());
    TC_TRY(launch_count_noalloc(desc, (n_rows + 31) / 32, n_rows + 1, sc, (int32_t *)(base + kOffScan), kScanTmp,
                                work, result, ds->tuned, s));
    noalloc_finish_kernel<<<1, 1, 0, s>>>(work, result, (unsigned long long *)d_out);
    TC_CUDA(cudaGetLastError());
    return TC_OK;
}
