// ref_launch.cu -- TEST INFRASTRUCTURE ONLY: launches the reference's own
// TC_128 kernel (Find_Triangle of src/WithoutPartition/ShareKernelTCV62_update_v1.cu:43-191),
// compiled from the reference sources into oracle/_ref/tc128_sm103a.cubin by
// oracle/build_ref.sh, with the reference's launch shape (one 128-thread block
// per vertex, :264).  Used by the tests to cross-check per-root counts and by
// bench.py to time the reference kernel on the same GPU.  Host code only.
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

extern "C" {

// Returns 0 on success; per_root[V] receives g_sum, *ms the kernel time of
// the last of `runs` launches (events around the launch, as :263-265).
int ref_tc128_run(const char *cubin, const int32_t *rp, const int32_t *col, int32_t V, int32_t nnz, int runs,
                  uint64_t *per_root, float *ms, char *err, int err_len) {
    cudaLibrary_t lib = nullptr;
    cudaKernel_t k = nullptr;
    int32_t *d_rp = nullptr, *d_col = nullptr;
    unsigned long long *d_sum = nullptr;
    void *d_flush = nullptr;  // written before each launch so the kernel starts with a cold L2
    const size_t flush_bytes = (size_t)512 << 20;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t e = cudaLibraryLoadFromFile(&lib, cubin, nullptr, nullptr, 0, nullptr, nullptr, 0);
    if (e == cudaSuccess) e = cudaLibraryGetKernel(&k, lib, "_Z13Find_TrianglePiS_iiPy");
    if (e == cudaSuccess) e = cudaMalloc(&d_rp, sizeof(int32_t) * ((size_t)V + 1));
    if (e == cudaSuccess) e = cudaMalloc(&d_col, sizeof(int32_t) * (size_t)(nnz ? nnz : 1));
    if (e == cudaSuccess) e = cudaMalloc(&d_sum, sizeof(unsigned long long) * (size_t)(V ? V : 1));
    if (e == cudaSuccess) e = cudaMalloc(&d_flush, flush_bytes);
    if (e == cudaSuccess) e = cudaMemcpy(d_rp, rp, sizeof(int32_t) * ((size_t)V + 1), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && nnz) e = cudaMemcpy(d_col, col, sizeof(int32_t) * (size_t)nnz, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    int edges = 0;  // the kernel's unused `edge` argument
    for (int r = 0; r < runs && e == cudaSuccess && V > 0; ++r) {
        void *args[] = {&d_col, &d_rp, &V, &edges, &d_sum};
        e = cudaMemset(d_flush, r & 0xff, flush_bytes);
        if (e == cudaSuccess) e = cudaEventRecord(e0);
        if (e == cudaSuccess) e = cudaLaunchKernel((const void *)k, dim3((unsigned)V), dim3(128), args, 0, nullptr);
        if (e == cudaSuccess) e = cudaEventRecord(e1);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        if (e == cudaSuccess) e = cudaEventElapsedTime(ms, e0, e1);
    }
    if (e == cudaSuccess && V > 0)
        e = cudaMemcpy(per_root, d_sum, sizeof(unsigned long long) * (size_t)V, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess && err) snprintf(err, (size_t)err_len, "%s", cudaGetErrorString(e));
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(d_rp);
    cudaFree(d_col);
    cudaFree(d_sum);
    cudaFree(d_flush);
    if (lib) cudaLibraryUnload(lib);
    return e == cudaSuccess ? 0 : (int)e;
}

// The reference's design-space variants of Find_Triangle (shareMemSize.cu,
// With_Atomic_op.cu, Without_ShareMemory_TC.cu in src/WithoutPartition/),
// launched as their drivers do: one block of `threads` per vertex.  idx64: the
// kernel takes u64 col / row_ptr and no vertex / edge arguments
// (Without_ShareMemory_TC.cu:53); total_only: it adds every hit to g_sum[0]
// (zeroed before each launch) instead of writing a per-vertex sum.  *total
// gets the count of the last run, *ms its kernel time.
int ref_variant_run(const char *cubin, const char *symbol, int threads, int idx64, int total_only,
                    const int32_t *rp, const int32_t *col, int32_t V, int32_t nnz, int runs, uint64_t *total,
                    float *ms, char *err, int err_len) {
    cudaLibrary_t lib = nullptr;
    cudaKernel_t k = nullptr;
    void *d_rp = nullptr, *d_col = nullptr;
    unsigned long long *d_sum = nullptr;
    void *d_flush = nullptr;
    const size_t flush_bytes = (size_t)512 << 20;
    const size_t isz = idx64 ? 8 : 4;
    const size_t n_sum = total_only ? 1 : (size_t)(V ? V : 1);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    uint64_t *h64 = nullptr;
    *total = 0;
    cudaError_t e = cudaLibraryLoadFromFile(&lib, cubin, nullptr, nullptr, 0, nullptr, nullptr, 0);
    if (e == cudaSuccess) e = cudaLibraryGetKernel(&k, lib, symbol);
    if (e == cudaSuccess) e = cudaMalloc(&d_rp, isz * ((size_t)V + 1));
    if (e == cudaSuccess) e = cudaMalloc(&d_col, isz * (size_t)(nnz ? nnz : 1));
    if (e == cudaSuccess) e = cudaMalloc(&d_sum, sizeof(unsigned long long) * n_sum);
    if (e == cudaSuccess) e = cudaMalloc(&d_flush, flush_bytes);
    if (e == cudaSuccess && idx64) {
        const size_t n = (size_t)V + 1 > (size_t)nnz ? (size_t)V + 1 : (size_t)nnz;
        h64 = (uint64_t *)malloc(8 * (n ? n : 1));
        if (!h64) e = cudaErrorMemoryAllocation;
        for (int32_t i = 0; e == cudaSuccess && i <= V; ++i) h64[i] = (uint64_t)rp[i];
        if (e == cudaSuccess) e = cudaMemcpy(d_rp, h64, 8 * ((size_t)V + 1), cudaMemcpyHostToDevice);
        for (int32_t i = 0; e == cudaSuccess && i < nnz; ++i) h64[i] = (uint64_t)col[i];
        if (e == cudaSuccess && nnz) e = cudaMemcpy(d_col, h64, 8 * (size_t)nnz, cudaMemcpyHostToDevice);
    } else if (e == cudaSuccess) {
        e = cudaMemcpy(d_rp, rp, 4 * ((size_t)V + 1), cudaMemcpyHostToDevice);
        if (e == cudaSuccess && nnz) e = cudaMemcpy(d_col, col, 4 * (size_t)nnz, cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    int edges = 0;  // the int32 kernels' unused `edge` argument
    for (int r = 0; r < runs && e == cudaSuccess && V > 0; ++r) {
        void *args32[] = {&d_col, &d_rp, &V, &edges, &d_sum};
        void *args64[] = {&d_col, &d_rp, &d_sum};
        e = cudaMemset(d_sum, 0, sizeof(unsigned long long) * n_sum);
        if (e == cudaSuccess) e = cudaMemset(d_flush, r & 0xff, flush_bytes);
        if (e == cudaSuccess) e = cudaEventRecord(e0);
        if (e == cudaSuccess)
            e = cudaLaunchKernel((const void *)k, dim3((unsigned)V), dim3((unsigned)threads), idx64 ? args64 : args32,
                                 0, nullptr);
        if (e == cudaSuccess) e = cudaEventRecord(e1);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        if (e == cudaSuccess) e = cudaEventElapsedTime(ms, e0, e1);
    }
    if (e == cudaSuccess && V > 0) {
        unsigned long long *h = (unsigned long long *)malloc(sizeof(unsigned long long) * n_sum);
        if (!h) e = cudaErrorMemoryAllocation;
        if (e == cudaSuccess) e = cudaMemcpy(h, d_sum, sizeof(unsigned long long) * n_sum, cudaMemcpyDeviceToHost);
        for (size_t i = 0; e == cudaSuccess && i < n_sum; ++i) *total += h[i];
        free(h);
    }
    if (e != cudaSuccess && err) snprintf(err, (size_t)err_len, "%s", cudaGetErrorString(e));
    free(h64);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(d_rp);
    cudaFree(d_col);
    cudaFree(d_sum);
    cudaFree(d_flush);
    if (lib) cudaLibraryUnload(lib);
    return e == cudaSuccess ? 0 : (int)e;
}

}  // extern "C"
