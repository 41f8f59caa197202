// TC_128 <file.csr> -- drop-in for the reference's TC_128
// (src/WithoutPartition/ShareKernelTCV62_update_v1.cu:192-310): reads the
// oriented int32 .csr text file, counts its triangles three times on the GPU
// and prints the reference's lines (:290, :296).  "Search" is the device time
// of the counting kernels, "Sum_result" the result read-back (the reference's
// separate CUB reduction is fused into the count here).
#include <vector>

#include "cli_common.h"

int main(int argc, char **argv) {
    if (argc < 2) {
        fprintf(stderr, "usage: %s <file.csr>\n", argv[0]);
        return 1;
    }
    if (!cli::file_exists(argv[1])) {  // :200-203
        printf("file not opened\n");
        return 0;
    }
    cli::Ints f;
    CLI_CHECK(tc_text_read_u64(argv[1], &f.v, &f.n));
    const uint64_t *h;
    if (!f.take(4, &h)) {
        fprintf(stderr, "%s: truncated header\n", argv[1]);
        return 1;
    }
    const int64_t V = (int64_t)h[0], rps = (int64_t)h[2], cis = (int64_t)h[3];
    const uint64_t *rp64, *col64;
    if (rps < 1 || !f.take(rps, &rp64) || !f.take(cis, &col64)) {
        fprintf(stderr, "%s: truncated row_ptr / col_idx (header says %lld and %lld values)\n", argv[1],
                (long long)rps, (long long)cis);
        return 1;
    }
    // the reference reads every value with "%d" (:207-230)
    std::vector<int32_t> rp((size_t)rps), col((size_t)cis);
    for (int64_t i = 0; i < rps; ++i) {
        if (rp64[i] > (uint64_t)INT32_MAX) {
            fprintf(stderr, "%s: row_ptr value %llu does not fit int32\n", argv[1], (unsigned long long)rp64[i]);
            return 1;
        }
        rp[(size_t)i] = (int32_t)rp64[i];
    }
    for (int64_t i = 0; i < cis; ++i) {
        if (col64[i] > (uint64_t)INT32_MAX) {
            fprintf(stderr, "%s: col_idx value %llu does not fit int32\n", argv[1], (unsigned long long)col64[i]);
            return 1;
        }
        col[(size_t)i] = (int32_t)col64[i];
    }
    tc_ctx *ctx = nullptr;
    CLI_CHECK(tc_ctx_create(0, &ctx));
    tc_graph *g = nullptr;
    CLI_CHECK(tc_graph_upload_i32(ctx, rp.data(), col.data(), rps - 1, cis, rps - 1, &g));
    float total = 0;
    for (int run = 0; run < 3; ++run) {
        uint64_t tri = 0;
        tc_count_stats st;
        CLI_CHECK(tc_count(ctx, g, &tri, &st));
        const float t = st.count_ms / 1000.0f + st.finalize_ms / 1000.0f;
        printf("\nSearch : %.6f sec Vertex : %d Edge : %d Triangle : %llu  Sum_result : %.6f Sec, total_time : %.6f "
               "Sec\n",
               st.count_ms / 1000.0f, (int)V, (int)cis, (unsigned long long)tri, st.finalize_ms / 1000.0f, t);
        total += t;
    }
    printf("\nTotal avg of 3 RUNS : %.6f Sec\n", total / 3);
    tc_graph_destroy(g);
    tc_ctx_destroy(ctx);
    return 0;
}
