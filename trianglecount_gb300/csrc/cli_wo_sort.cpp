// wo_sort_tc_256 <parts_output.csr> <k> [--batch] -- drop-in for the
// reference's partitioned counter (src/WithPartition/without_sorting_tc.cu:220-473):
// reads the halo-part file written by round_clean_sg, counts each part's
// triangles with roots = the part's own vertices (local ids [0, t_ver)) and
// prints the reference's lines (:256, :450, :466-470).  By default every part
// is its own launch with a host sync, as in the reference; --batch (or
// TC_BATCH=1) counts all parts in one persistent launch (a CUDA graph replay).
#include <string>
#include <vector>

#include "cli_common.h"

int main(int argc, char **argv) {
    if (argc < 3) {
        fprintf(stderr, "usage: %s <parts_output.csr> <k> [--batch]\n", argv[0]);
        return 1;
    }
    const uint64_t k = strtoull(argv[2], nullptr, 10);  // atoi(argv[2]) in the reference (:228-229)
    bool batch = getenv("TC_BATCH") && strcmp(getenv("TC_BATCH"), "1") == 0;
    for (int i = 3; i < argc; ++i)
        if (strcmp(argv[i], "--batch") == 0) batch = true;
    if (!cli::file_exists(argv[1])) {  // :234-238
        printf("\nFile Not Opened.........");
        return 0;
    }
    cli::Ints f;
    CLI_CHECK(tc_text_read_u64(argv[1], &f.v, &f.n));
    uint64_t V = 0, E = 0;
    if (!f.next(&V) || !f.next(&E)) {
        fprintf(stderr, "%s: truncated header\n", argv[1]);
        return 1;
    }
    tc_ctx *ctx = nullptr;
    CLI_CHECK(tc_ctx_create(0, &ctx));
    uint64_t total_tri = 0;
    float kernel_s = 0;
    double total_s = 0;
    std::vector<tc_graph *> parts;
    for (uint64_t i = 0; i < k; ++i) {
        const uint64_t *h, *rp, *col;
        if (!f.take(4, &h)) {
            fprintf(stderr, "%s: part %llu header missing (file has fewer than %llu parts)\n", argv[1],
                    (unsigned long long)i, (unsigned long long)k);
            return 1;
        }
        const int64_t rps = (int64_t)h[1], cis = (int64_t)h[2], t_ver = (int64_t)h[3];
        if (!batch) printf("\nPart %llu executing :", (unsigned long long)i);
        if (rps < 1 || !f.take(rps, &rp) || !f.take(cis, &col)) {
            fprintf(stderr, "%s: part %llu is truncated\n", argv[1], (unsigned long long)i);
            return 1;
        }
        const double t0 = cli::now_s();
        tc_graph *g = nullptr;
        CLI_CHECK(tc_graph_upload_u64(ctx, rp, col, rps - 1, cis, t_ver, &g));
        if (batch) {
            parts.push_back(g);
            total_s += cli::now_s() - t0;
            continue;
        }
        uint64_t tri = 0;
        tc_count_stats st;
        CLI_CHECK(tc_count(ctx, g, &tri, &st));
        total_s += cli::now_s() - t0;
        kernel_s += st.count_ms / 1000.0f + st.finalize_ms / 1000.0f;
        printf("\t%llu\n", (unsigned long long)tri);
        total_tri += tri;
        tc_graph_destroy(g);
    }
    if (batch && !parts.empty()) {
        tc_batch *b = nullptr;
        CLI_CHECK(tc_batch_create(ctx, parts.data(), (int)parts.size(), &b));
        std::vector<uint64_t> outs(parts.size());
        const double t0 = cli::now_s();
        CLI_CHECK(tc_batch_run(b, outs.data()));
        const double dt = cli::now_s() - t0;
        kernel_s += (float)dt;
        total_s += dt;
        for (size_t i = 0; i < parts.size(); ++i) {
            printf("\nPart %llu executing :", (unsigned long long)i);
            printf("\t%llu\n", (unsigned long long)outs[i]);
            total_tri += outs[i];
        }
        tc_batch_destroy(b);
        for (tc_graph *g : parts) tc_graph_destroy(g);
    }
    printf("\nTotal Vertex : %llu ", (unsigned long long)V);
    printf("\tTotal Edges : %llu ", (unsigned long long)(E / 2));
    printf("\tTotal Triangle : %llu ", (unsigned long long)total_tri);
    printf("\tTotal Kernel Time : %.4f sec", kernel_s);
    printf("\tTotal Time : %f \n\n", (float)total_s);
    tc_ctx_destroy(ctx);
    return 0;
}
