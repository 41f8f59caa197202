// round_clean_sg <k> <name_part.csr> <node_parts> -- drop-in for the
// reference's halo-subgraph extractor
// (preprocess_GPU/Halo_cleanned_preprocess/round_clean_subgraph.cu:904-989):
// reads the undirected CSR + degree file and the vertex -> part file, builds
// each part's halo subgraph on the GPU (part vertices, then their 1-hop halo,
// oriented edges among them, halo vertices of zero in-degree pruned until
// none is left) and writes <node_parts>_output.csr in the reference's layout
// (:371, :850-865).
#include <string>
#include <vector>

#include "cli_common.h"

int main(int argc, char **argv) {
    if (argc != 4) {
        fprintf(stderr, "Usage: %s <nopart> <name_part.csr> <node_parts>\n", argv[0]);
        return 1;
    }
    const int k = atoi(argv[1]);
    if (k < 1) {
        fprintf(stderr, "number of parts must be >= 1\n");
        return 1;
    }
    for (int i = 2; i < 4; ++i)
        if (!cli::file_exists(argv[i])) {
            fprintf(stderr, "Error opening file: %s\n", argv[i]);
            return 1;
        }
    const double t0 = cli::now_s();
    cli::Ints f;
    CLI_CHECK(tc_text_read_u64(argv[2], &f.v, &f.n));
    const uint64_t *h, *rp, *col, *deg;
    if (!f.take(6, &h)) {
        fprintf(stderr, "%s: truncated header\n", argv[2]);
        return 1;
    }
    const int64_t N = (int64_t)h[0], E = (int64_t)h[1], rps = (int64_t)h[3], cis = (int64_t)h[4];
    if (rps != N + 1 || !f.take(rps, &rp) || !f.take(cis, &col) || !f.take(N, &deg)) {
        fprintf(stderr, "%s: malformed or truncated _part.csr file\n", argv[2]);
        return 1;
    }
    cli::Ints pf;
    CLI_CHECK(tc_text_read_u64(argv[3], &pf.v, &pf.n));
    const uint64_t *pv;
    if (!pf.take(N, &pv)) {
        fprintf(stderr, "%s: needs %lld part ids\n", argv[3], (long long)N);
        return 1;
    }
    std::vector<int64_t> rp64(rp, rp + rps), col64(col, col + cis), deg64(deg, deg + N);
    std::vector<int32_t> part((size_t)N);
    for (int64_t v = 0; v < N; ++v) part[(size_t)v] = pv[v] > (uint64_t)INT32_MAX ? INT32_MAX : (int32_t)pv[v];
    tc_ctx *ctx = nullptr;
    CLI_CHECK(tc_ctx_create(0, &ctx));
    tc_ugraph *ug = nullptr;
    CLI_CHECK(tc_ugraph_upload_i64(ctx, rp64.data(), col64.data(), deg64.data(), N, cis, &ug));
    std::vector<tc_graph *> parts((size_t)k, nullptr);
    const double tk = cli::now_s();
    CLI_CHECK(tc_halo_extract(ctx, ug, part.data(), k, TC_TIE_REFERENCE, parts.data()));
    const double kernel_s = cli::now_s() - tk;
    const std::string out = std::string(argv[3]) + "_output.csr";
    const int64_t hdr[2] = {N, E};
    CLI_CHECK(tc_text_write_line(out.c_str(), hdr, 2, 8, 'w', 0));
    for (int p = 0; p < k; ++p) {
        int64_t n_rows = 0, nnz = 0, t_ver = 0;
        CLI_CHECK(tc_graph_info(parts[(size_t)p], &n_rows, &nnz, &t_ver));
        std::vector<int32_t> lrp((size_t)n_rows + 1), lcol((size_t)nnz);
        CLI_CHECK(tc_graph_download_i32(ctx, parts[(size_t)p], lrp.data(), lcol.data()));
        const int64_t ph[4] = {n_rows, n_rows + 1, nnz, t_ver};
        CLI_CHECK(tc_text_write_line(out.c_str(), ph, 4, 8, 'a', 0));
        CLI_CHECK(tc_text_write_line(out.c_str(), lrp.data(), n_rows + 1, 4, 'a', 1));
        CLI_CHECK(tc_text_write_line(out.c_str(), lcol.data(), nnz, 4, 'a', 1));
        printf("part %d: %lld vertices (%lld own, %lld halo), %lld oriented edges\n", p, (long long)n_rows,
               (long long)t_ver, (long long)(n_rows - t_ver), (long long)nnz);
        tc_graph_destroy(parts[(size_t)p]);
    }
    tc_ugraph_destroy(ug);
    tc_ctx_destroy(ctx);
    printf("Total EXE Time: %f seconds.\n", kernel_s);
    printf("Total Time measured:%f seconds.\n", cli::now_s() - t0);
    return 0;
}
