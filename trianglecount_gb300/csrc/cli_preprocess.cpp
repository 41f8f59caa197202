// tc_preprocess <edge-file> [--out-dir D] [--parts 2,4,8] [--seed S] [--tie reference|id_asc] [--tcsr]
//
// Replaces the reference's Python preprocessing on the GPU:
//   Med_dataset/without_part_preprocess.py (-> <name>_output.csr, the oriented
//     CSR read by TC_128) and
//   preprocess_GPU/generate_clean_undir_dataset/Halo_creation_preprocess.py
//     (-> <name>_part.csr, the undirected CSR + degree read by round_clean_sg,
//     and per k the node-parts files <name>_part.csr_node_parts_random_<k>
//     (seeded here where the reference's np.random.randint is unseeded),
//     _contig_<k>, and _lp_<k>: balanced label propagation on the device in
//     place of the reference's _metis_<k> (dgl.metis_partition_assignment)).
// Clean-up (self-loops, symmetrise, dedupe, isolated vertices) and orientation
// run on the device.  --tcsr also writes <name>.tcsr (binary oriented CSR).
#include <string>
#include <vector>

#include "cli_common.h"

static std::string stem(const char *path) {
    std::string s(path);
    const size_t slash = s.find_last_of('/');
    if (slash != std::string::npos) s = s.substr(slash + 1);
    const size_t dot = s.find_last_of('.');
    if (dot != std::string::npos && dot > 0) s = s.substr(0, dot);
    return s;
}

int main(int argc, char **argv) {
    if (argc < 2) {
        fprintf(stderr,
                "usage: %s <edge-file (.tsv/.txt/.mtx/.mmio)> [--out-dir D] [--parts 2,4,8] [--seed S] "
                "[--tie reference|id_asc] [--tcsr]\n",
                argv[0]);
        return 1;
    }
    std::string out_dir = ".";
    std::vector<int> ks = {2, 4, 8};
    uint64_t seed = 0x5EED9A27ull;
    int tie = TC_TIE_REFERENCE;
    bool tcsr = false;
    for (int i = 2; i < argc; ++i) {
        if (!strcmp(argv[i], "--out-dir") && i + 1 < argc) out_dir = argv[++i];
        else if (!strcmp(argv[i], "--seed") && i + 1 < argc) seed = strtoull(argv[++i], nullptr, 0);
        else if (!strcmp(argv[i], "--tcsr")) tcsr = true;
        else if (!strcmp(argv[i], "--tie") && i + 1 < argc) tie = !strcmp(argv[++i], "id_asc") ? TC_TIE_ID_ASC : TC_TIE_REFERENCE;
        else if (!strcmp(argv[i], "--parts") && i + 1 < argc) {
            ks.clear();
            for (char *t = strtok(argv[++i], ","); t; t = strtok(nullptr, ",")) ks.push_back(atoi(t));
        } else {
            fprintf(stderr, "unknown argument %s\n", argv[i]);
            return 1;
        }
    }
    const double t0 = cli::now_s();
    int64_t *src = nullptr, *dst = nullptr, m = 0;
    CLI_CHECK(tc_read_edges(argv[1], &src, &dst, &m));
    printf("read %lld edges in %.3f s\n", (long long)m, cli::now_s() - t0);
    tc_ctx *ctx = nullptr;
    CLI_CHECK(tc_ctx_create(0, &ctx));
    const double t1 = cli::now_s();
    tc_ugraph *ug = nullptr;
    CLI_CHECK(tc_ugraph_from_edges(ctx, src, dst, m, 0, &ug));
    tc_host_free(src);
    tc_host_free(dst);
    tc_graph *og = nullptr;
    CLI_CHECK(tc_orient(ctx, ug, tie, &og));
    printf("device clean-up + orientation in %.3f s\n", cli::now_s() - t1);
    int64_t N = 0, nnz2 = 0, V = 0, m_or = 0;
    CLI_CHECK(tc_ugraph_info(ug, &N, &nnz2));
    CLI_CHECK(tc_graph_info(og, &V, &m_or, nullptr));
    std::vector<int32_t> orp((size_t)V + 1), ocol((size_t)m_or);
    CLI_CHECK(tc_graph_download_i32(ctx, og, orp.data(), ocol.data()));
    const std::string base = out_dir + "/" + stem(argv[1]);
    // <name>_output.csr: "V E V+1 m \n" row_ptr col (without_part_preprocess.py:298-311)
    const std::string o1 = base + "_output.csr";
    const int64_t h1[4] = {V, nnz2, V + 1, m_or};
    CLI_CHECK(tc_text_write_line(o1.c_str(), h1, 4, 8, 'w', 1));
    CLI_CHECK(tc_text_write_line(o1.c_str(), orp.data(), V + 1, 4, 'a', 1));
    CLI_CHECK(tc_text_write_line(o1.c_str(), ocol.data(), m_or, 4, 'a', 1));
    // <name>_part.csr: "N E\n" "N N+1 2m 0 \n" row_ptr col in_deg (Halo_creation_preprocess.py:259-278)
    std::vector<int64_t> rp((size_t)N + 1), col((size_t)nnz2), deg((size_t)N);
    CLI_CHECK(tc_ugraph_download(ctx, ug, rp.data(), col.data(), deg.data()));
    const std::string o2 = base + "_part.csr";
    const int64_t h2a[2] = {N, nnz2}, h2b[4] = {N, N + 1, nnz2, 0};
    CLI_CHECK(tc_text_write_line(o2.c_str(), h2a, 2, 8, 'w', 0));
    CLI_CHECK(tc_text_write_line(o2.c_str(), h2b, 4, 8, 'a', 1));
    CLI_CHECK(tc_text_write_line(o2.c_str(), rp.data(), N + 1, 8, 'a', 1));
    CLI_CHECK(tc_text_write_line(o2.c_str(), col.data(), nnz2, 8, 'a', 1));
    CLI_CHECK(tc_text_write_line(o2.c_str(), deg.data(), N, 8, 'a', 1));
    std::vector<int32_t> part((size_t)N);
    for (int k : ks) {
        if (k < 1) continue;
        CLI_CHECK(tc_gen_parts_random(N, k, seed + (uint64_t)k, part.data()));
        const std::string o3 = o2 + "_node_parts_random_" + std::to_string(k);
        CLI_CHECK(tc_text_write_line(o3.c_str(), part.data(), N, 4, 'w', 1));
        CLI_CHECK(tc_gen_parts_contig(N, k, part.data()));
        const std::string o4 = o2 + "_node_parts_contig_" + std::to_string(k);
        CLI_CHECK(tc_text_write_line(o4.c_str(), part.data(), N, 4, 'w', 1));
        if (k <= 64) {
            CLI_CHECK(tc_gen_parts_lp(ctx, ug, k, seed + (uint64_t)k, 20, part.data()));
            const std::string o5 = o2 + "_node_parts_lp_" + std::to_string(k);
            CLI_CHECK(tc_text_write_line(o5.c_str(), part.data(), N, 4, 'w', 1));
        }
    }
    if (tcsr) {
        std::vector<int64_t> orp64(orp.begin(), orp.end());
        CLI_CHECK(tc_tcsr_write((base + ".tcsr").c_str(), orp64.data(), ocol.data(), V, m_or, V, nnz2));
    }
    printf("vertices %lld, undirected entries %lld, oriented edges %lld; wrote %s, %s\n", (long long)V,
           (long long)nnz2, (long long)m_or, o1.c_str(), o2.c_str());
    tc_graph_destroy(og);
    tc_ugraph_destroy(ug);
    tc_ctx_destroy(ctx);
    return 0;
}
