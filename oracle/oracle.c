/*
 * oracle.c -- CPU restatement of the reference triangle-counting path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: only the tests, the
 * smoke check and the CPU-baseline leg of bench.py load it.  The product
 * (libtc, the CLIs, the Python package) never links or calls it, and has no
 * CPU fallback.
 *
 * Every function cites the reference code it restates (paths are relative to
 * the KishantLab/TriangleCount tree).  Arithmetic is integer only.
 *
 *   orc_clean        DGL clean-up: remove_self_loop -> to_bidirected ->
 *                    remove isolated nodes -> adj_tensors('csr')
 *                    (Med_dataset/without_part_preprocess.py:193-228)
 *   orc_orient       degree orientation, count -> scan -> scatter, row order
 *                    preserved (Med_dataset/without_part_preprocess.py:19-111,
 *                    253-270; preprocess_CPU/Undir2Dir.c:107-133)
 *   orc_count        sum over roots of |N+(u) n N+(v)| for v in N+(u)
 *                    (src/WithoutPartition/ShareKernelTCV62_update_v1.cu:43-191
 *                    per-block g_sum; src/WithPartition/without_sorting_tc.cu:57-219
 *                    with roots 0..t_ver-1), as an OpenMP merge intersection
 *   orc_count_brute  independent O(sum d^2) count on the undirected graph
 *   orc_read_csr_fscanf  the TC_128 driver's .csr reader: one fscanf("%d")
 *                    per integer, single-threaded
 *                    (src/WithoutPartition/ShareKernelTCV62_update_v1.cu:206-230),
 *                    the CPU baseline of the library's parallel text parser
 *   orc_halo_part    per-part halo subgraph
 *                    (preprocess_GPU/Halo_cleanned_preprocess/round_clean_subgraph.cu:357-902)
 *                    with the prune loop of
 *                    preprocess_GPU/generate_clean_undir_dataset/Halo_creation_preprocess.py:566-589
 *
 *   orc_gen_rmat / orc_gen_parts_random  the benchmark's seeded inputs,
 *                    generated without the library so that the reference arm
 *                    of bench.py loads no product code: R-MAT quadrant draws
 *                    of 16 bits from the splitmix64 output function applied
 *                    to (seed, stream, index), a Fisher-Yates vertex
 *                    permutation, and uniform parts (they replace the
 *                    unseeded np.random.randint of
 *                    Halo_creation_preprocess.py:288); the tests check them
 *                    bit for bit against the library's generators
 *
 * Tie-break: the reference keeps u->w iff deg(u) < deg(w), or deg(u) == deg(w)
 * and w < u (without_part_preprocess.py:37-50).  ORC_TIE_ID_ASC selects the
 * other strict order, (deg u, u) < (deg w, w).  Both orient every undirected
 * edge exactly once, so the count is the same; the files differ.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_TIE_REFERENCE 0 /* keep u->w iff deg u < deg w || (== && w < u) */
#define ORC_TIE_ID_ASC 1    /* keep u->w iff deg u < deg w || (== && u < w) */

static int keep_edge(int64_t du, int64_t dw, int64_t u, int64_t w, int tie)
{
    if (du < dw) return 1;
    if (du > dw) return 0;
    return tie == ORC_TIE_REFERENCE ? (w < u) : (u < w);
}

static int cmp_i64(const void *a, const void *b)
{
    int64_t x = *(const int64_t *)a, y = *(const int64_t *)b;
    return (x > y) - (x < y);
}

int orc_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/*
 * orc_clean: edge list -> simple undirected CSR with sorted rows.
 *
 * dgl.graph((u, v)) has max(id)+1 nodes; remove_self_loop drops u == v;
 * to_bidirected returns the simple symmetric graph (each {u, v} once per
 * direction); isolated nodes (in == out == 0) are removed and the survivors
 * keep their relative order (without_part_preprocess.py:193-208).  The CSR of
 * adj_tensors('csr') lists each row ascending (:225-228).
 *
 * n_nodes may exceed max(id)+1 (extra vertices are isolated and dropped).
 * Buffers: row_ptr_out capacity >= N0 + 1 where N0 = max(n_nodes, max id + 1);
 * col_out capacity >= 2 * n; old_id_out (optional) capacity >= N0.
 * Returns nnz (= 2m) and writes *V_out, or -1 on a negative id.
 */
int64_t orc_clean(int64_t n, const int64_t *src, const int64_t *dst, int64_t n_nodes,
                  int64_t *row_ptr_out, int64_t *col_out, int64_t *V_out, int64_t *old_id_out)
{
    int64_t N0 = n_nodes;
    for (int64_t i = 0; i < n; i++) {
        if (src[i] < 0 || dst[i] < 0) return -1;
        if (src[i] + 1 > N0) N0 = src[i] + 1;
        if (dst[i] + 1 > N0) N0 = dst[i] + 1;
    }
    int64_t *cnt = (int64_t *)calloc((size_t)N0 + 1, sizeof(int64_t));
    for (int64_t i = 0; i < n; i++) {
        if (src[i] == dst[i]) continue;
        cnt[src[i] + 1]++;
        cnt[dst[i] + 1]++;
    }
    for (int64_t v = 0; v < N0; v++) cnt[v + 1] += cnt[v];
    int64_t total = cnt[N0];
    int64_t *tmp = (int64_t *)malloc(sizeof(int64_t) * (size_t)(total ? total : 1));
    int64_t *fill = (int64_t *)malloc(sizeof(int64_t) * (size_t)(N0 + 1));
    memcpy(fill, cnt, sizeof(int64_t) * (size_t)(N0 + 1));
    for (int64_t i = 0; i < n; i++) {
        if (src[i] == dst[i]) continue;
        tmp[fill[src[i]]++] = dst[i];
        tmp[fill[dst[i]]++] = src[i];
    }
    /* sort + dedupe each row (to_bidirected yields a simple graph) */
    int64_t *ulen = fill; /* reuse: unique length per row */
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t v = 0; v < N0; v++) {
        int64_t s = cnt[v], e = cnt[v + 1];
        qsort(tmp + s, (size_t)(e - s), sizeof(int64_t), cmp_i64);
        int64_t k = 0;
        for (int64_t j = s; j < e; j++)
            if (k == 0 || tmp[s + k - 1] != tmp[j]) tmp[s + (k++)] = tmp[j];
        ulen[v] = k;
    }
    /* isolated removal with order-preserving relabel */
    int64_t *newid = (int64_t *)malloc(sizeof(int64_t) * (size_t)(N0 ? N0 : 1));
    int64_t V = 0;
    for (int64_t v = 0; v < N0; v++) {
        if (ulen[v] > 0) {
            if (old_id_out) old_id_out[V] = v;
            newid[v] = V++;
        } else {
            newid[v] = -1;
        }
    }
    int64_t pos = 0;
    row_ptr_out[0] = 0;
    int64_t r = 0;
    for (int64_t v = 0; v < N0; v++) {
        if (ulen[v] == 0) continue;
        int64_t s = cnt[v];
        for (int64_t j = 0; j < ulen[v]; j++) col_out[pos++] = newid[tmp[s + j]];
        row_ptr_out[++r] = pos;
    }
    *V_out = V;
    free(cnt);
    free(tmp);
    free(fill);
    free(newid);
    return pos;
}

/*
 * orc_orient: undirected CSR -> degree-oriented CSR.
 * Find_size counts kept neighbours per row, cp.cumsum scans, Convert scatters
 * them in row order (without_part_preprocess.py:19-111, launches :253-270).
 * The degree is the row length (:29, :34).  Returns the oriented nnz.
 * out_row_ptr capacity V+1, out_col capacity >= row_ptr[V] / 2 (exactly half
 * for a symmetric simple graph).
 */
int64_t orc_orient(int64_t V, const int64_t *row_ptr, const int64_t *col, int tie,
                   int64_t *out_row_ptr, int64_t *out_col)
{
    int64_t *cnt = (int64_t *)malloc(sizeof(int64_t) * (size_t)(V + 1));
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t u = 0; u < V; u++) {
        int64_t du = row_ptr[u + 1] - row_ptr[u], c = 0;
        for (int64_t j = row_ptr[u]; j < row_ptr[u + 1]; j++) {
            int64_t w = col[j];
            c += keep_edge(du, row_ptr[w + 1] - row_ptr[w], u, w, tie);
        }
        cnt[u] = c;
    }
    out_row_ptr[0] = 0;
    for (int64_t u = 0; u < V; u++) out_row_ptr[u + 1] = out_row_ptr[u] + cnt[u];
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t u = 0; u < V; u++) {
        int64_t du = row_ptr[u + 1] - row_ptr[u], p = out_row_ptr[u];
        for (int64_t j = row_ptr[u]; j < row_ptr[u + 1]; j++) {
            int64_t w = col[j];
            if (keep_edge(du, row_ptr[w + 1] - row_ptr[w], u, w, tie)) out_col[p++] = w;
        }
    }
    free(cnt);
    return out_row_ptr[V];
}

/* Same orientation on int32 arrays, for the int32 .csr contract. */
int64_t orc_orient_i32(int64_t V, const int32_t *row_ptr, const int32_t *col, int tie,
                       int32_t *out_row_ptr, int32_t *out_col)
{
    int64_t *cnt = (int64_t *)malloc(sizeof(int64_t) * (size_t)(V + 1));
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t u = 0; u < V; u++) {
        int64_t du = row_ptr[u + 1] - row_ptr[u], c = 0;
        for (int64_t j = row_ptr[u]; j < row_ptr[u + 1]; j++) {
            int64_t w = col[j];
            c += keep_edge(du, row_ptr[w + 1] - row_ptr[w], u, w, tie);
        }
        cnt[u] = c;
    }
    out_row_ptr[0] = 0;
    for (int64_t u = 0; u < V; u++) out_row_ptr[u + 1] = (int32_t)(out_row_ptr[u] + cnt[u]);
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t u = 0; u < V; u++) {
        int64_t du = row_ptr[u + 1] - row_ptr[u], p = out_row_ptr[u];
        for (int64_t j = row_ptr[u]; j < row_ptr[u + 1]; j++) {
            int64_t w = col[j];
            if (keep_edge(du, row_ptr[w + 1] - row_ptr[w], u, w, tie)) out_col[p++] = (int32_t)w;
        }
    }
    free(cnt);
    return out_row_ptr[V];
}

/* |a n b| for ascending lists (two-pointer merge). */
static uint64_t merge_count_i64(const int64_t *a, int64_t na, const int64_t *b, int64_t nb)
{
    uint64_t c = 0;
    int64_t i = 0, j = 0;
    while (i < na && j < nb) {
        if (a[i] < b[j]) i++;
        else if (a[i] > b[j]) j++;
        else { c++; i++; j++; }
    }
    return c;
}

static uint64_t merge_count_i32(const int32_t *a, int64_t na, const int32_t *b, int64_t nb)
{
    uint64_t c = 0;
    int64_t i = 0, j = 0;
    while (i < na && j < nb) {
        if (a[i] < b[j]) i++;
        else if (a[i] > b[j]) j++;
        else { c++; i++; j++; }
    }
    return c;
}

/*
 * orc_count: triangles of an oriented CSR with ascending rows, roots
 * 0..n_roots-1.  per_root (optional, length n_roots) receives the reference's
 * g_sum[u] = sum_{v in N+(u)} |N+(u) n N+(v)|
 * (ShareKernelTCV62_update_v1.cu:175-186; without_sorting_tc.cu:207-217).
 * The total is sum over roots (the cub::DeviceReduce::Sum at :271-277 / :422-428).
 */
uint64_t orc_count(int64_t n_roots, const int64_t *row_ptr, const int64_t *col, uint64_t *per_root)
{
    uint64_t total = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : total)
    for (int64_t u = 0; u < n_roots; u++) {
        const int64_t *a = col + row_ptr[u];
        int64_t na = row_ptr[u + 1] - row_ptr[u];
        uint64_t t = 0;
        for (int64_t j = 0; j < na; j++) {
            int64_t v = a[j];
            t += merge_count_i64(a, na, col + row_ptr[v], row_ptr[v + 1] - row_ptr[v]);
        }
        if (per_root) per_root[u] = t;
        total += t;
    }
    return total;
}

uint64_t orc_count_i32(int64_t n_roots, const int32_t *row_ptr, const int32_t *col, uint64_t *per_root)
{
    uint64_t total = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : total)
    for (int64_t u = 0; u < n_roots; u++) {
        const int32_t *a = col + row_ptr[u];
        int64_t na = row_ptr[u + 1] - row_ptr[u];
        uint64_t t = 0;
        for (int64_t j = 0; j < na; j++) {
            int32_t v = a[j];
            t += merge_count_i32(a, na, col + row_ptr[v], row_ptr[v + 1] - row_ptr[v]);
        }
        if (per_root) per_root[u] = t;
        total += t;
    }
    return total;
}

/* Single-thread variant of orc_count_i32 for a bounded sample of roots
 * [r0, r1), used to time the scalar CPU baseline. */
uint64_t orc_count_i32_range(int64_t r0, int64_t r1, const int32_t *row_ptr, const int32_t *col)
{
    uint64_t total = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : total)
    for (int64_t u = r0; u < r1; u++) {
        const int32_t *a = col + row_ptr[u];
        int64_t na = row_ptr[u + 1] - row_ptr[u];
        for (int64_t j = 0; j < na; j++) {
            int32_t v = a[j];
            total += merge_count_i32(a, na, col + row_ptr[v], row_ptr[v + 1] - row_ptr[v]);
        }
    }
    return total;
}

static int has_edge(const int64_t *row_ptr, const int64_t *col, int64_t a, int64_t b)
{
    int64_t lo = row_ptr[a], hi = row_ptr[a + 1] - 1;
    while (lo <= hi) {
        int64_t mid = lo + (hi - lo) / 2;
        if (col[mid] < b) lo = mid + 1;
        else if (col[mid] > b) hi = mid - 1;
        else return 1;
    }
    return 0;
}

/* Independent count on the undirected sorted CSR: triangles u < v < w. */
uint64_t orc_count_brute(int64_t V, const int64_t *row_ptr, const int64_t *col)
{
    uint64_t total = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : total)
    for (int64_t u = 0; u < V; u++) {
        for (int64_t i = row_ptr[u]; i < row_ptr[u + 1]; i++) {
            int64_t v = col[i];
            if (v <= u) continue;
            for (int64_t j = i + 1; j < row_ptr[u + 1]; j++) {
                int64_t w = col[j];
                if (w <= v) continue;
                total += (uint64_t)has_edge(row_ptr, col, v, w);
            }
        }
    }
    return total;
}

/*
 * orc_halo_part: the halo subgraph of part p (round_clean_subgraph.cu:357-902).
 *
 *  1. part vertices P = {v : part[v] == p}, ascending (:390-397); t_ver = |P|.
 *  2. halo H = neighbours of P outside P, sorted and unique (find_halo_nodes1
 *     :69-120, MergeSort + Unique :468-495).
 *  3. combined = P ++ H; local id = position (:527-530, :600-602).
 *  4. for every combined src and neighbour dest with src -> dest kept by the
 *     orientation rule on the file's degree array (Find_size/Convert
 *     :160-272) and dest in combined: local edge lid(src) -> lid(dest); rows
 *     ascending by local id (sorting_col_idx :323-346).
 *  5. prune: repeatedly remove halo vertices (local id >= t_ver) whose
 *     in-degree in the current subgraph is 0, relabelling order-preservingly,
 *     until none is left (the intended loop, Halo_creation_preprocess.py:566-589;
 *     round_clean_subgraph.cu:671-838 implements round 1 correctly only).
 *
 * mode 1 (the library's counting halo, which has no reference counterpart):
 * step 2 keeps only the neighbours d of P outside P with s -> d kept by the
 * orientation rule for some s in P; steps 3-5 are unchanged (step 5 then
 * removes nothing: every halo vertex keeps its in-edge from P).
 *
 * Buffers: out_row_ptr capacity V+1, out_col capacity row_ptr[V].
 * Outputs *n_local, *t_ver; returns the local nnz.
 */
int64_t orc_halo_part(int64_t V, const int64_t *row_ptr, const int64_t *col, const int64_t *deg,
                      const int64_t *part, int64_t p, int tie, int mode, int64_t *out_row_ptr, int64_t *out_col,
                      int64_t *n_local_out, int64_t *t_ver_out)
{
    int64_t *lid = (int64_t *)malloc(sizeof(int64_t) * (size_t)(V ? V : 1));
    char *inH = (char *)calloc((size_t)(V ? V : 1), 1);
    int64_t t_ver = 0;
    for (int64_t v = 0; v < V; v++) {
        lid[v] = -1;
        if (part[v] == p) lid[v] = t_ver++;
    }
    for (int64_t v = 0; v < V; v++) {
        if (part[v] != p) continue;
        for (int64_t j = row_ptr[v]; j < row_ptr[v + 1]; j++)
            if (part[col[j]] != p && (mode == 0 || keep_edge(deg[v], deg[col[j]], v, col[j], tie)))
                inH[col[j]] = 1;
    }
    int64_t n_comb = t_ver;
    for (int64_t v = 0; v < V; v++)
        if (inH[v]) lid[v] = n_comb++;
    int64_t *comb = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n_comb ? n_comb : 1));
    for (int64_t v = 0; v < V; v++)
        if (lid[v] >= 0) comb[lid[v]] = v;
    /* step 4: oriented local CSR */
    int64_t *rp = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n_comb + 1));
    int64_t *cl = (int64_t *)malloc(sizeof(int64_t) * (size_t)(row_ptr[V] ? row_ptr[V] : 1));
    rp[0] = 0;
    int64_t pos = 0;
    for (int64_t i = 0; i < n_comb; i++) {
        int64_t s = comb[i], s0 = pos;
        for (int64_t j = row_ptr[s]; j < row_ptr[s + 1]; j++) {
            int64_t d = col[j];
            if (lid[d] >= 0 && keep_edge(deg[s], deg[d], s, d, tie)) cl[pos++] = lid[d];
        }
        qsort(cl + s0, (size_t)(pos - s0), sizeof(int64_t), cmp_i64);
        rp[i + 1] = pos;
    }
    /* step 5: prune to the fixpoint */
    int64_t *indeg = (int64_t *)calloc((size_t)(n_comb ? n_comb : 1), sizeof(int64_t));
    char *alive = (char *)malloc((size_t)(n_comb ? n_comb : 1));
    for (int64_t i = 0; i < n_comb; i++) alive[i] = 1;
    for (int64_t j = 0; j < pos; j++) indeg[cl[j]]++;
    int64_t *stack = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n_comb ? n_comb : 1));
    int64_t top = 0;
    for (int64_t i = t_ver; i < n_comb; i++)
        if (indeg[i] == 0) { alive[i] = 0; stack[top++] = i; }
    while (top > 0) {
        int64_t x = stack[--top];
        for (int64_t j = rp[x]; j < rp[x + 1]; j++) {
            int64_t d = cl[j];
            if (--indeg[d] == 0 && d >= t_ver && alive[d]) { alive[d] = 0; stack[top++] = d; }
        }
    }
    int64_t *nid = lid; /* reuse as old-local -> new-local */
    int64_t nl = 0;
    for (int64_t i = 0; i < n_comb; i++) nid[i] = alive[i] ? nl++ : -1;
    int64_t op = 0;
    int64_t r = 0;
    out_row_ptr[0] = 0;
    for (int64_t i = 0; i < n_comb; i++) {
        if (!alive[i]) continue;
        for (int64_t j = rp[i]; j < rp[i + 1]; j++) out_col[op++] = nid[cl[j]];
        out_row_ptr[++r] = op;
    }
    *n_local_out = nl;
    *t_ver_out = t_ver;
    free(lid);
    free(inH);
    free(comb);
    free(rp);
    free(cl);
    free(indeg);
    free(alive);
    free(stack);
    return op;
}

/* The .csr reader of the TC_128 driver
 * (src/WithoutPartition/ShareKernelTCV62_update_v1.cu:206-230): the header
 * "V E row_ptr_s col_idx_s", then row_ptr_s and col_idx_s integers, each read
 * by its own fscanf("%d").  hdr gets the four header values; *row_ptr and *col
 * are malloc'd (release with orc_free).  Returns 0, or -1 when the file cannot
 * be opened or ends early. */
int orc_read_csr_fscanf(const char *path, int64_t hdr[4], int32_t **row_ptr, int32_t **col)
{
    FILE *f = fopen(path, "r");
    int v[4], d;
    int32_t *rp = NULL, *cl = NULL;
    *row_ptr = NULL;
    *col = NULL;
    if (!f) return -1;
    for (int i = 0; i < 4; ++i)
        if (fscanf(f, "%d", &v[i]) != 1 || v[i] < 0) {
            fclose(f);
            return -1;
        }
    rp = (int32_t *)malloc(sizeof(int32_t) * (size_t)(v[2] ? v[2] : 1));
    cl = (int32_t *)malloc(sizeof(int32_t) * (size_t)(v[3] ? v[3] : 1));
    for (int i = 0; rp && cl && i < v[2]; ++i) {
        if (fscanf(f, "%d", &d) != 1) goto fail;
        rp[i] = d;
    }
    for (int j = 0; rp && cl && j < v[3]; ++j) {
        if (fscanf(f, "%d", &d) != 1) goto fail;
        cl[j] = d;
    }
    if (!rp || !cl) goto fail;
    fclose(f);
    for (int i = 0; i < 4; ++i) hdr[i] = v[i];
    *row_ptr = rp;
    *col = cl;
    return 0;
fail:
    fclose(f);
    free(rp);
    free(cl);
    return -1;
}

void orc_free(void *p) { free(p); }

/* ---- seeded inputs (independent of the library) ------------------------- */
/* splitmix64's output function (Steele, Lea, Flood, OOPSLA 2014) on a counter */
static uint64_t orc_mix(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

/* draw i of stream `stream` under `seed` */
static uint64_t orc_draw(uint64_t seed, uint64_t stream, uint64_t i)
{
    return orc_mix(orc_mix(seed ^ (stream * 0xD1B54A32D192ED03ull)) + i);
}

/* r mapped onto [0, range) by the high half of the 128-bit product (Lemire) */
static uint64_t orc_below(uint64_t r, uint64_t range)
{
    return (uint64_t)(((unsigned __int128)r * range) >> 64);
}

/* R-MAT: edge_factor << scale edges; at each of `scale` levels a 16-bit draw
 * picks quadrant (0,0) below a, (0,1) below a+b, (1,0) below a+b+c, else
 * (1,1) (probabilities as 16-bit fixed point, rounded); four levels share one
 * 64-bit draw (stream 1, index 8 i + level / 4).  permute != 0 relabels by a
 * Fisher-Yates shuffle (stream 2, index = the position swapped down). */
int orc_gen_rmat(int scale, int edge_factor, double a, double b, double c, uint64_t seed, int permute,
                 int64_t *src, int64_t *dst)
{
    if (scale < 1 || scale > 31 || edge_factor < 1) return -1;
    const int64_t n = (int64_t)edge_factor << scale, nv = (int64_t)1 << scale;
    const uint32_t qa = (uint32_t)llround(a * 65536.0), qab = (uint32_t)llround((a + b) * 65536.0),
                   qabc = (uint32_t)llround((a + b + c) * 65536.0);
    int64_t *perm = NULL;
    if (permute) {
        perm = (int64_t *)malloc(sizeof(int64_t) * (size_t)nv);
        if (!perm) return -1;
        for (int64_t i = 0; i < nv; i++) perm[i] = i;
        for (int64_t i = nv - 1; i > 0; i--) {
            const int64_t j = (int64_t)orc_below(orc_draw(seed, 2, (uint64_t)i), (uint64_t)i + 1);
            const int64_t t = perm[i];
            perm[i] = perm[j];
            perm[j] = t;
        }
    }
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < n; e++) {
        int64_t u = 0, v = 0;
        uint64_t bits = 0;
        for (int l = 0; l < scale; l++) {
            if (l % 4 == 0) bits = orc_draw(seed, 1, (uint64_t)e * 8 + (uint64_t)(l / 4));
            const uint32_t r = (uint32_t)(bits & 0xFFFFu);
            bits >>= 16;
            const int right = r >= qabc || (r >= qa && r < qab);
            const int down = r >= qab;
            u = 2 * u + down;
            v = 2 * v + right;
        }
        src[e] = permute ? perm[u] : u;
        dst[e] = permute ? perm[v] : v;
    }
    free(perm);
    return 0;
}

/* part[v] uniform in [0, k) (stream 5, index v) */
int orc_gen_parts_random(int64_t n, int k, uint64_t seed, int32_t *part)
{
    if (n < 0 || k < 1) return -1;
    for (int64_t v = 0; v < n; v++) part[v] = (int32_t)orc_below(orc_draw(seed, 5, (uint64_t)v), (uint64_t)k);
    return 0;
}
