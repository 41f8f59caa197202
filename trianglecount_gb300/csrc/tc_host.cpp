// tc_host.cpp -- host utilities of libtc: text and binary graph files, seeded
// synthetic graph generators.  No GPU is touched here.
#include <algorithm>
#include <atomic>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <thread>
#include <vector>

#include "tc_internal.h"

namespace {

using tc::set_error;

int n_workers(int64_t work, int64_t per_thread) {
    unsigned hc = std::thread::hardware_concurrency();
    if (hc == 0) hc = 4;
    int64_t t = work / std::max<int64_t>(per_thread, 1) + 1;
    return (int)std::max<int64_t>(1, std::min<int64_t>(t, hc));
}

// Runs f(i, t) for i in [0, n) split into contiguous ranges over t threads.
void parallel_ranges(int64_t n, int threads, const std::function<void(int64_t, int64_t, int)> &f) {
    if (threads <= 1 || n < 2) {
        f(0, n, 0);
        return;
    }
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t) {
        const int64_t a = n * t / threads, b = n * (t + 1) / threads;
        pool.emplace_back([=, &f] { f(a, b, t); });
    }
    for (auto &th : pool) th.join();
}

// ---- counter-based RNG: the splitmix64 output function (Steele, Lea, Flood,
// "Fast splittable pseudorandom number generators", OOPSLA 2014) applied to
// (seed, stream, index).  Integer-only, so every platform draws the same bits.
inline uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
inline uint64_t rng_at(uint64_t seed, uint64_t stream, uint64_t i) {
    return mix64(mix64(seed ^ (stream * 0xD1B54A32D192ED03ull)) + i);
}
// Lemire's multiply-shift map of a 64-bit draw onto [0, range).
inline uint64_t bounded(uint64_t r, uint64_t range) { return (uint64_t)(((__uint128_t)r * range) >> 64); }

void seeded_permutation(int64_t n, uint64_t seed, std::vector<int64_t> &perm) {
    perm.resize((size_t)n);
    for (int64_t i = 0; i < n; ++i) perm[(size_t)i] = i;
    for (int64_t i = n - 1; i > 0; --i) {
        const int64_t j = (int64_t)bounded(rng_at(seed, 2, (uint64_t)i), (uint64_t)i + 1);
        std::swap(perm[(size_t)i], perm[(size_t)j]);
    }
}

// ---- text -----------------------------------------------------------------------
inline bool is_ws(char c) { return c == ' ' || c == '\n' || c == '\t' || c == '\r' || c == '\v' || c == '\f'; }

int read_file(const char *path, std::vector<char> &buf) {
    FILE *f = fopen(path, "rb");
    if (!f) return set_error(TC_E_IO, "cannot open %s", path);
    if (fseek(f, 0, SEEK_END) != 0) {
        fclose(f);
        return set_error(TC_E_IO, "cannot seek %s", path);
    }
    long sz = ftell(f);
    fseek(f, 0, SEEK_SET);
    buf.resize((size_t)sz + 1);
    size_t got = sz > 0 ? fread(buf.data(), 1, (size_t)sz, f) : 0;
    fclose(f);
    if ((long)got != sz) return set_error(TC_E_IO, "short read on %s", path);
    buf[(size_t)sz] = ' ';
    return TC_OK;
}

char *format_u(char *p, uint64_t v) {
    char tmp[24];
    int k = 0;
    do {
        tmp[k++] = (char)('0' + v % 10);
        v /= 10;
    } while (v);
    while (k) *p++ = tmp[--k];
    return p;
}

char *format_i(char *p, int64_t v) {
    if (v < 0) {
        *p++ = '-';
        return format_u(p, (uint64_t)(-(v + 1)) + 1);
    }
    return format_u(p, (uint64_t)v);
}

struct TcsrHeader {
    char magic[8];
    int64_t n_rows, nnz, n_roots, aux;
    int64_t reserved[3];
};
const char kTcsrMagic[8] = {'T', 'C', 'S', 'R', '0', '0', '0', '1'};

}  // namespace

extern "C" {

void tc_host_free(void *p) { free(p); }

int tc_text_read_u64(const char *path, uint64_t **data, int64_t *n) {
    if (!path || !data || !n) return set_error(TC_E_INVALID, "null argument");
    *data = nullptr;
    *n = 0;
    std::vector<char> buf;
    TC_TRY(read_file(path, buf));
    const int64_t size = (int64_t)buf.size() - 1;
    const int T = n_workers(size, 1 << 20);
    std::vector<int64_t> cut((size_t)T + 1);
    cut[0] = 0;
    cut[(size_t)T] = size;
    for (int t = 1; t < T; ++t) {
        int64_t s = size * t / T;
        while (s < size && !is_ws(buf[(size_t)s])) ++s;
        cut[(size_t)t] = std::max(s, cut[(size_t)t - 1]);
    }
    std::vector<int64_t> counts((size_t)T, 0);
    std::atomic<int64_t> bad{-1};
    parallel_ranges(T, T, [&](int64_t a, int64_t b, int) {
        for (int64_t t = a; t < b; ++t) {
            int64_t c = 0;
            bool in = false;
            for (int64_t i = cut[(size_t)t]; i < cut[(size_t)t + 1]; ++i) {
                const bool w = is_ws(buf[(size_t)i]);
                if (!w && !in) ++c;
                in = !w;
            }
            counts[(size_t)t] = c;
        }
    });
    std::vector<int64_t> off((size_t)T + 1, 0);
    for (int t = 0; t < T; ++t) off[(size_t)t + 1] = off[(size_t)t] + counts[(size_t)t];
    uint64_t *out = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)std::max<int64_t>(off[(size_t)T], 1));
    if (!out) return set_error(TC_E_NOMEM, "host allocation of %lld values", (long long)off[(size_t)T]);
    parallel_ranges(T, T, [&](int64_t a, int64_t b, int) {
        for (int64_t t = a; t < b; ++t) {
            int64_t k = off[(size_t)t];
            const char *p = buf.data() + cut[(size_t)t];
            const char *e = buf.data() + cut[(size_t)t + 1];
            while (p < e) {
                while (p < e && is_ws(*p)) ++p;
                if (p >= e) break;
                const char *tok = p;
                uint64_t v = 0;
                bool ok = true;
                if (*p == '+') ++p;
                if (p >= e || !isdigit((unsigned char)*p)) ok = false;
                while (p < e && !is_ws(*p)) {
                    if (!isdigit((unsigned char)*p)) {
                        ok = false;
                        ++p;
                        continue;
                    }
                    v = v * 10 + (uint64_t)(*p - '0');
                    ++p;
                }
                if (!ok) {
                    int64_t pos = (int64_t)(tok - buf.data());
                    int64_t prev = bad.load();
                    while ((prev < 0 || pos < prev) && !bad.compare_exchange_weak(prev, pos)) {
                    }
                }
                out[k++] = v;
            }
        }
    });
    if (bad.load() >= 0) {
        free(out);
        return set_error(TC_E_FORMAT, "%s: non-integer token at byte %lld", path, (long long)bad.load());
    }
    *data = out;
    *n = off[(size_t)T];
    return TC_OK;
}

int tc_text_write_line(const char *path, const void *values, int64_t n, int elem_bytes, char mode, int trailing_space) {
    if (!path || (n > 0 && !values) || (elem_bytes != 4 && elem_bytes != 8) || (mode != 'w' && mode != 'a'))
        return set_error(TC_E_INVALID, "bad write arguments");
    FILE *f = fopen(path, mode == 'w' ? "wb" : "ab");
    if (!f) return set_error(TC_E_IO, "cannot open %s for writing", path);
    const int T = n_workers(n, 1 << 20);
    std::vector<std::vector<char>> parts((size_t)T);
    parallel_ranges(n, T, [&](int64_t a, int64_t b, int t) {
        std::vector<char> &o = parts[(size_t)t];
        o.resize((size_t)(b - a) * 21 + 2);
        char *p = o.data();
        for (int64_t i = a; i < b; ++i) {
            const int64_t v = elem_bytes == 4 ? (int64_t)((const int32_t *)values)[i] : ((const int64_t *)values)[i];
            p = format_i(p, v);
            if (trailing_space || i + 1 < n) *p++ = ' ';
        }
        o.resize((size_t)(p - o.data()));
    });
    bool ok = true;
    for (auto &o : parts)
        if (!o.empty() && fwrite(o.data(), 1, o.size(), f) != o.size()) ok = false;
    if (fputc('\n', f) == EOF) ok = false;
    if (fclose(f) != 0) ok = false;
    return ok ? TC_OK : set_error(TC_E_IO, "write to %s failed", path);
}

int tc_read_edges(const char *path, int64_t **src, int64_t **dst, int64_t *n_edges) {
    if (!path || !src || !dst || !n_edges) return set_error(TC_E_INVALID, "null argument");
    *src = *dst = nullptr;
    *n_edges = 0;
    std::vector<char> buf;
    TC_TRY(read_file(path, buf));
    const char *ext = strrchr(path, '.');
    const bool mtx = ext && (strcmp(ext, ".mtx") == 0 || strcmp(ext, ".mmio") == 0);
    std::vector<int64_t> s, d;
    const char *p = buf.data(), *end = buf.data() + buf.size() - 1;
    bool size_line_pending = mtx;
    int64_t line_no = 0;
    while (p < end) {
        const char *eol = (const char *)memchr(p, '\n', (size_t)(end - p));
        if (!eol) eol = end;
        ++line_no;
        const char *q = p;
        while (q < eol && (*q == ' ' || *q == '\t' || *q == '\r')) ++q;
        if (q < eol && *q != '#' && *q != '%') {
            int64_t v[2];
            int got = 0;
            while (got < 2 && q < eol) {
                while (q < eol && (*q == ' ' || *q == '\t' || *q == ',' || *q == '\r')) ++q;
                if (q >= eol) break;
                if (!isdigit((unsigned char)*q)) {
                    return set_error(TC_E_FORMAT, "%s:%lld: expected a vertex id", path, (long long)line_no);
                }
                int64_t x = 0;
                while (q < eol && isdigit((unsigned char)*q)) x = x * 10 + (*q++ - '0');
                v[got++] = x;
            }
            if (got < 2) return set_error(TC_E_FORMAT, "%s:%lld: expected two vertex ids", path, (long long)line_no);
            if (size_line_pending) {
                size_line_pending = false;  // Matrix Market "rows cols nnz" line
            } else if (mtx) {
                if (v[0] < 1 || v[1] < 1) return set_error(TC_E_FORMAT, "%s:%lld: Matrix Market ids are 1-based", path,
                                                           (long long)line_no);
                s.push_back(v[0] - 1);
                d.push_back(v[1] - 1);
            } else {
                s.push_back(v[0]);
                d.push_back(v[1]);
            }
        }
        p = eol + 1;
    }
    const int64_t n = (int64_t)s.size();
    *src = (int64_t *)malloc(sizeof(int64_t) * (size_t)std::max<int64_t>(n, 1));
    *dst = (int64_t *)malloc(sizeof(int64_t) * (size_t)std::max<int64_t>(n, 1));
    if (!*src || !*dst) {
        free(*src);
        free(*dst);
        *src = *dst = nullptr;
        return set_error(TC_E_NOMEM, "host allocation for %lld edges", (long long)n);
    }
    if (n) {
        memcpy(*src, s.data(), sizeof(int64_t) * (size_t)n);
        memcpy(*dst, d.data(), sizeof(int64_t) * (size_t)n);
    }
    *n_edges = n;
    return TC_OK;
}

int tc_tcsr_write(const char *path, const int64_t *row_ptr, const int32_t *col, int64_t n_rows, int64_t nnz,
                  int64_t n_roots, int64_t aux) {
    if (!path || !row_ptr || (nnz > 0 && !col)) return set_error(TC_E_INVALID, "null argument");
    FILE *f = fopen(path, "wb");
    if (!f) return set_error(TC_E_IO, "cannot open %s for writing", path);
    TcsrHeader h;
    memset(&h, 0, sizeof h);
    memcpy(h.magic, kTcsrMagic, 8);
    h.n_rows = n_rows;
    h.nnz = nnz;
    h.n_roots = n_roots;
    h.aux = aux;
    bool ok = fwrite(&h, sizeof h, 1, f) == 1;
    ok = ok && fwrite(row_ptr, sizeof(int64_t), (size_t)(n_rows + 1), f) == (size_t)(n_rows + 1);
    if (nnz > 0) ok = ok && fwrite(col, sizeof(int32_t), (size_t)nnz, f) == (size_t)nnz;
    ok = (fclose(f) == 0) && ok;
    return ok ? TC_OK : set_error(TC_E_IO, "write to %s failed", path);
}

static int tcsr_open(const char *path, TcsrHeader *h, FILE **fp) {
    FILE *f = fopen(path, "rb");
    if (!f) return set_error(TC_E_IO, "cannot open %s", path);
    if (fread(h, sizeof *h, 1, f) != 1 || memcmp(h->magic, kTcsrMagic, 8) != 0 || h->n_rows < 0 || h->nnz < 0) {
        fclose(f);
        return set_error(TC_E_FORMAT, "%s is not a .tcsr file", path);
    }
    *fp = f;
    return TC_OK;
}

int tc_tcsr_read_header(const char *path, int64_t *n_rows, int64_t *nnz, int64_t *n_roots, int64_t *aux) {
    TcsrHeader h;
    FILE *f = nullptr;
    TC_TRY(tcsr_open(path, &h, &f));
    fclose(f);
    if (n_rows) *n_rows = h.n_rows;
    if (nnz) *nnz = h.nnz;
    if (n_roots) *n_roots = h.n_roots;
    if (aux) *aux = h.aux;
    return TC_OK;
}

int tc_tcsr_read(const char *path, int64_t *row_ptr, int32_t *col) {
    TcsrHeader h;
    FILE *f = nullptr;
    TC_TRY(tcsr_open(path, &h, &f));
    bool ok = !row_ptr || fread(row_ptr, sizeof(int64_t), (size_t)(h.n_rows + 1), f) == (size_t)(h.n_rows + 1);
    if (ok && col && h.nnz > 0) {
        if (!row_ptr) fseek(f, (long)(sizeof(TcsrHeader) + sizeof(int64_t) * (size_t)(h.n_rows + 1)), SEEK_SET);
        ok = fread(col, sizeof(int32_t), (size_t)h.nnz, f) == (size_t)h.nnz;
    }
    fclose(f);
    return ok ? TC_OK : set_error(TC_E_FORMAT, "%s is truncated", path);
}

// ---- generators ---------------------------------------------------------------------
int tc_gen_rmat(int scale, int edge_factor, double a, double b, double c, uint64_t seed, int permute, int64_t *src,
                int64_t *dst) {
    if (scale < 1 || scale > 31 || edge_factor < 1 || !src || !dst || a < 0 || b < 0 || c < 0 || a + b + c > 1.0)
        return set_error(TC_E_INVALID, "bad R-MAT parameters");
    const int64_t n = (int64_t)edge_factor << scale;
    const uint32_t ta = (uint32_t)llround(a * 65536.0);
    const uint32_t tab = (uint32_t)llround((a + b) * 65536.0);
    const uint32_t tabc = (uint32_t)llround((a + b + c) * 65536.0);
    std::vector<int64_t> perm;
    if (permute) seeded_permutation((int64_t)1 << scale, seed, perm);
    const int T = n_workers(n, 1 << 18);
    parallel_ranges(n, T, [&](int64_t lo, int64_t hi, int) {
        for (int64_t i = lo; i < hi; ++i) {
            int64_t u = 0, v = 0;
            uint64_t w = 0;
            for (int l = 0; l < scale; ++l) {
                if ((l & 3) == 0) w = rng_at(seed, 1, (uint64_t)i * 8 + (uint64_t)(l >> 2));
                const uint32_t r = (uint32_t)(w & 0xFFFF);
                w >>= 16;
                int ub, vb;
                if (r < ta) ub = 0, vb = 0;
                else if (r < tab) ub = 0, vb = 1;
                else if (r < tabc) ub = 1, vb = 0;
                else ub = 1, vb = 1;
                u = (u << 1) | ub;
                v = (v << 1) | vb;
            }
            if (permute) {
                u = perm[(size_t)u];
                v = perm[(size_t)v];
            }
            src[i] = u;
            dst[i] = v;
        }
    });
    return TC_OK;
}

int tc_gen_road(int64_t width, int64_t height, double p_delete, double diag_rate, uint64_t seed, int64_t *src,
                int64_t *dst, int64_t *n_edges) {
    if (width < 1 || height < 1 || !src || !dst || !n_edges || p_delete < 0 || p_delete > 1 || diag_rate < 0 ||
        diag_rate > 1)
        return set_error(TC_E_INVALID, "bad road-grid parameters");
    const uint32_t t_keep = (uint32_t)llround((1.0 - p_delete) * 65536.0);
    const uint32_t t_diag = (uint32_t)llround(diag_rate * 65536.0);
    int64_t m = 0;
    for (int64_t y = 0; y < height; ++y)
        for (int64_t x = 0; x < width; ++x) {
            const int64_t id = y * width + x;
            const uint64_t r = rng_at(seed, 3, (uint64_t)id);
            if (x + 1 < width && (uint32_t)(r & 0xFFFF) < t_keep) src[m] = id, dst[m++] = id + 1;
            if (y + 1 < height && (uint32_t)((r >> 16) & 0xFFFF) < t_keep) src[m] = id, dst[m++] = id + width;
            if (x + 1 < width && y + 1 < height && (uint32_t)((r >> 32) & 0xFFFF) < t_diag) {
                if ((r >> 48) & 1) src[m] = id, dst[m++] = id + width + 1;
                else src[m] = id + 1, dst[m++] = id + width;
            }
        }
    *n_edges = m;
    return TC_OK;
}

int tc_gen_er(int64_t n, double p, uint64_t seed, int64_t *src, int64_t *dst, int64_t *n_edges) {
    // G(n, M) with M = round(p * n (n-1) / 2) uniform vertex pairs (integer
    // draws only); self-loops and repeats are removed by the clean-up stage.
    if (n < 2 || p < 0 || p > 1 || !src || !dst || !n_edges) return set_error(TC_E_INVALID, "bad ER parameters");
    const int64_t M = llround(p * (double)n * (double)(n - 1) / 2.0);
    if (M > *n_edges) return set_error(TC_E_INVALID, "ER needs %lld edges, buffer holds %lld", (long long)M, (long long)*n_edges);
    const int T = n_workers(M, 1 << 18);
    parallel_ranges(M, T, [&](int64_t lo, int64_t hi, int) {
        for (int64_t i = lo; i < hi; ++i) {
            src[i] = (int64_t)bounded(rng_at(seed, 4, (uint64_t)i * 2), (uint64_t)n);
            dst[i] = (int64_t)bounded(rng_at(seed, 4, (uint64_t)i * 2 + 1), (uint64_t)n);
        }
    });
    *n_edges = M;
    return TC_OK;
}

int tc_gen_chung_lu(int64_t n, double gamma, double avg_deg, uint64_t seed, int64_t *src, int64_t *dst,
                    int64_t n_edges) {
    if (n < 2 || gamma <= 1.0 || avg_deg <= 0 || !src || !dst || n_edges < 0)
        return set_error(TC_E_INVALID, "bad Chung-Lu parameters");
    std::vector<double> w((size_t)n);
    double sum = 0;
    const double ex = -1.0 / (gamma - 1.0);
    for (int64_t i = 0; i < n; ++i) sum += (w[(size_t)i] = pow((double)(i + 1), ex));
    const double scale = avg_deg * (double)n / sum;
    const double cap = sqrt(avg_deg * (double)n);  // sqrt(2E)
    double tot = 0;
    for (int64_t i = 0; i < n; ++i) tot += (w[(size_t)i] = std::min(w[(size_t)i] * scale, cap));
    // fixed-point CDF so the draw is an integer comparison
    std::vector<uint64_t> cdf((size_t)n);
    double run = 0;
    for (int64_t i = 0; i < n; ++i) {
        run += w[(size_t)i];
        cdf[(size_t)i] = (uint64_t)std::min(ldexp(run / tot, 62), ldexp(1.0, 62));
    }
    cdf[(size_t)n - 1] = (uint64_t)1 << 62;
    std::vector<int64_t> perm;
    seeded_permutation(n, seed ^ 0xC1u, perm);
    const int T = n_workers(n_edges, 1 << 18);
    parallel_ranges(n_edges, T, [&](int64_t lo, int64_t hi, int) {
        for (int64_t i = lo; i < hi; ++i) {
            for (int side = 0; side < 2; ++side) {
                const uint64_t r = rng_at(seed, 6, (uint64_t)i * 2 + (uint64_t)side) >> 2;
                const int64_t k = (int64_t)(std::upper_bound(cdf.begin(), cdf.end(), r) - cdf.begin());
                const int64_t v = perm[(size_t)std::min<int64_t>(k, n - 1)];
                if (side == 0) src[i] = v;
                else dst[i] = v;
            }
        }
    });
    return TC_OK;
}

int tc_gen_parts_contig(int64_t n, int k, int32_t *part) {
    // Halo_creation_preprocess.py:293-299: l = N // k; parts[i*l:(i+1)*l] = i on
    // a zero-filled array, so the last N mod k vertices stay in part 0.
    if (n < 0 || k < 1 || (n > 0 && !part)) return set_error(TC_E_INVALID, "bad partition arguments");
    const int64_t l = n / k;
    for (int64_t v = 0; v < n; ++v) part[v] = (l > 0 && v < l * k) ? (int32_t)(v / l) : 0;
    return TC_OK;
}

int tc_gen_parts_random(int64_t n, int k, uint64_t seed, int32_t *part) {
    if (n < 0 || k < 1 || (n > 0 && !part)) return set_error(TC_E_INVALID, "bad partition arguments");
    for (int64_t v = 0; v < n; ++v) part[v] = (int32_t)bounded(rng_at(seed, 5, (uint64_t)v), (uint64_t)k);
    return TC_OK;
}

}  // extern "C"
