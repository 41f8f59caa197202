// tc_tune.cpp -- autotuner for the counting kernel's strategy thresholds.
//
// The thresholds decide, per vertex task, warp vs block execution
// (warp_max_deg, light_max_work), the size of block units (unit_work) and,
// per partner list, whole-warp streaming vs lane flattening (long_list).
// probe_kicks picks the hash (cuckoo or linear probing); intersect the
// bulk-staged sorted lists instead of hash tables, for all tasks or per task.
// Their best values depend on the degree distribution, so they are picked per
// graph by timing the real count: coordinate descent from the current tuning,
// one parameter at a time over a small candidate grid, repeated until a pass
// changes nothing or the trial budget is spent.
#include <algorithm>
#include <vector>

#include "tc_internal.h"

namespace {

int time_count(tc_ctx *ctx, tc_graph *g, int reps, float *ms) {
    std::vector<float> t;
    for (int r = 0; r < reps; ++r) {
        uint64_t c = 0;
        tc_count_stats st;
        TC_TRY(tc_count(ctx, g, &c, &st));
        t.push_back(st.count_ms);
    }
    std::sort(t.begin(), t.end());
    *ms = t[t.size() / 2];
    return TC_OK;
}

}  // namespace

extern "C" int tc_autotune(tc_ctx *ctx, tc_graph *g, int max_trials, int reps, tc_tuning *best, float *best_ms) {
    return tc_autotune_ex(ctx, g, max_trials, reps, best, best_ms, nullptr);
}

extern "C" int tc_autotune_ex(tc_ctx *ctx, tc_graph *g, int max_trials, int reps, tc_tuning *best, float *best_ms,
                              int *trials_out) {
    if (!ctx || !g) return tc::set_error(TC_E_INVALID, "null argument");
    if (max_trials <= 0) max_trials = 32;
    if (reps <= 0) reps = 3;
    tc_tuning cur;
    TC_TRY(tc_ctx_get_tuning(ctx, &cur));
    cur.blocks_per_sm = 0;
    TC_TRY(tc_ctx_set_tuning(ctx, &cur));
    uint64_t warm = 0;
    TC_TRY(tc_count(ctx, g, &warm, nullptr));  // sizes the graph's scratch
    float cur_ms = 0;
    TC_TRY(time_count(ctx, g, reps, &cur_ms));
    int trials = 1;
    const std::vector<int32_t> grid[9] = {
        {64, 128, 256, 512},
        {4096, 8192, 16384, 32768, 65536, 131072},
        {131072, 262144, 524288, 1048576, 2097152, 4194304},
        {8, 16, 32, 64},
        {0, 32},
        {0, 1},
        {0, 1},
        {0, 4, 8},
        {0, 2, 1},
    };
    bool changed = true;
    while (changed && trials < max_trials) {
        changed = false;
        for (int p = 0; p < 9 && trials < max_trials; ++p) {
            for (int32_t v : grid[p]) {
                if (trials >= max_trials) break;
                tc_tuning t = cur;
                int32_t *field = p == 0   ? &t.warp_max_deg
                                 : p == 1 ? &t.light_max_work
                                 : p == 2 ? &t.unit_work
                                 : p == 3 ? &t.long_list
                                 : p == 4 ? &t.probe_kicks
                                 : p == 5 ? &t.heavy_bitmap
                                 : p == 6 ? &t.hash_pairs
                                 : p == 7 ? &t.flat_max_deg
                                          : &t.intersect;
                if (*field == v) continue;
                *field = v;
                TC_TRY(tc_ctx_set_tuning(ctx, &t));
                float ms = 0;
                TC_TRY(time_count(ctx, g, reps, &ms));
                ++trials;
                if (ms < cur_ms * 0.98f) {  // keep a change only if it clearly helps
                    cur = t;
                    cur_ms = ms;
                    changed = true;
                }
            }
        }
    }
    TC_TRY(tc_ctx_set_tuning(ctx, &cur));
    if (trials_out) *trials_out = trials;
    if (best) {
        *best = cur;
        best->blocks_per_sm = 0;
    }
    if (best_ms) *best_ms = cur_ms;
    return TC_OK;
}
