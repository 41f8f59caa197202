"""The autotuner (tc_autotune): it times at most max_trials candidates, leaves
every tuning field inside the documented range, and the counts under the
tuning it picks (whole and per root) still equal the oracle's."""
import numpy as np
import pytest

import oracle
from trianglecount_gb300 import generators as gen

pytestmark = pytest.mark.gpu

# documented ranges (include/tc.h, tc_tuning)
RANGES = {
    "warp_max_deg": lambda v: v in (32, 64, 128, 256, 512),
    "light_max_work": lambda v: v > 0,
    "unit_work": lambda v: v > 0,
    "long_list": lambda v: 0 <= v <= 4096,
    "probe_kicks": lambda v: 0 <= v <= 1024,
    "heavy_bitmap": lambda v: v in (0, 1),
    "hash_pairs": lambda v: v in (0, 1),
    "flat_max_deg": lambda v: 0 <= v <= 8,
    "intersect": lambda v: v in (0, 1, 2),
}


@pytest.fixture
def fresh(ctx):
    old = ctx.get_tuning()
    yield ctx
    ctx.set_tuning(old["warp_max_deg"], old["light_max_work"], old["unit_work"], old["long_list"],
                   old["probe_kicks"], old["heavy_bitmap"], 0, old["hash_pairs"], old["flat_max_deg"],
                   old["intersect"])


@pytest.mark.parametrize("maker", ["rmat14", "chung_lu"])
@pytest.mark.parametrize("max_trials", [1, 5, 12])
def test_autotune_respects_budget_ranges_and_counts(fresh, maker, max_trials):
    src, dst = gen.rmat(14) if maker == "rmat14" else gen.chung_lu(100000, 12.0, seed=77)
    orp, ocl, want = oracle.pipeline(src, dst)
    _, want_pr = oracle.count(orp, ocl, per_root=True)
    g = fresh.upload(orp, ocl)
    tuning, best_ms, trials = fresh.autotune(g, max_trials=max_trials, reps=2, with_trials=True)
    assert 1 <= trials <= max_trials
    assert best_ms > 0
    for k, ok in RANGES.items():
        assert ok(tuning[k]), (k, tuning[k])
    cur = fresh.get_tuning()
    assert all(cur[k] == tuning[k] for k in RANGES)  # the picked tuning is the context's
    assert fresh.count(g) == want
    assert np.array_equal(fresh.count_per_root(g), want_pr)
