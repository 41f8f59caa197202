"""Device halo extraction against the oracle (exact local CSRs) and the
sum-of-parts invariant."""
import numpy as np
import pytest

import oracle
from trianglecount_gb300 import generators as gen

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode", ["reference", "count"])
@pytest.mark.parametrize("k", [1, 2, 4, 8])
@pytest.mark.parametrize("maker", ["rmat13", "road", "chung_lu"])
def test_halo_parts_match_oracle(ctx, k, maker, mode):
    if maker == "rmat13":
        src, dst = gen.rmat(13)
    elif maker == "road":
        src, dst = gen.road(100)
    else:
        src, dst = gen.chung_lu(30000, 10.0, seed=12)
    rp, col = oracle.clean(src, dst)
    deg = np.diff(rp)
    whole = oracle.count(*oracle.orient(rp, col))
    part = gen.parts_random(len(rp) - 1, k)
    ug = ctx.upload_ugraph(rp, col, deg)
    parts = ctx.halo_extract(ug, part, k, mode=mode)
    total = 0
    for p, g in enumerate(parts):
        lrp, lcol, t_ver = oracle.halo_part(rp, col, deg, part, p, mode=mode)
        drp, dcol = g.download()
        assert g.n_roots == t_ver
        assert np.array_equal(drp, lrp) and np.array_equal(dcol, lcol), (maker, k, p)
        c = ctx.count(g)
        assert c == oracle.count(lrp, lcol, n_roots=t_ver)
        total += c
    assert total == whole
    assert sum(ctx.batch(parts).run()) == whole


def test_halo_with_empty_part(ctx):
    src, dst = gen.rmat(9)
    rp, col = oracle.clean(src, dst)
    part = np.zeros(len(rp) - 1, np.int32)  # parts 1, 2 empty
    ug = ctx.upload_ugraph(rp, col)
    parts = ctx.halo_extract(ug, part, 3)
    assert parts[1].n_rows == 0 and parts[2].n_rows == 0
    assert ctx.count(parts[0]) == oracle.count(*oracle.orient(rp, col))


@pytest.mark.parametrize("n", [1024, 2048, 1023])
@pytest.mark.parametrize("k", [1, 3])
def test_halo_tile_boundaries(ctx, n, k):
    """Circulant graphs C_n(1, 2): 4n undirected entries, so n = 1024 and 2048
    fill exactly one and two 4096-entry tiles (the last row ends on a tile
    boundary) and n = 1023 stops four entries short of one."""
    i = np.arange(n, dtype=np.int64)
    src = np.concatenate([i, i])
    dst = np.concatenate([(i + 1) % n, (i + 2) % n])
    rp, col = oracle.clean(src, dst)
    assert len(col) == 4 * n
    deg = np.diff(rp)
    part = gen.parts_random(n, k)
    ug = ctx.upload_ugraph(rp, col, deg)
    parts = ctx.halo_extract(ug, part, k)
    total = 0
    for p, g in enumerate(parts):
        lrp, lcol, t_ver = oracle.halo_part(rp, col, deg, part, p)
        drp, dcol = g.download()
        assert g.n_roots == t_ver
        assert np.array_equal(drp, lrp) and np.array_equal(dcol, lcol), (n, k, p)
        total += ctx.count(g)
    assert total == oracle.count(*oracle.orient(rp, col)) == n


@pytest.mark.parametrize("mode", ["reference", "count"])
@pytest.mark.parametrize("k, n_labels", [(40, 40), (3, 5), (3, 36)])
def test_halo_many_parts_and_unassigned_vertices(ctx, k, n_labels, mode):
    """k > 32 takes the per-part halo pass instead of the all-parts masks;
    labels >= k (also >= 32) put vertices in no extracted part, though they
    can still be in a part's halo."""
    src, dst = gen.rmat(12)
    rp, col = oracle.clean(src, dst)
    deg = np.diff(rp)
    part = np.random.default_rng(k * 100 + n_labels).integers(0, n_labels, len(rp) - 1).astype(np.int32)
    ug = ctx.upload_ugraph(rp, col, deg)
    parts = ctx.halo_extract(ug, part, k, mode=mode)
    assert len(parts) == k
    for p, g in enumerate(parts):
        lrp, lcol, t_ver = oracle.halo_part(rp, col, deg, part, p, mode=mode)
        drp, dcol = g.download()
        assert g.n_roots == t_ver
        assert np.array_equal(drp, lrp) and np.array_equal(dcol, lcol), (k, n_labels, p)


@pytest.mark.parametrize("tie", ["reference", "id_asc"])
def test_counting_halo_tie_breaks(ctx, tie):
    """Both tie-breaks: the counting halo follows the orientation's own rule."""
    src, dst = gen.rmat(12)
    rp, col = oracle.clean(src, dst)
    deg = np.diff(rp)
    part = gen.parts_random(len(rp) - 1, 4)
    ug = ctx.upload_ugraph(rp, col, deg)
    whole = oracle.count(*oracle.orient(rp, col, tie))
    total = 0
    for p, g in enumerate(ctx.halo_extract(ug, part, 4, tie=tie, mode="count")):
        lrp, lcol, t_ver = oracle.halo_part(rp, col, deg, part, p, tie=tie, mode="count")
        drp, dcol = g.download()
        assert np.array_equal(drp, lrp) and np.array_equal(dcol, lcol), (tie, p)
        total += ctx.count(g)
    assert total == whole


PART_TUNINGS = [
    {},  # defaults: the halo-part instance, heavy and light phases as two kernels
    {"warp_max_deg": 32, "light_max_work": 1, "unit_work": 1, "long_list": 0},  # heavy units everywhere
    {"warp_max_deg": 512, "light_max_work": 1 << 30, "unit_work": 1 << 30, "long_list": 4096},  # warps only
    {"heavy_bitmap": 1, "warp_max_deg": 32, "light_max_work": 64},  # heavy units on the bitmap kernel
    {"intersect": 1, "warp_max_deg": 32, "light_max_work": 64},  # sorted lists, bulk-staged
]


@pytest.mark.parametrize("tuning", PART_TUNINGS)
def test_halo_parts_per_root_match_oracle(ctx, tuning):
    """Per-root counts (the reference's g_sum) of halo parts, through the
    halo-part instance's two phase kernels under tunings that send the work to
    heavy units, to warps only, to the bitmap kernel or to sorted lists: each
    part's per-root array equals the oracle's, its total equals the plain
    count, and a batch of the parts agrees."""
    old = ctx.get_tuning()
    try:
        ctx.set_tuning(**tuning)
        src, dst = gen.rmat(13)
        rp, col = oracle.clean(src, dst)
        deg = np.diff(rp)
        whole = oracle.count(*oracle.orient(rp, col))
        part = gen.parts_random(len(rp) - 1, 4)
        ug = ctx.upload_ugraph(rp, col, deg)
        for mode in ("reference", "count"):
            parts = ctx.halo_extract(ug, part, 4, mode=mode)
            total = 0
            for p, g in enumerate(parts):
                lrp, lcol, t_ver = oracle.halo_part(rp, col, deg, part, p, mode=mode)
                want, want_pr = oracle.count(lrp, lcol, n_roots=t_ver, per_root=True)
                got_pr = ctx.count_per_root(g)
                assert len(got_pr) == t_ver and np.array_equal(got_pr, want_pr), (mode, p)
                assert ctx.count(g) == want == int(got_pr.sum())
                total += want
            assert total == whole
            assert list(ctx.batch(parts).run()) == [int(ctx.count(g)) for g in parts]
    finally:
        ctx.set_tuning(**old)
