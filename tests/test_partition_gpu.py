"""Balanced label-propagation parts (the stand-in for the reference's METIS
assignment, dgl.metis_partition_assignment in Halo_creation_preprocess.py:304):
seeded determinism, balance, fewer cut edges than random parts, and exact
halo-part counts."""
import numpy as np
import pytest

import oracle
import trianglecount_gb300 as tc
from trianglecount_gb300 import generators as gen

pytestmark = pytest.mark.gpu


def cut_fraction(rp, col, part):
    rows = np.repeat(np.arange(len(rp) - 1), np.diff(rp))
    return float((part[rows] != part[col]).mean())


@pytest.mark.parametrize("maker", ["rmat13", "chung_lu", "road"])
@pytest.mark.parametrize("k", [2, 8])
def test_parts_are_balanced_deterministic_and_cut_less(ctx, maker, k):
    if maker == "rmat13":
        src, dst = gen.rmat(13)
    elif maker == "chung_lu":
        src, dst = gen.chung_lu(20000, 12.0, seed=5)
    else:
        src, dst = gen.road(100)
    rp, col = oracle.clean(src, dst)
    ug = ctx.upload_ugraph(rp, col)
    n = len(rp) - 1
    part = ctx.parts_lp(ug, k, seed=11)
    assert part.dtype == np.int32 and len(part) == n
    assert part.min() >= 0 and part.max() < k
    assert np.bincount(part, minlength=k).max() <= 1.05 * n / k
    assert np.array_equal(part, ctx.parts_lp(ug, k, seed=11))  # seeded: the same parts again
    assert cut_fraction(rp, col, part) < cut_fraction(rp, col, gen.parts_random(n, k)) - 0.03


@pytest.mark.parametrize("maker", ["rmat12", "road"])
def test_halo_parts_of_lp_assignment_sum_to_whole(ctx, maker):
    src, dst = gen.rmat(12) if maker == "rmat12" else gen.road(60)
    rp, col = oracle.clean(src, dst)
    deg = np.diff(rp)
    ug = ctx.upload_ugraph(rp, col, deg)
    k = 4
    part = ctx.parts_lp(ug, k)
    parts = ctx.halo_extract(ug, part, k)
    for p, g in enumerate(parts):
        lrp, lcol, t_ver = oracle.halo_part(rp, col, deg, part, p)
        drp, dcol = g.download()
        assert g.n_roots == t_ver and np.array_equal(drp, lrp) and np.array_equal(dcol, lcol)
    assert sum(ctx.count(g) for g in parts) == oracle.count(*oracle.orient(rp, col))


def test_one_part_and_bad_k(ctx):
    src, dst = gen.rmat(10)
    rp, col = oracle.clean(src, dst)
    ug = ctx.upload_ugraph(rp, col)
    assert not ctx.parts_lp(ug, 1).any()
    with pytest.raises(tc.TCError) as e:
        ctx.parts_lp(ug, 65)
    assert e.value.code == "TC_E_INVALID"
