"""Device preprocessing (clean-up, orientation) against the oracle, exact arrays."""
import glob
import os

import numpy as np
import pytest

import families
import oracle
from trianglecount_gb300 import generators as gen

pytestmark = pytest.mark.gpu


def inputs():
    yield "rmat12", gen.rmat(12), 0
    yield "rmat17", gen.rmat(17), 0
    yield "road", gen.road(120), 0
    yield "er", gen.er(20000, 20.0, seed=5), 0
    yield "chung_lu", gen.chung_lu(50000, 12.0, seed=6), 0
    s, d, n = families.messy_complete(150)
    yield "messy", (s, d), n
    yield "selfloops_only", (np.arange(10, dtype=np.int64), np.arange(10, dtype=np.int64)), 0
    yield "empty", (np.empty(0, np.int64), np.empty(0, np.int64)), 5
    yield "isolated_hint", (np.array([3, 4], np.int64), np.array([4, 9], np.int64)), 40


@pytest.mark.parametrize("name,edges,n", list(inputs()), ids=[x[0] for x in inputs()])
def test_clean_matches_oracle(ctx, name, edges, n):
    src, dst = edges
    rp, col = oracle.clean(src, dst, n)
    ug = ctx.ugraph_from_edges(src, dst, n)
    grp, gcol, gdeg = ug.download()
    assert np.array_equal(grp, rp) and np.array_equal(gcol, col)
    assert np.array_equal(gdeg, np.diff(rp))
    for tie in ("reference", "id_asc"):
        orp, ocl = oracle.orient(rp, col, tie)
        g = ctx.orient(ug, tie)
        drp, dcol = g.download()
        assert np.array_equal(drp, orp) and np.array_equal(dcol, ocl), tie
        assert ctx.count(g) == oracle.count(orp, ocl)


def test_orientation_matches_reference_goldens(ctx, golden_dir):
    for f in sorted(glob.glob(os.path.join(golden_dir, "undir2dir_*.npz"))):
        z = np.load(f)
        ug = ctx.upload_ugraph(z["row_ptr"], z["col"])
        drp, dcol = ctx.orient(ug, "reference").download()
        assert np.array_equal(drp, z["oriented_row_ptr"]) and np.array_equal(dcol, z["oriented_col"]), f


def test_upload_ugraph_roundtrip(ctx):
    src, dst = gen.rmat(11)
    rp, col = oracle.clean(src, dst)
    deg = np.diff(rp)
    ug = ctx.upload_ugraph(rp, col, deg)
    r2, c2, d2 = ug.download()
    assert np.array_equal(r2, rp) and np.array_equal(c2, col) and np.array_equal(d2, deg)


def test_upload_ugraph_rejects_asymmetric_and_self_loops(ctx):
    """An undirected CSR lists every edge in both rows and has no self-loop;
    the halo extraction reads each edge from either end."""
    import trianglecount_gb300 as tc
    missing = (np.array([0, 2, 3, 3], np.int64), np.array([1, 2, 0], np.int64))  # 0-2 absent from row 2
    loop = (np.array([0, 2, 3, 5], np.int64), np.array([1, 2, 0, 0, 2], np.int64))  # self-loop 2-2
    for rp, col in (missing, loop):
        with pytest.raises(tc.TCError) as e:
            ctx.upload_ugraph(rp, col)
        assert e.value.code == "TC_E_INVALID"
    ug = ctx.upload_ugraph(np.array([0, 2, 3, 4], np.int64), np.array([1, 2, 0, 0], np.int64))  # 0-1, 0-2
    assert ug.info() == (3, 4)


@pytest.mark.parametrize("n", [1024, 2048, 1023, 1025, 3])
@pytest.mark.parametrize("tie", ["reference", "id_asc"])
def test_orientation_on_tile_boundaries(ctx, n, tie):
    """Circulant graphs C_n(1, 2) have 4n undirected entries: n = 1024 and
    2048 fill exactly one and two 4096-entry tiles, 1023 / 1025 stop just
    short of / just past one, and n = 3 (a triangle, 6 entries) is one
    partial warp; all vertices have the same degree, so the tie rule decides
    every edge."""
    i = np.arange(n, dtype=np.int64)
    src = np.concatenate([i, i])
    dst = np.concatenate([(i + 1) % n, (i + 2) % n])
    rp, col = oracle.clean(src, dst)
    ug = ctx.upload_ugraph(rp, col)
    orp, ocl = oracle.orient(rp, col, tie)
    drp, dcol = ctx.orient(ug, tie).download()
    assert np.array_equal(drp, orp) and np.array_equal(dcol, ocl)
    assert oracle.count(orp, ocl) == (1 if n == 3 else n)
