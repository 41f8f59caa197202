"""Parity at the benchmark sizes: R-MAT scale 21 and the 1448 x 1448 road grid
(plain path, both counting paths), R-MAT scale 23 whole and in k = 2, 4, 8
random halo parts (sum of parts == whole, batched == per part), against the
CPU oracle's counts committed in tests/golden/fullsize_counts.json."""
import json
import os

import numpy as np
import pytest

import trianglecount_gb300 as tc
from trianglecount_gb300 import generators as gen

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def full(golden_dir):
    return json.load(open(os.path.join(golden_dir, "fullsize_counts.json")))


def test_rmat21_plain_per_root_and_batched(ctx, full):
    want = full["rmat21"]
    g = ctx.graph_from_edges(*gen.rmat(21, 16))
    assert (g.n_rows, g.nnz) == (want["V"], want["oriented_nnz"])
    assert ctx.count(g) == want["triangles"]
    pr = ctx.count_per_root(g)
    assert int(pr.sum()) == want["triangles"] and len(pr) == g.n_roots
    b = ctx.batch([g, g])
    assert list(b.run()) == [want["triangles"]] * 2
    b.free()


def test_road_flat_and_chain(ctx, full):
    want = full["road"]
    g = ctx.graph_from_edges(*gen.road())
    assert (g.n_rows, g.nnz) == (want["V"], want["oriented_nnz"])
    old = ctx.get_tuning()
    try:
        got, st = ctx.count(g, stats=True)
        assert got == want["triangles"] and st["launches"] == 1  # one flat kernel
        ctx.set_tuning(flat_max_deg=0)
        got, st = ctx.count(g, stats=True)
        assert got == want["triangles"] and st["launches"] >= 4  # the full chain
    finally:
        ctx.set_tuning(flat_max_deg=old["flat_max_deg"])


@pytest.mark.parametrize("mode", ["reference", "count"])
def test_rmat23_halo_parts_sum_to_whole(ctx, full, mode):
    """R-MAT 23's k = 2, 4, 8 parts, in the reference's halo and in the
    counting halo: per-part launches and the batched launch agree part by
    part and sum to the oracle's count of the whole graph; the counting
    parts are no larger and count the same per part."""
    want = full["rmat23"]
    ug = ctx.ugraph_from_edges(*gen.rmat(23, 16))
    og = ctx.orient(ug)
    assert (og.n_rows, og.nnz) == (want["V"], want["oriented_nnz"])
    assert ctx.count(og) == want["triangles"]
    for k in (2, 4, 8):
        part = gen.parts_random(og.n_rows, k)
        parts = ctx.halo_extract(ug, part, k, mode=mode)
        each = ctx.count_each(parts)
        assert int(each.sum()) == want["triangles"], k
        b = ctx.batch(parts)
        assert np.array_equal(b.run(), each), k
        b.free()
        if mode == "count":
            ref = ctx.halo_extract(ug, part, k)
            assert all(c.nnz <= r.nnz and c.n_roots == r.n_roots for c, r in zip(parts, ref)), k
            assert np.array_equal(ctx.count_each(ref), each), k
            for p in ref:
                p.free()
        for p in parts:
            p.free()


def test_host_csr_counts_and_rejects_at_full_size(ctx, full):
    """tc_count_csr_i32 on a full-size host CSR (upload, validation, count,
    read-back): the golden count, twice; an id out of range, a row out of
    order and a non-monotone row_ptr are rejected with TC_E_FORMAT, and the
    context stays usable."""
    want = full["rmat21"]["triangles"]
    rp, col = ctx.graph_from_edges(*gen.rmat(21, 16)).download()
    assert ctx.count_csr(rp, col) == want
    assert ctx.count_csr(rp, col) == want
    bad_id = col.copy()
    bad_id[len(col) // 2] = len(rp) + 5  # an id out of range in a middle stage
    bad_order = col.copy()
    r = int(np.searchsorted(rp, 7 * len(col) // 8))  # a row with two entries late in the array
    while rp[r + 1] - rp[r] < 2:
        r += 1
    bad_order[rp[r]], bad_order[rp[r] + 1] = bad_order[rp[r] + 1], bad_order[rp[r]]
    bad_rp = rp.copy()
    bad_rp[len(rp) // 3] = bad_rp[len(rp) // 3 + 1] + 5  # row_ptr not monotone
    for r_, c_ in ((rp, bad_id), (rp, bad_order), (bad_rp, col)):
        with pytest.raises(tc.TCError) as e:
            ctx.count_csr(r_, c_)
        assert e.value.code == "TC_E_FORMAT"
    assert ctx.count_csr(rp, col) == want
    g = ctx.graph_from_edges(*gen.road(1600))  # > 4 M entries, rows <= 8: the flat count from host arrays
    rp2, col2 = g.download()
    assert len(col2) >= (1 << 22)
    assert ctx.count_csr(rp2, col2) == ctx.count(g)
