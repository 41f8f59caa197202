"""Batched persistent counting (one launch, CUDA-graph replay) against the
per-graph launch path and the oracle."""
import numpy as np
import pytest

import oracle
from trianglecount_gb300 import generators as gen

pytestmark = pytest.mark.gpu


def test_uneven_batch_matches_per_graph_and_oracle(ctx):
    specs = gen.batch_mix(48, scale=0.05)
    graphs, want = [], []
    for s in specs:
        src, dst = s.edges()
        orp, ocl, t = oracle.pipeline(src, dst)
        graphs.append(ctx.upload(orp, ocl))
        want.append(t)
    b = ctx.batch(graphs)
    for _ in range(3):  # graph replays give the same answer
        assert list(b.run()) == want
    assert list(ctx.count_each(graphs)) == want


def test_batch_async_and_single(ctx):
    src, dst = gen.rmat(13)
    orp, ocl, t = oracle.pipeline(src, dst)
    g = ctx.upload(orp, ocl)
    b = ctx.batch([g])
    b.run_async()
    assert list(b.results()) == [t]
    # the same graph several times in one batch
    assert list(ctx.batch([g, g, g]).run()) == [t, t, t]


def test_batch_mixes_degenerate_and_bounded_degree_graphs(ctx):
    """One batch holding an empty graph, an edgeless one, a single triangle, a
    halo-style graph (roots a prefix of the rows), a road grid (counted by the
    flat kernel on its own, by the chain inside a batch) and R-MAT graphs:
    every per-graph result equals its own plain count and the oracle."""
    cases = [(np.zeros(1, np.int32), np.zeros(0, np.int32), None),
             (np.zeros(7, np.int32), np.zeros(0, np.int32), None),
             (np.array([0, 2, 3, 3], np.int32), np.array([1, 2, 2], np.int32), None)]
    rp, col, _ = oracle.pipeline(*gen.rmat(11))
    cases.append((rp, col, len(rp) // 3))
    for src, dst in (gen.road(120), gen.rmat(12), gen.rmat(9)):
        rp, col, _ = oracle.pipeline(src, dst)
        cases.append((rp, col, None))
    graphs = [ctx.upload(rp, col, n_roots=nr) for rp, col, nr in cases]
    want = [oracle.count(rp, col, n_roots=nr) if nr is not None else oracle.count(rp, col)
            for rp, col, nr in cases]
    assert list(ctx.count_each(graphs)) == want
    b = ctx.batch(graphs)
    for _ in range(2):
        assert list(b.run()) == want
    b.free()


def test_batch_stats_and_parts_from_host(ctx):
    """tc_batch_stats times the replay's counting kernels; tc_count_parts_csr_i32
    counts halo parts from host arrays in one launch, exactly as the oracle."""
    src, dst = gen.rmat(13)
    rp, col = oracle.clean(src, dst)
    whole = oracle.count(*oracle.orient(rp, col))
    part = gen.parts_random(len(rp) - 1, 4)
    host = [oracle.halo_part(rp, col, np.diff(rp), part, p, mode="count") for p in range(4)]
    want = [oracle.count(lrp, lcol, n_roots=t) for lrp, lcol, t in host]
    got = ctx.count_parts_csr([(lrp.astype(np.int32), lcol.astype(np.int32), t) for lrp, lcol, t in host])
    assert list(got) == want and sum(want) == whole
    graphs = [ctx.upload(lrp, lcol, n_roots=t) for lrp, lcol, t in host]
    b = ctx.batch(graphs)
    st0 = b.stats()
    assert st0["launches"] > 0 and st0["count_kernel_ms"] == 0.0
    assert list(b.run()) == want
    st = b.stats()
    assert st["count_kernel_ms"] > 0.0 and st["launches"] == st0["launches"]
    b.free()


def test_parts_from_host_rejects_a_bad_part(ctx):
    import trianglecount_gb300 as tc
    rp = np.array([0, 2, 3, 3], np.int32)
    bad = np.array([2, 1, 2], np.int32)  # row 0 not ascending
    with pytest.raises(tc.TCError) as e:
        ctx.count_parts_csr([(rp, np.array([1, 2, 2], np.int32), 3), (rp, bad, 3)])
    assert e.value.code == "TC_E_FORMAT"


def test_parts_from_host_overlapped_uploads(ctx):
    """Large parts (over 4 M entries each) take the overlapped path: every
    upload goes out at once and each part is counted as soon as it is in and
    validated.  Counts equal the batched launch's and sum to the whole graph;
    a corrupt large part is still refused with TC_E_FORMAT."""
    import trianglecount_gb300 as tc
    src, dst = gen.rmat(20)
    ug = ctx.ugraph_from_edges(src, dst)
    whole = ctx.count(ctx.orient(ug))
    parts = ctx.halo_extract(ug, gen.parts_random(ug.info()[0], 2), 2, mode="count")
    host = [(*p.download(), p.n_roots) for p in parts]
    assert min(len(h[1]) for h in host) >= (1 << 22)
    want = [int(x) for x in ctx.batch(parts).run()]
    for _ in range(2):
        assert [int(x) for x in ctx.count_parts_csr(host)] == want
    assert sum(want) == whole
    rp1, col1, r1 = host[1]
    bad = col1.copy()
    bad[len(bad) // 2] = len(rp1) + 5  # an id out of range
    with pytest.raises(tc.TCError) as e:
        ctx.count_parts_csr([host[0], (rp1, bad, r1)])
    assert e.value.code == "TC_E_FORMAT"
    assert [int(x) for x in ctx.count_parts_csr(host)] == want  # the context is still usable


def test_batch_over_int32_pooled_edges_is_refused(ctx):
    """A launch pools its graphs' in-list offsets as int32: one graph listed
    often enough to pass 2^31 - 1 oriented edges in total is refused with
    TC_E_RANGE before anything is allocated, and the context stays usable."""
    import trianglecount_gb300 as tc
    src, dst = gen.rmat(18)
    orp, ocl, t = oracle.pipeline(src, dst)
    g = ctx.upload(orp, ocl)
    n = (1 << 31) // g.nnz + 1
    with pytest.raises(tc.TCError) as e:
        ctx.batch([g] * n)
    assert e.value.code == "TC_E_RANGE"
    assert list(ctx.batch([g] * 3).run()) == [t, t, t]


def test_parts_from_host_grouped_launches(ctx):
    """Five large parts take the overlapped path in groups [0], [1, 2],
    [3, 4] (sizes 1, 2, 4, ..., the last taking the rest): part 0 is counted
    on its own, the later groups in one pooled launch each.  Counts
    equal the batched launch's part by part and sum to the whole graph; a
    corrupt part inside a pooled group is refused with TC_E_FORMAT after
    part 0's count was already enqueued, and the context stays usable."""
    import trianglecount_gb300 as tc
    src, dst = gen.rmat(21)
    ug = ctx.ugraph_from_edges(src, dst)
    whole = ctx.count(ctx.orient(ug))
    parts = ctx.halo_extract(ug, gen.parts_random(ug.info()[0], 5), 5, mode="count")
    host = [(*p.download(), p.n_roots) for p in parts]
    assert sum(len(h[1]) for h in host) // len(host) >= (1 << 22)
    want = [int(x) for x in ctx.batch(parts).run()]
    for _ in range(2):
        assert [int(x) for x in ctx.count_parts_csr(host)] == want
    assert sum(want) == whole
    for k in (3, 4):  # three parts: groups [0], [1, 2]; four: [0], [1, 2, 3]
        assert [int(x) for x in ctx.count_parts_csr(host[:k])] == want[:k]
    rp2, col2, r2 = host[2]
    bad = col2.copy()
    bad[len(bad) // 3] = -1  # an id out of range inside the second group
    with pytest.raises(tc.TCError) as e:
        ctx.count_parts_csr(host[:2] + [(rp2, bad, r2)] + host[3:])
    assert e.value.code == "TC_E_FORMAT"
    assert [int(x) for x in ctx.count_parts_csr(host)] == want
