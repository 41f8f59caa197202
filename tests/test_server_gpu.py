"""Serving loop: continuous batching over resident graphs.  Each result is
the same alone and in the mix (exact integers), resident graphs are reused
by key and evicted LRU under the budget, and the host-side watchdog turns an
over-long batch into TC_E_TIMEOUT without any device-side fault."""
import threading
import time

import numpy as np
import pytest

import oracle
import trianglecount_gb300 as tc
from trianglecount_gb300 import generators as gen

pytestmark = pytest.mark.gpu


def _graphs():
    out = [gen.rmat(s, seed=100 + s) for s in (10, 12, 14, 15)]
    out += [gen.chung_lu(20000, 10.0, seed=7), gen.er(5000, 20.0, seed=8), gen.road(80)]
    return out


def test_results_identical_alone_and_in_the_mix(ctx):
    gs = _graphs()
    alone = [ctx.count(ctx.graph_from_edges(s, d)) for s, d in gs]
    assert alone[0] == oracle.pipeline(*gs[0])[2]
    with tc.Server(ctx, max_batch=64) as srv:
        ids = [srv.submit(s, d, key=0) for s, d in gs for _ in range(3)]
        got = [srv.wait(i)[0] for i in ids]
        st = srv.stats()
    assert got == [a for a in alone for _ in range(3)]
    assert st["completed"] == len(ids) and st["failed"] == 0 and st["batches"] >= 1


def test_resident_reuse_and_lru_eviction(ctx):
    gs = _graphs()[:4]
    want = [ctx.count(ctx.graph_from_edges(s, d)) for s, d in gs]
    # a budget just above the build footprint of the largest graph (about 58
    # bytes per input edge), so residents must be evicted to build it again
    budget = 58 * max(len(s) for s, _ in gs) + (3 << 20)
    with tc.Server(ctx, hbm_budget_bytes=budget, max_batch=8) as srv:
        for rnd in range(3):
            for k, (s, d) in enumerate(gs):
                c, lat = srv.wait(srv.submit(s, d, key=k + 1))
                assert c == want[k] and lat > 0
        rid = srv.submit(key=4)  # most recently used: still resident, no edges needed
        assert srv.wait(rid)[0] == want[3]
        st = srv.stats()
    assert st["evictions"] > 0 and st["cache_hits"] >= 1 and st["used_bytes"] <= st["budget_bytes"]


def test_request_errors_and_concurrent_clients(ctx):
    s, d = gen.rmat(12)
    want = ctx.count(ctx.graph_from_edges(s, d))
    with tc.Server(ctx, hbm_budget_bytes=8 << 20) as srv:
        big = srv.submit(*gen.rmat(18), key=0)  # needs more than the whole budget
        with pytest.raises(tc.TCError) as e:
            srv.wait(big)
        assert e.value.code == "TC_E_NOMEM"
        with pytest.raises(tc.TCError) as e:
            srv.wait(srv.submit(key=12345))  # unknown key and no edges
        assert e.value.code == "TC_E_STATE"
        results, errs = [], []

        def client():
            try:
                for _ in range(5):
                    results.append(srv.wait(srv.submit(s, d))[0])
            except Exception as ex:  # reported below
                errs.append(ex)

        th = [threading.Thread(target=client) for _ in range(4)]
        [t.start() for t in th]
        [t.join() for t in th]
        assert not errs and results == [want] * 20


def test_batch_watchdog_reports_timeout(ctx):
    """A 1 ms limit on a batch that takes longer: the request fails with
    TC_E_TIMEOUT (the launch itself completes normally on the device) and the
    server stops admitting new work."""
    s, d = gen.rmat(21)  # a count of several milliseconds
    with tc.Server(ctx, batch_timeout_ms=1) as srv:
        with pytest.raises(tc.TCError) as e:
            srv.wait(srv.submit(s, d))
        assert e.value.code == "TC_E_TIMEOUT"
        with pytest.raises(tc.TCError) as e:
            srv.wait(srv.submit(*gen.rmat(8)))
        assert e.value.code == "TC_E_STATE"


def test_small_requests_overtake_a_large_one_in_flight(ctx):
    """An R-MAT 23 request (134 M edges, the large lane; its count alone takes
    ~35 ms) is submitted first; once its batch has been taken for counting,
    three small requests (the small lane) arrive.  They are built and counted
    beside the large batch on their own streams and complete before it; every
    result equals its solo count (the plain per-graph count)."""
    big = gen.rmat(23)
    smalls = [gen.rmat(9, seed=300 + i) for i in range(2)] + [gen.chung_lu(3000, 8.0, seed=9)]
    want_big = ctx.count(ctx.graph_from_edges(*big))
    want_small = [ctx.count(ctx.graph_from_edges(s, d)) for s, d in smalls]
    assert want_small[0] == oracle.pipeline(*smalls[0])[2]
    with tc.Server(ctx, max_batch=64) as srv:
        # warm both lanes (first-use set-up stays out of the race below)
        srv.wait(srv.submit(*smalls[0]))
        srv.wait(srv.submit(*gen.rmat(20)))
        rb = srv.submit(*big, key=77)
        # wait until the large lane has taken the big batch (its build is done)
        t_end = time.monotonic() + 60
        while srv.stats()["large_batches"] < 2 and time.monotonic() < t_end:
            time.sleep(0.0005)
        ids = [srv.submit(s, d) for s, d in smalls]
        order = []
        pending = set(ids + [rb])
        t_end = time.monotonic() + 60
        while pending and time.monotonic() < t_end:
            for rid in list(pending):
                r = srv.poll(rid)
                if r is not None:
                    order.append((rid, r[0]))
                    pending.discard(rid)
            time.sleep(0.0002)
        st = srv.stats()
    assert not pending
    got = dict(order)
    assert got[rb] == want_big and [got[i] for i in ids] == want_small
    big_pos = [rid for rid, _ in order].index(rb)
    assert all([rid for rid, _ in order].index(i) < big_pos for i in ids), order
    assert st["small_batches"] >= 2 and st["large_batches"] >= 2


def test_one_lane_when_small_edges_is_negative(ctx):
    gs = _graphs()[:3]
    alone = [ctx.count(ctx.graph_from_edges(s, d)) for s, d in gs]
    with tc.Server(ctx, small_edges=-1) as srv:
        got = [srv.wait(srv.submit(s, d))[0] for s, d in gs]
        st = srv.stats()
    assert got == alone and st["small_batches"] == 0 and st["large_batches"] >= 1


@pytest.mark.parametrize("staging", [-1, 4 << 20])
def test_staging_area_full_or_absent(ctx, staging):
    """Edge lists that do not fit the pinned staging area (a 4 MiB area, or
    none) are kept in pageable memory; results are the same either way, and
    the area's ranges are reused once builds release them."""
    gs = _graphs()
    alone = [ctx.count(ctx.graph_from_edges(s, d)) for s, d in gs]
    with tc.Server(ctx, staging_bytes=staging) as srv:
        for _ in range(2):
            ids = [srv.submit(s, d) for s, d in gs]
            assert [srv.wait(i)[0] for i in ids] == alone


def test_one_key_built_by_both_lanes_at_once(ctx):
    """The same key submitted with its edge list (small lane) and with that
    list repeated 40 times (over 2^20 edges: the large lane; the clean-up
    drops the repeats, so it is the same graph) builds in both lanes at once.
    Both count it exactly; one build becomes the resident graph, the other
    stays the request's own; a key-only request then counts the resident one."""
    s, d = gen.rmat(14)
    want = ctx.count(ctx.graph_from_edges(s, d))
    big_s, big_d = np.tile(s, 40), np.tile(d, 40)
    assert len(s) <= (1 << 20) < len(big_s)
    with tc.Server(ctx) as srv:
        for _ in range(3):
            ids = [srv.submit(big_s, big_d, key=99), srv.submit(s, d, key=99)]
            assert [srv.wait(i)[0] for i in ids] == [want, want]
            assert srv.wait(srv.submit(key=99))[0] == want
        st = srv.stats()
    assert st["failed"] == 0 and st["resident_graphs"] == 1
