"""GPU counting kernels against the oracle and closed-form counts (bit-exact)."""
import json
import os

import numpy as np
import pytest

import families
import oracle
import trianglecount_gb300 as tc
from trianglecount_gb300 import generators as gen

pytestmark = pytest.mark.gpu

TUNINGS = [
    {},  # defaults (cuckoo hash)
    {"warp_max_deg": 32, "light_max_work": 1, "unit_work": 1, "long_list": 0},  # heavy path everywhere, 32-v slices
    {"warp_max_deg": 512, "light_max_work": 1 << 30, "unit_work": 1 << 30, "long_list": 4096,
     "probe_kicks": 0},  # warps only, flattened, linear probing
    {"warp_max_deg": 64, "light_max_work": 500, "unit_work": 3000, "long_list": 5, "blocks_per_sm": 1},
    {"probe_kicks": 1, "heavy_bitmap": 0},  # cuckoo give-ups: exercises the linear-probing fallback
    {"heavy_bitmap": 0, "warp_max_deg": 32, "light_max_work": 64},  # heavy work on shared hash tiles
    {"heavy_bitmap": 1, "warp_max_deg": 32, "light_max_work": 64},  # heavy work on the id bitmap kernel
    {"heavy_bitmap": 1},
    {"hash_pairs": 1},  # bucketed-pair tables, light and heavy
    {"flat_max_deg": 0},  # bounded-degree graphs through the full chain too
    {"hash_pairs": 1, "warp_max_deg": 32, "light_max_work": 64, "long_list": 5},
    {"intersect": 1},  # every task on its bulk-staged sorted list (binary search)
    {"intersect": 1, "warp_max_deg": 32, "light_max_work": 64, "long_list": 0},  # sorted heavy tiles, streamed lists
    {"intersect": 1, "warp_max_deg": 512, "light_max_work": 1 << 30, "unit_work": 1 << 30, "long_list": 4096},
    {"intersect": 2},  # per light task: sorted list when its work is below its length
    {"intersect": 2, "warp_max_deg": 512, "light_max_work": 1 << 30, "long_list": 5},
    {"intersect": 1, "hash_pairs": 1},  # pair tables ignore intersect
]


@pytest.fixture
def tuned(ctx):
    old = ctx.get_tuning()
    yield ctx
    ctx.set_tuning(old["warp_max_deg"], old["light_max_work"], old["unit_work"], old["long_list"],
                   old["probe_kicks"], old["heavy_bitmap"], 0, old["hash_pairs"], old["flat_max_deg"],
                   old["intersect"])


@pytest.mark.parametrize("tuning", TUNINGS)
def test_known_graphs(tuned, golden_dir, tuning):
    tuned.set_tuning(**tuning)
    for c in json.load(open(os.path.join(golden_dir, "known_graphs.json"))):
        src, dst, n = families.build(c["family"], c["args"])
        orp, ocl, _ = oracle.pipeline(src, dst, n)
        g = tuned.upload(orp, ocl)
        assert tuned.count(g) == c["expected"], (c["family"], c["args"], tuning)


@pytest.mark.parametrize("tuning", TUNINGS)
@pytest.mark.parametrize("scale", [8, 11, 14])
def test_rmat_per_root_matches_oracle(tuned, tuning, scale):
    tuned.set_tuning(**tuning)
    src, dst = gen.rmat(scale)
    orp, ocl, want = oracle.pipeline(src, dst)
    _, want_pr = oracle.count(orp, ocl, per_root=True)
    g = tuned.upload(orp, ocl)
    got_pr = tuned.count_per_root(g)
    assert np.array_equal(got_pr, want_pr)
    assert tuned.count(g) == want


@pytest.mark.parametrize("tie", ["reference", "id_asc"])
@pytest.mark.parametrize("maker", ["rmat16", "road", "er", "chung_lu", "complete_1500"])
def test_graph_families_match_oracle(ctx, maker, tie):
    if maker == "rmat16":
        src, dst = gen.rmat(16)
    elif maker == "road":
        src, dst = gen.road(300)
    elif maker == "er":
        src, dst = gen.er(50000, 40.0, seed=9)
    elif maker == "chung_lu":
        src, dst = gen.chung_lu(200000, 16.0, seed=10)
    else:
        src, dst, _ = families.complete(1500)
    orp, ocl, want = oracle.pipeline(src, dst, tie=tie)
    g = ctx.upload(orp, ocl)
    got, st = ctx.count(g, stats=True)
    assert got == want
    assert st["launches"] >= 1 and st["count_ms"] > 0


def test_rmat_golden_counts_on_device(ctx, golden_dir):
    for c in json.load(open(os.path.join(golden_dir, "rmat_counts.json"))):
        src, dst = gen.rmat(c["scale"], 16, seed=c["seed"])
        g = ctx.graph_from_edges(src, dst)
        assert (g.n_rows, g.nnz) == (c["V"], c["oriented_nnz"])
        assert ctx.count(g) == c["triangles"]


def test_halo_style_roots_subset(ctx):
    """n_roots < n_rows: only rows [0, n_roots) are roots (wo_sort_tc_256's t_ver)."""
    src, dst = gen.rmat(12)
    orp, ocl, _ = oracle.pipeline(src, dst)
    for nr in (0, 1, 100, len(orp) // 2, len(orp) - 1):
        g = ctx.upload(orp, ocl, n_roots=nr)
        assert ctx.count(g) == oracle.count(orp, ocl, n_roots=nr)


def test_edge_cases(ctx):
    # no vertices
    g = ctx.upload(np.zeros(1, np.int32), np.zeros(0, np.int32))
    assert ctx.count(g) == 0
    assert len(ctx.count_per_root(g)) == 0
    # vertices, no edges
    g = ctx.upload(np.zeros(6, np.int32), np.zeros(0, np.int32))
    assert ctx.count(g) == 0
    # one triangle 0->1, 0->2, 1->2
    g = ctx.upload(np.array([0, 2, 3, 3], np.int32), np.array([1, 2, 2], np.int32))
    assert ctx.count(g) == 1 and list(ctx.count_per_root(g)) == [1, 0, 0]
    # u64 upload path (the partitioned file's integer width)
    g = ctx.upload(np.array([0, 2, 3, 3], np.uint64), np.array([1, 2, 2], np.uint64))
    assert ctx.count(g) == 1


def test_invalid_csr_is_rejected(ctx):
    bad_order = (np.array([0, 2, 3, 3], np.int32), np.array([2, 1, 2], np.int32))
    bad_dup = (np.array([0, 2, 3, 3], np.int32), np.array([1, 1, 2], np.int32))
    bad_id = (np.array([0, 2, 3, 3], np.int32), np.array([1, 7, 2], np.int32))
    bad_rp = (np.array([0, 3, 2, 3], np.int32), np.array([1, 2, 2], np.int32))
    for rp, col in (bad_order, bad_dup, bad_id, bad_rp):
        with pytest.raises(tc.TCError) as e:
            ctx.upload(rp, col)
        assert e.value.code == "TC_E_FORMAT"
    with pytest.raises(tc.TCError) as e:
        ctx.upload(np.array([0, 1, 1], np.uint64), np.array([2**33], np.uint64))
    assert e.value.code == "TC_E_RANGE"
    with pytest.raises(tc.TCError):
        ctx.set_tuning(warp_max_deg=100)


def test_end_to_end_host_csr_and_repeatability(ctx):
    src, dst = gen.rmat(15)
    orp, ocl, want = oracle.pipeline(src, dst)
    assert ctx.count_csr(orp, ocl) == want
    g = ctx.upload(orp, ocl)
    assert {ctx.count(g) for _ in range(5)} == {want}


def test_context_outlives_its_graphs():
    """Closing a context while graphs / batches are alive defers its release
    until the last of them is freed (reference counting in the C ABI)."""
    src, dst = gen.rmat(10)
    orp, ocl, want = oracle.pipeline(src, dst)
    c = tc.Context(0)
    g = c.upload(orp, ocl)
    b = c.batch([g])
    c.close()
    assert list(b.run()) == [want]
    assert g.count() == want
    b.free()
    g.free()


def _bounded_degree_cases():
    """Graphs whose oriented rows are all at most 8 long (the flat count)."""
    yield "road300", gen.road(300)
    yield "road_tall", gen.road(64, height=900)
    s, d, _ = families.complete(5)  # out-degrees 4..0: 4-wide variant
    yield "K5", (s, d)
    s, d, _ = families.complete(9)  # out-degrees 8..0: 8-wide variant
    yield "K9", (s, d)
    yield "er_sparse", gen.er(20000, 2.5, seed=21)
    yield "er_deg6", gen.er(3000, 6.0, seed=5)  # out-degrees up to 7: 8-wide variant
    yield "road_full", gen.road()  # 2.1 M vertices; out-degree 5 under the id tie


@pytest.mark.parametrize("tie", ["reference", "id_asc"])
def test_flat_count_matches_chain_and_oracle(tuned, tie):
    for name, (src, dst) in _bounded_degree_cases():
        orp, ocl, want = oracle.pipeline(src, dst, tie=tie)
        assert np.diff(orp).max() <= 8, name
        _, want_pr = oracle.count(orp, ocl, per_root=True)
        g = tuned.upload(orp, ocl)
        tuned.set_tuning(flat_max_deg=8)
        got, st = tuned.count(g, stats=True)
        assert got == want and st["launches"] == 1, name
        assert np.array_equal(tuned.count_per_root(g), want_pr), name
        tuned.set_tuning(flat_max_deg=0)  # the same graph through the full chain
        got, st = tuned.count(g, stats=True)
        assert got == want and st["launches"] >= 4, name
        assert np.array_equal(tuned.count_per_root(g), want_pr), name
        tuned.set_tuning(flat_max_deg=8)


def test_flat_count_roots_subset_and_device_built(tuned):
    src, dst = gen.road(200)
    orp, ocl, _ = oracle.pipeline(src, dst)
    for nr in (0, 1, 777, len(orp) // 2, len(orp) - 1):
        g = tuned.upload(orp, ocl, n_roots=nr)
        assert tuned.count(g) == oracle.count(orp, ocl, n_roots=nr)
    g = tuned.graph_from_edges(src, dst)  # oriented on the device: the row bound is known too
    got, st = tuned.count(g, stats=True)
    assert got == oracle.count(orp, ocl) and st["launches"] == 1


def test_flat_count_not_used_above_the_bound(tuned):
    src, dst, _ = families.complete(10)  # out-degree 9 somewhere
    orp, ocl, want = oracle.pipeline(src, dst)
    got, st = tuned.count(tuned.upload(orp, ocl), stats=True)
    assert got == want and st["launches"] >= 4
    with pytest.raises(tc.TCError):
        tuned.set_tuning(flat_max_deg=9)


def test_repeated_counts_replay_a_captured_chain():
    """From its second count a graph replays its count chain as a captured
    CUDA graph: every replay gives the oracle's count and times the count
    kernel; results pointers that change every call are counted directly, a
    pointer used twice in a row or a tuning change re-captures, and per-root
    counts (never captured) still agree."""
    import torch
    c = tc.Context(0)  # its own context: the tuning changes below stay here
    rp, col, want = oracle.pipeline(*gen.rmat(12))
    g = c.upload(rp, col)
    launches = set()
    for _ in range(4):
        n, st = c.count(g, stats=True)
        assert n == want
        launches.add(st["launches"])
        assert c.last_count_kernel_ms() > 0
    assert len(launches) == 1  # a replay reports the captured chain's launches
    lib = tc.lib()
    outs = [torch.zeros(1, dtype=torch.int64, device="cuda") for _ in range(2)]
    torch.cuda.synchronize()
    for _ in range(2):
        for o in outs:  # a pointer that changes every call: direct launches
            assert lib.tc_count_async(c.handle, g.handle, o.data_ptr()) == 0
    c.synchronize()
    assert [int(o.item()) for o in outs] == [want, want]
    for _ in range(3):  # the same pointer twice in a row: captured, then replayed
        outs[0].zero_()
        torch.cuda.synchronize()
        assert lib.tc_count_async(c.handle, g.handle, outs[0].data_ptr()) == 0
        c.synchronize()
        assert int(outs[0].item()) == want
    c.set_tuning(light_max_work=512)
    assert c.count(g) == c.count(g) == want
    assert int(c.count_per_root(g).sum()) == want == c.count(g)
    g.free()
    c.close()


def test_repeated_counts_on_the_default_stream_and_under_a_caller_capture():
    """The legacy default stream cannot be captured, so repeated counts there
    launch the chain directly; a caller's own stream capture takes the chain's
    kernels into the caller's graph (the library starts no capture of its own)."""
    import torch
    rp, col, want = oracle.pipeline(*gen.rmat(12))
    c = tc.Context(0)
    g = c.upload(rp, col)
    c.set_stream(0)
    assert [c.count(g) for _ in range(3)] == [want] * 3
    s = torch.cuda.Stream()
    c.set_stream(s.cuda_stream)
    assert c.count(g) == want
    out = torch.zeros(1, dtype=torch.int64, device="cuda")
    torch.cuda.synchronize()
    cg = torch.cuda.CUDAGraph()
    with torch.cuda.graph(cg, stream=s):
        assert tc.lib().tc_count_async(c.handle, g.handle, out.data_ptr()) == 0
    for _ in range(2):
        out.zero_()
        torch.cuda.synchronize()
        cg.replay()
        torch.cuda.synchronize()
        assert int(out.item()) == want
    g.free()
    c.close()


@pytest.mark.parametrize("intersect", [1, 2])
def test_sorted_lists_on_a_misaligned_wrapped_graph(tuned, intersect):
    """Wrapped caller arrays need not be 16-byte aligned: the bulk copy is
    then skipped and the lists are staged by plain loads; counts and per-root
    counts stay exact."""
    torch = pytest.importorskip("torch")
    tuned.set_tuning(intersect=intersect, warp_max_deg=64, light_max_work=256)
    src, dst = gen.chung_lu(30000, 14.0, seed=5)
    orp, ocl, want = oracle.pipeline(src, dst)
    d_rp = torch.from_numpy(orp).cuda()
    buf = torch.zeros(len(ocl) + 1, dtype=torch.int32, device="cuda")
    buf[1:] = torch.from_numpy(ocl).cuda()  # col starts 4 bytes past an aligned base
    g = tuned.wrap_device(d_rp.data_ptr(), buf.data_ptr() + 4, len(orp) - 1, len(ocl))
    assert tuned.count(g) == want
    _, want_pr = oracle.count(orp, ocl, per_root=True)
    assert np.array_equal(tuned.count_per_root(g), want_pr)
