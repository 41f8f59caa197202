"""The CPU oracle against closed-form counts, an independent brute-force
counter, networkx, and the reference's own CPU orientation tool."""
import glob
import json
import os
import subprocess

import numpy as np
import pytest

import families
import oracle
from trianglecount_gb300 import generators as gen


def test_known_graphs(golden_dir):
    cases = json.load(open(os.path.join(golden_dir, "known_graphs.json")))
    assert len(cases) >= 20
    for c in cases:
        src, dst, n = families.build(c["family"], c["args"])
        _, _, t = oracle.pipeline(src, dst, n)
        assert t == c["expected"], (c["family"], c["args"])


@pytest.mark.parametrize("maker", ["rmat10", "rmat12", "road", "er", "cl"])
def test_count_matches_brute_force_and_networkx(maker):
    nx = pytest.importorskip("networkx")
    if maker.startswith("rmat"):
        src, dst = gen.rmat(int(maker[4:]))
    elif maker == "road":
        src, dst = gen.road(60)
    elif maker == "er":
        src, dst = gen.er(3000, 12.0, seed=3)
    else:
        src, dst = gen.chung_lu(5000, 10.0, seed=4)
    rp, col = oracle.clean(src, dst)
    orp, ocl = oracle.orient(rp, col)
    t = oracle.count(orp, ocl)
    assert t == oracle.count_brute(rp, col)
    G = nx.Graph()
    G.add_edges_from(zip(src.tolist(), dst.tolist()))
    G.remove_edges_from(list(nx.selfloop_edges(G)))
    assert t == sum(nx.triangles(G).values()) // 3


def test_tie_breaks_orient_each_edge_once():
    src, dst = gen.rmat(12)
    rp, col = oracle.clean(src, dst)
    counts = set()
    for tie in ("reference", "id_asc"):
        orp, ocl = oracle.orient(rp, col, tie)
        assert len(ocl) * 2 == len(col)
        counts.add(oracle.count(orp, ocl))
        # per-root sums equal the total
        t, pr = oracle.count(orp, ocl, per_root=True)
        assert int(pr.sum()) == t
    assert len(counts) == 1


def test_orientation_matches_reference_undir2dir_goldens(golden_dir):
    files = sorted(glob.glob(os.path.join(golden_dir, "undir2dir_*.npz")))
    assert files, "golden orientation vectors missing"
    for f in files:
        z = np.load(f)
        orp, ocl = oracle.orient(z["row_ptr"], z["col"], "reference")
        assert np.array_equal(orp, z["oriented_row_ptr"]), f
        assert np.array_equal(ocl, z["oriented_col"]), f


@pytest.mark.skipif(not os.path.exists(oracle.UNDIR2DIR), reason="reference tool not built here")
def test_orientation_matches_reference_undir2dir_live(tmp_path):
    src, dst = gen.er(2000, 9.0, seed=11)
    rp, col = oracle.clean(src, dst)
    V, deg = len(rp) - 1, np.diff(rp)
    inp, outp = tmp_path / "in.txt", tmp_path / "out.txt"
    with open(inp, "w") as f:
        f.write(f"{V}\n" + " ".join(map(str, deg)) + f"\n{V} {V + 1} {len(col)} {V}\n")
        f.write(" ".join(map(str, range(V))) + "\n" + " ".join(map(str, rp)) + "\n" + " ".join(map(str, col)) + "\n")
    subprocess.run([oracle.UNDIR2DIR, str(inp), str(outp), "1"], check=True, capture_output=True)
    vals = np.array(open(outp).read().split(), np.int64)
    rps, m = vals[1], vals[2]
    orp, ocl = oracle.orient(rp, col)
    assert np.array_equal(orp, vals[3:3 + rps]) and np.array_equal(ocl, vals[3 + rps:3 + rps + m])


def test_rmat_golden_counts(golden_dir):
    for c in json.load(open(os.path.join(golden_dir, "rmat_counts.json"))):
        src, dst = gen.rmat(c["scale"], 16, seed=c["seed"])
        assert int((src * 1000003 + dst).sum() % (1 << 61)) == c["edge_checksum"]
        rp, col = oracle.clean(src, dst)
        orp, ocl = oracle.orient(rp, col)
        assert (len(rp) - 1, len(col), len(ocl)) == (c["V"], c["undirected_nnz"], c["oriented_nnz"])
        assert oracle.count(orp, ocl) == c["triangles"]


def test_count_invariant_under_relabelling():
    src, dst = gen.rmat(11)
    t0 = oracle.pipeline(src, dst)[2]
    perm = np.random.default_rng(5).permutation(int(max(src.max(), dst.max())) + 1)
    assert oracle.pipeline(perm[src], perm[dst])[2] == t0


@pytest.mark.parametrize("k", [2, 4, 8])
def test_halo_parts_sum_to_whole(k):
    src, dst = gen.rmat(12)
    rp, col = oracle.clean(src, dst)
    deg = np.diff(rp)
    whole = oracle.count(*oracle.orient(rp, col))
    part = gen.parts_random(len(rp) - 1, k)
    total = 0
    for p in range(k):
        lrp, lcol, t_ver = oracle.halo_part(rp, col, deg, part, p)
        assert t_ver == int((part == p).sum())
        # every surviving halo vertex is pointed to by some edge (prune fixpoint)
        indeg = np.bincount(lcol, minlength=len(lrp) - 1)
        assert np.all(indeg[t_ver:] > 0)
        # rows ascending
        for u in range(0, len(lrp) - 1, 97):
            r = lcol[lrp[u]:lrp[u + 1]]
            assert np.all(np.diff(r) > 0)
        total += oracle.count(lrp, lcol, n_roots=t_ver)
    assert total == whole


@pytest.mark.parametrize("k", [2, 4, 8])
def test_counting_halo_parts_sum_to_whole_and_shrink(k):
    """The counting halo keeps the halo vertices with an oriented in-edge from
    the part: each part's count is unchanged, and the parts are subgraphs of
    the reference parts (fewer or equal rows and entries)."""
    src, dst = gen.chung_lu(20000, 10.0, seed=3)
    rp, col = oracle.clean(src, dst)
    deg = np.diff(rp)
    orp, ocl = oracle.orient(rp, col)
    whole = oracle.count(orp, ocl)
    part = gen.parts_random(len(rp) - 1, k)
    rows = np.repeat(np.arange(len(orp) - 1), np.diff(orp))
    total = 0
    for p in range(k):
        lrp, lcol, t_ver = oracle.halo_part(rp, col, deg, part, p, mode="count")
        rrp, rcol, rt = oracle.halo_part(rp, col, deg, part, p)
        assert t_ver == rt and len(lrp) <= len(rrp) and len(lcol) <= len(rcol)
        # the halo is exactly the oriented out-neighbours of the part outside it
        inP = part == p
        want_halo = np.unique(ocl[inP[rows] & ~inP[ocl]])
        assert len(lrp) - 1 == t_ver + len(want_halo)
        c = oracle.count(lrp, lcol, n_roots=t_ver)
        assert c == oracle.count(rrp, rcol, n_roots=rt)
        total += c
    assert total == whole


def test_planted_orientation_mistake_is_caught():
    """A non-strict orientation (keep u->w when degrees tie both ways) double
    counts; the known-answer check must notice."""
    src, dst, n = families.complete(12)
    rp, col = oracle.clean(src, dst, n)
    deg = np.diff(rp)
    keep = []
    for u in range(len(rp) - 1):
        keep.append([w for w in col[rp[u]:rp[u + 1]] if deg[u] <= deg[w]])
    orp = np.concatenate([[0], np.cumsum([len(k) for k in keep])])
    ocl = np.concatenate(keep).astype(np.int64)
    assert oracle.count(orp, ocl) != families.expected("complete", [12])


def test_fullsize_generators_are_pinned(golden_dir):
    """The benchmark-size inputs (R-MAT 21 / 23, road 1448 x 1448) are drawn
    with integer-only generators: their edge checksums match the committed
    ones on every platform, so the full-size golden counts apply."""
    full = json.load(open(os.path.join(golden_dir, "fullsize_counts.json")))
    for name, make in (("rmat21", lambda: gen.rmat(21, 16)), ("road", gen.road), ("rmat23", lambda: gen.rmat(23, 16))):
        src, dst = make()
        assert int((src * 1000003 + dst).sum() % (1 << 61)) == full[name]["edge_checksum"], name


def test_fscanf_reader_matches_parallel_parser(tmp_path):
    """The TC_128 driver's one-fscanf-per-integer reader (restated in the
    oracle) and the library's parallel text parser read the same .csr."""
    from trianglecount_gb300 import formats as F
    rp, col, _ = oracle.pipeline(*gen.rmat(11))
    p = tmp_path / "g_output.csr"
    F.write_csr(p, len(rp) - 1, 2 * len(col), rp, col)
    hdr, r1, c1 = oracle.read_csr_fscanf(p)
    fast = F.read_csr(p)
    assert list(hdr) == [len(rp) - 1, 2 * len(col), len(rp), len(col)] == [fast.V, fast.E, len(fast.row_ptr), len(fast.col)]
    assert np.array_equal(r1, rp) and np.array_equal(fast.row_ptr, rp)
    assert np.array_equal(c1, col) and np.array_equal(fast.col, col)
    p.write_text(p.read_text()[: len(p.read_text()) // 2])  # ends early
    with pytest.raises(OSError):
        oracle.read_csr_fscanf(p)


@pytest.mark.parametrize("scale, permute", [(10, True), (13, True), (12, False)])
def test_oracle_generators_match_the_library(scale, permute):
    """The reference arm of bench.py builds its input with the oracle's
    generators (no library loaded); they must give the library's bits."""
    s1, d1 = oracle.gen_rmat(scale, permute=permute)
    s2, d2 = gen.rmat(scale, permute=permute)
    assert np.array_equal(s1, s2) and np.array_equal(d1, d2)
    for k in (2, 8):
        assert np.array_equal(oracle.gen_parts_random(5000, k), gen.parts_random(5000, k))
