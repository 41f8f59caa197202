"""Command-line drop-ins without a GPU: argv / missing-file behaviour of the
reference tools, and the edge-list formats tc_preprocess reads."""
import os
import subprocess

import numpy as np
import pytest

from trianglecount_gb300 import build as B
from trianglecount_gb300 import formats as F

BIN = B.BIN


def run(tool, *args, **kw):
    return subprocess.run([os.path.join(BIN, tool), *map(str, args)], capture_output=True, text=True, timeout=120,
                          **kw)


@pytest.fixture(scope="module", autouse=True)
def tools():
    B.build_libtc()
    for t in ("TC_128", "wo_sort_tc_256", "round_clean_sg", "tc_preprocess"):
        assert os.path.exists(os.path.join(BIN, t)), t


def test_missing_files_behave_like_the_reference(tmp_path):
    r = run("TC_128", tmp_path / "nope.csr")  # ShareKernelTCV62_update_v1.cu:200-203
    assert r.returncode == 0 and r.stdout == "file not opened\n"
    r = run("wo_sort_tc_256", tmp_path / "nope.csr", 2)  # without_sorting_tc.cu:234-238
    assert r.returncode == 0 and r.stdout == "\nFile Not Opened........."
    r = run("round_clean_sg", 2, tmp_path / "a", tmp_path / "b")
    assert r.returncode == 1 and "Error opening file" in r.stderr
    r = run("round_clean_sg", 2)
    assert r.returncode == 1 and "Usage" in r.stderr
    r = run("TC_128")
    assert r.returncode == 1 and "usage" in r.stderr


def test_truncated_inputs_are_rejected(tmp_path):
    p = tmp_path / "t.csr"
    p.write_text("3 6 4 3\n0 2 3\n")
    r = run("TC_128", p)
    assert r.returncode == 1 and "truncated" in r.stderr
    q = tmp_path / "parts.csr"
    q.write_text("3 6\n3 4 3 3\n0 2 3 3\n1 2 2\n")
    r = run("wo_sort_tc_256", q, 2)
    assert r.returncode == 1


def test_edge_list_formats(tmp_path):
    edges = [(1, 2), (2, 3), (3, 1), (5, 6)]
    tsv = tmp_path / "g.tsv"
    tsv.write_text("".join(f"{u}\t{v}\t1\n" for u, v in edges))
    txt = tmp_path / "g.txt"
    txt.write_text("# Directed graph\n# Nodes: 6 Edges: 4\n# FromNodeId\tToNodeId\n#\n" +
                   "".join(f"{u}\t{v}\n" for u, v in edges))
    mtx = tmp_path / "g.mtx"
    mtx.write_text("%%MatrixMarket matrix coordinate pattern general\n% c\n7 7 4\n" +
                   "".join(f"{u + 1} {v + 1}\n" for u, v in edges))
    for p in (tsv, txt, mtx):
        s, d = F.read_edges(p)
        assert list(zip(s.tolist(), d.tolist())) == edges, p
    sp = pytest.importorskip("scipy.io")
    import warnings
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        m = sp.mmread(str(mtx)).tocoo()
    assert sorted(zip(m.row.tolist(), m.col.tolist())) == sorted(edges)
    bad = tmp_path / "bad.tsv"
    bad.write_text("1\tx\n")
    with pytest.raises(Exception):
        F.read_edges(bad)
