"""The drop-in tools end to end on the GPU, chained as the reference's README
runs them: edge file -> tc_preprocess -> TC_128; _part.csr + node parts ->
round_clean_sg -> wo_sort_tc_256.  Files are compared with the reference's
layouts and stdout with the reference's format strings."""
import os
import re
import subprocess

import numpy as np
import pytest

import oracle
from trianglecount_gb300 import build as B
from trianglecount_gb300 import formats as F
from trianglecount_gb300 import generators as gen

pytestmark = pytest.mark.gpu
BIN = B.BIN

SEARCH = re.compile(r"\nSearch : (\d+\.\d{6}) sec Vertex : (\d+) Edge : (\d+) Triangle : (\d+)  "
                    r"Sum_result : (\d+\.\d{6}) Sec, total_time : (\d+\.\d{6}) Sec\n")


def run(tool, *args):
    r = subprocess.run([os.path.join(BIN, tool), *map(str, args)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    return r.stdout


@pytest.fixture(scope="module")
def prepared(tmp_path_factory):
    d = tmp_path_factory.mktemp("cli")
    src, dst = gen.rmat(13)
    edge_file = d / "rmat13.tsv"
    with open(edge_file, "w") as f:
        for u, v in zip(src.tolist(), dst.tolist()):
            f.write(f"{u}\t{v}\t1\n")
    run("tc_preprocess", edge_file, "--out-dir", d, "--parts", "2,4,8", "--tcsr")
    rp, col = oracle.clean(src, dst)
    orp, ocl = oracle.orient(rp, col)
    return d, src, dst, rp, col, orp, ocl


def test_preprocess_files_match_reference_layout(prepared, tmp_path):
    d, src, dst, rp, col, orp, ocl = prepared
    ref = tmp_path / "ref_output.csr"
    F.write_csr(ref, len(rp) - 1, len(col), orp, ocl)
    assert open(d / "rmat13_output.csr", "rb").read() == open(ref, "rb").read()
    refp = tmp_path / "ref_part.csr"
    F.write_part_csr(refp, rp, col, np.diff(rp))
    assert open(d / "rmat13_part.csr", "rb").read() == open(refp, "rb").read()
    for k in (2, 4, 8):
        part = F.read_node_parts(d / f"rmat13_part.csr_node_parts_random_{k}", len(rp) - 1)
        assert np.array_equal(part, gen.parts_random(len(rp) - 1, k))
        part = F.read_node_parts(d / f"rmat13_part.csr_node_parts_contig_{k}", len(rp) - 1)
        assert np.array_equal(part, gen.parts_contig(len(rp) - 1, k))
        part = F.read_node_parts(d / f"rmat13_part.csr_node_parts_lp_{k}", len(rp) - 1)
        assert part.min() >= 0 and part.max() < k and np.bincount(part).max() <= 1.05 * len(part) / k
    trp, tcol, nr, aux = F.read_tcsr(d / "rmat13.tcsr")
    assert np.array_equal(trp, orp) and np.array_equal(tcol, ocl) and aux == len(col)


def test_tc128_stdout_and_count(prepared):
    d, src, dst, rp, col, orp, ocl = prepared
    out = run("TC_128", d / "rmat13_output.csr")
    runs = SEARCH.findall(out)
    assert len(runs) == 3
    want = oracle.count(orp, ocl)
    for s, v, e, t, sr, tt in runs:
        assert (int(v), int(e), int(t)) == (len(rp) - 1, len(ocl), want)
    assert re.search(r"\nTotal avg of 3 RUNS : \d+\.\d{6} Sec\n$", out)


@pytest.mark.parametrize("k", [2, 4, 8])
def test_round_clean_then_wo_sort(prepared, k):
    d, src, dst, rp, col, orp, ocl = prepared
    node_parts = d / f"rmat13_part.csr_node_parts_random_{k}"
    run("round_clean_sg", k, d / "rmat13_part.csr", node_parts)
    outf = str(node_parts) + "_output.csr"
    pf = F.read_parts_output(outf, k)
    assert (pf.V, pf.E) == (len(rp) - 1, len(col))
    part = gen.parts_random(len(rp) - 1, k)
    for p, hp in enumerate(pf.parts):
        lrp, lcol, t_ver = oracle.halo_part(rp, col, np.diff(rp), part, p)
        assert hp.t_ver == t_ver and np.array_equal(hp.row_ptr, lrp) and np.array_equal(hp.col, lcol)
    whole = oracle.count(orp, ocl)
    for extra in ([], ["--batch"]):
        out = run("wo_sort_tc_256", outf, k, *extra)
        per = [int(x) for x in re.findall(r"\nPart \d+ executing :\t(\d+)\n", out)]
        assert len(per) == k and sum(per) == whole
        m = re.search(r"\nTotal Vertex : (\d+) \tTotal Edges : (\d+) \tTotal Triangle : (\d+) "
                      r"\tTotal Kernel Time : \d+\.\d{4} sec\tTotal Time : \d+\.\d{6} \n\n$", out)
        assert m and int(m.group(1)) == len(rp) - 1 and int(m.group(2)) == len(col) // 2 and int(m.group(3)) == whole


def test_round_clean_on_label_propagation_parts(prepared):
    """The _node_parts_lp_<k> file (the stand-in for the reference's
    _node_parts_metis_<k>) drives round_clean_sg and wo_sort_tc_256 like the
    random parts: the parts' counts sum to the whole graph's."""
    d, src, dst, rp, col, orp, ocl = prepared
    k = 4
    node_parts = d / f"rmat13_part.csr_node_parts_lp_{k}"
    run("round_clean_sg", k, d / "rmat13_part.csr", node_parts)
    out = run("wo_sort_tc_256", str(node_parts) + "_output.csr", k)
    per = [int(x) for x in re.findall(r"\nPart \d+ executing :\t(\d+)\n", out)]
    assert len(per) == k and sum(per) == oracle.count(orp, ocl)
