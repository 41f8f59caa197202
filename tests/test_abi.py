"""libtc's C ABI without a GPU: the library loads, every declared entry point
is exported, host utilities (formats, generators) behave, and device entry
points fail cleanly when no GPU is present."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import trianglecount_gb300 as tc
from trianglecount_gb300 import _native as N
from trianglecount_gb300 import formats as F
from trianglecount_gb300 import generators as gen

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    txt = open(os.path.join(ROOT, "include", "tc.h")).read()
    return sorted(set(re.findall(r"TC_API\s+[\w\s\*]+?\b(tc_\w+)\s*\(", txt)))


def test_every_declared_symbol_is_exported():
    syms = header_symbols()
    assert len(syms) >= 40
    L = tc.lib()
    for s in syms:
        assert hasattr(L, s), s
    assert sorted(N.declared_symbols()) == syms


def test_version_and_status_strings():
    L = tc.lib()
    assert L.tc_version() >= 10000
    assert L.tc_status_string(0) == b"ok"
    assert L.tc_status_string(-5) == b"malformed input"


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_has_gpu(), reason="checks the no-GPU error path")
def test_context_without_gpu_fails_cleanly():
    with pytest.raises(tc.TCError) as e:
        tc.Context(0)
    assert e.value.code == "TC_E_NO_DEVICE"


def test_text_roundtrip_and_reference_byte_layout(tmp_path):
    rp = np.array([0, 2, 3, 3], np.int64)
    col = np.array([1, 2, 2], np.int64)
    p = tmp_path / "g_output.csr"
    F.write_csr(p, 3, 6, rp, col)
    # without_part_preprocess.py:298-311 writes "%i " per value and "\n" per line
    assert open(p).read() == "3 6 4 3 \n0 2 3 3 \n1 2 2 \n"
    g = F.read_csr(p)
    assert (g.V, g.E) == (3, 6) and np.array_equal(g.row_ptr, rp) and np.array_equal(g.col, col)
    q = tmp_path / "x_part.csr"
    F.write_part_csr(q, np.array([0, 1, 2]), np.array([1, 0]), np.array([1, 1]))
    assert open(q).read() == "2 2\n2 3 2 0 \n0 1 2 \n1 0 \n1 1 \n"
    pc = F.read_part_csr(q)
    assert pc.N == 2 and list(pc.in_deg) == [1, 1]
    o = tmp_path / "parts_output.csr"
    F.write_parts_output(o, 2, 2, [F.HaloPart(2, 1, np.array([0, 1, 1]), np.array([1]))])
    # round_clean_subgraph.cu:371, 850-865
    assert open(o).read() == "2 2\n2 3 1 1\n0 1 1 \n1 \n"
    po = F.read_parts_output(o, 1)
    assert po.parts[0].t_ver == 1 and list(po.parts[0].col) == [1]


def test_text_reader_errors(tmp_path):
    with pytest.raises(tc.TCError) as e:
        F.read_ints(tmp_path / "missing.csr")
    assert e.value.code == "TC_E_IO"
    bad = tmp_path / "bad.csr"
    bad.write_text("1 2 x3 4\n")
    with pytest.raises(tc.TCError) as e:
        F.read_ints(bad)
    assert e.value.code == "TC_E_FORMAT"
    trunc = tmp_path / "trunc.csr"
    trunc.write_text("3 6 4 3\n0 2 3 3\n1 2\n")
    with pytest.raises(F.FormatError):
        F.read_csr(trunc)


def test_large_text_parse_is_exact(tmp_path):
    vals = np.random.default_rng(1).integers(0, 2**40, size=3_000_000, dtype=np.int64)
    p = tmp_path / "big.txt"
    F.write_line(p, vals, "w")
    F.write_line(p, vals[:7], "a", trailing_space=False)
    got = F.read_ints(p)
    assert np.array_equal(got[:len(vals)].astype(np.int64), vals)
    assert np.array_equal(got[len(vals):].astype(np.int64), vals[:7])


def test_tcsr_roundtrip(tmp_path):
    rp = np.array([0, 2, 2, 5], np.int64)
    col = np.array([1, 2, 0, 1, 2], np.int32)
    p = tmp_path / "g.tcsr"
    F.write_tcsr(p, rp, col, n_roots=2, aux=7)
    r2, c2, nr, aux = F.read_tcsr(p)
    assert np.array_equal(r2, rp) and np.array_equal(c2, col) and nr == 2 and aux == 7


def test_generators_are_deterministic():
    a = gen.rmat(10, seed=123)
    b = gen.rmat(10, seed=123)
    c = gen.rmat(10, seed=124)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]) and not np.array_equal(a[0], c[0])
    assert a[0].max() < 1024 and a[0].min() >= 0
    r = gen.road(50)
    assert np.array_equal(r[0], gen.road(50)[0])
    assert len(r[0]) > 2 * 50 * 50 * 0.8
    e = gen.er(1000, 10, seed=1)
    assert abs(len(e[0]) - 5000) < 10
    cl = gen.chung_lu(10000, 8.0, seed=2)
    deg = np.bincount(np.concatenate(cl), minlength=10000)
    assert deg.max() <= 4 * np.sqrt(10000 * 8.0)
    p = gen.parts_random(100000, 4)
    assert set(np.unique(p)) == {0, 1, 2, 3} and abs((p == 0).mean() - 0.25) < 0.01


def test_batch_mix_spec():
    specs = gen.batch_mix(256)
    kinds = [s.kind for s in specs]
    assert len(specs) == 256 and kinds.count("er") == 86 and kinds.count("rmat") == 85
    for s in specs:
        if s.kind == "er":
            assert 1000 <= s.params["n"] <= 100000 and 8 <= s.params["avg_deg"] <= 64
        if s.kind == "chung_lu":
            assert 10000 <= s.params["n"] <= 1000000
        if s.kind == "rmat":
            assert 10 <= s.params["scale"] <= 18
    assert [s.seed for s in gen.batch_mix(256)] == [s.seed for s in specs]
