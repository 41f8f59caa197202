"""bench.py's JSON line against the benchmark contract: the reference arm
on the CPU, the GPU arm on R-MAT 16 (marked gpu)."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_contract_line():
    """The default (partitioned) workload at a small scale: the same code path
    as R-MAT 23, which takes minutes of CPU here."""
    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0",
                          "--scale", "14"],
                         cwd=ROOT, capture_output=True, text=True, timeout=600, check=True).stdout
    lines = [line for line in out.splitlines() if line.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == "oriented edges/s" and d["unit"] == "edges/s"
    assert d["value"] > 0 and d["ms_per_step"] > 0 and d["higher_is_better"] is True
    assert (d["n_gpus"], d["steps"], d["warmup"]) == (1, 1, 0)
    assert d["scaling"] == "strong" and d["vs_baseline"] is None and d["dtype"] == "int32"
    assert d["config"]["workload"] == "rmat14_ef16_halo_parts" and d["config"]["oriented_edges"] == 213184
    assert d["config"]["parts_k"] == [2, 4, 8]
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["unit"] == d["unit"] and cb["cores"] >= 1
    assert cb["kind"] in ("port", "reference") and cb["sample"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["unit"] == d["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


@pytest.mark.gpu
def test_gpu_arm_line_carries_roofline_baseline_e2e_and_clocks():
    """The GPU arm on R-MAT 16: roofline of the dominant kernel, the CPU
    baseline, the end-to-end number with its host copies, clocks and the
    launch count, with the count checked against the oracle inside."""
    out = subprocess.run([sys.executable, "bench.py", "--workload", "rmat16", "--steps", "3", "--warmup", "3"],
                         cwd=ROOT, capture_output=True, text=True, timeout=900, check=True).stdout
    lines = [line for line in out.splitlines() if line.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["metric"] == "oriented edges/s" and d["value"] > 0 and d["n_gpus"] == 1 and d["steps"] == 3
    r = d["roofline"]
    assert r["bound"] == "hbm" and r["unit"] == "GB/s" and r["achieved"] > 0 and r["peak"] > 0
    assert abs(r["frac"] - r["achieved"] / r["peak"]) < 1e-9
    assert d["cpu_baseline"]["value"] > 0 and d["cpu_baseline"]["cores"] >= 1
    e2e = d["e2e"]
    assert e2e["value"] > 0 and e2e["h2d_bytes_per_step"] > 0 and e2e["d2h_bytes_per_step"] > 0
    assert d["gpu_launches"] > 0 and "sm_mhz" in d["clocks"] and "reasons" in d["clocks"]
    assert d["config"]["workload"] == "rmat16_ef16_plain"


def test_reference_arm_loads_no_library_code():
    """The reference arm builds its input with the oracle's generators: the
    process never maps libtc.so."""
    code = ("import sys, runpy; sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '0', "
            "'--scale', '12']; runpy.run_path('bench.py', run_name='__main__'); "
            "maps = open('/proc/self/maps').read(); print('LIBTC' if 'libtc.so' in maps else 'CLEAN')")
    out = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=600,
                         check=True).stdout
    assert out.strip().splitlines()[-1] == "CLEAN"


@pytest.mark.gpu
def test_gpu_arm_partitioned_line_is_complete():
    """The default workload at scale 16: per-k timings in both halo modes,
    the roofline with its three figures, the end-to-end parts path, clocks."""
    out = subprocess.run([sys.executable, "bench.py", "--steps", "2", "--warmup", "3", "--scale", "16"],
                         cwd=ROOT, capture_output=True, text=True, timeout=900, check=True).stdout
    lines = [line for line in out.splitlines() if line.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["config"]["workload"] == "rmat16_ef16_halo_parts" and d["value"] > 0 and d["scaling"] == "strong"
    r = d["roofline"]
    assert r["achieved"] > 0 and abs(r["frac"] - r["achieved"] / r["peak"]) < 1e-9
    assert r["wedge_model_bytes"] >= r["algorithmic_bytes_per_launch"] > 0
    for k in ("2", "4", "8"):
        row = d["detail"]["parts"][k]
        assert row["count"]["parts_nnz_total"] <= row["reference"]["parts_nnz_total"]
        assert sum(row["count"]["per_part_counts"]) == d["detail"]["triangles"]
    e2e = d["e2e"]
    assert e2e["value"] > 0 and e2e["h2d_bytes_per_step"] > 0 and e2e["d2h_bytes_per_step"] > 0
    assert d["gpu_launches"] > 0 and "sm_mhz" in d["clocks"]
    assert d["cpu_baseline"]["count_matches"] is True
