"""bench.py's JSON line against the benchmark contract: the reference arm
on the CPU, the GPU arm on R-MAT 16 (marked gpu)."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_contract_line():
    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0"],
                         cwd=ROOT, capture_output=True, text=True, timeout=600, check=True).stdout
    lines = [line for line in out.splitlines() if line.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == "oriented edges/s" and d["unit"] == "edges/s"
    assert d["value"] > 0 and d["ms_per_step"] > 0 and d["higher_is_better"] is True
    assert (d["n_gpus"], d["steps"], d["warmup"]) == (1, 1, 0)
    assert d["scaling"] == "weak" and d["vs_baseline"] is None and d["dtype"] == "int32"
    assert d["config"]["workload"] == "rmat21_ef16_plain" and d["config"]["oriented_edges"] == 31769277
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
