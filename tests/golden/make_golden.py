"""Generates the committed golden fixtures of tests/golden/.

  known_graphs.json      closed-form counts of the families in families.py
  rmat_counts.json       counts of seeded R-MAT graphs (scales 8..14) from the
                         CPU oracle; the generator draws integers only, so these
                         pin the generator + pipeline on every platform
  fullsize_counts.json   the same for the benchmark-size workloads (R-MAT 21,
                         road 1448 x 1448, R-MAT 23)
  undir2dir_*.npz        orientation golden vectors produced by the reference's
                         own CPU converter (preprocess_CPU/Undir2Dir.c, built by
                         oracle/build_ref.sh into oracle/_ref/undir2dir) on small
                         cleaned graphs, with its input

Run from the repo root after building (needs oracle/_ref for the npz files):
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

import families  # noqa: E402
import oracle  # noqa: E402
from trianglecount_gb300 import generators as gen  # noqa: E402


def known_graphs():
    out = [{"family": n, "args": a, "expected": families.expected(n, a)} for n, a in families.CASES]
    with open(os.path.join(HERE, "known_graphs.json"), "w") as f:
        json.dump(out, f, indent=1)


def rmat_counts():
    out = []
    for scale in range(8, 15):
        src, dst = gen.rmat(scale, 16, seed=0x5EED0000 + scale)
        rp, col = oracle.clean(src, dst)
        orp, ocl = oracle.orient(rp, col)
        out.append({"scale": scale, "seed": 0x5EED0000 + scale, "V": len(rp) - 1, "undirected_nnz": len(col),
                    "oriented_nnz": len(ocl), "triangles": oracle.count(orp, ocl),
                    "edge_checksum": int((src * 1000003 + dst).sum() % (1 << 61))})
    with open(os.path.join(HERE, "rmat_counts.json"), "w") as f:
        json.dump(out, f, indent=1)


def fullsize_counts():
    """Counts of the benchmark-size workloads (R-MAT scale 21 and 23 with their
    default seeds, the 1448 x 1448 road grid), from the CPU oracle: the GPU
    tests compare the device counts and the halo-part sums with these."""
    out = {}
    cases = {"rmat21": lambda: gen.rmat(21, 16), "road": lambda: gen.road(), "rmat23": lambda: gen.rmat(23, 16)}
    for name, make in cases.items():
        src, dst = make()
        rp, col = oracle.clean(src, dst)
        orp, ocl = oracle.orient(rp, col)
        out[name] = {"V": len(rp) - 1, "undirected_nnz": len(col), "oriented_nnz": len(ocl),
                     "triangles": oracle.count(orp, ocl),
                     "edge_checksum": int((src * 1000003 + dst).sum() % (1 << 61))}
        print(name, out[name], flush=True)
    with open(os.path.join(HERE, "fullsize_counts.json"), "w") as f:
        json.dump(out, f, indent=1)


def undir2dir_goldens():
    exe = oracle.UNDIR2DIR
    if not os.path.exists(exe):
        print("oracle/_ref/undir2dir missing: run oracle/build_ref.sh first; skipping npz goldens")
        return
    cases = {"rmat9": gen.rmat(9, 16, seed=0x5EED0009), "road24": gen.road(24, seed=0x5EED0024),
             "k40": families.complete(40)[:2]}
    for name, (src, dst) in cases.items():
        rp, col = oracle.clean(src, dst)
        V = len(rp) - 1
        deg = np.diff(rp)
        with tempfile.TemporaryDirectory() as td:
            inp, outp = os.path.join(td, "in.txt"), os.path.join(td, "out.txt")
            with open(inp, "w") as f:
                # legacy input (Undir2Dir.c:33-90): in_deg_s, in_deg[], then per part
                # org_id_s row_ptr_s col_idx_s t_ver, org_id[], row_ptr[], col_idx[]
                f.write(f"{V}\n" + " ".join(map(str, deg)) + "\n")
                f.write(f"{V} {V + 1} {len(col)} {V}\n")
                f.write(" ".join(map(str, range(V))) + "\n")
                f.write(" ".join(map(str, rp)) + "\n")
                f.write(" ".join(map(str, col)) + "\n")
            subprocess.run([exe, inp, outp, "1"], check=True, capture_output=True)
            vals = np.array(open(outp).read().split(), np.int64)
        t_ver, rps, m = vals[:3]
        orp = vals[3:3 + rps]
        ocl = vals[3 + rps:3 + rps + m]
        np.savez_compressed(os.path.join(HERE, f"undir2dir_{name}.npz"), row_ptr=rp, col=col, oriented_row_ptr=orp,
                            oriented_col=ocl)


if __name__ == "__main__":
    known_graphs()
    rmat_counts()
    if "--fullsize" in sys.argv:  # minutes of CPU time
        fullsize_counts()
    undir2dir_goldens()
    print("golden fixtures written to", HERE)
