"""In-tree build of libtc (CUDA, sm_103a), its command-line tools and the oracle.

Every translation unit is compiled in parallel; an object is rebuilt only when
its source or a header is newer.  Outputs (all git-ignored):

  trianglecount_gb300/lib/libtc.so      the engine + C ABI (include/tc.h)
  trianglecount_gb300/bin/<tool>        TC_128, wo_sort_tc_256, round_clean_sg, tc_preprocess
  oracle/_build/liboracle.so            the CPU checker (tests and bench baseline only)
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "lib")
BIN = os.path.join(PKG, "bin")
LIBTC = os.path.join(LIB, "libtc.so")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-fvisibility=hidden,-O3",
                     "-I" + INCLUDE, "-I" + CSRC] + os.environ.get("TC_NVCC_EXTRA", "").split()
CXX = os.environ.get("CXX", "g++")
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-fvisibility=hidden", "-pthread", "-Wall",
             "-I" + INCLUDE, "-I" + CSRC, "-I" + os.path.join(CUDA_HOME, "include")]
TOOLS = {
    "TC_128": "cli_tc128.cpp",
    "wo_sort_tc_256": "cli_wo_sort.cpp",
    "round_clean_sg": "cli_round_clean.cpp",
    "tc_preprocess": "cli_preprocess.cpp",
}


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers() -> list[str]:
    return glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))


def build_libtc(jobs: int | None = None, verbose: bool = False) -> str:
    """Compile libtc.so and the CLI tools; returns the library path."""
    if not os.path.exists(NVCC):
        raise RuntimeError(f"nvcc not found at {NVCC}")
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIB, exist_ok=True)
    os.makedirs(BIN, exist_ok=True)
    hdrs = _headers()
    cli_srcs = set(TOOLS.values())
    steps = []
    objs = []
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp"))):
        if os.path.basename(src) in cli_srcs:
            continue
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(obj)
        if _stale(obj, [src] + hdrs):
            if src.endswith(".cu"):
                steps.append([NVCC] + NVCC_FLAGS + ["-c", src, "-o", obj])
            else:
                steps.append([CXX] + CXX_FLAGS + ["-c", src, "-o", obj])
    with ThreadPoolExecutor(max_workers=jobs or max(2, os.cpu_count() or 2)) as ex:
        for cmd in steps:
            if verbose:
                print(" ".join(cmd), file=sys.stderr)
        list(ex.map(_run, steps))
    if _stale(LIBTC, objs):
        _run([NVCC] + ARCH + ["-shared", "-o", LIBTC] + objs + ["-Xcompiler", "-pthread"])
    tool_steps = []
    for tool, src in TOOLS.items():
        path = os.path.join(CSRC, src)
        out = os.path.join(BIN, tool)
        if os.path.exists(path) and _stale(out, [path, LIBTC] + hdrs):
            tool_steps.append([CXX, "-O2", "-std=c++17", "-Wall", "-I" + INCLUDE, path, "-o", out,
                               "-L" + LIB, "-ltc", "-Wl,-rpath,$ORIGIN/../lib", "-pthread"])
    with ThreadPoolExecutor(max_workers=jobs or max(2, os.cpu_count() or 2)) as ex:
        list(ex.map(_run, tool_steps))
    return LIBTC


def build_oracle() -> str:
    """Compile the CPU oracle (test infrastructure) into oracle/_build."""
    odir = os.path.join(ROOT, "oracle")
    out_dir = os.path.join(odir, "_build")
    os.makedirs(out_dir, exist_ok=True)
    src = os.path.join(odir, "oracle.c")
    out = os.path.join(out_dir, "liboracle.so")
    if _stale(out, [src]):
        cc = os.environ.get("CC", "gcc")
        _run([cc, "-O3", "-fopenmp", "-shared", "-fPIC", "-Wall", src, "-o", out])
    # host-only launcher of the reference kernel cubin (oracle/_ref, when built)
    lsrc = os.path.join(odir, "ref_launch.cu")
    lout = os.path.join(out_dir, "libref_launch.so")
    if os.path.exists(lsrc) and os.path.exists(NVCC) and _stale(lout, [lsrc]):
        _run([NVCC] + ARCH + ["-O2", "-shared", "-Xcompiler", "-fPIC", lsrc, "-o", lout])
    return out


def clean() -> None:
    for d in (BUILD, LIB, BIN, os.path.join(ROOT, "oracle", "_build")):
        shutil.rmtree(d, ignore_errors=True)


if __name__ == "__main__":
    print(build_libtc(verbose="-v" in sys.argv))
    print(build_oracle())
