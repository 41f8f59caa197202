"""CPU oracle for the triangle-counting path -- TEST INFRASTRUCTURE ONLY.

Imported only by tests/, __graft_entry__.smoke() and the cpu_baseline /
reference legs of bench.py, as the checker.  The product never calls it.

ctypes wrapper of oracle/oracle.c (built into oracle/_build/liboracle.so by
trianglecount_gb300/build.py: build_oracle()).  See oracle.c for the
reference file:line each function restates.

Pinning: the reference ships no golden vectors or tests for this path.  The
orientation is pinned against the reference's own CPU converter
(preprocess_CPU/Undir2Dir.c) compiled from source by oracle/build_ref.sh; the
counts are pinned by closed-form graphs (tests/golden/) and an independent
brute-force counter; the DGL clean-up step is restated (parity of that step
rests on the invariance checks in tests/).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
TIE = {"reference": 0, "id_asc": 1}
_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            import sys
            sys.path.insert(0, os.path.dirname(_HERE))
            from trianglecount_gb300.build import build_oracle
            build_oracle()
        L = C.CDLL(LIB_PATH)
        vp, i64, u64 = C.c_void_p, C.c_int64, C.c_uint64
        L.orc_clean.restype = i64
        L.orc_clean.argtypes = [i64, vp, vp, i64, vp, vp, C.POINTER(i64), vp]
        L.orc_orient.restype = i64
        L.orc_orient.argtypes = [i64, vp, vp, C.c_int, vp, vp]
        L.orc_orient_i32.restype = i64
        L.orc_orient_i32.argtypes = [i64, vp, vp, C.c_int, vp, vp]
        L.orc_count.restype = u64
        L.orc_count.argtypes = [i64, vp, vp, vp]
        L.orc_count_i32.restype = u64
        L.orc_count_i32.argtypes = [i64, vp, vp, vp]
        L.orc_count_i32_range.restype = u64
        L.orc_count_i32_range.argtypes = [i64, i64, vp, vp]
        L.orc_count_brute.restype = u64
        L.orc_count_brute.argtypes = [i64, vp, vp]
        L.orc_halo_part.restype = i64
        L.orc_halo_part.argtypes = [i64, vp, vp, vp, vp, i64, C.c_int, C.c_int, vp, vp, C.POINTER(i64),
                                    C.POINTER(i64)]
        L.orc_num_threads.restype = C.c_int
        L.orc_num_threads.argtypes = []
        L.orc_read_csr_fscanf.restype = C.c_int
        L.orc_read_csr_fscanf.argtypes = [C.c_char_p, vp, C.POINTER(C.POINTER(C.c_int32)), C.POINTER(C.POINTER(C.c_int32))]
        L.orc_gen_rmat.restype = C.c_int
        L.orc_gen_rmat.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, u64, C.c_int, vp, vp]
        L.orc_gen_parts_random.restype = C.c_int
        L.orc_gen_parts_random.argtypes = [i64, C.c_int, u64, vp]
        L.orc_free.restype = None
        L.orc_free.argtypes = [vp]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def num_threads() -> int:
    return lib().orc_num_threads()


def clean(src, dst, n_nodes: int = 0, return_old_ids: bool = False):
    """DGL clean-up (without_part_preprocess.py:193-228) -> (row_ptr, col) int64."""
    s = np.ascontiguousarray(src, np.int64)
    d = np.ascontiguousarray(dst, np.int64)
    n0 = max(int(n_nodes), int(max(s.max(initial=-1), d.max(initial=-1))) + 1)
    rp = np.empty(n0 + 1, np.int64)
    col = np.empty(max(2 * len(s), 1), np.int64)
    old = np.empty(max(n0, 1), np.int64) if return_old_ids else None
    V = C.c_int64()
    nnz = lib().orc_clean(len(s), _p(s), _p(d), int(n_nodes), _p(rp), _p(col), C.byref(V), _p(old))
    if nnz < 0:
        raise ValueError("negative vertex id")
    out = (rp[:V.value + 1].copy(), col[:nnz].copy())
    if return_old_ids:
        return out + (old[:V.value].copy(),)
    return out


def orient(row_ptr, col, tie="reference"):
    """Degree orientation (without_part_preprocess.py:19-111) -> (row_ptr, col) int64."""
    rp = np.ascontiguousarray(row_ptr, np.int64)
    cl = np.ascontiguousarray(col, np.int64)
    V = len(rp) - 1
    orp = np.empty(V + 1, np.int64)
    ocl = np.empty(max(len(cl), 1), np.int64)
    m = lib().orc_orient(V, _p(rp), _p(cl), TIE[tie] if isinstance(tie, str) else int(tie), _p(orp), _p(ocl))
    return orp, ocl[:m].copy()


def count(row_ptr, col, n_roots: int | None = None, per_root: bool = False):
    """Exact count (the reference's g_sum summed); int32 or int64 arrays."""
    rp = np.ascontiguousarray(row_ptr)
    cl = np.ascontiguousarray(col)
    n_roots = len(rp) - 1 if n_roots is None else int(n_roots)
    pr = np.zeros(max(n_roots, 1), np.uint64) if per_root else None
    if rp.dtype == np.int32 and cl.dtype == np.int32:
        t = lib().orc_count_i32(n_roots, _p(rp), _p(cl), _p(pr))
    else:
        rp = rp.astype(np.int64, copy=False)
        cl = cl.astype(np.int64, copy=False)
        t = lib().orc_count(n_roots, _p(rp), _p(cl), _p(pr))
    return (int(t), pr[:n_roots]) if per_root else int(t)


def count_range_i32(row_ptr: np.ndarray, col: np.ndarray, r0: int, r1: int) -> int:
    """Count over roots [r0, r1) of an int32 CSR (bounded CPU-baseline sample)."""
    return int(lib().orc_count_i32_range(r0, r1, _p(row_ptr), _p(col)))


def count_brute(row_ptr, col) -> int:
    """Independent count on the undirected sorted CSR (u < v < w)."""
    rp = np.ascontiguousarray(row_ptr, np.int64)
    cl = np.ascontiguousarray(col, np.int64)
    return int(lib().orc_count_brute(len(rp) - 1, _p(rp), _p(cl)))


def halo_part(row_ptr, col, deg, part, p: int, tie="reference", mode: str = "reference"):
    """Halo subgraph of part p -> (row_ptr, col, t_ver), local ids.  mode
    "reference" follows the reference's extraction; "count" keeps only the halo
    vertices with an oriented in-edge from the part (the library's counting
    halo)."""
    rp = np.ascontiguousarray(row_ptr, np.int64)
    cl = np.ascontiguousarray(col, np.int64)
    dg = np.ascontiguousarray(deg, np.int64)
    pt = np.ascontiguousarray(part, np.int64)
    V = len(rp) - 1
    orp = np.empty(V + 1, np.int64)
    ocl = np.empty(max(len(cl), 1), np.int64)
    nl, tv = C.c_int64(), C.c_int64()
    m = lib().orc_halo_part(V, _p(rp), _p(cl), _p(dg), _p(pt), int(p), TIE[tie] if isinstance(tie, str) else int(tie),
                            {"reference": 0, "count": 1}[mode], _p(orp), _p(ocl), C.byref(nl), C.byref(tv))
    return orp[:nl.value + 1].copy(), ocl[:m].copy(), tv.value


def pipeline(src, dst, n_nodes: int = 0, tie="reference"):
    """Edge list -> oriented CSR (int32) and its count, all on the CPU."""
    rp, col = clean(src, dst, n_nodes)
    orp, ocl = orient(rp, col, tie)
    return orp.astype(np.int32), ocl.astype(np.int32), count(orp, ocl)


# ---- the reference's own TC_128 kernel (oracle/_ref, built by build_ref.sh) ----
REF_DIR = os.path.join(_HERE, "_ref")
REF_CUBIN = os.path.join(REF_DIR, "tc128_sm103a.cubin")
REF_LAUNCH = os.path.join(_HERE, "_build", "libref_launch.so")
UNDIR2DIR = os.path.join(_HERE, "_ref", "undir2dir")


def ref_kernel_available() -> bool:
    return os.path.exists(REF_CUBIN) and os.path.exists(REF_LAUNCH)


# The reference's design-space variants of its Find_Triangle kernel
# (src/WithoutPartition/): name -> (cubin, kernel symbol, threads per block,
# u64 indices, adds every hit to one counter).
REF_VARIANTS = {
    "tc128": ("tc128_sm103a.cubin", "_Z13Find_TrianglePiS_iiPy", 128, 0, 0),   # ShareKernelTCV62_update_v1.cu
    "smem64": ("var_smem64_sm103a.cubin", "_Z13Find_TrianglePiS_iiPy", 64, 0, 0),  # shareMemSize.cu
    "atomic256": ("var_atomic256_sm103a.cubin", "_Z13Find_TrianglePiS_iiPy", 256, 0, 1),  # With_Atomic_op.cu
    "nosmem2": ("var_nosmem2_sm103a.cubin", "_Z13Find_TrianglePyS_S_", 2, 1, 1),  # Without_ShareMemory_TC.cu
}


def ref_variant_available(name: str) -> bool:
    return os.path.exists(os.path.join(REF_DIR, REF_VARIANTS[name][0])) and os.path.exists(REF_LAUNCH)


def ref_variant(name: str, row_ptr, col, runs: int = 1):
    """Run one of the reference's kernel variants on cuda:0 with its own launch
    shape -> (total count, last kernel time in ms)."""
    cubin, sym, threads, idx64, total_only = REF_VARIANTS[name]
    L = C.CDLL(REF_LAUNCH)
    L.ref_variant_run.restype = C.c_int
    L.ref_variant_run.argtypes = [C.c_char_p, C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                  C.c_int32, C.c_int32, C.c_int, C.POINTER(C.c_uint64), C.POINTER(C.c_float),
                                  C.c_char_p, C.c_int]
    rp = np.ascontiguousarray(row_ptr, np.int32)
    cl = np.ascontiguousarray(col, np.int32)
    tot, ms = C.c_uint64(), C.c_float()
    err = C.create_string_buffer(256)
    rc = L.ref_variant_run(os.path.join(REF_DIR, cubin).encode(), sym.encode(), threads, idx64, total_only, _p(rp),
                           _p(cl), len(rp) - 1, len(cl), int(runs), C.byref(tot), C.byref(ms), err, 256)
    if rc != 0:
        raise RuntimeError(f"reference variant {name} failed: {err.value.decode()}")
    return int(tot.value), ms.value


def ref_tc128(row_ptr, col, runs: int = 1):
    """Run the reference TC_128 kernel (one 128-thread block per vertex) on
    cuda:0 -> (per_root g_sum as uint64, last kernel time in ms)."""
    L = C.CDLL(REF_LAUNCH)
    L.ref_tc128_run.restype = C.c_int
    L.ref_tc128_run.argtypes = [C.c_char_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int,
                                C.c_void_p, C.POINTER(C.c_float), C.c_char_p, C.c_int]
    rp = np.ascontiguousarray(row_ptr, np.int32)
    cl = np.ascontiguousarray(col, np.int32)
    V = len(rp) - 1
    out = np.zeros(max(V, 1), np.uint64)
    ms = C.c_float()
    err = C.create_string_buffer(256)
    rc = L.ref_tc128_run(REF_CUBIN.encode(), _p(rp), _p(cl), V, len(cl), int(runs), _p(out), C.byref(ms), err, 256)
    if rc != 0:
        raise RuntimeError(f"reference kernel launch failed: {err.value.decode()}")
    return out[:V], ms.value


def read_csr_fscanf(path):
    """The TC_128 driver's .csr reader restated (one fscanf per integer,
    ShareKernelTCV62_update_v1.cu:206-230): (header[4], row_ptr, col)."""
    L = lib()
    hdr = np.zeros(4, np.int64)
    rp, cl = C.POINTER(C.c_int32)(), C.POINTER(C.c_int32)()
    if L.orc_read_csr_fscanf(os.fsencode(path), hdr.ctypes.data_as(C.c_void_p), C.byref(rp), C.byref(cl)) != 0:
        raise OSError(f"cannot read {path}")
    try:
        row_ptr = np.ctypeslib.as_array(rp, shape=(int(hdr[2]),)).copy() if hdr[2] else np.zeros(0, np.int32)
        col = np.ctypeslib.as_array(cl, shape=(int(hdr[3]),)).copy() if hdr[3] else np.zeros(0, np.int32)
    finally:
        L.orc_free(C.cast(rp, C.c_void_p))
        L.orc_free(C.cast(cl, C.c_void_p))
    return hdr, row_ptr, col


# ---- seeded benchmark inputs without the library (bench.py's reference arm) ----
RMAT_ABC = (0.57, 0.19, 0.19)
SEED_RMAT = {16: 0x5EED0016, 21: 0x5EED0021, 23: 0x5EED0023}
SEED_PARTS = 0x5EED9A27


def gen_rmat(scale: int, edge_factor: int = 16, seed: int | None = None, permute: bool = True):
    """The benchmark's R-MAT edge list (same bits as the library's generator)."""
    n = edge_factor << scale
    src = np.empty(n, np.int64)
    dst = np.empty(n, np.int64)
    seed = SEED_RMAT.get(scale, 0x5EED0000 + scale) if seed is None else seed
    a, b, c = RMAT_ABC
    if lib().orc_gen_rmat(scale, edge_factor, a, b, c, seed, 1 if permute else 0, _p(src), _p(dst)) != 0:
        raise ValueError("bad R-MAT parameters")
    return src, dst


def gen_parts_random(n: int, k: int, seed: int | None = None):
    """Seeded uniform parts (same bits as the library's generator)."""
    part = np.empty(n, np.int32)
    if lib().orc_gen_parts_random(n, k, (SEED_PARTS + k) if seed is None else seed, _p(part)) != 0:
        raise ValueError("bad partition arguments")
    return part
