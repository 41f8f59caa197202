"""The reference's on-disk formats, read and written through libtc's parser.

All files are whitespace-separated unsigned integers read in order, exactly as
the reference's fscanf / ifstream loops consume them:

  .csr (oriented, TC_128 input; writer without_part_preprocess.py:298-311,
        reader ShareKernelTCV62_update_v1.cu:207-230):
        V E row_ptr_s col_idx_s / row_ptr[row_ptr_s] / col[col_idx_s]
        (E = 2m of the bidirected graph, row_ptr_s = V+1, col_idx_s = m)
  _part.csr (undirected + degree, Halo_creation_preprocess.py:259-278,
        reader round_clean_subgraph.cu:924-968):
        N E / N N+1 2m 0 / row_ptr / col / in_deg[N]
  node parts (Halo_creation_preprocess.py:306-312): one part id per vertex
  <parts>_output.csr (round_clean_subgraph.cu:371, 850-865; reader
        without_sorting_tc.cu:242-286):
        V E / per part: v_pos rp_pos ci_pos t_ver / row_ptr[rp_pos] / col[ci_pos]
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

from . import _native as N


def read_ints(path: str | os.PathLike) -> np.ndarray:
    """All integers of a text file, in order (uint64)."""
    data = C.POINTER(C.c_uint64)()
    n = C.c_int64()
    N.call("tc_text_read_u64", os.fsencode(path), C.byref(data), C.byref(n))
    try:
        if n.value == 0:
            return np.empty(0, np.uint64)
        arr = np.ctypeslib.as_array(data, shape=(n.value,)).copy()
    finally:
        N.lib().tc_host_free(C.cast(data, C.c_void_p))
    return arr


def write_line(path, values, mode: str = "a", trailing_space: bool = True) -> None:
    a = np.ascontiguousarray(values)
    if a.dtype not in (np.int32, np.int64):
        a = a.astype(np.int64)
    N.call("tc_text_write_line", os.fsencode(path), a.ctypes.data_as(C.c_void_p), len(a), a.itemsize,
           C.c_char(mode.encode()), 1 if trailing_space else 0)


class FormatError(ValueError):
    pass


def _take(a: np.ndarray, pos: int, n: int, what: str) -> tuple[np.ndarray, int]:
    if n < 0 or pos + n > len(a):
        raise FormatError(f"truncated file: {what} needs {n} values at offset {pos}, file has {len(a)}")
    return a[pos:pos + n], pos + n


@dataclass
class OrientedCSR:
    V: int
    E: int          # header E (2m)
    row_ptr: np.ndarray
    col: np.ndarray


def read_csr(path) -> OrientedCSR:
    a = read_ints(path)
    hdr, p = _take(a, 0, 4, "header")
    V, E, rps, cis = (int(x) for x in hdr)
    rp, p = _take(a, p, rps, "row_ptr")
    col, p = _take(a, p, cis, "col_idx")
    return OrientedCSR(V, E, rp.astype(np.int64), col.astype(np.int64))


def write_csr(path, V: int, E: int, row_ptr: np.ndarray, col: np.ndarray) -> None:
    """Byte layout of without_part_preprocess.py:298-311."""
    write_line(path, np.array([V, E, len(row_ptr), len(col)], np.int64), "w")
    write_line(path, row_ptr, "a")
    write_line(path, col, "a")


@dataclass
class PartCSR:
    N: int
    E: int
    row_ptr: np.ndarray
    col: np.ndarray
    in_deg: np.ndarray


def read_part_csr(path) -> PartCSR:
    a = read_ints(path)
    hdr, p = _take(a, 0, 6, "header")
    n, e, _nm, rps, cis, _nh = (int(x) for x in hdr)
    rp, p = _take(a, p, rps, "row_ptr")
    col, p = _take(a, p, cis, "col_idx")
    deg, p = _take(a, p, n, "in_deg")
    return PartCSR(n, e, rp.astype(np.int64), col.astype(np.int64), deg.astype(np.int64))


def write_part_csr(path, row_ptr: np.ndarray, col: np.ndarray, in_deg: np.ndarray) -> None:
    """Byte layout of Halo_creation_preprocess.py:259-278."""
    n = len(row_ptr) - 1
    write_line(path, np.array([n, len(col)], np.int64), "w", trailing_space=False)
    write_line(path, np.array([n, n + 1, len(col), 0], np.int64), "a")
    write_line(path, row_ptr, "a")
    write_line(path, col, "a")
    write_line(path, in_deg, "a")


def read_node_parts(path, n: int | None = None) -> np.ndarray:
    a = read_ints(path)
    if n is not None:
        a, _ = _take(a, 0, n, "node parts")
    return a.astype(np.int32)


def write_node_parts(path, part: np.ndarray) -> None:
    write_line(path, np.asarray(part, np.int64), "w")


@dataclass
class HaloPart:
    v_pos: int
    t_ver: int
    row_ptr: np.ndarray
    col: np.ndarray


@dataclass
class PartsFile:
    V: int
    E: int
    parts: list


def read_parts_output(path, k: int) -> PartsFile:
    a = read_ints(path)
    hdr, p = _take(a, 0, 2, "header")
    V, E = int(hdr[0]), int(hdr[1])
    parts = []
    for i in range(k):
        h, p = _take(a, p, 4, f"part {i} header")
        v_pos, rps, cis, t_ver = (int(x) for x in h)
        rp, p = _take(a, p, rps, f"part {i} row_ptr")
        col, p = _take(a, p, cis, f"part {i} col_idx")
        parts.append(HaloPart(v_pos, t_ver, rp.astype(np.int64), col.astype(np.int64)))
    return PartsFile(V, E, parts)


def write_parts_output(path, V: int, E: int, parts: list) -> None:
    """Byte layout of round_clean_subgraph.cu:371, 850-865."""
    write_line(path, np.array([V, E], np.int64), "w", trailing_space=False)
    for hp in parts:
        n = len(hp.row_ptr) - 1
        write_line(path, np.array([n, n + 1, len(hp.col), hp.t_ver], np.int64), "a", trailing_space=False)
        write_line(path, hp.row_ptr, "a")
        write_line(path, hp.col, "a")


def read_edges(path) -> tuple[np.ndarray, np.ndarray]:
    """Edge list of a .tsv / .txt / .mtx / .mmio graph file (int64 src, dst)."""
    s = C.POINTER(C.c_int64)()
    d = C.POINTER(C.c_int64)()
    n = C.c_int64()
    N.call("tc_read_edges", os.fsencode(path), C.byref(s), C.byref(d), C.byref(n))
    try:
        if n.value == 0:
            return np.empty(0, np.int64), np.empty(0, np.int64)
        return (np.ctypeslib.as_array(s, shape=(n.value,)).copy(), np.ctypeslib.as_array(d, shape=(n.value,)).copy())
    finally:
        N.lib().tc_host_free(C.cast(s, C.c_void_p))
        N.lib().tc_host_free(C.cast(d, C.c_void_p))


def write_tcsr(path, row_ptr: np.ndarray, col: np.ndarray, n_roots: int | None = None, aux: int = 0) -> None:
    rp = np.ascontiguousarray(row_ptr, np.int64)
    cl = np.ascontiguousarray(col, np.int32)
    n_rows = len(rp) - 1
    N.call("tc_tcsr_write", os.fsencode(path), rp.ctypes.data_as(C.c_void_p), cl.ctypes.data_as(C.c_void_p),
           n_rows, len(cl), n_rows if n_roots is None else n_roots, aux)


def read_tcsr(path) -> tuple[np.ndarray, np.ndarray, int, int]:
    n_rows, nnz, n_roots, aux = C.c_int64(), C.c_int64(), C.c_int64(), C.c_int64()
    N.call("tc_tcsr_read_header", os.fsencode(path), C.byref(n_rows), C.byref(nnz), C.byref(n_roots), C.byref(aux))
    rp = np.empty(n_rows.value + 1, np.int64)
    col = np.empty(nnz.value, np.int32)
    N.call("tc_tcsr_read", os.fsencode(path), rp.ctypes.data_as(C.c_void_p), col.ctypes.data_as(C.c_void_p))
    return rp, col, n_roots.value, aux.value
