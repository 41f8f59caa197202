"""Python host side of libtc: contexts, device graphs, counting, batching,
preprocessing and halo extraction.  Thin wrappers over the C ABI; every
computation runs in libtc's CUDA kernels.

The operations mirror the reference's processing stages:

  Context.ugraph_from_edges  ~ without_part_preprocess.py:193-228 (DGL clean-up)
  Context.orient             ~ without_part_preprocess.py:19-111 (Find_size/Convert)
  Context.upload + count     ~ TC_128 (ShareKernelTCV62_update_v1.cu:192-310)
  Context.halo_extract       ~ round_clean_sg (round_clean_subgraph.cu:357-902)
  Batch / Context.count_each ~ wo_sort_tc_256's per-part loop (without_sorting_tc.cu:244-465)
"""
from __future__ import annotations

import ctypes as C
from typing import Sequence

import numpy as np

from . import _native as N


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _tie(tie) -> int:
    if isinstance(tie, str):
        return N.TIE[tie]
    return int(tie)


class Graph:
    """A device-resident oriented CSR (int32).  Roots are rows [0, n_roots)."""

    def __init__(self, ctx: "Context", handle: C.c_void_p):
        self.ctx = ctx
        self._h = handle

    @property
    def handle(self):
        if self._h is None:
            raise ValueError("graph already freed")
        return self._h

    def info(self) -> tuple[int, int, int]:
        r, n, k = C.c_int64(), C.c_int64(), C.c_int64()
        N.call("tc_graph_info", self.handle, C.byref(r), C.byref(n), C.byref(k))
        return r.value, n.value, k.value

    @property
    def n_rows(self) -> int:
        return self.info()[0]

    @property
    def nnz(self) -> int:
        return self.info()[1]

    @property
    def n_roots(self) -> int:
        return self.info()[2]

    def download(self) -> tuple[np.ndarray, np.ndarray]:
        n_rows, nnz, _ = self.info()
        rp = np.empty(n_rows + 1, np.int32)
        col = np.empty(nnz, np.int32)
        N.call("tc_graph_download_i32", self.ctx.handle, self.handle, _ptr(rp), _ptr(col))
        return rp, col

    def count(self) -> int:
        return self.ctx.count(self)

    def free(self) -> None:
        if self._h is not None:
            N.lib().tc_graph_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class UGraph:
    """A device-resident simple undirected CSR (int32) with its degree column."""

    def __init__(self, ctx: "Context", handle: C.c_void_p):
        self.ctx = ctx
        self._h = handle

    @property
    def handle(self):
        if self._h is None:
            raise ValueError("graph already freed")
        return self._h

    def info(self) -> tuple[int, int]:
        r, n = C.c_int64(), C.c_int64()
        N.call("tc_ugraph_info", self.handle, C.byref(r), C.byref(n))
        return r.value, n.value

    def download(self) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        n_rows, nnz = self.info()
        rp = np.empty(n_rows + 1, np.int64)
        col = np.empty(nnz, np.int64)
        deg = np.empty(n_rows, np.int64)
        N.call("tc_ugraph_download", self.ctx.handle, self.handle, _ptr(rp), _ptr(col), _ptr(deg))
        return rp, col, deg

    def free(self) -> None:
        if self._h is not None:
            N.lib().tc_ugraph_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Batch:
    """Many graphs counted by one persistent launch, replayed as a CUDA graph."""

    def __init__(self, ctx: "Context", graphs: Sequence[Graph]):
        self.ctx = ctx
        self.graphs = list(graphs)  # keeps the graphs alive
        arr = (C.c_void_p * len(self.graphs))(*[g.handle for g in self.graphs])
        h = C.c_void_p()
        N.call("tc_batch_create", ctx.handle, arr, len(self.graphs), C.byref(h))
        self._h = h
        self._out = np.empty(len(self.graphs), np.uint64)

    def run(self) -> np.ndarray:
        N.call("tc_batch_run", self._h, _ptr(self._out))
        return self._out.copy()

    def run_async(self) -> None:
        N.call("tc_batch_run_async", self._h)

    def results(self) -> np.ndarray:
        N.call("tc_batch_results", self._h, _ptr(self._out))
        return self._out.copy()

    def stats(self) -> dict:
        """Of the last replay: counting-kernel device time (ms), kernels per
        replay, heavy block units."""
        st = N.CountStats()
        N.call("tc_batch_stats", self._h, C.byref(st))
        return {"count_kernel_ms": st.count_ms, "launches": st.launches, "heavy_units": st.heavy_units}

    def free(self) -> None:
        if getattr(self, "_h", None) is not None:
            N.lib().tc_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Server:
    """Continuous-batching triangle-count server (tc_server_* in the C ABI)."""

    def __init__(self, ctx: "Context", hbm_budget_frac: float = 0.8, hbm_budget_bytes: int = 0,
                 max_batch: int = 256, tie="reference", batch_timeout_ms: int = 60000, reserve_blocks: int = 0,
                 small_edges: int = 0, staging_bytes: int = 0):
        """small_edges: requests with at most this many edges take the small
        lane (0: 2^20, < 0: one lane); reserve_blocks: count-kernel block slots
        per SM the large lane leaves to the small one (0: 1, < 0: none);
        staging_bytes: pinned host area for submitted edge lists (0: 1 GiB,
        < 0: none)."""
        cfg = N.ServerConfig(hbm_budget_frac, hbm_budget_bytes, max_batch, _tie(tie), batch_timeout_ms,
                             reserve_blocks, small_edges, staging_bytes)
        h = C.c_void_p()
        N.call("tc_server_create", ctx.handle, C.byref(cfg), C.byref(h))
        self._h = h
        self.ctx = ctx

    def submit(self, src=None, dst=None, key: int = 0, n_nodes: int = 0) -> int:
        rid = C.c_uint64()
        if src is None:
            N.call("tc_server_submit", self._h, int(key), None, None, 0, int(n_nodes), C.byref(rid))
        else:
            s = np.ascontiguousarray(src, np.int64)
            d = np.ascontiguousarray(dst, np.int64)
            N.call("tc_server_submit", self._h, int(key), _ptr(s), _ptr(d), len(s), int(n_nodes), C.byref(rid))
        return rid.value

    def poll(self, rid: int):
        """(count, latency_ms) when done, None while pending; raises on failure."""
        c, lat = C.c_uint64(), C.c_double()
        st = N.lib().tc_server_poll(self._h, int(rid), C.byref(c), C.byref(lat))
        if st == -7:
            return None
        N.check(st, "tc_server_poll")
        return c.value, lat.value

    def wait(self, rid: int, timeout_ms: int = -1):
        c, lat = C.c_uint64(), C.c_double()
        N.call("tc_server_wait", self._h, int(rid), int(timeout_ms), C.byref(c), C.byref(lat))
        return c.value, lat.value

    def stats(self) -> dict:
        st = N.ServerStats()
        N.call("tc_server_get_stats", self._h, C.byref(st))
        return {k: getattr(st, k) for k, _ in N.ServerStats._fields_}

    def close(self) -> None:
        if getattr(self, "_h", None) is not None:
            N.lib().tc_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Context:
    """A CUDA device, a stream and libtc's scratch pool."""

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        N.call("tc_ctx_create", int(device), C.byref(h))
        self._h = h
        self.device = device

    @property
    def handle(self):
        return self._h

    def close(self) -> None:
        if getattr(self, "_h", None) is not None:
            N.lib().tc_ctx_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- device / stream / tuning ----
    @property
    def stream(self) -> int:
        return N.lib().tc_ctx_get_stream(self._h) or 0

    def set_stream(self, stream_ptr: int) -> None:
        N.call("tc_ctx_set_stream", self._h, C.c_void_p(stream_ptr))

    def synchronize(self) -> None:
        N.call("tc_ctx_synchronize", self._h)

    def last_count_kernel_ms(self) -> float:
        """Device time of the last plain count's counting kernel (CUDA events
        on the context's stream around it; waits for it)."""
        ms = C.c_float()
        N.call("tc_ctx_last_count_kernel_ms", self._h, C.byref(ms))
        return ms.value

    def device_info(self) -> dict:
        sm, f, t = C.c_int(), C.c_size_t(), C.c_size_t()
        N.call("tc_ctx_device_info", self._h, C.byref(sm), C.byref(f), C.byref(t))
        return {"sm_count": sm.value, "free_bytes": f.value, "total_bytes": t.value}

    def get_tuning(self) -> dict:
        t = N.Tuning()
        N.call("tc_ctx_get_tuning", self._h, C.byref(t))
        return {k: getattr(t, k) for k, _ in N.Tuning._fields_}

    def set_tuning(self, warp_max_deg: int = 0, light_max_work: int = 0, unit_work: int = 0, long_list: int = -1,
                   probe_kicks: int = -1, heavy_bitmap: int = -1, blocks_per_sm: int = -1,
                   hash_pairs: int = -1, flat_max_deg: int = -1, intersect: int = -1) -> None:
        t = N.Tuning(warp_max_deg, light_max_work, unit_work, long_list, probe_kicks, heavy_bitmap, blocks_per_sm,
                     hash_pairs, flat_max_deg, intersect)
        N.call("tc_ctx_set_tuning", self._h, C.byref(t))

    def autotune(self, g: "Graph", max_trials: int = 32, reps: int = 3, with_trials: bool = False):
        """Picks the fastest strategy thresholds for g by timing (sets them);
        returns (tuning, best ms) or, with_trials, (tuning, best ms, trials)."""
        t = N.Tuning()
        ms = C.c_float()
        n = C.c_int()
        N.call("tc_autotune_ex", self._h, g.handle, int(max_trials), int(reps), C.byref(t), C.byref(ms), C.byref(n))
        tun = {k: getattr(t, k) for k, _ in N.Tuning._fields_}
        return (tun, ms.value, n.value) if with_trials else (tun, ms.value)

    # ---- graphs ----
    def wrap_device(self, d_row_ptr: int, d_col: int, n_rows: int, nnz: int, n_roots: int | None = None) -> Graph:
        """A graph over caller-owned int32 device arrays (addresses), not copied
        and not validated; the caller keeps them alive."""
        h = C.c_void_p()
        N.call("tc_graph_wrap_device_i32", self._h, C.c_void_p(d_row_ptr), C.c_void_p(d_col), int(n_rows), int(nnz),
               int(n_rows if n_roots is None else n_roots), C.byref(h))
        return Graph(self, h)

    def upload(self, row_ptr: np.ndarray, col: np.ndarray, n_roots: int | None = None) -> Graph:
        """Upload an oriented CSR (int32, or u64 narrowed on the device)."""
        n_rows = len(row_ptr) - 1
        n_roots = n_rows if n_roots is None else int(n_roots)
        h = C.c_void_p()
        if row_ptr.dtype in (np.uint64, np.int64):
            rp = np.ascontiguousarray(row_ptr, np.uint64)
            cl = np.ascontiguousarray(col, np.uint64)
            N.call("tc_graph_upload_u64", self._h, _ptr(rp), _ptr(cl), n_rows, len(cl), n_roots, C.byref(h))
        else:
            rp = np.ascontiguousarray(row_ptr, np.int32)
            cl = np.ascontiguousarray(col, np.int32)
            N.call("tc_graph_upload_i32", self._h, _ptr(rp), _ptr(cl), n_rows, len(cl), n_roots, C.byref(h))
        return Graph(self, h)

    def count(self, g: Graph, stats: bool = False):
        out = C.c_uint64()
        st = N.CountStats()
        N.call("tc_count", self._h, g.handle, C.byref(out), C.byref(st))
        if stats:
            return out.value, {"count_ms": st.count_ms, "finalize_ms": st.finalize_ms,
                               "launches": st.launches, "heavy_units": st.heavy_units}
        return out.value

    def count_per_root(self, g: Graph) -> np.ndarray:
        out = np.empty(max(g.n_roots, 0), np.uint64)
        tot = C.c_uint64()
        N.call("tc_count_per_root", self._h, g.handle, _ptr(out), C.byref(tot))
        return out

    def count_csr(self, row_ptr: np.ndarray, col: np.ndarray) -> int:
        """End to end from host arrays: upload, validate, count, read back."""
        rp = np.ascontiguousarray(row_ptr, np.int32)
        cl = np.ascontiguousarray(col, np.int32)
        out = C.c_uint64()
        N.call("tc_count_csr_i32", self._h, _ptr(rp), _ptr(cl), len(rp) - 1, len(cl), C.byref(out))
        return out.value

    def count_parts_csr(self, parts: Sequence[tuple]) -> np.ndarray:
        """The partitioned path from host arrays: parts = [(row_ptr, col,
        n_roots), ...] (int32); upload, validate, one batched count."""
        rps = [np.ascontiguousarray(p[0], np.int32) for p in parts]
        cls = [np.ascontiguousarray(p[1], np.int32) for p in parts]
        n = len(parts)
        arr_rp = (C.c_void_p * n)(*[a.ctypes.data for a in rps])
        arr_cl = (C.c_void_p * n)(*[a.ctypes.data for a in cls])
        nr = (C.c_int64 * n)(*[len(a) - 1 for a in rps])
        nz = (C.c_int64 * n)(*[len(a) for a in cls])
        ro = (C.c_int64 * n)(*[int(p[2]) for p in parts])
        out = np.empty(n, np.uint64)
        tot = C.c_uint64()
        N.call("tc_count_parts_csr_i32", self._h, n, arr_rp, arr_cl, nr, nz, ro, _ptr(out), C.byref(tot))
        return out

    def count_each(self, graphs: Sequence[Graph]) -> np.ndarray:
        arr = (C.c_void_p * len(graphs))(*[g.handle for g in graphs])
        out = np.empty(len(graphs), np.uint64)
        N.call("tc_count_each", self._h, arr, len(graphs), _ptr(out))
        return out

    def batch(self, graphs: Sequence[Graph]) -> Batch:
        return Batch(self, graphs)

    def server(self, **kw) -> "Server":
        return Server(self, **kw)

    # ---- preprocessing ----
    def ugraph_from_edges(self, src: np.ndarray, dst: np.ndarray, n_nodes: int = 0) -> UGraph:
        s = np.ascontiguousarray(src, np.int64)
        d = np.ascontiguousarray(dst, np.int64)
        h = C.c_void_p()
        N.call("tc_ugraph_from_edges", self._h, _ptr(s), _ptr(d), len(s), int(n_nodes), C.byref(h))
        return UGraph(self, h)

    def upload_ugraph(self, row_ptr: np.ndarray, col: np.ndarray, deg: np.ndarray | None = None) -> UGraph:
        rp = np.ascontiguousarray(row_ptr, np.int64)
        cl = np.ascontiguousarray(col, np.int64)
        dg = None if deg is None else np.ascontiguousarray(deg, np.int64)
        h = C.c_void_p()
        N.call("tc_ugraph_upload_i64", self._h, _ptr(rp), _ptr(cl), _ptr(dg), len(rp) - 1, len(cl), C.byref(h))
        return UGraph(self, h)

    def orient(self, ug: UGraph, tie="reference") -> Graph:
        h = C.c_void_p()
        N.call("tc_orient", self._h, ug.handle, _tie(tie), C.byref(h))
        return Graph(self, h)

    def graph_from_edges(self, src: np.ndarray, dst: np.ndarray, n_nodes: int = 0, tie="reference") -> Graph:
        s = np.ascontiguousarray(src, np.int64)
        d = np.ascontiguousarray(dst, np.int64)
        h = C.c_void_p()
        N.call("tc_graph_from_edges", self._h, _ptr(s), _ptr(d), len(s), int(n_nodes), _tie(tie), C.byref(h))
        return Graph(self, h)

    def parts_lp(self, ug: UGraph, k: int, seed: int = 0x5EED1AB0, iterations: int = 20) -> np.ndarray:
        """Balanced label-propagation parts of ug's vertices (the stand-in for
        the reference's METIS assignment); int32 array of ug's row count."""
        out = np.empty(ug.info()[0], np.int32)
        N.call("tc_gen_parts_lp", self._h, ug.handle, int(k), int(seed), int(iterations), _ptr(out))
        return out

    def halo_extract(self, ug: UGraph, part: np.ndarray, k: int, tie="reference", mode="reference") -> list[Graph]:
        """Per-part halo subgraphs.  mode "reference": the round_clean_sg parts
        (1-hop halo, zero-in-degree halo peeled); "count": only halo vertices
        with an oriented in-edge from the part (smaller, same per-part counts)."""
        p = np.ascontiguousarray(part, np.int32)
        outs = (C.c_void_p * k)()
        if mode == "reference":
            N.call("tc_halo_extract", self._h, ug.handle, _ptr(p), int(k), _tie(tie), outs)
        else:
            N.call("tc_halo_extract_ex", self._h, ug.handle, _ptr(p), int(k), _tie(tie), N.HALO[mode], outs)
        return [Graph(self, C.c_void_p(outs[i])) for i in range(k)]
