"""ctypes binding of libtc (include/tc.h).

The library is the in-tree build at trianglecount_gb300/lib/libtc.so.  There is
no fallback: if it is missing, loading raises with the build command.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "lib", "libtc.so")

TC_OK = 0
STATUS = {
    -1: "TC_E_INVALID", -2: "TC_E_CUDA", -3: "TC_E_NOMEM", -4: "TC_E_RANGE", -5: "TC_E_FORMAT",
    -6: "TC_E_IO", -7: "TC_E_NOT_READY", -8: "TC_E_TIMEOUT", -9: "TC_E_NO_DEVICE", -10: "TC_E_STATE",
}
TIE = {"reference": 0, "id_asc": 1}
HALO = {"reference": 0, "count": 1}  # tc_halo_extract_ex modes (TC_HALO_*)


class TCError(RuntimeError):
    """A libtc call returned a negative status."""

    def __init__(self, status: int, func: str, message: str):
        self.status = status
        self.code = STATUS.get(status, str(status))
        super().__init__(f"{func}: {self.code}: {message}")


class Tuning(C.Structure):
    _fields_ = [("warp_max_deg", C.c_int32), ("light_max_work", C.c_int32), ("unit_work", C.c_int32),
                ("long_list", C.c_int32), ("probe_kicks", C.c_int32), ("heavy_bitmap", C.c_int32),
                ("blocks_per_sm", C.c_int32), ("hash_pairs", C.c_int32),
                ("flat_max_deg", C.c_int32), ("intersect", C.c_int32)]


class CountStats(C.Structure):
    _fields_ = [("count_ms", C.c_float), ("finalize_ms", C.c_float),
                ("launches", C.c_int32), ("heavy_units", C.c_int32)]


class ServerConfig(C.Structure):
    _fields_ = [("hbm_budget_frac", C.c_double), ("hbm_budget_bytes", C.c_int64), ("max_batch", C.c_int32),
                ("tie", C.c_int32), ("batch_timeout_ms", C.c_int32), ("reserve_blocks", C.c_int32),
                ("small_edges", C.c_int64), ("staging_bytes", C.c_int64)]


class ServerStats(C.Structure):
    _fields_ = [(n, C.c_int64) for n in ("submitted", "completed", "failed", "batches", "cache_hits", "evictions",
                                         "max_batch_seen", "budget_bytes", "used_bytes", "resident_graphs",
                                         "queued", "small_batches", "large_batches")]


vp = C.c_void_p
i64 = C.c_int64
i32 = C.c_int32
u64 = C.c_uint64
P = C.POINTER

# name -> (restype, argtypes); restype c_int means a status to check
_SIGS = {
    "tc_last_error": (C.c_char_p, []),
    "tc_status_string": (C.c_char_p, [C.c_int]),
    "tc_version": (C.c_int, []),
    "tc_ctx_create": (C.c_int, [C.c_int, P(vp)]),
    "tc_ctx_destroy": (C.c_int, [vp]),
    "tc_ctx_set_stream": (C.c_int, [vp, vp]),
    "tc_ctx_get_stream": (vp, [vp]),
    "tc_ctx_synchronize": (C.c_int, [vp]),
    "tc_ctx_last_count_kernel_ms": (C.c_int, [vp, P(C.c_float)]),
    "tc_ctx_device_info": (C.c_int, [vp, P(C.c_int), P(C.c_size_t), P(C.c_size_t)]),
    "tc_ctx_get_tuning": (C.c_int, [vp, P(Tuning)]),
    "tc_ctx_set_tuning": (C.c_int, [vp, P(Tuning)]),
    "tc_autotune": (C.c_int, [vp, vp, C.c_int, C.c_int, P(Tuning), P(C.c_float)]),
    "tc_autotune_ex": (C.c_int, [vp, vp, C.c_int, C.c_int, P(Tuning), P(C.c_float), P(C.c_int)]),
    "tc_graph_upload_i32": (C.c_int, [vp, vp, vp, i64, i64, i64, P(vp)]),
    "tc_graph_upload_u64": (C.c_int, [vp, vp, vp, i64, i64, i64, P(vp)]),
    "tc_graph_wrap_device_i32": (C.c_int, [vp, vp, vp, i64, i64, i64, P(vp)]),
    "tc_graph_info": (C.c_int, [vp, P(i64), P(i64), P(i64)]),
    "tc_graph_download_i32": (C.c_int, [vp, vp, vp, vp]),
    "tc_graph_destroy": (C.c_int, [vp]),
    "tc_count": (C.c_int, [vp, vp, P(u64), P(CountStats)]),
    "tc_count_async": (C.c_int, [vp, vp, vp]),
    "tc_count_per_root": (C.c_int, [vp, vp, vp, P(u64)]),
    "tc_count_csr_i32": (C.c_int, [vp, vp, vp, i64, i64, P(u64)]),
    "tc_count_noalloc_i32": (C.c_int, [vp, vp, i64, i64, i64, vp, vp]),
    "tc_batch_create": (C.c_int, [vp, P(vp), C.c_int, P(vp)]),
    "tc_batch_run": (C.c_int, [vp, vp]),
    "tc_batch_run_async": (C.c_int, [vp]),
    "tc_batch_results": (C.c_int, [vp, vp]),
    "tc_batch_destroy": (C.c_int, [vp]),
    "tc_batch_stats": (C.c_int, [vp, P(CountStats)]),
    "tc_count_parts_csr_i32": (C.c_int, [vp, C.c_int, P(vp), P(vp), P(i64), P(i64), P(i64), vp, P(u64)]),
    "tc_count_each": (C.c_int, [vp, P(vp), C.c_int, vp]),
    "tc_ugraph_from_edges": (C.c_int, [vp, vp, vp, i64, i64, P(vp)]),
    "tc_ugraph_upload_i64": (C.c_int, [vp, vp, vp, vp, i64, i64, P(vp)]),
    "tc_ugraph_info": (C.c_int, [vp, P(i64), P(i64)]),
    "tc_ugraph_download": (C.c_int, [vp, vp, vp, vp, vp]),
    "tc_ugraph_destroy": (C.c_int, [vp]),
    "tc_orient": (C.c_int, [vp, vp, C.c_int, P(vp)]),
    "tc_graph_from_edges": (C.c_int, [vp, vp, vp, i64, i64, C.c_int, P(vp)]),
    "tc_halo_extract": (C.c_int, [vp, vp, vp, C.c_int, C.c_int, P(vp)]),
    "tc_halo_extract_ex": (C.c_int, [vp, vp, vp, C.c_int, C.c_int, C.c_int, P(vp)]),
    "tc_server_create": (C.c_int, [vp, P(ServerConfig), P(vp)]),
    "tc_server_submit": (C.c_int, [vp, u64, vp, vp, i64, i64, P(u64)]),
    "tc_server_poll": (C.c_int, [vp, u64, P(u64), P(C.c_double)]),
    "tc_server_wait": (C.c_int, [vp, u64, i64, P(u64), P(C.c_double)]),
    "tc_server_get_stats": (C.c_int, [vp, P(ServerStats)]),
    "tc_server_destroy": (C.c_int, [vp]),
    "tc_text_read_u64": (C.c_int, [C.c_char_p, P(P(u64)), P(i64)]),
    "tc_host_free": (None, [vp]),
    "tc_text_write_line": (C.c_int, [C.c_char_p, vp, i64, C.c_int, C.c_char, C.c_int]),
    "tc_host_alloc_pinned": (C.c_int, [C.c_size_t, P(vp)]),
    "tc_host_free_pinned": (C.c_int, [vp]),
    "tc_read_edges": (C.c_int, [C.c_char_p, P(P(i64)), P(P(i64)), P(i64)]),
    "tc_tcsr_write": (C.c_int, [C.c_char_p, vp, vp, i64, i64, i64, i64]),
    "tc_tcsr_read_header": (C.c_int, [C.c_char_p, P(i64), P(i64), P(i64), P(i64)]),
    "tc_tcsr_read": (C.c_int, [C.c_char_p, vp, vp]),
    "tc_gen_rmat": (C.c_int, [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, u64, C.c_int, vp, vp]),
    "tc_gen_road": (C.c_int, [i64, i64, C.c_double, C.c_double, u64, vp, vp, P(i64)]),
    "tc_gen_er": (C.c_int, [i64, C.c_double, u64, vp, vp, P(i64)]),
    "tc_gen_chung_lu": (C.c_int, [i64, C.c_double, C.c_double, u64, vp, vp, i64]),
    "tc_gen_parts_random": (C.c_int, [i64, C.c_int, u64, vp]),
    "tc_gen_parts_contig": (C.c_int, [i64, C.c_int, vp]),
    "tc_gen_parts_lp": (C.c_int, [vp, vp, C.c_int, u64, C.c_int, vp]),
}

_lib = None


def lib() -> C.CDLL:
    """The loaded libtc, with prototypes set.  Raises if it is not built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"libtc.so is not built ({LIB_PATH}); run: python -c 'import __graft_entry__ as g; g.build()'")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(status: int, func: str) -> None:
    if status != TC_OK:
        msg = lib().tc_last_error().decode(errors="replace")
        raise TCError(status, func, msg)


def call(name: str, *args) -> None:
    """Call a status-returning entry point and raise TCError on failure."""
    check(getattr(lib(), name)(*args), name)


def declared_symbols() -> list[str]:
    return sorted(_SIGS)
