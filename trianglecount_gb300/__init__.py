"""GB300-native exact triangle counting (drop-in for the KishantLab/TriangleCount
TC_128 / wo_sort_tc_256 / round_clean_sg path).

The compute lives in libtc (CUDA, sm_103a; C ABI in include/tc.h).  This
package is its Python host side: ctypes bindings, the reference's file
formats and seeded synthetic inputs.
"""
from ._native import TCError, lib  # noqa: F401
from .api import Batch, Context, Graph, Server, UGraph  # noqa: F401

__all__ = ["Context", "Graph", "UGraph", "Batch", "Server", "TCError", "lib"]
