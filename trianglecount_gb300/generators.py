"""Seeded synthetic graphs for the benchmark workloads (libtc's host
generators; integer-only draws for R-MAT, road grid, ER and partitions).

The reference's real datasets are not available, so these stand in for them:

  rmat(16|21|23)  R-MAT, edge factor 16, (a, b, c) = (0.57, 0.19, 0.19), seeded
                  vertex permutation
  road()          jittered-grid planar graph, 1448 x 1448 = 2,096,704 vertices,
                  4-neighbour edges each deleted with p = 0.15, random diagonals
  er / chung_lu   the uneven-batch families
  batch_mix()     256 graphs: ER n in [1e3, 1e5] with mean degree in [8, 64],
                  Chung-Lu gamma 2.1 n in [1e4, 1e6] capped at sqrt(2E),
                  R-MAT scale in [10, 18]; one third each, sizes log-uniform
  parts_random()  seeded uniform vertex -> part map (the reference's
                  np.random.randint, Halo_creation_preprocess.py:288, is unseeded)
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field

import numpy as np

from . import _native as N

RMAT_A, RMAT_B, RMAT_C = 0.57, 0.19, 0.19
SEED = {
    "rmat16": 0x5EED0016, "rmat21": 0x5EED0021, "rmat23": 0x5EED0023, "road": 0x5EED20AD,
    "parts": 0x5EED9A27, "batch": 0x5EEDBA7C, "serve": 0x5EED5E7E,
}
ROAD_SIDE = 1448
ROAD_P_DELETE = 0.15
ROAD_DIAG_RATE = 0.05


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def rmat(scale: int, edge_factor: int = 16, a: float = RMAT_A, b: float = RMAT_B, c: float = RMAT_C,
         seed: int | None = None, permute: bool = True) -> tuple[np.ndarray, np.ndarray]:
    n = edge_factor << scale
    src = np.empty(n, np.int64)
    dst = np.empty(n, np.int64)
    seed = SEED.get(f"rmat{scale}", 0x5EED0000 + scale) if seed is None else seed
    N.call("tc_gen_rmat", scale, edge_factor, a, b, c, seed, 1 if permute else 0, _p(src), _p(dst))
    return src, dst


def road(side: int = ROAD_SIDE, p_delete: float = ROAD_P_DELETE, diag_rate: float = ROAD_DIAG_RATE,
         seed: int | None = None, height: int | None = None) -> tuple[np.ndarray, np.ndarray]:
    h = side if height is None else height
    cap = 3 * side * h
    src = np.empty(cap, np.int64)
    dst = np.empty(cap, np.int64)
    m = C.c_int64()
    N.call("tc_gen_road", side, h, p_delete, diag_rate, SEED["road"] if seed is None else seed, _p(src), _p(dst),
           C.byref(m))
    return src[:m.value].copy(), dst[:m.value].copy()


def er(n: int, avg_deg: float, seed: int) -> tuple[np.ndarray, np.ndarray]:
    p = min(1.0, avg_deg / (n - 1))
    cap = int(round(p * n * (n - 1) / 2)) + 1
    src = np.empty(cap, np.int64)
    dst = np.empty(cap, np.int64)
    m = C.c_int64(cap)
    N.call("tc_gen_er", n, p, seed, _p(src), _p(dst), C.byref(m))
    return src[:m.value].copy(), dst[:m.value].copy()


def chung_lu(n: int, avg_deg: float, seed: int, gamma: float = 2.1) -> tuple[np.ndarray, np.ndarray]:
    m = int(round(n * avg_deg / 2))
    src = np.empty(m, np.int64)
    dst = np.empty(m, np.int64)
    N.call("tc_gen_chung_lu", n, gamma, avg_deg, seed, _p(src), _p(dst), m)
    return src, dst


def parts_random(n: int, k: int, seed: int | None = None) -> np.ndarray:
    part = np.empty(n, np.int32)
    N.call("tc_gen_parts_random", n, k, (SEED["parts"] + k) if seed is None else seed, _p(part))
    return part


def parts_contig(n: int, k: int) -> np.ndarray:
    """Contiguous parts as Halo_creation_preprocess.py:293-299 builds them."""
    part = np.empty(n, np.int32)
    N.call("tc_gen_parts_contig", n, k, _p(part))
    return part


class SplitMix64:
    """Deterministic parameter draws (same on every platform)."""

    def __init__(self, seed: int):
        self.s = seed & 0xFFFFFFFFFFFFFFFF

    def next(self) -> int:
        self.s = (self.s + 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF
        z = self.s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & 0xFFFFFFFFFFFFFFFF
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & 0xFFFFFFFFFFFFFFFF
        return z ^ (z >> 31)

    def uniform(self) -> float:
        return (self.next() >> 11) * (1.0 / (1 << 53))

    def log_uniform(self, lo: float, hi: float) -> float:
        return math.exp(math.log(lo) + self.uniform() * (math.log(hi) - math.log(lo)))

    def randint(self, lo: int, hi: int) -> int:  # inclusive
        return lo + (self.next() * (hi - lo + 1) >> 64)


@dataclass
class GraphSpec:
    kind: str
    params: dict = field(default_factory=dict)
    seed: int = 0

    def edges(self) -> tuple[np.ndarray, np.ndarray]:
        if self.kind == "er":
            return er(self.params["n"], self.params["avg_deg"], self.seed)
        if self.kind == "chung_lu":
            return chung_lu(self.params["n"], self.params["avg_deg"], self.seed)
        if self.kind == "rmat":
            return rmat(self.params["scale"], 16, seed=self.seed)
        raise ValueError(self.kind)

    def label(self) -> str:
        return self.kind + "(" + ",".join(f"{k}={v}" for k, v in self.params.items()) + ")"


def batch_mix(n_graphs: int = 256, seed: int | None = None, scale: float = 1.0) -> list[GraphSpec]:
    """The uneven batch: ER / Chung-Lu / R-MAT in turn, sizes log-uniform.
    scale < 1 shrinks every size range (for quick tests)."""
    r = SplitMix64(SEED["batch"] if seed is None else seed)
    out = []
    for i in range(n_graphs):
        kind = ("er", "chung_lu", "rmat")[i % 3]
        gseed = r.next()
        if kind == "er":
            n = int(r.log_uniform(1e3 * scale, 1e5 * scale))
            out.append(GraphSpec("er", {"n": max(n, 16), "avg_deg": round(r.log_uniform(8, 64), 3)}, gseed))
        elif kind == "chung_lu":
            n = int(r.log_uniform(1e4 * scale, 1e6 * scale))
            out.append(GraphSpec("chung_lu", {"n": max(n, 16), "avg_deg": round(r.log_uniform(8, 32), 3)}, gseed))
        else:
            hi = 18 if scale >= 1.0 else max(10, int(18 + math.log2(scale)))
            out.append(GraphSpec("rmat", {"scale": r.randint(10 if scale >= 1.0 else 6, hi)}, gseed))
    return out
