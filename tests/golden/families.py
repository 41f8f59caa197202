"""Closed-form graph families with known triangle counts (known-answer tests).

Each builder returns (src, dst, n_nodes) as int64 numpy arrays; expected()
gives the count from the family's formula, not from any counter.
"""
from __future__ import annotations

from math import comb

import numpy as np


def _arr(edges):
    if not edges:
        return np.empty(0, np.int64), np.empty(0, np.int64)
    a = np.asarray(edges, np.int64)
    return a[:, 0].copy(), a[:, 1].copy()


def complete(n):
    i, j = np.triu_indices(n, 1)
    return i.astype(np.int64), j.astype(np.int64), n


def cycle(n):
    return _arr([(i, (i + 1) % n) for i in range(n)]) + (n,)


def star(n):
    return _arr([(0, i) for i in range(1, n + 1)]) + (n + 1,)


def wheel(n):  # hub 0 + rim 1..n
    e = [(0, i) for i in range(1, n + 1)] + [(i, i % n + 1) for i in range(1, n + 1)]
    return _arr(e) + (n + 1,)


def grid(a, b, diag=False):
    e = []
    for y in range(a):
        for x in range(b):
            v = y * b + x
            if x + 1 < b:
                e.append((v, v + 1))
            if y + 1 < a:
                e.append((v, v + b))
            if diag and x + 1 < b and y + 1 < a:
                e.append((v, v + b + 1))
    return _arr(e) + (a * b,)


def bipartite(a, b):
    return _arr([(i, a + j) for i in range(a) for j in range(b)]) + (a + b,)


def tripartite(a, b, c):
    parts = [range(0, a), range(a, a + b), range(a + b, a + b + c)]
    e = [(u, v) for p in range(3) for q in range(p + 1, 3) for u in parts[p] for v in parts[q]]
    return _arr(e) + (a + b + c,)


def friendship(k):  # k triangles sharing vertex 0
    e = []
    for t in range(k):
        x, y = 2 * t + 1, 2 * t + 2
        e += [(0, x), (0, y), (x, y)]
    return _arr(e) + (2 * k + 1,)


def book(k):  # k triangles sharing edge (0, 1)
    e = [(0, 1)] + [(0, i) for i in range(2, k + 2)] + [(1, i) for i in range(2, k + 2)]
    return _arr(e) + (k + 2,)


def windmill(k, n):  # k copies of K_n sharing vertex 0
    e = []
    for c in range(k):
        vs = [0] + [1 + c * (n - 1) + i for i in range(n - 1)]
        e += [(vs[i], vs[j]) for i in range(n) for j in range(i + 1, n)]
    return _arr(e) + (1 + k * (n - 1),)


def disjoint_complete(sizes):
    e, base = [], 0
    for s in sizes:
        e += [(base + i, base + j) for i in range(s) for j in range(i + 1, s)]
        base += s
    return _arr(e) + (base,)


def messy_complete(n, seed=7):
    """K_n relabelled, every edge listed twice (both directions), plus self-loops
    and isolated ids: the clean-up must reduce it to K_n."""
    rng = np.random.default_rng(seed)
    perm = rng.permutation(3 * n)[:n] + 5
    i, j = np.triu_indices(n, 1)
    u = np.concatenate([perm[i], perm[j], perm[:10]])
    v = np.concatenate([perm[j], perm[i], perm[:10]])
    order = rng.permutation(len(u))
    return u[order].astype(np.int64), v[order].astype(np.int64), int(perm.max()) + 3


def empty(n):
    return np.empty(0, np.int64), np.empty(0, np.int64), n


FAMILIES = {
    "complete": (complete, lambda n: comb(n, 3)),
    "cycle": (cycle, lambda n: 1 if n == 3 else 0),
    "star": (star, lambda n: 0),
    "wheel": (wheel, lambda n: 4 if n == 3 else n),
    "grid": (lambda a, b: grid(a, b), lambda a, b: 0),
    "tri_grid": (lambda a, b: grid(a, b, True), lambda a, b: 2 * (a - 1) * (b - 1)),
    "bipartite": (bipartite, lambda a, b: 0),
    "tripartite": (tripartite, lambda a, b, c: a * b * c),
    "friendship": (friendship, lambda k: k),
    "book": (book, lambda k: k),
    "windmill": (windmill, lambda k, n: k * comb(n, 3)),
    "disjoint_complete": (lambda *s: disjoint_complete(s), lambda *s: sum(comb(x, 3) for x in s)),
    "messy_complete": (messy_complete, lambda n: comb(n, 3)),
    "empty": (empty, lambda n: 0),
}

CASES = [
    ("complete", [3]), ("complete", [4]), ("complete", [5]), ("complete", [33]), ("complete", [200]),
    ("complete", [700]), ("cycle", [3]), ("cycle", [4]), ("cycle", [1000]), ("star", [5000]),
    ("wheel", [3]), ("wheel", [10]), ("wheel", [3000]), ("grid", [40, 50]), ("tri_grid", [40, 50]),
    ("bipartite", [30, 70]), ("tripartite", [5, 20, 40]), ("friendship", [300]), ("book", [2000]),
    ("windmill", [20, 40]), ("disjoint_complete", [5, 7, 130]), ("messy_complete", [150]), ("empty", [10]),
]


def build(name, args):
    return FAMILIES[name][0](*args)


def expected(name, args):
    return FAMILIES[name][1](*args)
