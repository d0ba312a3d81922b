"""Small graphs with known triangle counts (pairs arrays), shared by the tests."""
from __future__ import annotations

import numpy as np
from math import comb


def complete(n: int, offset: int = 0):
    p = np.array([[i, j] for i in range(n) for j in range(i + 1, n)], dtype=np.int32).reshape(-1, 2)
    return p + offset, comb(n, 3)


def grid(n: int, diagonals: int, offset: int = 0):
    """n x n grid; diagonals = 0 (none), 1 (one per cell: a triangulated mesh), 2 (king graph)."""
    ids = np.arange(n * n).reshape(n, n) + offset
    e = [np.stack([ids[:, :-1].ravel(), ids[:, 1:].ravel()], 1), np.stack([ids[:-1, :].ravel(), ids[1:, :].ravel()], 1)]
    if diagonals >= 1:
        e.append(np.stack([ids[:-1, :-1].ravel(), ids[1:, 1:].ravel()], 1))
    if diagonals >= 2:
        e.append(np.stack([ids[:-1, 1:].ravel(), ids[1:, :-1].ravel()], 1))
    tri = {0: 0, 1: 2 * (n - 1) ** 2, 2: 4 * (n - 1) ** 2}[diagonals]
    return np.concatenate(e).astype(np.int32), tri


def star(n: int, offset: int = 0):
    return np.array([[offset, offset + i] for i in range(1, n)], dtype=np.int32).reshape(-1, 2), 0


def path(n: int, offset: int = 0):
    return np.array([[offset + i, offset + i + 1] for i in range(n - 1)], dtype=np.int32).reshape(-1, 2), 0


def bipartite(a: int, b: int, offset: int = 0):
    return np.array([[offset + i, offset + a + j] for i in range(a) for j in range(b)], dtype=np.int32).reshape(-1, 2), 0


def union(*parts):
    """Disjoint union: each part is (pairs, triangles) built with distinct offsets."""
    return np.concatenate([p for p, _ in parts]).astype(np.int32), sum(t for _, t in parts)


def kat_cases():
    """(name, pairs, triangles) known-answer cases."""
    cases = [("K3", *complete(3)), ("K4", *complete(4)), ("K30", *complete(30)), ("K200", *complete(200)),
             ("grid20_0", *grid(20, 0)), ("grid20_1", *grid(20, 1)), ("grid20_2", *grid(20, 2)),
             ("star500", *star(500)), ("path300", *path(300)), ("K40_60", *bipartite(40, 60))]
    u = union(complete(25), grid(15, 2, offset=25), star(50, offset=25 + 225), complete(7, offset=300))
    cases.append(("union", *u))
    return cases


def random_csr(rng, n: int, max_deg: int, dup_prob: float = 0.1, self_prob: float = 0.02):
    """Arbitrary (not oriented, unsorted, with duplicates and self-loops) CSR for formula tests."""
    deg = rng.integers(0, max_deg + 1, size=n)
    beg = np.zeros(n + 1, dtype=np.int64)
    beg[1:] = np.cumsum(deg)
    adj = rng.integers(0, n, size=int(beg[-1])).astype(np.int32)
    for v in range(n):
        row = adj[beg[v]:beg[v + 1]]
        if row.size > 1 and rng.random() < dup_prob:
            row[-1] = row[0]
        if row.size and rng.random() < self_prob:
            row[0] = v
    return beg, adj
