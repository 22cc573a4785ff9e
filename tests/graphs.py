"""Small graphs for parity tests: CSR built from an edge list in `add_edge` order
(terrain-graph appends (b, w) to a's row and (a, w) to b's row), as fastlem's
builder fills the graph (builder.rs:251-268)."""
import math
from dataclasses import dataclass

import numpy as np


@dataclass
class Graph:
    n: int
    row_ptr: np.ndarray
    col: np.ndarray
    length: np.ndarray
    area: np.ndarray
    default_outlets: np.ndarray
    xs: np.ndarray = None
    ys: np.ndarray = None


def from_edges(n, edges, area=None, default_outlets=(), xs=None, ys=None):
    rows = [[] for _ in range(n)]
    for a, b, w in edges:
        rows[a].append((b, w))
        rows[b].append((a, w))
    row_ptr = np.zeros(n + 1, np.uint32)
    for i in range(n):
        row_ptr[i + 1] = row_ptr[i] + len(rows[i])
    col = np.array([j for r in rows for (j, _) in r], np.uint32)
    length = np.array([w for r in rows for (_, w) in r], np.float64)
    area = np.ones(n, np.float64) if area is None else np.asarray(area, np.float64)
    return Graph(n, row_ptr, col, length, area, np.asarray(default_outlets, np.uint32),
                 None if xs is None else np.asarray(xs, np.float64),
                 None if ys is None else np.asarray(ys, np.float64))


def from_csr(c):
    """Graph from a golden-fixture dict (row_ptr, col, length, area, default_outlets)."""
    return Graph(c["n"], np.array(c["row_ptr"], np.uint32), np.array(c["col"], np.uint32),
                 np.array(c["length"], np.float64), np.array(c["area"], np.float64),
                 np.array(c["default_outlets"], np.uint32))


def from_model(m):
    return Graph(m.n, m.row_ptr, m.col, m.length, m.area, m.default_outlets, m.xs, m.ys)


def line(n=6):
    """0 - 1 - ... - n-1, outlet 0 by default."""
    return from_edges(n, [(i, i + 1, 1.0 + 0.25 * i) for i in range(n - 1)], default_outlets=[0])


def star(leaves=6):
    """Centre 0 joined to leaves; every leaf-to-centre edge has length 1 (ties)."""
    return from_edges(leaves + 1, [(0, i, 1.0) for i in range(1, leaves + 1)],
                      default_outlets=list(range(1, leaves + 1)))


def grid(w, h, jitter=0.0, seed=0, unit_lengths=False):
    """w x h lattice with diagonals; unit_lengths makes every edge length 1.0 (ties
    everywhere); otherwise lengths are Euclidean on jittered points."""
    rng = np.random.default_rng(seed)
    xs = np.repeat(np.arange(w, dtype=np.float64)[None, :], h, 0).ravel()
    ys = np.repeat(np.arange(h, dtype=np.float64)[:, None], w, 1).ravel()
    if jitter:
        xs = xs + rng.uniform(-jitter, jitter, xs.shape)
        ys = ys + rng.uniform(-jitter, jitter, ys.shape)
    idx = lambda x, y: y * w + x
    edges = []
    for y in range(h):
        for x in range(w):
            for dx, dy in ((1, 0), (0, 1), (1, 1)):
                X, Y = x + dx, y + dy
                if X < w and Y < h:
                    a, b = idx(x, y), idx(X, Y)
                    d = 1.0 if unit_lengths else math.sqrt((xs[a] - xs[b]) ** 2 + (ys[a] - ys[b]) ** 2)
                    edges.append((a, b, d))
    hull = [idx(x, 0) for x in range(w)] + [idx(w - 1, y) for y in range(1, h)] + \
           [idx(x, h - 1) for x in range(w - 2, -1, -1)] + [idx(0, y) for y in range(h - 2, 0, -1)]
    return from_edges(w * h, edges, area=rng.uniform(0.5, 1.5, w * h), default_outlets=hull,
                      xs=xs, ys=ys)


def two_components():
    """A path 0-1-2 (outlet 0) and a separate triangle 3-4-5 with no outlet."""
    return from_edges(6, [(0, 1, 1.0), (1, 2, 1.0), (3, 4, 1.0), (4, 5, 2.0), (3, 5, 1.5)],
                      default_outlets=[0])


def random_delaunay(n, seed, side=10.0):
    """Delaunay graph of n uniform sites via the product's own builder."""
    from fastlem_gb300 import TerrainModel2DBulider, Site2D
    m = TerrainModel2DBulider.from_random_sites(n, Site2D(0, 0), Site2D(side, side), seed=seed).build()
    return from_model(m)
