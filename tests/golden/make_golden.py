"""Writes tests/golden/small_graphs.json: hand-made graphs with the oracle's
generate() results (elevation bit patterns, iteration counts).

Run from the repository root:  python tests/golden/make_golden.py
Each case is solved by the C++ oracle and by the pure-Python restatement
(tests/pyref.py); the file is only written when the two agree bit for bit.
"""
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle as orc  # noqa: E402
from tests import graphs, pyref  # noqa: E402


def cases():
    rng = np.random.default_rng(2024)
    out = []

    def add(name, g, base=None, k=None, u=None, outlets=(), ms=None):
        n = g.n
        out.append(dict(
            name=name, g=g,
            base=list(map(float, np.zeros(n) if base is None else base)),
            k=list(map(float, np.ones(n) if k is None else k)),
            u=list(map(float, np.ones(n) if u is None else u)),
            is_outlet=[1 if i in set(outlets) else 0 for i in range(n)],
            max_slope=None if ms is None else [float(ms)] * n))

    add("line_default_outlet", graphs.line(8))
    add("star_lake_touching_all_outlets", graphs.star(6))
    # lake between two outlets: a low interior site adjacent to outlets 0 and 4
    g = graphs.from_edges(5, [(0, 1, 1.0), (1, 2, 1.0), (2, 3, 1.0), (3, 4, 1.0), (1, 3, 1.5)])
    add("lake_touching_two_outlets", g, base=[0, 0.5, 0.1, 0.5, 0], outlets=[0, 4])
    # two adjacent lakes sharing a ridge
    g = graphs.from_edges(7, [(0, 1, 1.0), (1, 2, 1.0), (2, 3, 1.0), (3, 4, 1.0), (4, 5, 1.0),
                              (5, 6, 1.0), (1, 3, 2.0), (3, 5, 2.0)])
    add("two_lakes_touching", g, base=[0, 0.6, 0.2, 0.7, 0.1, 0.8, 0], outlets=[0, 6])
    add("grid_equal_lengths", graphs.grid(5, 4, unit_lengths=True, seed=5))
    add("grid_jitter_noise_k", graphs.grid(6, 5, jitter=0.3, seed=6), k=rng.uniform(0.5, 2, 30),
        u=rng.uniform(0.5, 1.5, 30))
    add("unreached_component", graphs.two_components())
    add("grid_max_slope", graphs.grid(6, 6, jitter=0.25, seed=7), ms=0.314)
    g = graphs.random_delaunay(60, seed=8)
    add("delaunay60_outlets_listed", g, outlets=[int(o) for o in g.default_outlets[::2]],
        k=rng.uniform(0.5, 2, 60))
    return out


def main():
    result = []
    for c in cases():
        g = c.pop("g")
        base, k, u = np.array(c["base"]), np.array(c["k"]), np.array(c["u"])
        iso = np.array(c["is_outlet"], np.uint8)
        ms = None if c["max_slope"] is None else np.array(c["max_slope"])
        r = orc.generate(g, base, k, u, iso, max_slope=ms)
        pe, pit, _ = pyref.generate(g, base, k, u, iso, ms)
        bits = [pyref.f64_bits(x) for x in r["elev"]]
        assert r["iters"] == pit and bits == [pyref.f64_bits(x) for x in pe], c["name"]
        c.update(n=g.n, row_ptr=list(map(int, g.row_ptr)), col=list(map(int, g.col)),
                 length=list(map(float, g.length)), area=list(map(float, g.area)),
                 default_outlets=list(map(int, g.default_outlets)), iters=r["iters"],
                 elev_bits=["%016x" % b for b in bits])
        result.append(c)
        print(c["name"], "iters", r["iters"])
    with open(os.path.join(os.path.dirname(__file__), "small_graphs.json"), "w") as f:
        json.dump(result, f, indent=1)


if __name__ == "__main__":
    main()
