"""Writes tests/golden/c2_converged.json: the oracle's converged solve of the 1M-site
configuration (1,000,000 sites in [0,1000]^2, seed 7, one Lloyd relaxation, border
outlets within 5.0, erodibility clamp(exp(N(0,0.5)) * (0.5 + V), 0.1, 4)).

The oracle needs about 800 iterations (several minutes on one core) to reach the
iteration that changes nothing, too long to repeat inside every GPU test run, so the
result is recorded here as digests: SHA-256 of the model and parameter arrays (the
inputs), the iteration count, and SHA-256 of the elevation bit patterns.  The GPU test
compares against these digests when its inputs hash the same (the generators use
numpy's exp and normal sampler, whose last bits may differ between machines), and runs
the oracle itself otherwise.

    python tests/golden/make_c2_converged.py
"""
import hashlib
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)


def input_digest(g, p):
    h = hashlib.sha256()
    for a in (g.row_ptr, g.col, g.length, g.area, g.default_outlets, p.base, p.erodibility,
              p.uplift, p.is_outlet):
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def elev_digest(e):
    return hashlib.sha256(np.ascontiguousarray(e, np.float64).view(np.uint64).tobytes()).hexdigest()


def main():
    from fastlem_gb300 import workloads
    from oracle import oracle as orc
    from tests import graphs
    w = workloads.one_million()
    g, p = graphs.from_model(w.model), w.params
    t = time.time()
    r = orc.generate(g, p.base, p.erodibility, p.uplift, p.is_outlet)
    out = {"config": "1m", "sites": int(g.n), "input_sha256": input_digest(g, p),
           "iterations": int(r["iters"]), "elev_sha256": elev_digest(r["elev"]),
           "elev_bits_head": [f"{int(b):016x}" for b in r["elev"][:8].view(np.uint64)],
           "oracle_seconds": round(time.time() - t, 1)}
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "c2_converged.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
