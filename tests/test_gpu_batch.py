"""Batched form: terrains packed into one graph (fl_batch_create / fl_batch_generate)
must give, terrain by terrain, the bit-identical elevations and the same iteration
counts as solving each terrain alone with fl_generate -- and, for one of them, the
oracle's."""
import math

import numpy as np
import pytest

from fastlem_gb300 import ParameterArrays, TerrainGenerator, workloads
from fastlem_gb300.batch import BatchGenerator, TerrainBatch

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a, np.float64).view(np.uint64)


def terrain_cases():
    """Uneven sizes; border outlets, default (hull) outlets, a slope limit, lakes."""
    out = []
    specs = [(300, 11, "border", None), (2500, 12, "default", None), (900, 13, "border", 0.2),
             (4000, 14, "one", None), (64, 15, "border", None), (1500, 16, "border", None)]
    for n, seed, outl, slope in specs:
        side = math.sqrt(n)
        m = workloads.build_model(n, side, seed, 1 if n > 100 else 0)
        r = np.random.default_rng(seed)
        k = np.exp(r.normal(0.0, 0.5, n))
        # uplift 1 and base 0 (fastlem's defaults) settle in a few tens of iterations;
        # two terrains get uneven uplift and base elevations and run to the bound
        uneven = seed in (13, 14)
        u = r.uniform(0.5, 1.5, n) if uneven else np.ones(n)
        base = r.uniform(0.0, 2.0, n) if uneven else np.zeros(n)
        if outl == "border":
            is_o = workloads.border_outlets(m, side, 0.05 * side)
        elif outl == "one":              # a single outlet: every other basin is a lake
            is_o = np.zeros(n, bool)
            is_o[int(np.argmin(m.xs))] = True
        else:
            is_o = np.zeros(n, bool)
        p = ParameterArrays(n, base_elevation=base, erodibility=k, uplift_rate=u, is_outlet=is_o,
                            max_slope=slope)
        out.append((m, p))
    return out


@pytest.fixture(scope="module")
def cases():
    return terrain_cases()


def solo(m, p, max_iteration=None):
    g = TerrainGenerator.default().set_model(m).set_parameters(p)
    if max_iteration is not None:
        g.set_max_iteration(max_iteration)
    t = g.generate()
    return t.elevations(), g.last_iterations


# fastlem iterates until an iteration changes nothing; terrains with random uplift can
# take very long to get there, so the comparisons run a bounded number of iterations
# (the batch's fixed-point handling is covered by terrains converging before the bound)
@pytest.mark.parametrize("max_iteration", [40, 3])
def test_batch_matches_solo_generate(cases, max_iteration):
    want = [solo(m, p, max_iteration) for m, p in cases]
    bg = BatchGenerator().set_models([m for m, _ in cases]).set_parameters([p for _, p in cases])
    if max_iteration is not None:
        bg.set_max_iteration(max_iteration)
    got = bg.generate()
    for t, ((we, wi), ge) in enumerate(zip(want, got)):
        bad = np.nonzero(bits(ge.elevations()) != bits(we))[0]
        assert len(bad) == 0, f"terrain {t}: {len(bad)} sites differ"
        assert int(bg.last_terrain_iterations[t]) == wi, f"terrain {t} iterations"
    assert bg.last_iterations == max(wi for _, wi in want)
    if max_iteration == 40:               # some terrains converged inside the bound
        assert min(wi for _, wi in want) < 40


def test_batch_matches_oracle(cases, orc):
    m, p = cases[3]
    from tests.graphs import from_model
    g = from_model(m)
    r = orc.generate(g, p.base, p.erodibility, p.uplift, p.is_outlet, max_slope=p.max_slope,
                     max_iter=40)
    bg = BatchGenerator().set_models([mm for mm, _ in cases]).set_parameters([pp for _, pp in cases])
    got = bg.set_max_iteration(40).generate()[3].elevations()
    assert np.array_equal(bits(got), bits(r["elev"]))
    assert int(bg.last_terrain_iterations[3]) == r["iters"]


def test_batch_of_one_and_repeated_generate(cases):
    m, p = cases[1]
    we, wi = solo(m, p, 40)
    b = TerrainBatch([m])
    bg = BatchGenerator().set_batch(b).set_parameters([p]).set_max_iteration(40)
    for _ in range(2):                     # the packed graph stays resident
        got = bg.generate()[0].elevations()
        assert np.array_equal(bits(got), bits(we))
        assert int(bg.last_terrain_iterations[0]) == wi


def test_batch_to_convergence_matches_solo(cases):
    """Without a bound every terrain runs to its own first unchanged iteration; the
    terrains that settle first sit out the later iterations of the packed solve (their
    sites take no part in the passes) and must still equal their solo solves."""
    picked = [cases[i] for i in (0, 1, 4, 5)]        # fastlem's default uplift: they settle
    want = [solo(m, p) for m, p in picked]
    assert len(set(wi for _, wi in want)) > 1         # they settle at different iterations
    bg = BatchGenerator().set_models([m for m, _ in picked]).set_parameters([p for _, p in picked])
    got = bg.generate()
    for t, ((we, wi), ge) in enumerate(zip(want, got)):
        assert np.array_equal(bits(ge.elevations()), bits(we)), f"terrain {t}"
        assert int(bg.last_terrain_iterations[t]) == wi, f"terrain {t} iterations"
    assert bg.last_iterations == max(wi for _, wi in want)
