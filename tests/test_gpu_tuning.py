"""Every launch shape the schedule can choose gives the same bits.

The top-down Kahn rounds (1, 2 or 4 sites in flight per thread), the number of chain
walkers per SM, whole-GPU or model-sized cooperative grids and the Kahn stop width (where the chain walks take over) only change
how the exact recurrences are scheduled, never their evaluation order, so generate()
must return the oracle's elevations and iteration count under each of them."""
import numpy as np
import pytest

from fastlem_gb300 import TerrainGenerator, workloads
from fastlem_gb300 import _lib
from tests import graphs

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cases(orc):
    out = []
    for w, iters in ((workloads.one_million(scale=0.2), 6),
                     (workloads.small(scale=0.5, max_slope=0.314), 10)):
        p = w.params
        r = orc.generate(graphs.from_model(w.model), p.base, p.erodibility, p.uplift,
                         p.is_outlet, max_slope=p.max_slope, max_iter=iters)
        out.append((w, iters, r))
    return out


def _check(cases):
    for w, iters, r in cases:
        w.model.release()                      # a new model picks up the stop width
        gen = TerrainGenerator.default().set_model(w.model).set_parameters(w.params)
        got = gen.set_max_iteration(iters).generate().elevations()
        assert gen.last_iterations == r["iters"], w.name
        assert np.array_equal(got.view(np.uint64), r["elev"].view(np.uint64)), w.name
        w.model.release()


@pytest.mark.parametrize("sized_grids", [0, 1])
@pytest.mark.parametrize("walk_per_sm", [0, 2])
@pytest.mark.parametrize("low_ilp", [1, 2, 4])
def test_launch_shapes_give_the_oracle_bits(cases, walk_per_sm, low_ilp, sized_grids):
    old = _lib.set_tuning(low_ilp=low_ilp, walk_per_sm=walk_per_sm, sized_grids=sized_grids)
    try:
        _check(cases)
    finally:
        _lib.set_tuning(**old)


@pytest.mark.parametrize("width", [256, 4096, 65536])
def test_kahn_stop_widths_give_the_oracle_bits(cases, width):
    old = _lib.set_tuning(kahn_min_width=width)
    try:
        _check(cases)
    finally:
        _lib.set_tuning(**old)
