"""Served form: requests run concurrently through fl_server_* must each return exactly
what fl_generate returns for the same model and parameters alone -- with continuous
batching (waiting requests solved together as one packed model) or without, and when a
small HBM budget forces instances to be evicted and re-created."""
import math

import numpy as np
import pytest

from fastlem_gb300 import ParameterArrays, TerrainGenerator, workloads
from fastlem_gb300._lib import lib
from fastlem_gb300.serve import TerrainServer

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def requests():
    out = []
    for i, n in enumerate([2000, 9000, 600, 20000, 4000, 9000, 1200]):
        side = math.sqrt(n)
        m = workloads.build_model(n, side, 100 + i, 1)
        r = np.random.default_rng(100 + i)
        p = ParameterArrays(n, erodibility=np.exp(r.normal(0.0, 0.5, n)),
                            is_outlet=workloads.border_outlets(m, side, 0.03 * side),
                            max_slope=0.3 if i == 2 else None)
        out.append((m, p))
    return out


def solo(m, p, cap):
    g = TerrainGenerator.default().set_model(m).set_parameters(p).set_max_iteration(cap)
    return g.generate().elevations(), g.last_iterations


@pytest.mark.parametrize("budget_models,slots,packing", [(None, 3, True), (2, 2, True),
                                                          (None, 3, False), (2, 2, False)])
def test_requests_in_the_mix_equal_alone(requests, budget_models, slots, packing):
    cap = 30
    want = [solo(m, p, cap) for m, p in requests]
    # room for `budget_models` of the largest instance (admission reserves the bound
    # fl_model_device_bytes until an instance exists, then its measured size)
    bound = max(lib().fl_model_device_bytes(m.n, int(m.row_ptr[-1])) for m, _ in requests)
    real = max(lib().fl_graph_device_bytes(m.handle()) for m, _ in requests)
    assert real <= bound
    budget = 120 * 10**9 if budget_models is None else budget_models * bound
    with TerrainServer(hbm_budget_bytes=budget, slots=slots) as srv:
        srv.set_packing(packing)
        ids = [srv.add_model(m) for m, _ in requests]
        # every model twice, interleaved: resident instances get reused
        order = list(range(len(requests))) * 2
        tickets = [srv.submit(ids[i], requests[i][1], cap) for i in order]
        got = [srv.wait(t) for t in tickets]
        stats = srv.stats()
    for i, (t, info) in zip(order, got):
        we, wi = want[i]
        assert np.array_equal(t.elevations().view(np.uint64), we.view(np.uint64)), f"request {i}"
        assert info["iterations"] == wi
        assert info["latency_ms"] >= info["solve_ms"] >= 0
    assert stats["completed"] == len(order)
    if not packing:
        assert stats["packed_solves"] == 0
    elif budget_models is None:
        assert stats["packed_requests"] >= 2      # the burst shares packed solves
    if budget_models is not None:
        if not packing:
            assert stats["instances_evicted"] > 0
        assert stats["peak_device_bytes"] <= budget
