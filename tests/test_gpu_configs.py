"""GPU parity on the benchmarked configurations themselves.

The 16M-site terrain (16,000,000 sites uniform in [0,4000]^2, seed 11, outlets within
5.0 of the left and bottom borders, erodibility 1 + 0.8 * (2V - 1)) is the workload of
every throughput figure, and the one whose long rivers (~23,000 sites), deep receiver
forest and tens of thousands of skeleton chains reach the paths that small cases
barely touch: long exact folds, chain hand-offs at confluences, full chain tables.
Its solve is checked for two bounded iterations through the public API, and the
receivers, basin labels and re-routed receivers of both iterations' inputs through
the probes, all against the oracle, bit for bit.

The 1M-site configuration (1,000,000 sites in [0,1000]^2, seed 7, one Lloyd
relaxation, border outlets within 5.0, log-normal erodibility modulated by value
noise) is solved to convergence: fastlem's loop runs until an iteration changes no
elevation (src/lem/generator.rs:140-210), and the GPU must stop at the same iteration
with the same bits.
"""
import ctypes

import numpy as np
import pytest

from fastlem_gb300 import TerrainGenerator, workloads
from fastlem_gb300._lib import check, lib, ptr
from tests import graphs

pytestmark = pytest.mark.gpu


def _bits_equal(got, want, what):
    g = np.ascontiguousarray(got, np.float64).view(np.uint64)
    w = np.ascontiguousarray(want, np.float64).view(np.uint64)
    bad = np.nonzero(g != w)[0]
    assert len(bad) == 0, f"{what}: {len(bad)} sites differ, first {bad[:5]}"


def _check_stream_tree(orc, g, h, elev, table, outlets, want_final):
    """Receivers, labels and re-routed receivers for elevations `elev` through the
    probes, against the oracle's initial tree, roots and lake heap."""
    n = g.n
    want_next = orc.initial_tree(g, elev, table)
    got_next = np.empty(n, np.uint32)
    hl = ctypes.c_int()
    check(lib().fl_probe_receivers(h, ptr(elev), ptr(table), ptr(got_next), ctypes.byref(hl)))
    assert np.array_equal(got_next, want_next), \
        f"receivers: {int((got_next != want_next).sum())} differ"
    sub, has_lake = orc.roots(table, want_next)
    assert bool(hl.value) == has_lake
    if not has_lake:
        assert np.array_equal(want_next, want_final)
        return 0
    rerouted = np.empty(n, np.uint32)
    labels = np.empty(n, np.uint32)
    check(lib().fl_probe_lakes(h, ptr(outlets), len(outlets), ptr(want_next), ptr(rerouted),
                               ptr(labels)))
    assert np.array_equal(labels, sub), f"labels: {int((labels != sub).sum())} differ"
    assert np.array_equal(rerouted, want_final), \
        f"re-routed receivers: {int((rerouted != want_final).sum())} differ"
    return int(np.count_nonzero((sub == np.arange(n)) & (table == 0)))


def test_sixteen_million_two_iterations_bit_exact(orc):
    w = workloads.sixteen_million()
    m, p = w.model, w.params
    g = graphs.from_model(m)
    r = orc.generate(g, p.base, p.erodibility, p.uplift, p.is_outlet, max_iter=2, trace_cap=2)
    assert r["iters"] == 2
    gen = TerrainGenerator.default().set_model(m).set_parameters(p).set_max_iteration(2)
    terrain = gen.generate()
    assert gen.last_iterations == r["iters"]
    _bits_equal(terrain.elevations(), r["elev"], "16M elevations after 2 iterations")

    # each iteration's stream tree on the oracle's inputs
    outlets = orc.resolve_outlets(p.is_outlet, g.default_outlets)
    table = np.zeros(g.n, np.uint8)
    table[outlets] = 1
    initial = p.base + orc.rng_f64(g.n) * np.finfo(np.float64).eps
    h = m.handle()
    lakes1 = _check_stream_tree(orc, g, h, initial, table, outlets, r["trace_next"][0])
    assert lakes1 > 0, "the initial noise leaves lakes to re-route"
    _check_stream_tree(orc, g, h, r["trace_elev"][0], table, outlets, r["trace_next"][1])
    m.release()


def test_one_million_config_to_convergence(orc):
    """C2 solved until an iteration changes nothing (821 iterations on the oracle).
    When the model and parameters hash as they did where the fixture was made, the
    GPU's iteration count and elevation digest must equal the oracle's recorded ones;
    otherwise the oracle is run here to convergence.  Either way, one oracle iteration
    from the GPU's final elevations must change nothing (the reference's loop would stop
    there)."""
    import json
    import os
    from tests.golden import make_c2_converged as fx
    with open(os.path.join(os.path.dirname(__file__), "golden", "c2_converged.json")) as f:
        want = json.load(f)
    w = workloads.one_million()
    m, p = w.model, w.params
    g = graphs.from_model(m)
    gen = TerrainGenerator.default().set_model(m).set_parameters(p)
    elev = gen.generate().elevations()
    if fx.input_digest(g, p) == want["input_sha256"]:
        assert gen.last_iterations == want["iterations"]
        assert fx.elev_digest(elev) == want["elev_sha256"], "1M converged elevations differ"
    else:
        r = orc.generate(g, p.base, p.erodibility, p.uplift, p.is_outlet)
        assert gen.last_iterations == r["iters"]
        _bits_equal(elev, r["elev"], f"1M elevations after {r['iters']} iterations")
    # a fixed point of the reference's iteration
    outlets = orc.resolve_outlets(p.is_outlet, g.default_outlets)
    table = np.zeros(g.n, np.uint8)
    table[outlets] = 1
    nxt = orc.initial_tree(g, elev, table)
    sub, has_lake = orc.roots(table, nxt)
    if has_lake:
        nxt = orc.remove_lakes_heap(g, nxt, outlets, sub)
    changed, again, _, _ = orc.tree_pass(g, nxt, outlets, p.erodibility, p.uplift,
                                         np.full(g.n, np.nan), elev)
    assert not changed
    _bits_equal(again, elev, "one more oracle iteration")
    m.release()
