"""GPU parity: every solver stage and whole generate() runs, through the C ABI,
compared bit for bit with the CPU oracle on the same inputs.  Integer outputs
(receivers, labels) must be identical; floating outputs (drainage, response time,
elevation) are compared by bit pattern -- the tolerance is zero ulp, tighter than the
1e-10 relative bound the solve is specified to."""
import ctypes
import json
import math
import os

import numpy as np
import pytest

from fastlem_gb300 import (ParameterArrays, Site2D, TerrainGenerator, TerrainModel2DBulider,
                           TopographicalParameters, workloads)
from fastlem_gb300._lib import FL_OK, check, lib, ptr
from tests import graphs, pyref

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


class Handle:
    def __init__(self, g):
        self.g = g
        h = ctypes.c_void_p()
        xs = None if getattr(g, "xs", None) is None else np.ascontiguousarray(g.xs)
        ys = None if getattr(g, "ys", None) is None else np.ascontiguousarray(g.ys)
        check(lib().fl_graph_create(g.n, ptr(g.row_ptr), ptr(g.col), ptr(g.length), ptr(g.area),
                                    ptr(g.default_outlets), len(g.default_outlets), ptr(xs),
                                    ptr(ys), ctypes.byref(h)))
        self.h = h

    def __enter__(self):
        return self

    def __exit__(self, *a):
        lib().fl_graph_destroy(self.h)

    def generate(self, base, k, u, is_outlet, max_slope=None, max_iter=-1):
        n = self.g.n
        out = np.empty(n)
        it = ctypes.c_uint32()
        ms = None if max_slope is None else np.ascontiguousarray(max_slope, np.float64)
        rc = lib().fl_generate(self.h, n, ptr(np.ascontiguousarray(base, np.float64)),
                               ptr(np.ascontiguousarray(k, np.float64)),
                               ptr(np.ascontiguousarray(u, np.float64)),
                               ptr(np.ascontiguousarray(is_outlet, np.uint8)), ptr(ms), max_iter,
                               ptr(out), ctypes.byref(it))
        check(rc)
        return out, it.value


def bits(a):
    return np.ascontiguousarray(a, np.float64).view(np.uint64)


def assert_bits_equal(got, want, what):
    g, w = bits(got), bits(want)
    bad = np.nonzero(g != w)[0]
    assert len(bad) == 0, f"{what}: {len(bad)} sites differ, first {bad[:5]} got {got[bad[:3]]} want {want[bad[:3]]}"


def graph_cases():
    yield "grid_ties", graphs.grid(12, 9, unit_lengths=True, seed=1)
    yield "grid_jitter", graphs.grid(15, 11, jitter=0.3, seed=2)
    yield "delaunay2k", graphs.random_delaunay(2000, seed=3)
    yield "two_components", graphs.two_components()


CASES = list(graph_cases())


def test_device_rng_matches_oracle(orc):
    for first, count in ((0, 1000), (13, 77), (1 << 20, 64)):
        out = np.empty(count)
        check(lib().fl_probe_rng_f64(0, first, count, ptr(out)))
        assert_bits_equal(out, orc.rng_f64(count, first=first), "rng")
    out = np.empty(50)
    check(lib().fl_probe_rng_f64(11, 0, 50, ptr(out)))
    assert_bits_equal(out, orc.rng_f64(50, seed=11), "rng seed 11")


@pytest.mark.parametrize("name,g", CASES, ids=[c[0] for c in CASES])
def test_receivers_parity(orc, name, g):
    rng = np.random.default_rng(5)
    with Handle(g) as h:
        for trial in range(4):
            elev = rng.uniform(0, 1, g.n)
            if trial % 2:
                elev = np.round(elev * 3) / 3        # plateaus: equal elevations
            table = (rng.uniform(size=g.n) < 0.1).astype(np.uint8)
            want = orc.initial_tree(g, elev, table)
            got = np.empty(g.n, np.uint32)
            hl = ctypes.c_int()
            check(lib().fl_probe_receivers(h.h, ptr(elev), ptr(table), ptr(got), ctypes.byref(hl)))
            assert np.array_equal(got, want)
            _, has_lake = orc.roots(table, want)
            assert bool(hl.value) == has_lake


def _hard_elevations(rng, n, family):
    """Elevations that stress the receivers' f32 slope estimates."""
    if family == "offset":        # one binary exponent, differences ~1e-9 of the value
        return 1000.0 + rng.uniform(0, 1e-6, n)
    if family == "binades":       # around powers of two: neighbours in different binades
        return np.ldexp(1.0, rng.integers(-3, 4, n)) * (1.0 + rng.uniform(-1e-6, 1e-6, n))
    if family == "extreme":       # far outside the f32 range, subnormals, zeros
        pick = rng.integers(0, 6, n)
        vals = np.array([0.0, 5e-324, 1e-300, 1e300, 1e-40, 3e38])
        return vals[pick] * (1.0 + rng.uniform(0, 1e-3, n))
    # special values scattered over a smooth field
    e = rng.uniform(0, 1, n)
    pick = rng.integers(0, 40, n)
    e[pick == 0] = np.nan
    e[pick == 1] = np.inf
    e[pick == 2] = -np.inf
    e[pick == 3] = -rng.uniform(0, 1, int((pick == 3).sum()))
    e[pick == 4] = 0.0
    e[pick == 5] = -0.0
    return e


@pytest.mark.parametrize("family", ["offset", "binades", "extreme", "special"])
@pytest.mark.parametrize("lengths", ["plain", "degenerate"])
def test_receivers_parity_hard_values(orc, family, lengths):
    g = graphs.random_delaunay(3000, seed=21)
    if lengths == "degenerate":
        # zero, subnormal, tiny and huge edge lengths (rows then take the exact scan)
        rng = np.random.default_rng(4)
        ln = g.length.copy()
        pick = rng.integers(0, 30, len(ln))
        ln[pick == 0] = 0.0
        ln[pick == 1] = 1e-310
        ln[pick == 2] = 1e-45
        ln[pick == 3] = 1e300
        ln[pick == 4] = 1e39
        g = graphs.Graph(g.n, g.row_ptr, g.col, ln, g.area, g.default_outlets, g.xs, g.ys)
    rng = np.random.default_rng(17)
    with Handle(g) as h:
        for trial in range(3):
            elev = _hard_elevations(rng, g.n, family)
            table = (rng.uniform(size=g.n) < 0.05).astype(np.uint8)
            want = orc.initial_tree(g, elev, table)
            got = np.empty(g.n, np.uint32)
            hl = ctypes.c_int()
            check(lib().fl_probe_receivers(h.h, ptr(elev), ptr(table), ptr(got), ctypes.byref(hl)))
            assert np.array_equal(got, want), f"{family}/{lengths} trial {trial}"
            _, has_lake = orc.roots(table, want)
            assert bool(hl.value) == has_lake


@pytest.mark.parametrize("name,g", CASES, ids=[c[0] for c in CASES])
def test_lake_rerouting_parity(orc, name, g):
    rng = np.random.default_rng(9)
    with Handle(g) as h:
        for trial in range(4):
            elev = rng.uniform(0, 1, g.n)
            if trial % 2:
                elev = np.round(elev * 4) / 4
            k = max(1, g.n // 30)
            outlets = np.array(sorted(rng.choice(g.n, size=k, replace=False)), np.uint32)
            if trial == 3:
                outlets = outlets[::-1].copy()
            table = np.zeros(g.n, np.uint8)
            table[outlets] = 1
            nxt = orc.initial_tree(g, elev, table)
            sub, has_lake = orc.roots(table, nxt)
            want = orc.remove_lakes_heap(g, nxt, outlets, sub)
            got = np.empty(g.n, np.uint32)
            lab = np.empty(g.n, np.uint32)
            check(lib().fl_probe_lakes(h.h, ptr(outlets), len(outlets), ptr(nxt), ptr(got), ptr(lab)))
            assert np.array_equal(lab, sub), "basin labels"
            assert np.array_equal(got, want), "re-routed receivers"


@pytest.mark.parametrize("with_slope", [False, True])
def test_tree_pass_parity(orc, with_slope):
    w = workloads.small(scale=0.3, max_slope=0.314 if with_slope else None)
    m, p = w.model, w.params
    g = graphs.from_model(m)
    r = orc.generate(g, p.base, p.erodibility, p.uplift, p.is_outlet, max_slope=p.max_slope,
                     trace_cap=6, max_iter=6)
    outlets = orc.resolve_outlets(p.is_outlet, g.default_outlets)
    tanms = np.tan(p.max_slope) if p.max_slope is not None else np.full(g.n, np.nan)
    with Handle(g) as h:
        for it in range(1, len(r["trace_next"])):
            nxt = r["trace_next"][it]
            elev_in = r["trace_elev"][it - 1]
            ch, e_want, a_want, t_want = orc.tree_pass(g, nxt, outlets, p.erodibility, p.uplift,
                                                        tanms, elev_in)
            e = elev_in.copy()
            a = np.empty(g.n)
            t = np.empty(g.n)
            changed = ctypes.c_int()
            check(lib().fl_probe_tree_pass(h.h, ptr(outlets), len(outlets), ptr(nxt),
                                           ptr(p.erodibility), ptr(p.uplift), ptr(p.max_slope),
                                           ptr(e), ptr(a), ptr(t), ctypes.byref(changed)))
            reached = np.zeros(g.n, bool)
            reached[np.isfinite(t_want) & (t_want > 0)] = True
            assert_bits_equal(a[reached], a_want[reached], f"drainage it{it}")
            assert_bits_equal(t[reached], t_want[reached], f"response it{it}")
            assert_bits_equal(e, e_want, f"elevation it{it}")
            assert bool(changed.value) == ch


def test_generate_golden_cases():
    with open(os.path.join(GOLDEN, "small_graphs.json")) as f:
        cases = json.load(f)
    for c in cases:
        g = graphs.from_csr(c)
        ms = None if c["max_slope"] is None else np.array(c["max_slope"])
        with Handle(g) as h:
            e, it = h.generate(np.array(c["base"]), np.array(c["k"]), np.array(c["u"]),
                               np.array(c["is_outlet"], np.uint8), max_slope=ms)
        assert it == c["iters"], c["name"]
        assert e.view(np.uint64).tolist() == [int(b, 16) for b in c["elev_bits"]], c["name"]


def _parity_run(orc, w, max_iter=-1):
    m, p = w.model, w.params
    g = graphs.from_model(m)
    r = orc.generate(g, p.base, p.erodibility, p.uplift, p.is_outlet, max_slope=p.max_slope,
                     max_iter=max(0, max_iter))
    gen = (TerrainGenerator.default().set_model(m).set_parameters(p))
    if max_iter >= 0:
        gen = gen.set_max_iteration(max_iter)
    terrain = gen.generate()
    assert gen.last_iterations == r["iters"]
    assert_bits_equal(terrain.elevations(), r["elev"], w.name)
    m.release()
    return r["iters"]


def test_generate_small_config_full_convergence(orc):
    assert _parity_run(orc, workloads.small()) > 10


def test_generate_small_config_with_max_slope(orc):
    _parity_run(orc, workloads.small(max_slope=0.314))


@pytest.mark.parametrize("max_slope", [None, 0.314])
def test_pinned_host_buffers_give_the_same_result(max_slope):
    """Parameters in page-locked memory (ParameterArrays.pinned) and a reused pinned
    output array give the bits of the pageable path, call after call."""
    from fastlem_gb300 import pinned_empty
    w = workloads.small(scale=0.5, max_slope=max_slope)
    m, p = w.model, w.params
    want = TerrainGenerator.default().set_model(m).set_parameters(p).set_max_iteration(12)
    want = want.generate().elevations()
    pp = p.pinned()
    assert all(np.array_equal(getattr(pp, k), getattr(p, k), equal_nan=True)
               for k in ("base", "erodibility", "uplift", "is_outlet"))
    out = pinned_empty(m.num(), np.float64)
    gen = TerrainGenerator.default().set_model(m).set_parameters(pp).set_max_iteration(12)
    for _ in range(2):
        out[:] = np.nan
        got = gen.generate(out=out).elevations()
        assert_bits_equal(got, want, "pinned")
        assert_bits_equal(out, want, "pinned out buffer")
    m.release()


def test_generate_reference_landscape_evolution_test(orc):
    """The setup of fastlem's tests/landscape_evolution.rs:9-34: 10,000 random sites in
    [0,200]x[0,100], one relaxation, all default parameters but max_slope 3.14*0.1, no
    outlets (so the hull)."""
    num = 10000
    model = (TerrainModel2DBulider.from_random_sites(num, Site2D(0.0, 0.0), Site2D(200.0, 100.0))
             .relaxate_sites(1).build())
    params = [TopographicalParameters().set_base_elevation(0.0).set_erodibility(1.0)
              .set_uplift_rate(1.0).set_is_outlet(False).set_max_slope(3.14 * 0.1)] * num
    g = graphs.from_model(model)
    pa = ParameterArrays.from_list(params)
    r = orc.generate(g, pa.base, pa.erodibility, pa.uplift, pa.is_outlet, max_slope=pa.max_slope)
    gen = TerrainGenerator.default().set_model(model).set_parameters(params)
    terrain = gen.generate()
    assert gen.last_iterations == r["iters"]
    assert_bits_equal(terrain.elevations(), r["elev"], "landscape_evolution")


def test_generate_1m_scaled_full_convergence(orc):
    """The 1M config's generator at 50k sites (same density), solved to convergence."""
    _parity_run(orc, workloads.one_million(scale=0.05))


def test_generate_1m_bounded_iterations(orc):
    _parity_run(orc, workloads.one_million(), max_iter=3)


def test_max_iteration_zero_returns_initial_elevations(orc):
    w = workloads.small(scale=0.1)
    n = w.model.num()
    terrain = (TerrainGenerator.default().set_model(w.model).set_parameters(w.params)
               .set_max_iteration(0).generate())
    want = w.params.base + orc.rng_f64(n) * np.finfo(np.float64).eps
    assert_bits_equal(terrain.elevations(), want, "max_iteration=0")
