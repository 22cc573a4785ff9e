"""The lake heap's order computed on the GPU (fl_probe_lake_rank_gpu) against the
oracle's restatement of the reference's BinaryHeap traversal
(src/lem/stream_tree.rs:175-243), rank for rank.

The GPU path replays only the outlets' tied prefix on the host and derives the rest
from the minimum spanning tree; where equal lengths could let the heap's arrangement
decide (rounded or unit lengths) or a length is zero, it must decline, and the solver
then keeps the host heap."""
import ctypes

import numpy as np
import pytest

from fastlem_gb300 import workloads
from fastlem_gb300 import _lib
from fastlem_gb300._lib import check, lib, ptr
from tests import graphs
from tests.test_lake_rank import cases

pytestmark = pytest.mark.gpu

CASES = list(cases())
# lengths rounded to 0.1, zero lengths, unit grids and the two-component case (two
# edges of length 1.0 from the same site) hold ties the keys cannot order
TIED = {"delaunay-rounded", "delaunay-zero-lengths", "grid-unit", "two-components"}


def gpu_rank(g, outlets):
    h = ctypes.c_void_p()
    check(lib().fl_graph_create(g.n, ptr(g.row_ptr), ptr(g.col), ptr(g.length), ptr(g.area),
                                ptr(g.default_outlets), len(g.default_outlets),
                                ptr(getattr(g, "xs", None)), ptr(getattr(g, "ys", None)),
                                ctypes.byref(h)))
    try:
        o = np.ascontiguousarray(outlets, np.uint32)
        rank = np.full(g.n, 7, np.uint32)
        used = ctypes.c_int(-1)
        check(lib().fl_probe_lake_rank_gpu(h, ptr(o), len(o), ptr(rank), ctypes.byref(used)))
        return rank, used.value
    finally:
        lib().fl_graph_destroy(h)


@pytest.mark.parametrize("name,g,outlets", CASES, ids=[c[0] for c in CASES])
def test_gpu_rank_equals_heap_order(orc, name, g, outlets):
    rank, used = gpu_rank(g, outlets)
    if name in TIED:
        assert used == 0, "ties must send the order back to the host heap"
        return
    assert used == 1, _lib.last_error()
    want = orc.prim_rank(g, outlets)
    assert np.array_equal(rank, want), f"{int((rank != want).sum())} ranks differ"


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_gpu_rank_random_delaunay(orc, seed):
    g = graphs.random_delaunay(20000, seed=seed)
    rng = np.random.default_rng(seed)
    outlets = rng.choice(g.n, 50 * seed, replace=False).astype(np.uint32)
    rank, used = gpu_rank(g, outlets)
    assert used == 1, _lib.last_error()
    assert np.array_equal(rank, orc.prim_rank(g, outlets))


def test_gpu_rank_unreached_component(orc):
    g = graphs.two_components()
    outlets = np.array([0], np.uint32)
    rank, used = gpu_rank(g, outlets)
    want = orc.prim_rank(g, outlets)
    if used:
        assert np.array_equal(rank, want)
    assert (want == 0xFFFFFFFF).any()


def test_gpu_rank_one_million_config(orc):
    w = workloads.one_million()
    g = graphs.from_model(w.model)
    outlets = orc.resolve_outlets(w.params.is_outlet, g.default_outlets)
    rank, used = gpu_rank(g, outlets)
    assert used == 1, _lib.last_error()
    assert np.array_equal(rank, orc.prim_rank(g, outlets))
