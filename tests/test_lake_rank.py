"""The solver's host lake-heap order (fl_lake_rank) against the oracle's restatement of
the reference's BinaryHeap traversal (lem/stream_tree.rs:175-243), on graphs whose
order is decided by keys alone and on graphs full of ties (equal lengths, zero
lengths, repeated outlets), where the solver must fall back to the reference's heap
arrangement."""
import numpy as np
import pytest

from fastlem_gb300._lib import FL_ERR_INVALID_ARGUMENT, FL_OK, lib, ptr
from oracle import oracle as orc
from tests import graphs


def product_rank(g, outlets):
    o = np.ascontiguousarray(outlets, np.uint32)
    rank = np.empty(g.n, np.uint32)
    rc = lib().fl_lake_rank(g.n, ptr(g.row_ptr), ptr(g.col), ptr(g.length), ptr(o), len(o),
                            ptr(rank))
    return rc, rank


def with_lengths(g, length):
    return graphs.Graph(g.n, g.row_ptr, g.col, np.ascontiguousarray(length, np.float64), g.area,
                        g.default_outlets, g.xs, g.ys)


def cases():
    r = np.random.default_rng(11)
    d = graphs.random_delaunay(3000, seed=4)
    yield "delaunay", d, np.sort(r.choice(d.n, 60, replace=False))
    yield "delaunay-unsorted-outlets", d, r.choice(d.n, 60, replace=False)
    yield "delaunay-repeated-outlets", d, np.r_[r.choice(d.n, 30, replace=False), [5, 5, 17]]
    yield "delaunay-one-outlet", d, np.array([123])
    # rounded lengths: many equal keys after the outlets
    yield "delaunay-rounded", with_lengths(d, np.round(d.length, 1)), r.choice(d.n, 40, replace=False)
    # zero-length edges: ties with the outlets' 0.0
    z = d.length.copy()
    z[r.random(len(z)) < 0.05] = 0.0
    yield "delaunay-zero-lengths", with_lengths(d, z), r.choice(d.n, 40, replace=False)
    yield "grid-unit", graphs.grid(30, 20, unit_lengths=True, seed=1), np.arange(0, 600, 37)
    yield "grid-jitter", graphs.grid(30, 20, jitter=0.3, seed=2), np.arange(0, 600, 41)
    yield "star", graphs.star(8), np.arange(1, 9)
    yield "line", graphs.line(9), np.array([4])
    yield "two-components", graphs.two_components(), np.array([0])
    yield "no-outlets", d, np.array([], np.int64)


CASES = list(cases())


@pytest.mark.parametrize("name,g,outlets", CASES, ids=[c[0] for c in CASES])
def test_lake_rank_equals_the_reference_heap(name, g, outlets):
    rc, got = product_rank(g, outlets)
    assert rc == FL_OK
    want = orc.prim_rank(g, np.asarray(outlets, np.uint32))
    assert np.array_equal(got, want), name


def test_lake_rank_rejects_bad_input():
    g = graphs.line(5)
    rc, _ = product_rank(g, np.array([7]))
    assert rc == FL_ERR_INVALID_ARGUMENT
    bad = g.length.copy()
    bad[0] = np.nan
    rc, _ = product_rank(with_lengths(g, bad), np.array([0]))
    assert rc == FL_ERR_INVALID_ARGUMENT
