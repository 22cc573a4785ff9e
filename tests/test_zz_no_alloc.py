"""The allocation-free basin-label entry point (fl_basin_labels_noalloc).

Some callers cannot allocate device memory -- a service that hands its GPU memory
out from its own fixed pool must not let a library call cudaMalloc behind the pool's
back (nor synchronise the device to do it).  fl_basin_labels_noalloc serves them from
a fixed scratch array inside the library.  This test gives it device arrays it did
not allocate, runs it twice in a row (the second call finds the first call's data in
the shared scratch), and checks both results against the labels of the existing
entry point, fl_probe_lakes, and against the oracle's find_roots_with_lakes, exactly
(labels are site ids).  Bad receivers -- one outside [0, n), cycles of length 2 and 3
that drain to no outlet -- must be reported as errors, and a valid call right after
them must still give the right labels.  It lives in its own file, collected last, and
works alone in a fresh process as well as after the other tests.
"""
import ctypes

import numpy as np
import pytest

from fastlem_gb300 import _lib
from fastlem_gb300._lib import check, lib, ptr
from tests import graphs

pytestmark = pytest.mark.gpu

MAX_SITES = 4 << 20


def _existing_labels(g, elev, table):
    """Receivers and labels through the existing C-ABI entry points."""
    h = ctypes.c_void_p()
    check(lib().fl_graph_create(g.n, ptr(g.row_ptr), ptr(g.col), ptr(g.length), ptr(g.area),
                                ptr(g.default_outlets), len(g.default_outlets), ptr(g.xs),
                                ptr(g.ys), ctypes.byref(h)))
    try:
        nxt = np.empty(g.n, np.uint32)
        hl = ctypes.c_int()
        check(lib().fl_probe_receivers(h, ptr(elev), ptr(table), ptr(nxt), ctypes.byref(hl)))
        outlets = np.nonzero(table)[0].astype(np.uint32)
        rerouted = np.empty(g.n, np.uint32)
        labels = np.empty(g.n, np.uint32)
        check(lib().fl_probe_lakes(h, ptr(outlets), len(outlets), ptr(nxt), ptr(rerouted),
                                   ptr(labels)))
        return nxt, labels, bool(hl.value)
    finally:
        lib().fl_graph_destroy(h)


def _torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    return torch


def _noalloc(torch, nxt, table):
    """One call on caller-owned device arrays; returns (rc, labels, has_lake)."""
    n = len(nxt)
    d_next = torch.from_numpy(np.ascontiguousarray(nxt, np.uint32).view(np.int32).copy()).cuda()
    d_table = torch.from_numpy(np.ascontiguousarray(table, np.uint8).copy()).cuda()
    d_labels = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    has_lake = ctypes.c_int(-1)
    rc = lib().fl_basin_labels_noalloc(n, ctypes.c_void_p(d_next.data_ptr()),
                                       ctypes.c_void_p(d_table.data_ptr()),
                                       ctypes.c_void_p(d_labels.data_ptr()),
                                       ctypes.byref(has_lake), None)
    torch.cuda.synchronize()
    return rc, d_labels.cpu().numpy().view(np.uint32), has_lake.value


def test_noalloc_labels_match_existing_entry_point(fl_lib, orc):
    torch = _torch_cuda()
    g = graphs.random_delaunay(30000, seed=21, side=170.0)
    rng = np.random.default_rng(4)
    for call in range(2):
        elev = rng.uniform(0.0, 1.0, g.n)
        if call == 1:
            elev = np.round(elev * 8) / 8          # plateaus: many more lakes
        table = (rng.uniform(size=g.n) < 0.03).astype(np.uint8)
        nxt, want, want_lake = _existing_labels(g, elev, table)
        sub, orc_lake = orc.roots(table, nxt)
        assert np.array_equal(want, sub) and want_lake == orc_lake

        # device arrays owned by the caller (allocated here, not by the library)
        rc, got, has_lake = _noalloc(torch, nxt, table)
        assert rc == _lib.FL_OK, _lib.last_error()
        assert np.array_equal(got, want), f"call {call}: {int((got != want).sum())} labels differ"
        assert bool(has_lake) == want_lake


def _chain_forest(n, seed):
    """A random receiver forest: site i drains to a lower-numbered site or to itself;
    every tenth root is an outlet."""
    rng = np.random.default_rng(seed)
    nxt = np.arange(n, dtype=np.uint32)
    for i in range(1, n):
        if rng.uniform() < 0.9:
            nxt[i] = rng.integers(max(0, i - 50), i)
    table = np.zeros(n, np.uint8)
    roots = np.nonzero(nxt == np.arange(n))[0]
    table[roots[::10]] = 1
    return nxt, table


@pytest.mark.parametrize("bad", ["out_of_range", "cycle2", "cycle3", "cycle4"])
def test_noalloc_reports_bad_receivers_then_recovers(fl_lib, orc, bad):
    torch = _torch_cuda()
    n = 5000
    nxt, table = _chain_forest(n, seed=8)
    broken = nxt.copy()
    a, b, c, d = 4000, 4001, 4002, 4003
    table[[a, b, c, d]] = 0
    if bad == "out_of_range":
        broken[a] = n + 7
        want_rc = _lib.FL_ERR_INVALID_ARGUMENT
    elif bad == "cycle2":                      # settles after one round: the final check
        broken[a], broken[b] = b, a
        want_rc = _lib.FL_ERR_DEVICE_LIMIT
    elif bad == "cycle3":                      # never settles: the round limit
        broken[a], broken[b], broken[c] = b, c, a
        want_rc = _lib.FL_ERR_DEVICE_LIMIT
    else:                                      # settles after two rounds
        broken[a], broken[b], broken[c], broken[d] = b, c, d, a
        want_rc = _lib.FL_ERR_DEVICE_LIMIT
    broken[4100:4200] = a                      # sites draining into the bad part
    rc, _, _ = _noalloc(torch, broken, table)
    assert rc == want_rc, (bad, rc, _lib.last_error())
    # the shared scratch holds the failed call's data: a valid call is unaffected
    rc, got, has_lake = _noalloc(torch, nxt, table)
    assert rc == _lib.FL_OK, _lib.last_error()
    sub, orc_lake = orc.roots(table, nxt)
    assert np.array_equal(got, sub)
    assert bool(has_lake) == orc_lake


def test_noalloc_empty_input_reads_nothing(fl_lib):
    has_lake = ctypes.c_int(-1)
    assert lib().fl_basin_labels_noalloc(0, None, None, None, ctypes.byref(has_lake), None) == _lib.FL_OK
    assert has_lake.value == 0


def test_noalloc_rejects_sizes_beyond_its_scratch(fl_lib):
    dummy = ctypes.c_void_p(16)   # never dereferenced: the size check comes first
    rc = lib().fl_basin_labels_noalloc(MAX_SITES + 1, dummy, dummy, dummy, None, None)
    assert rc == _lib.FL_ERR_INVALID_ARGUMENT
    assert "4194304" in _lib.last_error()
