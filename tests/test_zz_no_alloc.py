"""The allocation-free basin-label entry point (fl_basin_labels_noalloc).

Some callers cannot allocate device memory -- a service that hands its GPU memory
out from its own fixed pool must not let a library call cudaMalloc behind the pool's
back (nor synchronise the device to do it).  fl_basin_labels_noalloc serves them from
a fixed scratch array inside the library.  This test gives it device arrays it did
not allocate, runs it twice in a row (the second call finds the first call's data in
the shared scratch), and checks both results against the labels of the existing
entry point, fl_probe_lakes, exactly (labels are site ids).  It lives in its own file,
collected last, and works alone in a fresh process as well as after the other tests.
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


def test_noalloc_labels_match_existing_entry_point(fl_lib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    g = graphs.random_delaunay(30000, seed=21, side=170.0)
    rng = np.random.default_rng(4)
    for call in range(2):
        elev = rng.uniform(0.0, 1.0, g.n)
        if call == 1:
            elev = np.round(elev * 8) / 8          # plateaus: many more lakes
        table = (rng.uniform(size=g.n) < 0.03).astype(np.uint8)
        nxt, want, want_lake = _existing_labels(g, elev, table)

        # device arrays owned by the caller (allocated here, not by the library)
        d_next = torch.from_numpy(nxt.view(np.int32).copy()).cuda()
        d_table = torch.from_numpy(table.copy()).cuda()
        d_labels = torch.full((g.n,), -1, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        has_lake = ctypes.c_int(-1)
        rc = lib().fl_basin_labels_noalloc(g.n, ctypes.c_void_p(d_next.data_ptr()),
                                           ctypes.c_void_p(d_table.data_ptr()),
                                           ctypes.c_void_p(d_labels.data_ptr()),
                                           ctypes.byref(has_lake), None)
        assert rc == _lib.FL_OK, _lib.last_error()
        torch.cuda.synchronize()
        got = d_labels.cpu().numpy().view(np.uint32)
        assert np.array_equal(got, want), f"call {call}: {int((got != want).sum())} labels differ"
        assert bool(has_lake.value) == want_lake


def test_noalloc_rejects_sizes_beyond_its_scratch(fl_lib):
    dummy = ctypes.c_void_p(16)   # never dereferenced: the size check comes first
    rc = lib().fl_basin_labels_noalloc(MAX_SITES + 1, dummy, dummy, dummy, None, None)
    assert rc == _lib.FL_ERR_INVALID_ARGUMENT
    assert "4194304" in _lib.last_error()
