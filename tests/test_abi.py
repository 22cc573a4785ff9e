"""CPU tests of the C-ABI library: it builds, loads without a GPU, exports every
symbol include/fastlem_gb300.h declares, and reports fastlem's errors in
fastlem's order before touching the device."""
import ctypes
import os
import re

import numpy as np
import pytest

from fastlem_gb300 import (GenerationError, ParameterArrays, TerrainGenerator,
                           TopographicalParameters)
from fastlem_gb300 import _lib

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                      "fastlem_gb300.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(fl_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_the_exported_list():
    assert declared_functions() == sorted(_lib.EXPORTS)


def test_library_exports_every_declared_symbol(fl_lib):
    for name in declared_functions():
        assert hasattr(fl_lib, name), name


def test_status_codes_match_header():
    src = open(HEADER).read()
    for name, val in re.findall(r"#define (FL_[A-Z_]+) (\d+)", src):
        assert getattr(_lib, name) == int(val), name


def test_generate_errors_in_reference_order(fl_lib):
    # ModelNotSet comes first (generator.rs:91-97), whatever else is missing
    z = np.zeros(4)
    assert fl_lib.fl_generate(None, 4, None, None, None, None, None, -1, None, None) == 1
    with pytest.raises(GenerationError) as e:
        TerrainGenerator.default().generate()
    assert e.value.kind == "ModelNotSet"

    class FakeModel:
        def num(self):
            return 4

    with pytest.raises(GenerationError) as e:
        TerrainGenerator.default().set_model(FakeModel()).generate()
    assert e.value.kind == "ParametersNotSet"
    with pytest.raises(GenerationError) as e:
        (TerrainGenerator.default().set_model(FakeModel())
         .set_parameters([TopographicalParameters()] * 3).generate())
    assert e.value.kind == "InvalidNumberOfParameters"
    with pytest.raises(GenerationError) as e:
        TerrainGenerator.default().set_model(FakeModel()).set_parameters(ParameterArrays(5)).generate()
    assert e.value.kind == "InvalidNumberOfParameters"


def test_parameter_defaults_and_setters():
    p = TopographicalParameters()
    assert (p.base_elevation, p.erodibility, p.uplift_rate, p.is_outlet, p.max_slope) == \
        (0.0, 1.0, 1.0, False, None)
    q = p.set_erodibility(2.0).set_is_outlet(True).set_max_slope(0.3)
    assert (q.erodibility, q.is_outlet, q.max_slope) == (2.0, True, 0.3)
    arr = ParameterArrays.from_list([p, q])
    assert arr.is_outlet.tolist() == [0, 1]
    assert np.isnan(arr.max_slope[0]) and arr.max_slope[1] == 0.3


def _two_joined_terrains():
    import numpy as np
    # two 2-site terrains; site 1 (terrain 0) is joined to site 2 (terrain 1)
    return (np.array([0, 2, 4], np.uint32), np.array([0, 1, 3, 5, 6], np.uint32),
            np.array([1, 0, 2, 1, 3, 2], np.uint32), np.ones(6), np.ones(4),
            np.array([0, 1, 2], np.uint32), np.array([0, 3], np.uint32))


@pytest.mark.gpu
def test_batch_create_rejects_edges_across_terrains(fl_lib):
    """Packed terrains must not share an edge (checked on the device with the rest of
    the graph, before the model is returned)."""
    import ctypes
    from fastlem_gb300._lib import FL_ERR_INVALID_ARGUMENT, ptr
    site_off, row_ptr, col, length, area, def_off, defs = _two_joined_terrains()
    h = ctypes.c_void_p()
    rc = fl_lib.fl_batch_create(2, ptr(site_off), ptr(row_ptr), ptr(col), ptr(length), ptr(area),
                                ptr(def_off), ptr(defs), None, None, ctypes.byref(h))
    assert rc == FL_ERR_INVALID_ARGUMENT
    assert b"cross" in fl_lib.fl_last_error()


def test_batch_create_rejects_bad_offsets(fl_lib):
    """Terrain offsets that do not cover the sites (checked before any device work)."""
    import ctypes
    import numpy as np
    from fastlem_gb300._lib import FL_ERR_INVALID_ARGUMENT, ptr
    site_off, row_ptr, col, length, area, def_off, defs = _two_joined_terrains()
    h = ctypes.c_void_p()
    # offsets that do not cover the sites
    rc = fl_lib.fl_batch_create(2, ptr(np.array([0, 2, 3], np.uint32)), ptr(row_ptr), ptr(col),
                                ptr(length), ptr(area), ptr(def_off), ptr(defs), None, None,
                                ctypes.byref(h))
    assert rc == FL_ERR_INVALID_ARGUMENT


def test_server_host_checks(fl_lib):
    """Server argument checks that run before any device work."""
    import ctypes
    import numpy as np
    from fastlem_gb300._lib import (FL_ERR_INVALID_ARGUMENT, FL_ERR_MODEL_NOT_SET,
                                    FL_ERR_OUT_OF_MEMORY, ptr)
    s = ctypes.c_void_p()
    assert fl_lib.fl_server_create(0, 2, ctypes.byref(s)) == FL_ERR_INVALID_ARGUMENT
    assert fl_lib.fl_server_create(1 << 14, 1, ctypes.byref(s)) == 0
    try:
        row_ptr = np.array([0, 1, 2], np.uint32)
        col = np.array([1, 0], np.uint32)
        length = np.ones(2)
        area = np.ones(2)
        defs = np.array([0], np.uint32)
        mid = ctypes.c_uint32()
        # adjacency slots without their columns or lengths
        assert fl_lib.fl_server_add_model(s, 2, ptr(row_ptr), None, ptr(length), ptr(area),
                                          ptr(defs), 1, None, None,
                                          ctypes.byref(mid)) == FL_ERR_INVALID_ARGUMENT
        assert fl_lib.fl_server_add_model(s, 2, ptr(row_ptr), ptr(col), None, ptr(area),
                                          ptr(defs), 1, None, None,
                                          ctypes.byref(mid)) == FL_ERR_INVALID_ARGUMENT
        assert fl_lib.fl_server_add_model(s, 2, ptr(row_ptr), ptr(col), ptr(length), ptr(area),
                                          ptr(defs), 1, None, None, ctypes.byref(mid)) == 0
        z, o = np.zeros(2), np.ones(2)
        out = np.empty(2)
        t = ctypes.c_uint64()
        outl = np.zeros(2, np.uint8)
        # unknown model, then a model whose instance can never fit a 16 KiB budget
        assert fl_lib.fl_server_submit(s, 7, ptr(z), ptr(o), ptr(o), ptr(outl), None, -1,
                                       ptr(out), ctypes.byref(t)) == FL_ERR_MODEL_NOT_SET
        assert fl_lib.fl_server_submit(s, mid.value, ptr(z), ptr(o), ptr(o), ptr(outl), None, -1,
                                       ptr(out), ctypes.byref(t)) == FL_ERR_OUT_OF_MEMORY
        assert fl_lib.fl_server_wait(s, 12345, None, None, None, None) == FL_ERR_INVALID_ARGUMENT
    finally:
        fl_lib.fl_server_destroy(s)


def test_host_alloc_argument_checks(fl_lib):
    """fl_host_alloc rejects a zero size or a missing out pointer before any CUDA call;
    fl_host_free ignores NULL."""
    from fastlem_gb300._lib import FL_ERR_INVALID_ARGUMENT
    p = ctypes.c_void_p(1234)
    assert fl_lib.fl_host_alloc(0, ctypes.byref(p)) == FL_ERR_INVALID_ARGUMENT
    assert p.value is None
    assert fl_lib.fl_host_alloc(64, None) == FL_ERR_INVALID_ARGUMENT
    fl_lib.fl_host_free(None)


def test_model_device_bytes_bound_grows_with_the_model(fl_lib):
    """The admission bound covers the per-site and per-slot arrays of a model."""
    b1 = fl_lib.fl_model_device_bytes(1000, 6000)
    b2 = fl_lib.fl_model_device_bytes(2000, 12000)
    assert b2 > b1 >= 1000 * 360 + 6000 * 16
    assert fl_lib.fl_model_device_bytes(1000, 7000) - b1 == 1000 * 16


def test_generate_rejects_a_bad_output_buffer():
    """generate(out=...) wants a contiguous float64 array of num() sites."""
    import math
    from fastlem_gb300 import workloads
    w = workloads.small(scale=0.01)
    gen = TerrainGenerator.default().set_model(w.model).set_parameters(w.params)
    for bad in (np.empty(w.model.num(), np.float32), np.empty(w.model.num() + 1),
                np.empty(2 * w.model.num())[::2]):
        with pytest.raises(ValueError):
            gen.generate(out=bad)


def test_graph_create_rejects_missing_arrays(fl_lib):
    """Null columns or lengths are rejected before anything is read or allocated."""
    from fastlem_gb300._lib import FL_ERR_INVALID_ARGUMENT, ptr
    row_ptr = np.array([0, 1, 2], np.uint32)
    col = np.array([1, 0], np.uint32)
    length = np.ones(2)
    area = np.ones(2)
    h = ctypes.c_void_p()
    assert fl_lib.fl_graph_create(2, ptr(row_ptr), ptr(col), None, ptr(area), None, 0, None,
                                  None, ctypes.byref(h)) == FL_ERR_INVALID_ARGUMENT
    assert fl_lib.fl_graph_create(2, ptr(row_ptr), None, ptr(length), ptr(area), None, 0, None,
                                  None, ctypes.byref(h)) == FL_ERR_INVALID_ARGUMENT


def test_compiled_schedule_is_the_committed_one(fl_lib):
    """The library's compiled-in launch-shape schedule equals fastlem_gb300/schedule.json
    (the schedule sweep's output), class for class."""
    import json
    import os
    from fastlem_gb300 import _lib
    path = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                        "fastlem_gb300", "schedule.json")
    with open(path) as f:
        classes = json.load(f)["classes"]
    want = [(c["max_sites"], int(c["packed"]), c["best"]["low_ilp"], c["best"]["walk_per_sm"],
             c["best"]["kahn_min_width"], int(c["best"].get("sized_grids", 0))) for c in classes]
    assert _lib.schedule() == want


def test_tuning_knobs_reject_bad_values(fl_lib):
    """fl_set_tuning takes only the documented names and ranges; fl_get_tuning reports -2
    for an unknown name; a rejected call leaves the knob as it was."""
    from fastlem_gb300 import _lib
    from fastlem_gb300._lib import FL_ERR_INVALID_ARGUMENT
    before = _lib.get_tuning()
    for name, bad in (("low_ilp", 3), ("low_ilp", 8), ("walk_per_sm", 65), ("sized_grids", 2),
                      ("gpu_rank", 2), ("kahn_min_width", 100), ("kahn_min_width", 1 << 25),
                      ("no_such_knob", 1)):
        assert fl_lib.fl_set_tuning(name.encode(), bad) == FL_ERR_INVALID_ARGUMENT, name
    assert fl_lib.fl_set_tuning(None, 1) == FL_ERR_INVALID_ARGUMENT
    assert fl_lib.fl_get_tuning(b"no_such_knob") == -2
    assert _lib.get_tuning() == before
    old = _lib.set_tuning(low_ilp=2, kahn_min_width=4096)
    try:
        assert _lib.get_tuning()["low_ilp"] == 2 and _lib.get_tuning()["kahn_min_width"] == 4096
    finally:
        _lib.set_tuning(**old)
    assert _lib.get_tuning() == before
