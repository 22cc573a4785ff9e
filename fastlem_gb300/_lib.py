"""ctypes binding of libfastlem_gb300.so (include/fastlem_gb300.h).

There is no fallback: if the library is missing or cannot be loaded, every call
raises.  Build it with `python -m fastlem_gb300.build` (or `__graft_entry__.build()`).
"""
import ctypes
import os

import numpy as np

from . import build as _build

_lib = None

FL_OK = 0
FL_ERR_MODEL_NOT_SET = 1
FL_ERR_PARAMETERS_NOT_SET = 2
FL_ERR_INVALID_NUM_PARAMETERS = 3
FL_ERR_BUILDER_SITES_NOT_SET = 4
FL_ERR_BUILDER_BOUNDS_NOT_SET = 5
FL_ERR_BUILDER_VORONOI = 6
FL_ERR_INVALID_ARGUMENT = 20
FL_ERR_CUDA = 21
FL_ERR_OUT_OF_MEMORY = 22
FL_ERR_DEVICE_LIMIT = 23

# Every symbol include/fastlem_gb300.h declares.
EXPORTS = [
    "fl_graph_create", "fl_graph_destroy", "fl_generate", "fl_generate_timed",
    "fl_graph_num_sites", "fl_graph_num_slots", "fl_last_error", "fl_select_device",
    "fl_graph_set_timing", "fl_graph_reset_stats", "fl_graph_host_syncs", "fl_set_tuning",
    "fl_get_tuning", "fl_graph_rank_info", "fl_probe_lake_rank_gpu",
    "fl_schedule_entry", "fl_graph_set_sized_grids", "fl_batch_create_parts",
    "fl_batch_generate_parts", "fl_server_set_packing", "fl_num_kernel_classes",
    "fl_graph_kernel_stats",
    "fl_graph_basin_stats", "fl_graph_round_trace", "fl_basin_labels_noalloc",
    "fl_batch_create", "fl_graph_num_terrains", "fl_batch_generate", "fl_graph_device_bytes",
    "fl_model_device_bytes", "fl_host_alloc", "fl_host_free",
    "fl_server_create", "fl_server_add_model", "fl_server_submit", "fl_server_wait",
    "fl_server_stats", "fl_server_destroy",
    "fl_probe_receivers", "fl_probe_lakes", "fl_probe_tree_pass", "fl_probe_prim_rank",
    "fl_probe_rng_f64", "fl_probe_chain_fold", "fl_random_sites", "fl_relax_sites", "fl_build_graph", "fl_triangulate",
    "fl_interpolator_create", "fl_interpolator_destroy", "fl_interpolate", "fl_lake_rank",
    "fl_interpolate_gpu", "fl_interpolate_device", "fl_interpolator_last_deferred",
    "fl_probe_interp_query", "fl_probe_prefilters",
]

c_u32, c_u64, c_int, c_dbl, vp = ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int, ctypes.c_double, ctypes.c_void_p
P = ctypes.POINTER


class FastlemError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"fastlem_gb300 error {code}: {msg}")
        self.code = code


def lib():
    """The loaded library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path):
        raise FastlemError(-1, f"{path} is missing; build it with `python -m fastlem_gb300.build`")
    L = ctypes.CDLL(path)
    L.fl_graph_create.argtypes = [c_u32, vp, vp, vp, vp, vp, c_u32, vp, vp, P(vp)]
    L.fl_graph_destroy.argtypes = [vp]
    L.fl_graph_destroy.restype = None
    gen = [vp, c_u32, vp, vp, vp, vp, vp, ctypes.c_int64, vp, P(c_u32)]
    L.fl_generate.argtypes = gen
    L.fl_generate_timed.argtypes = gen + [P(c_dbl), P(c_dbl)]
    L.fl_batch_create.argtypes = [c_u32, vp, vp, vp, vp, vp, vp, vp, vp, vp, P(vp)]
    L.fl_graph_num_terrains.argtypes = [vp]
    L.fl_graph_num_terrains.restype = c_u32
    L.fl_graph_device_bytes.argtypes = [vp]
    L.fl_graph_device_bytes.restype = c_u64
    L.fl_model_device_bytes.argtypes = [c_u32, c_u64]
    L.fl_model_device_bytes.restype = c_u64
    L.fl_host_alloc.argtypes = [c_u64, P(vp)]
    L.fl_host_free.argtypes = [vp]
    L.fl_host_free.restype = None
    L.fl_interpolator_create.argtypes = [c_u32, vp, vp, P(vp)]
    L.fl_interpolator_destroy.argtypes = [vp]
    L.fl_interpolator_destroy.restype = None
    L.fl_interpolate.argtypes = [vp, vp, c_u64, vp, vp, vp, vp]
    L.fl_interpolate_gpu.argtypes = [vp, vp, c_u64, vp, vp, vp, vp]
    L.fl_interpolate_device.argtypes = [vp, vp, c_u64, vp, vp, vp, vp]
    L.fl_interpolator_last_deferred.argtypes = [vp]
    L.fl_interpolator_last_deferred.restype = c_u64
    L.fl_probe_interp_query.argtypes = [vp, vp, c_u64, vp, vp, c_int, vp, vp]
    L.fl_probe_prefilters.argtypes = [c_u64, vp, vp]
    L.fl_lake_rank.argtypes = [c_u32, vp, vp, vp, vp, c_u32, vp]
    L.fl_server_create.argtypes = [c_u64, c_u32, P(vp)]
    L.fl_server_add_model.argtypes = [vp, c_u32, vp, vp, vp, vp, vp, c_u32, vp, vp, P(c_u32)]
    L.fl_server_submit.argtypes = [vp, c_u32, vp, vp, vp, vp, vp, ctypes.c_int64, vp, P(c_u64)]
    L.fl_server_wait.argtypes = [vp, c_u64, P(c_u32), P(c_dbl), P(c_dbl), P(c_dbl)]
    L.fl_server_stats.argtypes = [vp, vp, c_u32]
    L.fl_server_destroy.argtypes = [vp]
    L.fl_server_destroy.restype = None
    L.fl_batch_generate.argtypes = [vp, c_u32, vp, vp, vp, vp, vp, ctypes.c_int64, vp, vp,
                                    P(c_u32), P(c_dbl), P(c_dbl)]
    L.fl_graph_num_sites.argtypes = [vp]
    L.fl_graph_num_sites.restype = c_u32
    L.fl_graph_num_slots.argtypes = [vp]
    L.fl_graph_num_slots.restype = c_u64
    L.fl_last_error.restype = ctypes.c_char_p
    L.fl_select_device.argtypes = [c_int]
    L.fl_graph_set_timing.argtypes = [vp, c_int]
    L.fl_graph_reset_stats.argtypes = [vp]
    L.fl_graph_reset_stats.restype = None
    L.fl_graph_host_syncs.argtypes = [vp]
    L.fl_graph_host_syncs.restype = c_u64
    L.fl_set_tuning.argtypes = [ctypes.c_char_p, ctypes.c_int64]
    L.fl_get_tuning.argtypes = [ctypes.c_char_p]
    L.fl_get_tuning.restype = ctypes.c_int64
    L.fl_graph_rank_info.argtypes = [vp, P(c_dbl), P(c_int)]
    L.fl_schedule_entry.argtypes = [c_u32, P(c_u32), P(c_int), P(c_int), P(c_u32), P(c_u32),
                                    P(c_int)]
    L.fl_probe_lake_rank_gpu.argtypes = [vp, vp, c_u32, vp, P(c_int)]
    L.fl_num_kernel_classes.restype = c_u32
    L.fl_graph_kernel_stats.argtypes = [vp, c_u32, P(ctypes.c_char_p), P(c_u64), P(c_dbl), P(c_dbl)]
    L.fl_graph_basin_stats.argtypes = [vp, vp, c_u32]
    L.fl_graph_round_trace.argtypes = [vp, c_u32, P(c_u32), vp, vp, vp]
    L.fl_basin_labels_noalloc.argtypes = [c_u32, vp, vp, vp, P(c_int), vp]
    L.fl_probe_receivers.argtypes = [vp, vp, vp, vp, P(c_int)]
    L.fl_probe_lakes.argtypes = [vp, vp, c_u32, vp, vp, vp]
    L.fl_probe_tree_pass.argtypes = [vp, vp, c_u32, vp, vp, vp, vp, vp, vp, vp, P(c_int)]
    L.fl_probe_prim_rank.argtypes = [vp, vp, c_u32, vp]
    L.fl_probe_rng_f64.argtypes = [c_u64, c_u64, c_u64, vp]
    L.fl_probe_chain_fold.argtypes = [vp, c_u32, c_dbl, vp]
    L.fl_random_sites.argtypes = [c_u64, c_dbl, c_dbl, c_dbl, c_dbl, c_u64, c_int, vp, vp]
    L.fl_relax_sites.argtypes = [c_u32, vp, vp, c_dbl, c_dbl, c_dbl, c_dbl, c_u32]
    L.fl_build_graph.argtypes = [c_u32, vp, vp, c_dbl, c_dbl, c_dbl, c_dbl, vp, vp, vp, c_u64,
                                 vp, vp, P(c_u64), P(c_u32)]
    L.fl_triangulate.argtypes = [c_u32, vp, vp, vp, c_u64]
    L.fl_triangulate.restype = ctypes.c_int64
    _lib = L
    return L


def last_error():
    return lib().fl_last_error().decode()


def check(rc):
    if rc != FL_OK:
        raise FastlemError(rc, last_error())
    return rc


def ptr(a):
    """Raw pointer of a C-contiguous numpy array (None passes NULL)."""
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(vp)


class _PinnedBlock:
    """Owner of one fl_host_alloc block; freed when the last array over it is gone."""

    def __init__(self, nbytes):
        p = vp()
        check(lib().fl_host_alloc(nbytes, ctypes.byref(p)))
        self.p = p.value

    def __del__(self):
        if self.p and _lib is not None:
            _lib.fl_host_free(vp(self.p))
            self.p = None


def pinned_empty(n, dtype):
    """An uninitialised 1-D numpy array of n elements in page-locked host memory
    (fl_host_alloc): host<->device copies of it run by DMA at the link's rate."""
    dtype = np.dtype(dtype)
    nbytes = max(1, int(n) * dtype.itemsize)
    block = _PinnedBlock(nbytes)
    raw = (ctypes.c_uint8 * nbytes).from_address(block.p)
    raw._block = block               # the buffer keeps its block alive
    return np.frombuffer(raw, dtype=dtype, count=int(n))


def as_u32(a):
    return np.ascontiguousarray(a, dtype=np.uint32)


def as_f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def as_u8(a):
    return np.ascontiguousarray(a, dtype=np.uint8)


def kernel_stats(handle):
    """{class name: (launches, device_ms, algorithmic_bytes)} of a model handle."""
    L = lib()
    out = {}
    for c in range(L.fl_num_kernel_classes()):
        name = ctypes.c_char_p()
        n = c_u64()
        ms = c_dbl()
        b = c_dbl()
        check(L.fl_graph_kernel_stats(handle, c, ctypes.byref(name), ctypes.byref(n), ctypes.byref(ms),
                                      ctypes.byref(b)))
        out[name.value.decode()] = (n.value, ms.value, b.value)
    return out


TUNING = ("low_ilp", "walk_per_sm", "sized_grids", "gpu_rank", "kahn_min_width")


def set_tuning(**kw):
    """Sets launch-shape / switch-point knobs (see fl_set_tuning); returns the previous
    values of the ones set."""
    L = lib()
    old = {}
    for k, v in kw.items():
        old[k] = int(L.fl_get_tuning(k.encode()))
        check(L.fl_set_tuning(k.encode(), int(v)))
    return old


def schedule():
    """The library's compiled-in schedule: [(max_sites, packed, low_ilp, walk_per_sm,
    kahn_min_width, sized_grids)]."""
    out = []
    i = 0
    while True:
        v = [c_u32(), c_int(), c_int(), c_u32(), c_u32(), c_int()]
        if lib().fl_schedule_entry(i, *[ctypes.byref(x) for x in v]) != FL_OK:
            return out
        out.append(tuple(int(x.value) for x in v))
        i += 1


def get_tuning():
    L = lib()
    return {k: int(L.fl_get_tuning(k.encode())) for k in TUNING}


def rank_info(handle):
    """(ms, where) of the model's last lake-order computation: where is "gpu", "host" or
    None."""
    ms = c_dbl()
    on = c_int()
    check(lib().fl_graph_rank_info(handle, ctypes.byref(ms), ctypes.byref(on)))
    return ms.value, {1: "gpu", 0: "host"}.get(on.value)


def host_syncs(handle):
    """Blocking host synchronisations of a model handle since its last stats reset."""
    return int(lib().fl_graph_host_syncs(handle))


BASIN_STATS = ["kahn_rounds", "leaves", "skeleton_sites", "chains", "longest_chain", "slow_sites",
               "wait_spins_up", "wait_spins_down", "up_slowest_ns", "up_slowest_pull_cycles",
               "up_slowest_pulls", "down_slowest_ns", "down_slowest_wait_cycles",
               "down_slowest_len"]


def basin_stats(handle):
    """Shape of the last basin pass of a model handle."""
    out = np.zeros(len(BASIN_STATS), np.uint64)
    check(lib().fl_graph_basin_stats(handle, out.ctypes.data_as(vp), len(BASIN_STATS)))
    return dict(zip(BASIN_STATS, (int(x) for x in out)))


def round_trace(handle, cap=1 << 16):
    """Kahn-round structure of the last basin pass: (offsets, up_ns, down_ns), each
    of length rounds + 1 (device clock in ns; see fl_graph_round_trace)."""
    r = ctypes.c_uint32(0)
    off = np.zeros(cap, np.uint32)
    up = np.zeros(cap, np.uint64)
    down = np.zeros(cap, np.uint64)
    check(lib().fl_graph_round_trace(handle, cap, ctypes.byref(r), off.ctypes.data_as(vp),
                                     up.ctypes.data_as(vp), down.ctypes.data_as(vp)))
    k = min(cap, r.value + 1)
    return off[:k], up[:k], down[:k]
