"""Batched form: many TerrainGenerator.generate() calls solved as one packed graph.

fastlem generates one terrain per generate() call (lem/generator.rs:90-213).  A batch
packs the CSR graphs of many TerrainModel2D into one device graph (global site ids,
per-terrain offsets) and runs every iteration's kernels over all of them at once;
fl_batch_generate keeps each terrain's own outlet resolution, noise stream and lake
order, so every terrain's elevations are bit-identical to its solo generate().
"""
import ctypes

import numpy as np

from ._lib import check, lib, ptr
from .api import GenerationError, ParameterArrays, Terrain2D, TerrainModel2D, _GEN_ERR


class TerrainBatch:
    """Models packed into one resident device graph (created on first use)."""

    def __init__(self, models):
        if not models:
            raise ValueError("a batch needs at least one model")
        self.models = list(models)
        ns = np.array([m.num() for m in self.models], np.int64)
        self.site_off = np.zeros(len(ns) + 1, np.uint32)
        self.site_off[1:] = np.cumsum(ns)
        if int(self.site_off[-1]) >= 0xFFFFFFFF:
            raise ValueError("a batch holds fewer than 2^32 - 1 sites")
        self.n = int(self.site_off[-1])
        self._handle = None

    def num_terrains(self):
        return len(self.models)

    def handle(self):
        """The packed device graph, built from every model's own arrays (no
        concatenated host copy: fl_batch_create_parts)."""
        if self._handle is not None:
            return self._handle
        k = len(self.models)
        if sum(int(m.row_ptr[-1]) for m in self.models) >= 0xFFFFFFFF:
            raise ValueError("a batch holds fewer than 2^32 - 1 adjacency slots")
        arr = lambda ctype, xs: (ctype * k)(*[x.ctypes.data_as(ctype) for x in xs])
        u32p, f64p = ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_double)
        ms = self.models
        sites = np.array([m.num() for m in ms], np.uint32)
        ndef = np.array([len(m.default_outlets) for m in ms], np.uint32)
        have_xy = all(m.xs is not None and m.ys is not None for m in ms)
        h = ctypes.c_void_p()
        check(lib().fl_batch_create_parts(
            k, ptr(sites), arr(u32p, [m.row_ptr for m in ms]), arr(u32p, [m.col for m in ms]),
            arr(f64p, [m.length for m in ms]), arr(f64p, [m.area for m in ms]), ptr(ndef),
            arr(u32p, [m.default_outlets for m in ms]),
            arr(f64p, [m.xs for m in ms]) if have_xy else None,
            arr(f64p, [m.ys for m in ms]) if have_xy else None, ctypes.byref(h)))
        self._handle = h
        return h

    def release(self):
        if self._handle is not None:
            lib().fl_graph_destroy(self._handle)
            self._handle = None

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass


class BatchGenerator:
    """TerrainGenerator for many (model, parameters) pairs at once.

    generate() returns one Terrain2D per pair, in order, each equal to what
    TerrainGenerator().set_model(model).set_parameters(parameters).generate() returns;
    last_terrain_iterations holds each terrain's own iteration count."""

    def __init__(self):
        self.batch = None
        self.parameters = None
        self.max_iteration = None
        self.last_terrain_iterations = None
        self.last_iterations = None
        self.last_loop_ms = None
        self.last_total_ms = None

    def set_batch(self, batch: TerrainBatch):
        self.batch = batch
        return self

    def set_models(self, models):
        return self.set_batch(TerrainBatch(models))

    def set_parameters(self, parameters):
        """One parameter list or ParameterArrays per model."""
        self.parameters = list(parameters)
        return self

    def set_max_iteration(self, max_iteration: int):
        self.max_iteration = int(max_iteration)
        return self

    def generate(self):
        if self.batch is None:
            raise GenerationError("ModelNotSet")
        if self.parameters is None:
            raise GenerationError("ParametersNotSet")
        b = self.batch
        ps = [p if isinstance(p, ParameterArrays) else ParameterArrays.from_list(p)
              for p in self.parameters]
        if len(ps) != b.num_terrains() or any(len(p) != m.num() for p, m in zip(ps, b.models)):
            raise GenerationError("InvalidNumberOfParameters")
        k = b.num_terrains()
        f64p = ctypes.POINTER(ctypes.c_double)
        u8p = ctypes.POINTER(ctypes.c_uint8)
        # the arrays stay referenced here while the call reads them
        keep = [[np.ascontiguousarray(getattr(p, f), dt) for p in ps]
                for f, dt in (("base", np.float64), ("erodibility", np.float64),
                              ("uplift", np.float64), ("is_outlet", np.uint8))]
        keep_slope = [None if p.max_slope is None else np.ascontiguousarray(p.max_slope, np.float64)
                      for p in ps]
        arr = lambda ctype, xs: (ctype * k)(*[None if x is None else x.ctypes.data_as(ctype)
                                              for x in xs])
        slopes = arr(f64p, keep_slope) if any(x is not None for x in keep_slope) else None
        outs = [np.empty(m.num(), np.float64) for m in b.models]
        t_iters = np.zeros(k, np.uint32)
        iters = ctypes.c_uint32()
        loop_ms, total_ms = ctypes.c_double(), ctypes.c_double()
        mi = -1 if self.max_iteration is None else self.max_iteration
        rc = lib().fl_batch_generate_parts(
            b.handle(), arr(f64p, keep[0]), arr(f64p, keep[1]), arr(f64p, keep[2]),
            arr(u8p, keep[3]), slopes, mi,
            arr(f64p, outs), ptr(t_iters), ctypes.byref(iters), ctypes.byref(loop_ms),
            ctypes.byref(total_ms))
        if rc in _GEN_ERR:
            raise GenerationError(_GEN_ERR[rc])
        check(rc)
        self.last_terrain_iterations = t_iters
        self.last_iterations = iters.value
        self.last_loop_ms = loop_ms.value
        self.last_total_ms = total_ms.value
        return [m.create_terrain_from_result(o) for m, o in zip(b.models, outs)]
