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
        if self._handle is not None:
            return self._handle
        rows, cols, lens, areas, xs, ys, defs = [], [], [], [], [], [], []
        slot = 0
        def_off = np.zeros(len(self.models) + 1, np.uint32)
        for t, m in enumerate(self.models):
            base = int(self.site_off[t])
            rows.append(m.row_ptr[:-1].astype(np.uint64) + slot)
            cols.append(m.col.astype(np.uint64) + base)
            slot += int(m.row_ptr[-1])
            lens.append(m.length)
            areas.append(m.area)
            xs.append(m.xs)
            ys.append(m.ys)
            defs.append(m.default_outlets.astype(np.uint64) + base)
            def_off[t + 1] = def_off[t] + len(m.default_outlets)
        if slot >= 0xFFFFFFFF:
            raise ValueError("a batch holds fewer than 2^32 - 1 adjacency slots")
        row_ptr = np.concatenate(rows + [np.array([slot], np.uint64)]).astype(np.uint32)
        col = np.concatenate(cols).astype(np.uint32)
        length = np.ascontiguousarray(np.concatenate(lens), np.float64)
        area = np.ascontiguousarray(np.concatenate(areas), np.float64)
        x = np.ascontiguousarray(np.concatenate(xs), np.float64)
        y = np.ascontiguousarray(np.concatenate(ys), np.float64)
        d = np.concatenate(defs).astype(np.uint32)
        h = ctypes.c_void_p()
        check(lib().fl_batch_create(len(self.models), ptr(self.site_off), ptr(row_ptr), ptr(col),
                                    ptr(length), ptr(area), ptr(def_off), ptr(d), ptr(x), ptr(y),
                                    ctypes.byref(h)))
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
        cat = lambda f: np.ascontiguousarray(np.concatenate([getattr(p, f) for p in ps]))
        base, k, u = cat("base"), cat("erodibility"), cat("uplift")
        outl = np.ascontiguousarray(np.concatenate([p.is_outlet for p in ps]), np.uint8)
        slopes = None
        if any(p.max_slope is not None for p in ps):
            slopes = np.ascontiguousarray(np.concatenate(
                [p.max_slope if p.max_slope is not None else np.full(len(p), np.nan) for p in ps]))
        out = np.empty(b.n, np.float64)
        t_iters = np.zeros(b.num_terrains(), np.uint32)
        iters = ctypes.c_uint32()
        loop_ms, total_ms = ctypes.c_double(), ctypes.c_double()
        mi = -1 if self.max_iteration is None else self.max_iteration
        rc = lib().fl_batch_generate(b.handle(), b.n, ptr(base), ptr(k), ptr(u), ptr(outl),
                                     ptr(slopes) if slopes is not None else None, mi, ptr(out),
                                     ptr(t_iters), ctypes.byref(iters), ctypes.byref(loop_ms),
                                     ctypes.byref(total_ms))
        if rc in _GEN_ERR:
            raise GenerationError(_GEN_ERR[rc])
        check(rc)
        self.last_terrain_iterations = t_iters
        self.last_iterations = iters.value
        self.last_loop_ms = loop_ms.value
        self.last_total_ms = total_ms.value
        res = []
        for t, m in enumerate(b.models):
            a, e = int(b.site_off[t]), int(b.site_off[t + 1])
            res.append(m.create_terrain_from_result(out[a:e].copy()))
        return res
