"""Served form: generate() calls of different sizes taken as they arrive and run
concurrently on one GPU (fl_server_* in include/fastlem_gb300.h).

Models are registered once; every submitted request names a model and carries its
own TopographicalParameters, and its result equals TerrainGenerator.generate() for the
same model and parameters (lem/generator.rs:90-213).
"""
import ctypes
from dataclasses import dataclass

import numpy as np

from ._lib import check, lib, ptr
from .api import GenerationError, ParameterArrays, Terrain2D, TerrainModel2D, _GEN_ERR


@dataclass
class Ticket:
    id: int
    model: TerrainModel2D
    out: np.ndarray
    keep: tuple          # parameter arrays kept alive until the request is done


class TerrainServer:
    def __init__(self, hbm_budget_bytes=120 * 10**9, slots=4):
        h = ctypes.c_void_p()
        check(lib().fl_server_create(int(hbm_budget_bytes), int(slots), ctypes.byref(h)))
        self._h = h
        self._models = []
        # every submitted request's buffers stay referenced here until it is waited for
        # (or the server is closed): the workers write into them
        self._pending = {}

    def add_model(self, model: TerrainModel2D) -> int:
        mid = ctypes.c_uint32()
        check(lib().fl_server_add_model(self._h, model.n, ptr(model.row_ptr), ptr(model.col),
                                        ptr(model.length), ptr(model.area),
                                        ptr(model.default_outlets), len(model.default_outlets),
                                        ptr(model.xs), ptr(model.ys), ctypes.byref(mid)))
        self._models.append(model)
        return mid.value

    def submit(self, model_id: int, parameters, max_iteration=None) -> Ticket:
        m = self._models[model_id]
        p = parameters if isinstance(parameters, ParameterArrays) else ParameterArrays.from_list(parameters)
        if len(p) != m.num():
            raise GenerationError("InvalidNumberOfParameters")
        out = np.empty(m.num(), np.float64)
        t = ctypes.c_uint64()
        mi = -1 if max_iteration is None else int(max_iteration)
        rc = lib().fl_server_submit(self._h, model_id, ptr(p.base), ptr(p.erodibility),
                                    ptr(p.uplift), ptr(p.is_outlet),
                                    ptr(p.max_slope) if p.max_slope is not None else None, mi,
                                    ptr(out), ctypes.byref(t))
        if rc in _GEN_ERR:
            raise GenerationError(_GEN_ERR[rc])
        check(rc)
        ticket = Ticket(t.value, m, out, (p,))
        self._pending[ticket.id] = ticket
        return ticket

    def wait(self, ticket: Ticket):
        """(Terrain2D, {"iterations", "latency_ms", "queue_ms", "solve_ms"})"""
        it = ctypes.c_uint32()
        lat, qu, so = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        rc = lib().fl_server_wait(self._h, ticket.id, ctypes.byref(it), ctypes.byref(lat),
                                  ctypes.byref(qu), ctypes.byref(so))
        self._pending.pop(ticket.id, None)
        if rc in _GEN_ERR:
            raise GenerationError(_GEN_ERR[rc])
        check(rc)
        info = {"iterations": it.value, "latency_ms": lat.value, "queue_ms": qu.value,
                "solve_ms": so.value}
        return ticket.model.create_terrain_from_result(ticket.out), info

    STATS = ["completed", "peak_active", "peak_device_bytes", "device_bytes", "instances_created",
             "instances_evicted", "waiting", "packed_solves", "packed_requests"]

    def set_packing(self, enable: bool):
        """Continuous batching of small requests into packed solves (on by default)."""
        check(lib().fl_server_set_packing(self._h, 1 if enable else 0))
        return self

    def stats(self):
        out = np.zeros(len(self.STATS), np.uint64)
        check(lib().fl_server_stats(self._h, ptr(out), len(self.STATS)))
        return dict(zip(self.STATS, (int(x) for x in out)))

    def close(self):
        """Stops the server after the requests it is running; waiting ones are dropped."""
        if self._h is not None:
            lib().fl_server_destroy(self._h)   # joins the workers: no buffer is written after
            self._h = None
            self._pending.clear()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
