"""fastlem's public API over the GB300 C ABI.

The names, builder-style setters, argument meaning and error behaviour follow fastlem
0.1.4:
  Site2D                  src/models/surface/sites.rs:7-35
  TopographicalParameters src/core/parameters.rs:24-74
  TerrainModel2DBulider   src/models/surface/builder.rs:31-322  (sic, fastlem's spelling)
  TerrainModel2D          src/models/surface/model.rs:18-69
  TerrainGenerator        src/lem/generator.rs:37-214
  Terrain2D               src/models/surface/terrain.rs:8-39
  GenerationError         src/lem/generator.rs:18-26
  ModelBuilderError       src/models/surface/builder.rs:14-21
The solve itself runs in libfastlem_gb300.so on the GPU; this module only moves
arrays.  Per-site parameters may also be given as arrays (ParameterArrays), which is
how large models should be driven.
"""
import ctypes
import math
from dataclasses import dataclass, replace
from typing import Optional, Sequence

import numpy as np

from . import _lib
from ._lib import as_f64, as_u32, as_u8, check, lib, pinned_empty, ptr


class GenerationError(Exception):
    """lem/generator.rs:18-26."""
    InvalidNumberOfParameters = "InvalidNumberOfParameters"
    ParametersNotSet = "ParametersNotSet"
    ModelNotSet = "ModelNotSet"

    _MSG = {
        "InvalidNumberOfParameters": "The number of topographical parameters must be equal to the number of sites",
        "ParametersNotSet": "You must set topographical parameters before generating terrain",
        "ModelNotSet": "You must set `TerrainModel` before generating terrain",
    }

    def __init__(self, kind):
        super().__init__(self._MSG[kind])
        self.kind = kind


class ModelBuilderError(Exception):
    """models/surface/builder.rs:14-21."""
    SitesNotSet = "SitesNotSet"
    BoundsNotSet = "BoundsNotSet"
    VoronoiError = "VoronoiError"

    _MSG = {
        "SitesNotSet": "You must set sites using `set_sites`",
        "BoundsNotSet": "You must set the bounding box using `set_bounding_box`",
        "VoronoiError": "Failed to calculate voronoi diagram",
    }

    def __init__(self, kind):
        super().__init__(self._MSG[kind])
        self.kind = kind


_GEN_ERR = {_lib.FL_ERR_MODEL_NOT_SET: "ModelNotSet",
            _lib.FL_ERR_PARAMETERS_NOT_SET: "ParametersNotSet",
            _lib.FL_ERR_INVALID_NUM_PARAMETERS: "InvalidNumberOfParameters"}


@dataclass(frozen=True)
class Site2D:
    x: float = 0.0
    y: float = 0.0

    def distance(self, other: "Site2D") -> float:
        return math.sqrt((self.x - other.x) ** 2 + (self.y - other.y) ** 2)

    def squared_distance(self, other: "Site2D") -> float:
        return (self.x - other.x) ** 2 + (self.y - other.y) ** 2


@dataclass(frozen=True)
class TopographicalParameters:
    """Defaults as core/parameters.rs:37-47; setters return a modified copy."""
    base_elevation: float = 0.0
    erodibility: float = 1.0
    uplift_rate: float = 1.0
    is_outlet: bool = False
    max_slope: Optional[float] = None

    def set_base_elevation(self, v):
        return replace(self, base_elevation=float(v))

    def set_erodibility(self, v):
        return replace(self, erodibility=float(v))

    def set_uplift_rate(self, v):
        return replace(self, uplift_rate=float(v))

    def set_is_outlet(self, v):
        return replace(self, is_outlet=bool(v))

    def set_max_slope(self, v):
        return replace(self, max_slope=None if v is None else float(v))


class ParameterArrays:
    """Structure-of-arrays form of a Vec<TopographicalParameters> (same meaning per
    site; max_slope NaN = None)."""

    def __init__(self, n, base_elevation=0.0, erodibility=1.0, uplift_rate=1.0, is_outlet=False,
                 max_slope=None):
        def full(v, dt):
            a = np.asarray(v, dtype=dt)
            return np.ascontiguousarray(np.broadcast_to(a, (n,)) if a.ndim == 0 else a)
        self.base = full(base_elevation, np.float64)
        self.erodibility = full(erodibility, np.float64)
        self.uplift = full(uplift_rate, np.float64)
        self.is_outlet = full(is_outlet, np.uint8)
        self.max_slope = None if max_slope is None else full(max_slope, np.float64)

    def __len__(self):
        return len(self.base)

    def pinned(self) -> "ParameterArrays":
        """A copy whose arrays live in page-locked host memory, so generate() uploads
        them by DMA, overlapped with its host-side work."""
        q = ParameterArrays.__new__(ParameterArrays)
        for name in ("base", "erodibility", "uplift", "is_outlet", "max_slope"):
            a = getattr(self, name)
            if a is not None:
                b = pinned_empty(len(a), a.dtype)
                b[:] = a
                a = b
            setattr(q, name, a)
        return q

    @staticmethod
    def from_list(params: Sequence[TopographicalParameters]) -> "ParameterArrays":
        n = len(params)
        ms = [p.max_slope for p in params]
        has_ms = any(m is not None for m in ms)
        return ParameterArrays(
            n,
            [p.base_elevation for p in params],
            [p.erodibility for p in params],
            [p.uplift_rate for p in params],
            [p.is_outlet for p in params],
            [math.nan if m is None else m for m in ms] if has_ms else None)


class TerrainModel2D:
    """Sites, cell areas, the adjacency graph (CSR in insertion order) and default
    outlets.  The graph is uploaded to the GPU on the first generate() and stays
    resident until the model is dropped."""

    def __init__(self, xs, ys, areas, row_ptr, col, length, default_outlets):
        self.xs = as_f64(xs)
        self.ys = as_f64(ys)
        self.area = as_f64(areas)
        self.row_ptr = as_u32(row_ptr)
        self.col = as_u32(col)
        self.length = as_f64(length)
        self.default_outlets = as_u32(default_outlets)
        self.n = len(self.row_ptr) - 1
        self._handle = None

    # Model trait (core/traits.rs:12-19)
    def num(self):
        return self.n

    def sites(self):
        return [Site2D(float(x), float(y)) for x, y in zip(self.xs, self.ys)]

    def areas(self):
        return self.area

    def default_outlets_list(self):
        return self.default_outlets

    def neighbors_of(self, i):
        s, e = self.row_ptr[i], self.row_ptr[i + 1]
        return list(zip(self.col[s:e].tolist(), self.length[s:e].tolist()))

    def handle(self):
        """Device-resident graph (created on first use)."""
        if self._handle is None:
            h = ctypes.c_void_p()
            check(lib().fl_graph_create(self.n, ptr(self.row_ptr), ptr(self.col), ptr(self.length),
                                        ptr(self.area), ptr(self.default_outlets),
                                        len(self.default_outlets), ptr(self.xs), ptr(self.ys),
                                        ctypes.byref(h)))
            self._handle = h
        return self._handle

    def release(self):
        if self._handle is not None:
            lib().fl_graph_destroy(self._handle)
            self._handle = None

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass

    def interpolator(self):
        """The sites' natural-neighbour interpolator (built on first use, host memory),
        shared by every Terrain2D of this model (models/surface/model.rs:62-68)."""
        if getattr(self, "_interp", None) is None:
            self._interp = TerrainInterpolator2D(self.xs, self.ys)
        return self._interp

    def create_terrain_from_result(self, elevations):
        return Terrain2D(self.xs, self.ys, elevations, interpolator=self.interpolator)


class TerrainModel2DBulider:
    """models/surface/builder.rs:31-322 (fastlem spells it `Bulider`)."""

    def __init__(self, xs=None, ys=None, bound_min=None, bound_max=None):
        self.xs = None if xs is None else as_f64(xs)
        self.ys = None if ys is None else as_f64(ys)
        self.bound_min = bound_min
        self.bound_max = bound_max

    @staticmethod
    def default():
        return TerrainModel2DBulider()

    @staticmethod
    def from_random_sites(num, bound_min: Site2D, bound_max: Site2D, seed=None):
        """builder.rs:38-52 (StdRng::from_seed([0; 32])); `seed` switches to
        StdRng::seed_from_u64(seed) for seeded synthetic workloads."""
        xs = np.empty(num, np.float64)
        ys = np.empty(num, np.float64)
        check(lib().fl_random_sites(num, bound_min.x, bound_min.y, bound_max.x, bound_max.y,
                                    0 if seed is None else seed, 1 if seed is None else 0,
                                    ptr(xs), ptr(ys)))
        return TerrainModel2DBulider(xs, ys, bound_min, bound_max)

    def set_sites(self, sites):
        if isinstance(sites, tuple) and len(sites) == 2:
            xs, ys = sites
        else:
            xs = [s.x for s in sites]
            ys = [s.y for s in sites]
        return TerrainModel2DBulider(xs, ys, self.bound_min, self.bound_max)

    def set_bounding_box(self, bound_min: Optional[Site2D], bound_max: Optional[Site2D]):
        return TerrainModel2DBulider(self.xs, self.ys, bound_min, bound_max)

    def _query_bounds(self):
        if self.bound_min is not None:
            bmin = self.bound_min
        elif self.xs is not None:
            bmin = Site2D(float(np.min(self.xs)), float(np.min(self.ys)))
        else:
            raise ModelBuilderError("BoundsNotSet")
        if self.bound_max is not None:
            bmax = self.bound_max
        elif self.xs is not None:
            bmax = Site2D(float(np.max(self.xs)), float(np.max(self.ys)))
        else:
            raise ModelBuilderError("BoundsNotSet")
        return bmin, bmax

    @staticmethod
    def _box(bmin, bmax):
        # voronoice BoundingBox::new(center, width, height) as builder.rs:162-171 builds it
        cx, cy = (bmax.x + bmin.x) / 2.0, (bmax.y + bmin.y) / 2.0
        w, h = bmax.x - bmin.x, bmax.y - bmin.y
        return cx - w / 2.0, cy - h / 2.0, cx + w / 2.0, cy + h / 2.0

    def add_edge_sites(self, edge_num_x: Optional[int], edge_num_y: Optional[int]):
        """builder.rs:54-131: evenly spaced sites along the four box edges."""
        if self.xs is None:
            raise ModelBuilderError("SitesNotSet")
        if self.bound_min is None or self.bound_max is None:
            raise ModelBuilderError("BoundsNotSet")
        bmin, bmax = self.bound_min, self.bound_max
        n = len(self.xs)
        corners = [(bmin.x, bmin.y), (bmin.x, bmax.y), (bmax.x, bmax.y), (bmax.x, bmin.y)]
        ex, ey = [], []
        for i, c in enumerate(corners):
            nx_ = corners[(i + 1) % 4]
            if i % 2 == 1:
                num = edge_num_x if edge_num_x is not None else int(
                    math.sqrt(n / (bmax.y - bmin.y) * (bmax.x - bmin.x)))
            else:
                num = edge_num_y if edge_num_y is not None else int(
                    math.sqrt(n / (bmax.x - bmin.x) * (bmax.y - bmin.y)))
            for j in range(num):
                t = j / num
                ex.append(c[0] * (1.0 - t) + nx_[0] * t)
                ey.append(c[1] * (1.0 - t) + nx_[1] * t)
        xs = np.concatenate([self.xs, np.asarray(ex, np.float64)])
        ys = np.concatenate([self.ys, np.asarray(ey, np.float64)])
        return TerrainModel2DBulider(xs, ys, self.bound_min, self.bound_max)

    def relaxate_sites(self, times: int):
        """builder.rs:155-200: `times` Lloyd iterations inside the bounding box."""
        if times == 0:
            return self
        bmin, bmax = self._query_bounds()
        if self.xs is None:
            raise ModelBuilderError("SitesNotSet")
        xs, ys = self.xs.copy(), self.ys.copy()
        x0, y0, x1, y1 = self._box(bmin, bmax)
        rc = lib().fl_relax_sites(len(xs), ptr(xs), ptr(ys), x0, y0, x1, y1, times)
        if rc == _lib.FL_ERR_BUILDER_VORONOI:
            raise ModelBuilderError("VoronoiError")
        check(rc)
        return TerrainModel2DBulider(xs, ys, self.bound_min, self.bound_max)

    def build(self) -> TerrainModel2D:
        """builder.rs:202-281."""
        if self.xs is None:
            raise ModelBuilderError("SitesNotSet")
        bmin, bmax = self._query_bounds()
        n = len(self.xs)
        x0, y0, x1, y1 = self._box(bmin, bmax)
        cap = 6 * n + 6
        row = np.empty(n + 1, np.uint32)
        col = np.empty(cap, np.uint32)
        ln = np.empty(cap, np.float64)
        area = np.empty(n, np.float64)
        hull = np.empty(n, np.uint32)
        nnz = ctypes.c_uint64()
        nh = ctypes.c_uint32()
        rc = lib().fl_build_graph(n, ptr(self.xs), ptr(self.ys), x0, y0, x1, y1, ptr(row), ptr(col),
                                  ptr(ln), cap, ptr(area), ptr(hull), ctypes.byref(nnz),
                                  ctypes.byref(nh))
        if rc == _lib.FL_ERR_BUILDER_VORONOI:
            raise ModelBuilderError("VoronoiError")
        check(rc)
        m = nnz.value
        return TerrainModel2D(self.xs, self.ys, area, row, col[:m].copy(), ln[:m].copy(),
                              hull[:nh.value].copy())


class TerrainInterpolator2D:
    """models/surface/interpolator.rs:6-29: Sibson natural-neighbour interpolation over
    the sites' Delaunay triangulation (fl_interpolator_*); None outside the convex hull."""

    def __init__(self, xs, ys):
        self.xs, self.ys = as_f64(xs), as_f64(ys)
        h = ctypes.c_void_p()
        check(lib().fl_interpolator_create(len(self.xs), ptr(self.xs), ptr(self.ys),
                                           ctypes.byref(h)))
        self._h = h

    def interpolate_many(self, elevations, qx, qy, gpu=False):
        """(values, found) for arrays of query coordinates; values are NaN where the
        query lies outside the hull (found False).  gpu=True answers them on the GPU
        (fl_interpolate_gpu), with the same bits."""
        e = as_f64(elevations)
        if len(e) != len(self.xs):
            raise ValueError("one elevation per site")
        qx, qy = as_f64(qx), as_f64(qy)
        if qx.shape != qy.shape:
            raise ValueError("qx and qy differ in shape")
        out = np.empty(qx.shape, np.float64)
        found = np.empty(qx.shape, np.uint8)
        call = lib().fl_interpolate_gpu if gpu else lib().fl_interpolate
        check(call(self._h, ptr(e), qx.size, ptr(qx), ptr(qy), ptr(out), ptr(found)))
        return out, found.astype(bool)

    def interpolate_device(self, elevations, qx, qy, out, found):
        """fl_interpolate_device on torch CUDA tensors (float64 elevations, queries and
        out, uint8 found), all on the device the interpolator uses."""
        import torch
        for name, t, dt in (("elevations", elevations, torch.float64), ("qx", qx, torch.float64),
                            ("qy", qy, torch.float64), ("out", out, torch.float64),
                            ("found", found, torch.uint8)):
            if not (t.is_cuda and t.dtype == dt and t.is_contiguous()):
                raise ValueError(f"{name}: a contiguous CUDA tensor of {dt} is wanted")
        if elevations.numel() != len(self.xs):
            raise ValueError("one elevation per site")
        m = qx.numel()
        if qy.numel() != m or out.numel() != m or found.numel() != m:
            raise ValueError("qx, qy, out and found differ in size")
        torch.cuda.current_stream().synchronize()      # inputs written by torch are complete
        check(lib().fl_interpolate_device(self._h, elevations.data_ptr(), m, qx.data_ptr(),
                                          qy.data_ptr(), out.data_ptr(), found.data_ptr()))

    def interpolate(self, elevations, site):
        v, ok = self.interpolate_many(elevations, np.array([site.x]), np.array([site.y]))
        return float(v[0]) if ok[0] else None

    def __del__(self):
        try:
            if getattr(self, "_h", None) is not None:
                lib().fl_interpolator_destroy(self._h)
                self._h = None
        except Exception:
            pass


class Terrain2D:
    """models/surface/terrain.rs:8-39."""

    def __init__(self, xs, ys, elevations, interpolator=None):
        self.xs = xs
        self.ys = ys
        self._elev = elevations
        self._interp = interpolator      # a TerrainInterpolator2D or a callable making one

    def sites(self):
        return [Site2D(float(x), float(y)) for x, y in zip(self.xs, self.ys)]

    def elevations(self):
        return self._elev

    def _interpolator(self):
        if self._interp is None:
            self._interp = TerrainInterpolator2D(self.xs, self.ys)
        elif not isinstance(self._interp, TerrainInterpolator2D):
            self._interp = self._interp()
        return self._interp

    def get_elevation(self, site: Site2D):
        """Interpolated elevation at `site` (terrain.rs:35-38), None outside the hull."""
        return self._interpolator().interpolate(self._elev, site)

    def get_elevations(self, xs, ys, gpu=False):
        """get_elevation for arrays of coordinates at once: NaN where it is None
        (gpu=True: computed on the GPU, the same values)."""
        return self._interpolator().interpolate_many(self._elev, xs, ys, gpu=gpu)[0]


class TerrainGenerator:
    """lem/generator.rs:37-214: builder-style configuration, then generate()."""

    def __init__(self):
        self.model = None
        self.parameters = None
        self.max_iteration = None
        self.last_iterations = None
        self.last_loop_ms = None
        self.last_total_ms = None

    @staticmethod
    def default():
        return TerrainGenerator()

    def set_model(self, model: TerrainModel2D):
        self.model = model
        return self

    def set_parameters(self, parameters):
        self.parameters = parameters
        return self

    def set_max_iteration(self, max_iteration: int):
        self.max_iteration = int(max_iteration)
        return self

    def generate(self, out=None) -> Terrain2D:
        """`out`: optional float64 array of num() sites that receives the elevations
        (e.g. one from pinned_empty, reused across calls); the result wraps it."""
        # error order as generator.rs:91-116
        if self.model is None:
            raise GenerationError("ModelNotSet")
        if self.parameters is None:
            raise GenerationError("ParametersNotSet")
        p = self.parameters
        if not isinstance(p, ParameterArrays):
            p = ParameterArrays.from_list(p)
        m = self.model
        if len(p) != m.num():
            raise GenerationError("InvalidNumberOfParameters")
        if out is None:
            out = np.empty(m.num(), np.float64)
        elif out.dtype != np.float64 or out.shape != (m.num(),) or not out.flags["C_CONTIGUOUS"]:
            raise ValueError("out must be a contiguous float64 array of num() elements")
        iters = ctypes.c_uint32()
        loop_ms = ctypes.c_double()
        total_ms = ctypes.c_double()
        mi = -1 if self.max_iteration is None else self.max_iteration
        rc = lib().fl_generate_timed(m.handle(), len(p), ptr(p.base), ptr(p.erodibility),
                                     ptr(p.uplift), ptr(p.is_outlet),
                                     ptr(p.max_slope) if p.max_slope is not None else None,
                                     mi, ptr(out), ctypes.byref(iters),
                                     ctypes.byref(loop_ms), ctypes.byref(total_ms))
        if rc in _GEN_ERR:
            raise GenerationError(_GEN_ERR[rc])
        check(rc)
        self.last_iterations = iters.value
        self.last_loop_ms = loop_ms.value
        self.last_total_ms = total_ms.value
        return m.create_terrain_from_result(out)

