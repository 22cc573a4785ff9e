"""Terrain2D::get_elevation on the GPU (fl_interpolate_gpu / fl_interpolate_device,
src/models/surface/interpolator.rs:17-29): the device queries give the host queries'
bits (tests/test_interp.py pins the host queries against Sibson's definition), on
random sites, on sites where the predicates' filters cannot decide (lattices, sites on
one circle, queries on edges, on circumcircles, at sites, on the hull), for batches
below and above the size that is sorted by grid cell, and through the device-array
form."""
import ctypes

import numpy as np
import pytest

from fastlem_gb300 import Site2D, TerrainModel2DBulider
from fastlem_gb300._lib import FL_ERR_INVALID_ARGUMENT, FL_OK, FastlemError, ptr
from fastlem_gb300.api import Terrain2D, TerrainInterpolator2D


def both(it, f, qx, qy):
    host, hok = it.interpolate_many(f, qx, qy)
    dev, dok = it.interpolate_many(f, qx, qy, gpu=True)
    return host, hok, dev, dok


def assert_same_bits(it, f, qx, qy):
    host, hok, dev, dok = both(it, f, qx, qy)
    assert np.array_equal(hok, dok)
    assert np.array_equal(host.view(np.uint64), dev.view(np.uint64))
    return host, hok


def test_gpu_interp_argument_checks(fl_lib):
    """Null arguments fail before any CUDA call; an empty batch does nothing."""
    xs, ys = np.array([0.0, 1.0, 0.0]), np.array([0.0, 0.0, 1.0])
    it = TerrainInterpolator2D(xs, ys)
    z = np.zeros(1)
    found = np.zeros(1, np.uint8)
    for call in (fl_lib.fl_interpolate_gpu, fl_lib.fl_interpolate_device):
        assert call(None, ptr(z), 1, ptr(z), ptr(z), ptr(z), ptr(found)) == FL_ERR_INVALID_ARGUMENT
        assert call(it._h, None, 1, ptr(z), ptr(z), ptr(z), ptr(found)) == FL_ERR_INVALID_ARGUMENT
        assert call(it._h, ptr(z), 1, ptr(z), None, ptr(z), ptr(found)) == FL_ERR_INVALID_ARGUMENT
        assert call(it._h, None, 0, None, None, None, None) == FL_OK


@pytest.mark.gpu
@pytest.mark.parametrize("count", [5_000, 300_000])
def test_random_sites_same_bits(count):
    r = np.random.default_rng(11)
    xs, ys = r.uniform(0, 100, 20_000), r.uniform(0, 100, 20_000)
    it = TerrainInterpolator2D(xs, ys)
    f = r.normal(0, 1, len(xs))
    qx, qy = r.uniform(-5, 105, count), r.uniform(-5, 105, count)
    qx[:3], qy[:3] = np.nan, [1.0, np.inf, np.nan]
    v, ok = assert_same_bits(it, f, qx, qy)
    assert 0.8 < ok.mean() < 0.9 and not ok[:3].any()


@pytest.mark.gpu
def test_lattice_edges_sites_and_hull_same_bits():
    """Sites on a lattice: every cell's four corners share a circle, queries at sites,
    on edges (orientation exactly zero), on hull edges and cell centres."""
    g = np.arange(0.0, 60.0, 2.0)
    X, Y = np.meshgrid(g, g)
    xs, ys = X.ravel(), Y.ravel()
    it = TerrainInterpolator2D(xs, ys)
    r = np.random.default_rng(2)
    f = r.normal(0, 1, len(xs))
    h = np.arange(-1.0, 60.0, 1.0)                  # sites, edge midpoints, cell centres
    QX, QY = np.meshgrid(h, h)
    qx = np.concatenate([QX.ravel(), r.uniform(-1, 60, 50_000)])
    qy = np.concatenate([QY.ravel(), r.uniform(-1, 60, 50_000)])
    v, ok = assert_same_bits(it, f, qx, qy)
    site = np.isin(qx, g) & np.isin(qy, g)
    assert ok[site].all()
    on_sites = (qx[site] / 2).astype(int) + 30 * (qy[site] / 2).astype(int)
    assert np.array_equal(v[site], f[on_sites])


@pytest.mark.gpu
def test_queries_on_a_circle_of_sites_same_bits():
    """Twelve lattice points of x^2 + y^2 = 25, one left out and asked for: the in-circle
    determinant is exactly zero for triangles of the remaining eleven."""
    ring = [(3, 4), (4, 3), (0, 5), (-3, 4), (-4, 3), (-5, 0), (-3, -4), (-4, -3), (0, -5),
            (3, -4), (4, -3)]
    r = np.random.default_rng(4)
    ang = r.uniform(0, 2 * np.pi, 60)
    rad = r.uniform(8, 10, 60)
    xs = np.array([p[0] for p in ring] + list(rad * np.cos(ang)), np.float64)
    ys = np.array([p[1] for p in ring] + list(rad * np.sin(ang)), np.float64)
    it = TerrainInterpolator2D(xs, ys)
    f = r.normal(0, 1, len(xs))
    qx = np.array([5.0, 0.0, 0.5, -4.0, 3.0, 1.0])
    qy = np.array([0.0, 0.0, 0.25, 3.0, -4.0, 2.0])
    v, ok = assert_same_bits(it, f, qx, qy)
    assert ok.all()


@pytest.mark.gpu
def test_large_cavity_same_bits_and_too_large_fails():
    """Sites on one circle: a query near the centre is inside every circumcircle, so its
    cavity holds every triangle (the exact pass's global tables)."""
    def circle(n):
        t = np.linspace(0, 2 * np.pi, n, endpoint=False)
        return 100 * np.cos(t), 100 * np.sin(t)

    xs, ys = circle(1500)
    it = TerrainInterpolator2D(xs, ys)
    f = np.random.default_rng(8).normal(0, 1, len(xs))
    assert_same_bits(it, f, np.array([0.5, -3.0, 40.0]), np.array([0.25, 2.0, -20.0]))
    xs, ys = circle(3000)
    it = TerrainInterpolator2D(xs, ys)
    f = np.arange(len(xs), dtype=np.float64)
    with pytest.raises(FastlemError) as e:
        it.interpolate_many(f, np.array([0.5]), np.array([0.25]), gpu=True)
    assert "2048" in str(e.value)
    # the interpolator stays usable after the refusal (every point inside this hull has
    # the whole triangulation as its cavity, so ask at sites)
    v, ok = it.interpolate_many(f, xs[[0, 7]], ys[[0, 7]], gpu=True)
    assert ok.all() and v.tolist() == [0.0, 7.0]


@pytest.mark.gpu
def test_builder_model_render_grid_same_bits():
    """The fastlem-shaped path: a relaxed model's terrain rendered on a pixel grid that
    includes the bounding box's edges (hull edges lined with the builder's edge sites)."""
    model = (TerrainModel2DBulider.from_random_sites(30_000, Site2D(0.0, 0.0), Site2D(200.0, 100.0))
             .relaxate_sites(1).add_edge_sites(None, None).build())
    elev = np.random.default_rng(6).uniform(0, 50, model.num())
    terrain = model.create_terrain_from_result(elev)
    px = np.linspace(0.0, 200.0, 640)
    py = np.linspace(0.0, 100.0, 320)
    QX, QY = np.meshgrid(px, py)
    qx, qy = QX.ravel(), QY.ravel()
    host = terrain.get_elevations(qx, qy)
    dev = terrain.get_elevations(qx, qy, gpu=True)
    assert np.array_equal(host.view(np.uint64), dev.view(np.uint64))
    assert np.isfinite(dev).mean() > 0.99


@pytest.mark.gpu
def test_device_arrays_same_bits():
    torch = pytest.importorskip("torch")
    r = np.random.default_rng(13)
    xs, ys = r.uniform(0, 50, 8_000), r.uniform(0, 50, 8_000)
    it = TerrainInterpolator2D(xs, ys)
    f = r.normal(0, 1, len(xs))
    qx, qy = r.uniform(0, 50, 100_000), r.uniform(0, 50, 100_000)
    host, hok = it.interpolate_many(f, qx, qy)
    dev = torch.device("cuda", 0)
    t = lambda a: torch.from_numpy(a).to(dev)
    out = torch.empty(len(qx), dtype=torch.float64, device=dev)
    found = torch.empty(len(qx), dtype=torch.uint8, device=dev)
    it.interpolate_device(t(f), t(qx), t(qy), out, found)
    assert np.array_equal(found.cpu().numpy().astype(bool), hok)
    assert np.array_equal(out.cpu().numpy().view(np.uint64), host.view(np.uint64))
