"""Terrain2D::get_elevation (models/surface/terrain.rs:35-38): Sibson natural-neighbour
interpolation, None outside the convex hull.  The checker restates the definition
directly -- the query's Voronoi cell among the sites and the query, and the part of it
each site's own cell covered, both cut from a large box by half-planes -- so it shares
no code or construction with fl_interpolate's circumcentre polygons."""
import numpy as np
import pytest

from fastlem_gb300 import Site2D, TerrainModel2DBulider
from fastlem_gb300.api import Terrain2D, TerrainInterpolator2D
from fastlem_gb300._lib import FastlemError


def clip(poly, px, py, nx, ny):
    """Part of convex polygon `poly` with (x - p) . n <= 0."""
    out = []
    m = len(poly)
    for k in range(m):
        ax, ay = poly[k]
        bx, by = poly[(k + 1) % m]
        da = (ax - px) * nx + (ay - py) * ny
        db = (bx - px) * nx + (by - py) * ny
        if da <= 0:
            out.append((ax, ay))
        if (da < 0) != (db < 0) and da != db:
            t = da / (da - db)
            out.append((ax + t * (bx - ax), ay + t * (by - ay)))
    return out


def area(poly):
    s = 0.0
    for k in range(len(poly)):
        ax, ay = poly[k]
        bx, by = poly[(k + 1) % len(poly)]
        s += ax * by - bx * ay
    return abs(s) / 2


def closer_to(poly, a, others):
    """Cut `poly` to the points at least as close to a as to every point of others."""
    for b in others:
        mx, my = (a[0] + b[0]) / 2, (a[1] + b[1]) / 2
        poly = clip(poly, mx, my, b[0] - a[0], b[1] - a[1])
        if not poly:
            break
    return poly


def sibson_by_definition(xs, ys, f, qx, qy):
    pts = list(zip(xs.tolist(), ys.tolist()))
    big = 1e4
    box = [(qx - big, qy - big), (qx + big, qy - big), (qx + big, qy + big), (qx - big, qy + big)]
    cell = closer_to(box, (qx, qy), pts)
    num = den = 0.0
    for i, p in enumerate(pts):
        piece = closer_to(cell, p, pts[:i] + pts[i + 1:])
        if len(piece) >= 3:
            a = area(piece)
            num += a * f[i]
            den += a
    return num / den


def test_sibson_weights_match_the_definition():
    r = np.random.default_rng(3)
    xs, ys = r.uniform(0, 10, 70), r.uniform(0, 10, 70)
    it = TerrainInterpolator2D(xs, ys)
    for trial in range(2):
        f = r.normal(0, 1, len(xs))
        qx, qy = r.uniform(2, 8, 12), r.uniform(2, 8, 12)   # well inside the hull
        got, ok = it.interpolate_many(f, qx, qy)
        assert ok.all()
        for k in range(len(qx)):
            want = sibson_by_definition(xs, ys, f, qx[k], qy[k])
            assert got[k] == pytest.approx(want, rel=1e-9, abs=1e-9), (trial, k)


def test_linear_precision_constants_and_sites():
    r = np.random.default_rng(5)
    xs, ys = r.uniform(0, 100, 5000), r.uniform(0, 100, 5000)
    it = TerrainInterpolator2D(xs, ys)
    qx, qy = r.uniform(0, 100, 20000), r.uniform(0, 100, 20000)
    lin = 2.0 + 3.0 * xs - 5.0 * ys
    v, ok = it.interpolate_many(lin, qx, qy)
    assert ok.mean() > 0.95
    assert np.abs(v[ok] - (2.0 + 3.0 * qx[ok] - 5.0 * qy[ok])).max() < 1e-9
    assert np.isnan(v[~ok]).all()
    c, _ = it.interpolate_many(np.full(len(xs), 7.25), qx, qy)
    assert np.abs(c[ok] - 7.25).max() < 1e-12
    # a query at a site returns its value exactly
    f = r.normal(0, 1, len(xs))
    s, sok = it.interpolate_many(f, xs[:500], ys[:500])
    assert sok.all() and np.array_equal(s, f[:500])


def test_outside_the_hull_is_none():
    spatial = pytest.importorskip("scipy.spatial")
    r = np.random.default_rng(7)
    xs, ys = r.uniform(0, 10, 400), r.uniform(0, 10, 400)
    it = TerrainInterpolator2D(xs, ys)
    qx, qy = r.uniform(-2, 12, 5000), r.uniform(-2, 12, 5000)
    _, ok = it.interpolate_many(np.zeros(len(xs)), qx, qy)
    hull = spatial.Delaunay(np.c_[xs, ys])
    inside = hull.find_simplex(np.c_[qx, qy]) >= 0
    # points within rounding of the hull boundary may go either way
    assert (ok == inside).mean() > 0.999
    assert not ok[(qx < 0) | (qx > 10) | (qy < 0) | (qy > 10)].any()


def test_on_a_hull_edge_is_linear_along_it():
    xs = np.array([0.0, 4.0, 4.0, 0.0, 1.5])
    ys = np.array([0.0, 0.0, 4.0, 4.0, 2.5])
    f = np.array([1.0, 5.0, -3.0, 2.0, 10.0])
    it = TerrainInterpolator2D(xs, ys)
    v, ok = it.interpolate_many(f, np.array([1.0, 4.0]), np.array([0.0, 1.0]))
    assert ok.all()
    assert v[0] == pytest.approx(1.0 + 0.25 * 4.0)          # 1/4 of the way 0 -> 1
    assert v[1] == pytest.approx(5.0 + 0.25 * (-8.0))        # 1/4 of the way 1 -> 2


def test_degenerate_site_sets_are_rejected():
    with pytest.raises(FastlemError):
        TerrainInterpolator2D(np.array([0.0, 1.0]), np.array([0.0, 1.0]))
    with pytest.raises(FastlemError):
        TerrainInterpolator2D(np.array([0.0, 1.0, 2.0]), np.array([0.0, 1.0, 2.0]))


def test_terrain_get_elevation_through_the_model():
    """The fastlem-shaped path: a model's terrain answers get_elevation (None outside)."""
    model = (TerrainModel2DBulider.from_random_sites(2000, Site2D(0.0, 0.0), Site2D(50.0, 50.0))
             .relaxate_sites(1).build())
    xs, ys = model.xs, model.ys
    elev = 0.5 * xs + 0.25 * ys
    terrain = model.create_terrain_from_result(elev)
    v = terrain.get_elevation(Site2D(20.0, 30.0))
    assert v == pytest.approx(0.5 * 20.0 + 0.25 * 30.0, abs=1e-9)
    assert terrain.get_elevation(Site2D(-5.0, 10.0)) is None
    got = terrain.get_elevations(np.array([10.0, 60.0]), np.array([10.0, 10.0]))
    assert got[0] == pytest.approx(7.5, abs=1e-9) and np.isnan(got[1])
    # a Terrain2D made directly from sites builds its own interpolator
    t2 = Terrain2D(xs, ys, elev)
    assert t2.get_elevation(Site2D(20.0, 30.0)) == v
