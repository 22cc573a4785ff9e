"""CPU tests of the host model builder (builder.rs restated): Delaunay triangulation,
clipped Voronoi areas, the a<b edge rule and the hull outlets."""
import numpy as np
import pytest

from fastlem_gb300 import ModelBuilderError, Site2D, TerrainModel2DBulider
from fastlem_gb300._lib import lib, ptr


def _tri(xs, ys):
    cap = 2 * len(xs) + 8
    t = np.empty(cap * 3, np.uint32)
    m = lib().fl_triangulate(len(xs), ptr(xs), ptr(ys), ptr(t), cap)
    assert m > 0
    return t[:3 * m].reshape(-1, 3)


@pytest.mark.parametrize("n,seed", [(50, 1), (2000, 2), (20000, 3)])
def test_triangulation_is_delaunay(fl_lib, n, seed):
    scipy_spatial = pytest.importorskip("scipy.spatial")
    b = TerrainModel2DBulider.from_random_sites(n, Site2D(0, 0), Site2D(100, 50), seed=seed)
    tri = _tri(b.xs, b.ys)
    mine = {tuple(sorted(t)) for t in tri.tolist()}
    ref = {tuple(sorted(t)) for t in scipy_spatial.Delaunay(np.c_[b.xs, b.ys]).simplices.tolist()}
    assert mine == ref
    a, bb, c = tri.T
    x, y = b.xs, b.ys
    assert (((x[a] - x[c]) * (y[bb] - y[c]) - (y[a] - y[c]) * (x[bb] - x[c])) > 0).all()


def test_build_graph_contract(fl_lib):
    b = TerrainModel2DBulider.from_random_sites(3000, Site2D(0, 0), Site2D(200, 100), seed=5)
    m = b.build()
    n = m.num()
    assert n == 3000
    # areas: clipped cells tile the box
    assert abs(m.areas().sum() - 200 * 100) < 1e-6 * 200 * 100
    assert (m.areas() > 0).all()
    # symmetric adjacency, lengths are Euclidean distances
    rows = [set(m.col[m.row_ptr[i]:m.row_ptr[i + 1]].tolist()) for i in range(n)]
    for i in range(n):
        for j in rows[i]:
            assert i in rows[j]
    s = np.repeat(np.arange(n), np.diff(m.row_ptr.astype(np.int64)))
    d = np.sqrt((m.xs[s] - m.xs[m.col]) ** 2 + (m.ys[s] - m.ys[m.col]) ** 2)
    assert np.array_equal(d, m.length)
    # the a<b rule over counter-clockwise triangles drops some hull edges
    tri = _tri(m.xs, m.ys)
    edges = set()
    for a, bb, c in tri.tolist():
        for p, q in ((a, bb), (bb, c), (c, a)):
            if p < q:
                edges.add((p, q))
    assert sum(len(r) for r in rows) == 2 * len(edges)
    # default outlets are the convex hull
    hull = set(m.default_outlets.tolist())
    sp = pytest.importorskip("scipy.spatial")
    assert hull == set(sp.ConvexHull(np.c_[m.xs, m.ys]).vertices.tolist())


def test_from_random_sites_is_deterministic(fl_lib):
    a = TerrainModel2DBulider.from_random_sites(100, Site2D(0, 0), Site2D(10, 10))
    b = TerrainModel2DBulider.from_random_sites(100, Site2D(0, 0), Site2D(10, 10))
    assert np.array_equal(a.xs, b.xs) and np.array_equal(a.ys, b.ys)
    assert (a.xs >= 0).all() and (a.xs < 10).all()
    c = TerrainModel2DBulider.from_random_sites(100, Site2D(0, 0), Site2D(10, 10), seed=3)
    assert not np.array_equal(a.xs, c.xs)


def test_relaxation_moves_sites_inside_box(fl_lib):
    b = TerrainModel2DBulider.from_random_sites(2000, Site2D(0, 0), Site2D(100, 100), seed=9)
    r = b.relaxate_sites(1)
    assert (r.xs >= 0).all() and (r.xs <= 100).all() and (r.ys >= 0).all() and (r.ys <= 100).all()
    # Lloyd spreads the sites: the minimum pairwise spacing grows
    def min_edge(m):
        return m.length.min()
    assert min_edge(r.build()) > min_edge(b.build())


def test_builder_errors(fl_lib):
    with pytest.raises(ModelBuilderError) as e:
        TerrainModel2DBulider.default().build()
    assert e.value.kind == "SitesNotSet"
    with pytest.raises(ModelBuilderError) as e:
        TerrainModel2DBulider.default().set_sites([Site2D(0, 0), Site2D(1, 1)]).add_edge_sites(None, None)
    assert e.value.kind == "BoundsNotSet"
    with pytest.raises(ModelBuilderError) as e:
        TerrainModel2DBulider.default().set_sites([Site2D(0, 0), Site2D(1, 1), Site2D(2, 2)]).build()
    assert e.value.kind == "VoronoiError"


def test_add_edge_sites(fl_lib):
    b = TerrainModel2DBulider.from_random_sites(400, Site2D(0, 0), Site2D(100, 100), seed=2)
    e = b.add_edge_sites(None, None)
    # sqrt(400 / 100 * 100) = 20 sites per side, 4 sides
    assert len(e.xs) == 400 + 80
    assert e.build().num() == 480


def test_builder_entry_points_reject_null_arrays(fl_lib):
    """The C builder calls check their arrays before touching them."""
    from fastlem_gb300._lib import FL_ERR_INVALID_ARGUMENT
    import ctypes
    xs = np.array([0.0, 1.0, 0.0, 1.0])
    ys = np.array([0.0, 0.0, 1.0, 1.0])
    assert fl_lib.fl_random_sites(4, 0.0, 0.0, 1.0, 1.0, 0, 0, None, None) == FL_ERR_INVALID_ARGUMENT
    assert fl_lib.fl_relax_sites(4, None, None, 0.0, 0.0, 1.0, 1.0, 1) == FL_ERR_INVALID_ARGUMENT
    nnz, nh = ctypes.c_uint64(), ctypes.c_uint32()
    assert fl_lib.fl_build_graph(4, ptr(xs), ptr(ys), 0.0, 0.0, 1.0, 1.0, None, None, None, 24,
                                 None, None, ctypes.byref(nnz), ctypes.byref(nh)) == FL_ERR_INVALID_ARGUMENT
    assert fl_lib.fl_triangulate(4, None, None, None, 0) == -1
