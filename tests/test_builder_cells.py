"""Per-cell checks of the host builder against the definition of a Voronoi cell.

TerrainModel2DBulider::build (src/models/surface/builder.rs:202-281) gives every site
the area of its Voronoi cell clipped to the bounding box (shoelace over the cell's
vertices, builder.rs:236-247), and relaxate_sites (builder.rs:155-200) moves every site
to the centroid of that clipped cell, `times` rounds.  The checker here builds each
cell by definition -- the box cut by the half-planes "closer to site i than to site j"
for i's Delaunay neighbours j (scipy's triangulation, not the builder's) -- and compares
area and centroid per cell, to 1e-9 relative.  It shares no code with the builder's
circumcentre polygons."""
import numpy as np
import pytest

from fastlem_gb300 import Site2D, TerrainModel2DBulider
from tests.test_interp import area, clip


def _cells(xs, ys, box):
    sp = pytest.importorskip("scipy.spatial")
    tri = sp.Delaunay(np.c_[xs, ys])
    ptr_, nbr = tri.vertex_neighbor_vertices
    x0, y0, x1, y1 = box
    out = []
    for i in range(len(xs)):
        poly = [(x0, y0), (x1, y0), (x1, y1), (x0, y1)]
        for j in nbr[ptr_[i]:ptr_[i + 1]]:
            mx, my = (xs[i] + xs[j]) / 2, (ys[i] + ys[j]) / 2
            poly = clip(poly, mx, my, xs[j] - xs[i], ys[j] - ys[i])
            if not poly:
                break
        out.append(poly)
    return out


def _centroid(poly):
    s = sx = sy = 0.0
    for k in range(len(poly)):
        ax, ay = poly[k]
        bx, by = poly[(k + 1) % len(poly)]
        c = ax * by - bx * ay
        s += c
        sx += (ax + bx) * c
        sy += (ay + by) * c
    return sx / (3 * s), sy / (3 * s)


@pytest.mark.parametrize("n,seed,w,h", [(400, 1, 100.0, 60.0), (1500, 2, 40.0, 40.0)])
def test_clipped_cell_areas_per_site(fl_lib, n, seed, w, h):
    b = TerrainModel2DBulider.from_random_sites(n, Site2D(0.0, 0.0), Site2D(w, h), seed=seed)
    m = b.build()
    cells = _cells(m.xs, m.ys, (0.0, 0.0, w, h))
    want = np.array([area(c) if len(c) >= 3 else 0.0 for c in cells])
    got = m.areas()
    rel = np.abs(got - want) / np.maximum(want, 1e-300)
    assert rel.max() < 1e-9, f"worst cell {int(rel.argmax())}: {got[rel.argmax()]} vs {want[rel.argmax()]}"


@pytest.mark.parametrize("times", [1, 2])
def test_lloyd_moves_each_site_to_its_cell_centroid(fl_lib, times):
    w, h = 80.0, 50.0
    b = TerrainModel2DBulider.from_random_sites(600, Site2D(0.0, 0.0), Site2D(w, h), seed=7)
    xs, ys = b.xs.copy(), b.ys.copy()
    for _ in range(times):                       # the definition, round by round
        cells = _cells(xs, ys, (0.0, 0.0, w, h))
        c = np.array([_centroid(p) for p in cells])
        xs, ys = c[:, 0], c[:, 1]
    r = b.relaxate_sites(times)
    scale = max(w, h)
    assert np.abs(r.xs - xs).max() < 1e-9 * scale
    assert np.abs(r.ys - ys).max() < 1e-9 * scale
