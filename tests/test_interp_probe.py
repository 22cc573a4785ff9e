"""The GPU natural-neighbour query code, compiled for the host (fl_probe_interp_query),
against the host queries (fl_interpolate) on CPU: the first pass gives the host's bits
wherever it does not defer, the second pass everywhere, including the degenerate site
sets the first pass defers (lattices, queries at sites, on edges and on hull edges)."""
import numpy as np
import pytest

from fastlem_gb300._lib import ptr
from fastlem_gb300.api import TerrainInterpolator2D

OUTSIDE, FOUND, DEFER, TOO_LARGE = 0, 1, 2, 3


def probe(fl_lib, it, f, qx, qy, exact):
    out = np.empty(len(qx))
    st = np.empty(len(qx), np.int32)
    assert fl_lib.fl_probe_interp_query(it._h, ptr(f), len(qx), ptr(qx), ptr(qy), exact, ptr(out),
                                        ptr(st)) == 0
    return out, st


def check_passes(fl_lib, it, f, qx, qy):
    host, ok = it.interpolate_many(f, qx, qy)
    fast, st = probe(fl_lib, it, f, qx, qy, 0)
    done = st != DEFER
    assert np.array_equal(st[done] == FOUND, ok[done])
    assert np.array_equal(fast[done].view(np.uint64), host[done].view(np.uint64))
    exact, st2 = probe(fl_lib, it, f, qx, qy, 1)
    assert np.array_equal(st2 == FOUND, ok)
    assert np.array_equal(exact.view(np.uint64), host.view(np.uint64))
    return st


def test_random_sites_first_pass_settles_almost_all(fl_lib):
    r = np.random.default_rng(21)
    xs, ys = r.uniform(0, 100, 5000), r.uniform(0, 100, 5000)
    it = TerrainInterpolator2D(xs, ys)
    f = r.normal(0, 1, len(xs))
    qx, qy = r.uniform(-3, 103, 20_000), r.uniform(-3, 103, 20_000)
    st = check_passes(fl_lib, it, f, qx, qy)
    assert (st == DEFER).mean() < 1e-3


def test_lattice_defers_to_the_exact_pass(fl_lib):
    g = np.arange(0.0, 40.0, 2.0)
    X, Y = np.meshgrid(g, g)
    it = TerrainInterpolator2D(X.ravel(), Y.ravel())
    f = np.random.default_rng(3).normal(0, 1, X.size)
    h = np.arange(-1.0, 40.0, 1.0)                  # sites, edges, diagonals: all degenerate
    QX, QY = np.meshgrid(h, h)
    r = np.random.default_rng(4)
    qx = np.concatenate([QX.ravel(), r.uniform(-1, 40, 2000)])
    qy = np.concatenate([QY.ravel(), r.uniform(-1, 40, 2000)])
    st = check_passes(fl_lib, it, f, qx, qy)
    assert (st[:QX.size] != FOUND).all() and (st[:QX.size] == DEFER).any()
    assert (st[QX.size:] == FOUND).mean() > 0.8


def test_cocircular_sites_and_large_cavities(fl_lib):
    t = np.linspace(0, 2 * np.pi, 300, endpoint=False)
    it = TerrainInterpolator2D(100 * np.cos(t), 100 * np.sin(t))
    f = np.random.default_rng(5).normal(0, 1, len(t))
    qx, qy = np.array([0.5, -30.0, 99.0]), np.array([0.25, 10.0, 1.0])
    st = check_passes(fl_lib, it, f, qx, qy)
    assert (st == DEFER).all()                      # cavities of 298 triangles
    t = np.linspace(0, 2 * np.pi, 2100, endpoint=False)
    it = TerrainInterpolator2D(100 * np.cos(t), 100 * np.sin(t))
    _, st = probe(fl_lib, it, np.zeros(len(t)), np.array([0.5]), np.array([0.25]), 1)
    assert st[0] == TOO_LARGE


def near_degenerate_cases(rng, m, scale, jitter):
    """a, b, c on a circle of radius ~scale around a centre; q on the circle, on the
    chord a-b or at a random point, each moved by ~jitter (relative)."""
    centre = rng.uniform(-scale, scale, (m, 2)) * rng.choice([0.0, 1.0, 1e3], (m, 1))
    r = scale * rng.uniform(0.5, 2.0, (m, 1))
    ang = rng.uniform(0, 2 * np.pi, (m, 4))
    pts = centre[:, None, :] + r[:, :, None] * np.stack([np.cos(ang), np.sin(ang)], -1)
    kind = rng.integers(0, 3, m)
    t = rng.uniform(-0.5, 1.5, m)
    chord = pts[:, 0] + t[:, None] * (pts[:, 1] - pts[:, 0])
    pts[kind == 1, 3] = chord[kind == 1]
    pts[kind == 2, 3] = centre[kind == 2] + r[kind == 2] * rng.normal(0, 1, ((kind == 2).sum(), 2))
    pts *= 1.0 + jitter * rng.normal(0, 1, pts.shape)
    # counter-clockwise a, b, c as the in-circle predicate expects
    cross = ((pts[:, 1, 0] - pts[:, 0, 0]) * (pts[:, 2, 1] - pts[:, 0, 1]) -
             (pts[:, 1, 1] - pts[:, 0, 1]) * (pts[:, 2, 0] - pts[:, 0, 0]))
    swap = cross < 0
    pts[swap, 1], pts[swap, 2] = pts[swap, 2].copy(), pts[swap, 1].copy()
    return np.ascontiguousarray(pts.reshape(m, 8))


@pytest.mark.parametrize("scale", [1e-30, 1e-3, 1.0, 4000.0, 1e7, 1e9])
def test_float_prefilters_never_contradict_the_exact_sign(fl_lib, scale):
    """Cases with q on or near a circumcircle or an edge line, at magnitudes from tiny to
    beyond the prefilter's range: a decided prefilter sign equals the exact sign."""
    rng = np.random.default_rng(int(abs(np.log10(scale))) + 1)
    decided = 0
    for jitter in (0.0, 1e-16, 1e-12, 1e-8, 1e-5, 1e-2):
        cases = near_degenerate_cases(rng, 4000, scale, jitter)
        out = np.empty((len(cases), 4), np.int32)
        assert fl_lib.fl_probe_prefilters(len(cases), ptr(cases), ptr(out)) == 0
        for f, e in ((0, 2), (1, 3)):
            d = out[:, f] != 0
            assert np.array_equal(out[d, f], out[d, e]), (jitter, f)
            decided += d.sum()
    if 1e-3 <= scale <= 4000.0:        # far below, the float products underflow: undecided
        assert decided > 0
