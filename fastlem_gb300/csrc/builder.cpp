// builder.cpp -- host-side terrain model construction (no GPU code).
//
// The GB300 solve consumes a graph that the host builds once per model, as
// fastlem's `TerrainModel2DBulider` does (src/models/surface/builder.rs:31-322):
//   * sites: `from_random_sites` draws x then y per site with `gen_range` from
//     StdRng::from_seed([0; 32]) (builder.rs:38-52); the synthetic workloads use the
//     same sampler seeded with StdRng::seed_from_u64(seed).
//   * Delaunay triangulation of the sites (builder.rs:213-228 via voronoice).  This
//     file implements its own sweep-hull triangulation (points added in order of
//     distance from a seed circumcircle, Lawson edge flips) with exact
//     orientation / in-circle predicates (floating filter + expansion arithmetic).
//   * Voronoi cells clipped to the bounding box; area by the shoelace formula
//     (builder.rs:236-247) and centroid for Lloyd relaxation (builder.rs:155-200).
//   * the undirected edge list: for every triangle (a, b, c), edges a-b, b-c, c-a are
//     added only when the first index is the smaller (builder.rs:254-266), with
//     length sqrt(dx^2 + dy^2) (sites.rs:28-30); adjacency rows keep insertion
//     order, so the CSR row of site i is `graph.neighbors_of(i)`.
//   * default outlets: the convex hull (builder.rs:270).
// Triangles are counter-clockwise (y up).  The triangle order is this builder's own,
// so adjacency order can differ from fastlem's for the same sites; the solve is
// defined on whatever CSR it is given.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <system_error>
#include <thread>
#include <vector>

#include "delaunay.h"
#include "fastlem_gb300.h"
#include "rng.h"

namespace fl {
namespace {

// ---------------------------------------------------------------------------
// Exact arithmetic on non-overlapping expansions (Shewchuk 1997): sums and
// products of doubles kept as unevaluated sums of doubles with no rounding error.
// Requires IEEE double evaluation without contraction or reassociation.
// ---------------------------------------------------------------------------
inline void two_sum(double a, double b, double& x, double& y) {
    x = a + b;
    double bv = x - a;
    double av = x - bv;
    y = (a - av) + (b - bv);
}
inline void two_diff(double a, double b, double& x, double& y) {
    x = a - b;
    double bv = a - x;
    double av = x + bv;
    y = (a - av) + (bv - b);
}
inline void two_prod(double a, double b, double& x, double& y) {
    x = a * b;
    y = std::fma(a, b, -x);
}

using Exp = std::vector<double>;

Exp grow(const Exp& e, double b) {
    Exp h;
    h.reserve(e.size() + 1);
    double q = b;
    for (double ei : e) {
        double qn, hh;
        two_sum(q, ei, qn, hh);
        q = qn;
        if (hh != 0.0) h.push_back(hh);
    }
    if (q != 0.0 || h.empty()) h.push_back(q);
    return h;
}
Exp add(const Exp& e, const Exp& f) {
    Exp h = e;
    for (double fi : f) h = grow(h, fi);
    return h;
}
Exp neg(Exp e) {
    for (double& v : e) v = -v;
    return e;
}
Exp scale(const Exp& e, double b) {
    Exp h;
    h.reserve(2 * e.size());
    double q, hh;
    two_prod(e[0], b, q, hh);
    if (hh != 0.0) h.push_back(hh);
    for (size_t i = 1; i < e.size(); ++i) {
        double t1, t0, s1, s0;
        two_prod(e[i], b, t1, t0);
        two_sum(q, t0, s1, s0);
        if (s0 != 0.0) h.push_back(s0);
        q = t1 + s1;                  // fast two-sum: |t1| >= |s1|
        double z = s1 - (q - t1);
        if (z != 0.0) h.push_back(z);
    }
    if (q != 0.0 || h.empty()) h.push_back(q);
    return h;
}
Exp mul(const Exp& e, const Exp& f) {
    Exp h{0.0};
    for (double fi : f) h = add(h, scale(e, fi));
    return h;
}
inline double sign_of(const Exp& e) {
    for (size_t i = e.size(); i-- > 0;)
        if (e[i] != 0.0) return e[i];
    return 0.0;
}
inline Exp diff2(double a, double b) {
    double x, y;
    two_diff(a, b, x, y);
    return y != 0.0 ? Exp{y, x} : Exp{x};
}

const double kEps = 1.1102230246251565e-16;               // 2^-53
const double kOrientBound = (3.0 + 16.0 * kEps) * kEps;
const double kIncircleBound = (10.0 + 96.0 * kEps) * kEps;

// > 0 when (a, b, c) turn counter-clockwise.
double orient(double ax, double ay, double bx, double by, double cx, double cy) {
    double l = (ax - cx) * (by - cy);
    double r = (ay - cy) * (bx - cx);
    double det = l - r;
    double bound = kOrientBound * (std::fabs(l) + std::fabs(r));
    if (std::fabs(det) > bound) return det;
    Exp acx = diff2(ax, cx), bcy = diff2(by, cy), acy = diff2(ay, cy), bcx = diff2(bx, cx);
    return sign_of(add(mul(acx, bcy), neg(mul(acy, bcx))));
}

// > 0 when d lies inside the circle through the counter-clockwise a, b, c.
double incircle(double ax, double ay, double bx, double by, double cx, double cy, double dx,
                double dy) {
    double adx = ax - dx, ady = ay - dy, bdx = bx - dx, bdy = by - dy, cdx = cx - dx,
           cdy = cy - dy;
    double bc = bdx * cdy - cdx * bdy, ca = cdx * ady - adx * cdy, ab = adx * bdy - bdx * ady;
    double al = adx * adx + ady * ady, bl = bdx * bdx + bdy * bdy, cl = cdx * cdx + cdy * cdy;
    double det = al * bc + bl * ca + cl * ab;
    double perm = (std::fabs(bdx * cdy) + std::fabs(cdx * bdy)) * al +
                  (std::fabs(cdx * ady) + std::fabs(adx * cdy)) * bl +
                  (std::fabs(adx * bdy) + std::fabs(bdx * ady)) * cl;
    if (std::fabs(det) > kIncircleBound * perm) return det;
    Exp eadx = diff2(ax, dx), eady = diff2(ay, dy), ebdx = diff2(bx, dx), ebdy = diff2(by, dy),
        ecdx = diff2(cx, dx), ecdy = diff2(cy, dy);
    Exp ebc = add(mul(ebdx, ecdy), neg(mul(ecdx, ebdy)));
    Exp eca = add(mul(ecdx, eady), neg(mul(eadx, ecdy)));
    Exp eab = add(mul(eadx, ebdy), neg(mul(ebdx, eady)));
    Exp eal = add(mul(eadx, eadx), mul(eady, eady));
    Exp ebl = add(mul(ebdx, ebdx), mul(ebdy, ebdy));
    Exp ecl = add(mul(ecdx, ecdx), mul(ecdy, ecdy));
    return sign_of(add(add(mul(eal, ebc), mul(ebl, eca)), mul(ecl, eab)));
}

inline uint32_t nxt3(uint32_t e) { return (e % 3 == 2) ? e - 2 : e + 1; }
inline uint32_t prv3(uint32_t e) { return (e % 3 == 0) ? e + 2 : e - 1; }

struct SweepHull {
    const double* X;
    const double* Y;
    uint32_t n;
    std::vector<uint32_t> tri;     // 3 vertices per triangle, counter-clockwise
    std::vector<int64_t> half;     // opposite half-edge, -1 on the hull
    std::vector<uint32_t> hnext, hprev, htri;
    std::vector<uint8_t> on_hull;
    std::vector<int64_t> hash;
    double ccx = 0, ccy = 0;
    uint32_t hsize = 1;
    std::vector<uint32_t> stack;
    uint32_t hull_start = 0;

    uint32_t hkey(double x, double y) const {
        double dx = x - ccx, dy = y - ccy;
        double den = std::fabs(dx) + std::fabs(dy);
        double p = den > 0 ? dx / den : 0.0;
        double a = (dy > 0 ? 3.0 - p : 1.0 + p) / 4.0;   // monotone in the angle, [0, 1)
        int64_t k = (int64_t)std::floor(a * hsize);
        k %= (int64_t)hsize;
        if (k < 0) k += hsize;
        return (uint32_t)k;
    }
    void link(int64_t a, int64_t b) {
        half[a] = b;
        if (b >= 0) half[b] = a;
    }
    uint32_t add_tri(uint32_t a, uint32_t b, uint32_t c, int64_t ha, int64_t hb, int64_t hc) {
        uint32_t t = (uint32_t)tri.size();
        tri.push_back(a); tri.push_back(b); tri.push_back(c);
        half.push_back(-1); half.push_back(-1); half.push_back(-1);
        link(t, ha); link(t + 1, hb); link(t + 2, hc);
        return t;
    }
    // Lawson flips starting from half-edge a (the edge opposite the new point).
    void legalize(uint32_t a0) {
        stack.clear();
        stack.push_back(a0);
        while (!stack.empty()) {
            uint32_t a = stack.back();
            stack.pop_back();
            int64_t hb = half[a];
            if (hb < 0) continue;
            uint32_t b = (uint32_t)hb;
            uint32_t al = nxt3(a), ar = prv3(a);
            uint32_t br = nxt3(b), bl = prv3(b);
            uint32_t p0 = tri[ar], pr = tri[a], pl = tri[al], p1 = tri[bl];
            if (incircle(X[pr], Y[pr], X[pl], Y[pl], X[p0], Y[p0], X[p1], Y[p1]) <= 0.0) continue;
            // (pr, pl, p0) + (pl, pr, p1)  ->  (p1, pl, p0) + (p0, pr, p1)
            tri[a] = p1;
            tri[b] = p0;
            int64_t hbl = half[bl], har = half[ar];
            if (hbl < 0) htri[p1] = a;
            if (har < 0) htri[p0] = b;
            link(a, hbl);
            link(b, har);
            link(ar, bl);
            stack.push_back(br);
            stack.push_back(a);
        }
    }

    bool run() {
        if (n < 3) return false;
        double minx = INFINITY, miny = INFINITY, maxx = -INFINITY, maxy = -INFINITY;
        for (uint32_t i = 0; i < n; ++i) {
            minx = std::min(minx, X[i]); maxx = std::max(maxx, X[i]);
            miny = std::min(miny, Y[i]); maxy = std::max(maxy, Y[i]);
        }
        double cx = (minx + maxx) / 2, cy = (miny + maxy) / 2;
        auto d2 = [&](uint32_t i, double x, double y) {
            double dx = X[i] - x, dy = Y[i] - y;
            return dx * dx + dy * dy;
        };
        uint32_t i0 = 0, i1 = UINT32_MAX, i2 = UINT32_MAX;
        double best = INFINITY;
        for (uint32_t i = 0; i < n; ++i) {
            double d = d2(i, cx, cy);
            if (d < best) { best = d; i0 = i; }
        }
        best = INFINITY;
        for (uint32_t i = 0; i < n; ++i) {
            if (i == i0) continue;
            double d = d2(i, X[i0], Y[i0]);
            if (d < best && d > 0) { best = d; i1 = i; }
        }
        if (i1 == UINT32_MAX) return false;
        auto circumradius2 = [&](uint32_t a, uint32_t b, uint32_t c) {
            double dx = X[b] - X[a], dy = Y[b] - Y[a], ex = X[c] - X[a], ey = Y[c] - Y[a];
            double bl = dx * dx + dy * dy, cl = ex * ex + ey * ey, d = 0.5 / (dx * ey - dy * ex);
            double x = (ey * bl - dy * cl) * d, y = (dx * cl - ex * bl) * d;
            return x * x + y * y;
        };
        best = INFINITY;
        for (uint32_t i = 0; i < n; ++i) {
            if (i == i0 || i == i1) continue;
            double r = circumradius2(i0, i1, i);
            if (r < best) { best = r; i2 = i; }
        }
        if (i2 == UINT32_MAX || !std::isfinite(best)) return false;   // all collinear
        if (orient(X[i0], Y[i0], X[i1], Y[i1], X[i2], Y[i2]) < 0) std::swap(i1, i2);
        {
            double ax = X[i0], ay = Y[i0];
            double dx = X[i1] - ax, dy = Y[i1] - ay, ex = X[i2] - ax, ey = Y[i2] - ay;
            double bl = dx * dx + dy * dy, cl = ex * ex + ey * ey, d = 0.5 / (dx * ey - dy * ex);
            ccx = ax + (ey * bl - dy * cl) * d;
            ccy = ay + (dx * cl - ex * bl) * d;
        }
        std::vector<double> dist(n);
        for (uint32_t i = 0; i < n; ++i) dist[i] = d2(i, ccx, ccy);
        std::vector<uint32_t> ids(n);
        std::iota(ids.begin(), ids.end(), 0u);
        std::sort(ids.begin(), ids.end(), [&](uint32_t a, uint32_t b) {
            return dist[a] < dist[b] || (dist[a] == dist[b] && a < b);
        });

        hsize = (uint32_t)std::ceil(std::sqrt((double)n));
        hash.assign(hsize, -1);
        hnext.assign(n, 0); hprev.assign(n, 0); htri.assign(n, 0); on_hull.assign(n, 0);
        tri.reserve(6ull * n); half.reserve(6ull * n);

        add_tri(i0, i1, i2, -1, -1, -1);
        hnext[i0] = i1; hnext[i1] = i2; hnext[i2] = i0;
        hprev[i1] = i0; hprev[i2] = i1; hprev[i0] = i2;
        htri[i0] = 0; htri[i1] = 1; htri[i2] = 2;
        on_hull[i0] = on_hull[i1] = on_hull[i2] = 1;
        hash[hkey(X[i0], Y[i0])] = i0;
        hash[hkey(X[i1], Y[i1])] = i1;
        hash[hkey(X[i2], Y[i2])] = i2;
        hull_start = i0;

        double px_prev = NAN, py_prev = NAN;
        for (uint32_t idx = 0; idx < n; ++idx) {
            uint32_t p = ids[idx];
            double px = X[p], py = Y[p];
            if (px == px_prev && py == py_prev) continue;     // exact duplicate: skipped
            px_prev = px; py_prev = py;
            if (p == i0 || p == i1 || p == i2) continue;
            uint32_t key = hkey(px, py);
            int64_t s = -1;
            for (uint32_t j = 0; j < hsize; ++j) {
                int64_t c = hash[(key + j) % hsize];
                if (c >= 0 && on_hull[c]) { s = c; break; }
            }
            if (s < 0) continue;
            uint32_t start = hprev[(uint32_t)s];
            uint32_t e = start;
            bool found = false;
            while (true) {
                uint32_t q = hnext[e];
                if (orient(X[e], Y[e], X[q], Y[q], px, py) < 0) { found = true; break; }
                e = q;
                if (e == start) break;
            }
            if (!found) continue;          // on the hull boundary: degenerate, skipped

            uint32_t q = hnext[e];
            uint32_t t = add_tri(e, p, q, -1, -1, (int64_t)htri[e]);
            htri[e] = t;          // e -> p
            htri[p] = t + 1;      // p -> q
            on_hull[p] = 1;
            legalize(t + 2);
            // walk forward: edges q -> hnext[q] visible from p
            while (true) {
                uint32_t q2 = hnext[q];
                if (!(orient(X[q], Y[q], X[q2], Y[q2], px, py) < 0)) break;
                uint32_t t2 = add_tri(q, p, q2, (int64_t)htri[p], -1, (int64_t)htri[q]);
                htri[p] = t2 + 1;     // p -> q2
                on_hull[q] = 0;
                legalize(t2 + 2);
                q = q2;
            }
            // walk backward: edges hprev[e] -> e visible from p
            while (true) {
                uint32_t e0 = hprev[e];
                if (!(orient(X[e0], Y[e0], X[e], Y[e], px, py) < 0)) break;
                uint32_t t2 = add_tri(e0, p, e, -1, (int64_t)htri[e], (int64_t)htri[e0]);
                htri[e0] = t2;        // e0 -> p
                on_hull[e] = 0;
                legalize(t2 + 2);
                e = e0;
            }
            hprev[p] = e; hnext[p] = q;
            hnext[e] = p; hprev[q] = p;
            hash[hkey(px, py)] = p;
            hash[hkey(X[e], Y[e])] = e;
            hull_start = e;
        }
        return true;
    }

    std::vector<uint32_t> hull() const {
        // start at the smallest hull index, counter-clockwise
        uint32_t s = hull_start, m = hull_start;
        uint32_t v = s;
        do { m = std::min(m, v); v = hnext[v]; } while (v != s);
        std::vector<uint32_t> h;
        v = m;
        do { h.push_back(v); v = hnext[v]; } while (v != m);
        return h;
    }
};

inline void circumcenter(double ax, double ay, double bx, double by, double cx, double cy,
                         double& ox, double& oy) {
    double dx = bx - ax, dy = by - ay, ex = cx - ax, ey = cy - ay;
    double bl = dx * dx + dy * dy, cl = ex * ex + ey * ey, d = 0.5 / (dx * ey - dy * ex);
    ox = ax + (ey * bl - dy * cl) * d;
    oy = ay + (dx * cl - ex * bl) * d;
}

// Sutherland-Hodgman clip of polygon (xs, ys) to one half-plane.
template <class Inside, class Cross>
void clip_edge(std::vector<double>& xs, std::vector<double>& ys, Inside inside, Cross cross) {
    std::vector<double> ox, oy;
    size_t m = xs.size();
    for (size_t i = 0; i < m; ++i) {
        size_t j = (i + 1) % m;
        bool ii = inside(xs[i], ys[i]), ij = inside(xs[j], ys[j]);
        if (ii) { ox.push_back(xs[i]); oy.push_back(ys[i]); }
        if (ii != ij) {
            double x, y;
            cross(xs[i], ys[i], xs[j], ys[j], x, y);
            ox.push_back(x); oy.push_back(y);
        }
    }
    xs.swap(ox);
    ys.swap(oy);
}

void clip_box(std::vector<double>& xs, std::vector<double>& ys, double x0, double y0, double x1,
              double y1) {
    auto cx = [](double v) {
        return [v](double ax, double ay, double bx, double by, double& x, double& y) {
            double t = (v - ax) / (bx - ax);
            x = v;
            y = ay + t * (by - ay);
        };
    };
    auto cy = [](double v) {
        return [v](double ax, double ay, double bx, double by, double& x, double& y) {
            double t = (v - ay) / (by - ay);
            y = v;
            x = ax + t * (bx - ax);
        };
    };
    clip_edge(xs, ys, [&](double x, double) { return x >= x0; }, cx(x0));
    if (xs.empty()) return;
    clip_edge(xs, ys, [&](double x, double) { return x <= x1; }, cx(x1));
    if (xs.empty()) return;
    clip_edge(xs, ys, [&](double, double y) { return y >= y0; }, cy(y0));
    if (xs.empty()) return;
    clip_edge(xs, ys, [&](double, double y) { return y <= y1; }, cy(y1));
}

// Voronoi cell of every site clipped to the box: area (shoelace, builder.rs:236-247)
// and centroid.  Cells of hull sites are closed with far points along the outward
// normals of their two hull edges before clipping.  Sites [v0, v1) only.
void voronoi_cells_range(const SweepHull& d, const std::vector<double>& ccx,
                         const std::vector<double>& ccy, const std::vector<int64_t>& start,
                         const std::vector<uint8_t>& hullv, double x0, double y0, double x1,
                         double y1, uint32_t v0, uint32_t v1, double* area, double* cenx,
                         double* ceny) {
    const double* X = d.X;
    const double* Y = d.Y;
    double diag = std::hypot(x1 - x0, y1 - y0);
    double bcx = (x0 + x1) / 2, bcy = (y0 + y1) / 2;
    std::vector<double> xs, ys, px, py;
    xs.reserve(64); ys.reserve(64); px.reserve(64); py.reserve(64);
    for (uint32_t v = v0; v < v1; ++v) {
        area[v] = 0.0;
        cenx[v] = X[v];
        ceny[v] = Y[v];
        if (start[v] < 0) continue;   // duplicate site, not triangulated
        xs.clear();
        ys.clear();
        uint32_t e = (uint32_t)start[v];
        uint32_t first = e, last = e;
        bool inside = true;
        do {
            uint32_t t = e / 3;
            double cx = ccx[t], cy = ccy[t];
            inside = inside && cx >= x0 && cx <= x1 && cy >= y0 && cy <= y1;
            xs.push_back(cx);
            ys.push_back(cy);
            last = e;
            int64_t tw = d.half[prv3(e)];
            if (tw < 0) break;
            e = (uint32_t)tw;
        } while (e != first);
        if (hullv[v]) {
            // first hull edge v -> hnext[v] (half-edge `first`), last edge hprev[v] -> v
            uint32_t w1 = d.tri[nxt3(first)];
            uint32_t w0 = d.tri[prv3(last)];
            double n1x = Y[w1] - Y[v], n1y = -(X[w1] - X[v]);
            double n2x = Y[v] - Y[w0], n2y = -(X[v] - X[w0]);
            double l1 = std::hypot(n1x, n1y), l2 = std::hypot(n2x, n2y);
            n1x /= l1; n1y /= l1; n2x /= l2; n2y /= l2;
            auto far = [&](double ox, double oy) {
                return 4.0 * (diag + std::hypot(ox - bcx, oy - bcy)) + 1.0;
            };
            double r1 = far(xs.front(), ys.front()), r2 = far(xs.back(), ys.back());
            double mx = n1x + n2x, my = n1y + n2y, ml = std::hypot(mx, my);
            px.assign(1, xs.front() + r1 * n1x);
            py.assign(1, ys.front() + r1 * n1y);
            px.insert(px.end(), xs.begin(), xs.end());
            py.insert(py.end(), ys.begin(), ys.end());
            px.push_back(xs.back() + r2 * n2x);
            py.push_back(ys.back() + r2 * n2y);
            if (ml > 1e-12) {
                double r3 = 2.0 * std::max(r1, r2);
                double ox = 0.5 * (xs.front() + xs.back()), oy = 0.5 * (ys.front() + ys.back());
                px.push_back(ox + r3 * mx / ml);
                py.push_back(oy + r3 * my / ml);
            }
            xs.swap(px);
            ys.swap(py);
            inside = false;
        }
        if (!inside) clip_box(xs, ys, x0, y0, x1, y1);
        size_t m = xs.size();
        if (m < 3) continue;
        double s = 0.0, sx = 0.0, sy = 0.0;
        for (size_t i = 0; i < m; ++i) {
            size_t j = (i + 1) % m;
            double c = xs[i] * ys[j] - xs[j] * ys[i];
            s += c;
            sx += (xs[i] + xs[j]) * c;
            sy += (ys[i] + ys[j]) * c;
        }
        area[v] = std::fabs(s) / 2.0;
        if (s != 0.0) {
            cenx[v] = sx / (3.0 * s);
            ceny[v] = sy / (3.0 * s);
        }
    }
}

void voronoi_cells(const SweepHull& d, double x0, double y0, double x1, double y1, double* area,
                   double* cenx, double* ceny) {
    const uint32_t n = d.n;
    uint64_t ntri = d.tri.size() / 3;
    std::vector<double> ccx(ntri), ccy(ntri);
    for (uint64_t t = 0; t < ntri; ++t) {
        uint32_t a = d.tri[3 * t], b = d.tri[3 * t + 1], c = d.tri[3 * t + 2];
        circumcenter(d.X[a], d.Y[a], d.X[b], d.Y[b], d.X[c], d.Y[c], ccx[t], ccy[t]);
    }
    std::vector<int64_t> start(n, -1);
    for (uint64_t e = 0; e < d.tri.size(); ++e) start[d.tri[e]] = (int64_t)e;
    std::vector<uint8_t> hullv(n, 0);
    for (uint32_t v : d.hull()) { hullv[v] = 1; start[v] = d.htri[v]; }
    unsigned nt = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    if (n < 100000) nt = 1;
    std::vector<std::thread> th;
    uint32_t chunk = (n + nt - 1) / nt;
    for (unsigned t = 0; t < nt; ++t) {
        uint32_t a = std::min<uint64_t>((uint64_t)t * chunk, n);
        uint32_t b = std::min<uint64_t>((uint64_t)a + chunk, n);
        auto cells = [&, a, b] {
            voronoi_cells_range(d, ccx, ccy, start, hullv, x0, y0, x1, y1, a, b, area, cenx, ceny);
        };
        try {
            th.emplace_back(cells);
        } catch (const std::system_error&) {   // no thread to spare: run it here
            cells();
        }
    }
    for (auto& t : th) t.join();
}

}  // namespace

bool delaunay(uint32_t n, const double* xs, const double* ys, std::vector<uint32_t>& tri,
              std::vector<int64_t>& half) {
    SweepHull d{xs, ys, n};
    if (!d.run()) return false;
    tri = std::move(d.tri);
    half = std::move(d.half);
    return true;
}

double orient2d(double ax, double ay, double bx, double by, double cx, double cy) {
    return orient(ax, ay, bx, by, cx, cy);
}

double incircle2d(double ax, double ay, double bx, double by, double cx, double cy, double dx,
                  double dy) {
    return incircle(ax, ay, bx, by, cx, cy, dx, dy);
}

}  // namespace fl

// ---------------------------------------------------------------------------
// C ABI (declared in include/fastlem_gb300.h)
// ---------------------------------------------------------------------------
extern "C" {

// Uniform sites in [x0,x1) x [y0,y1): per site x = gen_range(x0..x1) then
// y = gen_range(y0..y1) from StdRng::seed_from_u64(seed), or from
// StdRng::from_seed([0; 32]) when zero_seed != 0 (fastlem's from_random_sites).
int fl_random_sites(uint64_t n, double x0, double y0, double x1, double y1, uint64_t seed,
                    int zero_seed, double* xs, double* ys) {
    if (!(x0 < x1) || !(y0 < y1) || (n && (!xs || !ys))) return FL_ERR_INVALID_ARGUMENT;
    fl::StdRng rng = zero_seed ? fl::StdRng::zero_key() : fl::StdRng::seed_from_u64(seed);
    for (uint64_t i = 0; i < n; ++i) {
        xs[i] = rng.gen_range(x0, x1);
        ys[i] = rng.gen_range(y0, y1);
    }
    return FL_OK;
}

// Lloyd relaxation (builder.rs:155-200): `times` rounds of moving every site to the
// centroid of its Voronoi cell clipped to the box.  In place.  FL_OK, or
// FL_ERR_BUILDER_VORONOI when the triangulation fails (ModelBuilderError::VoronoiError).
int fl_relax_sites(uint32_t n, double* xs, double* ys, double x0, double y0, double x1, double y1,
                   uint32_t times) {
    if (times && (!xs || !ys)) return FL_ERR_INVALID_ARGUMENT;
    std::vector<double> area(n), cx(n), cy(n);
    for (uint32_t r = 0; r < times; ++r) {
        fl::SweepHull d{xs, ys, n};
        if (!d.run()) return FL_ERR_BUILDER_VORONOI;
        fl::voronoi_cells(d, x0, y0, x1, y1, area.data(), cx.data(), cy.data());
        std::memcpy(xs, cx.data(), n * sizeof(double));
        std::memcpy(ys, cy.data(), n * sizeof(double));
    }
    return 0;
}

// build() (builder.rs:202-281): triangulate, clip Voronoi cells to the box, build the
// CSR adjacency with the a<b edge rule in triangle order, and the hull outlets.
// row_ptr has n + 1 entries, col / len hold `cap` slots (6n always suffices for a
// planar graph), area n entries, hull n entries.  Returns FL_OK,
// FL_ERR_BUILDER_VORONOI when the sites cannot be triangulated
// (ModelBuilderError::VoronoiError), FL_ERR_INVALID_ARGUMENT when cap is too small.
int fl_build_graph(uint32_t n, const double* xs, const double* ys, double x0, double y0,
                   double x1, double y1, uint32_t* row_ptr, uint32_t* col, double* len,
                   uint64_t cap, double* area, uint32_t* hull, uint64_t* out_nnz,
                   uint32_t* out_nhull) {
    if (!xs || !ys || !row_ptr || !col || !len || !area || !hull || !out_nnz || !out_nhull)
        return FL_ERR_INVALID_ARGUMENT;
    fl::SweepHull d{xs, ys, n};
    if (!d.run()) return FL_ERR_BUILDER_VORONOI;
    std::vector<uint32_t> h = d.hull();
    uint64_t ntri = d.tri.size() / 3;
    std::vector<uint32_t> deg(n, 0);
    auto each_edge = [&](auto&& f) {
        for (uint64_t t = 0; t < ntri; ++t) {
            uint32_t a = d.tri[3 * t], b = d.tri[3 * t + 1], c = d.tri[3 * t + 2];
            if (a < b) f(a, b);
            if (b < c) f(b, c);
            if (c < a) f(c, a);
        }
    };
    each_edge([&](uint32_t a, uint32_t b) { ++deg[a]; ++deg[b]; });
    uint64_t nnz = 0;
    for (uint32_t i = 0; i < n; ++i) nnz += deg[i];
    *out_nnz = nnz;
    *out_nhull = (uint32_t)h.size();
    if (nnz > cap || nnz >= 0xffffffffull) return FL_ERR_INVALID_ARGUMENT;
    row_ptr[0] = 0;
    for (uint32_t i = 0; i < n; ++i) row_ptr[i + 1] = row_ptr[i] + deg[i];
    std::vector<uint32_t> fill(row_ptr, row_ptr + n);
    each_edge([&](uint32_t a, uint32_t b) {
        double dx = xs[a] - xs[b], dy = ys[a] - ys[b];
        double l = std::sqrt(dx * dx + dy * dy);
        col[fill[a]] = b; len[fill[a]++] = l;
        col[fill[b]] = a; len[fill[b]++] = l;
    });
    std::vector<double> cx(n), cy(n);
    fl::voronoi_cells(d, x0, y0, x1, y1, area, cx.data(), cy.data());
    std::copy(h.begin(), h.end(), hull);
    return 0;
}

// Raw triangulation (tests): counter-clockwise triangles; returns the triangle
// count, or -1 on failure.  `tri` holds up to `cap` triangles.
int64_t fl_triangulate(uint32_t n, const double* xs, const double* ys, uint32_t* tri,
                       uint64_t cap) {
    if (!xs || !ys) return -1;
    fl::SweepHull d{xs, ys, n};
    if (!d.run()) return -1;
    uint64_t ntri = d.tri.size() / 3;
    if (tri && ntri <= cap) std::memcpy(tri, d.tri.data(), d.tri.size() * sizeof(uint32_t));
    return (int64_t)ntri;
}

}  // extern "C"
