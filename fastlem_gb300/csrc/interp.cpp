// interp.cpp -- Terrain2D::get_elevation (src/models/surface/terrain.rs:35-38 through
// src/models/surface/interpolator.rs:17-29): natural-neighbour interpolation of the
// elevations at a query point, None outside the sites' convex hull.
//
// fastlem delegates to the naturalneighbor crate (1.2.2, not vendored); this restates
// the published method, Sibson's interpolant: inserting the query q into the Voronoi
// diagram of the sites, q's new cell takes a piece of the cell of each of its natural
// neighbours v; the weight of v is the area of that piece over the area of q's cell.
// In Delaunay terms (Bowyer-Watson / Watson's construction):
//   * the triangles whose circumcircle holds q form a star-shaped cavity around q; its
//     boundary vertices are the natural neighbours and its boundary edges (a -> b,
//     counter-clockwise) become the new triangles (a, b, q);
//   * the piece taken from v is the polygon through the circumcentre of the new
//     triangle ending at v, the circumcentres of the cavity triangles around v (the
//     old Voronoi vertices q's cell swallows), and the circumcentre of the new
//     triangle starting at v.
// Points on a hull edge take the linear interpolant along that edge (the limit of the
// weights from inside); a query equal to a site returns that site's value.
// Predicates are exact (the builder's expansion arithmetic); areas are computed
// relative to q.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <system_error>
#include <thread>
#include <vector>

#include "delaunay.h"
#include "fastlem_gb300.h"
#include "interp.h"

namespace fl {
void set_last_error(const char* msg);
}

namespace {

inline uint32_t nxt3(uint32_t e) { return (e % 3 == 2) ? e - 2 : e + 1; }

inline void circumcentre(double ax, double ay, double bx, double by, double cx, double cy,
                         double& ox, double& oy) {
    const double dx = bx - ax, dy = by - ay, ex = cx - ax, ey = cy - ay;
    const double bl = dx * dx + dy * dy, cl = ex * ex + ey * ey;
    const double d = 0.5 / (dx * ey - dy * ex);
    ox = ax + (ey * bl - dy * cl) * d;
    oy = ay + (dx * cl - ex * bl) * d;
}

constexpr uint32_t kOutside = UINT32_MAX;

// Walk from triangle t to the triangle holding (x, y) (inside or on its boundary), or
// kOutside beyond the hull, with *last the triangle the walk stopped in: a visibility
// walk, the edge tests rotating from edge (step mod 3), which terminates on a Delaunay
// triangulation with exact orientation tests.
uint32_t walk(const fl_interpolator& it, uint32_t t, double x, double y, uint32_t* last) {
    const uint64_t limit = 4ull * it.tri.size() + 16;
    for (uint64_t step = 0; step < limit; ++step) {
        bool moved = false;
        for (uint32_t k = 0; k < 3 && !moved; ++k) {
            const uint32_t e = 3 * t + (uint32_t)((k + step) % 3);
            const uint32_t a = it.tri[e], b = it.tri[nxt3(e)];
            if (fl::orient2d(it.X[a], it.Y[a], it.X[b], it.Y[b], x, y) < 0.0) {
                if (it.half[e] < 0) {                      // beyond a hull edge
                    *last = t;
                    return kOutside;
                }
                t = (uint32_t)(it.half[e] / 3);
                moved = true;
            }
        }
        if (!moved) return *last = t;
    }
    *last = t;
    return kOutside;
}

uint32_t locate(const fl_interpolator& it, double x, double y) {
    const uint32_t cx = (uint32_t)std::min<double>(it.gw - 1, std::max(0.0, (x - it.gx0) / it.gsx));
    const uint32_t cy = (uint32_t)std::min<double>(it.gh - 1, std::max(0.0, (y - it.gy0) / it.gsy));
    uint32_t last;
    return walk(it, it.gtri[(uint64_t)cy * it.gw + cx], x, y, &last);
}

// Sibson interpolant at (x, y); false outside the hull.
bool interpolate_one(const fl_interpolator& it, const double* f, double x, double y,
                     double* out) {
    if (!std::isfinite(x) || !std::isfinite(y)) return false;
    const uint32_t t0 = locate(it, x, y);
    if (t0 == kOutside) return false;
    for (uint32_t k = 0; k < 3; ++k) {
        const uint32_t v = it.tri[3 * t0 + k];
        if (it.X[v] == x && it.Y[v] == y) {
            *out = f[v];
            return true;
        }
    }
    // the cavity: triangles whose circumcircle holds q (connected, contains t0)
    std::vector<uint32_t> cav{t0}, seen{t0};
    auto in = [](const std::vector<uint32_t>& s, uint32_t t) {
        return std::find(s.begin(), s.end(), t) != s.end();
    };
    for (size_t i = 0; i < cav.size(); ++i) {
        const uint32_t t = cav[i];
        for (uint32_t k = 0; k < 3; ++k) {
            const int64_t o = it.half[3 * t + k];
            if (o < 0) continue;
            const uint32_t u = (uint32_t)(o / 3);
            if (in(seen, u)) continue;
            seen.push_back(u);
            const uint32_t a = it.tri[3 * u], b = it.tri[3 * u + 1], c = it.tri[3 * u + 2];
            if (fl::incircle2d(it.X[a], it.Y[a], it.X[b], it.Y[b], it.X[c], it.Y[c], x, y) > 0.0)
                cav.push_back(u);
        }
    }
    // boundary edges a -> b (counter-clockwise around q)
    std::vector<uint32_t> bnd;
    for (uint32_t t : cav)
        for (uint32_t k = 0; k < 3; ++k) {
            const uint32_t e = 3 * t + k;
            const int64_t o = it.half[e];
            if (o >= 0 && in(cav, (uint32_t)(o / 3))) continue;
            const uint32_t a = it.tri[e], b = it.tri[nxt3(e)];
            if (o < 0 && fl::orient2d(it.X[a], it.Y[a], it.X[b], it.Y[b], x, y) == 0.0) {
                // on a hull edge: linear along it
                const double dx = it.X[b] - it.X[a], dy = it.Y[b] - it.Y[a];
                const double s = ((x - it.X[a]) * dx + (y - it.Y[a]) * dy) / (dx * dx + dy * dy);
                *out = f[a] + s * (f[b] - f[a]);
                return true;
            }
            bnd.push_back(e);
        }
    // new circumcentres, relative to q
    const size_t m = bnd.size();
    std::vector<double> nx(m), ny(m);
    for (size_t i = 0; i < m; ++i) {
        const uint32_t a = it.tri[bnd[i]], b = it.tri[nxt3(bnd[i])];
        circumcentre(it.X[a] - x, it.Y[a] - y, it.X[b] - x, it.Y[b] - y, 0.0, 0.0, nx[i], ny[i]);
    }
    double num = 0.0, den = 0.0;
    std::vector<double> px, py;
    for (size_t o = 0; o < m; ++o) {                 // o: the edge leaving v
        const uint32_t eo = bnd[o];
        const uint32_t v = it.tri[eo];
        size_t i = m;                                // the edge arriving at v
        for (size_t j = 0; j < m; ++j)
            if (it.tri[nxt3(bnd[j])] == v) { i = j; break; }
        if (i == m) return false;
        px.assign(1, nx[i]);
        py.assign(1, ny[i]);
        // cavity triangles around v, from the arriving edge's to the leaving edge's
        uint32_t h = nxt3(bnd[i]);
        for (size_t guard = 0;; ++guard) {
            const uint32_t t = h / 3;
            px.push_back(it.ccx[t] - x);
            py.push_back(it.ccy[t] - y);
            if (h == eo) break;
            const int64_t tw = it.half[h];
            if (tw < 0 || guard > cav.size() || !in(cav, (uint32_t)(tw / 3))) return false;
            h = nxt3((uint32_t)tw);
        }
        px.push_back(nx[o]);
        py.push_back(ny[o]);
        double area2 = 0.0;                          // shoelace, closed polygon
        for (size_t k = 0; k < px.size(); ++k) {
            const size_t l = (k + 1) % px.size();
            area2 += px[k] * py[l] - px[l] * py[k];
        }
        const double w = std::fabs(area2);
        num += w * f[v];
        den += w;
    }
    if (!(den > 0.0)) return false;
    *out = num / den;
    return true;
}

}  // namespace

extern "C" {

int fl_interpolator_create(uint32_t n, const double* xs, const double* ys, fl_interpolator** out) {
    if (!out || !xs || !ys) {
        fl::set_last_error("fl_interpolator_create: null argument");
        return FL_ERR_INVALID_ARGUMENT;
    }
    *out = nullptr;
    auto* it = new fl_interpolator;
    it->n = n;
    it->X.assign(xs, xs + n);
    it->Y.assign(ys, ys + n);
    for (uint32_t i = 0; i < n; ++i)
        if (!std::isfinite(xs[i]) || !std::isfinite(ys[i])) {
            delete it;
            fl::set_last_error("fl_interpolator_create: non-finite site");
            return FL_ERR_INVALID_ARGUMENT;
        }
    if (!fl::delaunay(n, it->X.data(), it->Y.data(), it->tri, it->half)) {
        delete it;
        fl::set_last_error("fl_interpolator_create: fewer than three sites, or all collinear");
        return FL_ERR_INVALID_ARGUMENT;
    }
    const size_t nt = it->tri.size() / 3;
    it->ccx.resize(nt);
    it->ccy.resize(nt);
    for (size_t t = 0; t < nt; ++t) {
        const uint32_t a = it->tri[3 * t], b = it->tri[3 * t + 1], c = it->tri[3 * t + 2];
        circumcentre(it->X[a], it->Y[a], it->X[b], it->Y[b], it->X[c], it->Y[c], it->ccx[t],
                     it->ccy[t]);
    }
    it->vedge.assign(n, -1);
    for (size_t e = 0; e < it->tri.size(); ++e) it->vedge[it->tri[e]] = (int64_t)e;
    // grid over the triangulated sites' bounding box, about four sites per cell
    double x0 = INFINITY, y0 = INFINITY, x1 = -INFINITY, y1 = -INFINITY;
    std::vector<uint32_t> used;
    for (uint32_t v = 0; v < n; ++v)
        if (it->vedge[v] >= 0) {
            used.push_back(v);
            x0 = std::min(x0, it->X[v]); x1 = std::max(x1, it->X[v]);
            y0 = std::min(y0, it->Y[v]); y1 = std::max(y1, it->Y[v]);
        }
    const uint32_t g = (uint32_t)std::max(1.0, std::floor(std::sqrt(used.size() / 4.0)));
    it->gw = it->gh = g;
    it->gx0 = x0;
    it->gy0 = y0;
    it->gsx = (x1 > x0 ? (x1 - x0) : 1.0) / g;
    it->gsy = (y1 > y0 ? (y1 - y0) : 1.0) / g;
    std::vector<uint32_t> gsite((uint64_t)g * g, UINT32_MAX);
    for (uint32_t v : used) {
        const uint32_t cx = (uint32_t)std::min<double>(g - 1, (it->X[v] - x0) / it->gsx);
        const uint32_t cy = (uint32_t)std::min<double>(g - 1, (it->Y[v] - y0) / it->gsy);
        gsite[(uint64_t)cy * g + cx] = v;
    }
    // empty cells take the site of a nearest filled cell (breadth-first over the grid from
    // every filled cell at once, in cell order)
    std::vector<uint32_t> queue;
    queue.reserve(gsite.size());
    for (uint32_t c = 0; c < gsite.size(); ++c)
        if (gsite[c] != UINT32_MAX) queue.push_back(c);
    for (size_t h = 0; h < queue.size(); ++h) {
        const uint32_t c = queue[h], cx = c % g, cy = c / g;
        const uint32_t nb[4] = {cx > 0 ? c - 1 : UINT32_MAX, cx + 1 < g ? c + 1 : UINT32_MAX,
                                cy > 0 ? c - g : UINT32_MAX, cy + 1 < g ? c + g : UINT32_MAX};
        for (uint32_t d : nb)
            if (d != UINT32_MAX && gsite[d] == UINT32_MAX) {
                gsite[d] = gsite[c];
                queue.push_back(d);
            }
    }
    // each cell's start: walk from a triangle of its site to the cell's centre
    it->gtri.resize(gsite.size());
    auto starts = [&](uint64_t a, uint64_t b) {
        for (uint64_t c = a; c < b; ++c) {
            const double x = x0 + ((double)(c % g) + 0.5) * it->gsx;
            const double y = y0 + ((double)(c / g) + 0.5) * it->gsy;
            walk(*it, (uint32_t)(it->vedge[gsite[c]] / 3), x, y, &it->gtri[c]);
        }
    };
    const uint64_t cells = gsite.size();
    const unsigned workers =
        cells < 65536 ? 1u : std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    std::vector<std::thread> th;
    const uint64_t chunk = (cells + workers - 1) / workers;
    for (unsigned w = 1; w < workers; ++w) {
        const uint64_t a = std::min<uint64_t>(w * chunk, cells), b = std::min<uint64_t>(a + chunk, cells);
        try {
            th.emplace_back(starts, a, b);
        } catch (const std::system_error&) {
            starts(a, b);
        }
    }
    starts(0, std::min<uint64_t>(chunk, cells));
    for (auto& t : th) t.join();
    *out = it;
    return FL_OK;
}

void fl_interpolator_destroy(fl_interpolator* it) {
    if (!it) return;
    fl::interp_device_release(it->dev);
    delete it;
}

int fl_interpolate(const fl_interpolator* it, const double* values, uint64_t count,
                   const double* qx, const double* qy, double* out, uint8_t* found) {
    if (!it || (count && (!values || !qx || !qy || !out || !found))) {
        fl::set_last_error("fl_interpolate: null argument");
        return FL_ERR_INVALID_ARGUMENT;
    }
    // large batches run in grid-cell order (a counting sort of the queries), so that
    // neighbouring queries walk the same triangles; every query is independent
    std::vector<uint64_t> order;
    if (count >= 4096) {
        const uint64_t cells = (uint64_t)it->gw * it->gh;
        std::vector<uint64_t> cell(count), start(cells + 1, 0);
        for (uint64_t i = 0; i < count; ++i) {
            const double fx = (qx[i] - it->gx0) / it->gsx, fy = (qy[i] - it->gy0) / it->gsy;
            const uint64_t cx = fx > 0 ? (uint64_t)std::min<double>(it->gw - 1, fx) : 0;
            const uint64_t cy = fy > 0 ? (uint64_t)std::min<double>(it->gh - 1, fy) : 0;
            cell[i] = cy * it->gw + cx;
            ++start[cell[i] + 1];
        }
        for (uint64_t c = 0; c < cells; ++c) start[c + 1] += start[c];
        order.resize(count);
        for (uint64_t i = 0; i < count; ++i) order[start[cell[i]]++] = i;
    }
    auto run = [&](uint64_t a, uint64_t b) {
        for (uint64_t k = a; k < b; ++k) {
            const uint64_t i = order.empty() ? k : order[k];
            double v = NAN;
            found[i] = interpolate_one(*it, values, qx[i], qy[i], &v) ? 1 : 0;
            out[i] = found[i] ? v : NAN;
        }
    };
    unsigned nt = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    if (count < 4096) nt = 1;
    std::vector<std::thread> th;
    const uint64_t chunk = (count + nt - 1) / nt;
    for (unsigned t = 0; t < nt; ++t) {
        const uint64_t a = std::min<uint64_t>(t * chunk, count), b = std::min<uint64_t>(a + chunk, count);
        if (a >= b) continue;
        try {
            th.emplace_back(run, a, b);
        } catch (const std::system_error&) {   // no thread to spare: run it here
            run(a, b);
        }
    }
    for (auto& t : th) t.join();
    return FL_OK;
}

}  // extern "C"
