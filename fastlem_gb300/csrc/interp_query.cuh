// interp_query.cuh -- one natural-neighbour query over the interpolator's
// triangulation, for the device kernels of interp_gpu.cu and for their host-side probe
// (the same code compiled for the host, so the CPU tests can run it): interp.cpp's
// construction with the same IEEE double operations in the same order.
#pragma once
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "expansion.cuh"

namespace fl {
namespace iq {

constexpr uint64_t kFastWalk = 256;        // pass 1: walk steps per query

enum QueryStatus { kQOutside = 0, kQFound = 1, kQDefer = 2, kQTooLarge = 3 };
// Device status words: the round's deferred count, the too-large flag, and (words 2-3, a
// u64) the deferred queries of the whole call.
enum StatusWord { kDeferred = 0, kTooLarge = 1, kDeferredTotal = 2, kStatusWords = 4 };

struct View {
    const double2* __restrict__ xy;
    const uint32_t* __restrict__ tri;
    const int32_t* __restrict__ half;
    const double2* __restrict__ cc;
    const uint32_t* __restrict__ gtri;
    double gx0, gy0, gsx, gsy;
    uint32_t gw, gh;
    uint64_t walk_limit;                   // the host walk's limit: 4 x half-edges + 16
    const float2* __restrict__ xyf;        // the vertices rounded to float
    float smax;                            // largest |coordinate| of a vertex
};

// Single-precision prefilters of the orientation and in-circle signs (the first pass
// only): a sign they return is the exact sign of the double-precision predicate on the
// original coordinates; 0 means undecided and the double-precision filter follows.
//
// Inputs: the vertices and q rounded to float (relative error u = 2^-24 each, or an
// absolute 2^-150 below the normal range) and their differences in float.  With S the
// largest |coordinate| involved, each float difference is within
//   delta = 2^-21 S + 2^-140
// of the exact difference of the doubles (|fl(a) - A| + |fl(q) - Q| <= 2uS, the float
// subtraction adds at most u(|fl(a)| + |fl(q)|) <= 2uS(1 + u): 4uS + 2u^2 S <= 2^-21 S).
// A determinant is a sum of monomials of these differences; with every difference off
// by at most delta, the exact determinant of the float differences is off from the
// exact one of the true differences by at most P(|d| + delta) - P(|d|), P the
// determinant's permanent (each monomial with absolute values).  Evaluating the
// determinant in float adds Shewchuk's bound (3 + 16u)u or (10 + 96u)u times the
// permanent.  Both bounds are evaluated in float, scaled up by (1 + 2^-10) to cover
// their own rounding, plus 2^-126 for underflow.  Requires S <= 2^29 (no overflow in
// the degree-4 permanents); otherwise the caller skips the prefilter.
struct QueryF {
    float x, y, delta;
    bool ok;                               // the prefilter applies
};

FL_HD __forceinline__ QueryF query_f(const View& V, double x, double y) {
    QueryF q;
    q.x = (float)x;
    q.y = (float)y;
    const float s = fmaxf(V.smax, fmaxf(fabsf(q.x), fabsf(q.y))) * (1.0f + 1.0f / 1024.0f);
    q.ok = s <= 536870912.0f;                              // 2^29
    q.delta = s * (1.0f / 2097152.0f) + 7.174648e-43f;     // 2^-21 S + 2^-140
    return q;
}

constexpr float kU32 = 5.9604645e-08f;                     // 2^-24
constexpr float kBoundSlack = 1.0f + 1.0f / 1024.0f;
constexpr float kTiny = 1.1754944e-38f;                    // 2^-126

// +1 / -1: the sign of orient2d(a, b, q); 0: undecided.
FL_HD __forceinline__ int orient_f(float2 a, float2 b, const QueryF& q) {
    const float d1x = a.x - q.x, d1y = a.y - q.y, d2x = b.x - q.x, d2y = b.y - q.y;
    const float p1 = d1x * d2y, p2 = d1y * d2x;
    const float det = p1 - p2;
    const float dl = q.delta;
    const float ax = fabsf(d1x), ay = fabsf(d1y), bx = fabsf(d2x), by = fabsf(d2y);
    const float round = (3.0f + 16.0f * kU32) * kU32 * (fabsf(p1) + fabsf(p2));
    const float input = dl * (ax + by + ay + bx + 2.0f * dl);
    const float err = (round + input) * kBoundSlack + kTiny;
    return det > err ? 1 : (det < -err ? -1 : 0);
}

// Permanent of the in-circle determinant at non-negative differences.
FL_HD __forceinline__ float incircle_perm(float ax, float ay, float bx, float by, float cx, float cy) {
    return (ax * ax + ay * ay) * (bx * cy + cx * by) + (bx * bx + by * by) * (cx * ay + ax * cy) +
           (cx * cx + cy * cy) * (ax * by + bx * ay);
}

// +1 / -1: the sign of incircle2d(a, b, c, q); 0: undecided.
FL_HD __forceinline__ int incircle_f(float2 a, float2 b, float2 c, const QueryF& q) {
    const float adx = a.x - q.x, ady = a.y - q.y, bdx = b.x - q.x, bdy = b.y - q.y, cdx = c.x - q.x,
                cdy = c.y - q.y;
    const float bc = bdx * cdy - cdx * bdy, ca = cdx * ady - adx * cdy, ab = adx * bdy - bdx * ady;
    const float al = adx * adx + ady * ady, bl = bdx * bdx + bdy * bdy, cl = cdx * cdx + cdy * cdy;
    const float det = al * bc + bl * ca + cl * ab;
    const float dl = q.delta;
    const float ax = fabsf(adx), ay = fabsf(ady), bx = fabsf(bdx), by = fabsf(bdy), cx = fabsf(cdx),
                cy = fabsf(cdy);
    // each permanent is evaluated in float with all terms non-negative, so within a
    // factor (1 + u)^7 < 1 + 8u of its exact value; the difference needs
    // p1 (1 + 8u) - p0 (1 - 8u), and with 12u instead of 8u its own three roundings
    // cannot take the float result below that
    const float p0 = incircle_perm(ax, ay, bx, by, cx, cy);
    const float p1 = incircle_perm(ax + dl, ay + dl, bx + dl, by + dl, cx + dl, cy + dl);
    const float round = (10.0f + 96.0f * kU32) * kU32 * p0;
    const float input = p1 * (1.0f + 12.0f * kU32) - p0 * (1.0f - 12.0f * kU32);
    const float err = (round + input) * kBoundSlack + kTiny;
    return det > err ? 1 : (det < -err ? -1 : 0);
}


FL_HD __forceinline__ uint32_t nxt3(uint32_t e) { return (e % 3 == 2) ? e - 2 : e + 1; }

// interp.cpp's circumcentre, operation for operation.
FL_HD __forceinline__ double2 circumcentre(double ax, double ay, double bx, double by,
                                                double cx, double cy) {
    const double dx = bx - ax, dy = by - ay, ex = cx - ax, ey = cy - ay;
    const double bl = dx * dx + dy * dy, cl = ex * ex + ey * ey;
    const double d = 0.5 / (dx * ey - dy * ex);
    return make_double2(ax + (ey * bl - dy * cl) * d, ay + (dx * cl - ex * bl) * d);
}

// Circumcentre, relative to q, of the new triangle (a, b, q) on boundary edge e.
FL_HD __forceinline__ double2 new_centre(const View& V, uint32_t e, double x, double y) {
    const double2 a = V.xy[V.tri[e]], b = V.xy[V.tri[nxt3(e)]];
    return circumcentre(a.x - x, a.y - y, b.x - x, b.y - y, 0.0, 0.0);
}

// Sign of orient2d (a, b, q): the filter, then (kExact) the expansions; without them an
// inconclusive filter sets `defer`.
template <bool kExact>
FL_HD __forceinline__ double orient(double2 a, double2 b, double x, double y, double* xs,
                                         bool& defer) {
    const double l = (a.x - x) * (b.y - y);
    const double r = (a.y - y) * (b.x - x);
    const double det = l - r;
    if (fabs(det) > xp::kOrientBound * (fabs(l) + fabs(r))) return det;
    if (!kExact) {
        defer = true;
        return 0.0;
    }
    return xp::orient_exact(a.x, a.y, b.x, b.y, x, y, xs);
}

template <bool kExact>
FL_HD __forceinline__ double incircle(double2 a, double2 b, double2 c, double x, double y,
                                           double* xs, bool& defer) {
    const double adx = a.x - x, ady = a.y - y, bdx = b.x - x, bdy = b.y - y, cdx = c.x - x,
                 cdy = c.y - y;
    const double bc = bdx * cdy - cdx * bdy, ca = cdx * ady - adx * cdy, ab = adx * bdy - bdx * ady;
    const double al = adx * adx + ady * ady, bl = bdx * bdx + bdy * bdy, cl = cdx * cdx + cdy * cdy;
    const double det = al * bc + bl * ca + cl * ab;
    const double perm = (fabs(bdx * cdy) + fabs(cdx * bdy)) * al +
                        (fabs(cdx * ady) + fabs(adx * cdy)) * bl +
                        (fabs(adx * bdy) + fabs(bdx * ady)) * cl;
    if (fabs(det) > xp::kIncircleBound * perm) return det;
    if (!kExact) {
        defer = true;
        return 0.0;
    }
    return xp::incircle_exact(a.x, a.y, b.x, b.y, c.x, c.y, x, y, xs);
}

FL_HD __forceinline__ bool holds(const uint32_t* s, uint32_t n, uint32_t t) {
    for (uint32_t i = 0; i < n; ++i)
        if (s[i] == t) return true;
    return false;
}

// Grid cell coordinate of q, clamped as interp.cpp's locate clamps it.
FL_HD __forceinline__ uint32_t cell_coord(double q, double q0, double step, uint32_t cells) {
    double f = (q - q0) / step;
    f = (0.0 < f) ? f : 0.0;
    const double hi = (double)(cells - 1);
    f = (f < hi) ? f : hi;
    return (uint32_t)f;
}

// One query: the status and, when found, the value.  cav holds cap triangles, bnd
// cap + 2 edges; xs is the exact stages' scratch (kExact only).
template <bool kExact>
FL_HD int query(const View& V, const double* __restrict__ f, double x, double y,
                     uint32_t* cav, uint32_t* bnd, uint32_t cap, double* xs, double& out) {
    if (!isfinite(x) || !isfinite(y)) return kQOutside;
    bool defer = false;
    const uint32_t cx = cell_coord(x, V.gx0, V.gsx, V.gw);
    const uint32_t cy = cell_coord(y, V.gy0, V.gsy, V.gh);
    uint32_t t = V.gtri[(uint64_t)cy * V.gw + cx];
    const uint64_t limit = kExact ? V.walk_limit : kFastWalk;
    uint64_t step = 0;
    uint32_t rot = 0;                                     // step mod 3
    for (; step < limit; ++step) {
        bool moved = false;
        for (uint32_t k = 0; k < 3 && !moved; ++k) {
            const uint32_t e = 3 * t + (k + rot) % 3;
            const double s = orient<kExact>(V.xy[V.tri[e]], V.xy[V.tri[nxt3(e)]], x, y, xs, defer);
            if (defer) return kQDefer;
            if (s < 0.0) {
                const int32_t o = V.half[e];
                if (o < 0) return kQOutside;              // beyond a hull edge
                t = (uint32_t)o / 3;
                moved = true;
            }
        }
        if (!moved) break;
        rot = rot == 2 ? 0 : rot + 1;
    }
    if (step == limit) return kExact ? kQOutside : kQDefer;
    for (uint32_t k = 0; k < 3; ++k) {
        const uint32_t v = V.tri[3 * t + k];
        const double2 p = V.xy[v];
        if (p.x == x && p.y == y) {
            out = f[v];
            return kQFound;
        }
    }
    // the cavity
    uint32_t nc = 1;
    cav[0] = t;
    for (uint32_t i = 0; i < nc; ++i) {
        const uint32_t ti = cav[i];
        for (uint32_t k = 0; k < 3; ++k) {
            const int32_t o = V.half[3 * ti + k];
            if (o < 0) continue;
            const uint32_t u = (uint32_t)o / 3;
            if (holds(cav, nc, u)) continue;
            const double s = incircle<kExact>(V.xy[V.tri[3 * u]], V.xy[V.tri[3 * u + 1]],
                                              V.xy[V.tri[3 * u + 2]], x, y, xs, defer);
            if (defer) return kQDefer;
            if (s > 0.0) {
                if (nc == cap) return kExact ? kQTooLarge : kQDefer;
                cav[nc++] = u;
            }
        }
    }
    // boundary edges a -> b, counter-clockwise around q
    uint32_t nb = 0;
    for (uint32_t i = 0; i < nc; ++i)
        for (uint32_t k = 0; k < 3; ++k) {
            const uint32_t e = 3 * cav[i] + k;
            const int32_t o = V.half[e];
            if (o >= 0 && holds(cav, nc, (uint32_t)o / 3)) continue;
            const uint32_t a = V.tri[e], b = V.tri[nxt3(e)];
            if (o < 0) {
                const double2 pa = V.xy[a], pb = V.xy[b];
                const double s = orient<kExact>(pa, pb, x, y, xs, defer);
                if (defer) return kQDefer;
                if (s == 0.0) {                           // on a hull edge: linear along it
                    const double dx = pb.x - pa.x, dy = pb.y - pa.y;
                    const double w = ((x - pa.x) * dx + (y - pa.y) * dy) / (dx * dx + dy * dy);
                    out = f[a] + w * (f[b] - f[a]);
                    return kQFound;
                }
            }
            if (nb == cap + 2) return kExact ? kQTooLarge : kQDefer;
            bnd[nb++] = e;
        }
    double num = 0.0, den = 0.0;
    for (uint32_t o = 0; o < nb; ++o) {                   // o: the edge leaving v
        const uint32_t eo = bnd[o];
        const uint32_t v = V.tri[eo];
        uint32_t i = nb;                                  // the edge arriving at v
        for (uint32_t j = 0; j < nb; ++j)
            if (V.tri[nxt3(bnd[j])] == v) {
                i = j;
                break;
            }
        if (i == nb) return kQOutside;
        const double2 first = new_centre(V, bnd[i], x, y);
        double2 prev = first;
        double area2 = 0.0;                               // shoelace, closed polygon
        uint32_t h = nxt3(bnd[i]);
        for (uint32_t guard = 0;; ++guard) {
            const double2 c = V.cc[h / 3];
            const double2 p = make_double2(c.x - x, c.y - y);
            area2 += prev.x * p.y - p.x * prev.y;
            prev = p;
            if (h == eo) break;
            const int32_t tw = V.half[h];
            if (tw < 0 || guard > nc || !holds(cav, nc, (uint32_t)tw / 3)) return kQOutside;
            h = nxt3((uint32_t)tw);
        }
        const double2 last = new_centre(V, eo, x, y);
        area2 += prev.x * last.y - last.x * prev.y;
        area2 += last.x * first.y - first.x * last.y;
        const double w = fabs(area2);
        num += w * f[v];
        den += w;
    }
    if (!(den > 0.0)) return kQOutside;
    out = num / den;
    return kQFound;
}


constexpr uint32_t kFastCap = 32;          // pass 1: cavity triangles per query

// Warp-wide vote and reconvergence on the device; on the host (the probe) a "warp" is
// one thread.
FL_HD __forceinline__ bool warp_any(bool p) {
#ifdef __CUDA_ARCH__
    return __any_sync(0xffffffffu, p);
#else
    return p;
#endif
}
FL_HD __forceinline__ void warp_sync() {
#ifdef __CUDA_ARCH__
    __syncwarp();
#endif
}

constexpr int kQRun = -1;                  // still being answered

// The first pass's query: query<false>'s construction (filters only; anything the
// filters or the small tables cannot settle is deferred), run by all 32 threads of a
// warp together (`active` false for a thread without a query).  Every loop is
// warp-synchronous: its trip count is a warp vote, each iteration does at most one
// predicate or one polygon point per thread, and the threads meet before the
// double-precision work, so that they issue it together (the FP64 pipe is charged
// for the whole warp whatever the active threads).  Per thread the arithmetic is
// query<false>'s, operation for operation.  cav: kFastCap triangles; bnd and centre:
// kFastCap + 2 boundary edges and their new circumcentres.
FL_HD int query_fast(const View& V, const double* __restrict__ f, bool active, double x, double y,
                     uint32_t* cav, uint32_t* bnd, double2* centre, double& out) {
    int st = (active && isfinite(x) && isfinite(y)) ? kQRun : kQOutside;
    bool defer = false;
    uint32_t t = 0;
    if (st == kQRun)
        t = V.gtri[(uint64_t)cell_coord(y, V.gy0, V.gsy, V.gh) * V.gw + cell_coord(x, V.gx0, V.gsx, V.gw)];
    const QueryF qf = query_f(V, x, y);
    // the sign of a predicate: the float prefilter, then the double filter
    auto orient_sign = [&](uint32_t a, uint32_t b) -> double {
        const int s = qf.ok ? orient_f(V.xyf[a], V.xyf[b], qf) : 0;
        return s ? (double)s : orient<false>(V.xy[a], V.xy[b], x, y, nullptr, defer);
    };
    auto incircle_sign = [&](uint32_t a, uint32_t b, uint32_t c) -> double {
        const int s = qf.ok ? incircle_f(V.xyf[a], V.xyf[b], V.xyf[c], qf) : 0;
        return s ? (double)s : incircle<false>(V.xy[a], V.xy[b], V.xy[c], x, y, nullptr, defer);
    };
    // walk: one edge test per iteration
    uint32_t k = 0, rot = 0, steps = 0;
    bool busy = st == kQRun;
    while (warp_any(busy)) {
        if (busy) {
            const uint32_t e = 3 * t + (k + rot) % 3;
            const double s = orient_sign(V.tri[e], V.tri[nxt3(e)]);
            if (defer) {
                st = kQDefer;
                busy = false;
            } else if (s < 0.0) {
                const int32_t o = V.half[e];
                if (o < 0) {                              // beyond a hull edge
                    st = kQOutside;
                    busy = false;
                } else {
                    t = (uint32_t)o / 3;
                    if (++steps == kFastWalk) {
                        st = kQDefer;
                        busy = false;
                    }
                    rot = rot == 2 ? 0 : rot + 1;
                    k = 0;
                }
            } else if (++k == 3) {
                busy = false;
            }
        }
    }
    if (st == kQRun)
        for (uint32_t j = 0; j < 3; ++j) {
            const uint32_t v = V.tri[3 * t + j];
            const double2 p = V.xy[v];
            if (p.x == x && p.y == y) {
                out = f[v];
                st = kQFound;
                break;
            }
        }
    // cavity: one in-circle test per iteration, the scan to the next candidate before it
    uint32_t nc = 1, ci = 0, ck = 0;
    if (st == kQRun) cav[0] = t;
    busy = st == kQRun;
    while (warp_any(busy)) {
        uint32_t u = 0xffffffffu;
        while (busy && ci < nc) {
            const int32_t o = V.half[3 * cav[ci] + ck];
            if (++ck == 3) {
                ck = 0;
                ++ci;
            }
            if (o < 0 || holds(cav, nc, (uint32_t)o / 3)) continue;
            u = (uint32_t)o / 3;
            break;
        }
        if (u == 0xffffffffu) busy = false;
        warp_sync();
        if (busy) {
            const double s = incircle_sign(V.tri[3 * u], V.tri[3 * u + 1], V.tri[3 * u + 2]);
            if (defer) {
                st = kQDefer;
                busy = false;
            } else if (s > 0.0) {
                if (nc == kFastCap) {
                    st = kQDefer;
                    busy = false;
                } else {
                    cav[nc++] = u;
                }
            }
        }
    }
    // boundary edges a -> b, counter-clockwise around q (integer work; orientation only
    // for hull edges)
    uint32_t nb = 0;
    if (st == kQRun)
        for (uint32_t i = 0; i < nc && st == kQRun; ++i)
            for (uint32_t j = 0; j < 3; ++j) {
                const uint32_t e = 3 * cav[i] + j;
                const int32_t o = V.half[e];
                if (o >= 0 && holds(cav, nc, (uint32_t)o / 3)) continue;
                const uint32_t a = V.tri[e], b = V.tri[nxt3(e)];
                if (o < 0) {
                    const double2 pa = V.xy[a], pb = V.xy[b];
                    const double s = orient_sign(a, b);
                    if (defer) {
                        st = kQDefer;
                        break;
                    }
                    if (s == 0.0) {                       // on a hull edge: linear along it
                        const double dx = pb.x - pa.x, dy = pb.y - pa.y;
                        const double w = ((x - pa.x) * dx + (y - pa.y) * dy) / (dx * dx + dy * dy);
                        out = f[a] + w * (f[b] - f[a]);
                        st = kQFound;
                        break;
                    }
                }
                if (nb == kFastCap + 2) {
                    st = kQDefer;
                    break;
                }
                bnd[nb++] = e;
            }
    // the new circumcentres, once each
    const uint32_t ncentres = st == kQRun ? nb : 0;
    for (uint32_t j = 0; warp_any(j < ncentres); ++j)
        if (j < ncentres) centre[j] = new_centre(V, bnd[j], x, y);
    // weights: one polygon point per iteration
    double num = 0.0, den = 0.0, area2 = 0.0;
    double2 first = make_double2(0.0, 0.0), prev = first;
    uint32_t o = 0, eo = 0, v = 0, h = 0, guard = 0;
    bool open = false;
    busy = st == kQRun && nb > 0;
    while (warp_any(busy)) {
        if (busy && !open) {                              // o: the edge leaving v
            eo = bnd[o];
            v = V.tri[eo];
            uint32_t i = nb;                              // the edge arriving at v
            for (uint32_t j = 0; j < nb; ++j)
                if (V.tri[nxt3(bnd[j])] == v) {
                    i = j;
                    break;
                }
            if (i == nb) {
                st = kQOutside;
                busy = false;
            } else {
                first = prev = centre[i];
                area2 = 0.0;
                h = nxt3(bnd[i]);
                guard = 0;
                open = true;
            }
        }
        warp_sync();
        if (busy) {
            const double2 c = V.cc[h / 3];
            const double2 p = make_double2(c.x - x, c.y - y);
            area2 += prev.x * p.y - p.x * prev.y;
            prev = p;
            if (h == eo) {
                const double2 last = centre[o];
                area2 += prev.x * last.y - last.x * prev.y;
                area2 += last.x * first.y - first.x * last.y;
                const double w = fabs(area2);
                num += w * f[v];
                den += w;
                open = false;
                if (++o == nb) busy = false;
            } else {
                const int32_t tw = V.half[h];
                if (tw < 0 || guard > nc || !holds(cav, nc, (uint32_t)tw / 3)) {
                    st = kQOutside;
                    busy = false;
                } else {
                    h = nxt3((uint32_t)tw);
                    ++guard;
                }
            }
        }
    }
    if (st == kQRun) {
        if (!(den > 0.0)) return kQOutside;
        out = num / den;
        return kQFound;
    }
    return st;
}

}  // namespace iq
}  // namespace fl
