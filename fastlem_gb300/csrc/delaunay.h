// delaunay.h -- the host builder's triangulation and exact predicates, for the other
// host-side translation units (builder.cpp defines them).
#pragma once
#include <cstdint>
#include <vector>

namespace fl {

// Delaunay triangulation of (xs, ys): counter-clockwise triangles (3 vertex ids each)
// and, per half-edge (3 t + k runs from tri[3 t + k] to the next vertex of triangle
// t), the opposite half-edge or -1 on the convex hull.  False for fewer than three
// sites or all sites collinear.
bool delaunay(uint32_t n, const double* xs, const double* ys, std::vector<uint32_t>& tri,
              std::vector<int64_t>& half);

// Exact signs: > 0 when (a, b, c) turn counter-clockwise; > 0 when d lies inside the
// circle through the counter-clockwise a, b, c.
double orient2d(double ax, double ay, double bx, double by, double cx, double cy);
double incircle2d(double ax, double ay, double bx, double by, double cx, double cy, double dx,
                  double dy);

}  // namespace fl
