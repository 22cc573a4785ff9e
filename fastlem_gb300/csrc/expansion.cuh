// expansion.cuh -- exact signs of the orientation and in-circle determinants in
// device code, for the natural-neighbour queries.
//
// Floating-point expansions after Shewchuk (1997), "Adaptive Precision Floating-Point
// Arithmetic and Fast Robust Geometric Predicates": a number is kept as an unevaluated
// sum of doubles in increasing magnitude with no rounding error (Two-Sum,
// Two-Product, Grow-Expansion and Scale-Expansion, zero components dropped).  Each
// routine writes into a caller-provided buffer whose size bounds are stated beside it.
// The sequence of operations is the host builder's (builder.cpp) step for step, so
// both sides take the same decisions; only the sign of the sum is used.  Needs IEEE
// double arithmetic without contraction (-fmad=false) in round-to-nearest.
#pragma once
#include <cuda_runtime.h>

#include <cmath>

// Compiled for the device and, for the host-side probe of the same query code, the host.
#ifndef FL_HD
#define FL_HD __host__ __device__
#endif

namespace fl {
namespace xp {

// Shewchuk's filter bounds: |det| above these times the magnitude sum fixes the sign.
constexpr double kEps = 1.1102230246251565e-16;               // 2^-53
constexpr double kOrientBound = (3.0 + 16.0 * kEps) * kEps;
constexpr double kIncircleBound = (10.0 + 96.0 * kEps) * kEps;

FL_HD __forceinline__ void two_sum(double a, double b, double& x, double& y) {
    x = a + b;
    const double bv = x - a;
    const double av = x - bv;
    y = (a - av) + (b - bv);
}
FL_HD __forceinline__ void two_diff(double a, double b, double& x, double& y) {
    x = a - b;
    const double bv = a - x;
    const double av = x + bv;
    y = (a - av) + (bv - b);
}
FL_HD __forceinline__ void two_prod(double a, double b, double& x, double& y) {
    x = a * b;
#ifdef __CUDA_ARCH__
    y = __fma_rn(a, b, -x);
#else
    y = std::fma(a, b, -x);
#endif
}

// h <- h + b in place; h holds nh components and has room for nh + 1.
FL_HD inline int grow(double* h, int nh, double b) {
    double q = b;
    int k = 0;
    for (int i = 0; i < nh; ++i) {
        double qn, hh;
        two_sum(q, h[i], qn, hh);
        q = qn;
        if (hh != 0.0) h[k++] = hh;                // k <= i: never overwrites unread input
    }
    if (q != 0.0 || k == 0) h[k++] = q;
    return k;
}

// h <- e * b; h (not e) has room for 2 ne components.
FL_HD inline int scale(const double* e, int ne, double b, double* h) {
    int k = 0;
    double q, hh;
    two_prod(e[0], b, q, hh);
    if (hh != 0.0) h[k++] = hh;
    for (int i = 1; i < ne; ++i) {
        double t1, t0, s1, s0;
        two_prod(e[i], b, t1, t0);
        two_sum(q, t0, s1, s0);
        if (s0 != 0.0) h[k++] = s0;
        q = t1 + s1;                               // fast two-sum: |t1| >= |s1|
        const double z = s1 - (q - t1);
        if (z != 0.0) h[k++] = z;
    }
    if (q != 0.0 || k == 0) h[k++] = q;
    return k;
}

// h <- e * f as the sum over f's components of e scaled by each; h has room for
// 2 ne nf + 1 components, t for 2 ne.
FL_HD inline int mul(const double* e, int ne, const double* f, int nf, double* h, double* t) {
    int nh = 1;
    h[0] = 0.0;
    for (int j = 0; j < nf; ++j) {
        const int nt = scale(e, ne, f[j], t);
        for (int k = 0; k < nt; ++k) nh = grow(h, nh, t[k]);
    }
    return nh;
}

// e <- e - f (each of f's components negated and grown in); e has room for ne + nf.
FL_HD inline int sub_into(double* e, int ne, const double* f, int nf) {
    for (int k = 0; k < nf; ++k) ne = grow(e, ne, -f[k]);
    return ne;
}
FL_HD inline int add_into(double* e, int ne, const double* f, int nf) {
    for (int k = 0; k < nf; ++k) ne = grow(e, ne, f[k]);
    return ne;
}

FL_HD __forceinline__ double sign_of(const double* e, int ne) {
    for (int i = ne; i-- > 0;)
        if (e[i] != 0.0) return e[i];
    return 0.0;
}

// a - b exactly: {roundoff, difference}, or {difference} when the difference is exact.
FL_HD __forceinline__ int diff2(double a, double b, double* h) {
    double x, y;
    two_diff(a, b, x, y);
    if (y != 0.0) {
        h[0] = y;
        h[1] = x;
        return 2;
    }
    h[0] = x;
    return 1;
}

// Scratch of the exact stages, in doubles.
constexpr int kSmall = 24;                          // products of two differences: <= 18
constexpr int kProduct = 656;                       // products of two smalls: <= 2*18*18+1
constexpr int kAccum = 1952;                        // three such products: <= 1947
constexpr int kScratch = kAccum + kProduct + 40 + 6 * kSmall + 16;

// Sign of (a - c) x (b - c): > 0 counter-clockwise.  xs: kScratch doubles.
FL_HD inline double orient_exact(double ax, double ay, double bx, double by, double cx,
                                      double cy, double* xs) {
    double* d = xs;                                 // 4 differences, 2 each
    double* p = xs + 8;                             // kSmall
    double* q = p + kSmall;                         // kSmall
    double* t = q + kSmall;                         // 40
    const int n0 = diff2(ax, cx, d), n1 = diff2(by, cy, d + 2), n2 = diff2(ay, cy, d + 4),
              n3 = diff2(bx, cx, d + 6);
    int np = mul(d, n0, d + 2, n1, p, t);
    const int nq = mul(d + 4, n2, d + 6, n3, q, t);
    np = sub_into(p, np, q, nq);
    return sign_of(p, np);
}

// Sign of the in-circle determinant: > 0 when d is inside the circle through the
// counter-clockwise a, b, c.  xs: kScratch doubles.
FL_HD inline double incircle_exact(double ax, double ay, double bx, double by, double cx,
                                        double cy, double dx, double dy, double* xs) {
    double* acc = xs;                               // kAccum
    double* prod = acc + kAccum;                    // kProduct
    double* t = prod + kProduct;                    // 40 (scale temporaries, <= 36)
    double* s = t + 40;                             // 6 x kSmall
    double* df = s + 6 * kSmall;                    // 6 differences, 2 each
    double* adx = df;
    double* ady = df + 2;
    double* bdx = df + 4;
    double* bdy = df + 6;
    double* cdx = df + 8;
    double* cdy = df + 10;
    const int nadx = diff2(ax, dx, adx), nady = diff2(ay, dy, ady), nbdx = diff2(bx, dx, bdx),
              nbdy = diff2(by, dy, bdy), ncdx = diff2(cx, dx, cdx), ncdy = diff2(cy, dy, cdy);
    double* bc = s;
    double* ca = s + kSmall;
    double* ab = s + 2 * kSmall;
    double* al = s + 3 * kSmall;
    double* bl = s + 4 * kSmall;
    double* cl = s + 5 * kSmall;
    // each small term: one product of differences (<= 9), another grown in (<= 18); the
    // second product goes through prod, which is free until the large products
    int nbc = mul(bdx, nbdx, cdy, ncdy, bc, t);
    int nt = mul(cdx, ncdx, bdy, nbdy, prod, t);
    nbc = sub_into(bc, nbc, prod, nt);
    int nca = mul(cdx, ncdx, ady, nady, ca, t);
    nt = mul(adx, nadx, cdy, ncdy, prod, t);
    nca = sub_into(ca, nca, prod, nt);
    int nab = mul(adx, nadx, bdy, nbdy, ab, t);
    nt = mul(bdx, nbdx, ady, nady, prod, t);
    nab = sub_into(ab, nab, prod, nt);
    int nal = mul(adx, nadx, adx, nadx, al, t);
    nt = mul(ady, nady, ady, nady, prod, t);
    nal = add_into(al, nal, prod, nt);
    int nbl = mul(bdx, nbdx, bdx, nbdx, bl, t);
    nt = mul(bdy, nbdy, bdy, nbdy, prod, t);
    nbl = add_into(bl, nbl, prod, nt);
    int ncl = mul(cdx, ncdx, cdx, ncdx, cl, t);
    nt = mul(cdy, ncdy, cdy, ncdy, prod, t);
    ncl = add_into(cl, ncl, prod, nt);
    // al bc + bl ca + cl ab, summed left to right
    int nacc = mul(al, nal, bc, nbc, acc, t);
    nt = mul(bl, nbl, ca, nca, prod, t);
    nacc = add_into(acc, nacc, prod, nt);
    nt = mul(cl, ncl, ab, nab, prod, t);
    nacc = add_into(acc, nacc, prod, nt);
    return sign_of(acc, nacc);
}

}  // namespace xp
}  // namespace fl
