// ordering.cpp -- device memory order of a model's sites.
//
// Synthetic and builder-made sites come in random order, so a site's neighbours,
// receiver and donors are scattered over the whole array and every gather misses
// the caches.  The solver therefore stores sites in the order of a Hilbert curve
// through the bounding box of their coordinates: neighbours and river paths land on
// nearby indices.  Relabelling never changes results: every row keeps its slot
// order (the adjacency order the reference's tie-breaks and sums follow), outlet
// lists keep their order, and all inputs / outputs are translated at the boundary.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <system_error>
#include <thread>
#include <vector>

namespace fl {

// Position of grid cell (x, y) along the Hilbert curve filling a 2^order square
// (the classic quadrant-rotation construction).
static uint64_t hilbert_index(uint32_t order, uint32_t x, uint32_t y) {
    uint64_t d = 0;
    for (uint32_t s = 1u << (order - 1); s > 0; s >>= 1) {
        uint32_t rx = (x & s) ? 1u : 0u;
        uint32_t ry = (y & s) ? 1u : 0u;
        d += (uint64_t)s * s * ((3u * rx) ^ ry);
        if (ry == 0) {
            if (rx == 1) {
                x = s - 1 - (x & (s - 1)) + (x & ~(s - 1));
                y = s - 1 - (y & (s - 1)) + (y & ~(s - 1));
            }
            uint32_t t = x;
            x = y;
            y = t;
        }
    }
    return d;
}

// Threads for a host pass over `work` items: all cores for large passes.
static unsigned host_threads(uint64_t work) {
    unsigned t = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    return work < (1u << 18) ? 1u : t;
}

// Runs f(a, b) over [0, n) split into `nt` contiguous ranges on as many threads.
template <class F>
static void parallel_ranges(uint64_t n, unsigned nt, F f) {
    if (nt <= 1) {
        f((uint64_t)0, n);
        return;
    }
    std::vector<std::thread> th;
    const uint64_t chunk = (n + nt - 1) / nt;
    for (unsigned t = 0; t < nt; ++t) {
        const uint64_t a = std::min<uint64_t>((uint64_t)t * chunk, n);
        const uint64_t b = std::min<uint64_t>(a + chunk, n);
        if (a >= b) continue;
        try {
            th.emplace_back(f, a, b);
        } catch (const std::system_error&) {   // no thread to spare: run it here
            f(a, b);
        }
    }
    for (auto& x : th) x.join();
}

// perm[new] = old for the Hilbert order of (xs, ys); ties keep index order.
void hilbert_order(uint32_t n, const double* xs, const double* ys, std::vector<uint32_t>& perm) {
    double x0 = INFINITY, y0 = INFINITY, x1 = -INFINITY, y1 = -INFINITY;
    for (uint32_t i = 0; i < n; ++i) {
        if (std::isfinite(xs[i])) { x0 = std::min(x0, xs[i]); x1 = std::max(x1, xs[i]); }
        if (std::isfinite(ys[i])) { y0 = std::min(y0, ys[i]); y1 = std::max(y1, ys[i]); }
    }
    const uint32_t order = 16;
    const double cells = (double)((1u << order) - 1);
    double sx = (x1 > x0) ? cells / (x1 - x0) : 0.0;
    double sy = (y1 > y0) ? cells / (y1 - y0) : 0.0;
    // (key << 32 | index): an LSD radix sort on the key bytes keeps index order on ties
    std::vector<uint64_t> a(n), b(n);
    parallel_ranges(n, host_threads(n), [&](uint64_t lo, uint64_t hi) {
        for (uint64_t i = lo; i < hi; ++i) {
            double fx = std::isfinite(xs[i]) ? (xs[i] - x0) * sx : 0.0;
            double fy = std::isfinite(ys[i]) ? (ys[i] - y0) * sy : 0.0;
            uint32_t cx = (uint32_t)std::min(cells, std::max(0.0, fx));
            uint32_t cy = (uint32_t)std::min(cells, std::max(0.0, fy));
            const uint64_t key = hilbert_index(order, cx, cy);   // < 2^32 for order 16
            a[i] = (key << 32) | i;
        }
    });
    for (int shift = 32; shift < 64; shift += 8) {
        uint64_t cnt[257] = {0};
        for (uint32_t i = 0; i < n; ++i) ++cnt[((a[i] >> shift) & 255u) + 1];
        for (int k = 0; k < 256; ++k) cnt[k + 1] += cnt[k];
        for (uint32_t i = 0; i < n; ++i) b[cnt[(a[i] >> shift) & 255u]++] = a[i];
        a.swap(b);
    }
    perm.resize(n);
    for (uint32_t i = 0; i < n; ++i) perm[i] = (uint32_t)a[i];
}

// CSR of the relabelled graph: new row j is old row perm[j] with columns mapped
// through inv, slot order unchanged.
void relabel_csr(uint32_t n, const uint32_t* row, const uint32_t* col, const double* len,
                 const std::vector<uint32_t>& perm, const std::vector<uint32_t>& inv,
                 std::vector<uint32_t>& nrow, std::vector<uint32_t>& ncol, std::vector<double>& nlen) {
    nrow.assign(n + 1, 0);
    for (uint32_t j = 0; j < n; ++j) nrow[j + 1] = nrow[j] + (row[perm[j] + 1] - row[perm[j]]);
    ncol.resize(nrow[n]);
    nlen.resize(nrow[n]);
    parallel_ranges(n, host_threads(nrow[n]), [&](uint64_t lo, uint64_t hi) {
        for (uint64_t j = lo; j < hi; ++j) {
            const uint32_t o = perm[j];
            uint32_t d = nrow[j];
            for (uint32_t s = row[o]; s < row[o + 1]; ++s, ++d) {
                ncol[d] = inv[col[s]];
                nlen[d] = len[s];
            }
        }
    });
}

}  // namespace fl
