// interp_gpu.cu -- Terrain2D::get_elevation (src/models/surface/terrain.rs:35-38,
// src/models/surface/interpolator.rs:17-29) for whole batches of query points on the
// GPU: rendering grids of millions of points in one call.
//
// One thread per query repeats interp.cpp's construction with the same IEEE double
// operations in the same order (no contraction), so both give the same bits:
//   locate   a visibility walk from the triangle of the point-location grid cell's
//            site, the edge tests rotating from edge (step mod 3);
//   site     a query equal to a vertex of that triangle takes the vertex's value;
//   cavity   breadth-first over neighbours: a triangle joins when its circumcircle
//            strictly holds q.  A neighbour found outside is tested again when met
//            again instead of being remembered (the same answer, so the same order);
//   hull     q on a hull edge of the cavity takes the linear interpolant along it;
//   weights  per boundary vertex, the shoelace area of the polygon through the new
//            and the swallowed circumcentres, relative to q; value = sum(w f) / sum(w).
// Pass 1 runs every query with the predicates' floating-point filters only and small
// per-thread tables (32 cavity triangles, 256 walk steps).  A query that needs more --
// an inconclusive filter (q on or very near an edge line or a circumcircle, q at a
// site), a larger cavity, a longer walk -- is deferred to pass 2, where a few threads
// redo it with exact expansion arithmetic and tables in global memory (up to 2,048
// cavity triangles: more only happens with over two thousand sites on one circle, and
// the call then fails with FL_ERR_INVALID_ARGUMENT).  Large batches are sorted by grid
// cell first, so that the threads of a warp walk the same triangles.
//
// Layout: vertices as (x, y) pairs, triangles as vertex triples, twins as int32 (-1 on
// the hull), circumcentres as pairs, and the start triangle of every grid cell.

#include <cuda_runtime.h>

#include <cub/device/device_radix_sort.cuh>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <mutex>
#include <string>
#include <vector>

#include "expansion.cuh"
#include "fastlem_gb300.h"
#include "interp.h"

namespace fl {
void set_last_error(const char* msg);

namespace {

constexpr uint32_t kFastCap = 32;          // pass 1: cavity triangles per query
constexpr uint64_t kFastWalk = 256;        // pass 1: walk steps per query
constexpr uint32_t kWideCap = 2048;        // pass 2: cavity triangles per query
constexpr unsigned kWideBlocks = 32, kWideThreads = 32;
constexpr uint64_t kChunk = 1ull << 26;    // queries per device round
constexpr uint64_t kSortFrom = 1ull << 16; // batches this large run in grid-cell order
constexpr int kThreads = 128;

// bytes of one pass-2 thread's tables: expansion scratch, cavity, boundary
constexpr size_t kSlabBytes =
    ((xp::kScratch * sizeof(double) + (2 * kWideCap + 2) * sizeof(uint32_t)) + 255) & ~size_t(255);

enum QueryStatus { kQOutside = 0, kQFound = 1, kQDefer = 2, kQTooLarge = 3 };
enum StatusWord { kDeferred = 0, kTooLarge = 1, kStatusWords = 2 };

struct View {
    const double2* __restrict__ xy;
    const uint32_t* __restrict__ tri;
    const int32_t* __restrict__ half;
    const double2* __restrict__ cc;
    const uint32_t* __restrict__ gtri;
    double gx0, gy0, gsx, gsy;
    uint32_t gw, gh;
    uint64_t walk_limit;                   // the host walk's limit: 4 x half-edges + 16
};

}  // namespace

struct InterpDevice {
    int device = 0;
    cudaStream_t stream = nullptr;
    double2* xy = nullptr;
    uint32_t* tri = nullptr;
    int32_t* half = nullptr;
    double2* cc = nullptr;
    uint32_t* gtri = nullptr;
    View view{};
    // per-call buffers, grown on demand
    double* values = nullptr;
    uint32_t n = 0;
    uint64_t cap = 0;                      // queries the sort and deferral buffers hold
    uint64_t qcap = 0;                     // queries the host-staging buffers hold
    double *qx = nullptr, *qy = nullptr, *out = nullptr;
    uint8_t* found = nullptr;
    uint32_t *keys = nullptr, *keys_alt = nullptr, *idx = nullptr, *idx_alt = nullptr;
    uint32_t* deferred = nullptr;
    void* sort_tmp = nullptr;
    size_t sort_bytes = 0;
    int* status = nullptr;
    int* h_status = nullptr;
    unsigned char* slab = nullptr;
};

void interp_device_release(InterpDevice* d) {
    if (!d) return;
    int cur = 0;
    cudaGetDevice(&cur);
    cudaSetDevice(d->device);
    if (d->stream) cudaStreamSynchronize(d->stream);
    void* ptrs[] = {d->xy,   d->tri,      d->half,     d->cc,  d->gtri,    d->values, d->qx,
                    d->qy,   d->out,      d->found,    d->keys, d->keys_alt, d->idx,  d->idx_alt,
                    d->deferred, d->sort_tmp, d->status, d->slab};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (d->h_status) cudaFreeHost(d->h_status);
    if (d->stream) cudaStreamDestroy(d->stream);
    cudaSetDevice(cur);
    delete d;
}

namespace {

int cuda_fail(const char* what, cudaError_t e) {
    char buf[256];
    snprintf(buf, sizeof buf, "%s: %s", what, cudaGetErrorString(e));
    set_last_error(buf);
    return e == cudaErrorMemoryAllocation ? FL_ERR_OUT_OF_MEMORY : FL_ERR_CUDA;
}

#define IG_CU(call)                                 \
    do {                                            \
        cudaError_t e_ = (call);                    \
        if (e_ != cudaSuccess) return cuda_fail(#call, e_); \
    } while (0)

__device__ __forceinline__ uint32_t nxt3(uint32_t e) { return (e % 3 == 2) ? e - 2 : e + 1; }

// interp.cpp's circumcentre, operation for operation.
__device__ __forceinline__ double2 circumcentre(double ax, double ay, double bx, double by,
                                                double cx, double cy) {
    const double dx = bx - ax, dy = by - ay, ex = cx - ax, ey = cy - ay;
    const double bl = dx * dx + dy * dy, cl = ex * ex + ey * ey;
    const double d = 0.5 / (dx * ey - dy * ex);
    return make_double2(ax + (ey * bl - dy * cl) * d, ay + (dx * cl - ex * bl) * d);
}

// Circumcentre, relative to q, of the new triangle (a, b, q) on boundary edge e.
__device__ __forceinline__ double2 new_centre(const View& V, uint32_t e, double x, double y) {
    const double2 a = V.xy[V.tri[e]], b = V.xy[V.tri[nxt3(e)]];
    return circumcentre(a.x - x, a.y - y, b.x - x, b.y - y, 0.0, 0.0);
}

// Sign of orient2d (a, b, q): the filter, then (kExact) the expansions; without them an
// inconclusive filter sets `defer`.
template <bool kExact>
__device__ __forceinline__ double orient(double2 a, double2 b, double x, double y, double* xs,
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
__device__ __forceinline__ double incircle(double2 a, double2 b, double2 c, double x, double y,
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

__device__ __forceinline__ bool holds(const uint32_t* s, uint32_t n, uint32_t t) {
    for (uint32_t i = 0; i < n; ++i)
        if (s[i] == t) return true;
    return false;
}

// Grid cell coordinate of q, clamped as interp.cpp's locate clamps it.
__device__ __forceinline__ uint32_t cell_coord(double q, double q0, double step, uint32_t cells) {
    double f = (q - q0) / step;
    f = (0.0 < f) ? f : 0.0;
    const double hi = (double)(cells - 1);
    f = (f < hi) ? f : hi;
    return (uint32_t)f;
}

// One query: the status and, when found, the value.  cav holds cap triangles, bnd
// cap + 2 edges; xs is the exact stages' scratch (kExact only).
template <bool kExact>
__device__ int query(const View& V, const double* __restrict__ f, double x, double y,
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

// Grid cell of every query (non-finite coordinates: cell 0) and the identity order.
__global__ void k_cell_keys(View V, uint64_t count, const double* __restrict__ qx,
                            const double* __restrict__ qy, uint32_t* __restrict__ keys,
                            uint32_t* __restrict__ idx) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= count) return;
    const double x = qx[i], y = qy[i];
    uint32_t key = 0;
    if (isfinite(x) && isfinite(y))
        key = cell_coord(y, V.gy0, V.gsy, V.gh) * V.gw + cell_coord(x, V.gx0, V.gsx, V.gw);
    keys[i] = key;
    idx[i] = (uint32_t)i;
}

// Pass 1: every query (in `order` when given), filters only; the rest is deferred.
__global__ void __launch_bounds__(kThreads) k_interp_fast(View V, const double* __restrict__ f,
                                                          uint64_t count, const double* __restrict__ qx,
                                                          const double* __restrict__ qy,
                                                          const uint32_t* __restrict__ order,
                                                          double* __restrict__ out,
                                                          uint8_t* __restrict__ found,
                                                          uint32_t* __restrict__ deferred,
                                                          int* __restrict__ status) {
    const uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (k >= count) return;
    const uint32_t i = order ? order[k] : (uint32_t)k;
    uint32_t cav[kFastCap], bnd[kFastCap + 2];
    double v = 0.0;
    const int s = query<false>(V, f, qx[i], qy[i], cav, bnd, kFastCap, nullptr, v);
    if (s == kQDefer) {
        deferred[atomicAdd(&status[kDeferred], 1)] = i;
        return;
    }
    out[i] = s == kQFound ? v : __longlong_as_double(0x7ff8000000000000ll);
    found[i] = s == kQFound;
}

// Pass 2: the deferred queries, exact predicates, tables in each thread's slab.
__global__ void __launch_bounds__(kWideThreads) k_interp_exact(View V, const double* __restrict__ f,
                                                               const double* __restrict__ qx,
                                                               const double* __restrict__ qy,
                                                               double* __restrict__ out,
                                                               uint8_t* __restrict__ found,
                                                               const uint32_t* __restrict__ deferred,
                                                               int* __restrict__ status,
                                                               unsigned char* __restrict__ slab) {
    const uint32_t w = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned char* mine = slab + (size_t)w * kSlabBytes;
    double* xs = reinterpret_cast<double*>(mine);
    uint32_t* cav = reinterpret_cast<uint32_t*>(mine + xp::kScratch * sizeof(double));
    uint32_t* bnd = cav + kWideCap;
    const uint32_t nd = (uint32_t)status[kDeferred];
    for (uint32_t k = w; k < nd; k += gridDim.x * blockDim.x) {
        const uint32_t i = deferred[k];
        double v = 0.0;
        const int s = query<true>(V, f, qx[i], qy[i], cav, bnd, kWideCap, xs, v);
        if (s == kQTooLarge) atomicExch(&status[kTooLarge], 1);
        out[i] = s == kQFound ? v : __longlong_as_double(0x7ff8000000000000ll);
        found[i] = s == kQFound;
    }
}

template <class T>
int grow_buffer(T*& p, uint64_t count) {
    if (p) cudaFree(p);
    p = nullptr;
    IG_CU(cudaMalloc((void**)&p, std::max<uint64_t>(1, count) * sizeof(T)));
    return FL_OK;
}

// The triangulation on the current device (once per interpolator).
int ensure_device(fl_interpolator* it) {
    if (it->dev) {
        IG_CU(cudaSetDevice(it->dev->device));
        return FL_OK;
    }
    const uint64_t halves = it->tri.size(), tris = halves / 3;
    if (halves >= (1ull << 31)) {
        set_last_error("fl_interpolate_gpu: more than 2^31 half-edges");
        return FL_ERR_INVALID_ARGUMENT;
    }
    auto* d = new InterpDevice;
    auto fail = [&](int rc) {
        interp_device_release(d);
        return rc;
    };
    if (cudaGetDevice(&d->device) != cudaSuccess) return fail(cuda_fail("cudaGetDevice", cudaGetLastError()));
    cudaError_t e;
    if ((e = cudaStreamCreateWithFlags(&d->stream, cudaStreamNonBlocking)) != cudaSuccess)
        return fail(cuda_fail("cudaStreamCreate", e));
    std::vector<double2> xy(it->n), cc(tris);
    for (uint32_t v = 0; v < it->n; ++v) xy[v] = make_double2(it->X[v], it->Y[v]);
    for (uint64_t t = 0; t < tris; ++t) cc[t] = make_double2(it->ccx[t], it->ccy[t]);
    std::vector<int32_t> half(halves);
    for (uint64_t h = 0; h < halves; ++h) half[h] = (int32_t)it->half[h];
    std::vector<uint32_t> gtri(it->gsite.size());
    for (size_t c = 0; c < gtri.size(); ++c) gtri[c] = (uint32_t)(it->vedge[it->gsite[c]] / 3);
    struct Up { void** dst; const void* src; size_t bytes; } ups[] = {
        {(void**)&d->xy, xy.data(), xy.size() * sizeof(double2)},
        {(void**)&d->tri, it->tri.data(), halves * sizeof(uint32_t)},
        {(void**)&d->half, half.data(), halves * sizeof(int32_t)},
        {(void**)&d->cc, cc.data(), cc.size() * sizeof(double2)},
        {(void**)&d->gtri, gtri.data(), gtri.size() * sizeof(uint32_t)},
    };
    for (auto& u : ups) {
        if ((e = cudaMalloc(u.dst, std::max<size_t>(16, u.bytes))) != cudaSuccess)
            return fail(cuda_fail("cudaMalloc", e));
        if ((e = cudaMemcpy(*u.dst, u.src, u.bytes, cudaMemcpyHostToDevice)) != cudaSuccess)
            return fail(cuda_fail("cudaMemcpy", e));
    }
    if ((e = cudaMalloc((void**)&d->status, kStatusWords * sizeof(int))) != cudaSuccess ||
        (e = cudaHostAlloc((void**)&d->h_status, kStatusWords * sizeof(int), cudaHostAllocDefault)) !=
            cudaSuccess ||
        (e = cudaMalloc((void**)&d->slab, (size_t)kWideBlocks * kWideThreads * kSlabBytes)) != cudaSuccess)
        return fail(cuda_fail("cudaMalloc", e));
    d->view = View{d->xy, d->tri, d->half, d->cc, d->gtri, it->gx0, it->gy0, it->gsx, it->gsy,
                   it->gw, it->gh, 4ull * halves + 16};
    it->dev = d;
    return FL_OK;
}

int ensure_queries(InterpDevice* d, uint64_t count, bool host_arrays) {
    if (host_arrays && count > d->qcap) {
        int rc;
        if ((rc = grow_buffer(d->qx, count)) || (rc = grow_buffer(d->qy, count)) ||
            (rc = grow_buffer(d->out, count)) || (rc = grow_buffer(d->found, count)))
            return rc;
        d->qcap = count;
    }
    if (count <= d->cap) return FL_OK;
    int rc;
    if ((rc = grow_buffer(d->keys, count)) || (rc = grow_buffer(d->keys_alt, count)) ||
        (rc = grow_buffer(d->idx, count)) || (rc = grow_buffer(d->idx_alt, count)) ||
        (rc = grow_buffer(d->deferred, count)))
        return rc;
    size_t bytes = 0;
    cub::DoubleBuffer<uint32_t> kb(d->keys, d->keys_alt), ib(d->idx, d->idx_alt);
    IG_CU(cub::DeviceRadixSort::SortPairs(nullptr, bytes, kb, ib, (int)count, 0, 32, d->stream));
    if (d->sort_tmp) cudaFree(d->sort_tmp);
    d->sort_tmp = nullptr;
    IG_CU(cudaMalloc(&d->sort_tmp, std::max<size_t>(16, bytes)));
    d->sort_bytes = bytes;
    d->cap = count;
    return FL_OK;
}

// Enqueues one round of queries (device arrays) on the interpolator's stream.
int run_round(InterpDevice* d, const double* f, uint64_t count, const double* qx, const double* qy,
              double* out, uint8_t* found) {
    const View& V = d->view;
    IG_CU(cudaMemsetAsync(d->status, 0, sizeof(int), d->stream));   // the deferred count
    const uint32_t* order = nullptr;
    const unsigned blocks = (unsigned)((count + kThreads - 1) / kThreads);
    if (count >= kSortFrom) {
        k_cell_keys<<<blocks, kThreads, 0, d->stream>>>(V, count, qx, qy, d->keys, d->idx);
        IG_CU(cudaGetLastError());
        uint32_t cells = V.gw * V.gh, bits = 1;
        while (bits < 32 && (1ull << bits) < cells) ++bits;
        cub::DoubleBuffer<uint32_t> kb(d->keys, d->keys_alt), ib(d->idx, d->idx_alt);
        size_t bytes = 0;
        IG_CU(cub::DeviceRadixSort::SortPairs(nullptr, bytes, kb, ib, (int)count, 0, (int)bits,
                                              d->stream));
        if (bytes > d->sort_bytes) {
            IG_CU(cudaStreamSynchronize(d->stream));
            cudaFree(d->sort_tmp);
            d->sort_tmp = nullptr;
            d->sort_bytes = 0;
            IG_CU(cudaMalloc(&d->sort_tmp, bytes));
            d->sort_bytes = bytes;
        }
        bytes = d->sort_bytes;
        IG_CU(cub::DeviceRadixSort::SortPairs(d->sort_tmp, bytes, kb, ib, (int)count, 0, (int)bits,
                                              d->stream));
        order = ib.Current();
    }
    k_interp_fast<<<blocks, kThreads, 0, d->stream>>>(V, f, count, qx, qy, order, out, found,
                                                      d->deferred, d->status);
    IG_CU(cudaGetLastError());
    k_interp_exact<<<kWideBlocks, kWideThreads, 0, d->stream>>>(V, f, qx, qy, out, found,
                                                               d->deferred, d->status, d->slab);
    IG_CU(cudaGetLastError());
    return FL_OK;
}

int finish(InterpDevice* d, const char* who) {
    IG_CU(cudaMemcpyAsync(d->h_status, d->status, kStatusWords * sizeof(int), cudaMemcpyDeviceToHost,
                          d->stream));
    IG_CU(cudaStreamSynchronize(d->stream));
    if (d->h_status[kTooLarge]) {
        std::string m = std::string(who) +
                        ": a query's natural-neighbour cavity exceeds 2048 triangles (sites on one circle)";
        set_last_error(m.c_str());
        return FL_ERR_INVALID_ARGUMENT;
    }
    return FL_OK;
}

int check_args(const fl_interpolator* it, uint64_t count, const double* values, const double* qx,
               const double* qy, const double* out, const uint8_t* found, const char* who) {
    if (!it || (count && (!values || !qx || !qy || !out || !found))) {
        set_last_error((std::string(who) + ": null argument").c_str());
        return FL_ERR_INVALID_ARGUMENT;
    }
    return FL_OK;
}

}  // namespace
}  // namespace fl

extern "C" {

int fl_interpolate_gpu(fl_interpolator* it, const double* values, uint64_t count, const double* qx,
                       const double* qy, double* out, uint8_t* found) {
    using namespace fl;
    if (int rc = check_args(it, count, values, qx, qy, out, found, "fl_interpolate_gpu")) return rc;
    if (!count) return FL_OK;
    std::lock_guard<std::mutex> lock(it->device_mu);
    if (int rc = ensure_device(it)) return rc;
    InterpDevice* d = it->dev;
    if (int rc = ensure_queries(d, std::min(count, kChunk), true)) return rc;
    if (!d->values || d->n != it->n) {
        if (int rc = grow_buffer(d->values, it->n)) return rc;
        d->n = it->n;
    }
    IG_CU(cudaMemcpyAsync(d->values, values, it->n * sizeof(double), cudaMemcpyHostToDevice, d->stream));
    IG_CU(cudaMemsetAsync(d->status, 0, kStatusWords * sizeof(int), d->stream));
    for (uint64_t a = 0; a < count; a += kChunk) {
        const uint64_t m = std::min(kChunk, count - a);
        IG_CU(cudaMemcpyAsync(d->qx, qx + a, m * 8, cudaMemcpyHostToDevice, d->stream));
        IG_CU(cudaMemcpyAsync(d->qy, qy + a, m * 8, cudaMemcpyHostToDevice, d->stream));
        if (int rc = run_round(d, d->values, m, d->qx, d->qy, d->out, d->found)) return rc;
        IG_CU(cudaMemcpyAsync(out + a, d->out, m * 8, cudaMemcpyDeviceToHost, d->stream));
        IG_CU(cudaMemcpyAsync(found + a, d->found, m, cudaMemcpyDeviceToHost, d->stream));
    }
    return finish(d, "fl_interpolate_gpu");
}

int fl_interpolate_device(fl_interpolator* it, const double* values, uint64_t count, const double* qx,
                          const double* qy, double* out, uint8_t* found) {
    using namespace fl;
    if (int rc = check_args(it, count, values, qx, qy, out, found, "fl_interpolate_device")) return rc;
    if (!count) return FL_OK;
    std::lock_guard<std::mutex> lock(it->device_mu);
    if (int rc = ensure_device(it)) return rc;
    InterpDevice* d = it->dev;
    if (int rc = ensure_queries(d, std::min(count, kChunk), false)) return rc;
    IG_CU(cudaMemsetAsync(d->status, 0, kStatusWords * sizeof(int), d->stream));
    for (uint64_t a = 0; a < count; a += kChunk) {
        const uint64_t m = std::min(kChunk, count - a);
        if (int rc = run_round(d, values, m, qx + a, qy + a, out + a, found + a)) return rc;
    }
    return finish(d, "fl_interpolate_device");
}

}  // extern "C"
