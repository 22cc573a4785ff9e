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
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "expansion.cuh"
#include "fastlem_gb300.h"
#include "interp.h"
#include "interp_query.cuh"

namespace fl {
void set_last_error(const char* msg);
using namespace iq;

namespace {

constexpr uint32_t kWideCap = 2048;        // pass 2: cavity triangles per query
constexpr unsigned kWideBlocks = 32, kWideThreads = 32;
constexpr uint64_t kChunk = 1ull << 26;    // queries per device round
constexpr uint64_t kSortFrom = 1ull << 16; // batches this large run in grid-cell order
constexpr int kThreads = 128;

// bytes of one pass-2 thread's tables: expansion scratch, cavity, boundary
constexpr size_t kSlabBytes =
    ((xp::kScratch * sizeof(double) + (2 * kWideCap + 2) * sizeof(uint32_t)) + 255) & ~size_t(255);

}  // namespace

struct InterpDevice {
    int device = 0;
    cudaStream_t stream = nullptr;
    double2* xy = nullptr;
    float2* xyf = nullptr;
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
    uint64_t last_deferred = 0;            // queries of the last call the exact pass answered
    unsigned char* slab = nullptr;
};

void interp_device_release(InterpDevice* d) {
    if (!d) return;
    int cur = 0;
    cudaGetDevice(&cur);
    cudaSetDevice(d->device);
    if (d->stream) cudaStreamSynchronize(d->stream);
    void* ptrs[] = {d->xy,   d->xyf,  d->tri,      d->half,     d->cc,  d->gtri,    d->values, d->qx,
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
    // every thread of a warp takes part in the warp-synchronous query, with or without one
    const uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    const bool active = k < count;
    const uint32_t i = !active ? 0u : order ? order[k] : (uint32_t)k;
    uint32_t cav[kFastCap], bnd[kFastCap + 2];
    double2 centre[kFastCap + 2];
    double v = 0.0;
    const int s = query_fast(V, f, active, active ? qx[i] : 0.0, active ? qy[i] : 0.0, cav, bnd,
                             centre, v);
    if (!active) return;
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
    if (w == 0) atomicAdd(reinterpret_cast<unsigned long long*>(status + kDeferredTotal), nd);
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
    std::vector<float2> xyf(it->n);
    float smax = 0.0f;
    for (uint32_t v = 0; v < it->n; ++v) {
        xy[v] = make_double2(it->X[v], it->Y[v]);
        xyf[v] = make_float2((float)it->X[v], (float)it->Y[v]);
        smax = std::max(smax, std::max(std::fabs(xyf[v].x), std::fabs(xyf[v].y)));
    }
    for (uint64_t t = 0; t < tris; ++t) cc[t] = make_double2(it->ccx[t], it->ccy[t]);
    std::vector<int32_t> half(halves);
    for (uint64_t h = 0; h < halves; ++h) half[h] = (int32_t)it->half[h];
    const std::vector<uint32_t>& gtri = it->gtri;
    struct Up { void** dst; const void* src; size_t bytes; } ups[] = {
        {(void**)&d->xy, xy.data(), xy.size() * sizeof(double2)},
        {(void**)&d->xyf, xyf.data(), xyf.size() * sizeof(float2)},
        {(void**)&d->tri, it->tri.data(), halves * sizeof(uint32_t)},
        {(void**)&d->half, half.data(), halves * sizeof(int32_t)},
        {(void**)&d->cc, cc.data(), cc.size() * sizeof(double2)},
        {(void**)&d->gtri, (const void*)gtri.data(), gtri.size() * sizeof(uint32_t)},
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
                   it->gw, it->gh, 4ull * halves + 16, d->xyf, smax};
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
    uint64_t total;
    std::memcpy(&total, d->h_status + kDeferredTotal, 8);
    d->last_deferred = total;
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

// Probe of the float prefilters: per case (ax, ay, bx, by, cx, cy, qx, qy), the
// prefilter's orientation sign of (a, b, q) and in-circle sign of (a, b, c, q) (0:
// undecided) and the exact signs, in out[4 i .. 4 i + 3].
int fl_probe_prefilters(uint64_t count, const double* cases, int32_t* out) {
    using namespace fl;
    if (count && (!cases || !out)) {
        set_last_error("fl_probe_prefilters: null argument");
        return FL_ERR_INVALID_ARGUMENT;
    }
    std::vector<double> xs(xp::kScratch);
    for (uint64_t i = 0; i < count; ++i) {
        const double* c = cases + 8 * i;
        float smax = 0.0f;
        float2 f[3];
        for (int k = 0; k < 3; ++k) {
            f[k] = make_float2((float)c[2 * k], (float)c[2 * k + 1]);
            smax = std::max(smax, std::max(std::fabs(f[k].x), std::fabs(f[k].y)));
        }
        View V{};
        V.smax = smax;
        const QueryF q = query_f(V, c[6], c[7]);
        auto sgn = [](double v) { return v > 0.0 ? 1 : (v < 0.0 ? -1 : 0); };
        out[4 * i] = q.ok ? orient_f(f[0], f[1], q) : 0;
        out[4 * i + 1] = q.ok ? incircle_f(f[0], f[1], f[2], q) : 0;
        out[4 * i + 2] = sgn(xp::orient_exact(c[0], c[1], c[2], c[3], c[6], c[7], xs.data()));
        out[4 * i + 3] =
            sgn(xp::incircle_exact(c[0], c[1], c[2], c[3], c[4], c[5], c[6], c[7], xs.data()));
    }
    return FL_OK;
}

uint64_t fl_interpolator_last_deferred(const fl_interpolator* it) {
    return it && it->dev ? it->dev->last_deferred : 0;
}

// The device query code compiled for the host, one query after another: exact = 0 runs
// the first pass (status 2: deferred), exact = 1 the second (status 3: cavity too large).
int fl_probe_interp_query(const fl_interpolator* it, const double* values, uint64_t count,
                          const double* qx, const double* qy, int exact, double* out,
                          int32_t* status) {
    using namespace fl;
    if (!it || (count && (!values || !qx || !qy || !out || !status))) {
        set_last_error("fl_probe_interp_query: null argument");
        return FL_ERR_INVALID_ARGUMENT;
    }
    const uint64_t halves = it->tri.size();
    std::vector<double2> xy(it->n), cc(halves / 3);
    std::vector<float2> xyf(it->n);
    float smax = 0.0f;
    for (uint32_t v = 0; v < it->n; ++v) {
        xy[v] = make_double2(it->X[v], it->Y[v]);
        xyf[v] = make_float2((float)it->X[v], (float)it->Y[v]);
        smax = std::max(smax, std::max(std::fabs(xyf[v].x), std::fabs(xyf[v].y)));
    }
    for (uint64_t t = 0; t < halves / 3; ++t) cc[t] = make_double2(it->ccx[t], it->ccy[t]);
    std::vector<int32_t> half(halves);
    for (uint64_t h = 0; h < halves; ++h) half[h] = (int32_t)it->half[h];
    const std::vector<uint32_t>& gtri = it->gtri;
    const View V{xy.data(),  it->tri.data(), half.data(), cc.data(), gtri.data(),
                 it->gx0,    it->gy0,        it->gsx,     it->gsy,   it->gw,
                 it->gh,     4ull * halves + 16, xyf.data(), smax};
    std::vector<double> xs(xp::kScratch);
    std::vector<uint32_t> cav(kWideCap), bnd(kWideCap + 2);
    std::vector<double2> centre(kFastCap + 2);
    for (uint64_t i = 0; i < count; ++i) {
        double v = NAN;
        const int s = exact ? query<true>(V, values, qx[i], qy[i], cav.data(), bnd.data(), kWideCap,
                                          xs.data(), v)
                            : query_fast(V, values, true, qx[i], qy[i], cav.data(), bnd.data(),
                                         centre.data(), v);
        out[i] = s == kQFound ? v : NAN;
        status[i] = s;
    }
    return FL_OK;
}

}  // extern "C"
