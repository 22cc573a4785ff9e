// ordering.cu -- a model's graph on the device, in memory order.
//
// Synthetic and builder-made sites come in random order, so a site's neighbours,
// receiver and donors would be scattered over the whole array and every gather would
// miss the caches.  The solver stores sites in the order of a Hilbert curve through
// the bounding box of their coordinates (per terrain when terrains are packed):
// neighbours and river paths land on nearby indices.  Relabelling never changes
// results: every row keeps its slot order (the adjacency order the reference's
// tie-breaks and sums follow), outlet lists keep their order, and all inputs / outputs
// are translated at the boundary.
//
// Everything after the upload runs on the device: the input checks (monotone rows,
// columns in range, no NaN length, no edge across terrains), the curve keys, a stable
// radix sort of (terrain, key), and the relabelled CSR (degrees, scan, row copies),
// so creating a model costs about its upload.

#include <cuda_runtime.h>

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "common.cuh"
#include "kernels.h"
#include "ordering.h"

namespace fl {
namespace {

enum { kBadRow = 0, kBadSlot = 1, kCross = 2, kCheckWords = 4 };
constexpr uint32_t kOrder = 16;                         // 2^16 x 2^16 grid

inline unsigned grid_for(uint64_t n, unsigned t = 256) {
    return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((n + t - 1) / t, 152ull * 64));
}

// Terrain of site i: the t with so[t] <= i < so[t + 1] (k offsets + 1, increasing).
__device__ __forceinline__ uint32_t terrain_of(uint32_t i, const uint32_t* so, uint32_t k) {
    uint32_t lo = 0, hi = k;                             // so[lo] <= i < so[hi]
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (so[mid] <= i) lo = mid;
        else hi = mid;
    }
    return lo;
}

// Parts uploaded one after another: row entries and columns move by the part's first
// slot and first site.
__global__ void k_shift_parts(uint32_t n, uint64_t nnz, const uint32_t* __restrict__ so,
                              const unsigned long long* __restrict__ eo, uint32_t k,
                              uint32_t* __restrict__ row, uint32_t* __restrict__ col) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += stride)
        row[i] += (uint32_t)eo[terrain_of((uint32_t)i, so, k)];
    for (uint64_t sl = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; sl < nnz; sl += stride) {
        uint32_t lo = 0, hi = k;                         // eo[lo] <= sl < eo[hi]
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (eo[mid] <= sl) lo = mid;
            else hi = mid;
        }
        col[sl] += so[lo];
    }
}

__global__ void k_check_rows(uint32_t n, const uint32_t* __restrict__ row, uint32_t* st) {
    bool bad = false;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        bad |= row[i + 1] < row[i];
    if (__syncthreads_or(bad) && threadIdx.x == 0) st[kBadRow] = 1;
}

// Columns in range, no NaN length, and (packed terrains) no edge leaving its terrain.
__global__ void k_check_slots(uint32_t n, const uint32_t* __restrict__ row,
                              const uint32_t* __restrict__ col, const double* __restrict__ len,
                              const uint32_t* __restrict__ so, uint32_t k, uint32_t* st) {
    bool bad = false, cross = false;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint32_t lo = 0, hi = n;
        if (k > 1) {
            const uint32_t t = terrain_of(i, so, k);
            lo = so[t];
            hi = so[t + 1];
        }
        for (uint32_t s = row[i], e = row[i + 1]; s < e; ++s) {
            const uint32_t c = col[s];
            bad |= c >= n || isnan(len[s]);
            cross |= c < lo || c >= hi;
        }
    }
    if (__syncthreads_or(bad) && threadIdx.x == 0) st[kBadSlot] = 1;
    if (__syncthreads_or(cross) && threadIdx.x == 0) st[kCross] = 1;
}

// key = (terrain << 32) | Hilbert index of the site's cell in its terrain's box; the
// cell is floor((x - x0) * sx) clamped to the grid, non-finite coordinates at 0.
__global__ void k_curve_keys(uint32_t n, const double* __restrict__ xs,
                             const double* __restrict__ ys, const uint32_t* __restrict__ so,
                             uint32_t k, const double* __restrict__ box,
                             unsigned long long* __restrict__ key, uint32_t* __restrict__ val) {
    const double cells = (double)((1u << kOrder) - 1);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t t = k > 1 ? terrain_of(i, so, k) : 0;
        const double* b = box + 4 * t;                   // x0, y0, sx, sy
        const double x = xs[i], y = ys[i];
        const double fx = isfinite(x) ? __dmul_rn(__dsub_rn(x, b[0]), b[2]) : 0.0;
        const double fy = isfinite(y) ? __dmul_rn(__dsub_rn(y, b[1]), b[3]) : 0.0;
        const uint32_t cx = (uint32_t)fmin(cells, fmax(0.0, fx));
        const uint32_t cy = (uint32_t)fmin(cells, fmax(0.0, fy));
        key[i] = ((unsigned long long)t << 32) | hilbert_index(kOrder, cx, cy);
        val[i] = i;
    }
}

__global__ void k_iota_u32(uint32_t n, uint32_t* __restrict__ a) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        a[i] = i;
}

// inv[perm[j]] = j, the new row degrees and the cell areas in device order.
__global__ void k_order_maps(uint32_t n, const uint32_t* __restrict__ perm,
                             const uint32_t* __restrict__ row, const double* __restrict__ area,
                             uint32_t* __restrict__ inv, uint32_t* __restrict__ deg,
                             double* __restrict__ parea) {
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        const uint32_t o = perm[j];
        inv[o] = j;
        deg[j] = row[o + 1] - row[o];
        parea[j] = area[o];
    }
}

// New row j is old row perm[j], columns through inv, slot order kept.
__global__ void k_relabel_rows(uint32_t n, const uint32_t* __restrict__ perm,
                               const uint32_t* __restrict__ row, const uint32_t* __restrict__ col,
                               const double* __restrict__ len, const uint32_t* __restrict__ inv,
                               const uint32_t* __restrict__ nrow, uint32_t* __restrict__ ncol,
                               double* __restrict__ nlen) {
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        const uint32_t o = perm[j];
        uint32_t d = nrow[j];
        for (uint32_t s = row[o], e = row[o + 1]; s < e; ++s, ++d) {
            ncol[d] = inv[col[s]];
            nlen[d] = len[s];
        }
    }
}

// Packed terrains, per device site: its terrain and its sample index in that terrain's
// noise stream (its caller index within the terrain).
__global__ void k_terrain_maps(uint32_t n, const uint32_t* __restrict__ perm,
                               const uint32_t* __restrict__ so, uint32_t k,
                               uint32_t* __restrict__ tid, uint32_t* __restrict__ nidx) {
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        const uint32_t t = terrain_of(j, so, k);
        tid[j] = t;
        nidx[j] = perm[j] - so[t];
    }
}

struct Temps {
    cudaStream_t st;
    std::vector<void*> bufs;
    cudaError_t err = cudaSuccess;
    explicit Temps(cudaStream_t s) : st(s) {}
    template <class T>
    T* get(uint64_t count) {
        void* p = nullptr;
        if (err != cudaSuccess) return nullptr;
        err = cudaMallocAsync(&p, std::max<uint64_t>(1, count) * sizeof(T), st);
        if (err != cudaSuccess) return nullptr;
        bufs.push_back(p);
        return (T*)p;
    }
    ~Temps() {
        for (void* p : bufs) cudaFreeAsync(p, st);
    }
};

}  // namespace

int build_device_graph(cudaStream_t st, const GraphInput& in, const GraphOutput& out,
                       std::string* err) {
    const uint32_t n = in.n, k = in.terrains;
    const uint64_t nnz = in.nnz;
    Temps tmp(st);
    auto cuda_fail = [&](cudaError_t e, const char* what) {
        *err = std::string(what) + ": " + cudaGetErrorString(e);
        return e == cudaErrorMemoryAllocation ? 22 /* FL_ERR_OUT_OF_MEMORY */ : 21 /* FL_ERR_CUDA */;
    };
#define OB_CU(x, what)                        \
    do {                                      \
        cudaError_t e_ = (x);                 \
        if (e_ != cudaSuccess) return cuda_fail(e_, what); \
    } while (0)
    uint32_t* row = tmp.get<uint32_t>(n + 1ull);
    uint32_t* col = tmp.get<uint32_t>(nnz);
    double* len = tmp.get<double>(nnz);
    double* area = tmp.get<double>(n);
    uint32_t* so = tmp.get<uint32_t>(k + 1ull);
    uint32_t* st_w = tmp.get<uint32_t>(kCheckWords);
    if (!st_w) return cuda_fail(tmp.err, "graph upload");
    OB_CU(cudaMemcpyAsync(so, in.site_off, (k + 1ull) * 4, cudaMemcpyHostToDevice, st), "graph upload");
    const uint32_t nnz32 = (uint32_t)nnz;
    if (!in.parts) {
        OB_CU(cudaMemcpyAsync(row, in.row_ptr, (n + 1ull) * 4, cudaMemcpyHostToDevice, st), "graph upload");
        if (nnz) {
            OB_CU(cudaMemcpyAsync(col, in.col, nnz * 4, cudaMemcpyHostToDevice, st), "graph upload");
            OB_CU(cudaMemcpyAsync(len, in.len, nnz * 8, cudaMemcpyHostToDevice, st), "graph upload");
        }
        OB_CU(cudaMemcpyAsync(area, in.area, n * 8ull, cudaMemcpyHostToDevice, st), "graph upload");
    } else {
        unsigned long long* eo = tmp.get<unsigned long long>(k + 1ull);
        if (!eo) return cuda_fail(tmp.err, "graph upload");
        for (uint32_t t = 0; t < k; ++t) {
            const GraphPart& pt = in.parts[t];
            const uint32_t a = in.site_off[t], m = in.site_off[t + 1] - a;
            const uint64_t e0 = in.slot_off[t], ne = in.slot_off[t + 1] - e0;
            OB_CU(cudaMemcpyAsync(row + a, pt.row_ptr, m * 4ull, cudaMemcpyHostToDevice, st), "graph upload");
            if (ne) {
                OB_CU(cudaMemcpyAsync(col + e0, pt.col, ne * 4, cudaMemcpyHostToDevice, st), "graph upload");
                OB_CU(cudaMemcpyAsync(len + e0, pt.len, ne * 8, cudaMemcpyHostToDevice, st), "graph upload");
            }
            OB_CU(cudaMemcpyAsync(area + a, pt.area, m * 8ull, cudaMemcpyHostToDevice, st), "graph upload");
        }
        OB_CU(cudaMemcpyAsync(row + n, &nnz32, 4, cudaMemcpyHostToDevice, st), "graph upload");
        OB_CU(cudaMemcpyAsync(eo, in.slot_off, (k + 1ull) * 8, cudaMemcpyHostToDevice, st), "graph upload");
        k_shift_parts<<<grid_for(std::max<uint64_t>(n, nnz)), 256, 0, st>>>(n, nnz, so, eo, k, row, col);
    }
    OB_CU(cudaMemsetAsync(st_w, 0, kCheckWords * 4, st), "graph upload");
    k_check_rows<<<grid_for(n), 256, 0, st>>>(n, row, st_w);
    uint32_t h[kCheckWords];
    OB_CU(cudaMemcpyAsync(h, st_w, sizeof h, cudaMemcpyDeviceToHost, st), "graph checks");
    OB_CU(cudaStreamSynchronize(st), "graph checks");
    if (h[kBadRow]) {
        *err = "row_ptr not monotone";
        return 20;
    }
    k_check_slots<<<grid_for(n), 256, 0, st>>>(n, row, col, len, so, k, st_w);
    OB_CU(cudaMemcpyAsync(h, st_w, sizeof h, cudaMemcpyDeviceToHost, st), "graph checks");
    OB_CU(cudaStreamSynchronize(st), "graph checks");
    if (h[kBadSlot]) {
        *err = "column out of range or NaN length";
        return 20;
    }
    if (h[kCross]) {
        *err = "an edge crosses two terrains";
        return 20;
    }
    // the memory order: per-terrain curve keys sorted stably (ties keep index order)
    const bool coords = in.parts ? (in.parts[0].xs && in.parts[0].ys) : (in.xs && in.ys);
    if (coords) {
        double* xs = tmp.get<double>(n);
        double* ys = tmp.get<double>(n);
        double* box = tmp.get<double>(4ull * k);
        unsigned long long* key = tmp.get<unsigned long long>(n);
        unsigned long long* key2 = tmp.get<unsigned long long>(n);
        uint32_t* val = tmp.get<uint32_t>(n);
        if (!val) return cuda_fail(tmp.err, "memory order");
        for (uint32_t t = 0; t < k; ++t) {
            const uint32_t a = in.site_off[t], m = in.site_off[t + 1] - a;
            const double* px = in.parts ? in.parts[t].xs : in.xs + a;
            const double* py = in.parts ? in.parts[t].ys : in.ys + a;
            if (in.parts && (!px || !py)) {
                *err = "coordinates given for some terrains only";
                return 20;
            }
            if (in.parts || t == 0) {
                const uint32_t cnt = in.parts ? m : n;
                OB_CU(cudaMemcpyAsync(xs + a, px, cnt * 8ull, cudaMemcpyHostToDevice, st), "graph upload");
                OB_CU(cudaMemcpyAsync(ys + a, py, cnt * 8ull, cudaMemcpyHostToDevice, st), "graph upload");
            }
        }
        // every terrain's bounding box (finite coordinates) on the host meanwhile
        std::vector<double> hb(4ull * k);
        const double cells = (double)((1u << kOrder) - 1);
        for (uint32_t t = 0; t < k; ++t) {
            double x0 = INFINITY, y0 = INFINITY, x1 = -INFINITY, y1 = -INFINITY;
            const uint32_t a = in.site_off[t], m = in.site_off[t + 1] - a;
            const double* px = in.parts ? in.parts[t].xs : in.xs + a;
            const double* py = in.parts ? in.parts[t].ys : in.ys + a;
            for (uint32_t i = 0; i < m; ++i) {
                if (std::isfinite(px[i])) { x0 = std::min(x0, px[i]); x1 = std::max(x1, px[i]); }
                if (std::isfinite(py[i])) { y0 = std::min(y0, py[i]); y1 = std::max(y1, py[i]); }
            }
            hb[4 * t] = x0;
            hb[4 * t + 1] = y0;
            hb[4 * t + 2] = (x1 > x0) ? cells / (x1 - x0) : 0.0;
            hb[4 * t + 3] = (y1 > y0) ? cells / (y1 - y0) : 0.0;
        }
        OB_CU(cudaMemcpyAsync(box, hb.data(), hb.size() * 8, cudaMemcpyHostToDevice, st), "memory order");
        k_curve_keys<<<grid_for(n), 256, 0, st>>>(n, xs, ys, so, k, box, key, val);
        int end_bit = 32;
        while (end_bit < 64 && (1ull << (end_bit - 32)) < k) ++end_bit;
        size_t tb = 0;
        OB_CU(cub::DeviceRadixSort::SortPairs(nullptr, tb, key, key2, val, out.perm, (int)n, 0,
                                              end_bit, st), "memory order");
        void* ws = tmp.get<uint8_t>(tb);
        if (!ws) return cuda_fail(tmp.err, "memory order");
        OB_CU(cub::DeviceRadixSort::SortPairs(ws, tb, key, key2, val, out.perm, (int)n, 0, end_bit, st),
              "memory order");
        // the host's copy of the boxes must outlive the copy above
        OB_CU(cudaStreamSynchronize(st), "memory order");
    } else {
        k_iota_u32<<<grid_for(n), 256, 0, st>>>(n, out.perm);
    }
    // relabelled CSR
    uint32_t* deg = tmp.get<uint32_t>(n + 1ull);
    if (!deg) return cuda_fail(tmp.err, "relabelling");
    OB_CU(cudaMemsetAsync(deg + n, 0, 4, st), "relabelling");
    k_order_maps<<<grid_for(n), 256, 0, st>>>(n, out.perm, row, area, out.inv, deg, out.area);
    size_t tb = 0;
    OB_CU(cub::DeviceScan::ExclusiveSum(nullptr, tb, deg, out.row, (int)n + 1, st), "relabelling");
    void* ws = tmp.get<uint8_t>(tb);
    if (!ws) return cuda_fail(tmp.err, "relabelling");
    OB_CU(cub::DeviceScan::ExclusiveSum(ws, tb, deg, out.row, (int)n + 1, st), "relabelling");
    k_relabel_rows<<<grid_for(n), 256, 0, st>>>(n, out.perm, row, col, len, out.inv, out.row,
                                                out.col, out.len);
    if (k > 1) k_terrain_maps<<<grid_for(n), 256, 0, st>>>(n, out.perm, so, k, out.tid, out.noise_idx);
    OB_CU(cudaGetLastError(), "graph kernels");
    return 0;
#undef OB_CU
}

}  // namespace fl
