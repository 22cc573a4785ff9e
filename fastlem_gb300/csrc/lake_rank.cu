// lake_rank.cu -- the lake heap's processing order, computed on the GPU.
//
// fastlem re-routes lakes with a min-heap traversal from the outlets keyed by edge
// length (src/lem/stream_tree.rs:175-243).  Which sites it pops, in which order, does
// not depend on the receivers, so the order ("rank") is computed once per model and
// outlet list.  The outlets all enter with key 0.0 and are popped first, in an order
// the heap's arrangement decides; that tied prefix is replayed on the host
// (lake_rank_prefix).  From then on, when every edge is longer than zero and the keys
// that compete are distinct, the traversal is Prim's algorithm from the prefix
// contracted to one source R, and its order follows from the minimum spanning tree T
// rooted at R:
//   * give every site v != R the weight W(v) of the tree edge to its parent;
//   * let nga(v) be v's nearest proper ancestor a with W(a) > W(v) (R when there is
//     none; W(R) = infinity);
//   * the traversal visits the forest v -> nga(v) in pre-order, children in ascending
//     W.
// (The sites below v reachable over edges lighter than W(v) form the component Prim
// completes right after entering v; a child u of v in that forest is entered once
// the part of the component lighter than W(u) is complete, so lighter children come
// first.)  Each step is a data-parallel tree computation:
//   1. T by Boruvka rounds (per component the lightest outgoing edge by a 64-bit
//      atomicMin of the length's bit pattern, hooking, pointer jumping);
//   2. T rooted at R by an Euler tour and list ranking (pointer jumping);
//   3. nga by binary lifting over (ancestor, largest weight rank above);
//   4. the forest's children sorted by (nga, weight rank), a second Euler tour and
//      list ranking give every site its pre-order position.
// The keyed order is the same as the heap's exactly when no two competing keys are
// equal.  Two checks make sure of that: every Boruvka minimum is strict (the tree is
// then the only minimum spanning tree), and the tree's edge weights are pairwise
// distinct (so two frontier sites never share the smallest key).  If either fails, or
// an edge length is not positive, the caller falls back to the host heap.

#include <cuda_runtime.h>

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include <algorithm>
#include <cstdint>
#include <vector>

#include "common.cuh"
#include "kernels.h"

namespace fl {
namespace {

constexpr uint32_t kEnd = 0xffffffffu;
constexpr unsigned long long kInfKey = ~0ull;

// status words
enum { kStTie = 0, kStBadLen = 1, kStMerged = 2, kStEdges = 3, kStJumped = 4, kStCount = 8 };

inline unsigned grid_for(uint64_t n, unsigned t = 256) {
    return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((n + t - 1) / t, 152ull * 64));
}

// Every length must be > 0 (NaN, zero and negative lengths take the host heap).
__global__ void k_check_len(uint64_t nnz, const double* __restrict__ len, uint32_t* st) {
    bool bad = false;
    for (uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; s < nnz;
         s += (uint64_t)gridDim.x * blockDim.x)
        bad |= !(len[s] > 0.0);
    if (__syncthreads_or(bad) && threadIdx.x == 0) st[kStBadLen] = 1;
}

// comp[v] = v for v in [0, n]; id n is the contracted source R.
__global__ void k_iota(uint32_t cnt, uint32_t* __restrict__ a) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x)
        a[i] = i;
}

__global__ void k_mark_prefix(uint32_t k, const uint32_t* __restrict__ prefix, uint32_t n,
                              uint32_t* __restrict__ comp, uint8_t* __restrict__ inpre) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < k) {
        comp[prefix[i]] = n;
        inpre[prefix[i]] = 1;
    }
}

__global__ void k_bv_reset(uint32_t nc, unsigned long long* __restrict__ bw,
                           unsigned long long* __restrict__ emin,
                           unsigned long long* __restrict__ emax, uint32_t* __restrict__ hook) {
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
        bw[c] = kInfKey;
        emin[c] = kInfKey;
        emax[c] = 0;
        hook[c] = c;
    }
}

// Per component: the smallest length bit pattern of an edge leaving it (lengths are
// positive, so bit patterns order like values).
__global__ void k_bv_minw(uint32_t n, const uint32_t* __restrict__ row,
                          const uint32_t* __restrict__ col, const double* __restrict__ len,
                          const uint32_t* __restrict__ comp, unsigned long long* bw) {
    for (uint32_t u = blockIdx.x * blockDim.x + threadIdx.x; u < n; u += gridDim.x * blockDim.x) {
        const uint32_t cu = comp[u];
        unsigned long long m = kInfKey;
        for (uint32_t s = row[u], e = row[u + 1]; s < e; ++s)
            if (comp[col[s]] != cu) m = min(m, (unsigned long long)__double_as_longlong(len[s]));
        if (m != kInfKey) atomicMin(&bw[cu], m);
    }
}

// Per component: the smallest and largest edge (as an endpoint pair, prefix sites
// standing for R) among those of the minimum length; they differ on a tie.
__global__ void k_bv_mine(uint32_t n, const uint32_t* __restrict__ row,
                          const uint32_t* __restrict__ col, const double* __restrict__ len,
                          const uint32_t* __restrict__ comp, const uint8_t* __restrict__ inpre,
                          const unsigned long long* __restrict__ bw, unsigned long long* emin,
                          unsigned long long* emax) {
    for (uint32_t u = blockIdx.x * blockDim.x + threadIdx.x; u < n; u += gridDim.x * blockDim.x) {
        const uint32_t cu = comp[u];
        const unsigned long long target = bw[cu];
        if (target == kInfKey) continue;
        const uint32_t mu = inpre[u] ? n : u;
        for (uint32_t s = row[u], e = row[u + 1]; s < e; ++s) {
            const uint32_t v = col[s];
            if (comp[v] == cu || (unsigned long long)__double_as_longlong(len[s]) != target) continue;
            const uint32_t mv = inpre[v] ? n : v;
            const unsigned long long pr =
                ((unsigned long long)min(mu, mv) << 32) | (unsigned long long)max(mu, mv);
            atomicMin(&emin[cu], pr);
            atomicMax(&emax[cu], pr);
        }
    }
}

// Per live component: hook to the component across its lightest edge.
__global__ void k_bv_hook(uint32_t nc, const uint32_t* __restrict__ comp,
                          const unsigned long long* __restrict__ bw,
                          const unsigned long long* __restrict__ emin,
                          const unsigned long long* __restrict__ emax, uint32_t* __restrict__ hook,
                          unsigned long long* __restrict__ selp, uint32_t* st) {
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
        if (bw[c] == kInfKey) continue;
        const unsigned long long pr = emin[c];
        if (pr != emax[c]) st[kStTie] = 1;
        const uint32_t a = (uint32_t)(pr >> 32), b = (uint32_t)pr;
        const uint32_t ca = comp[a], cb = comp[b];
        hook[c] = ca == c ? cb : ca;
        selp[c] = pr;
    }
}

// Mutual hooks (both sides chose the same edge, the minima being strict) keep the
// smaller id as the root; every other hook records its edge once.
__global__ void k_bv_break(uint32_t nc, const unsigned long long* __restrict__ bw,
                           uint32_t* hook, const unsigned long long* __restrict__ selp,
                           unsigned long long* __restrict__ mst_pair,
                           unsigned long long* __restrict__ mst_w, uint32_t cap, uint32_t* st) {
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
        if (bw[c] == kInfKey) continue;
        const uint32_t d = hook[c];
        if (c < d && hook[d] == c) {            // only the smaller side of a pair writes
            hook[c] = c;
            continue;
        }
        const uint32_t i = atomicAdd(&st[kStEdges], 1u);
        if (i < cap) {
            mst_pair[i] = selp[c];
            mst_w[i] = bw[c];
        }
        st[kStMerged] = 1;
    }
}

// Pointer jumping on the hooks, in place (a pointer only ever moves to an ancestor).
__global__ void k_bv_jump(uint32_t nc, uint32_t* hook, uint32_t* st) {
    bool moved = false;
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
        const uint32_t h = hook[c];
        const uint32_t hh = hook[h];
        if (hh != h) {
            hook[c] = hh;
            moved = true;
        }
    }
    if (__syncthreads_or(moved) && threadIdx.x == 0) st[kStJumped] = 1;
}

__global__ void k_bv_relabel(uint32_t cnt, uint32_t* __restrict__ comp,
                             const uint32_t* __restrict__ hook) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < cnt; v += gridDim.x * blockDim.x)
        comp[v] = hook[comp[v]];
}

// ---- the tree rooted at R --------------------------------------------------------

// Tree edges of R's component; arc 2i is a -> b, arc 2i + 1 is b -> a.
__global__ void k_tree_filter(uint32_t m, const unsigned long long* __restrict__ pair,
                              const unsigned long long* __restrict__ w,
                              const uint32_t* __restrict__ comp, uint32_t rcomp,
                              unsigned long long* __restrict__ tpair,
                              unsigned long long* __restrict__ tw, uint32_t* cnt) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
        if (comp[(uint32_t)pair[i]] != rcomp) continue;
        const uint32_t j = atomicAdd(cnt, 1u);
        tpair[j] = pair[i];
        tw[j] = w[i];
    }
}

__global__ void k_edge_index(uint32_t m, uint32_t* __restrict__ idx) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x)
        idx[i] = i;
}

// Weight rank of every tree edge (its position in the sorted weights); equal
// neighbours in sorted order are a tie.
__global__ void k_weight_rank(uint32_t m, const unsigned long long* __restrict__ sk,
                              const uint32_t* __restrict__ sv, uint32_t* __restrict__ wrank,
                              uint32_t* st) {
    bool tie = false;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
        wrank[sv[i]] = i;
        if (i > 0 && sk[i] == sk[i - 1]) tie = true;
    }
    if (__syncthreads_or(tie) && threadIdx.x == 0) st[kStTie] = 1;
}

__global__ void k_arc_degree(uint32_t m, const unsigned long long* __restrict__ pair,
                             uint32_t* deg) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
        atomicAdd(&deg[(uint32_t)(pair[i] >> 32)], 1u);
        atomicAdd(&deg[(uint32_t)pair[i]], 1u);
    }
}

__global__ void k_arc_place(uint32_t m, const unsigned long long* __restrict__ pair,
                            const uint32_t* __restrict__ start, uint32_t* cursor,
                            uint32_t* __restrict__ adj, uint32_t* __restrict__ apos) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
        const uint32_t a = (uint32_t)(pair[i] >> 32), b = (uint32_t)pair[i];
        const uint32_t pa = start[a] + atomicAdd(&cursor[a], 1u);
        const uint32_t pb = start[b] + atomicAdd(&cursor[b], 1u);
        adj[pa] = 2 * i;          // a -> b
        apos[2 * i] = pa;
        adj[pb] = 2 * i + 1;      // b -> a
        apos[2 * i + 1] = pb;
    }
}

// Euler tour successor of arc x -> y: the arc after y -> x in y's list, cyclically;
// the tour starts at R's first arc and the arc leading back to it ends the list.
__global__ void k_arc_succ(uint32_t m, const unsigned long long* __restrict__ pair,
                           const uint32_t* __restrict__ start, const uint32_t* __restrict__ adj,
                           const uint32_t* __restrict__ apos, uint32_t first,
                           uint32_t* __restrict__ succ, uint32_t* __restrict__ val) {
    for (uint32_t a = blockIdx.x * blockDim.x + threadIdx.x; a < 2 * m; a += gridDim.x * blockDim.x) {
        const unsigned long long pr = pair[a >> 1];
        const uint32_t y = (a & 1) ? (uint32_t)(pr >> 32) : (uint32_t)pr;   // the arc's head
        const uint32_t p = apos[a ^ 1];
        const uint32_t q = p + 1 < start[y + 1] ? p + 1 : start[y];
        const uint32_t s = adj[q];
        succ[a] = s == first ? kEnd : s;
        val[a] = 1;
    }
}

// One list-ranking round: every entry adds its successor's value and jumps over it.
__global__ void k_list_rank(uint32_t cnt, const uint32_t* __restrict__ s0,
                            const uint32_t* __restrict__ v0, uint32_t* __restrict__ s1,
                            uint32_t* __restrict__ v1) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x) {
        const uint32_t s = s0[i];
        if (s == kEnd) {
            s1[i] = kEnd;
            v1[i] = v0[i];
        } else {
            s1[i] = s0[s];
            v1[i] = v0[i] + v0[s];
        }
    }
}

// Parent and weight rank of every tree vertex: an edge's earlier arc in the tour (more
// arcs after it) runs from the parent to the child.  wr[R] is the largest rank.
__global__ void k_tree_parent(uint32_t m, const unsigned long long* __restrict__ pair,
                              const uint32_t* __restrict__ after, const uint32_t* __restrict__ wrank,
                              uint32_t* __restrict__ parent, uint32_t* __restrict__ wr) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
        const uint32_t a = (uint32_t)(pair[i] >> 32), b = (uint32_t)pair[i];
        const bool a_up = after[2 * i] > after[2 * i + 1];
        const uint32_t child = a_up ? b : a;
        parent[child] = a_up ? a : b;
        wr[child] = wrank[i];
    }
}

// Binary lifting level 0: up = parent, mx = weight rank of the parent.
__global__ void k_lift0(uint32_t cnt, const uint32_t* __restrict__ parent,
                        const uint32_t* __restrict__ wr, uint32_t* __restrict__ up,
                        uint32_t* __restrict__ mx) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < cnt; v += gridDim.x * blockDim.x) {
        const uint32_t p = parent[v];
        up[v] = p;
        mx[v] = wr[p];
    }
}

__global__ void k_lift(uint32_t cnt, const uint32_t* __restrict__ up0,
                       const uint32_t* __restrict__ mx0, uint32_t* __restrict__ up1,
                       uint32_t* __restrict__ mx1) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < cnt; v += gridDim.x * blockDim.x) {
        const uint32_t u = up0[v];
        up1[v] = up0[u];
        mx1[v] = max(mx0[v], mx0[u]);
    }
}

// nga(v): jump while the next 2^j ancestors are all lighter than v's own edge.
__global__ void k_nga(uint32_t n, const uint32_t* __restrict__ intree,
                      const uint32_t* __restrict__ wr, const uint32_t* __restrict__ up,
                      const uint32_t* __restrict__ mx, uint32_t levels, uint64_t stride,
                      uint32_t* __restrict__ nga, uint32_t* __restrict__ items, uint32_t* cnt) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        if (!intree[v]) continue;
        const uint32_t w = wr[v];
        uint32_t cur = v;
        for (int j = (int)levels - 1; j >= 0; --j)
            if (mx[j * stride + cur] < w) cur = up[j * stride + cur];
        nga[v] = up[cur];
        items[atomicAdd(cnt, 1u)] = v;
    }
}

__global__ void k_sort_keys(uint32_t cnt, const uint32_t* __restrict__ items,
                            const uint32_t* __restrict__ nga, const uint32_t* __restrict__ wr,
                            unsigned long long* __restrict__ key) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x) {
        const uint32_t v = items[i];
        key[i] = ((unsigned long long)nga[v] << 32) | wr[v];
    }
}

// First child and next sibling in the forest v -> nga(v), children by weight rank.
__global__ void k_children(uint32_t cnt, const unsigned long long* __restrict__ key,
                           const uint32_t* __restrict__ sv, uint32_t* __restrict__ fc,
                           uint32_t* __restrict__ ns) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x) {
        const uint32_t p = (uint32_t)(key[i] >> 32);
        if (i == 0 || (uint32_t)(key[i - 1] >> 32) != p) fc[p] = sv[i];
        ns[sv[i]] = (i + 1 < cnt && (uint32_t)(key[i + 1] >> 32) == p) ? sv[i + 1] : kEnd;
    }
}

// Pre-order tour of that forest: down(v) = v, up(v) = n + 1 + v; only down arcs count.
__global__ void k_forest_succ(uint32_t n, const uint32_t* __restrict__ intree,
                              const uint32_t* __restrict__ fc, const uint32_t* __restrict__ ns,
                              const uint32_t* __restrict__ nga, uint32_t* __restrict__ succ,
                              uint32_t* __restrict__ val) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v <= n; v += gridDim.x * blockDim.x) {
        const uint32_t up = n + 1 + v;
        if (v == n || !intree[v]) {
            succ[v] = succ[up] = kEnd;
            val[v] = val[up] = 0;
            continue;
        }
        succ[v] = fc[v] != kEnd ? fc[v] : up;
        val[v] = 1;
        succ[up] = ns[v] != kEnd ? ns[v] : (nga[v] == n ? kEnd : n + 1 + nga[v]);
        val[up] = 0;
    }
}

__global__ void k_ranks(uint32_t n, const uint32_t* __restrict__ intree,
                        const uint32_t* __restrict__ after, uint32_t total, uint32_t k,
                        uint32_t* __restrict__ rank) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
        if (intree[v]) rank[v] = k + (total - after[v]);
}

__global__ void k_prefix_ranks(uint32_t k, const uint32_t* __restrict__ prefix,
                               uint32_t* __restrict__ rank) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < k) rank[prefix[i]] = i;
}

__global__ void k_in_tree(uint32_t n, const uint32_t* __restrict__ comp, uint32_t rcomp,
                          const uint8_t* __restrict__ inpre, uint32_t* __restrict__ intree) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
        intree[v] = (comp[v] == rcomp && !inpre[v]) ? 1u : 0u;
}

__global__ void k_site_of_rank(uint32_t n, const uint32_t* __restrict__ rank,
                               uint32_t* __restrict__ sor) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
        if (rank[v] < n) sor[rank[v]] = v;
}

__global__ void k_fill_u32(uint32_t cnt, uint32_t* __restrict__ a, uint32_t v) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x)
        a[i] = v;
}

// Stream-ordered scratch, released when the computation returns.
struct Scratch {
    cudaStream_t st;
    std::vector<void*> bufs;
    cudaError_t err = cudaSuccess;
    explicit Scratch(cudaStream_t s) : st(s) {}
    template <class T>
    T* get(uint64_t count) {
        void* p = nullptr;
        if (err != cudaSuccess) return nullptr;
        err = cudaMallocAsync(&p, std::max<uint64_t>(1, count) * sizeof(T), st);
        if (err != cudaSuccess) return nullptr;
        bufs.push_back(p);
        return (T*)p;
    }
    ~Scratch() {
        for (void* p : bufs) cudaFreeAsync(p, st);
    }
};

}  // namespace

#define LR_CU(x)                                \
    do {                                        \
        cudaError_t e_ = (x);                   \
        if (e_ != cudaSuccess) {                \
            info->error = e_;                   \
            return kRankError;                  \
        }                                       \
    } while (0)
#define LR_OK(ptr)                              \
    do {                                        \
        if (!(ptr)) {                           \
            info->error = sc.err;               \
            return kRankError;                  \
        }                                       \
    } while (0)

RankResult gpu_lake_rank(cudaStream_t st, uint32_t n, const uint32_t* row, const uint32_t* col,
                         const double* len, uint64_t nnz, const std::vector<uint32_t>& prefix,
                         uint32_t* rank, uint32_t* sor, GpuRankInfo* info) {
    *info = GpuRankInfo{};
    Scratch sc(st);
    const uint32_t nc = n + 1;                     // vertex ids and R = n
    const uint32_t k = (uint32_t)prefix.size();
    uint32_t* d_st = sc.get<uint32_t>(kStCount);
    uint32_t* comp = sc.get<uint32_t>(nc);
    uint32_t* hook = sc.get<uint32_t>(nc);
    uint8_t* inpre = sc.get<uint8_t>(nc);
    unsigned long long* bw = sc.get<unsigned long long>(nc);
    unsigned long long* emin = sc.get<unsigned long long>(nc);
    unsigned long long* emax = sc.get<unsigned long long>(nc);
    unsigned long long* selp = sc.get<unsigned long long>(nc);
    unsigned long long* mst_pair = sc.get<unsigned long long>(nc);
    unsigned long long* mst_w = sc.get<unsigned long long>(nc);
    uint32_t* d_prefix = sc.get<uint32_t>(k);
    LR_OK(d_prefix);
    uint32_t h[kStCount];
    auto read_status = [&]() -> cudaError_t {
        cudaError_t e = cudaMemcpyAsync(h, d_st, sizeof h, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        info->host_syncs++;
        return e;
    };
    LR_CU(cudaMemsetAsync(d_st, 0, kStCount * sizeof(uint32_t), st));
    LR_CU(cudaMemsetAsync(inpre, 0, nc, st));
    if (k) LR_CU(cudaMemcpyAsync(d_prefix, prefix.data(), k * 4ull, cudaMemcpyHostToDevice, st));
    k_check_len<<<grid_for(nnz), 256, 0, st>>>(nnz, len, d_st);
    k_iota<<<grid_for(nc), 256, 0, st>>>(nc, comp);
    if (k) k_mark_prefix<<<grid_for(k), 256, 0, st>>>(k, d_prefix, n, comp, inpre);
    LR_CU(cudaGetLastError());

    // 1. Boruvka rounds
    uint32_t rounds = 0;
    for (;; ++rounds) {
        if (rounds > 64) {
            info->error = cudaErrorUnknown;
            return kRankError;
        }
        LR_CU(cudaMemsetAsync(d_st + kStMerged, 0, sizeof(uint32_t), st));
        k_bv_reset<<<grid_for(nc), 256, 0, st>>>(nc, bw, emin, emax, hook);
        k_bv_minw<<<grid_for(n), 256, 0, st>>>(n, row, col, len, comp, bw);
        k_bv_mine<<<grid_for(n), 256, 0, st>>>(n, row, col, len, comp, inpre, bw, emin, emax);
        k_bv_hook<<<grid_for(nc), 256, 0, st>>>(nc, comp, bw, emin, emax, hook, selp, d_st);
        k_bv_break<<<grid_for(nc), 256, 0, st>>>(nc, bw, hook, selp, mst_pair, mst_w, nc, d_st);
        LR_CU(cudaGetLastError());
        LR_CU(read_status());
        if (h[kStBadLen] || h[kStTie]) {
            info->fallback_reason = h[kStBadLen] ? "an edge length is not positive"
                                                 : "equal lengths compete in the traversal";
            return kRankFallback;
        }
        if (!h[kStMerged]) break;
        for (int jr = 0;; ++jr) {                  // flatten the hook forest
            if (jr > 64) {
                info->error = cudaErrorUnknown;
                return kRankError;
            }
            LR_CU(cudaMemsetAsync(d_st + kStJumped, 0, sizeof(uint32_t), st));
            for (int rep = 0; rep < 4; ++rep) k_bv_jump<<<grid_for(nc), 256, 0, st>>>(nc, hook, d_st);
            LR_CU(cudaGetLastError());
            LR_CU(read_status());
            if (!h[kStJumped]) break;
        }
        k_bv_relabel<<<grid_for(nc), 256, 0, st>>>(nc, comp, hook);
        LR_CU(cudaGetLastError());
    }
    info->boruvka_rounds = rounds;
    const uint32_t medges = std::min(h[kStEdges], nc);
    uint32_t rcomp = 0;
    LR_CU(cudaMemcpyAsync(&rcomp, comp + n, 4, cudaMemcpyDeviceToHost, st));

    // R's tree
    unsigned long long* tpair = sc.get<unsigned long long>(medges);
    unsigned long long* tw = sc.get<unsigned long long>(medges);
    uint32_t* d_cnt = sc.get<uint32_t>(4);
    LR_OK(d_cnt);
    LR_CU(cudaMemsetAsync(d_cnt, 0, 4 * sizeof(uint32_t), st));
    LR_CU(cudaStreamSynchronize(st));
    info->host_syncs++;
    if (medges)
        k_tree_filter<<<grid_for(medges), 256, 0, st>>>(medges, mst_pair, mst_w, comp, rcomp, tpair,
                                                        tw, d_cnt);
    LR_CU(cudaGetLastError());
    uint32_t m = 0;
    LR_CU(cudaMemcpyAsync(&m, d_cnt, 4, cudaMemcpyDeviceToHost, st));
    LR_CU(cudaStreamSynchronize(st));
    info->host_syncs++;
    info->tree_edges = m;

    // ranks: prefix, then the keyed order; everything else never processed
    k_fill_u32<<<grid_for(n), 256, 0, st>>>(n, rank, kEnd);
    k_fill_u32<<<grid_for(n), 256, 0, st>>>(n, sor, kEnd);
    if (k) k_prefix_ranks<<<grid_for(k), 256, 0, st>>>(k, d_prefix, rank);
    LR_CU(cudaGetLastError());
    if (m == 0) {
        k_site_of_rank<<<grid_for(n), 256, 0, st>>>(n, rank, sor);
        LR_CU(cudaGetLastError());
        return kRankOk;
    }

    // 2a. weight ranks (and distinct weights)
    uint32_t* eidx = sc.get<uint32_t>(m);
    uint32_t* sidx = sc.get<uint32_t>(m);
    unsigned long long* skey = sc.get<unsigned long long>(m);
    uint32_t* wrank = sc.get<uint32_t>(m);
    LR_OK(wrank);
    k_edge_index<<<grid_for(m), 256, 0, st>>>(m, eidx);
    size_t tmp_bytes = 0, tb = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, tb, tw, skey, eidx, sidx, (int)m, 0, 64, st);
    tmp_bytes = std::max(tmp_bytes, tb);
    cub::DeviceRadixSort::SortPairs(nullptr, tb, (unsigned long long*)nullptr,
                                    (unsigned long long*)nullptr, (uint32_t*)nullptr,
                                    (uint32_t*)nullptr, (int)n, 0, 64, st);
    tmp_bytes = std::max(tmp_bytes, tb);
    cub::DeviceScan::ExclusiveSum(nullptr, tb, (uint32_t*)nullptr, (uint32_t*)nullptr, (int)nc + 1, st);
    tmp_bytes = std::max(tmp_bytes, tb);
    void* tmp = sc.get<uint8_t>(tmp_bytes);
    LR_OK(tmp);
    tb = tmp_bytes;
    LR_CU(cub::DeviceRadixSort::SortPairs(tmp, tb, tw, skey, eidx, sidx, (int)m, 0, 64, st));
    k_weight_rank<<<grid_for(m), 256, 0, st>>>(m, skey, sidx, wrank, d_st);
    LR_CU(cudaGetLastError());

    // 2b. Euler tour of the tree from R; list ranking
    uint32_t* deg = sc.get<uint32_t>(nc + 1);
    uint32_t* start = sc.get<uint32_t>(nc + 1);
    uint32_t* cursor = sc.get<uint32_t>(nc);
    uint32_t* adj = sc.get<uint32_t>(2ull * m);
    uint32_t* apos = sc.get<uint32_t>(2ull * m);
    const uint64_t L2 = std::max<uint64_t>(2ull * m, 2ull * nc);   // both tours' lists
    uint32_t* s0 = sc.get<uint32_t>(L2);
    uint32_t* v0 = sc.get<uint32_t>(L2);
    uint32_t* s1 = sc.get<uint32_t>(L2);
    uint32_t* v1 = sc.get<uint32_t>(L2);
    LR_OK(v1);
    LR_CU(cudaMemsetAsync(deg, 0, (nc + 1) * 4ull, st));
    LR_CU(cudaMemsetAsync(cursor, 0, nc * 4ull, st));
    k_arc_degree<<<grid_for(m), 256, 0, st>>>(m, tpair, deg);
    tb = tmp_bytes;
    LR_CU(cub::DeviceScan::ExclusiveSum(tmp, tb, deg, start, (int)nc + 1, st));
    k_arc_place<<<grid_for(m), 256, 0, st>>>(m, tpair, start, cursor, adj, apos);
    uint32_t first_pos = 0, first = 0;
    LR_CU(cudaMemcpyAsync(&first_pos, start + n, 4, cudaMemcpyDeviceToHost, st));
    LR_CU(cudaStreamSynchronize(st));
    info->host_syncs++;
    LR_CU(cudaMemcpyAsync(&first, adj + first_pos, 4, cudaMemcpyDeviceToHost, st));
    LR_CU(cudaStreamSynchronize(st));
    info->host_syncs++;
    k_arc_succ<<<grid_for(2ull * m), 256, 0, st>>>(m, tpair, start, adj, apos, first, s0, v0);
    LR_CU(cudaGetLastError());
    auto list_rank = [&](uint32_t cnt) -> uint32_t* {
        int r = 1;
        while ((1ull << r) < (uint64_t)cnt + 1) ++r;
        uint32_t *sa = s0, *va = v0, *sb = s1, *vb = v1;
        for (int i = 0; i <= r; ++i) {
            k_list_rank<<<grid_for(cnt), 256, 0, st>>>(cnt, sa, va, sb, vb);
            std::swap(sa, sb);
            std::swap(va, vb);
        }
        return va;                                    // arcs from each entry to the end
    };
    uint32_t* after1 = list_rank(2 * m);
    uint32_t* parent = sc.get<uint32_t>(nc);
    uint32_t* wr = sc.get<uint32_t>(nc);
    LR_OK(wr);
    k_iota<<<grid_for(nc), 256, 0, st>>>(nc, parent);   // R and sites outside: themselves
    k_fill_u32<<<grid_for(nc), 256, 0, st>>>(nc, wr, kEnd);
    k_tree_parent<<<grid_for(m), 256, 0, st>>>(m, tpair, after1, wrank, parent, wr);
    LR_CU(cudaGetLastError());

    // 3. binary lifting and nga
    uint32_t levels = 1;
    while ((1ull << levels) < (uint64_t)m + 1) ++levels;
    ++levels;
    uint32_t* up = sc.get<uint32_t>((uint64_t)levels * nc);
    uint32_t* mx = sc.get<uint32_t>((uint64_t)levels * nc);
    uint32_t* intree = sc.get<uint32_t>(nc);
    uint32_t* nga = sc.get<uint32_t>(nc);
    uint32_t* items = sc.get<uint32_t>(nc);
    LR_OK(items);
    info->lift_levels = levels;
    k_lift0<<<grid_for(nc), 256, 0, st>>>(nc, parent, wr, up, mx);
    for (uint32_t j = 0; j + 1 < levels; ++j)
        k_lift<<<grid_for(nc), 256, 0, st>>>(nc, up + (uint64_t)j * nc, mx + (uint64_t)j * nc,
                                             up + (uint64_t)(j + 1) * nc, mx + (uint64_t)(j + 1) * nc);
    k_in_tree<<<grid_for(n), 256, 0, st>>>(n, comp, rcomp, inpre, intree);
    LR_CU(cudaMemsetAsync(intree + n, 0, 4, st));
    LR_CU(cudaMemsetAsync(d_cnt, 0, 4, st));
    k_nga<<<grid_for(n), 256, 0, st>>>(n, intree, wr, up, mx, levels, nc, nga, items, d_cnt);
    LR_CU(cudaGetLastError());
    uint32_t cnt = 0;
    LR_CU(cudaMemcpyAsync(&cnt, d_cnt, 4, cudaMemcpyDeviceToHost, st));
    LR_CU(cudaMemcpyAsync(h, d_st, sizeof h, cudaMemcpyDeviceToHost, st));
    LR_CU(cudaStreamSynchronize(st));
    info->host_syncs++;
    if (h[kStTie]) {
        info->fallback_reason = "equal lengths in the spanning tree";
        return kRankFallback;
    }
    if (cnt != m) {                                 // every tree edge has one child vertex
        info->error = cudaErrorUnknown;
        return kRankError;
    }

    // 4. pre-order of the forest v -> nga(v), children by weight
    unsigned long long* key = sc.get<unsigned long long>(cnt);
    unsigned long long* skey2 = sc.get<unsigned long long>(cnt);
    uint32_t* sv = sc.get<uint32_t>(cnt);
    uint32_t* fc = sc.get<uint32_t>(nc);
    uint32_t* ns = sc.get<uint32_t>(nc);
    LR_OK(ns);
    k_sort_keys<<<grid_for(cnt), 256, 0, st>>>(cnt, items, nga, wr, key);
    tb = tmp_bytes;
    LR_CU(cub::DeviceRadixSort::SortPairs(tmp, tb, key, skey2, items, sv, (int)cnt, 0, 64, st));
    k_fill_u32<<<grid_for(nc), 256, 0, st>>>(nc, fc, kEnd);
    k_children<<<grid_for(cnt), 256, 0, st>>>(cnt, skey2, sv, fc, ns);
    k_forest_succ<<<grid_for(nc), 256, 0, st>>>(n, intree, fc, ns, nga, s0, v0);
    LR_CU(cudaGetLastError());
    uint32_t* after2 = list_rank(2 * nc);
    k_ranks<<<grid_for(n), 256, 0, st>>>(n, intree, after2, cnt, k, rank);
    k_site_of_rank<<<grid_for(n), 256, 0, st>>>(n, rank, sor);
    LR_CU(cudaGetLastError());
    return kRankOk;
}

}  // namespace fl
