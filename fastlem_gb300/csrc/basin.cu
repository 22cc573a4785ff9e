// basin.cu -- drainage area, response time and elevation over the receiver forest
// (src/lem/generator.rs:144-203, src/lem/drainage_basin.rs:13-46), bit-exact.
//
// The reference walks each outlet's basin breadth-first: drainage areas in reversed
// BFS order (a site's donors are added in reverse adjacency order), then response
// times and elevations in BFS order (parent before child).  Both are exact f64
// recurrences along the river paths, and river paths are long: on the 16M-site
// terrain the forest is ~24,000 levels deep with a few hundred sites per level, so
// level-by-level processing is launch- and latency-bound.  The passes here are:
//
//  1. Kahn rounds (bottom-up, one cooperative kernel, grid barrier per round).
//     Round r processes the sites of height r (all donors done): each pulls its
//     donors' areas walking its adjacency row backwards, which reproduces the
//     reference's addition order exactly.  Rounds stop once the ready frontier is
//     narrower than `kahn_min_width`; what is left -- the skeleton -- is the deep
//     trunk part of the rivers, a small fraction of the sites.
//  2. Skeleton chains.  Every skeleton site with skeleton donors designates one of
//     them (largest previous drainage area, i.e. the likely main stem) to continue
//     its chain, so the skeleton splits into chains, one per skeleton leaf.  The
//     chains are ranked by pointer jumping over the skeleton only and laid out
//     contiguously; per site, the part of the pull that does not involve the chain
//     predecessor is precomputed in parallel.
//  3. Skeleton bottom-up: one thread per chain walks it from its leaf to its bottom
//     doing only the dependent additions; a chain that reaches a confluence waits
//     (bounded acquire/release flags) for the other chain's bottom.  All chains are
//     co-resident, so the waits always end.
//  4. w_v = (1 / (k_v * sqrt(A_v))) * len_v for all sites, in parallel.
//  5. Skeleton top-down: the same chains from bottom to leaf, t_v = t_parent + w_v,
//     elevation and slope clamp; a chain starts once its parent site is published.
//  6. Remaining sites top-down by Kahn round, highest first (a site's receiver is
//     higher, so it is done earlier).
// Sites in components without an outlet are computed but never receive an
// elevation, as in the reference (they are in no basin).

#include <algorithm>

#include "common.cuh"
#include "fold.cuh"
#include "kernels.h"

namespace fl {
namespace {

// per-slot flags of the skeleton layout (SlotInfo::flags)
constexpr uint32_t kLeafSlot = 1;  // chain leaf: pre holds the complete area
constexpr uint32_t kTok = 2;       // donor list in tokval (a confluence with another chain's
                                   // bottom, or more than kMaxPost additions after the
                                   // predecessor)
constexpr uint32_t kSlow = 4;      // donor list too long: full pull at walk time
constexpr int kPostShift = 3;      // bits 3-4: additions after the chain predecessor
constexpr uint32_t kPend = 32;     // confluence whose operands (pre, posts) the last chain
                                   // bottom to arrive computes from the donor list
constexpr int kMaxPost = 3;
constexpr int kTokCntShift = 8;    // bits 8-11: donor-list length (cell area first)
constexpr int kHeavyShift = 12;    // bits 12-15: the predecessor's index in the list
constexpr int kMaxTok = 15;
// A chain bottom's area not pushed yet (a signalling NaN: never an arithmetic result,
// and pushed NaNs are quieted).
constexpr uint64_t kPendingBits = 0x7ff4000000000000ull;

// Rows up to this many slots are gathered with all loads in flight at once; longer
// rows (rare: hull sites) take the plain loop.
constexpr int kRowFast = 12;

// The reference's drainage area of v given final donor areas: a_v + donors in
// reverse adjacency order (generator.rs:154-159).  Column ids, then receivers,
// then donor areas are each loaded together, so a row costs three memory latencies
// rather than three per slot.
__device__ __forceinline__ double pull_area(uint32_t v, const uint32_t* __restrict__ row,
                                            const uint32_t* __restrict__ col,
                                            const uint32_t* __restrict__ next,
                                            const double* __restrict__ area, const double* A) {
    const uint32_t s0 = row[v], s1 = row[v + 1];
    double a = area[v];
    const uint32_t deg = s1 - s0;
    if (deg <= (uint32_t)kRowFast) {
        uint32_t d[kRowFast];
        bool don[kRowFast];
        double val[kRowFast];
#pragma unroll
        for (int k = 0; k < kRowFast; ++k)
            if ((uint32_t)k < deg) d[k] = col[s0 + k];
#pragma unroll
        for (int k = 0; k < kRowFast; ++k)
            don[k] = (uint32_t)k < deg && d[k] != v && next[d[k]] == v;
#pragma unroll
        for (int k = 0; k < kRowFast; ++k)
            if (don[k]) val[k] = __ldcg(&A[d[k]]);
#pragma unroll
        for (int k = kRowFast - 1; k >= 0; --k)
            if (don[k]) a = __dadd_rn(a, val[k]);
        return a;
    }
    for (uint32_t s = s1; s-- > s0;) {
        uint32_t dd = col[s];
        if (dd != v && next[dd] == v) a = __dadd_rn(a, __ldcg(&A[dd]));
    }
    return a;
}

// Packed terrains: a terrain whose first unchanged iteration is recorded sits at its
// fixed point; another pass over it would reproduce its values, so its sites take no
// part in the basin pass (they stay out of the leaves, the rounds and the skeleton,
// and keep their areas, records and elevations).
__device__ __forceinline__ bool settled(const uint32_t* tid, const uint32_t* titer, uint32_t v) {
    return tid && titer[tid[v]] != 0;
}

__global__ void k_count_donors(uint32_t n, const uint32_t* __restrict__ next,
                               uint32_t* __restrict__ pending, const uint32_t* __restrict__ tid,
                               const uint32_t* __restrict__ titer) {
    uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n || settled(tid, titer, v)) return;
    uint32_t p = next[v];
    if (p != v) atomicAdd(&pending[p], 1u);
}

// Leaves in site order per block range (one reservation per block).
__global__ void k_collect_leaves(uint32_t n, const uint32_t* __restrict__ pending,
                                 uint32_t* __restrict__ order, uint32_t* __restrict__ counter,
                                 const uint32_t* __restrict__ tid, const uint32_t* __restrict__ titer) {
    block_range_compact(
        n, counter, [&](uint32_t v) { return pending[v] == 0 && !settled(tid, titer, v); },
        [&](uint32_t v, uint32_t pos) { order[pos] = v; });
}

// Kahn rounds.  order[0, nleaves) holds the leaves; rounds append the next frontier
// after the current one.  Writes hgt (round) and A of processed sites, the round
// offsets roff[0..r_stop+1] and meta[kMetaRStop] = r_stop.
__global__ void k_kahn(uint32_t n, const uint32_t* __restrict__ row,
                       const uint32_t* __restrict__ col, const uint32_t* __restrict__ next,
                       const double* __restrict__ area, double* A, uint32_t* pending,
                       uint32_t* __restrict__ hgt, uint32_t* order, uint32_t* roff,
                       uint64_t* __restrict__ rtime, uint32_t max_rounds, uint32_t min_width,
                       uint32_t* meta, int* flags) {
    const uint32_t gtid = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t stride = gridDim.x * blockDim.x;
    uint32_t beg = 0, end = ld_acquire_u(&meta[kMetaLeaves]);
    uint32_t r = 0;
    if (gtid == 0) {
        roff[0] = 0;
        roff[1] = end;
    }
    while (true) {
        if (gtid == 0) rtime[r] = global_ns();
        uint32_t width = end - beg;
        if (width == 0 || width < min_width || r + 2 >= max_rounds) break;
        uint32_t* cnt = &meta[kMetaCnt0 + (r % 3)];
        if (gtid == 0) meta[kMetaCnt0 + ((r + 1) % 3)] = 0;
        // block-uniform trip count: block_append synchronises the block
        for (uint32_t tile = beg + blockIdx.x * blockDim.x; tile < end; tile += stride) {
            const uint32_t idx = tile + threadIdx.x;
            bool ready = false;
            uint32_t p = 0;
            if (idx < end) {
                uint32_t v = __ldcg(&order[idx]);
                // round 0 is the leaves: no donors, the drainage area is the cell area
                A[v] = (r == 0) ? area[v] : pull_area(v, row, col, next, area, A);
                hgt[v] = r;
                p = next[v];
                ready = p != v && atomicSub(&pending[p], 1u) == 1u;
            }
            uint32_t pos = block_append(cnt, ready);
            if (pos != kNone) {
                pos += end;
                if (pos < n) order[pos] = p;
                else set_error(flags, kErrForest);
            }
        }
        if (!grid_barrier(flags)) return;
        beg = end;
        end = end + ld_acquire_u(cnt);
        ++r;
        if (gtid == 0) roff[r + 1] = end;
    }
    if (gtid == 0) {
        meta[kMetaRStop] = r;
        meta[kMetaFrontBeg] = beg;
        meta[kMetaFrontEnd] = end;
    }
}

// ---- skeleton --------------------------------------------------------------------

// The pointer-jumping result sits in ping-pong buffer meta[kMetaRankBuf].
struct Ranks {
    const uint32_t* ptr[2];
    const uint32_t* dist[2];
    __device__ __forceinline__ const uint32_t* P(const uint32_t* meta) const { return ptr[meta[kMetaRankBuf]]; }
    __device__ __forceinline__ const uint32_t* D(const uint32_t* meta) const { return dist[meta[kMetaRankBuf]]; }
};

__global__ void k_s_collect(uint32_t n, const uint32_t* __restrict__ hgt,
                            uint32_t* __restrict__ sid, uint32_t* __restrict__ slist,
                            uint32_t* meta, const uint32_t* __restrict__ tid,
                            const uint32_t* __restrict__ titer) {
    block_range_compact(
        n, &meta[kMetaNs], [&](uint32_t v) { return hgt[v] == kNone && !settled(tid, titer, v); },
        [&](uint32_t v, uint32_t k) {
            sid[v] = k;
            slist[k] = v;
        });
}

// For skeleton site p: the skeleton donor that continues p's chain (largest
// previous drainage area, first in row order on ties), or none.
__global__ void k_s_designate(const uint32_t* __restrict__ row, const uint32_t* __restrict__ col,
                              const uint32_t* __restrict__ next, const uint32_t* __restrict__ hgt,
                              const double* __restrict__ A, const uint32_t* __restrict__ slist,
                              uint32_t* __restrict__ desig, const uint32_t* meta) {
    uint32_t ns = meta[kMetaNs];
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < ns; k += gridDim.x * blockDim.x) {
        uint32_t p = slist[k];
        uint32_t best = kNone;
        double ba = 0.0;
        const uint32_t s0 = row[p], s1 = row[p + 1];
        if (s1 - s0 <= (uint32_t)kRowFast) {
            // columns, receivers, then the donors' heights and areas: a phase at a time
            const uint32_t deg = s1 - s0;
            uint32_t dd[kRowFast], donm = 0, skelm = 0;
            double av[kRowFast];
#pragma unroll
            for (int j = 0; j < kRowFast; ++j)
                if ((uint32_t)j < deg) dd[j] = col[s0 + j];
#pragma unroll
            for (int j = 0; j < kRowFast; ++j)
                if ((uint32_t)j < deg && dd[j] != p && next[dd[j]] == p) donm |= 1u << j;
#pragma unroll
            for (int j = 0; j < kRowFast; ++j)
                if ((donm >> j) & 1u) {
                    if (hgt[dd[j]] == kNone) skelm |= 1u << j;
                    av[j] = A[dd[j]];
                }
#pragma unroll
            for (int j = 0; j < kRowFast; ++j)
                if ((skelm >> j) & 1u && (best == kNone || av[j] > ba)) {
                    best = dd[j];
                    ba = av[j];
                }
        } else {
            for (uint32_t s = s0; s < s1; ++s) {
                uint32_t d = col[s];
                if (d == p || next[d] != p || hgt[d] != kNone) continue;
                double a = A[d];
                if (best == kNone || a > ba) {
                    best = d;
                    ba = a;
                }
            }
        }
        desig[p] = best;
    }
}

// Chain successor (toward the root) in skeleton-index space, for pointer jumping.
__global__ void k_s_link(const uint32_t* __restrict__ next, const uint32_t* __restrict__ desig,
                         const uint32_t* __restrict__ hgt, const uint32_t* __restrict__ sid,
                         const uint32_t* __restrict__ slist, uint32_t* __restrict__ ptr,
                         uint32_t* __restrict__ dist, const uint32_t* meta) {
    uint32_t ns = meta[kMetaNs];
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < ns; k += gridDim.x * blockDim.x) {
        uint32_t v = slist[k];
        uint32_t p = next[v];
        // a skeleton site's receiver is a skeleton site; desig is only written there
        bool cont = (p != v) && hgt[p] == kNone && desig[p] == v;
        ptr[k] = cont ? sid[p] : k;
        dist[k] = cont ? 1u : 0u;
    }
}

// Pointer jumping to the chain bottom: dist = sites below on the chain.
__global__ void k_s_rank(uint32_t* ptr0, uint32_t* dist0, uint32_t* ptr1, uint32_t* dist1,
                         uint32_t* meta, int* flags) {
    const uint32_t ns = meta[kMetaNs];
    const uint32_t gtid = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t stride = gridDim.x * blockDim.x;
    uint32_t* P[2] = {ptr0, ptr1};
    uint32_t* D[2] = {dist0, dist1};
    int cur = 0;
    for (uint32_t round = 0; round < 64; ++round) {
        uint32_t* jf = &meta[kMetaJump0 + (round % 3)];
        if (gtid == 0) meta[kMetaJump0 + ((round + 1) % 3)] = 0;
        bool changed = false;
        for (uint32_t k = gtid; k < ns; k += stride) {
            uint32_t p = __ldcg(&P[cur][k]);
            uint32_t pp = __ldcg(&P[cur][p]);
            D[cur ^ 1][k] = __ldcg(&D[cur][k]) + (p != k ? __ldcg(&D[cur][p]) : 0u);
            P[cur ^ 1][k] = pp;
            changed |= (pp != p);
        }
        if (__syncthreads_or(changed) && threadIdx.x == 0) atomicOr(jf, 1u);
        if (!grid_barrier(flags)) return;
        cur ^= 1;
        if (ld_acquire_u(jf) == 0) {
            if (gtid == 0) meta[kMetaRankBuf] = cur;
            return;
        }
    }
    set_error(flags, kErrForest);
}

// Chain ids for chain bottoms.
// Chain ids for the chain bottoms (skeleton sites that point at themselves after the
// ranking), in skeleton order, one reservation per block.
__global__ void k_s_bottoms(const uint32_t* __restrict__ slist, Ranks rk,
                            uint32_t* __restrict__ cid, uint32_t* __restrict__ cbot,
                            uint32_t max_chains, uint32_t* meta, int* flags) {
    const uint32_t ns = meta[kMetaNs];
    const uint32_t* ptr = rk.P(meta);
    block_range_compact(
        ns, &meta[kMetaChains], [&](uint32_t k) { return ptr[k] == k; },
        [&](uint32_t k, uint32_t c) {
            if (c < max_chains) {
                cid[k] = c;
                cbot[c] = slist[k];
            } else {
                set_error(flags, kErrCapacity);
            }
        });
}

// Chain lengths from the skeleton leaves (the final Kahn frontier).
__global__ void k_s_lengths(const uint32_t* __restrict__ order, const uint32_t* __restrict__ sid,
                            Ranks rk, const uint32_t* __restrict__ cid, uint32_t* __restrict__ clen,
                            uint32_t max_chains, uint32_t* meta, const int* flags) {
    if (flags[kError]) return;
    uint32_t b = meta[kMetaFrontBeg], e = meta[kMetaFrontEnd];
    const uint32_t* ptr = rk.P(meta);
    const uint32_t* dist = rk.D(meta);
    for (uint32_t base = b + blockIdx.x * blockDim.x; base < e; base += gridDim.x * blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        uint32_t l = 0;
        if (i < e) {
            uint32_t k = sid[order[i]];
            uint32_t c = cid[ptr[k]];
            l = dist[k] + 1;
            if (c < max_chains) clen[c] = l;
        }
        l = __reduce_max_sync(0xffffffffu, l);      // one atomic per warp
        if ((threadIdx.x & 31) == 0 && l) atomicMax(&meta[kMetaMaxChain], l);
    }
}

// Exclusive scan of chain lengths (single block).
__global__ void k_s_scan(const uint32_t* __restrict__ clen, uint32_t* __restrict__ coff,
                         const uint32_t* meta, const int* flags) {
    __shared__ uint32_t part[1024];
    if (flags[kError]) return;
    uint32_t nc = meta[kMetaChains];
    uint32_t per = (nc + blockDim.x - 1) / blockDim.x;
    uint32_t b = threadIdx.x * per, e = min(nc, b + per);
    uint32_t s = 0;
    for (uint32_t i = b; i < e; ++i) s += clen[i];
    part[threadIdx.x] = s;
    __syncthreads();
    for (uint32_t off = 1; off < blockDim.x; off <<= 1) {
        uint32_t v = threadIdx.x >= off ? part[threadIdx.x - off] : 0;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    uint32_t run = part[threadIdx.x] - s;
    for (uint32_t i = b; i < e; ++i) {
        coff[i] = run;
        run += clen[i];
    }
}

__global__ void k_s_layout(const uint32_t* __restrict__ slist, Ranks rk,
                           const uint32_t* __restrict__ cid, const uint32_t* __restrict__ coff,
                           uint32_t* __restrict__ layout, uint32_t* __restrict__ slot_chain,
                           uint32_t* __restrict__ kslot, const uint32_t* meta, int* flags) {
    if (flags[kError]) return;
    uint32_t ns = meta[kMetaNs];
    const uint32_t* ptr = rk.P(meta);
    const uint32_t* dist = rk.D(meta);
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < ns; k += gridDim.x * blockDim.x) {
        uint32_t c = cid[ptr[k]];
        uint32_t q = coff[c] + dist[k];
        if (q < ns) {
            layout[q] = slist[k];
            slot_chain[q] = c;
            kslot[k] = q;
        } else {
            set_error(flags, kErrForest);
        }
    }
}

// Lanes of the warp holding the same key: one atomicAdd per distinct key; returns
// the lane's slot (old value + its rank among the lanes with that key).
__device__ __forceinline__ uint32_t grouped_add(uint32_t* base, uint32_t key, bool active) {
    const unsigned act = __ballot_sync(0xffffffffu, active);
    if (!active) return 0;
    const unsigned peers = __match_any_sync(act, key);
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(peers) - 1;
    uint32_t b = 0;
    if (lane == leader) b = atomicAdd(&base[key], (uint32_t)__popc(peers));
    b = __shfl_sync(peers, b, leader);
    return b + (uint32_t)__popc(peers & ((1u << lane) - 1u));
}

// Counting sort inside a cooperative kernel: positions of the chains c < nc by key[c]
// (stable within a key is not needed), written to out.  hist must be zero on entry up
// to the largest key, which the sort records in meta[maxslot].
__device__ bool grid_counting_sort(const uint32_t* key, uint32_t nc, uint32_t* hist,
                                   uint32_t* meta, int maxslot, uint32_t* __restrict__ out,
                                   int* flags) {
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x; base < nc; base += stride) {
        const uint32_t c = base + threadIdx.x;
        const bool act = c < nc;
        const uint32_t k = act ? key[c] : 0;
        grouped_add(hist, k, act);
        const uint32_t km = __reduce_max_sync(0xffffffffu, k);
        if ((threadIdx.x & 31) == 0) atomicMax(&meta[maxslot], km);
    }
    if (!grid_barrier(flags)) return false;
    if (blockIdx.x == 0) {                       // exclusive scan of the key counts
        __shared__ uint32_t part[1024];
        const uint32_t nb = meta[maxslot] + 1;
        const uint32_t per = (nb + blockDim.x - 1) / blockDim.x;
        const uint32_t b = threadIdx.x * per, e = min(nb, b + per);
        uint32_t sum = 0;
        for (uint32_t i = b; i < e; ++i) sum += hist[i];
        part[threadIdx.x] = sum;
        __syncthreads();
        for (uint32_t off = 1; off < blockDim.x; off <<= 1) {
            const uint32_t v = threadIdx.x >= off ? part[threadIdx.x - off] : 0;
            __syncthreads();
            part[threadIdx.x] += v;
            __syncthreads();
        }
        uint32_t run = part[threadIdx.x] - sum;
        for (uint32_t i = b; i < e; ++i) {
            const uint32_t h = hist[i];
            hist[i] = run;
            run += h;
        }
    }
    if (!grid_barrier(flags)) return false;
    for (uint32_t base = blockIdx.x * blockDim.x; base < nc; base += stride) {
        const uint32_t c = base + threadIdx.x;
        const bool act = c < nc;
        const uint32_t pos = grouped_add(hist, act ? key[c] : 0, act);
        if (act) out[pos] = c;
    }
    return grid_barrier(flags);
}

// The chain tree (cooperative).  A chain's parent is the chain holding the site its
// bottom drains to (itself for a chain that ends at a root).  Pointer jumping gives every
// chain its root chain (cpar) and the depth of its bottom in sites below the root (a
// child's bottom lies one site below a site of its parent, so it is strictly deeper than
// the parent's bottom).  A chain's height is the depth of the deepest chain bottom in
// its subtree minus its own depth: strictly smaller for every child than for its parent.
// A chain only ever waits for its children (bottom-up: the chains ending on it) or its
// parent (top-down), so walkers that claim chains by ascending height (corder_up) or by
// ascending depth (corder_down) never wait for an unclaimed chain.  By height, chains
// without children come first and the long main stems last, by depth a chain is
// claimed about when its parent's walk reaches it.
__global__ void k_s_chain_tree(const uint32_t* __restrict__ next, const uint32_t* __restrict__ layout,
                               const uint32_t* __restrict__ coff, const uint32_t* __restrict__ sid,
                               const uint32_t* __restrict__ kslot,
                               const uint32_t* __restrict__ slot_chain, uint32_t* par0,
                               uint32_t* dep0, uint32_t* par1, uint32_t* dep1,
                               uint32_t* __restrict__ cqp, uint32_t* cpar, uint32_t* hist,
                               uint32_t* __restrict__ corder_down,
                               uint32_t* __restrict__ corder_up, uint32_t walkers, uint32_t* meta,
                               int* flags) {
    const uint32_t gtid = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t stride = gridDim.x * blockDim.x;
    if (ld_acquire(&flags[kError])) return;
    const uint32_t nc = meta[kMetaChains];
    const uint32_t ns = meta[kMetaNs];
    // with a walker for every chain all chains run at once and their order is free
    const bool sort = nc > walkers;
    // the pointer jumping's rotating "moved" words (k_s_rank's before)
    if (gtid == 0) meta[kMetaJump0] = meta[kMetaJump1] = 0;
    for (uint32_t i = gtid; i <= ns; i += stride) hist[i] = 0;
    for (uint32_t c = gtid; c < nc; c += stride) {
        const uint32_t v = layout[coff[c]];
        const uint32_t p = next[v];
        if (p == v) {
            par0[c] = c;
            dep0[c] = 0;
            cqp[c] = kNone;
        } else {
            const uint32_t q = kslot[sid[p]];
            const uint32_t pc = slot_chain[q];
            cqp[c] = q;
            par0[c] = pc;
            dep0[c] = q - coff[pc] + 1;          // sites from the parent's bottom
        }
    }
    if (!grid_barrier(flags)) return;
    // ceil(log2(nc)) + 1 rounds reach every root; the rounds stop earlier once no pointer
    // moves (every pointer is then a root: the chain tree is shallow)
    int rounds = 1;
    while ((1u << (rounds - 1)) < nc && rounds < 32) ++rounds;
    uint32_t *pin = par0, *din = dep0, *pout = par1, *dout = dep1;
    for (int r = 0; r < rounds; ++r) {
        const uint32_t* moved_w = &meta[kMetaJump0 + (r % 3)];
        if (gtid == 0) meta[kMetaJump0 + ((r + 1) % 3)] = 0;
        bool moved = false;
        for (uint32_t c = gtid; c < nc; c += stride) {
            const uint32_t p = pin[c];
            const uint32_t pp = pin[p];
            pout[c] = pp;
            dout[c] = p == c ? din[c] : din[c] + din[p];
            moved |= pp != p;
        }
        if (__syncthreads_or(moved) && threadIdx.x == 0) atomicOr(&meta[kMetaJump0 + (r % 3)], 1u);
        if (!grid_barrier(flags)) return;
        uint32_t* t = pin; pin = pout; pout = t;
        t = din; din = dout; dout = t;
        if (ld_acquire_u(moved_w) == 0) break;
    }
    // root chains, consistency, and the subtree maxima start at the own depth
    uint32_t* maxd = dout;
    for (uint32_t c = gtid; c < nc; c += stride) {
        cpar[c] = pin[c];
        if (din[c] >= ns || pin[pin[c]] != pin[c]) set_error(flags, kErrForest);
        maxd[c] = din[c];
        if (!sort) corder_down[c] = corder_up[c] = c;
    }
    if (!sort) return;
    if (!grid_barrier(flags)) return;
    if (ld_acquire(&flags[kError])) return;
    // every chain raises its ancestors' subtree maximum to its depth; a walk stops at an
    // ancestor that already holds at least as much (its setter raises the rest)
    for (uint32_t c = gtid; c < nc; c += stride) {
        const uint32_t d = din[c];
        uint32_t q = cqp[c];
        for (uint32_t hops = 0; q != kNone && hops < nc; ++hops) {
            const uint32_t a = slot_chain[q];
            if (atomicMax(&maxd[a], d) >= d) break;
            q = cqp[a];
        }
    }
    if (!grid_barrier(flags)) return;
    for (uint32_t c = gtid; c < nc; c += stride) maxd[c] -= din[c];   // heights
    if (!grid_counting_sort(din, nc, hist, meta, kMetaMaxDepth, corder_down, flags)) return;
    const uint32_t top = meta[kMetaMaxDepth];
    for (uint32_t i = gtid; i <= top; i += stride) hist[i] = 0;
    if (!grid_barrier(flags)) return;
    grid_counting_sort(maxd, nc, hist, meta, kMetaMaxHeight, corder_up, flags);
}

// Per skeleton site (layout slot q): the part of its pull that precedes the chain
// predecessor (pre) and the single addition after it (post), or kSlow.  Also marks
// the sites whose response time another chain waits for.
__global__ void k_s_prepare(uint32_t n_sites, const uint32_t* __restrict__ row,
                            const uint32_t* __restrict__ col,
                            const uint32_t* __restrict__ next, const uint32_t* __restrict__ hgt,
                            const double* __restrict__ area, const double* __restrict__ A,
                            const uint32_t* __restrict__ layout,
                            const uint32_t* __restrict__ slot_chain,
                            const uint32_t* __restrict__ coff, const uint32_t* __restrict__ clen,
                            const uint32_t* __restrict__ cbot, SlotRec* __restrict__ rec,
                            SlotInfo* __restrict__ info, double* __restrict__ tokval,
                            uint32_t* __restrict__ tokslot, uint32_t* __restrict__ pend,
                            uint32_t tok_cap, uint64_t* __restrict__ push_to,
                            int* __restrict__ td_need, int stamp, uint32_t* meta,
                            int* flags) {
    if (flags[kError]) return;
    uint32_t ns = meta[kMetaNs];
    uint32_t nc = meta[kMetaChains];
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < ns; q += gridDim.x * blockDim.x) {
        uint32_t v = layout[q];
        if (v >= n_sites) {
            set_error(flags, kErrForest);
            return;
        }
        uint32_t c = slot_chain[q];
        uint32_t last = coff[c] + clen[c] - 1;
        uint32_t heavy = q < last ? layout[q + 1] : kNone;
        double a = area[v];
        double ps[kMaxPost] = {0.0, 0.0, 0.0};
        int np = 0, ndon = 0;
        uint32_t f = (q == last) ? kLeafSlot : 0;
        bool seen_heavy = false, list = false;
        // reverse row order: additions before the predecessor fold into pre, up to
        // kMaxPost after it are replayed by the walk; anything else keeps the whole
        // donor list
        auto visit = [&](uint32_t d, bool skel, double val) {     // donor d
            ++ndon;
            if (d == heavy) {
                seen_heavy = true;
                return;
            }
            if (skel) {                     // another chain's bottom: pushed at walk time
                list = true;
                return;
            }
            if (list) return;
            if (!seen_heavy) {
                a = __dadd_rn(a, val);
            } else if (np < kMaxPost) {
                if (np == 0) ps[0] = val;
                else if (np == 1) ps[1] = val;
                else ps[2] = val;
                ++np;
            } else {
                list = true;
            }
        };
        const uint32_t s0 = row[v], s1 = row[v + 1];
        if (s1 - s0 <= (uint32_t)kRowFast) {
            // columns, then receivers, then the donors' heights and areas, each phase's
            // loads in flight together
            const uint32_t deg = s1 - s0;
            uint32_t dd[kRowFast], donm = 0, skelm = 0;
            double av[kRowFast];
#pragma unroll
            for (int k = 0; k < kRowFast; ++k)
                if ((uint32_t)k < deg) dd[k] = col[s0 + k];
#pragma unroll
            for (int k = 0; k < kRowFast; ++k)
                if ((uint32_t)k < deg && dd[k] != v && next[dd[k]] == v) donm |= 1u << k;
#pragma unroll
            for (int k = 0; k < kRowFast; ++k)
                if ((donm >> k) & 1u) {
                    if (hgt[dd[k]] == kNone) skelm |= 1u << k;
                    av[k] = A[dd[k]];
                }
#pragma unroll
            for (int k = kRowFast - 1; k >= 0; --k)
                if ((donm >> k) & 1u) visit(dd[k], (skelm >> k) & 1u, av[k]);
        } else {
            for (uint32_t s = s1; s-- > s0;) {
                const uint32_t d = col[s];
                if (d == v || next[d] != v) continue;
                const bool skel = hgt[d] == kNone;
                visit(d, skel, skel ? 0.0 : A[d]);
            }
        }
        uint32_t toff = 0;
        if (list) {
            const uint32_t nt = 1 + (uint32_t)ndon;
            toff = kNone;
            if (nt <= (uint32_t)kMaxTok) {
                toff = atomicAdd(&meta[kMetaTok], nt);
                if (toff + nt > tok_cap) toff = kNone;
            }
            if (toff == kNone) {
                f |= kSlow;
                toff = 0;
            } else {
                tokval[toff] = area[v];
                uint32_t t = 1, hpos = 0, npend = 0;
                for (uint32_t s = s1; s-- > s0;) {
                    uint32_t d = col[s];
                    if (d == v || next[d] != v) continue;
                    double val = 0.0;
                    if (d == heavy) {
                        hpos = t;
                    } else if (hgt[d] == kNone) {
                        val = __longlong_as_double((long long)kPendingBits);
                        push_to[d] = ((uint64_t)(uint32_t)stamp << 32) | (toff + t);
                        tokslot[toff + t] = q;
                        ++npend;
                    } else {
                        val = A[d];
                    }
                    tokval[toff + t] = val;
                    ++t;
                }
                f |= (nt << kTokCntShift) | (hpos << kHeavyShift);
                const uint32_t npost = hpos ? nt - 1 - hpos : 0;
                if (hpos && npend && npost <= (uint32_t)kMaxPost) {
                    // an ordinary fold slot once its operands arrive: the last chain
                    // bottom to push computes pre and the posts from the list
                    f |= kPend;
                    pend[q] = npend;
                    np = (int)npost;
                    const double m = __longlong_as_double((long long)kPendingBits);
                    a = m;
                    ps[0] = ps[1] = ps[2] = m;
                } else {
                    f |= kTok;
                    np = 0;
                }
            }
            if (!(f & kPend)) np = 0;
        }
        rec[q] = SlotRec{a, ps[0], ps[1], ps[2]};
        info[q] = SlotInfo{f | ((uint32_t)np << kPostShift), toff};
        warp_append(&meta[kMetaSlow], (f & (kTok | kSlow | kPend)) != 0);
    }
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
        uint32_t b = cbot[c];
        uint32_t p = next[b];
        if (p != b) td_need[p] = stamp;
    }
}

constexpr unsigned kFull = 0xffffffffu;

// Keeps the slowest chain's walk statistic in meta[slot] (two words).
__device__ __forceinline__ void record_chain_stat(uint32_t* meta, int slot, uint64_t dur_ns,
                                                  uint64_t cycles, uint64_t count) {
    const uint64_t d = dur_ns >> 6, c = cycles >> 7;
    const uint64_t key = ((d < kStat22 ? d : kStat22) << kStatDurShift) |
                         ((c < kStat22 ? c : kStat22) << kStatCycShift) |
                         (count < kStat20 ? count : kStat20);
    atomicMax((unsigned long long*)&meta[slot], (unsigned long long)key);
}

// Full pull of v during the walk, by the whole warp: lane l takes slot s1-1-l (reverse
// row order), the values are folded in lane order.  The chain predecessor's value is
// x; another skeleton donor is a chain bottom, waited for through bu_done.
__device__ double warp_slow_pull(uint32_t v, uint32_t heavy, double x,
                                 const uint32_t* __restrict__ row, const uint32_t* __restrict__ col,
                                 const uint32_t* __restrict__ next, const uint32_t* __restrict__ hgt,
                                 const double* __restrict__ area, const double* A,
                                 const int* bu_done, int stamp, int* flags, bool* ok,
                                 uint32_t* spin_total) {
    const int lane = threadIdx.x & 31;
    const uint32_t s0 = row[v], s1 = row[v + 1];
    double acc = area[v];
    bool fail = false;
    for (int64_t hi = s1; hi > (int64_t)s0; hi -= 32) {
        const int64_t s = hi - 1 - lane;
        bool don = false;
        double val = 0.0;
        if (s >= (int64_t)s0) {
            uint32_t d = col[s];
            if (d != v && next[d] == v) {
                don = true;
                if (d == heavy) {
                    val = x;
                } else {
                    if (hgt[d] == kNone) {
                        uint32_t spins = 0;
                        while (ld_acquire(&bu_done[d]) != stamp) {
                            if (++spins > kSpinLimit ||
                                ((spins & 255) == 0 && ld_acquire(&flags[kError]))) {
                                set_error(flags, kErrWait);
                                fail = true;
                                break;
                            }
                            __nanosleep(32);
                        }
                        *spin_total += spins;
                    }
                    val = __ldcg(&A[d]);
                }
            }
        }
        unsigned dm = __ballot_sync(kFull, don);
        if (__any_sync(kFull, fail)) {
            *ok = false;
            return 0.0;
        }
        while (dm) {
            int j = __ffs(dm) - 1;
            acc = __dadd_rn(acc, __shfl_sync(kFull, val, j));
            dm &= dm - 1;
        }
    }
    return acc;
}

__device__ __forceinline__ uint64_t ld_relaxed_u64(const double* p) {
    uint64_t v;
    asm volatile("ld.relaxed.gpu.global.b64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_relaxed_u64(double* p, uint64_t v) {
    asm volatile("st.relaxed.gpu.global.b64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

__device__ __forceinline__ uint64_t ld_acquire_u64(const double* p) {
    uint64_t v;
    asm volatile("ld.acquire.gpu.global.b64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

// The last chain bottom to push into confluence slot q's donor list computes q's fold
// operands from it (by the whole warp): pre = cell area + the donors before the chain
// predecessor, in order, and the donors after it as posts; pre, stored last, is the
// flag the slot's walker waits for.
__device__ void finalize_pending(SlotRec* rec, const SlotInfo* info, const double* tokval,
                                 uint32_t q) {
    const int lane = threadIdx.x & 31;
    const uint32_t fl = info[q].flags, toff = info[q].tokoff;
    const uint32_t nt = (fl >> kTokCntShift) & 15u, hpos = (fl >> kHeavyShift) & 15u;
    double v = 0.0;
    if ((uint32_t)lane < nt) v = __longlong_as_double((long long)ld_relaxed_u64(&tokval[toff + lane]));
    double acc = __shfl_sync(0xffffffffu, v, 0);
    for (uint32_t t = 1; t < hpos; ++t) acc = __dadd_rn(acc, __shfl_sync(0xffffffffu, v, t));
    const double p0 = __shfl_sync(0xffffffffu, v, (hpos + 1) & 31);
    const double p1 = __shfl_sync(0xffffffffu, v, (hpos + 2) & 31);
    const double p2 = __shfl_sync(0xffffffffu, v, (hpos + 3) & 31);
    if (lane == 0) {
        const uint32_t npost = nt - 1 - hpos;
        if (npost > 0) st_relaxed_u64(&rec[q].p0, (uint64_t)__double_as_longlong(p0));
        if (npost > 1) st_relaxed_u64(&rec[q].p1, (uint64_t)__double_as_longlong(p1));
        if (npost > 2) st_relaxed_u64(&rec[q].p2, (uint64_t)__double_as_longlong(p2));
        __threadfence();
        uint64_t ab = (uint64_t)__double_as_longlong(acc);
        if (isnan(acc)) ab = 0x7ff8000000000000ull;   // never the pending marker
        st_relaxed_u64(&rec[q].pre, ab);
    }
}

// The full pull of a slot with a donor list, by the whole warp: lane t takes entry t
// (waiting for a chain bottom's push), then the entries are added in order to the cell
// area, x standing in for the chain predecessor.
__device__ double warp_list_pull(const double* tokval, uint32_t toff, uint32_t nt, uint32_t hpos,
                                 double x, int* flags, bool* ok, uint32_t* spin_total) {
    const int lane = threadIdx.x & 31;
    double v = 0.0;
    bool fail = false;
    if ((uint32_t)lane < nt) {
        uint64_t b = ld_relaxed_u64(&tokval[toff + lane]);
        uint32_t spins = 0;
        while (b == kPendingBits) {
            if (++spins > kSpinLimit || ((spins & 255) == 0 && ld_acquire(&flags[kError]))) {
                set_error(flags, kErrWait);
                fail = true;
                break;
            }
            __nanosleep(32);
            b = ld_relaxed_u64(&tokval[toff + lane]);
        }
        *spin_total += spins;
        v = __longlong_as_double((long long)b);
    }
    if (__any_sync(kFull, fail)) {
        *ok = false;
        return 0.0;
    }
    double acc = __shfl_sync(kFull, v, 0);
    for (uint32_t t = 1; t < nt; ++t) {
        const double vt = __shfl_sync(kFull, v, t);
        acc = __dadd_rn(acc, t == hpos ? x : vt);
    }
    return acc;
}

// One warp per chain, leaf to bottom.  Each round the lanes load 32 slots (lane l the
// slot l places below the round's top, coalesced) and issue the next round's loads;
// warp_fold then applies every slot's additions (pre, then post) to the running area
// exactly.  Chain leaves and slots with a donor list are evaluated one at a time by
// the warp.  Results go to Al (layout order); the chain bottom's area is also stored
// in A and published through bu_done, and pushed into the donor list that waits for
// it.
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    const uint32_t sa = (uint32_t)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
    const uint32_t sa = (uint32_t)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// Rounds of slot data in flight ahead of the one being folded (per warp, in shared
// memory: a lane only ever reads back what it copied itself).  A folded round takes
// well under the L2 / HBM latency, so several rounds must be in flight.
constexpr int kStages = 3;
constexpr int kStagesDown = 4;
// Consecutive slots per lane and round: one warp scan covers 32 * S slots.
constexpr int kUpSlots = 2;
constexpr int kDownSlots = 4;

__global__ void __launch_bounds__(kWalkWarps * 32, 7)
k_s_bottom_up(const uint32_t* __restrict__ row, const uint32_t* __restrict__ col,
              const uint32_t* __restrict__ next, const uint32_t* __restrict__ hgt,
              const double* __restrict__ area, double* A, const uint32_t* __restrict__ layout,
              const uint32_t* __restrict__ coff, const uint32_t* __restrict__ clen,
              SlotRec* rec, const SlotInfo* __restrict__ info, double* tokval,
              const uint32_t* __restrict__ tokslot, uint32_t* pend,
              const uint64_t* __restrict__ push_to, double* __restrict__ Al,
              const uint32_t* __restrict__ corder, int* bu_done, int stamp, uint32_t* meta,
              int* flags) {
    constexpr int S = kUpSlots;
    __shared__ SlotRec s_rec[kWalkWarps][kStages][32 * S];
    __shared__ SlotInfo s_info[kWalkWarps][kStages][32 * S];
    const int lane = threadIdx.x & 31;
    const int wb = threadIdx.x >> 5;
    const uint32_t nc = meta[kMetaChains];
    // persistent warps claim chains by ascending height (a chain waits only for the
    // chains ending on it, whose heights are smaller); warp-uniform exits only
    while (true) {
        if (__any_sync(kFull, ld_acquire(&flags[kError]) != 0)) return;
        uint32_t idx = 0;
        if (lane == 0) idx = atomicAdd(&meta[kMetaClaimUp], 1u);
        idx = __shfl_sync(kFull, idx, 0);
        if (idx >= nc) return;
        const uint32_t c = corder[idx];
        const uint32_t off = coff[c];
        const uint32_t len = clen[c];
        if (off + len > meta[kMetaNs] || len == 0) {
            if (lane == 0) set_error(flags, kErrForest);
            return;
        }
        const uint64_t t_start = global_ns();
        uint32_t slow_cycles = 0, slow_n = 0;
        // round r, lane l, slot s is the slot (32 r + l) S + s places below the chain's leaf
        const uint32_t per_round = 32 * S;
        const uint32_t nrounds = (len + per_round - 1) / per_round;
        const uint32_t top = off + len - 1;
        auto issue = [&](uint32_t r) {                   // one commit group per round
            if (r < nrounds) {
    #pragma unroll
                for (int sl = 0; sl < S; ++sl) {
                    const uint32_t back = r * per_round + lane * S + sl;
                    if (back < len) {
                        const uint32_t q = top - back;
                        SlotRec* dst = &s_rec[wb][r % kStages][lane * S + sl];
                        cp_async16(&dst->pre, &rec[q].pre);
                        cp_async16(&dst->p1, &rec[q].p1);
                        cp_async8(&s_info[wb][r % kStages][lane * S + sl], &info[q]);
                    }
                }
            }
            cp_async_commit();
        };
    #pragma unroll
        for (int r = 0; r < kStages - 1; ++r) issue(r);
        double x = 0.0;
        bool ok = true;
        uint32_t spins = 0;
        for (uint32_t r = 0; r < nrounds; ++r) {
            __syncwarp();                                // stage r - 1 is no longer read
            issue(r + kStages - 1);
            cp_async_wait<kStages - 1>();                // this round's copies have landed
            __syncwarp();                                // ... for every lane
            const int st = r % kStages;
            const uint32_t left = len - r * per_round;
            const int cnt = left < per_round ? (int)((left + S - 1) / S) : 32;
            const int nsl = (uint32_t)lane * S < left ? (int)min((uint32_t)S, left - lane * S) : 0;
            uint32_t nopm = 0, specm = 0;
    #pragma unroll
            for (int sl = 0; sl < S; ++sl) {
                if (sl < nsl) {
                    const uint32_t fl = s_info[wb][st][lane * S + sl].flags;
                    nopm |= ((fl >> kPostShift) & 3u) << (2 * sl);
                    if (fl & (kLeafSlot | kTok | kSlow)) specm |= 1u << sl;
                }
            }
            // confluences finalised by the chain bottoms ending there: wait (bounded) for
            // their operands if this round's copy predates them
            bool pend_fail = false;
#pragma unroll
            for (int sl = 0; sl < S; ++sl) {
                if (sl < nsl && (s_info[wb][st][lane * S + sl].flags & kPend)) {
                    SlotRec& sr = s_rec[wb][st][lane * S + sl];
                    const uint32_t npost = (s_info[wb][st][lane * S + sl].flags >> kPostShift) & 3u;
                    const auto pending = [](double x) {
                        return (uint64_t)__double_as_longlong(x) == kPendingBits;
                    };
                    if (pending(sr.pre) || (npost > 0 && pending(sr.p0)) ||
                        (npost > 1 && pending(sr.p1)) || (npost > 2 && pending(sr.p2))) {
                        const uint32_t q = top - (r * per_round + lane * S + sl);
                        uint32_t sp = 0;
                        uint64_t b = ld_acquire_u64(&rec[q].pre);
                        while (b == kPendingBits) {
                            if (++sp > kSpinLimit || ((sp & 255) == 0 && ld_acquire(&flags[kError]))) {
                                set_error(flags, kErrWait);
                                pend_fail = true;
                                break;
                            }
                            __nanosleep(32);
                            b = ld_acquire_u64(&rec[q].pre);
                        }
                        spins += sp;
                        sr.pre = __longlong_as_double((long long)b);
                        sr.p0 = __longlong_as_double((long long)ld_relaxed_u64(&rec[q].p0));
                        sr.p1 = __longlong_as_double((long long)ld_relaxed_u64(&rec[q].p1));
                        sr.p2 = __longlong_as_double((long long)ld_relaxed_u64(&rec[q].p2));
                    }
                }
            }
            if (__any_sync(kFull, pend_fail)) {
                ok = false;
                break;
            }
            __syncwarp();
            auto opnd = [&](int l, int sl, int j) -> double {
                return reinterpret_cast<const double*>(&s_rec[wb][st][l * S + sl])[j];
            };
            x = warp_fold_slots<S, 4>(
                x, cnt, nsl, nopm, specm, [&](int sl, int j) { return opnd(lane, sl, j); },
                [&](int l, int sl, int j) { return opnd(l, sl, j); },
                [&](int l, int sl, double xin) -> double {
                    const SlotInfo si = s_info[wb][st][l * S + sl];
                    const uint32_t q = top - (r * per_round + l * S + sl);
                    if (!ok) return xin;
                    const long long c0 = clock64();
                    double res;
                    if (si.flags & kTok) {
                        res = warp_list_pull(tokval, si.tokoff, (si.flags >> kTokCntShift) & 15u,
                                             (si.flags >> kHeavyShift) & 15u, xin, flags, &ok, &spins);
                    } else if (si.flags & kSlow) {
                        res = warp_slow_pull(layout[q], (si.flags & kLeafSlot) ? kNone : layout[q + 1],
                                             xin, row, col, next, hgt, area, A, bu_done, stamp, flags,
                                             &ok, &spins);
                    } else {
                        return opnd(l, sl, 0);             // chain leaf: its own complete pull
                    }
                    slow_cycles += (uint32_t)(clock64() - c0);
                    ++slow_n;
                    return res;
                },
                [&](int sl, double v) { Al[top - (r * per_round + lane * S + sl)] = v; });
            if (!ok) break;
        }
        cp_async_wait<0>();                              // nothing in flight at exit
        if (!ok) return;
        uint32_t fin = kNone;
        if (lane == 0) {
            uint32_t bottom = layout[off];
            A[bottom] = x;
            st_release(&bu_done[bottom], stamp);          // orders the store above
            const uint64_t pt = push_to[bottom];
            if ((uint32_t)(pt >> 32) == (uint32_t)stamp) {
                uint64_t xb = (uint64_t)__double_as_longlong(x);
                if (isnan(x)) xb = 0x7ff8000000000000ull;   // never the pending marker
                st_relaxed_u64(&tokval[(uint32_t)pt], xb);
                const uint32_t q = tokslot[(uint32_t)pt];
                if (info[q].flags & kPend) {
                    __threadfence();                          // the push, before the count
                    if (atomicSub(&pend[q], 1u) == 1u) {
                        __threadfence();                      // every push, before the reads
                        fin = q;
                    }
                }
            }
        }
        fin = __shfl_sync(kFull, fin, 0);
        if (fin != kNone) finalize_pending(rec, info, tokval, fin);
        spins = __reduce_add_sync(kFull, spins);
        if (lane == 0 && spins) atomicAdd(&meta[kMetaSpinUp], spins);
        if (lane == 0)
            record_chain_stat(meta, kMetaUpSlow, global_ns() - t_start, slow_cycles, slow_n);
    }
}

// Skeleton areas back to site order.
__global__ void k_s_scatter(const uint32_t* __restrict__ layout, const double* __restrict__ src,
                            double* __restrict__ dst, const uint32_t* meta, const int* flags) {
    if (flags[kError]) return;
    uint32_t ns = meta[kMetaNs];
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < ns; q += gridDim.x * blockDim.x)
        dst[layout[q]] = src[q];
}

// Top-down operands in layout order: w, and whether another chain waits for the site;
// every layout-order response time starts as the pending marker.
__global__ void k_s_gather_down(const uint32_t* __restrict__ layout, const double* __restrict__ w,
                                const int* __restrict__ td_need, int stamp,
                                double* __restrict__ wl, uint8_t* __restrict__ needl,
                                double* __restrict__ tl, const uint32_t* meta, const int* flags) {
    if (flags[kError]) return;
    uint32_t ns = meta[kMetaNs];
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < ns; q += gridDim.x * blockDim.x) {
        uint32_t v = layout[q];
        wl[q] = w[v];
        needl[q] = td_need[v] == stamp ? 1 : 0;
        tl[q] = __longlong_as_double((long long)kPendingBits);
    }
}

// w_v = (1 / (k_v * sqrt(A_v))) * len_v  (generator.rs:172-173).  The f64 square root
// and divide bound this kernel, and after the first iterations of a solve most drainage
// areas and receivers stay as they were: with `valid` (k unchanged since the previous
// pass, whose w, A and len are in w / wa / wl) a site whose A and len have the same bits
// keeps its w -- the same operands give the same result.  A warp issues its f64
// sequence if any lane needs it, and changed sites are scattered, so each block first
// packs its changed sites into shared memory and computes them on dense warps.
// blockDim.x == kThreads.
__global__ void k_w(uint32_t n, const double* __restrict__ A, const double* __restrict__ kk,
                    const double* __restrict__ rlen, double* __restrict__ w,
                    double* __restrict__ wa, double* __restrict__ wl, bool valid) {
    __shared__ uint32_t s_site[kThreads];
    __shared__ double s_a[kThreads], s_l[kThreads];
    __shared__ uint32_t s_cnt;
    if (threadIdx.x == 0) s_cnt = 0;
    __syncthreads();
    const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    bool need = false;
    double a = 0.0, l = 0.0;
    if (v < n) {
        a = A[v];
        l = rlen[v];
        need = !valid || __double_as_longlong(a) != __double_as_longlong(wa[v]) ||
               __double_as_longlong(l) != __double_as_longlong(wl[v]);
    }
    const int lane = threadIdx.x & 31;
    const unsigned m = __ballot_sync(0xffffffffu, need);
    uint32_t base = 0;
    if (lane == 0 && m) base = atomicAdd(&s_cnt, (uint32_t)__popc(m));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (need) {
        const uint32_t k = base + (uint32_t)__popc(m & ((1u << lane) - 1u));
        s_site[k] = v;
        s_a[k] = a;
        s_l[k] = l;
    }
    __syncthreads();
    if (threadIdx.x >= s_cnt) return;
    const uint32_t u = s_site[threadIdx.x];
    const double au = s_a[threadIdx.x], lu = s_l[threadIdx.x];
    const double cel = __dmul_rn(kk[u], __dsqrt_rn(au));
    w[u] = __dmul_rn(__ddiv_rn(1.0, cel), lu);
    wa[u] = au;
    wl[u] = lu;
}

struct TopDown {
    const uint32_t* next;
    const double* w;
    const double* uu;
    const double* tanms;
    const double* rlen;
    const uint8_t* outlet;
    TRec* rec;
    double* elev;
    int* flags;
    const uint32_t* tid;   // packed terrains: terrain of each site (else null)
    int* tchg;             // ... and its "elevation changed" word
};

// Records that v's elevation changed (per terrain as well when terrains are packed).
__device__ __forceinline__ void mark_changed(const TopDown& td, uint32_t v, bool* changed) {
    *changed = true;
    if (td.tid) td.tchg[td.tid[v]] = 1;
}

__device__ __forceinline__ bool has_outlet(double to) {
    return (uint64_t)__double_as_longlong(to) != kNoOutletBits;
}

__device__ __forceinline__ TRec load_rec(const TRec* r) {
    const double2 a = __ldcg(reinterpret_cast<const double2*>(r));
    const double2 b = __ldcg(reinterpret_cast<const double2*>(r) + 1);
    return TRec{a.x, a.y, b.x, b.y};
}

// Response time and elevation of v from its receiver's record rp (ignored for a root)
// and v's own inputs (w, uplift, tan of the maximum slope, receiver distance, current
// elevation, outlet flag).  Writes v's record -- the basin outlet's response time and
// new elevation carried along, or kNoOutletBits for a basin without an outlet -- and,
// in a basin with an outlet, its elevation.  Returns t_v.  A site that is nobody's
// receiver may skip its record (write_rec false) unless the records are read back.
__device__ __forceinline__ double settle_own(const TopDown& td, uint32_t v, bool root,
                                             const TRec& rp, double w, double u, double tn,
                                             double dist, double old_e, bool is_outlet,
                                             double* e_out, bool* changed,
                                             bool write_rec = true) {
    double tv, to, eo, ep;
    bool has_o;
    if (root) {                           // t = 0 + (0 + w), the outlet is v itself
        tv = plus_zero(plus_zero(w));
        has_o = is_outlet;
        to = tv;
        eo = old_e;
        ep = old_e;
    } else {
        tv = plus_zero(__dadd_rn(rp.t, w));
        has_o = has_outlet(rp.to);
        to = rp.to;
        eo = rp.eo;
        ep = rp.e;
    }
    double ne = old_e;
    if (has_o) {
        double dt = __dsub_rn(tv, to);
        ne = __dadd_rn(eo, __dmul_rn(u, dt > 0.0 ? dt : 0.0));
        if (!isnan(tn)) {
            double slope = __ddiv_rn(__dsub_rn(ne, ep), dist);
            if (slope > tn) ne = __dadd_rn(ep, __dmul_rn(tn, dist));
        }
        if (ne != old_e) mark_changed(td, v, changed);
        td.elev[v] = ne;
    }
    // below a root the outlet's elevation is its updated one
    const double to_below = has_o ? to : __longlong_as_double((long long)kNoOutletBits);
    TRec out{tv, ne, to_below, root ? ne : eo};
    if (write_rec) {
        reinterpret_cast<double2*>(&td.rec[v])[0] = make_double2(out.t, out.e);
        reinterpret_cast<double2*>(&td.rec[v])[1] = make_double2(out.to, out.eo);
    }
    *e_out = ne;
    return tv;
}

__device__ __forceinline__ double settle(const TopDown& td, uint32_t v, uint32_t p,
                                         const TRec& rp, double* e_out, bool* changed) {
    return settle_own(td, v, p == v, rp, td.w[v], td.uu[v], td.tanms[v], td.rlen[v],
                      __ldcg(&td.elev[v]), td.outlet[v] != 0, e_out, changed);
}

// Before the top-down walk: root chains settle their root site (t = 0 + (0 + w), the
// outlet's own elevation update) and store its response time / elevation in the layout
// arrays, publishing it for the slope-limited walk; then every chain takes its basin
// outlet and the outlet's response time and elevation from its root chain (cpar).
__global__ void k_s_settle_roots(TopDown td, const uint32_t* __restrict__ layout,
                                 const uint32_t* __restrict__ coff,
                                 const uint32_t* __restrict__ cqp, uint32_t* __restrict__ cbas,
                                 double* __restrict__ cto, double* __restrict__ ceo,
                                 double* __restrict__ tl, double* __restrict__ el, int* td_done,
                                 int stamp, const uint32_t* meta) {
    if (td.flags[kError]) return;
    const uint32_t nc = meta[kMetaChains];
    bool changed = false;
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
        if (cqp[c] != kNone) continue;
        const uint32_t off = coff[c];
        const uint32_t v = layout[off];
        double e;
        const double tv = settle(td, v, v, TRec{}, &e, &changed);
        tl[off] = tv;
        el[off] = e;
        cbas[c] = td.outlet[v] ? v : kNone;
        cto[c] = tv;
        ceo[c] = e;
        td_done[v] = stamp;
    }
    block_flag(td.flags, kChanged, changed);
}

__global__ void k_s_root_values(const uint32_t* __restrict__ cpar, uint32_t* __restrict__ cbas,
                                double* __restrict__ cto, double* __restrict__ ceo,
                                const uint32_t* meta, const int* flags) {
    if (flags[kError]) return;
    const uint32_t nc = meta[kMetaChains];
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
        const uint32_t r = cpar[c];
        if (r != c) {
            cbas[c] = cbas[r];
            cto[c] = cto[r];
            ceo[c] = ceo[r];
        }
    }
}

// One warp per chain, bottom to leaf: t_v = 0 + (t_parent + w_v) (below a root t is
// never -0.0, so that is t_parent + w_v), in rounds of 32 slots folded exactly.
// Without slope limits only t is needed (tl, layout order; elevations follow in
// k_s_finish): a chain waits until its parent slot's tl is no longer the pending
// marker, and every tl it writes is itself the publication for the chains below.
__global__ void __launch_bounds__(kWalkWarps * 32, 8)
k_s_top_down(const int* flags, const uint32_t* __restrict__ coff,
             const uint32_t* __restrict__ clen, const uint32_t* __restrict__ cqp,
             const double* __restrict__ wl, double* tl, const uint32_t* __restrict__ corder,
             uint32_t* meta) {
    __shared__ double s_w[kWalkWarps][kStagesDown][32 * kDownSlots];
    const int lane = threadIdx.x & 31;
    const int wb = threadIdx.x >> 5;
    const uint32_t nc = meta[kMetaChains];
    // persistent warps claim chains shallowest first (a chain waits only for its
    // parent); warp-uniform exits only
    while (true) {
        if (__any_sync(kFull, ld_acquire(&flags[kError]) != 0)) return;
        uint32_t idx = 0;
        if (lane == 0) idx = atomicAdd(&meta[kMetaClaimDown], 1u);
        idx = __shfl_sync(kFull, idx, 0);
        if (idx >= nc) return;
        const uint32_t c = corder[idx];
        const uint32_t off = coff[c], len = clen[c];
        if (off + len > meta[kMetaNs] || len == 0) {
            if (lane == 0) set_error(const_cast<int*>(flags), kErrForest);
            return;
        }
        const uint32_t end = off + len;
        const uint32_t qp = cqp[c];
        uint32_t q = off;
        uint64_t tb = 0;
        bool failed = false;
        if (qp == kNone) {                   // the root was settled before the walk
            tb = (uint64_t)__double_as_longlong(tl[off]);
            q = off + 1;
        } else if (lane == 0) {
            uint32_t spins = 0;
            const uint64_t t0 = global_ns();
            const long long c0 = clock64();
            tb = ld_relaxed_u64(&tl[qp]);
            while (tb == kPendingBits) {
                if (++spins > kSpinLimit || ((spins & 255) == 0 && ld_acquire(&flags[kError]))) {
                    set_error(const_cast<int*>(flags), kErrWait);
                    failed = true;
                    break;
                }
                __nanosleep(32);
                tb = ld_relaxed_u64(&tl[qp]);
            }
            // the chain that waited longest for its parent
            record_chain_stat(meta, kMetaDownSlow, global_ns() - t0, (uint64_t)(clock64() - c0), len);
            if (spins) atomicAdd(&meta[kMetaSpinDown], spins);
        }
        if (__shfl_sync(kFull, failed, 0)) return;
        double tp = __longlong_as_double((long long)__shfl_sync(kFull, (unsigned long long)tb, 0));
        constexpr int S = kDownSlots;
        constexpr uint32_t per_round = 32 * S;
        const uint32_t nrounds = (end - q + per_round - 1) / per_round;
        auto issue = [&](uint32_t r) {                   // one commit group per round
            if (r < nrounds) {
    #pragma unroll
                for (int sl = 0; sl < S; ++sl) {
                    const uint32_t qq = q + r * per_round + lane * S + sl;
                    if (qq < end) cp_async8(&s_w[wb][r % kStagesDown][lane * S + sl], &wl[qq]);
                }
            }
            cp_async_commit();
        };
    #pragma unroll
        for (int r = 0; r < kStagesDown - 1; ++r) issue(r);
        for (uint32_t r = 0; r < nrounds; ++r) {
            __syncwarp();                                // stage r - 1 is no longer read
            issue(r + kStagesDown - 1);
            cp_async_wait<kStagesDown - 1>();
            __syncwarp();
            const int st = r % kStagesDown;
            const uint32_t q0 = q + r * per_round;
            const uint32_t left = end - q0;
            const int cnt = left < per_round ? (int)((left + S - 1) / S) : 32;
            const int nsl = (uint32_t)lane * S < left ? (int)min((uint32_t)S, left - lane * S) : 0;
            tp = warp_fold_slots<S, 1>(
                tp, cnt, nsl, 0u, 0u, [&](int sl, int) { return s_w[wb][st][lane * S + sl]; },
                [&](int l, int sl, int) { return s_w[wb][st][l * S + sl]; },
                [](int, int, double xin) -> double { return xin; },
                [&](int sl, double v) {
                    st_relaxed_u64(&tl[q0 + lane * S + sl], (uint64_t)__double_as_longlong(v));
                });
        }
        cp_async_wait<0>();
    }
}

// With slope limits the elevation clamp e_v <= e_parent + tan * len chains through
// the elevations too: lane 0 walks the chain site by site with settle().  A chain
// starts once its parent site is published (t / elevation / basin written, then
// td_done released); sites another chain hangs from are published as they are
// passed.  Root chains start from the values the pre-pass settled.
__global__ void k_s_top_down_slope(TopDown td, const uint32_t* __restrict__ layout,
                                   const uint32_t* __restrict__ coff,
                                   const uint32_t* __restrict__ clen,
                                   const uint32_t* __restrict__ cqp,
                                   const uint8_t* __restrict__ needl, double* __restrict__ tl,
                                   double* __restrict__ el, const uint32_t* __restrict__ corder,
                                   int* td_done, int stamp, uint32_t* meta) {
    const int lane = threadIdx.x & 31;
    if (lane != 0) return;
    const uint32_t nc = meta[kMetaChains];
    // one thread per chain, claimed shallowest first (a chain waits only for its parent)
    while (true) {
        if (ld_acquire(&td.flags[kError]) != 0) return;
        const uint32_t idx = atomicAdd(&meta[kMetaClaimDown], 1u);
        if (idx >= nc) return;
        const uint32_t c = corder[idx];
        const uint32_t off = coff[c], len = clen[c];
        if (off + len > meta[kMetaNs] || len == 0) {
            set_error(td.flags, kErrForest);
            return;
        }
        const uint32_t end = off + len;
        uint32_t q = off;
        uint32_t p = td.next[layout[off]];
        if (cqp[c] == kNone) {                 // the root was settled before the walk
            p = layout[off];
            q = off + 1;
        } else {
            uint32_t spins = 0;
            const uint64_t t0 = global_ns();
            const long long c0 = clock64();
            while (ld_acquire(&td_done[p]) != stamp) {
                if (++spins > kSpinLimit || ((spins & 255) == 0 && ld_acquire(&td.flags[kError]))) {
                    set_error(td.flags, kErrWait);
                    return;
                }
                __nanosleep(32);
            }
            record_chain_stat(meta, kMetaDownSlow, global_ns() - t0, (uint64_t)(clock64() - c0), len);
            if (spins) atomicAdd(&meta[kMetaSpinDown], spins);
        }
        bool changed = false;
        TRec rp = load_rec(&td.rec[p]);
        for (; q < end; ++q) {
            const uint32_t v = layout[q];
            double e;
            const double tp = settle(td, v, p, rp, &e, &changed);
            rp = TRec{tp, e, rp.to, rp.eo};      // the basin outlet's values pass down
            tl[q] = tp;
            el[q] = e;
            p = v;
            if (needl[q]) st_release(&td_done[v], stamp);   // v's record written above
        }
        if (changed) td.flags[kChanged] = 1;
    }
}

// Skeleton response times and elevations back to site order (records and elevations;
// the slope-limited walk wrote its sites itself).
__global__ void k_s_finish(TopDown td, const uint32_t* __restrict__ layout,
                           const uint32_t* __restrict__ slot_chain, const double* __restrict__ tl,
                           const uint32_t* __restrict__ cbas, const double* __restrict__ cto,
                           const double* __restrict__ ceo, const uint32_t* meta) {
    if (td.flags[kError]) return;
    uint32_t ns = meta[kMetaNs];
    bool changed = false;
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < ns; q += gridDim.x * blockDim.x) {
        uint32_t v = layout[q];
        if (td.next[v] == v) continue;     // roots were settled before the walk
        const uint32_t c = slot_chain[q];
        const bool has_o = cbas[c] != kNone;
        const double tv = tl[q];
        const double to = cto[c], eo = ceo[c];
        double ne = 0.0;
        if (has_o) {
            const double old_e = td.elev[v];
            double dt = __dsub_rn(tv, to);
            ne = __dadd_rn(eo, __dmul_rn(td.uu[v], dt > 0.0 ? dt : 0.0));
            if (ne != old_e) mark_changed(td, v, &changed);
            td.elev[v] = ne;
        } else {
            ne = td.elev[v];
        }
        reinterpret_cast<double2*>(&td.rec[v])[0] = make_double2(tv, ne);
        reinterpret_cast<double2*>(&td.rec[v])[1] =
            make_double2(has_o ? to : __longlong_as_double((long long)kNoOutletBits), eo);
    }
    block_flag(td.flags, kChanged, changed);
}

// Top-down over the Kahn rounds, highest round first, a grid barrier between rounds.
// After the barrier a site only needs its receiver's record: each thread loads its
// first site of the next round (id at the start of the round, receiver and own inputs
// before the barrier), so a narrow round costs about one barrier and one load.  In a
// wide round a thread has further sites; it takes them K at a time, issuing all K ids,
// then all K sites' inputs, then all K receivers' records before settling any, so K
// dependent load chains are in flight per thread instead of one (the sites of a round
// are independent: every receiver belongs to a higher round).
// Round 0 is the leaves, which are nobody's receiver: their records are written only
// when all_records asks for every site's record.
constexpr int low_block(int K) { return K == 1 ? 1024 : K == 2 ? 512 : 256; }

template <bool kSlope, int K>
__global__ void __launch_bounds__(low_block(K))
k_low_top_down(TopDown td, const uint32_t* __restrict__ order,
               const uint32_t* __restrict__ roff, uint64_t* __restrict__ rtime,
               const uint32_t* meta, bool all_records) {
    const uint32_t gtid = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t stride = gridDim.x * blockDim.x;
    if (ld_acquire(&td.flags[kError])) return;
    const uint32_t rs = meta[kMetaRStop];
    bool changed = false;
    if (gtid == 0) rtime[0] = global_ns();
    struct Site {
        uint32_t v, p;
        double w, u, tn, dist, old_e;
    };
    // the slope inputs only with slope limits
    auto inputs = [&](uint32_t v, Site& f) {
        f.v = v;
        f.p = td.next[v];
        f.w = td.w[v];
        f.u = td.uu[v];
        f.tn = kSlope ? td.tanms[v] : __longlong_as_double(0x7ff8000000000000ll);
        f.dist = kSlope ? td.rlen[v] : 1.0;
        f.old_e = __ldcg(&td.elev[v]);
    };
    // the outlet flag only matters for a root
    auto settle_site = [&](const Site& f, const TRec& rp, bool write_rec) {
        const bool root = f.p == f.v;
        const bool is_outlet = root && td.outlet[f.v] != 0;
        double en;
        settle_own(td, f.v, root, rp, f.w, f.u, f.tn, f.dist, f.old_e, is_outlet, &en, &changed,
                   write_rec);
    };
    Site cur{};
    if (rs > 0 && roff[rs - 1] + gtid < roff[rs]) inputs(order[roff[rs - 1] + gtid], cur);
    for (uint32_t r = rs; r-- > 0;) {
        const uint32_t b = roff[r], e = roff[r + 1];
        const bool write_rec = r > 0 || all_records;
        const uint32_t nidx = (r > 0 && roff[r - 1] + gtid < b) ? roff[r - 1] + gtid : kNone;
        const uint32_t nv = nidx != kNone ? order[nidx] : kNone;   // next round, in flight
        uint32_t i = b + gtid;
        if (i < e) {                                   // the prefetched first site
            const TRec rp = cur.p != cur.v ? load_rec(&td.rec[cur.p]) : TRec{};
            settle_site(cur, rp, write_rec);
        }
        for (i += stride; i < e; i += K * stride) {
            uint32_t vid[K];
#pragma unroll
            for (int k = 0; k < K; ++k) {
                const uint32_t ii = i + (uint32_t)k * stride;
                vid[k] = ii < e ? order[ii] : kNone;
            }
            Site f[K];
#pragma unroll
            for (int k = 0; k < K; ++k)
                if (vid[k] != kNone) inputs(vid[k], f[k]);
            TRec rp[K];
#pragma unroll
            for (int k = 0; k < K; ++k)
                rp[k] = (vid[k] != kNone && f[k].p != f[k].v) ? load_rec(&td.rec[f[k].p]) : TRec{};
#pragma unroll
            for (int k = 0; k < K; ++k)
                if (vid[k] != kNone) settle_site(f[k], rp[k], write_rec);
        }
        if (nv != kNone) inputs(nv, cur);
        if (!grid_barrier(td.flags)) return;
        if (gtid == 0) rtime[rs - r] = global_ns();
    }
    block_flag(td.flags, kChanged, changed);
}

template <class K, class... Args>
cudaError_t coop_launch(K kernel, unsigned grid, unsigned block, cudaStream_t st, Args... args) {
    void* argv[] = {(void*)&args...};
    return cudaLaunchCooperativeKernel((const void*)kernel, dim3(grid), dim3(block), argv, 0, st);
}

template <class... Args>
cudaError_t coop_launch_ptr(const void* kernel, unsigned grid, unsigned block, cudaStream_t st,
                            Args... args) {
    void* argv[] = {(void*)&args...};
    return cudaLaunchCooperativeKernel(kernel, dim3(grid), dim3(block), argv, 0, st);
}

// Blocks of `block` threads at which `kernel` is co-resident on the current device.
unsigned coop_grid(const void* kernel, unsigned block, unsigned cap_per_sm) {
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, (int)block, 0);
    if (per < 1) per = 1;
    return (unsigned)(sms * std::min<unsigned>((unsigned)per, cap_per_sm));
}

// Round kernels synchronise the grid every round; big blocks keep the number of
// barrier arrivals (one per block) small.
constexpr unsigned kRoundBlock = 1024;

}  // namespace

// Probe: x_k after each operand of one chain (one operand per slot), by warp_fold.
__global__ void k_fold_probe(const double* __restrict__ y, uint32_t n, double x0,
                             double* __restrict__ out) {
    constexpr int S = kDownSlots;
    constexpr uint32_t per_round = 32 * S;
    const int lane = threadIdx.x & 31;
    double x = x0;
    for (uint32_t base = 0; base < n; base += per_round) {
        const uint32_t left = n - base;
        const int cnt = left < per_round ? (int)((left + S - 1) / S) : 32;
        const int nsl = (uint32_t)lane * S < left ? (int)min((uint32_t)S, left - lane * S) : 0;
        x = warp_fold_slots<S, 1>(
            x, cnt, nsl, 0u, 0u, [&](int sl, int) { return y[base + lane * S + sl]; },
            [&](int l, int sl, int) { return y[base + l * S + sl]; },
            [](int, int, double xin) -> double { return xin; },
            [&](int sl, double v) { out[base + lane * S + sl] = v; });
    }
}

cudaError_t fold_probe(const double* y, uint32_t n, double x0, double* out) {
    k_fold_probe<<<1, 32>>>(y, n, x0, out);
    return cudaGetLastError();
}

uint32_t walk_capacity() {
    int dev = 0, sms = 0, up = 0, down = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&up, k_s_bottom_up, kWalkWarps * 32, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&down, k_s_top_down, kWalkWarps * 32, 0);
    int down_slope = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&down_slope, k_s_top_down_slope, kWalkWarps * 32, 0);
    down = std::min(down, down_slope);
    int per = std::max(1, std::min(up, down));
    return (uint32_t)(sms * per * kWalkWarps);
}

uint32_t walk_grid(uint32_t per_sm) {
    static uint32_t cached = 0;            // the GPUs of a process match
    if (!cached) cached = std::max<uint32_t>(1, walk_capacity() / kWalkWarps);
    uint32_t g = cached;
    if (per_sm) {
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        g = std::min<uint32_t>(g, (uint32_t)std::max(1, sms) * per_sm);
    }
    return g;
}

cudaError_t basin_pass(const BasinArgs& a, cudaStream_t st, const Hooks& hk, uint32_t nnz) {
    const uint32_t n = a.n;
    const unsigned nb = (n + kThreads - 1) / kThreads;
    const bool sz = a.sized_grids;
    const unsigned g_kahn = sized_grid(sz, coop_grid((const void*)k_kahn, kThreads, 8), n, kThreads * 8);
    const unsigned g_rank = sized_grid(sz, coop_grid((const void*)k_s_rank, kRoundBlock, 2), n / 8,
                                       kRoundBlock * 4);
    // ordered compactions: one block range each, two blocks per SM
    const unsigned g_compact = coop_grid((const void*)k_collect_leaves, kRoundBlock, 2);
    // persistent chain walkers: every warp resident (they wait on one another)
    const unsigned g_chain = sized_grid(sz, a.walk_grid, n, 4096, 16);
    const unsigned g_tree = sized_grid(sz, coop_grid((const void*)k_s_chain_tree, kThreads, 4), n / 16,
                                       kThreads * 4);
    const unsigned gs = 152 * 8;   // grid-stride kernels over the skeleton
    Ranks rk{{a.sptr0, a.sptr1}, {a.sdist0, a.sdist1}};
    TopDown td{a.next, a.w, a.u, a.tanms, a.rlen, a.outlet, a.rec_t, a.elev, a.flags, a.tid, a.tchg};
    cudaError_t e;

    hk.begin(hk.ctx);
    cudaMemsetAsync(a.pending, 0, n * 4ull, st);
    cudaMemsetAsync(a.hgt, 0xff, n * 4ull, st);
    cudaMemsetAsync(a.meta, 0, kMetaCount * 4ull, st);
    const uint32_t* titer = a.tid ? a.titer : nullptr;
    k_count_donors<<<nb, kThreads, 0, st>>>(n, a.next, a.pending, a.tid, titer);
    k_collect_leaves<<<g_compact, kRoundBlock, 0, st>>>(n, a.pending, a.order, a.meta + kMetaLeaves,
                                                        a.tid, titer);
    hk.end(hk.ctx, kcBasinBuild, 20.0 * n);

    // Kahn rounds: order 4 + next 4 + row 8 + area 8 + A 8 + hgt 4 + pending 4 per site,
    // col 4 + next 4 per slot, donor areas 8 per site
    hk.begin(hk.ctx);
    e = coop_launch(k_kahn, g_kahn, kThreads, st, n, a.row, a.col, a.next, a.area, a.A, a.pending,
                    a.hgt, a.order, a.roff, a.rtime, a.max_rounds, a.kahn_min_width, a.meta,
                    a.flags);
    hk.end(hk.ctx, kcKahn, 48.0 * n + 8.0 * nnz);
    if (e != cudaSuccess) return e;

    hk.begin(hk.ctx);
    k_s_collect<<<g_compact, kRoundBlock, 0, st>>>(n, a.hgt, a.sid, a.slist, a.meta, a.tid, titer);
    k_s_designate<<<gs, kThreads, 0, st>>>(a.row, a.col, a.next, a.hgt, a.A, a.slist, a.desig,
                                           a.meta);
    k_s_link<<<gs, kThreads, 0, st>>>(a.next, a.desig, a.hgt, a.sid, a.slist, a.sptr0, a.sdist0,
                                      a.meta);
    hk.end(hk.ctx, kcBasinBuild, 4.0 * n);

    hk.begin(hk.ctx);
    e = coop_launch(k_s_rank, g_rank, kRoundBlock, st, a.sptr0, a.sdist0, a.sptr1, a.sdist1, a.meta,
                    a.flags);
    hk.end(hk.ctx, kcSkelRank, 0.0);
    if (e != cudaSuccess) return e;

    hk.begin(hk.ctx);
    k_s_bottoms<<<gs, kThreads, 0, st>>>(a.slist, rk, a.cid, a.cbot, a.kahn_min_width, a.meta,
                                         a.flags);
    k_s_lengths<<<gs, kThreads, 0, st>>>(a.order, a.sid, rk, a.cid, a.clen, a.kahn_min_width, a.meta,
                                         a.flags);
    k_s_scan<<<1, 1024, 0, st>>>(a.clen, a.coff, a.meta, a.flags);
    k_s_layout<<<gs, kThreads, 0, st>>>(a.slist, rk, a.cid, a.coff, a.layout, a.slot_chain, a.kslot,
                                        a.meta,
                                        a.flags);
    e = coop_launch(k_s_chain_tree, g_tree, kThreads, st, (const uint32_t*)a.next,
                    (const uint32_t*)a.layout, (const uint32_t*)a.coff, (const uint32_t*)a.sid,
                    (const uint32_t*)a.kslot, (const uint32_t*)a.slot_chain, a.cpar1, a.cdep,
                    a.cpar1 + a.kahn_min_width, a.cdep1, a.cqp, a.cpar, a.chist, a.corder,
                    a.corder_up, g_chain * kWalkWarps, a.meta, a.flags);
    if (e != cudaSuccess) return e;
    k_s_prepare<<<gs, kThreads, 0, st>>>(n, a.row, a.col, a.next, a.hgt, a.area, a.A, a.layout,
                                         a.slot_chain, a.coff, a.clen, a.cbot, a.rec, a.info,
                                         a.tokval, a.tokslot, a.pend, a.tok_cap, a.push_to,
                                         a.td_need, a.stamp, a.meta, a.flags);
    hk.end(hk.ctx, kcBasinBuild, 0.0);

    // chain walk bottom-up; results in layout order (in place over `pre`)
    hk.begin(hk.ctx);
    e = coop_launch(k_s_bottom_up, g_chain, kWalkWarps * 32, st, a.row, a.col, a.next,
                    (const uint32_t*)a.hgt, a.area, a.A, (const uint32_t*)a.layout,
                    (const uint32_t*)a.coff, (const uint32_t*)a.clen, a.rec,
                    (const SlotInfo*)a.info, a.tokval, (const uint32_t*)a.tokslot, a.pend,
                    (const uint64_t*)a.push_to, a.pre, (const uint32_t*)a.corder_up, a.bu_done,
                    a.stamp, a.meta, a.flags);
    hk.end(hk.ctx, kcSkelUp, 0.0);
    if (e != cudaSuccess) return e;

    hk.begin(hk.ctx);
    k_s_scatter<<<gs, kThreads, 0, st>>>(a.layout, a.pre, a.A, a.meta, a.flags);
    hk.end(hk.ctx, kcBasinBuild, 0.0);

    // w: A 8 + k 8 + rlen 8 + w 8 per site
    hk.begin(hk.ctx);
    k_w<<<nb, kThreads, 0, st>>>(n, a.A, a.k, a.rlen, a.w, a.w_area, a.w_dist, a.w_valid);
    hk.end(hk.ctx, kcW, 32.0 * n);

    hk.begin(hk.ctx);
    k_s_gather_down<<<gs, kThreads, 0, st>>>(a.layout, a.w, a.td_need, a.stamp, a.post, a.needl,
                                             a.pre, a.meta, a.flags);
    hk.end(hk.ctx, kcBasinBuild, 0.0);

    hk.begin(hk.ctx);
    k_s_settle_roots<<<gs, kThreads, 0, st>>>(td, (const uint32_t*)a.layout,
                                              (const uint32_t*)a.coff, (const uint32_t*)a.cqp,
                                              a.cbas, a.cto, a.ceo, a.pre, a.el, a.td_done,
                                              a.stamp, (const uint32_t*)a.meta);
    k_s_root_values<<<gs, kThreads, 0, st>>>((const uint32_t*)a.cpar, a.cbas, a.cto, a.ceo,
                                             (const uint32_t*)a.meta, (const int*)a.flags);
    if (a.slope) {
        e = coop_launch(k_s_top_down_slope, g_chain, kWalkWarps * 32, st, td,
                        (const uint32_t*)a.layout, (const uint32_t*)a.coff,
                        (const uint32_t*)a.clen, (const uint32_t*)a.cqp, (const uint8_t*)a.needl,
                        a.pre, a.el, (const uint32_t*)a.corder, a.td_done, a.stamp, a.meta);
    } else {
        e = coop_launch(k_s_top_down, g_chain, kWalkWarps * 32, st, (const int*)a.flags,
                        (const uint32_t*)a.coff, (const uint32_t*)a.clen, (const uint32_t*)a.cqp,
                        (const double*)a.post, a.pre, (const uint32_t*)a.corder, a.meta);
    }
    hk.end(hk.ctx, kcSkelDown, 0.0);
    if (e != cudaSuccess) return e;

    hk.begin(hk.ctx);
    if (!a.slope)
        k_s_finish<<<gs, kThreads, 0, st>>>(td, (const uint32_t*)a.layout,
                                            (const uint32_t*)a.slot_chain, (const double*)a.pre,
                                            (const uint32_t*)a.cbas, (const double*)a.cto,
                                            (const double*)a.ceo, (const uint32_t*)a.meta);
    hk.end(hk.ctx, kcBasinBuild, 0.0);

    // top-down rounds: order 4, next 4, w 8, u 8, tan 8, rlen 8, elev 8+8, t 8, bas 4,
    // parent t/elev/bas 20, outlet t/elev 16 per site
    hk.begin(hk.ctx);
    {
        const int K = a.low_ilp;
        const void* kern =
            a.slope ? (K == 4 ? (const void*)k_low_top_down<true, 4>
                              : K == 2 ? (const void*)k_low_top_down<true, 2>
                                       : (const void*)k_low_top_down<true, 1>)
                    : (K == 4 ? (const void*)k_low_top_down<false, 4>
                              : K == 2 ? (const void*)k_low_top_down<false, 2>
                                       : (const void*)k_low_top_down<false, 1>);
        const unsigned blk = (unsigned)low_block(K);
        e = coop_launch_ptr(kern, sized_grid(sz, coop_grid(kern, blk, 2048 / blk), n, blk * 16ull), blk, st, td,
                            (const uint32_t*)a.order, (const uint32_t*)a.roff,
                            a.rtime + a.max_rounds + 1, (const uint32_t*)a.meta, a.all_records);
    }
    hk.end(hk.ctx, kcLowDown, 112.0 * n);
    return e;
}

}  // namespace fl
