// oracle.cpp -- TEST INFRASTRUCTURE, NOT PART OF THE PRODUCT.
//
// A CPU restatement of fastlem 0.1.4's landscape-evolution solve
// (`TerrainGenerator::generate`), used only as the parity checker by the tests,
// by `__graft_entry__.smoke()` and by the `cpu_baseline` / `--impl reference` legs of
// `bench.py`.  The shipped library (fastlem_gb300) never links, loads or calls it.
//
// Parity status: the reference is Rust and no Rust toolchain exists where this runs,
// so the restatement could not be checked against fastlem's own output.  It is
// pinned against (a) published known-answer vectors for the ChaCha block function
// (RFC 7539 section 2.3.2, adapted to 20 rounds) and (b) hand-worked cases whose
// expected results follow from the reference source line by line
// (tests/golden/).  Everything else about parity with fastlem itself is
// "parity unpinned".
//
// Sources restated (paths inside the fastlem crate):
//   src/lem/generator.rs:90-213        generate()
//   src/lem/stream_tree.rs:72-243      StreamTree::construct and helpers
//   src/lem/drainage_basin.rs:13-46    DrainageBasin
//   Cargo.toml:16 rand = "0.8.5"       StdRng = ChaCha12 (rand_chacha 0.3), seeded by
//                                      rand_core 0.6's seed_from_u64 (PCG32 expansion)
//
// Conventions: the graph is a CSR whose row i lists `graph.neighbors_of(i)` in
// insertion order (terrain-graph 1.0.1 `add_edge(a, b, w)` appends (b, w) to a's
// list and (a, w) to b's list).  `has_edge(i, j)` returns the weight of the first
// entry of row i whose column is j.

#include <cmath>
#include <cstdint>
#include <cstring>
#include <chrono>
#include <vector>
#include <algorithm>

namespace {

// ---------------------------------------------------------------------------
// rand 0.8.5 StdRng: ChaCha with 12 rounds, 64-bit block counter in words 12-13,
// stream id 0 in words 14-15.  `seed_from_u64` (rand_core 0.6) fills the 32-byte
// seed with little-endian PCG32 outputs.  `gen::<f64>()` takes next_u64() >> 11
// and scales by 2^-53.  next_u64 reads two consecutive keystream words
// (low word first).
// ---------------------------------------------------------------------------
inline uint32_t rotl32(uint32_t v, int c) { return (v << c) | (v >> (32 - c)); }

inline void quarter(uint32_t& a, uint32_t& b, uint32_t& c, uint32_t& d) {
    a += b; d ^= a; d = rotl32(d, 16);
    c += d; b ^= c; b = rotl32(b, 12);
    a += b; d ^= a; d = rotl32(d, 8);
    c += d; b ^= c; b = rotl32(b, 7);
}

void chacha_block(const uint32_t key[8], uint64_t counter, uint64_t stream, int rounds,
                  uint32_t out[16]) {
    uint32_t s[16] = {0x61707865u, 0x3320646eu, 0x79622d32u, 0x6b206574u,
                      key[0], key[1], key[2], key[3], key[4], key[5], key[6], key[7],
                      (uint32_t)counter, (uint32_t)(counter >> 32),
                      (uint32_t)stream, (uint32_t)(stream >> 32)};
    uint32_t x[16];
    std::memcpy(x, s, sizeof x);
    for (int r = 0; r < rounds; r += 2) {
        quarter(x[0], x[4], x[8], x[12]);
        quarter(x[1], x[5], x[9], x[13]);
        quarter(x[2], x[6], x[10], x[14]);
        quarter(x[3], x[7], x[11], x[15]);
        quarter(x[0], x[5], x[10], x[15]);
        quarter(x[1], x[6], x[11], x[12]);
        quarter(x[2], x[7], x[8], x[13]);
        quarter(x[3], x[4], x[9], x[14]);
    }
    for (int i = 0; i < 16; ++i) out[i] = x[i] + s[i];
}

void seed_from_u64(uint64_t state, uint32_t key[8]) {
    const uint64_t MUL = 6364136223846793005ull;
    const uint64_t INC = 11634580027462260723ull;
    for (int w = 0; w < 8; ++w) {
        state = state * MUL + INC;
        uint32_t xorshifted = (uint32_t)(((state >> 18) ^ state) >> 27);
        uint32_t rot = (uint32_t)(state >> 59);
        key[w] = (xorshifted >> rot) | (xorshifted << ((32 - rot) & 31));
    }
}

// ---------------------------------------------------------------------------
// Rust std::collections::BinaryHeap<RidgeElement> (stream_tree.rs:15-44,184).
// RidgeElement's Ord is reversed on `dist`, so the heap pops the smallest dist.
// Equal keys are ordered by the heap's own sift rules, reproduced here:
//   push: append, sift_up while elem > parent (i.e. elem.dist < parent.dist).
//   pop:  take the last element, swap it into the root, sift_down_to_bottom
//         (always descend to the child c+1 when data[c] <= data[c+1], i.e. when
//         right.dist <= left.dist), then sift_up from where the hole stopped.
// `partial_cmp().unwrap()` panics on NaN; here a NaN key sets `nan_seen`.
// ---------------------------------------------------------------------------
struct Ridge { uint32_t index; double dist; };

struct RustMinHeap {
    std::vector<Ridge> d;
    bool nan_seen = false;
    // Ord::gt for RidgeElement: a > b  <=>  b.dist.partial_cmp(a.dist) == Greater
    bool gt(const Ridge& a, const Ridge& b) {
        if (std::isnan(a.dist) || std::isnan(b.dist)) nan_seen = true;
        return b.dist > a.dist;
    }
    size_t sift_up(size_t start, size_t pos) {
        Ridge e = d[pos];
        while (pos > start) {
            size_t parent = (pos - 1) / 2;
            if (!gt(e, d[parent])) break;   // hole.element() <= parent  -> stop
            d[pos] = d[parent];
            pos = parent;
        }
        d[pos] = e;
        return pos;
    }
    void sift_down_to_bottom(size_t pos) {
        size_t end = d.size();
        size_t start = pos;
        Ridge e = d[pos];
        size_t child = 2 * pos + 1;
        while (end >= 2 && child <= end - 2) {
            // child += (data[child] <= data[child+1])  ==  !(data[child] > data[child+1])
            if (!gt(d[child], d[child + 1])) child += 1;
            d[pos] = d[child];
            pos = child;
            child = 2 * pos + 1;
        }
        if (child == end - 1) {
            d[pos] = d[child];
            pos = child;
        }
        d[pos] = e;
        sift_up(start, pos);
    }
    void push(Ridge r) { d.push_back(r); sift_up(0, d.size() - 1); }
    bool pop(Ridge& out) {
        if (d.empty()) return false;
        Ridge item = d.back();
        d.pop_back();
        if (!d.empty()) {
            std::swap(item, d[0]);
            sift_down_to_bottom(0);
        }
        out = item;
        return true;
    }
};

struct Graph {
    uint32_t n;
    const uint32_t* row_ptr;  // n + 1
    const uint32_t* col;
    const double* len;
    const double* area;
};

// terrain-graph `has_edge(i, j)`: (true, w) for the first entry of row i with column j.
inline double edge_length_or_one(const Graph& g, uint32_t i, uint32_t j) {
    for (uint32_t s = g.row_ptr[i]; s < g.row_ptr[i + 1]; ++s)
        if (g.col[s] == j) return g.len[s];
    return 1.0;
}

// stream_tree.rs:109-137 construct_initial_stream_tree
void initial_stream_tree(const Graph& g, const double* elev, const uint8_t* is_outlet,
                         uint32_t* next) {
    for (uint32_t i = 0; i < g.n; ++i) {
        next[i] = i;
        if (is_outlet[i]) continue;
        double steepest = 0.0;
        for (uint32_t s = g.row_ptr[i]; s < g.row_ptr[i + 1]; ++s) {
            uint32_t j = g.col[s];
            if (elev[i] > elev[j]) {
                double slope = (elev[i] - elev[j]) / g.len[s];
                if (slope > steepest) {
                    steepest = slope;
                    next[i] = j;
                }
            }
        }
    }
}

// stream_tree.rs:139-173 find_roots_with_lakes
bool roots_with_lakes(uint32_t n, const uint8_t* is_outlet, const uint32_t* next,
                      uint32_t* subroot) {
    const uint32_t NONE = UINT32_MAX;
    for (uint32_t i = 0; i < n; ++i) subroot[i] = is_outlet[i] ? i : NONE;
    bool has_lake = false;
    for (uint32_t i = 0; i < n; ++i) {
        if (subroot[i] != NONE) continue;
        uint32_t iv = i;
        while (subroot[iv] == NONE && iv != next[iv]) iv = next[iv];
        uint32_t ir;
        if (subroot[iv] == NONE) {
            has_lake = true;
            ir = iv;
        } else {
            ir = subroot[iv];
        }
        iv = i;
        while (subroot[iv] == NONE && iv != next[iv]) {
            subroot[iv] = ir;
            iv = next[iv];
        }
        subroot[iv] = ir;
    }
    return has_lake;
}

// stream_tree.rs:175-243 remove_lakes_from_stream_tree, heap-driven as in the reference.
bool remove_lakes_heap(const Graph& g, const uint32_t* outlets, uint32_t n_out,
                       const uint32_t* subroot, uint32_t* next /* in/out */) {
    const uint32_t NONE = UINT32_MAX;
    std::vector<uint32_t> root(g.n, NONE);
    RustMinHeap heap;
    heap.d.reserve(g.n);
    for (uint32_t o = 0; o < n_out; ++o) {
        root[outlets[o]] = outlets[o];
        heap.push({outlets[o], 0.0});
    }
    std::vector<uint8_t> visited(g.n, 0);
    Ridge el;
    while (heap.pop(el)) {
        uint32_t i = el.index;
        if (visited[i]) continue;
        for (uint32_t s = g.row_ptr[i]; s < g.row_ptr[i + 1]; ++s) {
            uint32_t j = g.col[s];
            if (visited[j]) continue;
            if (root[subroot[j]] == NONE) {
                uint32_t k = j, nk = i;
                while (next[k] != k) {   // flip flow
                    uint32_t tmp = next[k];
                    next[k] = nk;
                    nk = k;
                    k = tmp;
                }
                next[k] = nk;
                root[subroot[j]] = root[subroot[i]];
            }
            heap.push({j, g.len[s]});
        }
        root[i] = root[subroot[i]];
        visited[i] = 1;
    }
    return !heap.nan_seen;
}

// The pop order of the loop above (the sequence of sites processed, i.e. popped
// while unvisited) depends only on the graph, the lengths and the outlet list:
// pushes happen for every unvisited neighbour whatever `next` holds.  This
// computes it without touching `next`: rank[v] = position of v in that order,
// UINT32_MAX for sites never processed.
bool prim_rank(const Graph& g, const uint32_t* outlets, uint32_t n_out, uint32_t* rank) {
    RustMinHeap heap;
    heap.d.reserve(g.n);
    for (uint32_t v = 0; v < g.n; ++v) rank[v] = UINT32_MAX;
    for (uint32_t o = 0; o < n_out; ++o) heap.push({outlets[o], 0.0});
    std::vector<uint8_t> visited(g.n, 0);
    uint32_t r = 0;
    Ridge el;
    while (heap.pop(el)) {
        uint32_t i = el.index;
        if (visited[i]) continue;
        for (uint32_t s = g.row_ptr[i]; s < g.row_ptr[i + 1]; ++s) {
            uint32_t j = g.col[s];
            if (visited[j]) continue;
            heap.push({j, g.len[s]});
        }
        visited[i] = 1;
        rank[i] = r++;
    }
    return !heap.nan_seen;
}

// The same lake re-routing expressed through `rank`: lake L (a basin whose root is
// not an outlet) is re-routed the first time the heap processes a site adjacent to
// it, i.e. through v* = argmin rank over sites v outside L with a neighbour in L,
// and j* = the first entry of v*'s row that lies in L.  The path j* -> bottom(L) is
// reversed and next[j*] = v*.  Lakes never touch each other's paths, so the order
// in which lakes are handled does not matter.
void remove_lakes_rank(const Graph& g, const uint8_t* is_outlet, const uint32_t* subroot,
                       const uint32_t* rank, uint32_t* next /* in/out */) {
    std::vector<uint64_t> best(g.n, UINT64_MAX);
    for (uint32_t v = 0; v < g.n; ++v) {
        if (rank[v] == UINT32_MAX) continue;
        for (uint32_t s = g.row_ptr[v]; s < g.row_ptr[v + 1]; ++s) {
            uint32_t L = subroot[g.col[s]];
            if (is_outlet[L] || L == subroot[v]) continue;
            uint64_t key = ((uint64_t)rank[v] << 32) | (uint64_t)(s - g.row_ptr[v]);
            if (key < best[L]) best[L] = key;
        }
    }
    std::vector<uint32_t> site_of_rank(g.n, UINT32_MAX);
    for (uint32_t v = 0; v < g.n; ++v)
        if (rank[v] != UINT32_MAX) site_of_rank[rank[v]] = v;
    for (uint32_t L = 0; L < g.n; ++L) {
        if (best[L] == UINT64_MAX) continue;
        uint32_t v = site_of_rank[best[L] >> 32];
        uint32_t j = g.col[g.row_ptr[v] + (uint32_t)(best[L] & 0xffffffffu)];
        uint32_t k = j, nk = v;
        while (next[k] != k) {
            uint32_t tmp = next[k];
            next[k] = nk;
            nk = k;
            k = tmp;
        }
        next[k] = nk;
    }
}

// drainage_basin.rs:13-36: BFS from `outlet` over donors (sites whose next is the
// visited site), donors taken in the visited site's adjacency order.
void drainage_basin(const Graph& g, const uint32_t* next, uint32_t outlet,
                    std::vector<uint32_t>& trav) {
    trav.clear();
    trav.push_back(outlet);
    size_t i = 0;
    while (true) {
        uint32_t it = trav[i];
        for (uint32_t s = g.row_ptr[it]; s < g.row_ptr[it + 1]; ++s) {
            uint32_t jt = g.col[s];
            if (next[jt] == it) trav.push_back(jt);
        }
        ++i;
        if (i >= trav.size()) break;
    }
}

struct Params {
    const double* k;       // erodibility
    const double* u;       // uplift rate
    const double* tanms;   // tan(max_slope) per site, NaN when max_slope is None
    bool use_pow;          // drainage^0.5 via pow() instead of sqrt()
};

// generator.rs:144-203: one pass of drainage area, response time and elevation
// over every outlet basin, in outlet-list order.  Returns `changed`.
bool tree_pass(const Graph& g, const uint32_t* next, const uint32_t* outlets, uint32_t n_out,
               const Params& p, double* elev, double* drain, double* resp,
               std::vector<uint32_t>& trav) {
    for (uint32_t i = 0; i < g.n; ++i) { drain[i] = g.area[i]; resp[i] = 0.0; }
    bool changed = false;
    for (uint32_t oi = 0; oi < n_out; ++oi) {
        uint32_t outlet = outlets[oi];
        drainage_basin(g, next, outlet, trav);
        for (size_t t = trav.size(); t-- > 0;) {           // for_each_downstream
            uint32_t i = trav[t];
            uint32_t j = next[i];
            if (j != i) drain[j] += drain[i];
        }
        for (size_t t = 0; t < trav.size(); ++t) {          // response times
            uint32_t i = trav[t];
            uint32_t j = next[i];
            double distance = edge_length_or_one(g, i, j);
            double a = p.use_pow ? std::pow(drain[i], 0.5) : std::sqrt(drain[i]);
            double celerity = p.k[i] * a;
            resp[i] += resp[j] + 1.0 / celerity * distance;
        }
        for (size_t t = 0; t < trav.size(); ++t) {          // elevations
            uint32_t i = trav[t];
            double dt = resp[i] - resp[outlet];
            double new_e = elev[outlet] + p.u[i] * (dt > 0.0 ? dt : 0.0);
            double tanv = p.tanms[i];
            if (!std::isnan(tanv)) {
                uint32_t j = next[i];
                double distance = edge_length_or_one(g, i, j);
                double slope = (new_e - elev[j]) / distance;
                if (slope > tanv) new_e = elev[j] + tanv * distance;
            }
            changed |= (new_e != elev[i]);
            elev[i] = new_e;
        }
    }
    return changed;
}

}  // namespace

extern "C" {

// Per-site f64 samples of StdRng::seed_from_u64(seed) `gen::<f64>()`, from the
// `first`-th sample on.
void orc_rng_f64(uint64_t seed, uint64_t first, uint64_t count, double* out) {
    uint32_t key[8];
    seed_from_u64(seed, key);
    uint32_t blk[16];
    uint64_t cur_block = UINT64_MAX;
    for (uint64_t m = 0; m < count; ++m) {
        uint64_t idx = first + m;
        uint64_t b = idx >> 3;
        if (b != cur_block) { chacha_block(key, b, 0, 12, blk); cur_block = b; }
        uint32_t w = (uint32_t)(idx & 7) * 2;
        uint64_t v = (uint64_t)blk[w] | ((uint64_t)blk[w + 1] << 32);
        out[m] = (double)(v >> 11) * (1.0 / 9007199254740992.0);
    }
}

// Raw ChaCha block (for the published known-answer vectors).
void orc_chacha_block(const uint32_t key[8], uint64_t counter, uint64_t stream, int rounds,
                      uint32_t out[16]) {
    chacha_block(key, counter, stream, rounds, out);
}

void orc_seed_from_u64(uint64_t seed, uint32_t key[8]) { seed_from_u64(seed, key); }

// generator.rs:120-132: the outlet list (ascending sites with is_outlet, else the
// model's default outlets).  Returns the count written to `out` (capacity n or n_def).
uint32_t orc_resolve_outlets(uint32_t n, const uint8_t* is_outlet, const uint32_t* def,
                             uint32_t n_def, uint32_t* out) {
    uint32_t c = 0;
    for (uint32_t i = 0; i < n; ++i)
        if (is_outlet[i]) out[c++] = i;
    if (c == 0) {
        for (uint32_t i = 0; i < n_def; ++i) out[i] = def[i];
        c = n_def;
    }
    return c;
}

void orc_initial_tree(uint32_t n, const uint32_t* row_ptr, const uint32_t* col,
                      const double* len, const double* elev, const uint8_t* outlet_table,
                      uint32_t* next) {
    Graph g{n, row_ptr, col, len, nullptr};
    initial_stream_tree(g, elev, outlet_table, next);
}

int orc_roots(uint32_t n, const uint8_t* outlet_table, const uint32_t* next, uint32_t* subroot) {
    return roots_with_lakes(n, outlet_table, next, subroot) ? 1 : 0;
}

int orc_remove_lakes_heap(uint32_t n, const uint32_t* row_ptr, const uint32_t* col,
                          const double* len, const uint32_t* outlets, uint32_t n_out,
                          const uint32_t* subroot, uint32_t* next) {
    Graph g{n, row_ptr, col, len, nullptr};
    return remove_lakes_heap(g, outlets, n_out, subroot, next) ? 0 : -1;
}

int orc_prim_rank(uint32_t n, const uint32_t* row_ptr, const uint32_t* col, const double* len,
                  const uint32_t* outlets, uint32_t n_out, uint32_t* rank) {
    Graph g{n, row_ptr, col, len, nullptr};
    return prim_rank(g, outlets, n_out, rank) ? 0 : -1;
}

void orc_remove_lakes_rank(uint32_t n, const uint32_t* row_ptr, const uint32_t* col,
                           const uint8_t* outlet_table, const uint32_t* subroot,
                           const uint32_t* rank, uint32_t* next) {
    Graph g{n, row_ptr, col, nullptr, nullptr};
    remove_lakes_rank(g, outlet_table, subroot, rank, next);
}

// One drainage/response/elevation pass on a given receiver array.
int orc_tree_pass(uint32_t n, const uint32_t* row_ptr, const uint32_t* col, const double* len,
                  const double* area, const uint32_t* outlets, uint32_t n_out,
                  const double* k, const double* u, const double* tanms, int use_pow,
                  const uint32_t* next, double* elev, double* drain, double* resp) {
    Graph g{n, row_ptr, col, len, area};
    Params p{k, u, tanms, use_pow != 0};
    std::vector<uint32_t> trav;
    trav.reserve(n);
    return tree_pass(g, next, outlets, n_out, p, elev, drain, resp, trav) ? 1 : 0;
}

// generate() (generator.rs:90-213) on a CSR graph.
//   base, k, u:   per-site base_elevation, erodibility, uplift_rate
//   is_outlet:    per-site flag (u8); empty set -> default outlets
//   max_slope:    per-site max_slope in radians, NaN = None; nullptr = all None
//   max_iter:     0 = unset (u32::MAX)
//   flags bit 0:  pow() instead of sqrt() for drainage^0.5
//   flags bit 1:  rank-based lake re-routing instead of the heap (reformulation)
//   trace_*:      optional; receivers / elevations after each of the first
//                 trace_cap iterations ([trace_cap][n] row-major)
//   out_seconds:  optional; wall time of the iteration loop
// Returns 0, or -1 on a NaN edge length (the reference panics there).
int orc_generate(uint32_t n, const uint32_t* row_ptr, const uint32_t* col, const double* len,
                 const double* area, const uint32_t* default_outlets, uint32_t n_def,
                 const double* base, const double* k, const double* u,
                 const uint8_t* is_outlet, const double* max_slope, uint32_t max_iter,
                 int flags, double* out_elev, uint32_t* out_iters,
                 uint32_t trace_cap, uint32_t* trace_next, double* trace_elev,
                 uint8_t* trace_has_lake, double* out_seconds) {
    Graph g{n, row_ptr, col, len, area};
    std::vector<uint32_t> outlets(std::max(n, n_def));
    uint32_t n_out = orc_resolve_outlets(n, is_outlet, default_outlets, n_def, outlets.data());
    outlets.resize(n_out);

    std::vector<double> tanms(n);
    for (uint32_t i = 0; i < n; ++i)
        tanms[i] = (max_slope && !std::isnan(max_slope[i])) ? std::tan(max_slope[i]) : NAN;
    Params p{k, u, tanms.data(), (flags & 1) != 0};

    // generator.rs:134-138
    std::vector<double> noise(n);
    orc_rng_f64(0, 0, n, noise.data());
    for (uint32_t i = 0; i < n; ++i) out_elev[i] = base[i] + noise[i] * 2.220446049250313e-16;

    std::vector<uint8_t> table(n, 0);
    for (uint32_t o : outlets) table[o] = 1;
    std::vector<uint32_t> next(n), subroot(n), rank;
    std::vector<double> drain(n), resp(n);
    std::vector<uint32_t> trav;
    trav.reserve(n);
    bool use_rank = (flags & 2) != 0;
    if (use_rank) {
        rank.resize(n);
        if (!prim_rank(g, outlets.data(), n_out, rank.data())) return -1;
    }

    auto t0 = std::chrono::steady_clock::now();
    uint64_t limit = max_iter ? max_iter : UINT32_MAX;
    uint32_t iters = 0;
    for (uint64_t it = 0; it < limit; ++it) {
        ++iters;
        initial_stream_tree(g, out_elev, table.data(), next.data());
        bool has_lake = roots_with_lakes(n, table.data(), next.data(), subroot.data());
        if (has_lake) {
            if (use_rank) {
                remove_lakes_rank(g, table.data(), subroot.data(), rank.data(), next.data());
            } else if (!remove_lakes_heap(g, outlets.data(), n_out, subroot.data(), next.data())) {
                return -1;
            }
        }
        bool changed = tree_pass(g, next.data(), outlets.data(), n_out, p, out_elev,
                                 drain.data(), resp.data(), trav);
        if (it < trace_cap) {
            if (trace_next) std::memcpy(trace_next + it * (uint64_t)n, next.data(), n * 4ull);
            if (trace_elev) std::memcpy(trace_elev + it * (uint64_t)n, out_elev, n * 8ull);
            if (trace_has_lake) trace_has_lake[it] = has_lake ? 1 : 0;
        }
        if (!changed) break;
    }
    auto t1 = std::chrono::steady_clock::now();
    if (out_seconds) *out_seconds = std::chrono::duration<double>(t1 - t0).count();
    *out_iters = iters;
    return 0;
}

// Counts sites where pow(x, 0.5) and sqrt(x) differ, for x in `vals`.
uint64_t orc_pow_sqrt_mismatches(const double* vals, uint64_t count) {
    uint64_t c = 0;
    for (uint64_t i = 0; i < count; ++i)
        if (std::pow(vals[i], 0.5) != std::sqrt(vals[i])) ++c;
    return c;
}

}  // extern "C"
