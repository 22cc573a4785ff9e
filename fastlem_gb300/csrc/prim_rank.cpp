// prim_rank.cpp -- host computation of the lake-heap processing order.
//
// fastlem re-routes lakes with a min-heap traversal started from the outlets
// (src/lem/stream_tree.rs:175-243).  Which sites the heap pushes and pops does not
// depend on the receivers: every unvisited neighbour of a processed site is pushed
// with its edge length as key, whatever `next` holds.  So the order in which sites
// are processed ("rank") is a function of (graph, edge lengths, outlet list) and is
// computed here once per generate() call -- cached per model and outlet list -- and
// the per-iteration GPU step only needs it to find, for every lake, the first
// processed site adjacent to it.
//
// The heap must break ties exactly like std::collections::BinaryHeap with the
// reversed `Ord` of RidgeElement (stream_tree.rs:34-38): outlets all enter with key
// 0.0 and equal edge lengths occur, so the pop order among equal keys is decided
// by the heap's sift rules:
//   push:  append, then move the new element up while its key is strictly smaller
//          than its parent's.
//   pop:   remove the last element and put it at the root in place of the popped
//          one; walk the hole down to a leaf, at each level taking the right child
//          when right.key <= left.key (a lone last child is taken too); then move
//          the element up from there while strictly smaller than its parent.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <unordered_map>
#include <vector>

#include "fastlem_gb300.h"

namespace fl {

namespace {
struct Entry {
    double key;
    uint32_t site;
};

class LakeHeap {
  public:
    explicit LakeHeap(size_t cap) { v_.reserve(cap); }
    bool empty() const { return v_.empty(); }
    bool nan_seen() const { return nan_; }
    double top_key() const { return v_.front().key; }
    template <class F>
    void drain(F f) {
        for (const Entry& e : v_) f(e.site, e.key);
        v_.clear();
    }

    void push(uint32_t site, double key) {
        if (std::isnan(key)) nan_ = true;
        v_.push_back({key, site});
        float_up(0, v_.size() - 1);
    }
    uint32_t pop() {
        Entry top = v_.front();
        Entry last = v_.back();
        v_.pop_back();
        if (!v_.empty()) {
            v_[0] = last;
            size_t pos = 0, end = v_.size();
            size_t c = 1;
            while (end >= 2 && c <= end - 2) {
                if (v_[c + 1].key <= v_[c].key) ++c;
                v_[pos] = v_[c];
                pos = c;
                c = 2 * pos + 1;
            }
            if (c == end - 1) {
                v_[pos] = v_[c];
                pos = c;
            }
            v_[pos] = last;
            float_up(0, pos);
        }
        return top.site;
    }

  private:
    void float_up(size_t start, size_t pos) {
        Entry e = v_[pos];
        while (pos > start) {
            size_t parent = (pos - 1) / 2;
            if (!(e.key < v_[parent].key)) break;
            v_[pos] = v_[parent];
            pos = parent;
        }
        v_[pos] = e;
    }
    std::vector<Entry> v_;
    bool nan_ = false;
};

// The reference's traversal, entry for entry: every unvisited neighbour pushed, stale
// entries skipped.  rank[v] = index of v in the processing order, UINT32_MAX for
// sites never reached.  Returns false when a NaN key was pushed (the reference panics).
bool exact_rank(uint32_t n, const uint32_t* row_ptr, const uint32_t* col, const double* len,
                const uint32_t* outlets, uint32_t n_out, uint32_t* rank) {
    LakeHeap heap((size_t)n + n_out);
    std::vector<uint8_t> visited(n, 0);
    for (uint32_t v = 0; v < n; ++v) rank[v] = UINT32_MAX;
    for (uint32_t o = 0; o < n_out; ++o) heap.push(outlets[o], 0.0);
    uint32_t r = 0;
    while (!heap.empty()) {
        uint32_t i = heap.pop();
        if (visited[i]) continue;
        for (uint32_t s = row_ptr[i]; s < row_ptr[i + 1]; ++s) {
            uint32_t j = col[s];
            if (!visited[j]) heap.push(j, len[s]);
        }
        visited[i] = 1;
        rank[i] = r++;
    }
    return !heap.nan_seen();
}

// Indexed 4-ary min-heap with one entry per site (key = the smallest pushed key).
class SiteHeap {
  public:
    explicit SiteHeap(uint32_t n) : pos_(n, kAbsent) {}
    bool empty() const { return k_.empty(); }
    double min_key() const { return k_[0]; }
    void push_or_decrease(uint32_t site, double key) {
        uint32_t p = pos_[site];
        if (p == kAbsent) {
            p = (uint32_t)k_.size();
            k_.push_back(key);
            s_.push_back(site);
            pos_[site] = p;
        } else if (key < k_[p]) {
            k_[p] = key;
        } else {
            return;
        }
        up(p);
    }
    void pop(double* key, uint32_t* site) {
        *key = k_[0];
        *site = s_[0];
        pos_[s_[0]] = kAbsent;
        const double lk = k_.back();
        const uint32_t ls = s_.back();
        k_.pop_back();
        s_.pop_back();
        if (k_.empty()) return;
        uint32_t p = 0;
        const uint32_t m = (uint32_t)k_.size();
        while (true) {
            const uint32_t c0 = 4 * p + 1;
            if (c0 >= m) break;
            uint32_t b = c0;
            const uint32_t ce = std::min(c0 + 4, m);
            for (uint32_t c = c0 + 1; c < ce; ++c)
                if (k_[c] < k_[b]) b = c;
            if (!(k_[b] < lk)) break;
            k_[p] = k_[b];
            s_[p] = s_[b];
            pos_[s_[p]] = p;
            p = b;
        }
        k_[p] = lk;
        s_[p] = ls;
        pos_[ls] = p;
    }

  private:
    static constexpr uint32_t kAbsent = UINT32_MAX;
    void up(uint32_t p) {
        const double key = k_[p];
        const uint32_t site = s_[p];
        while (p > 0) {
            const uint32_t q = (p - 1) / 4;
            if (!(key < k_[q])) break;
            k_[p] = k_[q];
            s_[p] = s_[q];
            pos_[s_[p]] = p;
            p = q;
        }
        k_[p] = key;
        s_[p] = site;
        pos_[site] = p;
    }
    std::vector<double> k_;
    std::vector<uint32_t> s_;
    std::vector<uint32_t> pos_;
};

// The same order, faster, when it is decided by keys alone.  The heap's arrangement
// only matters when two live entries share the smallest key: the outlets (all 0.0)
// do, so the traversal runs the reference's heap while 0.0 keys are queued.  After
// that a site's live entries count through their smallest key only (a site is
// processed at its first pop, later entries are stale), so an indexed heap with one
// entry per site gives the same order as long as each popped key is strictly the
// smallest.  Returns false (nothing decided) at the first tie or NaN.
bool keyed_rank(uint32_t n, const uint32_t* row_ptr, const uint32_t* col, const double* len,
                const uint32_t* outlets, uint32_t n_out, uint32_t* rank) {
    LakeHeap heap((size_t)n_out + 64);
    std::vector<uint8_t> visited(n, 0);
    for (uint32_t v = 0; v < n; ++v) rank[v] = UINT32_MAX;
    for (uint32_t o = 0; o < n_out; ++o) heap.push(outlets[o], 0.0);
    uint32_t r = 0;
    while (!heap.empty() && heap.top_key() == 0.0) {
        uint32_t i = heap.pop();
        if (visited[i]) continue;
        for (uint32_t s = row_ptr[i]; s < row_ptr[i + 1]; ++s) {
            uint32_t j = col[s];
            if (!visited[j]) heap.push(j, len[s]);
        }
        visited[i] = 1;
        rank[i] = r++;
    }
    if (heap.nan_seen()) return false;
    SiteHeap sh(n);
    heap.drain([&](uint32_t site, double key) {
        if (!visited[site]) sh.push_or_decrease(site, key);
    });
    while (!sh.empty()) {
        double key;
        uint32_t i;
        sh.pop(&key, &i);
        if (!sh.empty() && !(key < sh.min_key())) return false;   // a tie
        visited[i] = 1;
        rank[i] = r++;
        for (uint32_t s = row_ptr[i]; s < row_ptr[i + 1]; ++s) {
            const uint32_t j = col[s];
            if (visited[j]) continue;
            if (std::isnan(len[s])) return false;
            sh.push_or_decrease(j, len[s]);
        }
    }
    return true;
}

}  // namespace

// The tied prefix of the traversal: the sites the reference's heap processes while the
// smallest queued key is 0.0 (the outlets, in the order its arrangement gives them, and
// any site reached over a zero-length edge), in processing order.  With every edge
// longer than zero the rest of the order is decided by keys alone (the GPU rank).
// Returns false when a NaN key was pushed.
bool lake_rank_prefix(uint32_t n, const uint32_t* row_ptr, const uint32_t* col,
                      const double* len, const uint32_t* outlets, uint32_t n_out,
                      std::vector<uint32_t>& order) {
    LakeHeap heap((size_t)n_out + 64);
    std::vector<uint8_t> visited(n, 0);
    order.clear();
    for (uint32_t o = 0; o < n_out; ++o) heap.push(outlets[o], 0.0);
    while (!heap.empty() && heap.top_key() == 0.0) {
        uint32_t i = heap.pop();
        if (visited[i]) continue;
        for (uint32_t s = row_ptr[i]; s < row_ptr[i + 1]; ++s) {
            uint32_t j = col[s];
            if (!visited[j]) heap.push(j, len[s]);
        }
        visited[i] = 1;
        order.push_back(i);
    }
    return !heap.nan_seen();
}

// The same tied prefix from the outlets' own rows only (row i of orow / ocol / olen
// belongs to outlets[i], offsets absolute): with every edge longer than zero only
// outlets are processed at key 0.0.  Returns 0, 1 when a NaN key was pushed, 2 when a
// site that is not an outlet comes up at key 0.0 (a zero-length edge: the full graph
// is needed).
int lake_rank_prefix_rows(uint32_t n, const uint32_t* outlets, uint32_t n_out,
                          const uint32_t* orow, const uint32_t* ocol, const double* olen,
                          std::vector<uint32_t>& order) {
    std::unordered_map<uint32_t, uint32_t> at;            // site -> its first list position
    at.reserve(n_out * 2 + 1);
    for (uint32_t o = 0; o < n_out; ++o) at.emplace(outlets[o], o);
    // only outlets are processed here, so "visited" lives on their list positions
    std::vector<uint8_t> done(n_out, 0);
    auto visited = [&](uint32_t site) {
        const auto it = at.find(site);
        return it != at.end() && done[it->second];
    };
    (void)n;
    LakeHeap heap((size_t)n_out + 64);
    order.clear();
    for (uint32_t o = 0; o < n_out; ++o) heap.push(outlets[o], 0.0);
    while (!heap.empty() && heap.top_key() == 0.0) {
        const uint32_t i = heap.pop();
        const auto it = at.find(i);
        if (it == at.end()) return 2;
        const uint32_t p = it->second;
        if (done[p]) continue;
        for (uint32_t s = orow[p]; s < orow[p + 1]; ++s) {
            const uint32_t j = ocol[s];
            if (!visited(j)) heap.push(j, olen[s]);
        }
        done[p] = 1;
        order.push_back(i);
    }
    return heap.nan_seen() ? 1 : 0;
}

// rank[v] = index of v in the processing order, UINT32_MAX for sites the traversal
// never reaches.  Returns false when a NaN key was pushed (the reference panics).
bool lake_heap_rank(uint32_t n, const uint32_t* row_ptr, const uint32_t* col, const double* len,
                    const uint32_t* outlets, uint32_t n_out, uint32_t* rank) {
    if (keyed_rank(n, row_ptr, col, len, outlets, n_out, rank)) return true;
    return exact_rank(n, row_ptr, col, len, outlets, n_out, rank);
}

}  // namespace fl

extern "C" int fl_lake_rank(uint32_t n, const uint32_t* row_ptr, const uint32_t* col,
                            const double* len, const uint32_t* outlets, uint32_t n_out,
                            uint32_t* rank) {
    if (!row_ptr || (!col && n && row_ptr[n]) || (!len && n && row_ptr[n]) || !rank ||
        (n_out && !outlets))
        return FL_ERR_INVALID_ARGUMENT;
    for (uint32_t o = 0; o < n_out; ++o)
        if (outlets[o] >= n) return FL_ERR_INVALID_ARGUMENT;
    for (uint64_t s = 0; s < (n ? row_ptr[n] : 0); ++s)
        if (col[s] >= n) return FL_ERR_INVALID_ARGUMENT;
    return fl::lake_heap_rank(n, row_ptr, col, len, outlets, n_out, rank)
               ? FL_OK
               : FL_ERR_INVALID_ARGUMENT;
}
