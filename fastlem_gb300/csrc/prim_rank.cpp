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

#include <cmath>
#include <cstdint>
#include <vector>

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
}  // namespace

// rank[v] = index of v in the processing order, UINT32_MAX for sites the traversal
// never reaches.  Returns false when a NaN key was pushed (the reference panics).
bool lake_heap_rank(uint32_t n, const uint32_t* row_ptr, const uint32_t* col, const double* len,
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

}  // namespace fl
