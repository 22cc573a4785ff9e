// solver.cu -- GB300 (sm_103a) landscape-evolution solve and its C ABI.
//
// One fl_graph = one terrain model resident in HBM (CSR adjacency in the
// reference's per-row insertion order, cell areas) plus the solver workspace.
// fl_generate() runs fastlem's fixed-point loop (src/lem/generator.rs:140-210) on the
// device:
//   1. receivers      steepest-descent neighbour, first maximum wins (stream_tree.rs:109-137)
//   2. lakes          only when some non-outlet site has no lower neighbour:
//                     basin labels by pointer jumping (stream_tree.rs:139-173), then per
//                     lake the first site processed by the reference's lake heap that
//                     touches it -- a packed 64-bit atomicMin of (heap rank << 32 | slot)
//                     -- and the reversal of the receiver path from there to the lake
//                     bottom (stream_tree.rs:175-243)
//   3. basin pass     drainage area bottom-up, response time and elevation top-down,
//                     `changed` flag (generator.rs:144-203; basin.cu)
// All FP64 arithmetic is written with explicit round-to-nearest intrinsics, so no
// multiply-add is ever contracted and every value is bit-identical to the
// reference's evaluation order.

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdlib>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "common.cuh"
#include "fastlem_gb300.h"
#include "kernels.h"
#include "rng.h"

namespace fl {
bool lake_heap_rank(uint32_t n, const uint32_t* row_ptr, const uint32_t* col, const double* len,
                    const uint32_t* outlets, uint32_t n_out, uint32_t* rank);
int lake_rank_prefix_rows(uint32_t n, const uint32_t* outlets, uint32_t n_out,
                          const uint32_t* orow, const uint32_t* ocol, const double* olen,
                          std::vector<uint32_t>& order);
}

namespace {

using fl::kNone;
using fl::kNoKey;
using fl::kThreads;
using namespace fl;
constexpr double kEpsilon = 2.220446049250313e-16;   // f64::EPSILON
// Kahn rounds stop when the ready frontier is narrower than this; it also bounds
// the number of skeleton chains (one co-resident thread each).
// The Kahn rounds stop once fewer sites than this are ready (n / 512, between the two
// bounds); the rest (the deep part of the rivers) goes to the skeleton chains, walked by
// persistent warps.  Narrow rounds cost a grid barrier each, a wide skeleton costs its
// build and the chain hand-offs.
constexpr uint32_t kKahnMinWidth = 65536;
constexpr uint32_t kKahnMinWidthLow = 8192;
// ... and for the first passes of a generate(): the chains follow the largest drainage
// area of the previous pass, which is only the cell area on the first pass and a poor
// guide on the second, and a wide skeleton cut into badly chosen chains walks slowly.
constexpr uint32_t kKahnMinWidthEarly = 8192;
constexpr uint32_t kEarlyPasses = 2;

// The stop width for a model of n sites (packed: several terrains).
uint32_t kahn_min_width(uint32_t n, bool packed = false) {
    const uint32_t w = fl::shape_for(n, packed).kahn_min_width;
    if (w) return w;
    return std::max(kKahnMinWidthLow, std::min(kKahnMinWidth, n / 512));
}

thread_local std::string g_err;

std::mutex& status_mu() {
    static std::mutex m;
    return m;
}
std::vector<int*>& status_free() {
    static std::vector<int*> v;
    return v;
}

void set_err(const char* what, cudaError_t e) {
    char buf[256];
    snprintf(buf, sizeof buf, "%s: %s", what, cudaGetErrorString(e));
    g_err = buf;
}

#define FL_CU(call)                                                               \
    do {                                                                          \
        cudaError_t e_ = (call);                                                  \
        if (e_ != cudaSuccess) {                                                  \
            set_err(#call, e_);                                                   \
            return e_ == cudaErrorMemoryAllocation ? FL_ERR_OUT_OF_MEMORY : FL_ERR_CUDA; \
        }                                                                         \
    } while (0)

#define FL_TRY(expr)            \
    do {                        \
        int rc_ = (expr);       \
        if (rc_ != FL_OK) return rc_; \
    } while (0)

inline unsigned blocks_for(uint64_t n, int t = kThreads) {
    uint64_t b = (n + t - 1) / t;
    return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(b, 1u << 30));
}

// ---------------------------------------------------------------------------
// Kernels
// ---------------------------------------------------------------------------

// noise[i] = sample i of StdRng::seed_from_u64(0).gen::<f64>() (generator.rs:134-137),
// in the caller's site order.  One thread per ChaCha block = 8 consecutive samples.
__global__ void k_noise(uint32_t n, double* __restrict__ noise) {
    uint64_t b = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (b * 8 >= n) return;
    uint32_t key[8];
    fl::key_from_u64(0, key);
    uint32_t w[16];
    fl::chacha12_block(key, b, w);
#pragma unroll
    for (int m = 0; m < 8; ++m) {
        uint64_t i = b * 8 + m;
        if (i < n) noise[i] = fl::u64_to_unit_f64((uint64_t)w[2 * m] | ((uint64_t)w[2 * m + 1] << 32));
    }
}

// elev[j] = base[j] + noise[perm[j]] * f64::EPSILON (generator.rs:135-138), device order.
__global__ void k_initial_elevation(uint32_t n, const uint32_t* __restrict__ perm,
                                    const double* __restrict__ base,
                                    const double* __restrict__ noise, double* __restrict__ elev) {
    uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < n) elev[j] = __dadd_rn(base[j], __dmul_rn(noise[perm[j]], kEpsilon));
}

// dst[j] = src[idx[j]]: caller order <-> device order.
__global__ void k_gather_f64(uint32_t n, const uint32_t* __restrict__ idx,
                             const double* __restrict__ src, double* __restrict__ dst) {
    uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < n) dst[j] = src[idx[j]];
}

__global__ void k_rng_f64(uint64_t seed, uint64_t first, uint64_t count, double* out) {
    uint64_t m = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= count) return;
    uint32_t key[8];
    fl::key_from_u64(seed, key);
    uint64_t idx = first + m;
    uint32_t w[16];
    fl::chacha12_block(key, idx >> 3, w);
    uint32_t k = (uint32_t)(idx & 7) * 2;
    out[m] = fl::u64_to_unit_f64((uint64_t)w[k] | ((uint64_t)w[k + 1] << 32));
}

// Length of edge (i, j) as `graph.has_edge(i, j)` reports it: the first entry of
// row i with column j, else 1.0 (generator.rs:164-171).
__device__ __forceinline__ double edge_len_or_one(const uint32_t* __restrict__ row,
                                                  const uint32_t* __restrict__ col,
                                                  const double* __restrict__ len, uint32_t i,
                                                  uint32_t j) {
    for (uint32_t s = row[i], e = row[i + 1]; s < e; ++s)
        if (col[s] == j) return len[s];
    return 1.0;
}

__global__ void k_copy_u32(uint32_t n, const uint32_t* __restrict__ a, uint32_t* __restrict__ b) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = a[i];
}

// Basin labels of the receivers by pointer jumping, every round in one cooperative
// launch: lab = next, then lab[i] = lab[lab[i]] until no label moves.  Roots
// (next[r] == r) are fixed points, so after ceil(log2(depth)) rounds every site holds
// its basin root (stream_tree.rs:139-173, "subroot"); the rounds synchronise on the
// grid barrier and a rotating "moved" word, and the result ends in lab.  With a gate,
// nothing runs unless *gate is set (the receivers found a lake), so the launch can be
// enqueued before the host knows.
__global__ void k_labels(uint32_t n, const uint32_t* __restrict__ next, uint32_t* lab,
                         uint32_t* lab2, const int* gate, int* flags) {
    if (gate && *gate == 0) return;                      // the same verdict for every block
    const uint32_t gtid = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = gtid; i < n; i += stride) lab[i] = next[i];
    if (!grid_barrier(flags)) return;
    uint32_t* cur = lab;
    uint32_t* out = lab2;
    for (uint32_t round = 0; round < 64; ++round) {
        int* moved_word = &flags[kJump0 + round % 3];
        if (gtid == 0) flags[kJump0 + (round + 1) % 3] = 0;
        bool moved = false;
        for (uint32_t i = gtid; i < n; i += stride) {
            const uint32_t l = __ldcg(&cur[i]);
            const uint32_t ll = __ldcg(&cur[l]);
            out[i] = ll;
            moved |= ll != l;
        }
        if (__syncthreads_or(moved) && threadIdx.x == 0) atomicOr(moved_word, 1);
        if (!grid_barrier(flags)) return;
        uint32_t* t = cur;
        cur = out;
        out = t;
        if (ld_acquire(moved_word) == 0) {
            if (cur != lab)
                for (uint32_t i = gtid; i < n; i += stride) lab[i] = __ldcg(&cur[i]);
            return;
        }
    }
    if (gtid == 0) set_error(flags, kErrForest);          // a receiver cycle
}

// best[L] = no key, for every site (gated like k_labels).
__global__ void k_clear_keys(uint32_t n, unsigned long long* __restrict__ best,
                             const int* gate) {
    if (gate && *gate == 0) return;
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) best[i] = kNoKey;
}

// For every site v the lake heap processes (rank[v] != none) and every neighbour j
// lying in a lake L other than v's own basin: best[L] = min((rank[v] << 32) | slot).
// The minimum is the first processed site touching L and, within its row, the
// first entry in L -- the pair at which the reference flips L (stream_tree.rs:204-230).
__global__ void k_lake_keys(uint32_t n, const uint32_t* __restrict__ row,
                            const uint32_t* __restrict__ col, const uint32_t* __restrict__ rank,
                            const uint32_t* __restrict__ lab, const uint8_t* __restrict__ outlet,
                            unsigned long long* __restrict__ best, const int* gate) {
    if (gate && *gate == 0) return;
    uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    uint32_t r = rank[v];
    if (r == kNone) return;
    uint32_t lv = lab[v];
    const uint32_t s0 = row[v], s1 = row[v + 1];
    for (uint32_t s = s0; s < s1; ++s) {
        uint32_t L = lab[col[s]];
        if (outlet[L] || L == lv) continue;
        unsigned long long key = ((unsigned long long)r << 32) | (unsigned long long)(s - s0);
        if (key < best[L]) atomicMin(&best[L], key);
    }
}

// One thread per lake: reverse the receiver path from j* to the lake bottom and
// hang it on v* (stream_tree.rs:214-228).  Lakes are disjoint and each flip only
// touches its own lake's sites, so lakes run independently.
__global__ void k_lake_flip(uint32_t n, const uint32_t* __restrict__ row,
                            const uint32_t* __restrict__ col, const double* __restrict__ len,
                            const unsigned long long* __restrict__ best,
                            const uint32_t* __restrict__ site_of_rank, uint32_t* next,
                            double* rlen, int* flags, const int* gate) {
    if (gate && *gate == 0) return;
    uint32_t L = blockIdx.x * blockDim.x + threadIdx.x;
    if (L >= n) return;
    unsigned long long key = best[L];
    if (key == kNoKey) return;
    uint32_t v = site_of_rank[key >> 32];
    uint32_t j = col[row[v] + (uint32_t)(key & 0xffffffffu)];
    uint32_t k = j, nk = v;
    for (uint32_t steps = 0;; ++steps) {
        if (steps > n) {             // a cycle: cannot happen on a descent forest
            set_error(flags, kErrForest);
            return;
        }
        uint32_t nx = next[k];
        if (nx == k) break;
        next[k] = nk;
        rlen[k] = edge_len_or_one(row, col, len, k, nk);
        nk = k;
        k = nx;
    }
    next[k] = nk;
    rlen[k] = edge_len_or_one(row, col, len, k, nk);
}

__global__ void k_fill_nan(uint32_t n, double* __restrict__ d) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) d[i] = __longlong_as_double(0x7ff8000000000000ll);
}

__global__ void k_mark(uint32_t m, const uint32_t* __restrict__ ids, uint8_t* __restrict__ table) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m) table[ids[i]] = 1;
}

// Response times out of the per-site top-down records (probes).
__global__ void k_rec_times(uint32_t n, const fl::TRec* __restrict__ rec, double* __restrict__ t) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) t[i] = rec[i].t;
}

__global__ void k_fill_f64(uint32_t n, double* __restrict__ a, const double* __restrict__ src) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = src ? src[i] : 0.0;
}

// Packed terrains: a terrain whose elevations did not change in iteration `iter`
// (1-based) would have stopped there alone; its first such iteration is recorded, and
// the per-terrain "changed" words are cleared for the next iteration.
__global__ void k_terrain_iters(uint32_t terrains, int* __restrict__ tchg,
                                uint32_t* __restrict__ titer, uint32_t iter) {
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= terrains) return;
    if (!tchg[t] && titer[t] == 0) titer[t] = iter;
    tchg[t] = 0;
}

// Blocks of `block` threads at which `kernel` is co-resident on the current device,
// at most cap_per_sm per SM.
unsigned coop_blocks(const void* kernel, unsigned block, unsigned cap_per_sm) {
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, (int)block, 0);
    if (per < 1) per = 1;
    return (unsigned)(sms * std::min<unsigned>((unsigned)per, cap_per_sm));
}

}  // namespace

namespace fl {
void set_last_error(const char* msg) { g_err = msg ? msg : ""; }

Tuning& tuning() {
    static Tuning t = [] {
        Tuning d;
        auto env = [](const char* name, long lo, long hi, long dflt) {
            if (const char* v = std::getenv(name)) {
                const long x = std::strtol(v, nullptr, 10);
                if (x >= lo && x <= hi) return x;
            }
            return dflt;
        };
        const long ilp = env("FL_LOW_ILP", 1, 4, -1);
        d.low_ilp = ilp < 0 ? -1 : ilp >= 4 ? 4 : ilp >= 2 ? 2 : 1;
        d.walk_per_sm = (int)env("FL_WALK_PER_SM", 0, 64, -1);
        d.kahn_min_width = env("FL_KAHN_MIN_WIDTH", 256, 1l << 24, -1);
        d.gpu_rank = env("FL_GPU_RANK", 0, 1, 1) != 0;
        d.sized_grids = (int)env("FL_SIZED_GRIDS", 0, 1, -1);
        return d;
    }();
    return t;
}

// The committed schedule (fastlem_gb300/schedule.json, written by the schedule sweep
// fastlem_gb300/autotune.py); a CPU test keeps the two equal.
const std::vector<ScheduleEntry>& schedule() {
    static const std::vector<ScheduleEntry> s = {
        // max_sites, packed, {low_ilp, walk_per_sm, kahn_min_width}
        {0x20000u, false, {4, 2, 512, false}},
        {0x80000u, false, {4, 0, 1024, true}},
        {0x200000u, false, {4, 0, 2048, true}},
        {0x7d0000u, false, {4, 0, 4096, true}},
        {0xffffffffu, false, {4, 4, 0, true}},
        {0xffffffffu, true, {2, 0, 0, true}},
    };
    return s;
}

Shape shape_for(uint32_t n, bool packed) {
    Shape sh{4, 0, 0, false};
    for (const ScheduleEntry& e : schedule())
        if (e.packed == packed && n <= e.max_sites) {
            sh = e.shape;
            break;
        }
    const Tuning& t = tuning();
    if (t.low_ilp > 0) sh.low_ilp = t.low_ilp;
    if (t.walk_per_sm >= 0) sh.walk_per_sm = (uint32_t)t.walk_per_sm;
    if (t.kahn_min_width >= 0) sh.kahn_min_width = (uint32_t)t.kahn_min_width;
    if (t.sized_grids >= 0) sh.sized_grids = t.sized_grids != 0;
    return sh;
}
}  // namespace fl

// ---------------------------------------------------------------------------
// Model handle
// ---------------------------------------------------------------------------
const char* const kKClassName[kcCount] = {
    "initial_elevation", "receivers", "lake_reroute", "basin_build", "kahn_rounds",
    "skeleton_rank", "skeleton_up", "response_w", "skeleton_down", "rounds_down", "misc"};

struct fl_graph {
    uint32_t n = 0;
    uint64_t nnz = 0;
    int device = 0;
    uint64_t dev_bytes = 0;   // device memory the model holds
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaEvent_t ev_status[2] = {nullptr, nullptr};   // an iteration's status copy is done
    // host copies used by the host-side lake-heap rank
    std::vector<uint32_t> h_row, h_col;
    std::vector<double> h_len;
    std::vector<uint32_t> def_outlets;
    // cached rank for one outlet list
    std::vector<uint32_t> rank_key;
    bool rank_valid = false;
    bool rank_uploaded = false;
    std::vector<uint32_t> h_rank;        // host-computed rank (empty when computed on the GPU)
    int rank_gpu = -1;                   // where the last rank was computed: 1 GPU, 0 host
    int sized_grids = -1;                // model-sized cooperative grids: -1 the schedule's
    double* h_stage = nullptr;           // page-locked staging array (many packed terrains)
    double rank_ms = 0.0;                // its host wall time
    // device order: perm[device index] = caller index, inv the reverse
    std::vector<uint32_t> perm, inv;
    uint32_t *d_perm = nullptr, *d_inv = nullptr;
    // packed terrains (batched form): terrain t owns caller and device sites
    // [site_off[t], site_off[t+1]) and default outlets [def_off[t], def_off[t+1]);
    // a single terrain has terrains == 1 and no per-site terrain array
    uint32_t terrains = 1;
    std::vector<uint32_t> site_off, def_off;
    uint32_t noise_n = 0;              // RNG samples a terrain needs (its site count)
    uint32_t* d_noise_idx = nullptr;   // device site -> its sample (index within its terrain)
    uint32_t* d_tid = nullptr;
    int* d_tchg = nullptr;
    uint32_t* d_titer = nullptr;   // per terrain: first iteration without a change (0: none yet)
    // page-locked copy of the status words and basin-pass bookkeeping, read once per
    // iteration
    int* h_status = nullptr;
    uint64_t host_syncs = 0;       // blocking stream synchronisations inside generate()
    // model (device)
    uint32_t *d_row = nullptr, *d_col = nullptr;
    double *d_len = nullptr, *d_area = nullptr;
    float* d_ilen = nullptr;   // 1/len per slot in f32 (receiver slope estimates)
    // parameters and iteration state (device)
    double *d_k = nullptr, *d_u = nullptr, *d_tan = nullptr, *d_base = nullptr, *d_elev = nullptr,
           *d_A = nullptr, *d_t = nullptr, *d_w = nullptr, *d_rlen = nullptr,
           *d_wa = nullptr, *d_wl = nullptr;
    // d_w / d_wa / d_wl hold the last pass's w and the A and receiver distance it came
    // from, for the current parameters (cleared whenever d_w is reused or k uploaded)
    bool w_valid = false;
    uint32_t *d_next = nullptr, *d_lab = nullptr, *d_lab2 = nullptr, *d_rank = nullptr,
             *d_sor = nullptr, *d_outlets = nullptr, *d_bas = nullptr;
    uint8_t* d_outlet = nullptr;
    unsigned long long* d_best = nullptr;
    int* d_flags = nullptr;
    // basin pass workspace (device)
    uint64_t* d_rtime = nullptr;
    fl::TRec* d_trec = nullptr;
    uint32_t *d_pending = nullptr, *d_hgt = nullptr, *d_order = nullptr, *d_roff = nullptr,
             *d_meta = nullptr, *d_sid = nullptr, *d_slist = nullptr, *d_desig = nullptr,
             *d_sptr0 = nullptr, *d_sdist0 = nullptr, *d_sptr1 = nullptr, *d_sdist1 = nullptr,
             *d_cid = nullptr, *d_cbot = nullptr, *d_clen = nullptr, *d_coff = nullptr,
             *d_layout = nullptr, *d_slot_chain = nullptr, *d_cbas = nullptr;
    double *d_pre = nullptr, *d_post = nullptr, *d_tokval = nullptr,
           *d_el = nullptr, *d_cto = nullptr, *d_ceo = nullptr;
    bool slope = false;
    uint32_t *d_kslot = nullptr, *d_cpar = nullptr, *d_cqp = nullptr, *d_cdep = nullptr,
             *d_cpar1 = nullptr, *d_cdep1 = nullptr, *d_chist = nullptr, *d_corder = nullptr,
             *d_corder_up = nullptr;
    fl::SlotRec* d_rec = nullptr;
    fl::SlotInfo* d_info = nullptr;
    uint32_t *d_tokslot = nullptr, *d_pend = nullptr;
    uint8_t* d_needl = nullptr;
    uint64_t* d_push = nullptr;
    uint32_t tok_cap = 0;
    int *d_bu_done = nullptr, *d_td_need = nullptr, *d_td_done = nullptr;
    uint32_t max_rounds = 0, kahn_min_width = kKahnMinWidth;
    uint32_t passes = 0;   // basin passes since the drainage areas were reset
    int stamp = 0;
    uint32_t last_meta[kMetaCount] = {};
    // instrumentation: launches / algorithmic bytes always, device time when enabled
    bool timing = false;
    uint64_t k_launches[kcCount] = {};
    double k_ms[kcCount] = {};
    double k_bytes[kcCount] = {};
    std::vector<cudaEvent_t> ev_pool;
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> ev_pending;
    cudaEvent_t ev_open = nullptr;
};

namespace {

// Device bytes allocated on this thread are added here while a model is being created,
// from the stream-ordered pool on its stream: creating or destroying a model then never
// synchronises the device (solves of other models keep running).
thread_local uint64_t* t_alloc_bytes = nullptr;
thread_local cudaStream_t t_alloc_stream = nullptr;

// Freed model memory stays in the device's pool for the next model (no release to the
// driver, which would synchronise); set once per device.
void keep_pool_memory() {
    static std::mutex mu;
    static std::vector<int> done;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return;
    std::lock_guard<std::mutex> lk(mu);
    if (std::find(done.begin(), done.end(), dev) != done.end()) return;
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
        uint64_t thr = ~0ull;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
    done.push_back(dev);
}

template <class T>
int dalloc(T** p, uint64_t count) {
    const uint64_t bytes = std::max<uint64_t>(1, count) * sizeof(T);
    FL_CU(cudaMallocAsync((void**)p, bytes, t_alloc_stream));
    if (t_alloc_bytes) *t_alloc_bytes += bytes;
    return FL_OK;
}

// Page-locked 256-byte status blocks, recycled (freeing page-locked memory may
// synchronise the device).
// A page-locked status block: [0, kStatusSlot) for sync_status, then two slots of
// flags + bookkeeping words for the pipelined iterations.
constexpr uint32_t kStatusSlot = 64;
static_assert(kNumFlags + kMetaCount <= kStatusSlot, "status slot too small");

int* status_block_get() {
    std::lock_guard<std::mutex> lk(status_mu());
    auto& fl = status_free();
    if (!fl.empty()) {
        int* b = fl.back();
        fl.pop_back();
        return b;
    }
    void* p = nullptr;
    if (cudaHostAlloc(&p, 3 * kStatusSlot * sizeof(int), cudaHostAllocPortable) != cudaSuccess)
        return nullptr;
    return (int*)p;
}
void status_block_put(int* b) {
    if (!b) return;
    std::lock_guard<std::mutex> lk(status_mu());
    status_free().push_back(b);
}

void free_graph(fl_graph* g) {
    if (!g) return;
    void* ptrs[] = {g->d_row, g->d_col, g->d_len, g->d_area, g->d_k, g->d_u, g->d_tan, g->d_base,
                    g->d_elev, g->d_A, g->d_t, g->d_w, g->d_rlen, g->d_next, g->d_lab, g->d_lab2,
                    g->d_rank, g->d_sor, g->d_outlets, g->d_bas, g->d_outlet, g->d_best,
                    g->d_flags, g->d_pending, g->d_hgt, g->d_order, g->d_roff, g->d_meta,
                    g->d_sid, g->d_slist, g->d_desig, g->d_sptr0, g->d_sdist0, g->d_sptr1,
                    g->d_sdist1, g->d_cid, g->d_cbot, g->d_clen, g->d_coff, g->d_layout,
                    g->d_pre, g->d_post, g->d_rec, g->d_info, g->d_bu_done, g->d_td_need, g->d_td_done,
                    g->d_slot_chain, g->d_cbas, g->d_el, g->d_cto, g->d_ceo, g->d_perm, g->d_inv,
                    g->d_tokval, g->d_needl, g->d_push, g->d_rtime, g->d_kslot, g->d_cpar,
                    g->d_cqp, g->d_trec, g->d_noise_idx, g->d_tid, g->d_tchg, g->d_cdep,
                    g->d_cpar1, g->d_cdep1, g->d_chist, g->d_corder, g->d_tokslot, g->d_pend,
                    g->d_corder_up, g->d_wa, g->d_wl, g->d_ilen, g->d_titer};
    for (void* p : ptrs)
        if (p) cudaFreeAsync(p, g->stream);
    status_block_put(g->h_status);
    if (g->h_stage) cudaFreeHost(g->h_stage);
    for (cudaEvent_t e : g->ev_pool) cudaEventDestroy(e);
    for (auto& p : g->ev_pending) {
        cudaEventDestroy(p.second.first);
        cudaEventDestroy(p.second.second);
    }
    if (g->ev0) cudaEventDestroy(g->ev0);
    if (g->ev1) cudaEventDestroy(g->ev1);
    for (cudaEvent_t e : g->ev_status)
        if (e) cudaEventDestroy(e);
    if (g->stream) cudaStreamDestroy(g->stream);
    delete g;
}

cudaEvent_t pooled_event(fl_graph* g) {
    if (!g->ev_pool.empty()) {
        cudaEvent_t e = g->ev_pool.back();
        g->ev_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

// Bracket a launch group: counts it, adds its algorithmic bytes and, with timing
// on, records CUDA events on the model's stream around it.
void kbegin(void* ctx) {
    fl_graph* g = (fl_graph*)ctx;
    if (g->timing) {
        g->ev_open = pooled_event(g);
        cudaEventRecord(g->ev_open, g->stream);
    }
}
void kend(void* ctx, int cls, double bytes) {
    fl_graph* g = (fl_graph*)ctx;
    g->k_launches[cls] += 1;
    g->k_bytes[cls] += bytes;
    if (g->timing && g->ev_open) {
        cudaEvent_t e = pooled_event(g);
        cudaEventRecord(e, g->stream);
        g->ev_pending.push_back({cls, {g->ev_open, e}});
        g->ev_open = nullptr;
    }
}
// Folds finished event pairs into the per-class times (after a stream sync).
void kresolve(fl_graph* g) {
    for (auto& p : g->ev_pending) {
        float ms = 0;
        if (cudaEventElapsedTime(&ms, p.second.first, p.second.second) == cudaSuccess)
            g->k_ms[p.first] += ms;
        g->ev_pool.push_back(p.second.first);
        g->ev_pool.push_back(p.second.second);
    }
    g->ev_pending.clear();
}

#define FL_LAUNCH(g, cls, bytes, ...) \
    do {                              \
        kbegin(g);                    \
        __VA_ARGS__;                  \
        kend(g, cls, (double)(bytes)); \
    } while (0)

int alloc_workspace(fl_graph* g) {
    const uint32_t n = g->n;
    // the Kahn rounds stop once fewer sites are ready than walk warps fit on the GPU
    g->kahn_min_width = kahn_min_width(n, g->terrains > 1);
    FL_TRY(dalloc(&g->d_k, n));
    FL_TRY(dalloc(&g->d_u, n));
    FL_TRY(dalloc(&g->d_tan, n));
    FL_TRY(dalloc(&g->d_base, n));
    FL_TRY(dalloc(&g->d_elev, n));
    FL_TRY(dalloc(&g->d_A, n));
    FL_TRY(dalloc(&g->d_t, n));
    FL_TRY(dalloc(&g->d_w, n));
    FL_TRY(dalloc(&g->d_wa, n));
    FL_TRY(dalloc(&g->d_wl, n));
    FL_TRY(dalloc(&g->d_rlen, n));
    FL_TRY(dalloc(&g->d_next, n));
    FL_TRY(dalloc(&g->d_lab, n));
    FL_TRY(dalloc(&g->d_lab2, n));
    FL_TRY(dalloc(&g->d_rank, n));
    FL_TRY(dalloc(&g->d_sor, n));
    FL_TRY(dalloc(&g->d_outlets, n));
    FL_TRY(dalloc(&g->d_bas, n));
    FL_TRY(dalloc(&g->d_trec, n));
    FL_TRY(dalloc(&g->d_outlet, n));
    FL_TRY(dalloc(&g->d_best, n));
    FL_TRY(dalloc(&g->d_flags, kNumFlags));
    FL_TRY(dalloc(&g->d_pending, n));
    FL_TRY(dalloc(&g->d_hgt, n));
    FL_TRY(dalloc(&g->d_order, n));
    // each Kahn round retires at least kahn_min_width sites
    g->max_rounds = n / std::min(g->kahn_min_width, kKahnMinWidthEarly) + 64;
    FL_TRY(dalloc(&g->d_roff, g->max_rounds + 2));
    FL_TRY(dalloc(&g->d_rtime, 2ull * (g->max_rounds + 1)));
    FL_TRY(dalloc(&g->d_meta, kMetaCount));
    FL_TRY(dalloc(&g->d_sid, n));
    FL_TRY(dalloc(&g->d_slist, n));
    FL_TRY(dalloc(&g->d_desig, n));
    FL_TRY(dalloc(&g->d_sptr0, n));
    FL_TRY(dalloc(&g->d_sdist0, n));
    FL_TRY(dalloc(&g->d_sptr1, n));
    FL_TRY(dalloc(&g->d_sdist1, n));
    FL_TRY(dalloc(&g->d_cid, n));
    FL_TRY(dalloc(&g->d_cbot, g->kahn_min_width));
    FL_TRY(dalloc(&g->d_clen, g->kahn_min_width));
    FL_TRY(dalloc(&g->d_coff, g->kahn_min_width));
    FL_TRY(dalloc(&g->d_layout, n));
    FL_TRY(dalloc(&g->d_slot_chain, n));
    FL_TRY(dalloc(&g->d_kslot, n));
    FL_TRY(dalloc(&g->d_cpar, g->kahn_min_width));
    FL_TRY(dalloc(&g->d_cqp, g->kahn_min_width));
    FL_TRY(dalloc(&g->d_cdep, g->kahn_min_width));
    FL_TRY(dalloc(&g->d_cpar1, 2ull * g->kahn_min_width));   // pointer-jumping buffers
    FL_TRY(dalloc(&g->d_cdep1, g->kahn_min_width));
    FL_TRY(dalloc(&g->d_chist, n + 1ull));
    FL_TRY(dalloc(&g->d_corder, g->kahn_min_width));
    FL_TRY(dalloc(&g->d_corder_up, g->kahn_min_width));
    FL_TRY(dalloc(&g->d_el, n));
    FL_TRY(dalloc(&g->d_cbas, g->kahn_min_width));
    FL_TRY(dalloc(&g->d_cto, g->kahn_min_width));
    FL_TRY(dalloc(&g->d_ceo, g->kahn_min_width));
    FL_TRY(dalloc(&g->d_pre, n));
    FL_TRY(dalloc(&g->d_post, n));
    FL_TRY(dalloc(&g->d_rec, n));
    FL_TRY(dalloc(&g->d_info, n));
    FL_TRY(dalloc(&g->d_needl, n));
    FL_TRY(dalloc(&g->d_push, n));
    // donor lists: each site's list is its cell area plus its donors, so 2n entries
    // hold every list at once
    g->tok_cap = (uint32_t)std::min<uint64_t>(2ull * n + 64, 0xfffffff0ull);
    FL_TRY(dalloc(&g->d_tokval, g->tok_cap));
    FL_TRY(dalloc(&g->d_tokslot, g->tok_cap));
    FL_TRY(dalloc(&g->d_pend, n));
    FL_TRY(dalloc(&g->d_bu_done, n));
    FL_TRY(dalloc(&g->d_td_need, n));
    FL_TRY(dalloc(&g->d_td_done, n));
    // stamp-tagged words start below every stamp (stamps count from 1 per model, and
    // the memory may have belonged to an earlier model)
    FL_CU(cudaMemsetAsync(g->d_bu_done, 0, n * 4ull, g->stream));
    FL_CU(cudaMemsetAsync(g->d_td_need, 0, n * 4ull, g->stream));
    FL_CU(cudaMemsetAsync(g->d_td_done, 0, n * 4ull, g->stream));
    FL_CU(cudaMemsetAsync(g->d_push, 0, n * 8ull, g->stream));
    FL_CU(cudaMemsetAsync(g->d_flags, 0, kNumFlags * 4ull, g->stream));
    static_assert((kNumFlags + kMetaCount) * sizeof(int) <= 256, "status block size");
    g->h_status = status_block_get();
    if (!g->h_status) {
        g_err = "cudaHostAlloc failed";
        return FL_ERR_OUT_OF_MEMORY;
    }
    return FL_OK;
}

// The status words (and, with meta, the basin pass's bookkeeping words) back to the
// host: one blocking synchronisation of the model's stream.
int sync_status(fl_graph* g, int* h, bool meta = false) {
    FL_CU(cudaMemcpyAsync(g->h_status, g->d_flags, kNumFlags * sizeof(int), cudaMemcpyDeviceToHost,
                          g->stream));
    if (meta)
        FL_CU(cudaMemcpyAsync(g->h_status + kNumFlags, g->d_meta, kMetaCount * sizeof(uint32_t),
                              cudaMemcpyDeviceToHost, g->stream));
    FL_CU(cudaStreamSynchronize(g->stream));
    g->host_syncs++;
    std::memcpy(h, g->h_status, kNumFlags * sizeof(int));
    if (meta) std::memcpy(g->last_meta, g->h_status + kNumFlags, sizeof g->last_meta);
    return FL_OK;
}

// Clears the per-iteration status words: has_lake, changed, error, the exact-scan count
// and the pointer-jumping words (not the barrier words, which the grid barrier leaves
// consistent).
int clear_flags(fl_graph* g) {
    FL_CU(cudaMemsetAsync(g->d_flags, 0, 4 * sizeof(int), g->stream));
    FL_CU(cudaMemsetAsync(g->d_flags + kExact, 0, (kJump2 + 1 - kExact) * sizeof(int), g->stream));
    return FL_OK;
}

// Copies this iteration's status words and bookkeeping into pipeline slot `slot`
// behind its kernels.
int enqueue_status(fl_graph* g, int slot) {
    int* sb = g->h_status + kStatusSlot * (1 + slot);
    FL_CU(cudaMemcpyAsync(sb, g->d_flags, kNumFlags * sizeof(int), cudaMemcpyDeviceToHost, g->stream));
    FL_CU(cudaMemcpyAsync(sb + kNumFlags, g->d_meta, kMetaCount * sizeof(uint32_t),
                          cudaMemcpyDeviceToHost, g->stream));
    FL_CU(cudaEventRecord(g->ev_status[slot], g->stream));
    return FL_OK;
}

int device_error(const int* h) {
    static const char* what[] = {"", "receivers do not form a forest", "grid barrier timed out",
                                 "chain hand-off timed out", "skeleton chain table overflow"};
    int c = h[kError];
    if (c <= 0 || c > 4) return FL_OK;
    g_err = what[c];
    return FL_ERR_DEVICE_LIMIT;
}

// Outlet list as generate() resolves it (generator.rs:120-132).
// Returned in device ids, list order unchanged (the order matters to the lake heap).
// generator.rs:120-132, per terrain: the sites with is_outlet in ascending order, else
// the terrain's default outlets (device ids, terrain after terrain).
// A caller-order host array: one over all sites, or (packed terrains) one per terrain.
template <class T>
struct HostCols {
    T* whole = nullptr;
    T* const* parts = nullptr;
    HostCols() = default;
    HostCols(T* w) : whole(w) {}
    static HostCols of_parts(T* const* p) {
        HostCols c;
        c.parts = p;
        return c;
    }
    // every terrain has its array
    bool complete(const fl_graph* g) const {
        if (whole) return true;
        if (!parts) return false;
        for (uint32_t t = 0; t < g->terrains; ++t)
            if (!parts[t]) return false;
        return true;
    }
    bool any() const { return whole || parts; }
    // terrain t's slice, indexed by its own site index (null when absent)
    T* terrain(const fl_graph* g, uint32_t t) const {
        if (whole) return whole + g->site_off[t];
        return parts ? parts[t] : nullptr;
    }
};

// Runs f(lo, hi, w) over [0, m) cut into contiguous ranges, range w on host thread w:
// one range below 2^20 elements, else up to eight.  Ranges come in index order, so
// per-range results concatenated in w order are the serial scan's.
constexpr unsigned kHostRanges = 8;
template <class F>
void host_ranges(uint32_t m, F f) {
    const unsigned nt = m < (1u << 20) ? 1u
                                       : std::max(1u, std::min(kHostRanges, std::thread::hardware_concurrency()));
    const uint64_t step = (m + nt - 1) / nt;
    auto range = [&](unsigned w) {
        f((uint32_t)std::min<uint64_t>(m, w * step), (uint32_t)std::min<uint64_t>(m, (w + 1) * step), w);
    };
    std::vector<std::thread> th;
    for (unsigned w = 1; w < nt; ++w) th.emplace_back(range, w);
    range(0);
    for (auto& x : th) x.join();
}

// Appends base-relative site i (as its device id) for every nonzero a[i], i ascending.
void flagged_sites(const fl_graph* g, const uint8_t* a, uint32_t base, uint32_t m,
                   std::vector<uint32_t>& o) {
    std::vector<uint32_t> part[kHostRanges];
    host_ranges(m, [&](uint32_t lo, uint32_t hi, unsigned w) {
        std::vector<uint32_t>& out = w ? part[w] : o;
        uint32_t i = lo;
        while (i < hi) {
            // outlets are sparse: step over eight zero flags at a time
            if (i + 8 <= hi) {
                uint64_t word;
                std::memcpy(&word, a + i, 8);
                if (word == 0) {
                    i += 8;
                    continue;
                }
            }
            if (a[i]) out.push_back(g->inv[base + i]);
            ++i;
        }
    });
    for (unsigned w = 1; w < kHostRanges; ++w) o.insert(o.end(), part[w].begin(), part[w].end());
}

// Whether any of m max_slope entries is a number (NaN means no limit).
bool any_slope_limit(const double* ms, uint32_t m) {
    std::atomic<bool> found{false};
    host_ranges(m, [&](uint32_t lo, uint32_t hi, unsigned) {
        for (uint32_t a = lo; a < hi && !found.load(std::memory_order_relaxed); a += 4096) {
            const uint32_t e = std::min(hi, a + 4096);
            int num = 0;
            for (uint32_t i = a; i < e; ++i) num |= ms[i] == ms[i];   // false for NaN only
            if (num) found.store(true, std::memory_order_relaxed);
        }
    });
    return found.load();
}

std::vector<uint32_t> resolve_outlets(const fl_graph* g, HostCols<const uint8_t> is_outlet) {
    std::vector<uint32_t> o;
    for (uint32_t t = 0; t < g->terrains; ++t) {
        const size_t first = o.size();
        const uint32_t base = g->site_off[t], m = g->site_off[t + 1] - base;
        flagged_sites(g, is_outlet.terrain(g, t), base, m, o);
        if (o.size() == first)
            o.insert(o.end(), g->def_outlets.begin() + g->def_off[t],
                     g->def_outlets.begin() + g->def_off[t + 1]);
    }
    return o;
}

std::vector<uint32_t> to_device_ids(const fl_graph* g, const uint32_t* ids, uint32_t count) {
    std::vector<uint32_t> o(count);
    for (uint32_t i = 0; i < count; ++i) o[i] = g->inv[ids[i]];
    return o;
}

// Many terrains' arrays pass through one page-locked staging array (one transfer instead
// of one per terrain, each of which costs a fixed driver overhead).
constexpr uint32_t kStageTerrains = 32;

int host_stage(fl_graph* g) {
    if (g->h_stage) return FL_OK;
    FL_CU(cudaHostAlloc((void**)&g->h_stage, std::max<uint64_t>(1, g->n) * 8ull, cudaHostAllocPortable));
    return FL_OK;
}

// Copies between the staging array and the terrains' arrays on a few host threads.
template <class F>
void per_terrain_threads(const fl_graph* g, F f) {
    const unsigned nt = g->n < (1u << 20) ? 1u : std::max(1u, std::min(8u, std::thread::hardware_concurrency()));
    std::vector<std::thread> th;
    for (unsigned w = 1; w < nt; ++w)
        th.emplace_back([&, w] {
            for (uint32_t t = w; t < g->terrains; t += nt) f(t);
        });
    for (uint32_t t = 0; t < g->terrains; t += nt) f(t);
    for (auto& x : th) x.join();
}

// Uploads a caller-order f64 array (whole or per terrain) into device order.
int upload_permuted(fl_graph* g, HostCols<const double> src, double* dst) {
    if (src.whole) {
        FL_CU(cudaMemcpyAsync(g->d_t, src.whole, g->n * 8ull, cudaMemcpyHostToDevice, g->stream));
    } else if (g->terrains > kStageTerrains) {
        FL_TRY(host_stage(g));
        FL_CU(cudaStreamSynchronize(g->stream));       // the previous staged copy is done
        per_terrain_threads(g, [&](uint32_t t) {
            std::memcpy(g->h_stage + g->site_off[t], src.parts[t],
                        (g->site_off[t + 1] - g->site_off[t]) * 8ull);
        });
        FL_CU(cudaMemcpyAsync(g->d_t, g->h_stage, g->n * 8ull, cudaMemcpyHostToDevice, g->stream));
    } else {
        for (uint32_t t = 0; t < g->terrains; ++t)
            FL_CU(cudaMemcpyAsync(g->d_t + g->site_off[t], src.parts[t],
                                  (g->site_off[t + 1] - g->site_off[t]) * 8ull,
                                  cudaMemcpyHostToDevice, g->stream));
    }
    k_gather_f64<<<blocks_for(g->n), kThreads, 0, g->stream>>>(g->n, g->d_perm, g->d_t, dst);
    FL_CU(cudaGetLastError());
    return FL_OK;
}
int upload_permuted(fl_graph* g, const double* src, double* dst) {
    return upload_permuted(g, HostCols<const double>(src), dst);
}

// Downloads a device-order f64 array into caller order (whole or per terrain).
int download_permuted(fl_graph* g, const double* src, HostCols<double> dst) {
    // w is dead after a pass (and response times must survive the downloads)
    double* stage = (src == g->d_w) ? g->d_t : g->d_w;
    if (stage == g->d_w) g->w_valid = false;
    k_gather_f64<<<blocks_for(g->n), kThreads, 0, g->stream>>>(g->n, g->d_inv, src, stage);
    FL_CU(cudaGetLastError());
    if (dst.whole) {
        FL_CU(cudaMemcpyAsync(dst.whole, stage, g->n * 8ull, cudaMemcpyDeviceToHost, g->stream));
    } else if (g->terrains > kStageTerrains) {
        FL_TRY(host_stage(g));
        FL_CU(cudaMemcpyAsync(g->h_stage, stage, g->n * 8ull, cudaMemcpyDeviceToHost, g->stream));
        FL_CU(cudaStreamSynchronize(g->stream));
        per_terrain_threads(g, [&](uint32_t t) {
            std::memcpy(dst.parts[t], g->h_stage + g->site_off[t],
                        (g->site_off[t + 1] - g->site_off[t]) * 8ull);
        });
    } else {
        for (uint32_t t = 0; t < g->terrains; ++t)
            FL_CU(cudaMemcpyAsync(dst.parts[t], stage + g->site_off[t],
                                  (g->site_off[t + 1] - g->site_off[t]) * 8ull,
                                  cudaMemcpyDeviceToHost, g->stream));
    }
    return FL_OK;
}
int download_permuted(fl_graph* g, const double* src, double* dst) {
    return download_permuted(g, src, HostCols<double>(dst));
}

// The model's CSR (device order) on the host, for the host heap and the probes;
// downloaded on first use.
int ensure_host_csr(fl_graph* g) {
    if (g->h_row.size() == g->n + 1ull) return FL_OK;
    g->h_row.resize(g->n + 1ull);
    g->h_col.resize(g->nnz);
    g->h_len.resize(g->nnz);
    FL_CU(cudaMemcpyAsync(g->h_row.data(), g->d_row, (g->n + 1ull) * 4, cudaMemcpyDeviceToHost, g->stream));
    if (g->nnz) {
        FL_CU(cudaMemcpyAsync(g->h_col.data(), g->d_col, g->nnz * 4, cudaMemcpyDeviceToHost, g->stream));
        FL_CU(cudaMemcpyAsync(g->h_len.data(), g->d_len, g->nnz * 8, cudaMemcpyDeviceToHost, g->stream));
    }
    FL_CU(cudaStreamSynchronize(g->stream));
    return FL_OK;
}

// Rows of the listed sites gathered into a compact CSR (list order).
__global__ void k_row_degrees(uint32_t c, const uint32_t* __restrict__ ids,
                              const uint32_t* __restrict__ row, uint32_t* __restrict__ deg) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < c) deg[i] = row[ids[i] + 1] - row[ids[i]];
}
__global__ void k_row_gather(uint32_t c, const uint32_t* __restrict__ ids,
                             const uint32_t* __restrict__ row, const uint32_t* __restrict__ col,
                             const double* __restrict__ len, const uint32_t* __restrict__ off,
                             uint32_t* __restrict__ ocol, double* __restrict__ olen) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c) return;
    uint32_t d = off[i];
    for (uint32_t s = row[ids[i]], e = row[ids[i] + 1]; s < e; ++s, ++d) {
        ocol[d] = col[s];
        olen[d] = len[s];
    }
}

// The lake heap's tied prefix for an outlet list (device ids; packed terrains one after
// another, each replayed with its own heap), from the outlets' rows gathered on the
// device.  *status: FL_OK, 1 for a NaN length, 2 when a zero-length edge reaches a site
// that is not an outlet (then only the host heap over the whole graph can continue).
int lake_prefix(fl_graph* g, const std::vector<uint32_t>& outlets, std::vector<uint32_t>& prefix,
                int* status) {
    prefix.clear();
    *status = FL_OK;
    const uint32_t c = (uint32_t)outlets.size();
    if (c == 0) return FL_OK;
    uint32_t *d_ids = nullptr, *d_deg = nullptr, *d_ocol = nullptr;
    double* d_olen = nullptr;
    std::vector<uint32_t> orow(c + 1ull), ocol;
    std::vector<double> olen;
    cudaError_t e = cudaMallocAsync((void**)&d_ids, c * 8ull, g->stream);
    if (e == cudaSuccess) {
        d_deg = d_ids + c;
        e = cudaMemcpyAsync(d_ids, outlets.data(), c * 4ull, cudaMemcpyHostToDevice, g->stream);
    }
    if (e == cudaSuccess) {
        k_row_degrees<<<blocks_for(c), kThreads, 0, g->stream>>>(c, d_ids, g->d_row, d_deg);
        e = cudaMemcpyAsync(orow.data() + 1, d_deg, c * 4ull, cudaMemcpyDeviceToHost, g->stream);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    if (e == cudaSuccess) {
        orow[0] = 0;
        for (uint32_t i = 0; i < c; ++i) orow[i + 1] += orow[i];
        ocol.resize(orow[c]);
        olen.resize(orow[c]);
        e = cudaMallocAsync((void**)&d_ocol, (orow[c] + 2ull) * 12ull, g->stream);
    }
    if (e == cudaSuccess) {
        d_olen = (double*)(d_ocol + ((orow[c] + 1) & ~1u));   // 8-byte aligned after the columns
        e = cudaMemcpyAsync(d_deg, orow.data(), c * 4ull, cudaMemcpyHostToDevice, g->stream);
    }
    if (e == cudaSuccess) {
        k_row_gather<<<blocks_for(c), kThreads, 0, g->stream>>>(c, d_ids, g->d_row, g->d_col,
                                                                g->d_len, d_deg, d_ocol, d_olen);
        if (orow[c]) {
            e = cudaMemcpyAsync(ocol.data(), d_ocol, orow[c] * 4ull, cudaMemcpyDeviceToHost, g->stream);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(olen.data(), d_olen, orow[c] * 8ull, cudaMemcpyDeviceToHost, g->stream);
        }
    }
    if (d_ocol) cudaFreeAsync(d_ocol, g->stream);
    if (d_ids) cudaFreeAsync(d_ids, g->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    if (e != cudaSuccess) {
        set_err("outlet rows", e);
        return FL_ERR_CUDA;
    }
    std::vector<uint32_t> part;
    size_t p0 = 0;
    for (uint32_t t = 0; t < g->terrains; ++t) {
        const uint32_t b = g->site_off[t + 1];
        size_t p1 = p0;
        while (p1 < c && outlets[p1] < b) ++p1;
        const int r = fl::lake_rank_prefix_rows(g->n, outlets.data() + p0, (uint32_t)(p1 - p0),
                                                orow.data() + p0, ocol.data(), olen.data(), part);
        if (r != 0) {
            *status = r;
            return FL_OK;
        }
        prefix.insert(prefix.end(), part.begin(), part.end());
        p0 = p1;
    }
    return FL_OK;
}

// Uploads the outlet list and table, computing (or reusing) the lake-heap rank.
int set_outlets(fl_graph* g, const std::vector<uint32_t>& outlets, bool need_rank) {
    uint32_t n = g->n;
    // the outlet table from the list, on the device
    FL_CU(cudaMemsetAsync(g->d_outlet, 0, n, g->stream));
    if (!outlets.empty()) {
        FL_CU(cudaMemcpyAsync(g->d_outlets, outlets.data(), outlets.size() * 4,
                              cudaMemcpyHostToDevice, g->stream));
        k_mark<<<blocks_for((uint32_t)outlets.size()), kThreads, 0, g->stream>>>(
            (uint32_t)outlets.size(), g->d_outlets, g->d_outlet);
        FL_CU(cudaGetLastError());
        // pageable copies return before the DMA ends: keep the list until it is done
        FL_CU(cudaStreamSynchronize(g->stream));
    }
    if (!g->rank_valid || g->rank_key != outlets) {
        g->rank_valid = false;
        g->rank_uploaded = false;
        g->rank_key = outlets;
    }
    if (need_rank && !g->rank_uploaded && fl::tuning().gpu_rank) {
        // the keyed order on the GPU after the tied prefix replayed here; the host heap
        // when equal or non-positive lengths could let its arrangement decide.  Packed
        // terrains: each terrain's own prefix (its own heap), concatenated; one contracted
        // source for all of them keeps every terrain's order (a terrain's frontier only
        // moves by its own pops), and lakes compare ranks within their terrain only.
        const auto t0 = std::chrono::steady_clock::now();
        std::vector<uint32_t> prefix;
        int pr = FL_OK;
        FL_TRY(lake_prefix(g, outlets, prefix, &pr));
        if (pr == 1) {
            g_err = "NaN edge length in the lake traversal";
            return FL_ERR_INVALID_ARGUMENT;
        }
        fl::GpuRankInfo info;
        const fl::RankResult r =
            pr != FL_OK ? fl::kRankFallback   // a zero-length edge: the host heap decides
                        : fl::gpu_lake_rank(g->stream, n, g->d_row, g->d_col, g->d_len, g->nnz,
                                            prefix, g->d_rank, g->d_sor, &info);
        if (r == fl::kRankError) {
            set_err("lake order on the GPU", info.error);
            return FL_ERR_CUDA;
        }
        if (r == fl::kRankOk) {
            FL_CU(cudaStreamSynchronize(g->stream));
            g->h_rank.clear();
            g->rank_valid = g->rank_uploaded = true;
            g->rank_gpu = 1;
            g->rank_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
            return FL_OK;
        }
        g->rank_gpu = 0;                              // fall through to the host heap
    }
    if (need_rank && !g->rank_uploaded) {
        const auto t0 = std::chrono::steady_clock::now();
        if (!g->rank_valid || g->h_rank.size() != n) {
            FL_TRY(ensure_host_csr(g));
            g->h_rank.resize(n);
            if (g->terrains == 1) {
                if (!fl::lake_heap_rank(n, g->h_row.data(), g->h_col.data(), g->h_len.data(),
                                        outlets.data(), (uint32_t)outlets.size(),
                                        g->h_rank.data())) {
                    g_err = "NaN edge length in the lake traversal";
                    return FL_ERR_INVALID_ARGUMENT;
                }
            } else {
                // each terrain's own traversal (heap ties included), ranks offset by the
                // terrain's first site: lakes never compare ranks across terrains
                std::vector<uint32_t> lrow, lcol, lout, lrank;
                size_t oi = 0;
                for (uint32_t t = 0; t < g->terrains; ++t) {
                    const uint32_t a = g->site_off[t], b = g->site_off[t + 1], m = b - a;
                    const uint32_t s0 = g->h_row[a];
                    lrow.resize(m + 1);
                    for (uint32_t j = 0; j <= m; ++j) lrow[j] = g->h_row[a + j] - s0;
                    lcol.resize(g->h_row[b] - s0);
                    for (uint32_t s = s0; s < g->h_row[b]; ++s) lcol[s - s0] = g->h_col[s] - a;
                    lout.clear();
                    while (oi < outlets.size() && outlets[oi] < b) lout.push_back(outlets[oi++] - a);
                    lrank.resize(m);
                    if (!fl::lake_heap_rank(m, lrow.data(), lcol.data(), g->h_len.data() + s0,
                                            lout.data(), (uint32_t)lout.size(), lrank.data())) {
                        g_err = "NaN edge length in the lake traversal";
                        return FL_ERR_INVALID_ARGUMENT;
                    }
                    for (uint32_t j = 0; j < m; ++j)
                        g->h_rank[a + j] = lrank[j] == kNone ? kNone : a + lrank[j];
                }
            }
            g->rank_valid = true;
        }
        std::vector<uint32_t> sor(n, kNone);
        for (uint32_t v = 0; v < n; ++v)
            if (g->h_rank[v] != kNone && g->h_rank[v] < n) sor[g->h_rank[v]] = v;
        FL_CU(cudaMemcpyAsync(g->d_rank, g->h_rank.data(), n * 4ull, cudaMemcpyHostToDevice, g->stream));
        FL_CU(cudaMemcpyAsync(g->d_sor, sor.data(), n * 4ull, cudaMemcpyHostToDevice, g->stream));
        FL_CU(cudaStreamSynchronize(g->stream));
        g->rank_uploaded = true;
        g->rank_gpu = 0;
        g->rank_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
    return FL_OK;
}

// Receivers for the current elevations; the kernel raises flags[kHasLake].
int enqueue_receivers(fl_graph* g) {
    FL_LAUNCH(g, kcReceivers, 25.0 * g->n + 20.0 * g->nnz,
              fl::launch_receivers(g->stream, g->n, g->d_row, g->d_col, g->d_len, g->d_ilen,
                                   g->d_elev, g->d_outlet, g->d_next, g->d_rlen, g->d_flags,
                                   g->d_tid, g->d_titer));
    FL_CU(cudaGetLastError());
    return FL_OK;
}

// Basin labels of d_next into d_lab (pointer jumping, one cooperative launch); with a
// gate, only if *gate is set when the kernel runs.
int enqueue_labels(fl_graph* g, const int* gate) {
    uint32_t n = g->n;
    static const unsigned full = coop_blocks((const void*)k_labels, 1024, 2);
    const bool sized = g->sized_grids >= 0 ? g->sized_grids != 0
                                           : fl::shape_for(n, g->terrains > 1).sized_grids;
    const unsigned grid = fl::sized_grid(sized, full, n, 1024 * 8);
    const int* gt = gate;
    void* argv[] = {(void*)&n, (void*)&g->d_next, (void*)&g->d_lab, (void*)&g->d_lab2,
                    (void*)&gt, (void*)&g->d_flags};
    FL_LAUNCH(g, kcLakes, 8.0 * n,
              cudaLaunchCooperativeKernel((const void*)k_labels, dim3(grid), dim3(1024), argv, 0,
                                          g->stream));
    FL_CU(cudaGetLastError());
    return FL_OK;
}

// Lake re-routing on d_next (labels must be current), gated like enqueue_labels.
int enqueue_lakes(fl_graph* g, const int* gate) {
    uint32_t n = g->n;
    FL_LAUNCH(g, kcLakes, 8.0 * n,
              k_clear_keys<<<blocks_for(n), kThreads, 0, g->stream>>>(n, g->d_best, gate));
    FL_LAUNCH(g, kcLakes, 12.0 * n + 8.0 * g->nnz,
              k_lake_keys<<<blocks_for(n), kThreads, 0, g->stream>>>(
                  n, g->d_row, g->d_col, g->d_rank, g->d_lab, g->d_outlet, g->d_best, gate));
    FL_LAUNCH(g, kcLakes, 8.0 * n,
              k_lake_flip<<<blocks_for(n), kThreads, 0, g->stream>>>(
                  n, g->d_row, g->d_col, g->d_len, g->d_best, g->d_sor, g->d_next, g->d_rlen,
                  g->d_flags, gate));
    FL_CU(cudaGetLastError());
    return FL_OK;
}

// Drainage areas, response times, elevations on final receivers; *changed.
// Algorithmic bytes of the kernels that work on the skeleton, whose size is known
// only once the pass has run (the launch groups were counted with 0 bytes).
//   bottom-up: slot record (32) + slot info (8) + area out (8) per slot;
//              offset, length, bottom id, bottom area, hand-off flag (24) per chain
//   top-down:  w (8) + flags (1) + t out (8) [+ elevation out (8) with slope limits]
//              per slot; offset, length, parent t / elevation / outlet, chain outlet
//              t / elevation / id out (56) per chain
//   ranking:   per pointer-jumping round, own and successor's pointer and distance
//              in (16) and out (8) per skeleton site; ceil(log2(longest chain)) + 1
//              rounds
void account_skeleton(fl_graph* g) {
    const double ns = g->last_meta[kMetaNs], nc = g->last_meta[kMetaChains];
    const uint32_t longest = g->last_meta[kMetaMaxChain];
    int rounds = 1;
    while (rounds < 32 && (1u << (rounds - 1)) < longest) ++rounds;
    g->k_bytes[kcSkelUp] += 48.0 * ns + 24.0 * nc;
    g->k_bytes[kcSkelDown] += (g->slope ? 25.0 : 17.0) * ns + 56.0 * nc;
    g->k_bytes[kcSkelRank] += 24.0 * ns * rounds;
}

// Enqueues the pass; flags[kChanged] / flags[kError] and the bookkeeping words in meta
// hold its outcome once it has run (finish_basin_pass).  all_records: every site's
// top-down record is read afterwards (response times).
int enqueue_basin_pass(fl_graph* g, bool all_records = false) {
    g->stamp = g->stamp == 0x7ffffff0 ? 1 : g->stamp + 1;
    if (g->stamp == 1) {   // stamps wrapped (or first pass): clear hand-off words
        FL_CU(cudaMemsetAsync(g->d_bu_done, 0, g->n * 4ull, g->stream));
        FL_CU(cudaMemsetAsync(g->d_td_need, 0, g->n * 4ull, g->stream));
        FL_CU(cudaMemsetAsync(g->d_td_done, 0, g->n * 4ull, g->stream));
        FL_CU(cudaMemsetAsync(g->d_push, 0, g->n * 8ull, g->stream));
    }
    fl::BasinArgs a{};
    a.n = g->n;
    a.row = g->d_row;
    a.col = g->d_col;
    a.area = g->d_area;
    a.next = g->d_next;
    a.rlen = g->d_rlen;
    a.k = g->d_k;
    a.u = g->d_u;
    a.tanms = g->d_tan;
    a.outlet = g->d_outlet;
    a.A = g->d_A;
    a.rec_t = g->d_trec;
    a.w = g->d_w;
    a.w_area = g->d_wa;
    a.w_dist = g->d_wl;
    a.w_valid = g->w_valid;
    g->w_valid = false;   // until the pass, and with it k_w, has run
    a.elev = g->d_elev;
    a.pending = g->d_pending;
    a.hgt = g->d_hgt;
    a.order = g->d_order;
    a.roff = g->d_roff;
    a.rtime = g->d_rtime;
    a.max_rounds = g->max_rounds;
    a.kahn_min_width = g->passes < kEarlyPasses
                           ? std::min(g->kahn_min_width, kKahnMinWidthEarly)
                           : g->kahn_min_width;
    g->passes++;
    a.meta = g->d_meta;
    a.flags = g->d_flags;
    a.tid = g->d_tid;
    a.tchg = g->d_tchg;
    a.titer = g->d_titer;
    a.sid = g->d_sid;
    a.slist = g->d_slist;
    a.desig = g->d_desig;
    a.sptr0 = g->d_sptr0;
    a.sdist0 = g->d_sdist0;
    a.sptr1 = g->d_sptr1;
    a.sdist1 = g->d_sdist1;
    a.cid = g->d_cid;
    a.cbot = g->d_cbot;
    a.clen = g->d_clen;
    a.coff = g->d_coff;
    a.layout = g->d_layout;
    a.slot_chain = g->d_slot_chain;
    a.el = g->d_el;
    a.cbas = g->d_cbas;
    a.cto = g->d_cto;
    a.ceo = g->d_ceo;
    a.slope = g->slope;
    a.pre = g->d_pre;
    a.post = g->d_post;
    a.kslot = g->d_kslot;
    a.cpar = g->d_cpar;
    a.cqp = g->d_cqp;
    a.cdep = g->d_cdep;
    a.cpar1 = g->d_cpar1;
    a.cdep1 = g->d_cdep1;
    a.chist = g->d_chist;
    a.corder = g->d_corder;
    a.corder_up = g->d_corder_up;
    const fl::Shape sh = fl::shape_for(g->n, g->terrains > 1);
    a.walk_grid = fl::walk_grid(sh.walk_per_sm);
    a.low_ilp = sh.low_ilp;
    a.sized_grids = g->sized_grids >= 0 ? g->sized_grids != 0 : sh.sized_grids;
    a.rec = g->d_rec;
    a.info = g->d_info;
    a.needl = g->d_needl;
    a.tokval = g->d_tokval;
    a.tokslot = g->d_tokslot;
    a.pend = g->d_pend;
    a.tok_cap = g->tok_cap;
    a.push_to = g->d_push;
    a.bu_done = g->d_bu_done;
    a.td_need = g->d_td_need;
    a.td_done = g->d_td_done;
    a.stamp = g->stamp;
    a.all_records = all_records;
    fl::Hooks hk{g, kbegin, kend};
    cudaError_t e = fl::basin_pass(a, g->stream, hk, (uint32_t)std::min<uint64_t>(g->nnz, 0xffffffffu));
    if (e != cudaSuccess) {
        set_err("basin pass launch", e);
        return e == cudaErrorMemoryAllocation ? FL_ERR_OUT_OF_MEMORY : FL_ERR_CUDA;
    }
    FL_CU(cudaGetLastError());
    return FL_OK;
}

// After sync_status(.., meta = true) following a pass: its device error, if any, and
// the bookkeeping that needs the skeleton's size.
int finish_basin_pass(fl_graph* g, const int* h) {
    FL_TRY(device_error(h));
    g->w_valid = true;
    account_skeleton(g);
    return FL_OK;
}

// Waits for the status copied into pipeline slot `slot` (one host synchronisation)
// and takes it: h receives the status words, last_meta the bookkeeping.
int take_status(fl_graph* g, int slot, int* h) {
    FL_CU(cudaEventSynchronize(g->ev_status[slot]));
    g->host_syncs++;
    const int* sb = g->h_status + kStatusSlot * (1 + slot);
    std::memcpy(h, sb, kNumFlags * sizeof(int));
    std::memcpy(g->last_meta, sb + kNumFlags, sizeof g->last_meta);
    return finish_basin_pass(g, h);
}

// Parameters into device order.  The uploads share one staging buffer; stream order
// makes each copy wait for the previous gather, and a copy from pageable memory has
// taken its data by the time it returns, so no host synchronisation is needed.
// tan(max_slope) is computed on the host with the C library's tan, as fastlem's
// `max_slope.tan()` is; without any slope limit the device array is just NaN.
int upload_params(fl_graph* g, HostCols<const double> base, HostCols<const double> k,
                  HostCols<const double> u, HostCols<const double> max_slope) {
    uint32_t n = g->n;
    g->slope = false;
    if (base.any()) FL_TRY(upload_permuted(g, base, g->d_base));
    if (k.any()) {
        FL_TRY(upload_permuted(g, k, g->d_k));
        g->w_valid = false;
    }
    if (u.any()) FL_TRY(upload_permuted(g, u, g->d_u));
    // a terrain without max_slope array has no slope limit
    for (uint32_t t = 0; t < g->terrains && !g->slope; ++t) {
        const double* ms = max_slope.terrain(g, t);
        if (ms) g->slope = any_slope_limit(ms, g->site_off[t + 1] - g->site_off[t]);
    }
    if (g->slope) {
        std::vector<double> tanv(n, NAN);
        for (uint32_t t = 0; t < g->terrains; ++t) {
            const double* ms = max_slope.terrain(g, t);
            const uint32_t a = g->site_off[t], m = g->site_off[t + 1] - a;
            if (!ms) continue;
            host_ranges(m, [&](uint32_t lo, uint32_t hi, unsigned) {
                for (uint32_t i = lo; i < hi; ++i) tanv[a + i] = std::isnan(ms[i]) ? NAN : std::tan(ms[i]);
            });
        }
        FL_TRY(upload_permuted(g, tanv.data(), g->d_tan));
    } else {
        k_fill_nan<<<blocks_for(n), kThreads, 0, g->stream>>>(n, g->d_tan);
        FL_CU(cudaGetLastError());
    }
    return FL_OK;
}

int generate_impl(fl_graph* g, uint32_t n_params, HostCols<const double> base,
                  HostCols<const double> k, HostCols<const double> u,
                  HostCols<const uint8_t> is_outlet, HostCols<const double> max_slope,
                  int64_t max_iter, HostCols<double> out_elev, uint32_t* out_iters,
                  double* loop_ms, double* total_ms, uint32_t* terrain_iters = nullptr) {
    g_err.clear();
    if (!g) return FL_ERR_MODEL_NOT_SET;
    if (!base.complete(g) || !k.complete(g) || !u.complete(g) || !is_outlet.complete(g))
        return FL_ERR_PARAMETERS_NOT_SET;
    if (n_params != g->n) return FL_ERR_INVALID_NUM_PARAMETERS;
    if (!out_elev.complete(g)) return FL_ERR_INVALID_ARGUMENT;
    FL_CU(cudaSetDevice(g->device));
    auto t_start = std::chrono::steady_clock::now();
    uint32_t n = g->n;
    // the uploads are asynchronous from page-locked memory: scan the outlet flags on the
    // host meanwhile
    FL_TRY(upload_params(g, base, k, u, max_slope));
    std::vector<uint32_t> outlets = resolve_outlets(g, is_outlet);
    FL_TRY(set_outlets(g, outlets, false));
    // all status words, including the grid barrier's, start from zero
    FL_CU(cudaMemsetAsync(g->d_flags, 0, kNumFlags * sizeof(int), g->stream));
    // every terrain draws its own StdRng::seed_from_u64(0) stream, sample i for its site i
    FL_LAUNCH(g, kcNoise, 8.0 * g->noise_n,
              k_noise<<<blocks_for((g->noise_n + 7) / 8), kThreads, 0, g->stream>>>(g->noise_n, g->d_w));
    g->w_valid = false;
    FL_LAUNCH(g, kcNoise, 28.0 * n,
              k_initial_elevation<<<blocks_for(n), kThreads, 0, g->stream>>>(
                  n, g->d_noise_idx ? g->d_noise_idx : g->d_perm, g->d_base, g->d_w, g->d_elev));
    // previous-iteration drainage areas steer the skeleton's chain choice; start from
    // the cell areas
    FL_LAUNCH(g, kcMisc, 16.0 * n,
              k_fill_f64<<<blocks_for(n), kThreads, 0, g->stream>>>(n, g->d_A, g->d_area));
    FL_CU(cudaGetLastError());
    FL_CU(cudaEventRecord(g->ev0, g->stream));
    if (max_iter > 0xffffffffll) max_iter = 0xffffffffll;
    uint64_t limit = max_iter < 0 ? 0xffffffffull : (uint64_t)max_iter;
    uint32_t iters = 0;
    g->passes = 0;
    // a terrain alone stops at its first iteration without a change; packed with others
    // it keeps iterating at a fixed point, so its count is that first unchanged iteration
    if (g->d_titer) {
        FL_CU(cudaMemsetAsync(g->d_tchg, 0, g->terrains * sizeof(int), g->stream));
        FL_CU(cudaMemsetAsync(g->d_titer, 0, g->terrains * sizeof(uint32_t), g->stream));
    }
    // One host synchronisation per iteration, on the status of the iteration before:
    // whether an elevation changed (the loop's exit, generator.rs:207-209) and any
    // device error.  Iteration it is enqueued before the host waits for iteration
    // it - 1's status (copied into one of two page-locked slots behind its kernels), so
    // the device never waits for the host between iterations.  When iteration it - 1
    // changed nothing, iteration it -- already queued -- recomputes the same fixed
    // point (an iteration without a change leaves the elevations, hence everything the
    // next one computes, as they were) and is not counted.  After a device error the
    // queued work is drained before returning.
    // The lake stages are enqueued behind the receivers and skip themselves when the
    // receivers found no lake; only while the lake order for this outlet list is not on
    // the device yet does the host wait for the receivers' lake flag to compute it.
    int h[kNumFlags];
    auto drained = [&](int rc) {
        cudaStreamSynchronize(g->stream);
        return rc;
    };
    uint64_t it = 0;
    bool settled = false;
    for (; it < limit && !settled; ++it) {
        FL_TRY(clear_flags(g));
        FL_TRY(enqueue_receivers(g));
        bool lakes = true;
        const int* gate = g->d_flags + kHasLake;
        if (!g->rank_uploaded) {
            FL_TRY(sync_status(g, h));
            lakes = h[kHasLake] != 0;
            gate = nullptr;
            if (lakes) FL_TRY(set_outlets(g, outlets, true));
        }
        if (lakes) {
            FL_TRY(enqueue_labels(g, gate));
            FL_TRY(enqueue_lakes(g, gate));
        }
        FL_TRY(enqueue_basin_pass(g));
        if (g->d_titer) {
            k_terrain_iters<<<blocks_for(g->terrains), kThreads, 0, g->stream>>>(
                g->terrains, g->d_tchg, g->d_titer, (uint32_t)(it + 1));
            FL_CU(cudaGetLastError());
        }
        FL_TRY(enqueue_status(g, (int)(it & 1)));
        if (it > 0) {
            if (int rc = take_status(g, (int)((it - 1) & 1), h)) return drained(rc);
            if (!h[kChanged]) {                       // iteration it - 1 was the last
                iters = (uint32_t)it;
                settled = true;
            }
        }
    }
    if (!settled && it > 0) {                         // the last iteration's status
        if (int rc = take_status(g, (int)((it - 1) & 1), h)) return drained(rc);
        iters = (uint32_t)it;
    }
    if (terrain_iters) {
        if (g->d_titer) {
            FL_CU(cudaMemcpyAsync(terrain_iters, g->d_titer, g->terrains * sizeof(uint32_t),
                                  cudaMemcpyDeviceToHost, g->stream));
            FL_CU(cudaStreamSynchronize(g->stream));
            for (uint32_t t = 0; t < g->terrains; ++t)
                if (!terrain_iters[t]) terrain_iters[t] = iters;
        } else {
            terrain_iters[0] = iters;
        }
    }
    FL_CU(cudaEventRecord(g->ev1, g->stream));
    FL_TRY(download_permuted(g, g->d_elev, out_elev));
    FL_CU(cudaStreamSynchronize(g->stream));
    kresolve(g);
    if (out_iters) *out_iters = iters;
    if (loop_ms) {
        float ms = 0;
        FL_CU(cudaEventElapsedTime(&ms, g->ev0, g->ev1));
        *loop_ms = ms;
    }
    if (total_ms)
        *total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start).count();
    return FL_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

const char* fl_last_error(void) { return g_err.c_str(); }

}  // extern "C"

namespace {

// A model on the current device.  k_terr > 1 packs terrains: site_off / def_off give
// each terrain's caller sites and default outlets, no edge may cross terrains, and each
// terrain is ordered along its own Hilbert curve (coordinates are per terrain).
int create_graph(uint32_t n, const uint32_t* row_ptr, const uint32_t* col, const double* len,
                 const double* area, const uint32_t* default_outlets, uint32_t n_default,
                 const double* xs, const double* ys, uint32_t k_terr, const uint32_t* site_off,
                 const uint32_t* def_off, fl_graph** out, const fl::GraphPart* parts = nullptr) {
    g_err.clear();
    if (!out || (!parts && (!row_ptr || (!col && n) || (!len && n) || !area)) ||
        (n_default && !default_outlets) || n == 0 || n >= kNone || k_terr == 0 ||
        (k_terr > 1 && (!site_off || !def_off))) {
        g_err = "invalid graph arguments";
        return FL_ERR_INVALID_ARGUMENT;
    }
    *out = nullptr;
    std::vector<uint32_t> so(k_terr + 1), dof(k_terr + 1);
    if (k_terr == 1) {
        so = {0, n};
        dof = {0, n_default};
    } else {
        for (uint32_t t = 0; t <= k_terr; ++t) {
            so[t] = site_off[t];
            dof[t] = def_off[t];
        }
        if (so[0] != 0 || so[k_terr] != n || dof[0] != 0 || dof[k_terr] != n_default) {
            g_err = "terrain offsets do not cover the sites / default outlets";
            return FL_ERR_INVALID_ARGUMENT;
        }
        for (uint32_t t = 0; t < k_terr; ++t)
            if (so[t + 1] <= so[t] || dof[t + 1] < dof[t]) {
                g_err = "terrain offsets not increasing (empty terrain?)";
                return FL_ERR_INVALID_ARGUMENT;
            }
    }
    std::vector<uint64_t> eo;                 // with parts: every terrain's first slot
    uint64_t nnz = 0;
    if (parts) {
        eo.assign(k_terr + 1, 0);
        for (uint32_t t = 0; t < k_terr; ++t) {
            const fl::GraphPart& pt = parts[t];
            const uint32_t m = so[t + 1] - so[t];
            if (!pt.row_ptr || !pt.area || (pt.row_ptr[m] && (!pt.col || !pt.len))) {
                g_err = "invalid graph arguments";
                return FL_ERR_INVALID_ARGUMENT;
            }
            if (pt.row_ptr[0] != 0) { g_err = "row_ptr[0] != 0"; return FL_ERR_INVALID_ARGUMENT; }
            eo[t + 1] = eo[t] + pt.row_ptr[m];
        }
        nnz = eo[k_terr];
    } else {
        nnz = row_ptr[n];
        if (row_ptr[0] != 0) { g_err = "row_ptr[0] != 0"; return FL_ERR_INVALID_ARGUMENT; }
    }
    if (nnz >= 0xffffffffull) { g_err = "more than 2^32 - 2 adjacency slots"; return FL_ERR_INVALID_ARGUMENT; }
    // default outlets: in their terrain, not repeated (the rest is checked on the device)
    for (uint32_t t = 0; t < k_terr; ++t) {
        std::vector<uint8_t> seen(so[t + 1] - so[t], 0);
        for (uint32_t i = dof[t]; i < dof[t + 1]; ++i) {
            const uint32_t o = default_outlets[i];
            if (o < so[t] || o >= so[t + 1] || seen[o - so[t]]) {
                g_err = "default outlet out of its terrain's range or repeated";
                return FL_ERR_INVALID_ARGUMENT;
            }
            seen[o - so[t]] = 1;
        }
    }
    fl_graph* g = new fl_graph();
    if (cudaGetDevice(&g->device) != cudaSuccess) g->device = 0;
    g->n = n;
    g->nnz = nnz;
    g->terrains = k_terr;
    struct Track {
        explicit Track(uint64_t* b) { t_alloc_bytes = b; }
        ~Track() {
            t_alloc_bytes = nullptr;
            t_alloc_stream = nullptr;
        }
    } track(&g->dev_bytes);
    keep_pool_memory();
    g->site_off = so;
    g->def_off = dof;
    for (uint32_t t = 0; t < k_terr; ++t) g->noise_n = std::max(g->noise_n, so[t + 1] - so[t]);
    int rc = FL_OK;
    auto fail = [&](int r) { free_graph(g); return r; };
    cudaError_t e = cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) { set_err("cudaStreamCreate", e); return fail(FL_ERR_CUDA); }
    t_alloc_stream = g->stream;
    if (cudaEventCreate(&g->ev0) != cudaSuccess || cudaEventCreate(&g->ev1) != cudaSuccess ||
        cudaEventCreateWithFlags(&g->ev_status[0], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&g->ev_status[1], cudaEventDisableTiming) != cudaSuccess) {
        g_err = "cudaEventCreate failed";
        return fail(FL_ERR_CUDA);
    }
    if ((rc = dalloc(&g->d_row, n + 1)) || (rc = dalloc(&g->d_col, nnz)) ||
        (rc = dalloc(&g->d_len, nnz)) || (rc = dalloc(&g->d_ilen, nnz)) ||
        (rc = dalloc(&g->d_area, n)) ||
        (rc = dalloc(&g->d_perm, n)) || (rc = dalloc(&g->d_inv, n)) || (rc = alloc_workspace(g)))
        return fail(rc);
    if (k_terr > 1 &&
        ((rc = dalloc(&g->d_noise_idx, n)) || (rc = dalloc(&g->d_tid, n)) ||
         (rc = dalloc(&g->d_tchg, k_terr)) || (rc = dalloc(&g->d_titer, k_terr))))
        return fail(rc);
    // upload, check and relabel on the device
    fl::GraphInput gi{n, nnz, row_ptr, col, len, area, (xs && ys) ? xs : nullptr,
                      (xs && ys) ? ys : nullptr, k_terr, so.data(), parts,
                      parts ? eo.data() : nullptr};
    fl::GraphOutput go{g->d_row, g->d_col, g->d_len, g->d_area, g->d_perm, g->d_inv, g->d_tid,
                       g->d_noise_idx};
    std::string why;
    rc = fl::build_device_graph(g->stream, gi, go, &why);
    if (rc != FL_OK) {
        g_err = why;
        return fail(rc);
    }
    fl::launch_inv_len(g->stream, nnz, g->d_len, g->d_ilen);
    // the maps between caller and device order, kept on the host for the boundary
    g->perm.resize(n);
    g->inv.resize(n);
    if (cudaMemcpyAsync(g->perm.data(), g->d_perm, n * 4ull, cudaMemcpyDeviceToHost, g->stream) != cudaSuccess ||
        cudaMemcpyAsync(g->inv.data(), g->d_inv, n * 4ull, cudaMemcpyDeviceToHost, g->stream) != cudaSuccess ||
        cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(g->stream) != cudaSuccess) {
        g_err = "graph set-up on the device failed";
        return fail(FL_ERR_CUDA);
    }
    g->def_outlets.resize(n_default);
    for (uint32_t i = 0; i < n_default; ++i) g->def_outlets[i] = g->inv[default_outlets[i]];
    *out = g;
    return FL_OK;
}

}  // namespace

extern "C" {

int fl_graph_create(uint32_t n, const uint32_t* row_ptr, const uint32_t* col, const double* len,
                    const double* area, const uint32_t* default_outlets, uint32_t n_default,
                    const double* xs, const double* ys, fl_graph** out) {
    return create_graph(n, row_ptr, col, len, area, default_outlets, n_default, xs, ys, 1,
                        nullptr, nullptr, out);
}

int fl_batch_create(uint32_t terrains, const uint32_t* site_off, const uint32_t* row_ptr,
                    const uint32_t* col, const double* len, const double* area,
                    const uint32_t* def_off, const uint32_t* default_outlets, const double* xs,
                    const double* ys, fl_graph** out) {
    if (!site_off || !def_off || terrains == 0) {
        g_err = "invalid batch arguments";
        return FL_ERR_INVALID_ARGUMENT;
    }
    return create_graph(site_off[terrains], row_ptr, col, len, area, default_outlets,
                        def_off[terrains], xs, ys, terrains, site_off, def_off, out);
}

int fl_batch_create_parts(uint32_t terrains, const uint32_t* sites,
                          const uint32_t* const* row_ptr, const uint32_t* const* col,
                          const double* const* len, const double* const* area,
                          const uint32_t* n_default, const uint32_t* const* default_outlets,
                          const double* const* xs, const double* const* ys, fl_graph** out) {
    g_err.clear();
    if (!sites || !row_ptr || !col || !len || !area || !n_default || !default_outlets ||
        terrains == 0) {
        g_err = "invalid batch arguments";
        return FL_ERR_INVALID_ARGUMENT;
    }
    std::vector<uint32_t> so(terrains + 1, 0), dof(terrains + 1, 0), defs;
    std::vector<fl::GraphPart> parts(terrains);
    for (uint32_t t = 0; t < terrains; ++t) {
        if ((uint64_t)so[t] + sites[t] >= kNone || (n_default[t] && !default_outlets[t])) {
            g_err = "invalid batch arguments";
            return FL_ERR_INVALID_ARGUMENT;
        }
        so[t + 1] = so[t] + sites[t];
        dof[t + 1] = dof[t] + n_default[t];
        for (uint32_t i = 0; i < n_default[t]; ++i) defs.push_back(so[t] + default_outlets[t][i]);
        parts[t] = fl::GraphPart{row_ptr[t], col[t], len[t], area[t], xs ? xs[t] : nullptr,
                                 ys ? ys[t] : nullptr};
    }
    return create_graph(so[terrains], nullptr, nullptr, nullptr, nullptr, defs.data(),
                        dof[terrains], nullptr, nullptr, terrains, so.data(), dof.data(), out,
                        parts.data());
}

int fl_batch_generate_parts(fl_graph* g, const double* const* base,
                            const double* const* erodibility, const double* const* uplift,
                            const uint8_t* const* is_outlet, const double* const* max_slope,
                            int64_t max_iteration, double* const* out_elev,
                            uint32_t* out_terrain_iterations, uint32_t* out_iterations,
                            double* loop_ms, double* total_ms) {
    using D = HostCols<const double>;
    return generate_impl(g, g ? g->n : 0, D::of_parts(base), D::of_parts(erodibility),
                         D::of_parts(uplift), HostCols<const uint8_t>::of_parts(is_outlet),
                         D::of_parts(max_slope), max_iteration,
                         HostCols<double>::of_parts(out_elev), out_iterations, loop_ms, total_ms,
                         out_terrain_iterations);
}

uint32_t fl_graph_num_terrains(const fl_graph* g) { return g ? g->terrains : 0; }

uint64_t fl_graph_device_bytes(const fl_graph* g) { return g ? g->dev_bytes : 0; }

uint64_t fl_model_device_bytes(uint32_t n, uint64_t nnz) {
    // per site about 370 B of arrays (per-site state, lake ranks, basin workspace,
    // operand and top-down records, donor lists), per slot the CSR's 12 B and 4 B of 1/len; per-chain
    // tables of kahn_min_width entries (64 B each), per-round tables and status words
    const uint64_t width = kahn_min_width(n);
    const uint64_t rounds = n / std::min<uint64_t>(width, kKahnMinWidthEarly) + 64;
    return 400ull * n + 16ull * nnz + 64ull * width + 24ull * rounds + 4096;
}

int fl_batch_generate(fl_graph* g, uint32_t n_params, const double* base,
                      const double* erodibility, const double* uplift, const uint8_t* is_outlet,
                      const double* max_slope, int64_t max_iteration, double* out_elev,
                      uint32_t* out_terrain_iterations, uint32_t* out_iterations,
                      double* loop_ms, double* total_ms) {
    return generate_impl(g, n_params, base, erodibility, uplift, is_outlet, max_slope,
                         max_iteration, out_elev, out_iterations, loop_ms, total_ms,
                         out_terrain_iterations);
}

void fl_graph_destroy(fl_graph* g) { free_graph(g); }

int fl_host_alloc(uint64_t bytes, void** out) {
    g_err.clear();
    if (out) *out = nullptr;
    if (!out || bytes == 0) return FL_ERR_INVALID_ARGUMENT;
    cudaError_t e = cudaHostAlloc(out, bytes, cudaHostAllocPortable);
    if (e != cudaSuccess) {
        set_err("cudaHostAlloc", e);
        *out = nullptr;
        return e == cudaErrorMemoryAllocation ? FL_ERR_OUT_OF_MEMORY : FL_ERR_CUDA;
    }
    return FL_OK;
}

void fl_host_free(void* p) {
    if (p) cudaFreeHost(p);
}

uint32_t fl_graph_num_sites(const fl_graph* g) { return g ? g->n : 0; }
uint64_t fl_graph_num_slots(const fl_graph* g) { return g ? g->nnz : 0; }

int fl_generate(fl_graph* g, uint32_t n_params, const double* base, const double* erodibility,
                const double* uplift, const uint8_t* is_outlet, const double* max_slope,
                int64_t max_iteration, double* out_elev, uint32_t* out_iterations) {
    return generate_impl(g, n_params, base, erodibility, uplift, is_outlet, max_slope,
                         max_iteration, out_elev, out_iterations, nullptr, nullptr);
}

int fl_generate_timed(fl_graph* g, uint32_t n_params, const double* base,
                      const double* erodibility, const double* uplift, const uint8_t* is_outlet,
                      const double* max_slope, int64_t max_iteration, double* out_elev,
                      uint32_t* out_iterations, double* loop_ms, double* total_ms) {
    return generate_impl(g, n_params, base, erodibility, uplift, is_outlet, max_slope,
                         max_iteration, out_elev, out_iterations, loop_ms, total_ms);
}

// The probes take and return caller-order arrays and site ids.
int fl_probe_receivers(fl_graph* g, const double* elev, const uint8_t* outlet_table,
                       uint32_t* next_out, int* has_lake) {
    if (!g) return FL_ERR_MODEL_NOT_SET;
    FL_CU(cudaSetDevice(g->device));
    uint32_t n = g->n;
    std::vector<uint8_t> table(n);
    for (uint32_t j = 0; j < n; ++j) table[j] = outlet_table[g->perm[j]];
    FL_TRY(upload_permuted(g, elev, g->d_elev));
    FL_CU(cudaMemcpyAsync(g->d_outlet, table.data(), n, cudaMemcpyHostToDevice, g->stream));
    FL_CU(cudaMemsetAsync(g->d_flags, 0, kNumFlags * sizeof(int), g->stream));
    FL_TRY(enqueue_receivers(g));
    int h[kNumFlags];
    FL_TRY(sync_status(g, h));
    const int hl = h[kHasLake];
    std::vector<uint32_t> nx(n);
    FL_CU(cudaMemcpyAsync(nx.data(), g->d_next, n * 4ull, cudaMemcpyDeviceToHost, g->stream));
    FL_CU(cudaStreamSynchronize(g->stream));
    for (uint32_t i = 0; i < n; ++i) next_out[i] = g->perm[nx[g->inv[i]]];
    if (has_lake) *has_lake = hl;
    return FL_OK;
}

int fl_probe_lakes(fl_graph* g, const uint32_t* outlets, uint32_t n_outlets,
                   const uint32_t* next_in, uint32_t* next_out, uint32_t* label_out) {
    if (!g) return FL_ERR_MODEL_NOT_SET;
    FL_CU(cudaSetDevice(g->device));
    uint32_t n = g->n;
    FL_TRY(set_outlets(g, to_device_ids(g, outlets, n_outlets), true));
    FL_CU(cudaMemsetAsync(g->d_flags, 0, kNumFlags * sizeof(int), g->stream));
    std::vector<uint32_t> nx(n);
    for (uint32_t j = 0; j < n; ++j) nx[j] = g->inv[next_in[g->perm[j]]];
    FL_CU(cudaMemcpyAsync(g->d_next, nx.data(), n * 4ull, cudaMemcpyHostToDevice, g->stream));
    std::vector<double> ones(n, 1.0);
    FL_CU(cudaMemcpyAsync(g->d_rlen, ones.data(), n * 8ull, cudaMemcpyHostToDevice, g->stream));
    FL_TRY(enqueue_labels(g, nullptr));
    std::vector<uint32_t> lab(n);
    FL_CU(cudaMemcpyAsync(lab.data(), g->d_lab, n * 4ull, cudaMemcpyDeviceToHost, g->stream));
    FL_TRY(enqueue_lakes(g, nullptr));
    FL_CU(cudaMemcpyAsync(nx.data(), g->d_next, n * 4ull, cudaMemcpyDeviceToHost, g->stream));
    int h[kNumFlags];
    FL_TRY(sync_status(g, h));
    FL_TRY(device_error(h));
    for (uint32_t i = 0; i < n; ++i) {
        next_out[i] = g->perm[nx[g->inv[i]]];
        if (label_out) label_out[i] = g->perm[lab[g->inv[i]]];
    }
    return FL_OK;
}

int fl_probe_tree_pass(fl_graph* g, const uint32_t* outlets, uint32_t n_outlets,
                       const uint32_t* next, const double* erodibility, const double* uplift,
                       const double* max_slope, double* elev, double* drainage_out,
                       double* response_out, int* changed) {
    if (!g) return FL_ERR_MODEL_NOT_SET;
    FL_CU(cudaSetDevice(g->device));
    uint32_t n = g->n;
    FL_TRY(upload_params(g, nullptr, erodibility, uplift, max_slope));
    FL_TRY(set_outlets(g, to_device_ids(g, outlets, n_outlets), false));
    std::vector<uint32_t> nx(n);
    for (uint32_t j = 0; j < n; ++j) nx[j] = g->inv[next[g->perm[j]]];
    FL_CU(cudaMemcpyAsync(g->d_next, nx.data(), n * 4ull, cudaMemcpyHostToDevice, g->stream));
    FL_TRY(upload_permuted(g, elev, g->d_elev));
    // receiver lengths as has_edge reports them (device order)
    FL_TRY(ensure_host_csr(g));
    std::vector<double> rl(n);
    for (uint32_t j = 0; j < n; ++j) {
        rl[j] = 1.0;
        if (nx[j] != j)
            for (uint32_t s = g->h_row[j]; s < g->h_row[j + 1]; ++s)
                if (g->h_col[s] == nx[j]) { rl[j] = g->h_len[s]; break; }
    }
    FL_CU(cudaMemcpyAsync(g->d_rlen, rl.data(), n * 8ull, cudaMemcpyHostToDevice, g->stream));
    k_fill_f64<<<blocks_for(n), kThreads, 0, g->stream>>>(n, g->d_A, g->d_area);
    FL_CU(cudaMemsetAsync(g->d_flags, 0, kNumFlags * sizeof(int), g->stream));
    FL_CU(cudaStreamSynchronize(g->stream));
    FL_TRY(enqueue_basin_pass(g, true));
    int h[kNumFlags];
    FL_TRY(sync_status(g, h, true));
    FL_TRY(finish_basin_pass(g, h));
    const int ch = h[kChanged];
    FL_TRY(download_permuted(g, g->d_elev, elev));
    FL_CU(cudaStreamSynchronize(g->stream));
    if (drainage_out) {
        FL_TRY(download_permuted(g, g->d_A, drainage_out));
        FL_CU(cudaStreamSynchronize(g->stream));
    }
    if (response_out) {
        k_rec_times<<<blocks_for(n), kThreads, 0, g->stream>>>(n, g->d_trec, g->d_w);
        g->w_valid = false;
        FL_TRY(download_permuted(g, g->d_w, response_out));
        FL_CU(cudaStreamSynchronize(g->stream));
    }
    if (changed) *changed = ch;
    return FL_OK;
}

int fl_probe_prim_rank(fl_graph* g, const uint32_t* outlets, uint32_t n_outlets, uint32_t* rank) {
    if (!g) return FL_ERR_MODEL_NOT_SET;
    std::vector<uint32_t> o = to_device_ids(g, outlets, n_outlets);
    std::vector<uint32_t> r(g->n);
    FL_TRY(ensure_host_csr(g));
    if (!fl::lake_heap_rank(g->n, g->h_row.data(), g->h_col.data(), g->h_len.data(), o.data(),
                            n_outlets, r.data())) {
        g_err = "NaN edge length in the lake traversal";
        return FL_ERR_INVALID_ARGUMENT;
    }
    for (uint32_t i = 0; i < g->n; ++i) rank[i] = r[g->inv[i]];
    return FL_OK;
}

int fl_probe_chain_fold(const double* operands, uint32_t n, double start, double* out) {
    double* d = nullptr;
    FL_CU(cudaMalloc(&d, std::max<uint64_t>(1, 2ull * n) * 8));
    cudaError_t e = cudaMemcpy(d, operands, n * 8ull, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = fl::fold_probe(d, n, start, d + n);
    if (e == cudaSuccess) e = cudaMemcpy(out, d + n, n * 8ull, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) {
        set_err("fl_probe_chain_fold", e);
        return FL_ERR_CUDA;
    }
    return FL_OK;
}

int fl_select_device(int device) {
    FL_CU(cudaSetDevice(device));
    return FL_OK;
}

int fl_graph_set_timing(fl_graph* g, int enable) {
    if (!g) return FL_ERR_MODEL_NOT_SET;
    g->timing = enable != 0;
    return FL_OK;
}

uint64_t fl_graph_host_syncs(const fl_graph* g) { return g ? g->host_syncs : 0; }

int fl_graph_set_sized_grids(fl_graph* g, int sized) {
    if (!g) return FL_ERR_MODEL_NOT_SET;
    if (sized < -1 || sized > 1) return FL_ERR_INVALID_ARGUMENT;
    g->sized_grids = sized;
    return FL_OK;
}

int fl_set_tuning(const char* name, int64_t value) {
    g_err.clear();
    fl::Tuning& t = fl::tuning();
    const std::string k = name ? name : "";
    if (k == "low_ilp" && (value == -1 || value == 1 || value == 2 || value == 4)) {
        t.low_ilp = (int)value;
    } else if (k == "walk_per_sm" && value >= -1 && value <= 64) {
        t.walk_per_sm = (int)value;
    } else if (k == "sized_grids" && value >= -1 && value <= 1) {
        t.sized_grids = (int)value;
    } else if (k == "gpu_rank" && (value == 0 || value == 1)) {
        t.gpu_rank = value != 0;
    } else if (k == "kahn_min_width" &&
               (value == -1 || value == 0 || (value >= 256 && value <= (1 << 24)))) {
        t.kahn_min_width = value;
    } else {
        g_err = "fl_set_tuning: unknown name or value out of range";
        return FL_ERR_INVALID_ARGUMENT;
    }
    return FL_OK;
}

int64_t fl_get_tuning(const char* name) {
    const fl::Tuning& t = fl::tuning();
    const std::string k = name ? name : "";
    if (k == "low_ilp") return t.low_ilp;
    if (k == "walk_per_sm") return t.walk_per_sm;
    if (k == "kahn_min_width") return t.kahn_min_width;
    if (k == "gpu_rank") return t.gpu_rank ? 1 : 0;
    if (k == "sized_grids") return t.sized_grids;
    return -2;
}

int fl_schedule_entry(uint32_t i, uint32_t* max_sites, int* packed, int* low_ilp,
                      uint32_t* walk_per_sm, uint32_t* kahn_min_width, int* sized_grids) {
    const auto& s = fl::schedule();
    if (i >= s.size()) return FL_ERR_INVALID_ARGUMENT;
    if (max_sites) *max_sites = s[i].max_sites;
    if (packed) *packed = s[i].packed ? 1 : 0;
    if (low_ilp) *low_ilp = s[i].shape.low_ilp;
    if (walk_per_sm) *walk_per_sm = s[i].shape.walk_per_sm;
    if (kahn_min_width) *kahn_min_width = s[i].shape.kahn_min_width;
    if (sized_grids) *sized_grids = s[i].shape.sized_grids ? 1 : 0;
    return FL_OK;
}

int fl_graph_rank_info(const fl_graph* g, double* ms, int* on_gpu) {
    if (!g) return FL_ERR_MODEL_NOT_SET;
    if (ms) *ms = g->rank_ms;
    if (on_gpu) *on_gpu = g->rank_gpu;
    return FL_OK;
}

int fl_probe_lake_rank_gpu(fl_graph* g, const uint32_t* outlets, uint32_t n_outlets,
                           uint32_t* rank, int* used_gpu) {
    if (!g) return FL_ERR_MODEL_NOT_SET;
    if (!rank || (n_outlets && !outlets)) return FL_ERR_INVALID_ARGUMENT;
    FL_CU(cudaSetDevice(g->device));
    const uint32_t n = g->n;
    for (uint32_t i = 0; i < n_outlets; ++i)
        if (outlets[i] >= n) return FL_ERR_INVALID_ARGUMENT;
    std::vector<uint32_t> o = to_device_ids(g, outlets, n_outlets), prefix;
    int pr = FL_OK;
    if (g->terrains > 1) {                     // the prefix replays terrain after terrain
        g_err = "fl_probe_lake_rank_gpu takes a single-terrain model";
        return FL_ERR_INVALID_ARGUMENT;
    }
    FL_TRY(lake_prefix(g, o, prefix, &pr));
    if (pr == 1) {
        g_err = "NaN edge length in the lake traversal";
        return FL_ERR_INVALID_ARGUMENT;
    }
    // into the solver's rank arrays: the next lake pass recomputes its own order
    g->rank_valid = g->rank_uploaded = false;
    fl::GpuRankInfo info;
    if (pr == 2) info.fallback_reason = "a zero-length edge reaches a site at key 0.0";
    const fl::RankResult r =
        pr == 2 ? fl::kRankFallback
                : fl::gpu_lake_rank(g->stream, n, g->d_row, g->d_col, g->d_len, g->nnz, prefix,
                                    g->d_rank, g->d_sor, &info);
    if (r == fl::kRankError) {
        set_err("lake order on the GPU", info.error);
        return FL_ERR_CUDA;
    }
    if (used_gpu) *used_gpu = r == fl::kRankOk ? 1 : 0;
    if (r == fl::kRankFallback) {
        g_err = info.fallback_reason;
        return FL_OK;
    }
    std::vector<uint32_t> dr(n);
    FL_CU(cudaMemcpyAsync(dr.data(), g->d_rank, n * 4ull, cudaMemcpyDeviceToHost, g->stream));
    FL_CU(cudaStreamSynchronize(g->stream));
    for (uint32_t i = 0; i < n; ++i) rank[i] = dr[g->inv[i]];
    return FL_OK;
}

void fl_graph_reset_stats(fl_graph* g) {
    if (!g) return;
    g->host_syncs = 0;
    for (int c = 0; c < kcCount; ++c) {
        g->k_launches[c] = 0;
        g->k_ms[c] = 0;
        g->k_bytes[c] = 0;
    }
}

uint32_t fl_num_kernel_classes(void) { return kcCount; }

int fl_graph_basin_stats(const fl_graph* g, uint64_t* out, uint32_t cap) {
    if (!g) return FL_ERR_MODEL_NOT_SET;
    const uint32_t* m = g->last_meta;
    auto u64 = [&](int slot) { return (uint64_t)m[slot] | ((uint64_t)m[slot + 1] << 32); };
    const uint64_t up = u64(kMetaUpSlow), down = u64(kMetaDownSlow);
    const uint64_t vals[] = {m[kMetaRStop], m[kMetaLeaves], m[kMetaNs], m[kMetaChains],
                             m[kMetaMaxChain], m[kMetaSlow], m[kMetaSpinUp], m[kMetaSpinDown],
                             (up >> kStatDurShift) << 6, ((up >> kStatCycShift) & kStat22) << 7,
                             up & kStat20,
                             (down >> kStatDurShift) << 6, ((down >> kStatCycShift) & kStat22) << 7,
                             down & kStat20};
    for (uint32_t i = 0; i < cap && i < sizeof vals / sizeof vals[0]; ++i) out[i] = vals[i];
    return FL_OK;
}

int fl_graph_round_trace(fl_graph* g, uint32_t cap, uint32_t* rounds, uint32_t* offsets,
                         uint64_t* up_ns, uint64_t* down_ns) {
    if (!g) return FL_ERR_MODEL_NOT_SET;
    if (!rounds) return FL_ERR_INVALID_ARGUMENT;
    FL_CU(cudaSetDevice(g->device));
    const uint32_t r = g->last_meta[kMetaRStop];
    *rounds = r;
    const uint32_t k = std::min<uint32_t>(cap, r + 1);
    if (k == 0 || !g->d_rtime) return FL_OK;
    if (offsets) FL_CU(cudaMemcpy(offsets, g->d_roff, k * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    if (up_ns) FL_CU(cudaMemcpy(up_ns, g->d_rtime, k * sizeof(uint64_t), cudaMemcpyDeviceToHost));
    if (down_ns)
        FL_CU(cudaMemcpy(down_ns, g->d_rtime + g->max_rounds + 1, k * sizeof(uint64_t),
                         cudaMemcpyDeviceToHost));
    return FL_OK;
}

int fl_graph_kernel_stats(const fl_graph* g, uint32_t cls, const char** name, uint64_t* launches,
                          double* device_ms, double* bytes) {
    if (!g) return FL_ERR_MODEL_NOT_SET;
    if (cls >= (uint32_t)kcCount) return FL_ERR_INVALID_ARGUMENT;
    if (name) *name = kKClassName[cls];
    if (launches) *launches = g->k_launches[cls];
    if (device_ms) *device_ms = g->k_ms[cls];
    if (bytes) *bytes = g->k_bytes[cls];
    return FL_OK;
}

int fl_probe_rng_f64(uint64_t seed, uint64_t first, uint64_t count, double* out) {
    double* d = nullptr;
    FL_CU(cudaMalloc(&d, std::max<uint64_t>(1, count) * 8));
    k_rng_f64<<<blocks_for(count), kThreads>>>(seed, first, count, d);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpy(out, d, count * 8, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) {
        set_err("fl_probe_rng_f64", e);
        return FL_ERR_CUDA;
    }
    return FL_OK;
}

}  // extern "C"
