// kernels.h -- host-side entry points of the solver's CUDA translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

namespace fl {

// Kernel classes for launch counting and per-class device timing.
enum KClass {
    kcNoise = 0,      // initial elevations
    kcReceivers,      // steepest-descent receivers
    kcLakes,          // basin labels + lake re-routing
    kcBasinBuild,     // donor counts, leaves, skeleton collection / layout / preparation
    kcKahn,           // bottom-up Kahn rounds (drainage area)
    kcSkelRank,       // pointer jumping over the skeleton
    kcSkelUp,         // skeleton chains bottom-up (drainage area)
    kcW,              // 1 / (k sqrt(A)) * len
    kcSkelDown,       // skeleton chains top-down (response time, elevation)
    kcLowDown,        // Kahn rounds top-down (response time, elevation)
    kcMisc,
    kcCount
};

// Skeleton chains are walked one warp each, this many warps per block.
constexpr int kWalkWarps = 4;

// Launch shapes and switch points of one model's solve.
struct Shape {
    int low_ilp;              // top-down Kahn rounds: sites in flight per thread (1, 2 or 4)
    uint32_t walk_per_sm;     // chain walker blocks per SM; 0: as many as fit
    uint32_t kahn_min_width;  // Kahn rounds stop below this frontier width; 0: n / 512
                              // clamped to [8192, 65536]
    bool sized_grids;         // cooperative grids scaled to the model (else the whole GPU)
};
// The schedule: per size class (models of up to max_sites sites; packed batches apart)
// the shapes the schedule sweep chose on GB300 (fastlem_gb300/schedule.json).
struct ScheduleEntry {
    uint32_t max_sites;
    bool packed;
    Shape shape;
};
const std::vector<ScheduleEntry>& schedule();
// Process-wide overrides of the schedule (-1: none) and the GPU lake-order switch;
// FL_LOW_ILP, FL_WALK_PER_SM, FL_KAHN_MIN_WIDTH and FL_GPU_RANK set them at load,
// fl_set_tuning at run time.
struct Tuning {
    int low_ilp = -1;
    int walk_per_sm = -1;
    int64_t kahn_min_width = -1;
    int sized_grids = -1;
    bool gpu_rank = true;
};
Tuning& tuning();
// The shapes for a model of n sites (packed: several terrains), overrides applied.
Shape shape_for(uint32_t n, bool packed);

// Largest skeleton chain count whose walk kernels are all co-resident on the
// current device (one warp per chain), and the walkers' grid (blocks of kWalkWarps
// warps) for the current tuning.
uint32_t walk_capacity();
uint32_t walk_grid(uint32_t per_sm);
// A cooperative grid of `full` co-resident blocks cut to `units` of work at
// `per_block` each (at least min_blocks) when sized grids are on: a small model then
// leaves most of the GPU to the solves of other streams.
inline unsigned sized_grid(bool sized, unsigned full, uint64_t units, uint64_t per_block,
                           unsigned min_blocks = 4) {
    if (!sized) return full;
    const uint64_t want = (units + per_block - 1) / per_block;
    const uint64_t b = want < min_blocks ? min_blocks : want;
    return (unsigned)(b < full ? b : full);
}

// Device-side bookkeeping words of one basin pass (uint32 slots of BasinArgs::meta).
enum Meta {
    kMetaLeaves = 0,   // number of leaves (Kahn round 0)
    kMetaCnt0,         // rotating append counters of the Kahn rounds
    kMetaCnt1,
    kMetaCnt2,
    kMetaRStop,        // number of Kahn rounds run
    kMetaFrontBeg,     // the unprocessed frontier = skeleton leaves
    kMetaFrontEnd,
    kMetaNs,           // skeleton size
    kMetaJump0,        // rotating "changed" words of the pointer jumping
    kMetaJump1,
    kMetaJump2,
    kMetaRankBuf,      // which ping-pong buffer holds the ranks
    kMetaChains,       // number of skeleton chains
    kMetaSlow,         // skeleton sites needing the full pull at walk time
    kMetaSpinUp,       // wait iterations of the bottom-up chain hand-offs
    kMetaSpinDown,     // wait iterations of the top-down chain hand-offs
    kMetaMaxChain,     // longest skeleton chain
    kMetaClaimUp,      // chains claimed by the bottom-up walkers
    kMetaClaimDown,    // chains claimed by the top-down walkers
    kMetaTok,          // used entries of the donor-list buffer
    kMetaMaxDepth,     // largest chain-bottom depth (sites from the root)
    kMetaMaxHeight,    // largest chain height (sites)
    kMetaUpSlow,       // (2 words, u64) slowest bottom-up chain, packed by pack_chain_stat
    kMetaUpSlowHi,
    kMetaDownSlow,     // (2 words, u64) slowest top-down chain, packed by pack_chain_stat
    kMetaDownSlowHi,
    kMetaCount
};
static_assert(kMetaUpSlow % 2 == 0 && kMetaDownSlow % 2 == 0, "u64 meta words must be aligned");

// Per-chain walk statistic packed for atomicMax: duration / 64 ns (22 bits), a cycle
// count / 128 (22 bits), a count (20 bits).  The largest key is the slowest chain.
constexpr int kStatDurShift = 42;
constexpr int kStatCycShift = 20;
constexpr uint64_t kStat22 = (1ull << 22) - 1;
constexpr uint64_t kStat20 = (1ull << 20) - 1;

// Per skeleton layout slot, what the bottom-up walk adds to the chain's running area:
// pre (the cell area plus the donors before the chain predecessor, in the reference's
// order) and up to three donor areas after the predecessor.
struct __align__(32) SlotRec {
    double pre, p0, p1, p2;
};
// Per skeleton layout slot: kind bits, addition count, donor-list length and the
// predecessor's position in it (see basin.cu), and the donor list's offset.
struct __align__(8) SlotInfo {
    uint32_t flags;
    uint32_t tokoff;
};

// Per site, once its response time is final: t, elevation, and its basin outlet's
// response time and (updated) elevation -- everything a donor needs from its receiver
// in one 32-byte load.  to is kNoOutletBits in a basin without an outlet.
struct __align__(32) TRec {
    double t, e, to, eo;
};
constexpr uint64_t kNoOutletBits = 0x7ff5000000000000ull;   // a signalling NaN

struct BasinArgs {
    uint32_t n;
    const uint32_t* row;
    const uint32_t* col;
    const double* area;
    const uint32_t* next;
    const double* rlen;
    const double* k;
    const double* u;
    const double* tanms;
    const uint8_t* outlet;
    double* A;
    TRec* rec_t;
    double* w;
    double* w_area;            // the A and receiver distance each w was computed from
    double* w_dist;
    bool w_valid;              // w / w_area / w_dist hold the previous pass's values
    bool all_records;          // every site's record is read afterwards (else leaves skip it)
    double* elev;
    uint32_t* pending;
    uint32_t* hgt;
    uint32_t* order;
    uint32_t* roff;
    uint64_t* rtime;           // globaltimer at the start of each round: Kahn rounds at
                               // [0, max_rounds], top-down rounds after them
    uint32_t max_rounds;
    uint32_t kahn_min_width;   // also the chain capacity
    uint32_t* meta;
    int* flags;
    // packed terrains (batched form): terrain of each site, per-terrain "elevation
    // changed" words and first unchanged iteration (nonzero: the terrain is at its fixed
    // point and its sites take no part in the pass); all null for a single terrain
    const uint32_t* tid;
    int* tchg;
    const uint32_t* titer;
    // skeleton
    uint32_t* sid;
    uint32_t* slist;
    uint32_t* desig;
    uint32_t* sptr0;
    uint32_t* sdist0;
    uint32_t* sptr1;
    uint32_t* sdist1;
    uint32_t* cid;
    uint32_t* cbot;
    uint32_t* clen;
    uint32_t* coff;
    uint32_t* layout;
    uint32_t* slot_chain;   // layout slot -> chain
    uint32_t* kslot;        // skeleton index -> layout slot
    uint32_t* cpar;         // per chain: root chain of its chain tree
    uint32_t* cqp;          // per chain: layout slot of the site it hangs from, or kNone
    uint32_t* cdep;         // per chain: its bottom's depth in sites below the root (pointer
                            // jumping, 2 buffers)
    uint32_t* cpar1;
    uint32_t* cdep1;
    uint32_t* chist;        // per depth (n + 1 entries): chain count, then first position in corder
    uint32_t* corder;       // chains by depth, shallowest first: the top-down claim order
    uint32_t* corder_up;    // chains by height, lowest first: the bottom-up claim order
    uint32_t walk_grid;     // blocks of the persistent chain walkers (all co-resident)
    int low_ilp;            // top-down Kahn rounds: sites in flight per thread
    bool sized_grids;       // cooperative grids scaled to n (else the whole GPU)
    double* el;             // skeleton elevations in layout order (slope limits only)
    uint32_t* cbas;         // per chain: basin outlet, its response time and elevation
    double* cto;
    double* ceo;
    bool slope;             // some site has a maximum slope
    SlotRec* rec;
    SlotInfo* info;
    double* pre;            // layout-order areas (bottom-up), response times (top-down)
    double* post;           // layout-order w (top-down)
    uint8_t* needl;         // per layout slot: another chain starts below this site
    double* tokval;         // donor lists: final donor areas, chain bottoms pushed at walk time
    uint32_t* tokslot;      // per donor-list entry: the slot whose list it is
    uint32_t* pend;         // per layout slot: chain bottoms still to push into its list
    uint32_t tok_cap;
    uint64_t* push_to;      // per site: (stamp << 32) | tokval index its chain bottom fills
    int* bu_done;
    int* td_need;
    int* td_done;
    int stamp;       // distinct per pass: hand-off flags never need clearing
};

// Instrumentation callbacks around each launch group.
struct Hooks {
    void* ctx;
    void (*begin)(void* ctx);
    void (*end)(void* ctx, int cls, double bytes);
};

// Sets the message fl_last_error() returns on this thread.
void set_last_error(const char* msg);

// Packed terrains: sites of a terrain with titer[tid[v]] != 0 (converged) are left as
// they are (tid / titer null: every site is scanned).
void launch_receivers(cudaStream_t st, uint32_t n, const uint32_t* row, const uint32_t* col,
                      const double* len, const float* ilen, const double* elev,
                      const uint8_t* outlet, uint32_t* next, double* rlen, int* flags,
                      const uint32_t* tid = nullptr, const uint32_t* titer = nullptr);
// ilen[s] = 1/len[s] in f32 (NaN where not a normal f32), for launch_receivers.
void launch_inv_len(cudaStream_t st, uint64_t nnz, const double* len, float* ilen);

// A model as the caller gives it (host arrays; site_off has terrains + 1 offsets) and
// the device arrays ordering.cu fills in memory order (tid / noise_idx only for packed
// terrains).
// One terrain's arrays in its own site numbering (its row_ptr starts at 0).
struct GraphPart {
    const uint32_t* row_ptr;
    const uint32_t* col;
    const double* len;
    const double* area;
    const double* xs;
    const double* ys;
};
struct GraphInput {
    uint32_t n;
    uint64_t nnz;
    const uint32_t* row_ptr;
    const uint32_t* col;
    const double* len;
    const double* area;
    const double* xs;         // both null: caller order is kept
    const double* ys;
    uint32_t terrains;
    const uint32_t* site_off;
    const GraphPart* parts;   // instead of the arrays above: one part per terrain
    const uint64_t* slot_off; // with parts: first slot of every terrain (terrains + 1)
};
struct GraphOutput {
    uint32_t* row;
    uint32_t* col;
    double* len;
    double* area;
    uint32_t* perm;           // perm[device index] = caller index
    uint32_t* inv;
    uint32_t* tid;
    uint32_t* noise_idx;
};
// Uploads, checks (0, or 20 with *err for invalid input, 21 / 22 for CUDA errors /
// out of memory) and relabels; the arrays are ready when it returns.
int build_device_graph(cudaStream_t st, const GraphInput& in, const GraphOutput& out,
                       std::string* err);

// The lake heap's order on the GPU (lake_rank.cu): rank[v] (device order) and
// sor[rank] = site, from the tied prefix the host replayed (the sites processed while
// the smallest key is 0.0, in order).  kRankFallback: equal lengths could let the heap's
// arrangement decide, or some length is not positive -- the host heap must be used.
enum RankResult { kRankOk = 0, kRankFallback = 1, kRankError = 2 };
struct GpuRankInfo {
    cudaError_t error = cudaSuccess;
    const char* fallback_reason = "";
    uint32_t boruvka_rounds = 0, tree_edges = 0, lift_levels = 0, host_syncs = 0;
};
RankResult gpu_lake_rank(cudaStream_t st, uint32_t n, const uint32_t* row, const uint32_t* col,
                         const double* len, uint64_t nnz, const std::vector<uint32_t>& prefix,
                         uint32_t* rank, uint32_t* sor, GpuRankInfo* info);

// Runs the exact parallel fold over one chain of n operands starting at x0 (probe).
cudaError_t fold_probe(const double* y, uint32_t n, double x0, double* out);

// One drainage-area / response-time / elevation pass on final receivers.
cudaError_t basin_pass(const BasinArgs& a, cudaStream_t st, const Hooks& hk, uint32_t nnz);

}  // namespace fl
