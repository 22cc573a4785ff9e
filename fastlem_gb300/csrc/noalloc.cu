// noalloc.cu -- basin labels for callers that cannot allocate device memory.
//
// Some callers of this library must not call cudaMalloc: a service that hands out
// device memory from its own fixed, pre-sized pool has to keep every byte inside
// that pool's accounting, and cudaMalloc / cudaFree also synchronise the whole
// device, which such a service avoids while other requests are in flight.
// fl_basin_labels_noalloc gives them fastlem's basin labels (the root each site
// drains to, src/lem/stream_tree.rs:139-173) on device arrays they already own,
// allocating nothing: its only scratch is the fixed array below.
//
// Scratch: g_labels_scratch, kNoAllocMaxSites + kStatusWords uint32 words (16 MiB +
// 256 B).  Every GPU that loads this library holds it until the process exits.
// Host code cannot use the array's name as a device address, so the address is taken
// once per device with cudaGetSymbolAddress, by the first call made with that device
// current; make that first call before any stream capture.  The address is kept for
// the life of the process: after a cudaDeviceReset the module is loaded again and
// the array may move, so this entry point must not be called on a device after that
// device was reset.  All calls share the array and it keeps the last call's
// contents: the status words are cleared at the start of each call and round, the
// label buffer is fully rewritten.  Two calls that overlap on the same GPU (different
// streams or threads) race on the scratch, so callers must serialise them.
//
// Pointer jumping settles in ceil(log2(longest path)) rounds on a forest.  A receiver
// cycle either keeps moving (the round limit reports it) or, for a cycle whose length
// is a power of two, settles with every cycle site labelled as itself; the final check
// catches that case: every label must be an outlet or a site that is its own receiver.

#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>
#include <string>

#include "common.cuh"
#include "fastlem_gb300.h"
#include "kernels.h"

namespace {

constexpr uint32_t kNoAllocMaxSites = 4u << 20;   // 4,194,304 sites
constexpr uint32_t kStatusWords = 64;             // keeps the label buffer 256-byte aligned
constexpr int kMaxDevices = 64;
constexpr int kMaxRounds = 64;                    // 2^64 > any receiver path length

static __device__ __align__(256) uint32_t g_labels_scratch[kStatusWords + kNoAllocMaxSites];

std::mutex g_mu;
uint32_t* g_scratch_ptr[kMaxDevices] = {};

// Device address of the scratch on the current device (taken once per device).
int scratch_address(uint32_t** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        fl::set_last_error("fl_basin_labels_noalloc: no usable current CUDA device");
        return FL_ERR_CUDA;
    }
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_labels_scratch);
        if (e != cudaSuccess || !p) {
            fl::set_last_error((std::string("fl_basin_labels_noalloc: cudaGetSymbolAddress failed: ") +
                                cudaGetErrorString(e)).c_str());
            return FL_ERR_CUDA;
        }
        g_scratch_ptr[dev] = (uint32_t*)p;
    }
    *out = g_scratch_ptr[dev];
    return FL_OK;
}

// Outlets are roots whatever their receiver says (stream_tree.rs:140-142); every
// other site starts from its receiver.  A receiver outside [0, n) raises status[2]
// and is not followed.
__global__ void k_na_init(uint32_t n, const uint32_t* __restrict__ next,
                          const uint8_t* __restrict__ outlet, uint32_t* __restrict__ lab,
                          uint32_t* __restrict__ status) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    bool bad = false;
    if (i < n) {
        uint32_t r = next[i];
        bad = r >= n;
        lab[i] = (outlet[i] || bad) ? i : r;
    }
    if (__syncthreads_or(bad) && threadIdx.x == 0) status[2] = 1;
}

// One pointer-jumping round; status[0] is raised when some label moved.
__global__ void k_na_jump(uint32_t n, const uint32_t* __restrict__ in, uint32_t* __restrict__ out,
                          uint32_t* __restrict__ status) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    bool moved = false;
    if (i < n) {
        uint32_t l = in[i];
        uint32_t ll = in[l];
        out[i] = ll;
        moved = ll != l;
    }
    if (__syncthreads_or(moved) && threadIdx.x == 0) status[0] = 1;
}

// has_lake: some site drains to a root that is not an outlet (stream_tree.rs:156-158),
// status[1].  A label that is neither an outlet nor its own receiver is a site on a
// receiver cycle (pointer jumping settled on it): status[3].
__global__ void k_na_lake(uint32_t n, const uint32_t* __restrict__ next,
                          const uint32_t* __restrict__ lab, const uint8_t* __restrict__ outlet,
                          uint32_t* __restrict__ status) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    bool lake = false, cycle = false;
    if (i < n) {
        const uint32_t l = lab[i];
        lake = !outlet[l];
        cycle = lake && next[l] != l;
    }
    if (__syncthreads_or(lake) && threadIdx.x == 0) status[1] = 1;
    if (__syncthreads_or(cycle) && threadIdx.x == 0) status[3] = 1;
}

__global__ void k_na_copy(uint32_t n, const uint32_t* __restrict__ in, uint32_t* __restrict__ out) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = in[i];
}

#define NA_CU(call)                                                                     \
    do {                                                                                \
        cudaError_t e_ = (call);                                                        \
        if (e_ != cudaSuccess) {                                                        \
            fl::set_last_error(                                                         \
                (std::string("fl_basin_labels_noalloc: ") + cudaGetErrorString(e_)).c_str()); \
            return FL_ERR_CUDA;                                                         \
        }                                                                               \
    } while (0)

}  // namespace

extern "C" {

int fl_basin_labels_noalloc(uint32_t n, const uint32_t* next, const uint8_t* outlet_table,
                            uint32_t* labels, int* has_lake, void* stream) {
    fl::set_last_error("");
    if (n == 0) {                          // nothing to label: the arrays are not read
        if (has_lake) *has_lake = 0;
        return FL_OK;
    }
    if (n > kNoAllocMaxSites) {
        char buf[160];
        snprintf(buf, sizeof buf,
                 "fl_basin_labels_noalloc: %u sites exceed its fixed scratch of %u sites",
                 n, kNoAllocMaxSites);
        fl::set_last_error(buf);
        return FL_ERR_INVALID_ARGUMENT;
    }
    if (!next || !outlet_table || !labels) {
        fl::set_last_error("fl_basin_labels_noalloc: null device array");
        return FL_ERR_INVALID_ARGUMENT;
    }
    uint32_t* scratch = nullptr;
    int rc = scratch_address(&scratch);
    if (rc != FL_OK) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    uint32_t* status = scratch;
    uint32_t* other = scratch + kStatusWords;
    const unsigned grid = (n + fl::kThreads - 1) / fl::kThreads;

    NA_CU(cudaMemsetAsync(status, 0, 4 * sizeof(uint32_t), st));
    k_na_init<<<grid, fl::kThreads, 0, st>>>(n, next, outlet_table, labels, status);
    NA_CU(cudaGetLastError());
    uint32_t* cur = labels;
    uint32_t* nxt = other;
    bool converged = false;
    for (int round = 0; round < kMaxRounds; ++round) {
        if (round > 0) NA_CU(cudaMemsetAsync(status, 0, sizeof(uint32_t), st));
        k_na_jump<<<grid, fl::kThreads, 0, st>>>(n, cur, nxt, status);
        NA_CU(cudaGetLastError());
        uint32_t words[3] = {0, 0, 0};
        NA_CU(cudaMemcpyAsync(words, status, sizeof words, cudaMemcpyDeviceToHost, st));
        NA_CU(cudaStreamSynchronize(st));
        if (words[2]) {
            fl::set_last_error("fl_basin_labels_noalloc: a receiver is outside [0, n)");
            return FL_ERR_INVALID_ARGUMENT;
        }
        uint32_t moved = words[0];
        uint32_t* t = cur;
        cur = nxt;
        nxt = t;
        if (!moved) {
            converged = true;
            break;
        }
    }
    if (!converged) {
        fl::set_last_error("fl_basin_labels_noalloc: receivers contain a cycle");
        return FL_ERR_DEVICE_LIMIT;
    }
    if (cur != labels) {
        k_na_copy<<<grid, fl::kThreads, 0, st>>>(n, cur, labels);
        NA_CU(cudaGetLastError());
    }
    k_na_lake<<<grid, fl::kThreads, 0, st>>>(n, next, labels, outlet_table, status);
    NA_CU(cudaGetLastError());
    uint32_t words[4] = {0, 0, 0, 0};
    NA_CU(cudaMemcpyAsync(words, status, sizeof words, cudaMemcpyDeviceToHost, st));
    NA_CU(cudaStreamSynchronize(st));
    if (words[3]) {
        fl::set_last_error("fl_basin_labels_noalloc: receivers contain a cycle");
        return FL_ERR_DEVICE_LIMIT;
    }
    if (has_lake) *has_lake = words[1] ? 1 : 0;
    return FL_OK;
}

}  // extern "C"
