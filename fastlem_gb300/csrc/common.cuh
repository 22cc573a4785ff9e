// common.cuh -- shared device helpers of the GB300 solve.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace fl {

constexpr uint32_t kNone = 0xffffffffu;
constexpr unsigned long long kNoKey = ~0ull;
constexpr int kThreads = 256;

// Device status words (int32 slots of the solver's flag array).
enum Flag {
    kHasLake = 0,   // some non-outlet site has no lower neighbour
    kChanged = 1,   // some elevation changed this iteration
    kJumped = 2,    // a pointer-jumping round changed something
    kError = 3,     // device-side limit hit (see kErr* codes)
    kBarrier = 4,   // grid barrier arrival counter
    kBarrierGen = 5,// grid barrier generation
    kExact = 6,     // receiver scans that needed the exact f64 fallback
    kJump0 = 8,     // rotating "a label moved" words of the pointer-jumping rounds
    kJump1 = 9,
    kJump2 = 10,
    kNumFlags = 16
};

// Values stored in flags[kError].
enum DeviceError {
    kErrNone = 0,
    kErrForest = 1,       // receivers do not form a forest (cycle / over-visit)
    kErrBarrier = 2,      // a grid barrier wait ran out
    kErrWait = 3,         // a chain hand-off wait ran out
    kErrCapacity = 4,     // a fixed-size table overflowed
};

// Spin limits: a wait that exceeds them reports an error instead of hanging.
constexpr uint32_t kSpinLimit = 1u << 24;

__device__ __forceinline__ int ld_acquire(const int* p) {
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(int* p, int v) {
    asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned ld_acquire_u(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void set_error(int* flags, int code) { atomicCAS(&flags[kError], 0, code); }

// Grid-wide barrier for cooperative (co-resident) launches.  Every block's thread
// 0 arrives on a counter; the last arrival bumps the generation.  Waits are bounded:
// on timeout the error word is set and false is returned, after which callers
// leave the kernel.
__device__ __forceinline__ bool grid_barrier(int* flags) {
    __syncthreads();
    __shared__ int ok;
    if (threadIdx.x == 0) {
        ok = 1;
        int gen = ld_acquire(&flags[kBarrierGen]);
        __threadfence();
        unsigned nb = gridDim.x * gridDim.y * gridDim.z;
        int arrived = atomicAdd(&flags[kBarrier], 1);
        if ((unsigned)arrived == nb - 1) {
            atomicExch(&flags[kBarrier], 0);
            __threadfence();
            st_release(&flags[kBarrierGen], gen + 1);
        } else {
            uint32_t spins = 0;
            while (ld_acquire(&flags[kBarrierGen]) == gen) {
                if (++spins > kSpinLimit || ld_acquire(&flags[kError]) != 0) {
                    set_error(flags, kErrBarrier);
                    ok = 0;
                    break;
                }
                __nanosleep(64);
            }
        }
        if (ld_acquire(&flags[kError]) != 0) ok = 0;
    }
    __syncthreads();
    return ok != 0;   // the same verdict for every thread of the block
}

// Waits (bounded) until *flag becomes nonzero.  Returns false on timeout / error.
__device__ __forceinline__ bool wait_flag(const int* flag, int* flags) {
    uint32_t spins = 0;
    while (ld_acquire(flag) == 0) {
        if (++spins > kSpinLimit) {
            set_error(flags, kErrWait);
            return false;
        }
        if ((spins & 255) == 0 && ld_acquire(&flags[kError]) != 0) return false;
        __nanosleep(32);
    }
    return true;
}

// Appends for every lane with pred set: one atomicAdd per warp instead of one per
// lane (same-address atomics serialise in L2).  Returns the lane's slot, or kNone.
__device__ __forceinline__ uint32_t warp_append(uint32_t* counter, bool pred) {
    const unsigned mask = __activemask();
    const unsigned ballot = __ballot_sync(mask, pred);
    if (!pred) return kNone;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(ballot) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(counter, (uint32_t)__popc(ballot));
    base = __shfl_sync(ballot, base, leader);
    return base + (uint32_t)__popc(ballot & ((1u << lane) - 1u));
}

// Block-wide ordered append: the threads of the block whose pred is set get
// consecutive slots of *counter in thread order, with one atomicAdd per call (a warp-
// per-call scheme is limited by same-address atomic throughput on wide frontiers).
// Returns the thread's slot, or kNone.  Every thread of the block must call it, with
// blockDim.x a multiple of 32.
__device__ __forceinline__ uint32_t block_append(uint32_t* counter, bool pred) {
    __shared__ uint32_t s_cnt[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const unsigned ballot = __ballot_sync(0xffffffffu, pred);
    if (lane == 0) s_cnt[wid] = __popc(ballot);
    __syncthreads();
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
        const uint32_t own = lane < nw ? s_cnt[lane] : 0;
        uint32_t inc = own;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += t;
        }
        uint32_t base = 0;
        if (lane == 31 && inc) base = atomicAdd(counter, inc);
        base = __shfl_sync(0xffffffffu, base, 31);
        if (lane < nw) s_cnt[lane] = base + inc - own;
    }
    __syncthreads();
    const uint32_t pos = pred ? s_cnt[wid] + (uint32_t)__popc(ballot & ((1u << lane) - 1u)) : kNone;
    __syncthreads();
    return pos;
}

// Ordered compaction of the indices i in [0, n) with pred(i), with one atomicAdd
// per block: block b takes a contiguous range, counts it, reserves its slots of
// *counter and calls emit(i, slot) in index order.  Every thread of the block must
// call it, with blockDim.x a multiple of 32.
template <class Pred, class Emit>
__device__ __forceinline__ void block_range_compact(uint32_t n, uint32_t* counter, Pred pred,
                                                    Emit emit) {
    __shared__ uint32_t s_cnt[32];
    __shared__ uint32_t s_run;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int nw = blockDim.x >> 5;
    const uint64_t per = ((uint64_t)n + gridDim.x - 1) / gridDim.x;
    const uint32_t lo = (uint32_t)(blockIdx.x * per < n ? blockIdx.x * per : n);
    const uint32_t hi = (uint32_t)((blockIdx.x + 1) * per < n ? (blockIdx.x + 1) * per : n);
    uint32_t c = 0;
    for (uint32_t i = lo + threadIdx.x; i < hi; i += blockDim.x) c += pred(i) ? 1u : 0u;
    c = __reduce_add_sync(0xffffffffu, c);
    if (lane == 0) s_cnt[wid] = c;
    __syncthreads();
    if (wid == 0) {
        uint32_t t = lane < nw ? s_cnt[lane] : 0;
        t = __reduce_add_sync(0xffffffffu, t);
        if (lane == 0) s_run = t ? atomicAdd(counter, t) : 0;
    }
    __syncthreads();
    for (uint32_t tile = lo; tile < hi; tile += blockDim.x) {
        const uint32_t i = tile + threadIdx.x;
        const bool p = i < hi && pred(i);
        const unsigned ballot = __ballot_sync(0xffffffffu, p);
        if (lane == 0) s_cnt[wid] = __popc(ballot);
        __syncthreads();
        if (wid == 0) {
            const uint32_t own = lane < nw ? s_cnt[lane] : 0;
            uint32_t inc = own;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
                if (lane >= o) inc += t;
            }
            const uint32_t run = s_run;
            if (lane < nw) s_cnt[lane] = run + inc - own;
            if (lane == 31) s_run = run + inc;
        }
        __syncthreads();
        if (p) emit(i, s_cnt[wid] + (uint32_t)__popc(ballot & ((1u << lane) - 1u)));
        __syncthreads();
    }
}

// Raises flags[slot] once per block if any thread's pred is set.  Every thread of
// the block must call it (it contains __syncthreads).
__device__ __forceinline__ void block_flag(int* flags, int slot, bool pred) {
    if (__syncthreads_or(pred) && threadIdx.x == 0) flags[slot] = 1;
}

// `0.0 + x` exactly as IEEE evaluates it: x itself, except that -0.0 becomes +0.0.
__device__ __forceinline__ double plus_zero(double x) { return x == 0.0 ? 0.0 : x; }

// Nanosecond wall clock shared by all SMs (instrumentation).
__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

}  // namespace fl
