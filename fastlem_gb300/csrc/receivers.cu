// receivers.cu -- steepest-descent receivers (src/lem/stream_tree.rs:109-137).
//
// For site i (not an outlet) the reference takes, over its adjacency row in order,
// every neighbour j with e_i > e_j, the slope s_j = (e_i - e_j) / len_j in f64, and
// keeps the first j whose slope is strictly larger than the best so far (starting
// from 0.0).  The result must be bit-exact, but GB300 issues f64 at 1/64 of the f32
// rate and a correctly rounded f64 divide costs ~9 f64 operations, which made the
// straightforward scan FP64-bound.  Here every candidate's slope is first estimated
// in f32 from the exact bit patterns:
//   * e_i > e_j is an integer comparison of the bit patterns (both non-negative);
//   * d = e_i - e_j: when both share a binary exponent (the usual case for
//     neighbours) the bit patterns' difference is the exact difference in units of
//     that exponent's ulp, converted to f32 within 2^-23 relative; otherwise it is formed
//     in 64-bit integers, exactly when the exponents differ by <= 11 and truncated
//     (error < 2^-52 relative) otherwise, then cut to 24 bits;
//   * the estimate is d times the slot's 1/len, rounded to f32 once per graph, so it
//     has relative error below 2^-20.
// If the largest estimate exceeds every other by more than a factor (1 - 2^-17)^-1,
// its exact slope is strictly the largest, so it is the reference's receiver.
// Otherwise (near-ties, negative or non-finite values, values outside the f32
// range) the row is rescanned exactly as the reference does.

#include <algorithm>
#include <cfloat>

#include "common.cuh"
#include "kernels.h"

namespace fl {
namespace {

constexpr uint64_t kMant = (1ull << 52) - 1;
constexpr int kRowFast = 12;   // rows up to this length gather their elevations at once

// Float estimate of (a - b) for non-negative finite doubles with bits A > B.
// Returns false when the result falls outside the normal f32 range.
__device__ __forceinline__ bool diff_estimate(uint64_t A, uint64_t B, float& out) {
    int ea = (int)(A >> 52), eb = (int)(B >> 52);
    uint64_t ma = (A & kMant) | (ea ? (1ull << 52) : 0);
    uint64_t mb = (B & kMant) | (eb ? (1ull << 52) : 0);
    ea = ea ? ea : 1;
    eb = eb ? eb : 1;
    int sh = ea - eb;
    uint64_t D;
    int E;
    if (sh <= 11) {
        D = (ma << sh) - mb;
        E = eb;
    } else {
        D = ma - (sh < 64 ? (mb >> sh) : 0);
        E = ea;
    }
    if (D == 0) return false;
    int lz = __clzll((long long)D);
    uint64_t top = D << lz;                      // leading one at bit 63
    int e2 = (63 - lz) + E - 1075;               // d = 1.xxx * 2^e2
    int fe = e2 + 127;
    if (fe <= 0 || fe >= 255) return false;
    uint32_t fb = ((uint32_t)fe << 23) | (uint32_t)((top >> 40) & 0x7fffffu);
    out = __uint_as_float(fb);
    return true;
}

// f32 estimate of a - b for non-negative finite doubles with bits A > B.  Sharing
// the exponent field e in [949, 1149], A - B is the difference in units of 2^(e-1075)
// (below 2^52) and the scaled result is a normal f32 number.  The 52-bit difference is
// converted as two 32-bit halves (a 64-bit integer conversion issues on the f64 pipe):
// the high half is exact, the low half truncated and the fused sum rounded, within
// 2^-23 relative.
__device__ __forceinline__ bool slope_diff(uint64_t A, uint64_t B, float& out) {
    const uint32_t e = (uint32_t)(A >> 52);
    if (e == (uint32_t)(B >> 52) && e - 949u <= 200u) {
        const uint64_t D = A - B;
        const float d = fmaf(__uint2float_rz((uint32_t)(D >> 32)), 4294967296.0f,
                             __uint2float_rz((uint32_t)D));
        out = d * __uint_as_float((e - 948u) << 23);
        return true;
    }
    return diff_estimate(A, B, out);
}

// Site i's receiver and receiver distance.  s0 / s1 bound its row; dmax is the
// largest row length (up to kRowFast) among the warp's sites on the short-row path,
// so the unrolled gathers stop where the warp's rows do.
__device__ __forceinline__ void scan_site(uint32_t i, uint32_t s0, uint32_t s1, uint32_t dmax,
                                          const uint32_t* __restrict__ col,
                                          const double* __restrict__ len,
                                          const float* __restrict__ ilen,
                                          const double* __restrict__ elev,
                                          uint32_t* __restrict__ next, double* __restrict__ rlen,
                                          bool* lake, bool* went_exact) {
    const double ei = elev[i];
    const uint64_t EI = (uint64_t)__double_as_longlong(ei);
    bool exact = (EI >> 63) != 0 || (EI >> 52) == 0x7ff;   // negative or non-finite
    float best = 0.0f, second = 0.0f;
    uint32_t best_slot = kNone;
    bool any_lower = false;
    if (!exact) {
        // one candidate: exact comparison of the bit patterns, then the f32 estimate
        auto consider = [&](uint32_t s, uint64_t EJ) {
            if (exact) return;
            if ((EJ >> 63) || (EJ >> 52) == 0x7ff) { exact = true; return; }
            if (EI <= EJ) return;                          // not lower (bits are monotone)
            any_lower = true;
            float d;
            if (!slope_diff(EI, EJ, d)) {
                exact = true;
                return;
            }
            const float a = d * ilen[s];
            if (!(a > 1e-30f) || !(a < 1e30f)) { exact = true; return; }
            if (a > best) {
                second = best;
                best = a;
                best_slot = s;
            } else if (a > second) {
                second = a;
            }
        };
        const uint32_t deg = s1 - s0;
        if (deg <= (uint32_t)kRowFast) {
            // short rows: all neighbour elevations in flight at once
            uint32_t jj[kRowFast];
            uint64_t ej[kRowFast];
#pragma unroll
            for (int k = 0; k < kRowFast; ++k) {
                if ((uint32_t)k >= dmax) break;
                if ((uint32_t)k < deg) jj[k] = col[s0 + k];
            }
#pragma unroll
            for (int k = 0; k < kRowFast; ++k) {
                if ((uint32_t)k >= dmax) break;
                if ((uint32_t)k < deg) ej[k] = (uint64_t)__double_as_longlong(elev[jj[k]]);
            }
#pragma unroll
            for (int k = 0; k < kRowFast; ++k) {
                if ((uint32_t)k >= dmax) break;
                if ((uint32_t)k < deg) consider(s0 + k, ej[k]);
            }
        } else {
            for (uint32_t s = s0; s < s1; ++s)
                consider(s, (uint64_t)__double_as_longlong(elev[col[s]]));
        }
        if (!exact && any_lower && second > best * (1.0f - 7.62939453125e-06f)) exact = true;
    }
    if (exact) {
        *went_exact = true;
        double steepest = 0.0;
        best_slot = kNone;
        for (uint32_t s = s0; s < s1; ++s) {
            uint32_t j = col[s];
            double ej = elev[j];
            if (ei > ej) {
                double slope = __ddiv_rn(__dsub_rn(ei, ej), len[s]);
                if (slope > steepest) {
                    steepest = slope;
                    best_slot = s;
                }
            }
        }
    }
    if (best_slot == kNone) {
        next[i] = i;
        rlen[i] = 1.0;
        *lake = true;
        return;
    }
    // A duplicate of the receiver later in the row has the same slope and never wins
    // (strictly larger only; in the estimate it is a near-tie), so best_slot is the
    // receiver's first entry, the one has_edge reports.
    next[i] = col[best_slot];
    rlen[i] = len[best_slot];
}


__global__ void k_receivers(uint32_t n, const uint32_t* __restrict__ row,
                            const uint32_t* __restrict__ col, const double* __restrict__ len,
                            const float* __restrict__ ilen, const double* __restrict__ elev,
                            const uint8_t* __restrict__ outlet, uint32_t* __restrict__ next,
                            double* __restrict__ rlen, int* __restrict__ flags,
                            const uint32_t* __restrict__ tid, const uint32_t* __restrict__ titer) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    bool lake = false, went_exact = false, scan = false;
    uint32_t s0 = 0, s1 = 0;
    // a converged packed terrain keeps its routed receivers
    if (i < n && !(tid && titer[tid[i]])) {
        if (outlet[i]) {
            next[i] = i;
            rlen[i] = 1.0;
        } else {
            s0 = row[i];
            s1 = row[i + 1];
            scan = true;
        }
    }
    const uint32_t deg = s1 - s0;
    const uint32_t dmax = __reduce_max_sync(0xffffffffu, deg <= (uint32_t)kRowFast ? deg : 0u);
    if (scan) scan_site(i, s0, s1, dmax, col, len, ilen, elev, next, rlen, &lake, &went_exact);
    block_flag(flags, kHasLake, lake);
    if (__syncthreads_or(went_exact) && threadIdx.x == 0) atomicAdd(&flags[kExact], 1);
}

// 1/len per slot in f32 for the slope estimates, NaN where that is not a normal f32
// number (the row then takes the exact scan).
__global__ void k_inv_len(uint64_t nnz, const double* __restrict__ len, float* __restrict__ ilen) {
    for (uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; s < nnz;
         s += (uint64_t)gridDim.x * blockDim.x) {
        const float f = __double2float_rn(__ddiv_rn(1.0, len[s]));
        ilen[s] = (f >= FLT_MIN && f <= FLT_MAX) ? f : __int_as_float(0x7fc00000);
    }
}

}  // namespace

void launch_receivers(cudaStream_t st, uint32_t n, const uint32_t* row, const uint32_t* col,
                      const double* len, const float* ilen, const double* elev,
                      const uint8_t* outlet, uint32_t* next, double* rlen, int* flags,
                      const uint32_t* tid, const uint32_t* titer) {
    k_receivers<<<(n + kThreads - 1) / kThreads, kThreads, 0, st>>>(
        n, row, col, len, ilen, elev, outlet, next, rlen, flags, tid && titer ? tid : nullptr, titer);
}

void launch_inv_len(cudaStream_t st, uint64_t nnz, const double* len, float* ilen) {
    if (nnz == 0) return;
    const uint64_t blocks = std::min<uint64_t>((nnz + kThreads - 1) / kThreads, 152ull * 64);
    k_inv_len<<<(unsigned)blocks, kThreads, 0, st>>>(nnz, len, ilen);
}

}  // namespace fl
