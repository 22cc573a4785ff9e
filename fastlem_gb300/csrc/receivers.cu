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
//   * d = e_i - e_j is formed in 64-bit integers, exactly when the exponents differ
//     by <= 11 and truncated (error < 2^-52 relative) otherwise, then cut to 24 bits;
//   * the slope estimate d_f / len_f has relative error below 2^-20.
// If the largest estimate exceeds every other by more than a factor (1 - 2^-17)^-1,
// its exact slope is strictly the largest, so it is the reference's receiver.
// Otherwise (near-ties, negative or non-finite values, values outside the f32
// range) the row is rescanned exactly as the reference does.

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

// Float estimate of a positive finite double (truncated mantissa).
__device__ __forceinline__ bool to_float_estimate(uint64_t L, float& out) {
    int e = (int)(L >> 52);
    if ((L >> 63) || e == 0 || e == 0x7ff) return false;
    int fe = e - 1023 + 127;
    if (fe <= 0 || fe >= 255) return false;
    out = __uint_as_float(((uint32_t)fe << 23) | (uint32_t)((L >> 29) & 0x7fffffu));
    return true;
}

__device__ __forceinline__ void scan_site(uint32_t i, const uint32_t* __restrict__ row,
                                          const uint32_t* __restrict__ col,
                                          const double* __restrict__ len,
                                          const double* __restrict__ elev,
                                          const uint8_t* __restrict__ outlet,
                                          uint32_t* __restrict__ next, double* __restrict__ rlen,
                                          bool* lake, bool* went_exact) {
    if (outlet[i]) {
        next[i] = i;
        rlen[i] = 1.0;
        return;
    }
    const uint32_t s0 = row[i], s1 = row[i + 1];
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
            float d, l;
            if (!diff_estimate(EI, EJ, d) ||
                !to_float_estimate((uint64_t)__double_as_longlong(len[s]), l)) {
                exact = true;
                return;
            }
            float a = __fdividef(d, l);
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
            for (int k = 0; k < kRowFast; ++k)
                if ((uint32_t)k < deg) jj[k] = col[s0 + k];
#pragma unroll
            for (int k = 0; k < kRowFast; ++k)
                if ((uint32_t)k < deg) ej[k] = (uint64_t)__double_as_longlong(elev[jj[k]]);
#pragma unroll
            for (int k = 0; k < kRowFast; ++k)
                if ((uint32_t)k < deg) consider(s0 + k, ej[k]);
        } else {
            for (uint32_t s = s0; s < s1; ++s)
                consider(s, (uint64_t)__double_as_longlong(elev[col[s]]));
        }
        if (!exact && any_lower && second > best * (1.0f - 7.62939453125e-06f)) exact = true;
    }
    uint32_t nb = i;
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
    nb = col[best_slot];
    next[i] = nb;
    uint32_t s = s0;
    while (col[s] != nb) ++s;   // first entry of the receiver, as has_edge reports it
    rlen[i] = len[s];
}


__global__ void k_receivers(uint32_t n, const uint32_t* __restrict__ row,
                            const uint32_t* __restrict__ col, const double* __restrict__ len,
                            const double* __restrict__ elev, const uint8_t* __restrict__ outlet,
                            uint32_t* __restrict__ next, double* __restrict__ rlen,
                            int* __restrict__ flags) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    bool lake = false, went_exact = false;
    if (i < n) scan_site(i, row, col, len, elev, outlet, next, rlen, &lake, &went_exact);
    block_flag(flags, kHasLake, lake);
    if (__syncthreads_or(went_exact) && threadIdx.x == 0) atomicAdd(&flags[kExact], 1);
}

}  // namespace

void launch_receivers(cudaStream_t st, uint32_t n, const uint32_t* row, const uint32_t* col,
                      const double* len, const double* elev, const uint8_t* outlet,
                      uint32_t* next, double* rlen, int* flags) {
    k_receivers<<<(n + kThreads - 1) / kThreads, kThreads, 0, st>>>(n, row, col, len, elev, outlet,
                                                                     next, rlen, flags);
}

}  // namespace fl
