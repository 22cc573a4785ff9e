// fold.cuh -- exact parallel evaluation of a chain of rounded f64 additions.
//
// The skeleton walks evaluate, along each river chain, x_k = RN(...RN(RN(x + y_k,0) +
// y_k,1)...) -- one rounded addition per operand, in order, exactly as the reference's
// sequential loops do.  Done naively that is one dependent f64 add (64 cycles on GB300)
// per operand on the critical path.
//
// For a positive normal x in the binade [2^e, 2^(e+1)), x = M * u with M in
// [2^52, 2^53) and u = 2^(e-52).  For an operand y >= 0 write y / u = I + F
// (I integer, 0 <= F < 1).  As long as the sum stays in the binade, round-to-nearest-
// even gives
//        RN(x + y) = (M + I + r) * u,   r = [F > 1/2]   (F = 1/2 ties to even M + I)
// so, between ties and binade crossings, the running value is M plus an integer sum:
// a warp prefix scan.  Each lane computes its operands' (I, r) against the current
// binade, the warp scans the increments, and every lane checks, with the exact running
// mantissa in hand, that none of its steps ties or leaves the binade (M + I + 1 <
// 2^53).  Lanes before the first failing one are final; the failing lane is evaluated
// with real f64 additions (or a caller-supplied rule) and the scan resumes after it.
// Binade crossings happen O(log(x_end / x_start)) times along a chain and exact ties
// are rare, so a 32-site round costs a few scans instead of 32+ dependent additions.
#pragma once
#include <stdint.h>

namespace fl {

constexpr int kFoldOps = 4;   // operands per lane

struct FoldStep {
    uint64_t I;
    uint32_t r;
    bool ok;   // a plain step (non-negative finite, no tie, not absurdly large)
};

// (I, r) of adding y to a value of biased exponent E (ulp 2^(E-1075)).
__device__ __forceinline__ FoldStep fold_step(int E, double y) {
    FoldStep st{0, 0, true};
    const uint64_t Y = (uint64_t)__double_as_longlong(y);
    if (Y >> 63) { st.ok = false; return st; }                 // negative, -0.0
    int ey = (int)(Y >> 52);
    if (ey == 0x7ff) { st.ok = false; return st; }             // inf / nan
    uint64_t my = Y & ((1ull << 52) - 1);
    if (ey) my |= 1ull << 52; else ey = 1;
    if (my == 0) return st;                                     // +0.0
    const int d = E - ey;                                       // y / u = my * 2^-d
    if (d <= 0) {
        if (d < -10) { st.ok = false; return st; }             // y far above x
        st.I = my << (-d);
        return st;
    }
    if (d >= 64) return st;                                     // y < u / 2^11
    st.I = my >> d;
    const uint64_t rem = my & ((1ull << d) - 1);
    const uint64_t half = 1ull << (d - 1);
    if (rem == half) { st.ok = false; return st; }             // tie: parity-dependent
    st.r = rem > half ? 1u : 0u;
    return st;
}

__device__ __forceinline__ uint64_t shfl_up_u64(uint64_t v, int delta) {
    uint32_t lo = __shfl_up_sync(0xffffffffu, (uint32_t)v, delta);
    uint32_t hi = __shfl_up_sync(0xffffffffu, (uint32_t)(v >> 32), delta);
    return ((uint64_t)hi << 32) | lo;
}

__device__ __forceinline__ uint64_t shfl_u64(uint64_t v, int src) {
    uint32_t lo = __shfl_sync(0xffffffffu, (uint32_t)v, src);
    uint32_t hi = __shfl_sync(0xffffffffu, (uint32_t)(v >> 32), src);
    return ((uint64_t)hi << 32) | lo;
}

// Warp-wide exact fold.  Lane k (< cnt) owns operands y[0..nop) to be added in order to
// the running value after lane k-1; `special` lanes are evaluated by seq(k, x) (a
// warp-uniform callback returning the value after lane k).  Lanes with plain operands
// that cannot use the integer path are evaluated with sequential f64 additions.
// Returns the running value after lane cnt-1; `mine` receives the value after this
// lane.  Must be called by all 32 lanes with the same x and cnt.
template <class Seq>
__device__ __forceinline__ double warp_fold(double x, const double (&y)[kFoldOps], int nop,
                                            bool special, int cnt, double& mine, Seq seq) {
    const int lane = threadIdx.x & 31;
    int done = 0;
    while (done < cnt) {
        const uint64_t X = (uint64_t)__double_as_longlong(x);
        const int E = (int)(X >> 52);
        const bool x_plain = (X >> 63) == 0 && E >= 1 && E < 0x7ff;
        bool ok = false;
        uint64_t delta = 0;
        FoldStep st[kFoldOps];
        const bool active = lane >= done && lane < cnt;
        if (x_plain && active && !special) {
            ok = true;
#pragma unroll
            for (int j = 0; j < kFoldOps; ++j) {
                if (j < nop) {
                    st[j] = fold_step(E, y[j]);
                    ok = ok && st[j].ok && st[j].I < (1ull << 53);
                    delta += st[j].I + st[j].r;
                } else {
                    st[j] = FoldStep{0, 0, true};
                }
            }
            if (!ok) delta = 0;
        }
        // inclusive scan of delta over the warp (inactive lanes contribute 0)
        uint64_t incl = delta;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            uint64_t v = shfl_up_u64(incl, off);
            if (lane >= off) incl += v;
        }
        const uint64_t M = x_plain ? ((X & ((1ull << 52) - 1)) | (1ull << 52)) : 0;
        if (ok) {
            // every step must stay inside the binade with the exact running mantissa
            uint64_t run = M + (incl - delta);
#pragma unroll
            for (int j = 0; j < kFoldOps; ++j) {
                if (j < nop) {
                    ok = ok && (run + st[j].I + 1 < (1ull << 53));
                    run += st[j].I + st[j].r;
                }
            }
        }
        const unsigned bad = __ballot_sync(0xffffffffu, active && !ok);
        const int first_bad = bad ? __ffs(bad) - 1 : cnt;
        // lanes [done, first_bad) are final
        if (lane >= done && lane < first_bad)
            mine = __longlong_as_double((long long)(((uint64_t)E << 52) | (M + incl - (1ull << 52))));
        if (first_bad > done) {
            const uint64_t end = shfl_u64(incl, first_bad - 1);
            x = __longlong_as_double((long long)(((uint64_t)E << 52) | (M + end - (1ull << 52))));
        }
        if (first_bad >= cnt) break;
        // the failing lane, sequentially (uniform across the warp)
        const int s = first_bad;
        const bool s_special = __shfl_sync(0xffffffffu, special, s);
        if (s_special) {
            x = seq(s, x);
        } else {
            const int sn = __shfl_sync(0xffffffffu, nop, s);
#pragma unroll
            for (int j = 0; j < kFoldOps; ++j) {
                const double ys = __shfl_sync(0xffffffffu, y[j], s);
                if (j < sn) x = __dadd_rn(x, ys);
            }
        }
        if (lane == s) mine = x;
        done = s + 1;
    }
    return x;
}

}  // namespace fl
