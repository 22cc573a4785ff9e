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
//        RN(x + y) = (M + I + r) * u,   r = [F > 1/2],  or for a tie (F = 1/2)
//                                       r = (M + I) mod 2   (the result is even)
// so, inside a binade, the running value is M plus an integer sum: a warp prefix scan
// (each lane contributing the steps of its few consecutive slots).
// Ties make r depend on the parity of the running mantissa, but parity evolves by a
// one-bit function per operand -- "xor a constant" for a non-tie, "becomes 0" after a
// tie -- and such functions compose, so every lane's entry parity comes from two
// ballots and a popcount.  A lane's increment is then D + [tie] * (p xor h) for a
// constant D and bit h, i.e. a fixed scan plus a popcount of correction bits.
//
// Per binade the lanes compute their (I, r, tie) and scan D once.  Each lane then
// checks, with the exact running mantissa, that its steps stay inside the binade:
// partial sums only grow, so M_after + 1 < 2^53 covers every step's M + I + 1 < 2^53.
// Lanes before the first failing one are final; the failing lane
// (a binade crossing, an operand that is negative / non-finite / far above x, or a
// caller-evaluated lane) is evaluated with real f64 additions or by the caller, and
// the lanes after it are re-based on its result -- without a new scan when the
// result stayed in the binade.  Binade crossings happen O(log(x_end / x_start)) times
// along a chain, so a round normally costs one scan; each lane keeps its running
// increment at the end of each of its slots for the per-slot values.
#pragma once
#include <stdint.h>

namespace fl {

struct FoldStep {
    uint64_t I;
    uint32_t r;   // rounding increment when not a tie
    bool tie;     // F = 1/2: the increment is decided by the running parity
    bool ok;      // a plain step (non-negative finite, not absurdly large)
};

// (I, r) of adding y to a value of biased exponent E (ulp 2^(E-1075)).  The bits of
// y / u below the integer part, shifted out of I and left-aligned, decide r: above
// 1000...0 rounds up, exactly 1000...0 is a tie.
__device__ __forceinline__ FoldStep fold_step(int E, double y) {
    FoldStep st{0, 0, false, true};
    const uint64_t Y = (uint64_t)__double_as_longlong(y);
    int ey = (int)(Y >> 52);                                    // sign bit included
    if (ey >= 0x7ff) { st.ok = false; return st; }             // negative, -0.0, inf, nan
    uint64_t my = Y & ((1ull << 52) - 1);
    if (ey) my |= 1ull << 52; else ey = 1;
    const int d = E - ey;                                       // y / u = my * 2^-d
    if (d <= 0) {
        st.ok = d >= -10;                                       // y not far above x
        st.I = my << (-d);
        return st;
    }
    if (d >= 64) return st;                                     // y < u / 2^11
    st.I = my >> d;
    const uint64_t out = my << (64 - d);
    st.tie = out == (1ull << 63);
    st.r = out > (1ull << 63) ? 1u : 0u;
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

__device__ __forceinline__ double make_double(int E, uint64_t M) {
    return __longlong_as_double((long long)(((uint64_t)E << 52) | (M - (1ull << 52))));
}

// Warp-wide exact fold over one round of slots.  Lane l (< cnt) owns the round's
// slots l*S .. l*S + nsl - 1 (in walk order); slot s has 1 + ((nopm >> 2s) & 3) <= kOps
// operands, added in order to the running value; bit s of specm marks a slot that the
// caller evaluates itself.  Accessors:
//   own(s, j)      this lane's operand j of its slot s;
//   any(l, s, j)   lane l's operand (called by all lanes with the same l);
//   seq(l, s, x)   value after lane l's special slot s given the value x before it
//                  (called by all lanes with the same arguments);
//   out(s, v)      receives the value after this lane's slot s (called by the owning
//                  lane only).
// A lane whose slots cannot all take the integer path (a special slot, an operand that
// is negative / non-finite / far above the running value, a binade crossing) is
// evaluated slot by slot with f64 additions and seq.  Returns the value after the
// round.  Must be called by all 32 lanes with the same x and cnt.
template <int S, int kOps, class Own, class Any, class Seq, class Out>
__device__ __forceinline__ double warp_fold_slots(double x, int cnt, int nsl, uint32_t nopm,
                                                  uint32_t specm, Own own, Any any, Seq seq,
                                                  Out out) {
    constexpr unsigned kAll = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    int done = 0;
    while (done < cnt) {
        // ---- once per binade: every remaining lane's steps against x's exponent
        const uint64_t X = (uint64_t)__double_as_longlong(x);
        const int E = (int)(X >> 52);
        const bool x_plain = (X >> 63) == 0 && E >= 1 && E < 0x7ff;
        const bool active = lane >= done && lane < cnt;
        bool step_ok = false;
        uint64_t D = 0;                   // increment without the first tie's bit
        uint64_t DS[S];                   // ... up to the end of each slot
        int tslot = S;                    // slot of the first tie
        uint32_t g = 0, h = 0;            // has a tie; first tie's bit = p xor h
        uint32_t fa = 1, fb = 0;          // exit parity = fa ? p ^ fb : fb
#pragma unroll
        for (int s = 0; s < S; ++s) DS[s] = 0;
        if (x_plain && active && specm == 0) {
            step_ok = true;
            uint32_t c = 0;               // parity change since the last tie (or entry)
#pragma unroll
            for (int s = 0; s < S; ++s) {
                if (s < nsl) {
                    const int nop = kOps == 1 ? 1 : 1 + (int)((nopm >> (2 * s)) & 3u);
#pragma unroll 1
                    for (int j = 0; j < nop; ++j) {
                        const FoldStep st = fold_step(E, own(s, j));
                        step_ok = step_ok && st.ok && st.I < (1ull << 53);
                        D += st.I;
                        if (st.tie) {
                            const uint32_t ib = (uint32_t)st.I & 1u;
                            if (!g) {
                                g = 1;
                                h = c ^ ib;
                                tslot = s;
                            } else {
                                D += c ^ ib;      // parity after a tie is 0
                            }
                            c = 0;
                            fa = 0;
                        } else {
                            D += st.r;
                            c ^= (uint32_t)((st.I + st.r) & 1u);
                        }
                    }
                }
                DS[s] = D;
            }
            fb = c;
            if (!step_ok) D = 0;
        }
        // fixed part of the increments, scanned once per binade
        uint64_t inclD = D;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const uint64_t v = shfl_up_u64(inclD, off);
            if (lane >= off) inclD += v;
        }
        const unsigned C = __ballot_sync(kAll, step_ok && fa == 0);
        const unsigned F = __ballot_sync(kAll, step_ok && fb != 0);
        // ---- segments: re-based after each sequentially evaluated lane
        int seg = done;
        uint64_t Mseg = x_plain ? ((X & ((1ull << 52) - 1)) | (1ull << 52)) : 0;
        uint64_t Dbase = 0;               // inclD of the lane before seg
        bool rescan = false;
        while (!rescan) {
            const unsigned segm = ~((1u << seg) - 1u);   // lanes >= seg
            // entry parity: the last constant lane in [seg, lane), then xors
            const unsigned cm = C & segm & lt;
            const int jc = cm ? 31 - __clz(cm) : -1;
            const unsigned from = jc >= 0 ? ~((1u << jc) - 1u) : segm;
            uint32_t p = (uint32_t)__popc(F & from & lt) & 1u;
            if (jc < 0) p ^= (uint32_t)(Mseg & 1u);
            const uint32_t corr = g & (p ^ h);
            const unsigned CORR = C ? __ballot_sync(kAll, step_ok && lane >= seg && corr) : 0u;
            const uint64_t before = Mseg + (inclD - D - Dbase) + (uint64_t)__popc(CORR & segm & lt);
            const uint64_t after = before + D + corr;
            // The lane's partial sums only grow, so every step stays inside the binade
            // (M + I + 1 < 2^53 before its rounding) when after + 1 < 2^53.
            const bool ok = step_ok && lane >= seg && lane < cnt && after + 1 < (1ull << 53);
            const unsigned bad = __ballot_sync(kAll, lane >= seg && lane < cnt && !ok);
            const int first_bad = bad ? __ffs(bad) - 1 : cnt;
            if (lane >= seg && lane < first_bad) {
#pragma unroll
                for (int s = 0; s < S; ++s)
                    if (s < nsl) out(s, make_double(E, before + DS[s] + (s >= tslot ? corr : 0u)));
            }
            if (first_bad > seg) x = make_double(E, shfl_u64(after, first_bad - 1));
            if (first_bad >= cnt) return x;
            // the failing lane, slot by slot (uniform across the warp)
            const int sl = first_bad;
            const int n_s = __shfl_sync(kAll, nsl, sl);
            const uint32_t nopm_s = __shfl_sync(kAll, nopm, sl);
            const uint32_t specm_s = __shfl_sync(kAll, specm, sl);
#pragma unroll
            for (int s = 0; s < S; ++s) {
                if (s < n_s) {
                    if ((specm_s >> s) & 1u) {
                        x = seq(sl, s, x);
                    } else {
                        const int nop = kOps == 1 ? 1 : 1 + (int)((nopm_s >> (2 * s)) & 3u);
#pragma unroll 1
                        for (int j = 0; j < nop; ++j) x = __dadd_rn(x, any(sl, s, j));
                    }
                    if (lane == sl) out(s, x);
                }
            }
            done = sl + 1;
            if (done >= cnt) return x;
            // still in the binade: later lanes keep their steps, re-based on x
            const uint64_t Xn = (uint64_t)__double_as_longlong(x);
            if ((Xn >> 63) == 0 && (int)(Xn >> 52) == E && E >= 1 && E < 0x7ff) {
                seg = done;
                Mseg = (Xn & ((1ull << 52) - 1)) | (1ull << 52);
                Dbase = shfl_u64(inclD, sl);
            } else {
                rescan = true;
            }
        }
    }
    return x;
}

}  // namespace fl
