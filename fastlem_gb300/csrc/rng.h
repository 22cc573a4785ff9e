// rng.h -- rand 0.8.5's StdRng (ChaCha12, rand_chacha 0.3) as used by fastlem, for
// host and device code.
//
//   * StdRng::seed_from_u64(s) (rand_core 0.6): the 32-byte key is eight little-endian
//     PCG32 outputs (multiplier 6364136223846793005, increment 11634580027462260723,
//     state advanced before each output).
//   * StdRng::from_seed([0; 32]): all-zero key (builder.rs:39).
//   * ChaCha block: 12 rounds, 64-bit block counter in words 12-13, stream 0 in
//     words 14-15; next_u64() = word[2m] | word[2m+1] << 32 of the keystream.
//   * gen::<f64>(): (next_u64() >> 11) * 2^-53                     (generator.rs:137)
//   * gen_range(lo..hi): v = bits((next_u64() >> 12) | 0x3ff0...) - 1.0;
//     r = v * (hi - lo) + lo, redrawn while r >= hi                 (builder.rs:43-44)
// The keystream is random-access: sample m of gen::<f64>() depends only on block m/8,
// which is what lets the device draw one block per thread.
#pragma once
#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define FL_HD __host__ __device__ __forceinline__
#else
#define FL_HD inline
#endif

namespace fl {

FL_HD uint32_t rotl32(uint32_t v, int c) { return (v << c) | (v >> (32 - c)); }

FL_HD void chacha12_block(const uint32_t key[8], uint64_t counter, uint32_t out[16]) {
    uint32_t s[16] = {0x61707865u, 0x3320646eu, 0x79622d32u, 0x6b206574u,
                      key[0], key[1], key[2], key[3], key[4], key[5], key[6], key[7],
                      (uint32_t)counter, (uint32_t)(counter >> 32), 0u, 0u};
    uint32_t x[16];
    for (int i = 0; i < 16; ++i) x[i] = s[i];
#define FL_QR(a, b, c, d)                          \
    x[a] += x[b]; x[d] ^= x[a]; x[d] = rotl32(x[d], 16); \
    x[c] += x[d]; x[b] ^= x[c]; x[b] = rotl32(x[b], 12); \
    x[a] += x[b]; x[d] ^= x[a]; x[d] = rotl32(x[d], 8);  \
    x[c] += x[d]; x[b] ^= x[c]; x[b] = rotl32(x[b], 7);
    for (int r = 0; r < 12; r += 2) {
        FL_QR(0, 4, 8, 12) FL_QR(1, 5, 9, 13) FL_QR(2, 6, 10, 14) FL_QR(3, 7, 11, 15)
        FL_QR(0, 5, 10, 15) FL_QR(1, 6, 11, 12) FL_QR(2, 7, 8, 13) FL_QR(3, 4, 9, 14)
    }
#undef FL_QR
    for (int i = 0; i < 16; ++i) out[i] = x[i] + s[i];
}

FL_HD void key_from_u64(uint64_t state, uint32_t key[8]) {
    const uint64_t MUL = 6364136223846793005ull;
    const uint64_t INC = 11634580027462260723ull;
    for (int w = 0; w < 8; ++w) {
        state = state * MUL + INC;
        uint32_t xs = (uint32_t)(((state >> 18) ^ state) >> 27);
        uint32_t rot = (uint32_t)(state >> 59);
        key[w] = (xs >> rot) | (xs << ((32 - rot) & 31));
    }
}

FL_HD double u64_to_unit_f64(uint64_t v) { return (double)(v >> 11) * (1.0 / 9007199254740992.0); }

struct StdRng {
    uint32_t key[8];
    uint32_t buf[16];
    uint64_t block;   // next block to generate
    int pos;          // next word in buf (16 = empty)

    static StdRng seed_from_u64(uint64_t s) {
        StdRng r;
        key_from_u64(s, r.key);
        r.block = 0;
        r.pos = 16;
        return r;
    }
    static StdRng zero_key() {
        StdRng r;
        for (int i = 0; i < 8; ++i) r.key[i] = 0;
        r.block = 0;
        r.pos = 16;
        return r;
    }
    uint32_t next_u32() {
        if (pos >= 16) {
            chacha12_block(key, block++, buf);
            pos = 0;
        }
        return buf[pos++];
    }
    // Consecutive u64 reads start on even words here (no u32 draws are mixed in).
    uint64_t next_u64() {
        uint64_t lo = next_u32();
        uint64_t hi = next_u32();
        return lo | (hi << 32);
    }
    double gen_f64() { return u64_to_unit_f64(next_u64()); }
    double gen_range(double lo, double hi) {
        double scale = hi - lo;
        while (true) {
            uint64_t bits = (next_u64() >> 12) | 0x3ff0000000000000ull;
            double v12;
            memcpy(&v12, &bits, 8);
            double v01 = v12 - 1.0;
            double r = v01 * scale + lo;
            if (r < hi) return r;
        }
    }
};

}  // namespace fl
