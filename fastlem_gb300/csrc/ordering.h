// ordering.h -- the Hilbert curve index used to order a model's sites in memory.
#pragma once
#include <stdint.h>

#ifdef __CUDACC__
#define FL_HD __host__ __device__
#else
#define FL_HD
#endif

namespace fl {

// Position of grid cell (x, y) along the Hilbert curve filling a 2^order square
// (the classic quadrant-rotation construction).
FL_HD inline uint64_t hilbert_index(uint32_t order, uint32_t x, uint32_t y) {
    uint64_t d = 0;
    for (uint32_t s = 1u << (order - 1); s > 0; s >>= 1) {
        const uint32_t rx = (x & s) ? 1u : 0u;
        const uint32_t ry = (y & s) ? 1u : 0u;
        d += (uint64_t)s * s * ((3u * rx) ^ ry);
        if (ry == 0) {
            if (rx == 1) {
                x = s - 1 - (x & (s - 1)) + (x & ~(s - 1));
                y = s - 1 - (y & (s - 1)) + (y & ~(s - 1));
            }
            const uint32_t t = x;
            x = y;
            y = t;
        }
    }
    return d;
}

}  // namespace fl
