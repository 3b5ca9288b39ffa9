// Operand pairs for the integer-pipe binary64 arithmetic checks, shared by the
// host check (soft_fp64_host.cpp) and the device check (soft_fp64_device.cu).
// Every pair is a pure function of (seed, index), so both sides draw the same
// cases. Distributions:
//   0 nearby exponents (difference 0..65), full significands, random signs
//   1 short significands (only the top 0..52 bits set): exact ties when rounding
//   2 raw 64-bit patterns: zeros, subnormals, infinities and NaNs included
//   3 cancellation: b is -a moved by up to 1024 units in the last place
//   4 exponents over the whole normal range (overflow and underflow edges)
//   5 exponent pairs whose sum lies at the ends of the normal range (products)
//   6 exponents at most 9 apart (the nearby-exponent addition's own path), full or
//     short significands, random signs
#pragma once
#include <cstdint>

#if defined(__CUDACC__)
#define SOFT_CASES_FN __host__ __device__ inline
#else
#define SOFT_CASES_FN inline
#endif

namespace soft_cases {

SOFT_CASES_FN uint64_t mix(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

SOFT_CASES_FN uint64_t make(uint64_t r0, uint64_t r1, int exponent, bool short_significand) {
    uint64_t frac = r0 & 0x000FFFFFFFFFFFFFull;
    if (short_significand) {
        const int t = (int)(r1 % 53);
        frac &= ~((1ull << (52 - t)) - 1) & 0x000FFFFFFFFFFFFFull;
    }
    return ((r1 >> 63) << 63) | ((uint64_t)exponent << 52) | frac;
}

SOFT_CASES_FN int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// The bit patterns of operand pair `i` of distribution `dist`.
SOFT_CASES_FN void pair(int dist, uint64_t seed, uint64_t i, uint64_t *a, uint64_t *b) {
    const uint64_t r0 = mix(seed ^ (4 * i)), r1 = mix(seed ^ (4 * i + 1)), r2 = mix(seed ^ (4 * i + 2)),
                   r3 = mix(seed ^ (4 * i + 3));
    switch (dist) {
    case 0: {
        const int ea = 900 + (int)(r2 % 250), d = (int)((r2 >> 20) % 66);
        *a = make(r0, r1, ea, false);
        *b = make(r3, r2 ^ r1, ea - d, false);
        break;
    }
    case 1: {
        const int ea = 900 + (int)(r2 % 250), d = (int)((r2 >> 20) % 60);
        *a = make(r0, r1, ea, true);
        *b = make(r3, r2 ^ (r1 << 1), ea - d, true);
        break;
    }
    case 2:
        *a = r0;
        *b = r1;
        break;
    case 3:
        *a = make(r0, r1, 1 + (int)(r2 % 2045), false);
        *b = (*a ^ 0x8000000000000000ull) + (uint64_t)((int64_t)(r3 % 2049) - 1024);
        break;
    case 4:
        *a = make(r0, r1, 1 + (int)(r2 % 2046), false);
        *b = make(r3, r2 ^ r1, 1 + (int)((r2 >> 16) % 2046), false);
        break;
    case 6: {
        const int ea = 10 + (int)(r2 % 2028), d = (int)((r2 >> 20) % 19) - 9;  // both exponents in [1, 2046]
        *a = make(r0, r1, ea, (r3 & 1) != 0);
        *b = make(r3, r2 ^ r1, ea - d, (r3 & 2) != 0);
        break;
    }
    default: {
        const int ea = 1 + (int)(r2 % 2046);
        const int end = ((r2 >> 30) & 1) ? 1023 + 1 : 1023 + 0x7FE;
        const int eb = clampi(end + (int)((r2 >> 32) % 5) - 2 - ea, 1, 2046);
        *a = make(r0, r1, ea, (r3 & 1) != 0);
        *b = make(r3, r2 ^ r1, eb, (r3 & 2) != 0);
        break;
    }
    }
}

} // namespace soft_cases
