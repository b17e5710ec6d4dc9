// Operand generators shared by the CPU and GPU checks of exact_fp64.h: case k of family f
// from a 64-bit counter hash, so that both sides can draw the same inputs.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define XC_HD __host__ __device__ __forceinline__
#else
#define XC_HD static inline
#endif

XC_HD uint64_t xc_mix(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// families: 0 random positive normals over the whole exponent range; 1 exponents within
// +-32 of 1; 2 quotients within a few units of a rounding midpoint; 3 square roots within a
// few units of a midpoint; 4 pair-term-like operands (r2 of a few AU^2 down to 1e-20, masses
// of 1e-12 .. 1)
XC_HD void xc_case(uint64_t seed, uint64_t k, int family, uint64_t* a_bits, uint64_t* b_bits)
{
    const uint64_t M52 = (1ull << 52) - 1, H52 = 1ull << 52;
    const uint64_t u1 = xc_mix(seed ^ (k * 0xD1342543DE82EF95ull)), u2 = xc_mix(u1 + 0x632BE59BD9B4E019ull);
    switch (family) {
    case 0:
        *a_bits = (u1 & M52) | ((1 + (u1 >> 52) % 2046) << 52);
        *b_bits = (u2 & M52) | ((1 + (u2 >> 52) % 2046) << 52);
        break;
    case 1:
        *a_bits = (u1 & M52) | ((uint64_t)(1023 - 32 + (u1 >> 58)) << 52);
        *b_bits = (u2 & M52) | ((uint64_t)(1023 - 32 + (u2 >> 58)) << 52);
        break;
    case 2: {
        // A 2^52 ~ (Q + 1/2 + d) B with d a few units: (2Q + 1) B / 2^53 rounded, plus jitter
        const uint64_t B = (u2 & M52) | H52, Q = (u1 & M52) | H52;
        const uint64_t lo = (2 * Q + 1) * B;
#if defined(__CUDA_ARCH__)
        const uint64_t hi = __umul64hi(2 * Q + 1, B);
#else
        const uint64_t hi = (uint64_t)(((unsigned __int128)(2 * Q + 1) * B) >> 64);
#endif
        uint64_t A = (hi << 11) | (lo >> 53);
        A += (uint64_t)((int64_t)((u1 >> 60) & 7) - 3);
        if (A < H52) A = H52;
        if (A > 2 * H52 - 1) A = 2 * H52 - 1;
        *a_bits = (A & M52) | (1023ull << 52);
        *b_bits = (B & M52) | (1023ull << 52);
        break;
    }
    case 3: {
        // X 2^54 ~ (2T + 1)^2, the square of a midpoint of the result's significand T
        const uint64_t T = (u1 & M52) | H52;
        const uint64_t lo = (2 * T + 1) * (2 * T + 1);
#if defined(__CUDA_ARCH__)
        const uint64_t hi = __umul64hi(2 * T + 1, 2 * T + 1);
#else
        const uint64_t hi = (uint64_t)(((unsigned __int128)(2 * T + 1) * (2 * T + 1)) >> 64);
#endif
        const int odd = (int)(u2 & 1);  // an odd exponent doubles the significand
        uint64_t X = ((hi << 10) | (lo >> 54)) >> odd;
        X += (uint64_t)((int64_t)((u1 >> 60) & 7) - 3);
        if (X < H52) X = H52;
        if (X > 2 * H52 - 1) X = 2 * H52 - 1;
        *a_bits = (X & M52) | ((uint64_t)(1023 + 2 * (int)((u2 >> 1) & 63) - 64 + odd) << 52);
        *b_bits = (u2 & M52) | (1023ull << 52);
        break;
    }
    default: {
        // r2 in [1e-20, 30] AU^2 (exponent -67 .. 5), m in [1e-12, 1] Msun (exponent -40 .. 0)
        *a_bits = (u2 & M52) | ((uint64_t)(1023 - 40 + (int)((u2 >> 52) % 41)) << 52);
        *b_bits = (u1 & M52) | ((uint64_t)(1023 - 67 + (int)((u1 >> 52) % 73)) << 52);
        break;
    }
    }
}
