// Rows of terms for the check of the warp-parallel exact serial sum (exact_fp64.h:
// xf::quantize and warp_serial_sum), shared by the CPU and GPU checks.  A row is drawn from
// (seed, family, row) by a counter-based generator, so both checks see the same rows:
//   0  gravity-like: one to three large terms, then many terms 2^-8 .. 2^-40 of them
//   1  wide: random signs and exponents over 2^-60 .. 2^60 (the binade changes often)
//   2  ties: small integers times 2^-55 .. 2^-51 around an accumulator near 1 (many terms
//      fall on odd multiples of half a quantum)
//   3  cancellation: pairs t, -t (1 + e) and exact negations (sums through and at zero)
//   4  specials: family 0 with zeros of both signs, subnormals, infinities, NaNs, huge terms
#pragma once

#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define SC_HD __host__ __device__ __forceinline__
#define SC_MEMBER __host__ __device__ __forceinline__
#else
#define SC_HD static inline
#define SC_MEMBER inline
#endif

constexpr int SC_MAX_LEN = 2048;

SC_HD uint64_t sc_mix(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

struct ScRng {
    uint64_t s;
    SC_MEMBER uint64_t next() { return s = sc_mix(s); }
    SC_MEMBER double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
    SC_MEMBER int below(int n) { return (int)(next() % (uint64_t)n); }
};

SC_HD double sc_bits(uint64_t u)
{
    double x;
    memcpy(&x, &u, 8);
    return x;
}

SC_HD double sc_pow2(int e)  // 2^e for -1022 <= e <= 1023
{
    return sc_bits((uint64_t)(e + 1023) << 52);
}

SC_HD double sc_random_mag(ScRng& g, int emin, int emax)
{
    const int e = emin + g.below(emax - emin + 1);
    const uint64_t mant = g.next() & ((1ull << 52) - 1);
    return sc_bits(((uint64_t)(e + 1023) << 52) | mant);
}

// row `row` of family `fam`: its length, its initial accumulator and its terms
SC_HD int sc_row(uint64_t seed, int fam, uint64_t row, double* acc0, double* t)
{
    ScRng g{sc_mix(seed ^ sc_mix(((uint64_t)fam << 48) ^ row))};
    const int n = 1 + g.below(g.below(4) == 0 ? 64 : SC_MAX_LEN);
    *acc0 = g.below(4) == 0 ? (g.below(2) ? -1.0 : 1.0) * sc_random_mag(g, -3, 3) : 0.0;
    const int big = 1 + g.below(3);
    for (int k = 0; k < n; k++) {
        const double sgn = g.below(2) ? -1.0 : 1.0;
        double v;
        switch (fam) {
        case 0:
        case 4:
            v = sgn * (k < big ? sc_random_mag(g, -5, 5) : sc_random_mag(g, -45, -12));
            if (fam == 4 && g.below(16) == 0) {
                switch (g.below(8)) {
                case 0: v = 0.0; break;
                case 1: v = -0.0; break;
                case 2: v = sgn * sc_bits(1 + (g.next() & ((1ull << 52) - 1))); break;  // subnormal
                case 3: v = sgn * sc_bits(0x7ff0000000000000ull); break;                 // infinity
                case 4: v = sc_bits(0x7ff8000000000000ull); break;                       // NaN
                case 5: v = sgn * sc_random_mag(g, 900, 1000); break;
                case 6: v = sgn * sc_random_mag(g, -1000, -900); break;
                default: v = sgn * sc_pow2(-1022); break;
                }
            }
            break;
        case 1:
            v = sgn * sc_random_mag(g, -60, 60);
            break;
        case 2:
            v = sgn * (double)(1 + g.below(1024)) * sc_pow2(-55 + g.below(5));
            if (k == 0) v = 1.0 + (double)g.below(1 << 20) * sc_pow2(-52);
            break;
        default:
            if (k % 2 == 0 || k == 0) {
                v = sgn * sc_random_mag(g, -10, 10);
            } else {
                const double prev = t[k - 1];
                v = g.below(3) == 0 ? -prev : -prev * (1.0 + (double)(1 + g.below(64)) * sc_pow2(-52 + g.below(30)));
            }
            break;
        }
        t[k] = v;
    }
    return n;
}
