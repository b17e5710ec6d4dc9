// exact_fp64.h -- IEEE 754 binary64 square root and division, correctly rounded (round to
// nearest, ties to even), computed with 64-bit integer arithmetic instead of the FP64 pipe.
//
// Why: GB300 retires about two FP64 lanes per SM and clock (1/64 of its FP32 rate), and the
// reference's pair term m / (sqrt(r2) * r2) spends about half of its FP64 instructions in the
// square root and the division.  Both results are defined exactly by IEEE 754 (the correctly
// rounded value of the real result), so any method that returns that value gives the same
// bits as the FP64 pipe's sqrt.rn / div.rn and as the reference's CPU path.  The integer
// pipes and the FP32 seed instructions run beside the FP64 pipe, which keeps only the
// additions and multiplications of the pair term.
//
// Method (schoolbook fixed-point arithmetic with an exact remainder; no library code):
//  * the operands' significands are taken as 53-bit integers;
//  * division: a reciprocal V ~ 2^114 / B from an FP32 seed refined by two Newton steps
//    V += V (2^114 - B V) / 2^114, the quotient Q ~ A 2^s V / 2^114, then the exact
//    remainder R = A 2^s - Q B (it fits in 64 bits, so low-word arithmetic gives it exactly)
//    moves Q to floor(A 2^s / B); the rounding bit follows from 2R against B (an exact tie
//    cannot occur for a quotient of two 53-bit numbers, but ties to even are honoured);
//  * square root: S ~ sqrt(M), M = X' 2^54 with X' the significand (doubled for an odd
//    exponent), from an FP32 seed and two Newton steps S += (M - S^2) / (2S) on 128-bit
//    residuals; the exact remainder M - S^2 (again 64-bit) moves S to floor(sqrt(M)), and
//    the correctly rounded significand is (S + 1) / 2 (sqrt(M) is never a midpoint);
//  * every correction loop is bounded; an operand outside the fast path (zero, subnormal,
//    infinite, NaN, negative, or a result that would not be a normal number) or a loop that
//    did not settle falls back to the hardware's correctly rounded operation, so the result
//    is the IEEE result in every case.
//
// The seeds only need to be within a few parts in 2^20 of the true value: the Newton steps
// and the exact-remainder corrections absorb the rest.  XF_APPROX_RCP / XF_APPROX_RSQRT can
// be defined before including this header (a test perturbs them on the CPU to show that).
#pragma once

#include <stdint.h>
#include <string.h>
#include <math.h>

#if defined(__CUDACC__)
#define XF_HD __host__ __device__ __forceinline__
#else
#define XF_HD static inline
#endif

namespace redgb {
namespace xf {

constexpr uint64_t M52 = (1ull << 52) - 1;
constexpr uint64_t H52 = 1ull << 52;

XF_HD uint64_t dbits(double x)
{
#if defined(__CUDA_ARCH__)
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t u;
    memcpy(&u, &x, 8);
    return u;
#endif
}

XF_HD double bitsd(uint64_t u)
{
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)u);
#else
    double x;
    memcpy(&x, &u, 8);
    return x;
#endif
}

XF_HD uint32_t fbits(float x)
{
#if defined(__CUDA_ARCH__)
    return __float_as_uint(x);
#else
    uint32_t u;
    memcpy(&u, &x, 4);
    return u;
#endif
}

XF_HD uint64_t umulhi64(uint64_t a, uint64_t b)
{
#if defined(__CUDA_ARCH__)
    return __umul64hi(a, b);
#else
    return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

XF_HD int64_t smulhi64(int64_t a, int64_t b)
{
#if defined(__CUDA_ARCH__)
    return __mul64hi(a, b);
#else
    return (int64_t)(((__int128)a * b) >> 64);
#endif
}

#ifndef XF_APPROX_RCP
#if defined(__CUDA_ARCH__)
XF_HD float xf_rcp_seed(float x)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
XF_HD float xf_rsqrt_seed(float x)
{
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
#else
XF_HD float xf_rcp_seed(float x) { return 1.0f / x; }
XF_HD float xf_rsqrt_seed(float x) { return 1.0f / sqrtf(x); }
#endif
#define XF_APPROX_RCP(x) ::redgb::xf::xf_rcp_seed(x)
#define XF_APPROX_RSQRT(x) ::redgb::xf::xf_rsqrt_seed(x)
#endif

// A positive normal float f = sig 2^(e - 23) as the integer round(f 2^k) (k chosen by the
// caller so that the result fits in 63 bits; the shift is never negative here).
XF_HD uint64_t float_to_fixed(float f, int k)
{
    const uint32_t b = fbits(f);
    const int e = (int)((b >> 23) & 0xff) - 127;
    const uint64_t sig = (uint64_t)((b & 0x7fffffu) | 0x800000u);
    const int sh = e - 23 + k;
    return sh >= 0 ? sig << sh : sig >> (-sh);
}

// 128-bit (hi:lo) minus 128-bit, then arithmetic shift right by k (0 < k < 64) to int64;
// the caller guarantees the shifted difference fits.
XF_HD int64_t sub128_shr(uint64_t ahi, uint64_t alo, uint64_t bhi, uint64_t blo, int k)
{
    const uint64_t lo = alo - blo;
    const uint64_t hi = ahi - bhi - (alo < blo ? 1u : 0u);
    return (int64_t)((hi << (64 - k)) | (lo >> k));
}

// a / b for a, b > 0 normal with a normal quotient: returns false (nothing written) when the
// operands or the result leave that range or a correction did not settle.
XF_HD bool div_rn_fast(double a, double b, double* q)
{
    const uint64_t ua = dbits(a), ub = dbits(b);
    const int ea = (int)(ua >> 52), eb = (int)(ub >> 52);  // sign bit 0: the exponent field
    if (ea < 1 || ea > 2046 || eb < 1 || eb > 2046) return false;
    const uint64_t A = (ua & M52) | H52, B = (ub & M52) | H52;
    const int lt = A < B ? 1 : 0;
    int e = ea - eb + 1023 - lt;  // biased exponent of the quotient
    if (e < 1 || e > 2045) return false;
    const int s = 52 + lt;  // A 2^s / B lies in [2^52, 2^53)
    // V ~ 2^114 / B, in (2^61, 2^62]: the seed from the top 24 bits of B
    const float r = XF_APPROX_RCP((float)(uint32_t)(B >> 29));  // ~ 2^-(23..24)
    int64_t V = (int64_t)float_to_fixed(r, 85);                 // 2^114 / (B >> 29 << 29)
    for (int it = 0; it < 2; it++) {
        // E = 2^114 - B V (128-bit), V += V E / 2^114
        const uint64_t phi = umulhi64(B, (uint64_t)V), plo = B * (uint64_t)V;
        const int64_t E = sub128_shr(1ull << 50, 0ull, phi, plo, 50);  // E / 2^50
        V += smulhi64(V, E);                                           // V E / 2^114
    }
    // Q ~ A 2^s V / 2^114 = (A 2^11 V / 2^64) / 2^(61 - s)
    uint64_t Q = umulhi64(A << 11, (uint64_t)V) >> (61 - s);
    int64_t R = (int64_t)((A << s) - Q * B);  // exact: |R| < 2^63
    int k = 0;
    for (; k < 4 && R < 0; k++) {
        Q -= 1;
        R += (int64_t)B;
    }
    for (; k < 8 && R >= (int64_t)B; k++) {
        Q += 1;
        R -= (int64_t)B;
    }
    if (R < 0 || R >= (int64_t)B || Q < H52 || Q >= (H52 << 1)) return false;
    const int64_t twoR = 2 * R;
    if (twoR > (int64_t)B || (twoR == (int64_t)B && (Q & 1))) Q += 1;
    if (Q == (H52 << 1)) {
        Q = H52;
        e += 1;
    }
    *q = bitsd(((uint64_t)e << 52) | (Q & M52));
    return true;
}

// sqrt(x) for x > 0 normal (the result is then always normal)
XF_HD bool sqrt_rn_fast(double x, double* out)
{
    const uint64_t ux = dbits(x);
    const int eb = (int)(ux >> 52);
    if (eb < 1 || eb > 2046) return false;
    const uint64_t X = (ux & M52) | H52;
    const int odd = (eb & 1) ? 0 : 1;  // unbiased exponent eb - 1023 is odd when eb is even
    const uint64_t Xp = X << odd;        // [2^52, 2^54)
    const int ehalf = (eb - 1023 - odd) >> 1;  // exact: eb - 1023 - odd is even
    // M = Xp 2^54 as hi:lo; S = floor(sqrt(M)) in [2^53, 2^54)
    const uint64_t Mhi = Xp >> 10, Mlo = Xp << 54;
    const float xs = (float)(uint32_t)(Xp >> 30);  // [2^22, 2^24): exact
    const float y = XF_APPROX_RSQRT(xs);           // ~ 1 / sqrt(Xp >> 30), in (2^-12, 2^-11]
    const uint64_t yfix = float_to_fixed(y, 43);   // y 2^43, in (2^31, 2^32]
    uint64_t S = float_to_fixed(xs * y, 42);       // sqrt(Xp >> 30) 2^42 ~ sqrt(M)
    // Newton steps S += (M - S^2) / (2 S) with 1 / (2 S) ~ y 2^-43 = yfix 2^-86.  With a seed
    // within 2^-17 of the true value: |M - S0^2| < 2^91, then < 2^77 and < 2^60 after the
    // first and second steps (each step gains the ~17 bits the seed carries).
    {
        const int64_t D = sub128_shr(Mhi, Mlo, umulhi64(S, S), S * S, 40);  // (M - S^2) / 2^40
        S = (uint64_t)((int64_t)S + smulhi64(D, (int64_t)(yfix << 18)));      // D yfix 2^-46
    }
    {
        const int64_t D = sub128_shr(Mhi, Mlo, umulhi64(S, S), S * S, 20);  // (M - S^2) / 2^20
        S = (uint64_t)((int64_t)S + (smulhi64(D, (int64_t)yfix) >> 2));       // D yfix 2^-66
    }
    {
        const int64_t D = (int64_t)(Mlo - S * S);                      // exact: |M - S^2| < 2^63
        S = (uint64_t)((int64_t)S + (smulhi64(D, (int64_t)yfix) >> 22));  // D yfix 2^-86
    }
    int64_t R = (int64_t)(Mlo - S * S);  // exact: |M - S^2| < 2^63
    int k = 0;
    for (; k < 4 && R < 0; k++) {
        R += (int64_t)(2 * S - 1);
        S -= 1;
    }
    for (; k < 8 && R > (int64_t)(2 * S); k++) {
        R -= (int64_t)(2 * S + 1);
        S += 1;
    }
    if (R < 0 || R > (int64_t)(2 * S) || S < (H52 << 1) || S >= (H52 << 2)) return false;
    const uint64_t T = (S + 1) >> 1;  // [2^52, 2^53)
    *out = bitsd(((uint64_t)(ehalf + 1023) << 52) | (T & M52));
    return true;
}

// ---------------------------------------------------------------------------------------
// Serial sums.  Inside one binade [2^(ea-1023), 2^(ea-1022)) the doubles are the multiples of
// the quantum Q = 2^(ea-1075), so while a running sum acc stays in its binade, the correctly
// rounded acc + t is acc + (t rounded to a multiple of Q) -- ties to even, where a tie is a t
// at an odd multiple of Q/2.  The terms of a serial FP64 sum can therefore be rounded to
// quanta independently and added as integers, which is exact and associative, as long as
// every running sum stays strictly inside the binade and no term is a tie; the first term
// that breaks this is added by the FP64 pipe and the binade is taken afresh.

// t / Q rounded to the nearest integer, for the quantum Q = 2^(ea - 1075) of the binade with
// biased exponent ea (1..2046); false for a tie, a subnormal, an infinite or NaN t, or a t of
// 2^5 binades or more above the accumulator's (|r| then stays below 2^58, so 32 of them add
// without overflow).
XF_HD bool quantize(double t, int ea, int64_t* r)
{
    const uint64_t ut = dbits(t);
    const int et = (int)((ut >> 52) & 0x7ff);
    const uint64_t mant = ut & M52;
    if (et == 0) {
        if (mant != 0) return false;  // subnormal
        *r = 0;                        // +-0 adds nothing to a nonzero accumulator
        return true;
    }
    if (et == 2047) return false;
    const uint64_t M = mant | H52;
    const int sh = et - ea;
    uint64_t mag;
    if (sh >= 0) {
        if (sh > 4) return false;
        mag = M << sh;
    } else if (-sh >= 64) {
        mag = 0;  // |t| < 2^-11 Q
    } else {
        const int k = -sh;
        const uint64_t q0 = M >> k;
        const uint64_t rem = M - (q0 << k);
        const uint64_t half = 1ull << (k - 1);
        if (rem == half) return false;  // a tie: the result's parity decides
        mag = q0 + (rem > half ? 1u : 0u);
    }
    *r = (ut >> 63) ? -(int64_t)mag : (int64_t)mag;
    return true;
}

// the accumulator's signed significand in quanta of its own binade (2^52 <= |A| < 2^53)
XF_HD int64_t quanta_of(double acc)
{
    const uint64_t ua = dbits(acc);
    const int64_t A = (int64_t)((ua & M52) | H52);
    return (ua >> 63) ? -A : A;
}

// S quanta of the binade ea (2^52 < |S| < 2^53) as a double
XF_HD double from_quanta(int64_t S, int ea)
{
    const uint64_t sign = S < 0 ? (1ull << 63) : 0ull;
    const uint64_t mag = S < 0 ? (uint64_t)(-S) : (uint64_t)S;
    return bitsd(sign | ((uint64_t)ea << 52) | (mag & M52));
}

// whether S quanta (a running sum of an accumulator with significand A quanta) lies strictly
// inside the binade, on A's side of zero: then the rounded sum is the binade's S Q, and the
// exact sum, within Q/2 of it, lies inside the binade too
XF_HD bool inside_binade(int64_t A, int64_t S)
{
    return A > 0 ? (S > (int64_t)H52 && S < (int64_t)(H52 << 1)) : (S < -(int64_t)H52 && S > -(int64_t)(H52 << 1));
}

}  // namespace xf
}  // namespace redgb

#if defined(__CUDACC__)
namespace redgb {

// sqrt(x) and a / b rounded to nearest even, off the FP64 pipe where the fast path applies;
// the hardware's correctly rounded instructions take every other operand.
__device__ __forceinline__ double rn_sqrt(double x)
{
    double r;
    return xf::sqrt_rn_fast(x, &r) ? r : __dsqrt_rn(x);
}

__device__ __forceinline__ double rn_div(double a, double b)
{
    double r;
    return xf::div_rn_fast(a, b, &r) ? r : __ddiv_rn(a, b);
}

// acc + T[0] + T[1] + ... + T[m-1], rounded to nearest after every addition in that order --
// the bits of the serial FP64 loop -- computed by the 32 lanes of a warp together (m <= 32;
// every lane of the warp calls this with the same acc, T, m and state; lane k reads T[k]).
//
// Fast passes: the terms are rounded to quanta of the accumulator's binade in parallel and
// added by a warp prefix sum (xf::quantize); if the running sum stays in its binade and no
// term is a tie or special, one pass takes all the terms -- a few integer operations, five
// shuffles and a ballot, about 21 cycles per term on GB300 against 71 for each dependent FP64
// addition of the serial loop.  The first term that breaks this is added by lane 0 on the
// FP64 pipe; after a pass that took at least SERIAL_GOOD_PASS terms another pass follows,
// otherwise lane 0 adds the rest of the round in order (one active lane: the FP64 pipe's cost
// of a one-lane addition is small, its latency is what the serial loop pays).
//
// A running sum that keeps leaving its binade (a component hovering about zero, where the
// terms cancel) makes every pass short; after such a round the next `backoff` rounds are
// serial, the backoff going 0, 1, 2, 4, 8 while rounds keep failing that way and back to 0
// after a round whose passes were all long.  SerialSumState holds that per chain; it starts
// as {0, 0}.
struct SerialSumState {
    int skip;     // serial rounds still to do
    int backoff;  // serial rounds after the next poor round
};

constexpr int SERIAL_GOOD_PASS = 8;

// lane 0 adds T[from..m) in order; every lane returns the result
__device__ __forceinline__ double serial_tail(double acc, const double* T, int from, int m)
{
    if ((threadIdx.x & 31) == 0)
        for (int k = from; k < m; k++) acc = __dadd_rn(acc, T[k]);
    return __shfl_sync(0xffffffffu, acc, 0);
}

__device__ __forceinline__ double warp_serial_sum(double acc, const double* T, int m, SerialSumState& st)
{
    if (m <= 0) return acc;
    if (st.skip > 0) {
        st.skip--;
        return serial_tail(acc, T, 0, m);
    }
    const int lane = threadIdx.x & 31;
    const double tk = lane < m ? T[lane] : 0.0;
    int pos = 0;
    while (pos < m) {
        int ea = (int)((xf::dbits(acc) >> 52) & 0x7ff);
        if (ea == 0 || ea == 2047) {  // a zero, subnormal, infinite or NaN accumulator: one term first
            acc = serial_tail(acc, T, pos, pos + 1);
            pos++;
            continue;
        }
        int64_t r = 0;
        bool ok = true;
        const bool mine = lane >= pos && lane < m;
        if (mine) ok = xf::quantize(tk, ea, &r);
        if (!ok) r = 0;
        int64_t P = r;  // inclusive prefix over the lanes
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const long long o = __shfl_up_sync(0xffffffffu, (long long)P, off);
            if (lane >= off) P += o;
        }
        const int64_t A = xf::quanta_of(acc);
        const int64_t S = A + P;
        const unsigned bad = __ballot_sync(0xffffffffu, mine && !(ok && xf::inside_binade(A, S)));
        const int stop = bad ? __ffs(bad) - 1 : m;
        if (stop > pos) acc = xf::from_quanta(__shfl_sync(0xffffffffu, (long long)S, stop - 1), ea);
        if (stop >= m) break;
        if (stop - pos < SERIAL_GOOD_PASS) {  // a poor pass: the rest of the round serially
            st.skip = st.backoff;
            st.backoff = st.backoff ? min(2 * st.backoff, 8) : 1;
            return serial_tail(acc, T, stop, m);
        }
        acc = serial_tail(acc, T, stop, stop + 1);
        pos = stop + 1;
    }
    st.backoff = 0;
    return acc;
}

}  // namespace redgb
#endif
