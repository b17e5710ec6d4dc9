// gravity_mixed.cu -- mixed-precision direct-summation gravity for GB300.
//
// Same interaction model and event tests as the FP64 kernel (pp_disk.cu:217-296), but
// the arithmetic is placed on the pipes GB300 has: its FP64 rate is about 1/64 of its
// FP32 rate, so every FP64 operation per pair costs as much as ~64 FP32 operations.
//
//  * Heavy sources (the leading SI bodies: star, giant and rocky planets -- `heavy_end`
//    per tile) and near pairs (m_j / r^2 above `near_ratio` times the sink's pull from
//    the first heavy source) contribute double-float terms (below): FP64-class accuracy
//    computed on the FP32 pipes, added to the same compensated accumulators.  Their
//    displacement comes from the FP64 positions where the split positions would not
//    resolve it (heavy sources always; others closer than |x| / 256: close_r2).
//  * Every other pair uses the FP64 positions split into FP32 (hi, lo) pairs once per
//    force evaluation (split_positions, O(N) integer work).  The displacement is
//    (x_j^hi - x_i^hi) + (x_j^lo - x_i^lo): the hi difference is exact for neighbours
//    (Sterbenz), so the displacement carries the FP64 positions' information down to
//    FP32 resolution of the displacement itself.  1/r^3 comes from the FP32 rsqrt with a
//    first-order correction taken on r^-3 (light_w), and each warp-slice's 32 terms are
//    summed in FP32 and folded into compensated (two-sum) FP32 accumulators per component.
//  * Event tests (collision radius, Hill sphere) are re-evaluated in FP64 for every pair
//    whose FP32 distance is within a 1e-3 relative margin of a threshold, so the event
//    list is decided in FP64 exactly as in the FP64 kernel.
//
// Work split: a CTA holds 32 sinks x 4 (lane x register) and 8 warps; warp w walks the
// w-th slice of each source tile, so all 256 threads work however few sinks a tile has.
// Sources are staged in shared memory as FP32 (hi, lo) quads; the per-warp compensated
// partial sums are added in FP64 at the end.
#include <algorithm>
#include <atomic>
#include <string>

#include "../../include/redgb.h"
#include "common.cuh"
#include "dfloat.cuh"
#include "kernels.h"
#include "tma.cuh"

namespace redgb {

int set_error(int code, const std::string& msg);

struct SplitPos {
    float4 xy;  // x_hi, x_lo, y_hi, y_lo
    float4 zm;  // z_hi, z_lo, m_hi, m_lo
};

// inactive bodies (id < 0, pp_disk.cu:242) get mass 0 here, so the pair loop needs no
// per-pair activity test: their terms vanish.  Coordinates beyond 1e15 AU are clamped
// (split_coord, dfloat.cuh).
static_assert(sizeof(SplitPos) == 4 * sizeof(float2), "SplitPos: float2 #0 x, #1 y, #2 z, #3 m");

// |r_i - r_base| in FP32 from the split positions' leading parts (event screens)
__device__ __forceinline__ float star_dist_f(const SplitPos& pi, const SplitPos& p0)
{
    const float dx = pi.xy.x - p0.xy.x, dy = pi.xy.z - p0.xy.z, dz = pi.zm.x - p0.zm.x;
    return sqrtf(dx * dx + dy * dy + dz * dz);
}

// rf (optional): the radii rounded to FP32, for the event screens.  smax (optional, reset to
// zero before the launch): per system k, FP32 bits of the largest screened value over its
// light bodies that can be the source of an event test (screen_slot[i] = k, id >= 0) --
// smax[4k] the radius, smax[4k + 1] the mass and smax[4k + 2] the star distance (with hill),
// each the same FP32 value the screens read (base_of: each body's body 0, or nullptr for
// index 0).  Heavy bodies (screen_slot -1: stars, giant and rocky planets) are screened
// without a cutoff.
__global__ void split_positions_kernel(const double* __restrict__ x, const double* __restrict__ y,
                                       const double* __restrict__ z, const double* __restrict__ m,
                                       const int* __restrict__ id, const int* __restrict__ base_of,
                                       const int* __restrict__ screen_slot, const double* __restrict__ radius,
                                       int n, SplitPos* __restrict__ out, float* __restrict__ rf,
                                       unsigned int* smax, bool hill, float2* __restrict__ mass_f2)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    float rmax = 0.0f, mmax = 0.0f, dmax = 0.0f;
    int slot = -1;
    if (i < n) {
        SplitPos sp;
        split_coord(x[i], sp.xy.x, sp.xy.y);
        split_coord(y[i], sp.xy.z, sp.xy.w);
        split_coord(z[i], sp.zm.x, sp.zm.y);
        sp.zm.z = sp.zm.w = 0.0f;
        if (id[i] >= 0) split_bits(m[i], sp.zm.z, sp.zm.w);
        out[i] = sp;
        if (mass_f2) mass_f2[i] = make_float2(sp.zm.z, sp.zm.w);
        if (rf) {
            float rh, rl;
            split_bits(radius[i], rh, rl);
            rf[i] = rh;
            if (smax && id[i] >= 0) slot = screen_slot[i];
            if (slot >= 0) {
                rmax = rh;
                const int b = base_of ? base_of[i] : 0;
                if (hill) {
                    SplitPos p0;
                    split_coord(x[b], p0.xy.x, p0.xy.y);
                    split_coord(y[b], p0.xy.z, p0.xy.w);
                    split_coord(z[b], p0.zm.x, p0.zm.y);
                    mmax = sp.zm.z;
                    dmax = star_dist_f(sp, p0);
                }
            }
        }
    }
    if (!smax) return;
    // lanes of one system: one atomic per value and warp (non-negative floats order as their
    // bit patterns); a warp that spans systems or holds heavy bodies: one per lane
    const int slot0 = __shfl_sync(0xffffffffu, slot, 0);
    if (__all_sync(0xffffffffu, slot == slot0)) {
        for (int off = 16; off > 0; off >>= 1) {
            rmax = fmaxf(rmax, __shfl_xor_sync(0xffffffffu, rmax, off));
            mmax = fmaxf(mmax, __shfl_xor_sync(0xffffffffu, mmax, off));
            dmax = fmaxf(dmax, __shfl_xor_sync(0xffffffffu, dmax, off));
        }
        if ((threadIdx.x & 31) != 0) slot = -1;
    }
    if (slot >= 0) {
        unsigned int* s = smax + SCREEN_MAX_WORDS * slot;
        if (rmax > 0.0f) atomicMax(&s[0], __float_as_uint(rmax));
        if (mmax > 0.0f) atomicMax(&s[1], __float_as_uint(mmax));
        if (dmax > 0.0f) atomicMax(&s[2], __float_as_uint(dmax));
    }
}

__device__ __forceinline__ float rsqrt_approx(float x)
{
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// m r^-3 of a light pair from the FP32 rsqrt seed y0 = r^-1 (1 + d): with s = y0^2,
// y0^3 (2.5 - 1.5 r^2 s) = r^-3 (1 - 7.5 d^2 + O(d^3)) -- the first-order correction taken on
// y^3 itself, one multiplication fewer than a Newton step on y followed by y^3; |d| < 2^-22,
// so the truncation (~2e-13) is far below the FP32 rounding of the term.
__device__ __forceinline__ float light_w(float mj, float r2)
{
    const float y0 = rsqrt_approx(r2);
    const float s = y0 * y0;
    const float t = fmaf(-1.5f * r2, s, 2.5f);
    return (mj * (y0 * s)) * t;
}


__device__ __forceinline__ Acc2 two_sum_merge(Acc2 a, Acc2 b)
{
    two_sum_add(a, b.s);
    a.c += b.c;
    return a;
}


struct MixedArgs {
    GravArgs g;
    const SplitPos* sp;
    const int* heavy_end;  // per tile: sources [src_begin, heavy_end) are heavy
    float near_ratio;
    int chunk;             // sources per grid.y chunk (multiple of MX_T)
    double* partial;       // n_chunks x 3 x n_part doubles, or nullptr when grid.y == 1
    int n_part;            // row length of `partial`
    unsigned int* err;     // set to 1 when a tile copy did not arrive within the wait limit
    int hold;              // test hook: issue no tile copies (the waits run out)
};

constexpr int MX_WARPS = 8;
constexpr int MX_R = 4;          // sinks per lane
constexpr int MX_S = 32 * MX_R;  // sinks per CTA
static_assert(MX_S == MIXED_SINKS_PER_TILE, "tile size");
static_assert(sizeof(SplitPos) == SPLIT_POS_BYTES, "split size");
constexpr int MX_T = 256;        // sources per shared-memory tile

// an output row element and a velocity row element in the stage vectors' format (GravArgs::
// acc_f2, vel_f2: double-float pairs in the ensemble's mixed form, FP64 otherwise)
__device__ __forceinline__ void store_acc(const GravArgs& g, double* row, int i, double v)
{
    if (g.acc_f2)
        reinterpret_cast<float2*>(row)[i] = to_f2(v);
    else
        row[i] = v;
}

__device__ __forceinline__ double load_vel(const GravArgs& g, const double* row, int i)
{
    return g.vel_f2 ? f2_to_double(reinterpret_cast<const float2*>(row)[i]) : row[i];
}

__device__ __forceinline__ void exact_event_tests(const GravArgs& g, const Tile& tile, int i, int j, double xi,
                                                  double yi, double zi, double Ri, double mi, double rhoi)
{
    // __dadd_rn / __dmul_rn are never contracted into FMA: this file is built with FMA
    // contraction on, and these decisions must round exactly as the FP64 kernel's do.
    const double xj = g.px[j], yj = g.py[j], zj = g.pz[j];
    const double dx = __dadd_rn(xj, -xi), dy = __dadd_rn(yj, -yi), dz = __dadd_rn(zj, -zi);
    const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
    const double d = sqrt(r2);
    const int li = i - tile.base, lj = j - tile.base;
    const bool rad = g.record && li > 0 && li > lj && d < __dmul_rn(tile_f_rad(g, tile), __dadd_rn(Ri, g.radius[j]));
    bool hill = false;
    if (g.hill && tile.block != 2 && li > 0 && li > lj && lj > 0) {
        const double h = __dmul_rn(0.5, __dadd_rn(rhoi, g.rho[j]));
        const double lhs = __dmul_rn(__dmul_rn(d, d), d);
        const double rhs = __dmul_rn(__ddiv_rn(__dmul_rn(g.hill_f3, __dadd_rn(mi, g.mass[j])), __dmul_rn(3.0, g.mass[tile.base])),
                                     __dmul_rn(__dmul_rn(h, h), h));
        hill = lhs < rhs;
    }
    for (int kind = 0; kind < 2; kind++) {
        if (!(kind == 0 ? rad : hill)) continue;
        const EventBuf& eb = kind == 0 ? g.ev : g.hv;
        unsigned int slot = atomicAdd(eb.count, 1u);
        if (kind == 0 && g.sys_events) atomicAdd(&g.sys_events[tile.sys], 1u);
        if (slot < eb.cap) {
            DevEvent* e = &eb.rec[slot];
            e->seq = record_seq(g, tile, kind);
            e->kind = kind;
            e->i = i;
            e->j = j;
            e->sys = tile.sys;
            e->pad = 0;
            e->d = d;
            e->t = g.sys_t ? g.sys_t[tile.sys] : 0.0;
            const int b0 = tile.base;
            e->ri[0] = xi; e->ri[1] = yi; e->ri[2] = zi;
            e->rj[0] = xj; e->rj[1] = yj; e->rj[2] = zj;
            e->vi[0] = load_vel(g, g.vx, i); e->vi[1] = load_vel(g, g.vy, i); e->vi[2] = load_vel(g, g.vz, i);
            e->vj[0] = load_vel(g, g.vx, j); e->vj[1] = load_vel(g, g.vy, j); e->vj[2] = load_vel(g, g.vz, j);
            e->r0[0] = g.px[b0]; e->r0[1] = g.py[b0]; e->r0[2] = g.pz[b0];
            e->v0[0] = load_vel(g, g.vx, b0); e->v0[1] = load_vel(g, g.vy, b0); e->v0[2] = load_vel(g, g.vz, b0);
        }
    }
}

// ---------------------------------------------------------------------------------------
// Heavy pairs in double-float arithmetic.
//
// The pairs whose terms need more than FP32 accuracy -- sinks against the star and giant
// planets, and the star and giants' own rows -- would cost GB300 its scarce FP64 issue
// (grav_fp64_rowseq and the few-sink kernels spend about 35 FP64 operations per pair).
// Here they run on the FP32 pipes in unevaluated sums of two floats (hi + lo, about 44
// significant bits), built from the error-free transformations two-sum (Knuth) and
// two-product by FMA, with the double-double addition and multiplication of Hida, Li and
// Bailey (2001) carried out in float.  The inputs are the split positions and masses of
// split_positions_kernel (x = x_hi + x_lo to 2^-48 |x|), the displacement is formed from
// them exactly up to that split, 1/r^3 comes from the FP32 rsqrt refined by one Newton
// step evaluated in double-float (relative error about 2.5e-14), and the sums stay in
// double-float until one conversion to FP64 per sink and component.  Event decisions are
// screened in FP32 with the same 1e-3 margin as the mixed kernel and re-taken in FP64.


// the term m_j (r_j - r_i) / |r_j - r_i|^3 of one pair; r2f = |r_j - r_i|^2 in FP32
// the term from a double-float displacement r_j - r_i and the source's split mass
__device__ __forceinline__ void df_term_disp(DF dx, DF dy, DF dz, float mh, float ml, DF& tx, DF& ty, DF& tz,
                                             float& r2f)
{
    DF r2 = df_add_same_sign(df_add_same_sign(df_mul(dx, dx), df_mul(dy, dy)), df_mul(dz, dz));  // squares: no cancellation
    // a merged body parked at 1e20 AU (pp_disk.cu:1184) overflows r^2 in FP32; its mass is 0
    if (!(r2.hi < 1.0e30f)) r2 = DF{1.0e30f, 0.0f};
    const float y0 = rsqrt_approx(r2.hi);
    const DF p = df_mul(r2, df_two_prod(y0, y0));
    const float h = (1.0f - p.hi) - p.lo;  // 1 - r^2 y0^2, small: FP32 suffices
    const DF y = df_fast_sum(y0, 0.5f * y0 * h);
    const DF w = df_mul(df_mul(df_mul(y, y), y), DF{mh, ml});
    tx = df_mul(w, dx);
    ty = df_mul(w, dy);
    tz = df_mul(w, dz);
    r2f = r2.hi;
}

// the term from the split positions: the displacement (x_j^hi - x_i^hi) + (x_j^lo - x_i^lo)
// carries the positions to 2^-48 |x| (the split keeps 48 of FP64's 53 significant bits)
__device__ __forceinline__ void df_term(const SplitPos& si, const SplitPos& pj, DF& tx, DF& ty, DF& tz, float& r2f)
{
    df_term_disp(df_diff(pj.xy.x, pj.xy.y, si.xy.x, si.xy.y), df_diff(pj.xy.z, pj.xy.w, si.xy.z, si.xy.w),
                 df_diff(pj.zm.x, pj.zm.y, si.zm.x, si.zm.y), pj.zm.z, pj.zm.w, tx, ty, tz, r2f);
}

// r^2 below which a pair of this sink takes the FP64 displacement: beyond it the split
// positions' error, 2^-48 (|x_i| + |x_j|) per component, stays below ~1e-12 of |r_j - r_i|
__device__ __forceinline__ float close_r2(const SplitPos& p)
{
    const float m = fmaxf(fabsf(p.xy.x), fmaxf(fabsf(p.xy.z), fabsf(p.zm.x))) * (1.0f / 256.0f);
    return m * m;
}

// the term from the FP64 positions: the displacement is one FP64 subtraction per component
// (exact for neighbours, Sterbenz), kept to 2^-48 of itself -- for close pairs, where the
// split positions' 2^-48 |x| would be a large part of |r_j - r_i|
__device__ __forceinline__ void df_term_fp64(double xi, double yi, double zi, double xj, double yj, double zj,
                                             float mh, float ml, DF& tx, DF& ty, DF& tz, float& r2f)
{
    df_term_disp(split_df(__dadd_rn(xj, -xi)), split_df(__dadd_rn(yj, -yi)), split_df(__dadd_rn(zj, -zi)), mh, ml,
                 tx, ty, tz, r2f);
}

// FP32 screen of the event tests of pair_term (pp_disk.cu:262-280) with a 1e-3 margin;
// candidates are decided in FP64 by exact_event_tests
// frad: the tile's collision factor in FP32 (tile_frad_f, formed once per CTA: a per-pair load
// and conversion would run on GB300's FP64 pipe for every heavy pair)
__device__ __forceinline__ float tile_frad_f(const GravArgs& g, const Tile& tile)
{
    return g.sys_f_rad ? (float)g.sys_f_rad[tile.sys] : g.f_rad_f;
}

__device__ __forceinline__ void df_screen(const GravArgs& g, const Tile& tile, int i, int j, float r2f, float Ri,
                                          float Rj, float rhoi, float rhoj, float mi, float mj, float inv3M,
                                          float frad)
{
    const int li = i - tile.base, lj = j - tile.base;
    if (!(li > 0 && li > lj)) return;
    const float margin = 1.001f;
    bool cand = false;
    if (g.record) {
        const float lim = frad * (Ri + Rj) * margin;
        cand = r2f < lim * lim;
    }
    if (g.hill && tile.block != 2 && lj > 0) {
        const float h = 0.5f * (rhoi + rhoj);
        const float d3 = r2f * sqrtf(r2f);
        cand = cand || d3 < g.hill_f3_f * (mi + mj) * inv3M * (h * h * h) * (margin * margin * margin);
    }
    if (cand)
        exact_event_tests(g, tile, i, j, g.px[i], g.py[i], g.pz[i], g.radius[i], g.mass[i], g.hill ? g.rho[i] : 0.0);
}

// A sink's cutoff on the FP32 r^2 beyond which no pair of it with a light source passes the
// screens: each screen's limit grows with the source's radius, mass and star distance (FP32
// sums and products of non-negative factors round monotonically), so the limit computed, in
// the screens' own operation order, from the maxima over the system's light bodies (g.smax,
// split_positions) bounds it (heavy sources are screened by the heavy-source loop, without
// a cutoff).  The star-distance maximum gets a 1e-4 relative allowance for the rounding of
// its own evaluation; the Hill limit on r^2 is (the limit on r^3)^(2/3) x 1.001.  An
// undefined Hill limit (0 x inf) only arises where no Hill test can pass.  Without the
// maxima every pair is screened.
__device__ __forceinline__ float screen_cut2(const GravArgs& g, const Tile& tile, float Ri, float mi, float rhoi,
                                             float inv3M)
{
    if (!g.smax) return 3.0e38f;
    const unsigned int* sm = g.smax + SCREEN_MAX_WORDS * tile.sys;
    const float margin = 1.001f;
    float c = 0.0f;
    if (g.record) {
        const float lim = (g.sys_f_rad ? (float)g.sys_f_rad[tile.sys] : g.f_rad_f) * (Ri + __uint_as_float(sm[0])) * margin;
        c = lim * lim;
    }
    if (g.hill) {
        const float h = 0.5f * (rhoi + __uint_as_float(sm[2]) * 1.0001f);
        const float d3 = g.hill_f3_f * (mi + __uint_as_float(sm[1])) * inv3M * (h * h * h) *
                         (margin * margin * margin);
        const float cr = cbrtf(d3);
        c = fmaxf(c, cr * cr * 1.001f);
    }
    return c;
}

struct SinkD {
    double x, y, z, R, m, rho;
};


// The detailed FP32 screen of one light pair (sink i, source j) of the mixed kernel, with the
// same 1e-3 margin as df_screen; candidates are decided in FP64 by exact_event_tests.  sf:
// the sink's R, m, rho (FP32); Rj, rhoj: the source's.
__device__ __noinline__ void mixed_screen_pair(const GravArgs& g, const Tile& tile, int i, int j, float r2, float mj,
                                               float4 sf, float Rj, float rhoj, float inv3M, const SinkD& sd)
{
    const int li = i - tile.base, lj = j - tile.base;
    if (!(li > 0 && li > lj && mj >= 0.0f)) return;
    const float margin = 1.001f;
    bool cand = false;
    if (g.record) {
        const float lim = (g.sys_f_rad ? (float)g.sys_f_rad[tile.sys] : g.f_rad_f) * (sf.x + Rj) * margin;
        cand = r2 < lim * lim;
    }
    if (g.hill && tile.block != 2 && lj > 0) {
        const float h = 0.5f * (sf.z + rhoj);
        const float d3 = r2 * sqrtf(r2);
        cand = cand || (d3 < g.hill_f3_f * (sf.y + mj) * inv3M * (h * h * h) * (margin * margin * margin));
    }
    if (cand && 0 <= g.id[j]) exact_event_tests(g, tile, i, j, sd.x, sd.y, sd.z, sd.R, sd.m, sd.rho);
}

// The r^2 below which a pair of one sink and one warp-slice is flagged for the exact pass:
// every near pair (m_j > near_lim r^2, m_j <= mslice, the slice's largest mass), every
// self pair (r^2 = 0) and every screen candidate (r^2 < cut2) lies below it.  Proof of the
// near part: FP32 multiplication is monotone, so r^2 >= c gives fl(near_lim r^2) >=
// fl(near_lim c), which the check makes >= mslice.  A quotient that fails the check (no
// heavy source, an overflow) flags every pair of the slice.
__device__ __forceinline__ float flag_cut2(float mslice, float near_lim, float inv_near_lim, float cut2)
{
    float c = mslice > 0.0f ? mslice * inv_near_lim * 1.0001f : 0.0f;
    c = fmaxf(fmaxf(c, cut2), 1.17549435e-38f);  // FLT_MIN: self pairs (r^2 = 0) are flagged
    return near_lim * c >= mslice ? c : 3.0e38f;
}

// One warp-slice of a source tile (at most 32 sources) for MX_R sinks per lane: the FP32
// terms of the pairs whose r^2 is at or above the sink's flag cutoff (flag_cut2), one
// compare per pair, summed in FP32 over the slice and folded into the compensated
// accumulators once.  The flagged pairs add nothing here; their bits (source q - q_begin)
// go to `flags` for the warp's flagged-pair rounds.
__device__ __forceinline__ void mixed_slice(const SplitPos* s_sp, int q_begin, int q_end, const float* xh,
                                            const float* xl, const float* yh, const float* yl, const float* zh,
                                            const float* zl, const float* flag2, Acc2* ax, Acc2* ay, Acc2* az,
                                            unsigned* flags)
{
    float px[MX_R], py[MX_R], pz[MX_R];
#pragma unroll
    for (int r = 0; r < MX_R; r++) {
        px[r] = py[r] = pz[r] = 0.0f;
        flags[r] = 0u;
    }
    unsigned bit = 1u;
#pragma unroll 4
    for (int q = q_begin; q < q_end; q++, bit <<= 1) {
        const float4 pxy = s_sp[q].xy;
        const float4 pzm = s_sp[q].zm;
        const float mj = pzm.z;
#pragma unroll
        for (int r = 0; r < MX_R; r++) {
            const float dx = (pxy.x - xh[r]) + (pxy.y - xl[r]);
            const float dy = (pxy.z - yh[r]) + (pxy.w - yl[r]);
            const float dz = (pzm.x - zh[r]) + (pzm.y - zl[r]);
            // finite: split_positions clamps coordinates to 1e15 AU
            const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
            const bool flag = r2 < flag2[r];
            const float w = flag ? 0.0f : light_w(mj, r2);
            px[r] = fmaf(w, dx, px[r]);
            py[r] = fmaf(w, dy, py[r]);
            pz[r] = fmaf(w, dz, pz[r]);
            flags[r] |= flag ? bit : 0u;
        }
    }
#pragma unroll
    for (int r = 0; r < MX_R; r++) {
        two_sum_add(ax[r], px[r]);
        two_sum_add(ay[r], py[r]);
        two_sum_add(az[r], pz[r]);
    }
}

// One flagged pair (sink i, source j = j0 + q), classified exactly: a self pair adds
// nothing; a screen candidate (r^2 < cut2, the pair loop's FP32 r^2 recomputed by the same
// operations) goes to the detailed screen; a near pair (m_j > near_lim r^2) gives its
// double-float term, from the FP64 displacement where the split positions would not resolve
// the pair (close_r2); any other pair gives its FP32 term (lo parts 0).
struct FlagTerm {
    float hx, lx, hy, ly, hz, lz;
};

template <bool SCREEN>
__device__ __forceinline__ FlagTerm mixed_flag_term(const MixedArgs& a, const Tile& tile, int i, int j, int q,
                                                    const SplitPos* s_sp, const float* s_R, const float* s_rho,
                                                    const float4 sf, const SinkD& sd, const SplitPos sp,
                                                    float near_lim, float inv3M)
{
    const GravArgs& g = a.g;
    FlagTerm f{0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    if (j == i) return f;
    const SplitPos pj = s_sp[q];
    const float mj = pj.zm.z;
    const float dx = (pj.xy.x - sp.xy.x) + (pj.xy.y - sp.xy.y);
    const float dy = (pj.xy.z - sp.xy.z) + (pj.xy.w - sp.xy.w);
    const float dz = (pj.zm.x - sp.zm.x) + (pj.zm.y - sp.zm.y);
    const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    if (SCREEN && r2 < sf.w) mixed_screen_pair(g, tile, i, j, r2, mj, sf, s_R[q], s_rho[q], inv3M, sd);
    if (mj > near_lim * r2) {
        DF tx, ty, tz;
        float r2f;
        df_term(sp, pj, tx, ty, tz, r2f);
        if (r2f < close_r2(sp))
            df_term_fp64(sd.x, sd.y, sd.z, g.px[j], g.py[j], g.pz[j], mj, pj.zm.w, tx, ty, tz, r2f);
        f = FlagTerm{tx.hi, tx.lo, ty.hi, ty.lo, tz.hi, tz.lo};
    } else {
        const float w = light_w(mj, r2);
        f.hx = w * dx;
        f.hy = w * dy;
        f.hz = w * dz;
    }
    return f;
}

// Source tiles reach shared memory by TMA bulk copies (cp.async.bulk, one thread issues an
// 8 KB copy of MX_T split positions), double-buffered: tile t + 2 is requested while tile t
// is computed, each buffer's arrival is signalled on its own mbarrier (transaction bytes),
// and one CTA barrier per tile releases the buffer for reuse.  Every wait on a copy is
// bounded (tma.cuh: TMA_WAIT_NS of the GPU's global timer, or TMA_WAIT_POLLS polls should the
// timer not advance); a CTA whose copy does not arrive sets a.err, waits (again bounded)
// for the copies it issued, and returns.  `a.hold` (a test hook) issues no copies, so that
// the waits run out and the host sees the error status.

// dynamic shared memory of grav_mixed_kernel
struct MixedSmem {
    SplitPos sp[2][MX_T];              // double-buffered source tiles (TMA destination)
    SinkD sink[MX_S];
    float4 sinkf[MX_S];                // R, m, rho, r^2 cutoff of the sinks in FP32 (screens)
    float2 near_lim[MX_S];             // the sinks' near-pair limits and their reciprocals
    SplitPos sinksp[MX_S];             // the sinks' split positions
    FlagTerm fterm[MX_WARPS][32];      // one round of a warp's flagged-pair terms
    unsigned short fitem[MX_WARPS][32];  // the round's items: owner lane << 7 | row << 5 | source bit
    Acc2 part[MX_WARPS][3][MX_S];      // per-warp compensated partial sums
    float R[2][MX_T], rho[2][MX_T];    // screening data of the tiles (SCREEN only)
    unsigned long long bar[2];
    int fail;
};

template <bool SCREEN>
__global__ void __launch_bounds__(256, 2) grav_mixed_kernel(MixedArgs a)
{
    const GravArgs& g = a.g;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    MixedSmem& S = *reinterpret_cast<MixedSmem*>(smem_raw);

    const Tile tile = g.tiles[blockIdx.x];
    if (g.sys_active && !g.sys_active[tile.sys]) return;
    const int heavy_end = a.heavy_end[blockIdx.x];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int src_lo = tile.src_begin + blockIdx.y * a.chunk;
    const int src_hi = min(tile.src_end, src_lo + a.chunk);
    const int first = max(heavy_end, src_lo);
    const int n_tiles = first < src_hi ? (src_hi - first + MX_T - 1) / MX_T : 0;

    auto issue = [&](int t) {  // one thread
        const int j0 = first + t * MX_T;
        const int nj = min(MX_T, src_hi - j0);
        tma_tile(&S.sp[t & 1][0], a.sp + j0, (unsigned)(nj * sizeof(SplitPos)), &S.bar[t & 1]);
    };
    auto stage_screen = [&](int t) {  // all threads
        const int j0 = first + t * MX_T;
        const int nj = min(MX_T, src_hi - j0);
        for (int q = threadIdx.x; q < nj; q += blockDim.x) {
            S.R[t & 1][q] = g.rf[j0 + q];
            S.rho[t & 1][q] = g.hill ? star_dist_f(a.sp[j0 + q], a.sp[tile.base]) : 0.0f;
        }
    };

    if (threadIdx.x == 0) {
        mbar_init(&S.bar[0], 1);
        mbar_init(&S.bar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        S.fail = 0;
    }
    for (int s = threadIdx.x; s < MX_S; s += blockDim.x) {
        const int i = tile.sink_begin + s;
        SinkD sd{0, 0, 0, 0, 0, 0};
        if (i < tile.sink_end) {
            sd.x = g.px[i]; sd.y = g.py[i]; sd.z = g.pz[i];
            sd.R = g.radius[i]; sd.m = g.mass[i];
            sd.rho = g.hill ? g.rho[i] : 0.0;
        }
        S.sink[s] = sd;
        S.sinkf[s] = make_float4((float)sd.R, (float)sd.m, (float)sd.rho, 0.0f);
        SplitPos sp;
        sp.xy = sp.zm = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        float pull = 0.0f;
        if (i < tile.sink_end) {
            sp = a.sp[i];
            if (tile.src_begin < heavy_end) {  // m / r^2 of the first heavy source: the near-pair scale
                const int j = tile.src_begin;
                const double dx = g.px[j] - sd.x, dy = g.py[j] - sd.y, dz = g.pz[j] - sd.z;
                pull = (float)(g.mass[j] / (dx * dx + dy * dy + dz * dz));
            }
        }
        S.sinksp[s] = sp;
        // a pair is near when m_j > near_lim * r^2; without a heavy source there is no scale
        const float nl = pull > 0.0f ? a.near_ratio * pull : 3.0e38f;
        S.near_lim[s] = make_float2(nl, 1.0f / nl);
    }
    const float inv3M = (SCREEN && g.hill) ? (float)(1.0 / (3.0 * g.mass[tile.base])) : 0.0f;
    // .w: the sink's cutoff on r^2 (screen_cut2); padding sinks get none
    for (int s = threadIdx.x; s < MX_S; s += blockDim.x) {
        float4& sf = S.sinkf[s];
        sf.w = (SCREEN && tile.sink_begin + s < tile.sink_end) ? screen_cut2(g, tile, sf.x, sf.y, sf.z, inv3M)
                                                               : -1.0f;
    }
    __syncthreads();
    // the first two tiles travel while the heavy sources are summed
    if (threadIdx.x == 0 && !a.hold) {
        if (n_tiles > 0) issue(0);
        if (n_tiles > 1) issue(1);
    }
    if (SCREEN) {
        if (n_tiles > 0) stage_screen(0);
        if (n_tiles > 1) stage_screen(1);
    }

    int si[MX_R];
    float xh[MX_R], xl[MX_R], yh[MX_R], yl[MX_R], zh[MX_R], zl[MX_R];
    Acc2 ax[MX_R], ay[MX_R], az[MX_R];
#pragma unroll
    for (int r = 0; r < MX_R; r++) {
        const int s = lane + 32 * r;
        si[r] = tile.sink_begin + s;
        const SplitPos sp = S.sinksp[s];
        xh[r] = sp.xy.x; xl[r] = sp.xy.y; yh[r] = sp.xy.z; yl[r] = sp.xy.w;
        zh[r] = sp.zm.x; zl[r] = sp.zm.y;
        ax[r] = ay[r] = az[r] = Acc2{0.0f, 0.0f};
    }

    // heavy sources (first chunk only): double-float terms, split over the warps
    if (blockIdx.y == 0) {
        const float frad = SCREEN ? tile_frad_f(g, tile) : 0.0f;
        for (int j = tile.src_begin + warp; j < heavy_end; j += MX_WARPS) {
            if (0 > g.id[j]) continue;
            const SplitPos pj = a.sp[j];
            const double xj = g.px[j], yj = g.py[j], zj = g.pz[j];
            float Rj = 0.0f, rhoj = 0.0f;
            if (SCREEN) {
                Rj = (float)g.radius[j];
                rhoj = g.hill ? (float)g.rho[j] : 0.0f;
            }
#pragma unroll
            for (int r = 0; r < MX_R; r++) {
                const int s = lane + 32 * r;
                if (si[r] >= tile.sink_end || j == si[r]) continue;
                const SinkD& sd = S.sink[s];
                DF tx, ty, tz;
                float r2f;
                df_term_fp64(sd.x, sd.y, sd.z, xj, yj, zj, pj.zm.z, pj.zm.w, tx, ty, tz, r2f);
                acc_df(ax[r], tx);
                acc_df(ay[r], ty);
                acc_df(az[r], tz);
                if (SCREEN) {
                    const float4 sf = S.sinkf[s];
                    df_screen(g, tile, si[r], j, r2f, sf.x, Rj, sf.z, rhoj, sf.y, pj.zm.z, inv3M, frad);
                }
            }
        }
    }
    if (SCREEN) __syncthreads();  // the screening data of tiles 0 and 1 are visible

    constexpr int SLICE = MX_T / MX_WARPS;  // 32 sources per warp and tile: one flag bit each
    int t = 0;
    for (; t < n_tiles; t++) {
        const int b = t & 1;
        const int j0 = first + t * MX_T;
        const int nj = min(MX_T, src_hi - j0);
        // one answer per warp, so that the warp's shuffles below see all of its lanes
        const bool arrived = __all_sync(0xffffffffu, mbar_wait(&S.bar[b], (unsigned)((t >> 1) & 1)));
        if (!arrived) S.fail = 1;
        const int q_begin = warp * SLICE;
        const int q_end = min(nj, q_begin + SLICE);
        if (arrived && q_begin < q_end) {
            // the slice's largest mass, for the flag cutoffs
            float mslice = q_begin + lane < q_end ? S.sp[b][q_begin + lane].zm.z : 0.0f;
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) mslice = fmaxf(mslice, __shfl_xor_sync(0xffffffffu, mslice, off));
            float flag2[MX_R];
            unsigned flags[MX_R];
#pragma unroll
            for (int r = 0; r < MX_R; r++) {
                const float2 nl = S.near_lim[lane + 32 * r];
                flag2[r] = flag_cut2(mslice, nl.x, nl.y, S.sinkf[lane + 32 * r].w);
            }
            mixed_slice(S.sp[b], q_begin, q_end, xh, xl, yh, yl, zh, zl, flag2, ax, ay, az, flags);
            // The flagged pairs, shared out over the warp: each round, the lanes list up to 32
            // of their items (in row, source order) at an exclusive prefix of their counts,
            // each lane computes one listed item, and the owners add the round's terms in
            // their listing order -- the same order as a lane walking its own items.
            int cnt = 0;
#pragma unroll
            for (int r = 0; r < MX_R; r++) cnt += __popc(flags[r]);
            while (__any_sync(0xffffffffu, cnt > 0)) {
                int incl = cnt;
#pragma unroll
                for (int d = 1; d < 32; d <<= 1) {
                    const int v = __shfl_up_sync(0xffffffffu, incl, d);
                    if (lane >= d) incl += v;
                }
                const int off = incl - cnt;
                const int n_items = min(32, __shfl_sync(0xffffffffu, incl, 31));
                int take = max(0, min(cnt, 32 - off));
                cnt -= take;
                int taken[MX_R];
                int k = off;
#pragma unroll
                for (int r = 0; r < MX_R; r++) {
                    taken[r] = 0;
                    while (take > 0 && flags[r]) {
                        const int bit = __ffs(flags[r]) - 1;
                        flags[r] &= flags[r] - 1;
                        S.fitem[warp][k++] = (unsigned short)((lane << 7) | (r << 5) | bit);
                        taken[r]++;
                        take--;
                    }
                }
                __syncwarp();
                if (lane < n_items) {
                    const unsigned it = S.fitem[warp][lane];
                    const int s = (int)(it >> 7) + 32 * (int)((it >> 5) & 3u);
                    const int q = q_begin + (int)(it & 31u);
                    S.fterm[warp][lane] = mixed_flag_term<SCREEN>(a, tile, tile.sink_begin + s, j0 + q, q, S.sp[b], S.R[b],
                                                                  S.rho[b], S.sinkf[s], S.sink[s], S.sinksp[s],
                                                                  S.near_lim[s].x, inv3M);
                }
                __syncwarp();
                k = off;
#pragma unroll
                for (int r = 0; r < MX_R; r++) {
                    for (int u = 0; u < taken[r]; u++, k++) {
                        const FlagTerm f = S.fterm[warp][k];
                        acc_df(ax[r], DF{f.hx, f.lx});
                        acc_df(ay[r], DF{f.hy, f.ly});
                        acc_df(az[r], DF{f.hz, f.lz});
                    }
                }
                __syncwarp();  // the round's lists are read before the next round writes them
            }
        }
        __syncthreads();  // buffer b is free; the fail flag is visible
        if (S.fail) break;
        // tile t + 2 into buffer b; its screening data become visible at the next iteration's barrier
        if (t + 2 < n_tiles) {
            if (threadIdx.x == 0 && !a.hold) issue(t + 2);
            if (SCREEN) stage_screen(t + 2);
        }
    }
    if (S.fail) {
        if (threadIdx.x == 0) {
            atomicExch(a.err, 1u);
            // the copies this CTA issued and did not consume: tiles t and t + 1
            if (!a.hold)
                for (int u = t; u < min(t + 2, n_tiles); u++) mbar_wait(&S.bar[u & 1], (unsigned)((u >> 1) & 1));
        }
        return;
    }

    // per-sink total: fixed-order sum over the warps of the compensated partials
#pragma unroll
    for (int r = 0; r < MX_R; r++) {
        const int s = lane + 32 * r;
        S.part[warp][0][s] = ax[r];
        S.part[warp][1][s] = ay[r];
        S.part[warp][2][s] = az[r];
    }
    __syncthreads();
    for (int k = threadIdx.x; k < 3 * MX_S; k += blockDim.x) {
        const int comp = k / MX_S, s = k % MX_S;
        const int i = tile.sink_begin + s;
        if (i >= tile.sink_end) continue;
        double v = 0.0;
        for (int w = 0; w < MX_WARPS; w++) v += f2d_bits(S.part[w][comp][s].s) + f2d_bits(S.part[w][comp][s].c);
        if (!(0 < g.id[i])) v = 0.0;  // inactive sinks feel nothing (pp_disk.cu:235-236)
        if (a.partial)
            a.partial[((long long)blockIdx.y * 3 + comp) * a.n_part + i] = v;
        else
            store_acc(g, comp == 0 ? g.ax : (comp == 1 ? g.ay : g.az), i, v);
    }
}

// a_i = sum over source chunks of the partials, in chunk order
__global__ void mixed_reduce_kernel(const double* __restrict__ partial, int n_chunks, int n_part, const Tile* tiles,
                                    int n_tiles, const int* sys_active, double* ax, double* ay, double* az,
                                    int acc_f2)
{
    const Tile tile = tiles[blockIdx.x];
    if (sys_active && !sys_active[tile.sys]) return;
    const int i = tile.sink_begin + threadIdx.x;
    if (i >= tile.sink_end) return;
    for (int comp = 0; comp < 3; comp++) {
        double v = 0.0;
        for (int c = 0; c < n_chunks; c++) v += partial[((long long)c * 3 + comp) * n_part + i];
        double* row = comp == 0 ? ax : (comp == 1 ? ay : az);
        if (acc_f2)
            reinterpret_cast<float2*>(row)[i] = to_f2(v);
        else
            row[i] = v;
    }
}

// Row kernel: one thread per sink, the tile's sources (a few massive bodies) staged in
// shared memory -- the mixed-precision counterpart of grav_fp64_rowseq.
constexpr int DF_ROW_NT = 128;

template <bool SCREEN>
__global__ void __launch_bounds__(DF_ROW_NT, 8) grav_df_rowseq(GravArgs g, const SplitPos* __restrict__ sp)
{
    __shared__ SplitPos s_p[DF_ROW_NT];
    __shared__ float s_R[DF_ROW_NT], s_rho[DF_ROW_NT];
    __shared__ int s_id[DF_ROW_NT];
    const Tile tile = g.tiles[blockIdx.x];
    if (g.sys_active && !g.sys_active[tile.sys]) return;
    const int t = threadIdx.x;
    const int i = tile.sink_begin + t;
    const bool sink_ok = i < tile.sink_end;
    const bool active = sink_ok && 0 < g.id[i];
    SplitPos si{};
    float Ri = 0.0f, rhoi = 0.0f, mi = 0.0f, inv3M = 0.0f;
    const float frad = SCREEN ? tile_frad_f(g, tile) : 0.0f;
    SplitPos p0{};
    if (SCREEN && g.hill) {
        p0 = sp[tile.base];
        inv3M = 1.0f / (3.0f * p0.zm.z);
    }
    if (active) {
        si = sp[i];
        if (SCREEN) {
            Ri = g.rf[i];
            rhoi = g.hill ? star_dist_f(si, p0) : 0.0f;
            mi = si.zm.z;
        }
    }
    const float close2 = close_r2(si);
    Acc2 ax{0.0f, 0.0f}, ay{0.0f, 0.0f}, az{0.0f, 0.0f};  // compensated: a few terms per sink
    for (int j0 = tile.src_begin; j0 < tile.src_end; j0 += DF_ROW_NT) {
        const int nj = min(DF_ROW_NT, tile.src_end - j0);
        if (t < nj) {
            const int j = j0 + t;
            s_p[t] = sp[j];
            s_id[t] = g.id[j];
            if (SCREEN) {
                s_R[t] = g.rf[j];
                s_rho[t] = g.hill ? star_dist_f(s_p[t], p0) : 0.0f;
            }
        }
        __syncthreads();
        if (active) {
            for (int q = 0; q < nj; q++) {
                const int j = j0 + q;
                if (j == i || s_id[q] < 0) continue;
                DF tx, ty, tz;
                float r2f;
                df_term(si, s_p[q], tx, ty, tz, r2f);
                if (r2f < close2)
                    df_term_fp64(g.px[i], g.py[i], g.pz[i], g.px[j], g.py[j], g.pz[j], s_p[q].zm.z, s_p[q].zm.w, tx,
                                 ty, tz, r2f);
                acc_df(ax, tx);
                acc_df(ay, ty);
                acc_df(az, tz);
                if (SCREEN) df_screen(g, tile, i, j, r2f, Ri, s_R[q], rhoi, s_rho[q], mi, s_p[q].zm.z, inv3M, frad);
            }
        }
        __syncthreads();
    }
    if (sink_ok) {
        if (g.acc_f2) {  // the compensated sums as double-float pairs, no FP64 work
            const DF x = df_two_sum(ax.s, ax.c), y = df_two_sum(ay.s, ay.c), z = df_two_sum(az.s, az.c);
            reinterpret_cast<float2*>(g.ax)[i] = make_float2(x.hi, x.lo);
            reinterpret_cast<float2*>(g.ay)[i] = make_float2(y.hi, y.lo);
            reinterpret_cast<float2*>(g.az)[i] = make_float2(z.hi, z.lo);
        } else {
            g.ax[i] = f2d_bits(ax.s) + f2d_bits(ax.c);
            g.ay[i] = f2d_bits(ay.s) + f2d_bits(ay.c);
            g.az[i] = f2d_bits(az.s) + f2d_bits(az.c);
        }
    }
}

// Few-sink kernel: tiles of at most FEW_SINKS_MAX heavy sinks against many sources.
// grid (source chunks, tiles); a CTA takes `chunk` sources of one tile, every thread keeps
// double-float sums for all the tile's sinks, and the CTA's sums go to
// partial[(comp * rows + row) * pitch + chunk index] as FP64; df_few_final adds the chunks.
// The chunk is DF_FEW_CHUNK_MAX sources (the per-CTA reduction of the sums is then a small
// part of the work), halved -- down to one source per thread -- while the grid has fewer
// than DF_FEW_GRID_MIN CTAs (two per SM of a 152-SM GB300), e.g. for a single star row.
constexpr int DF_FEW_CHUNK_MAX = 2048;
constexpr int DF_FEW_CHUNK_MIN = 256;
constexpr int DF_FEW_GRID_MIN = 304;

struct DfFewArgs {
    GravArgs g;
    const SplitPos* sp;
    const int* tile_row0;  // first row of each tile
    double* partial;
    int rows;
    long long pitch;  // >= chunks of the longest row
    int chunk;        // sources per CTA
};

template <bool SCREEN, int SMAX>
__global__ void __launch_bounds__(256, SMAX <= 4 ? 3 : 2) grav_df_few(DfFewArgs a)
{
    const GravArgs& g = a.g;
    const Tile tile = g.tiles[blockIdx.y];
    if (g.sys_active && !g.sys_active[tile.sys]) return;
    const int nsrc = tile.src_end - tile.src_begin;
    const int c0 = blockIdx.x * a.chunk;
    if (c0 >= nsrc) return;
    const int ns = tile.sink_end - tile.sink_begin;  // <= SMAX
    __shared__ SplitPos s_sink[SMAX];
    __shared__ float s_R[SMAX], s_rho[SMAX], s_m[SMAX], s_close2[SMAX];
    __shared__ int s_act[SMAX];
    __shared__ DF s_red[8][3 * SMAX];
    SplitPos p0{};
    float inv3M = 0.0f;
    const float frad = SCREEN ? tile_frad_f(g, tile) : 0.0f;
    if (SCREEN && g.hill) {
        p0 = a.sp[tile.base];
        inv3M = 1.0f / (3.0f * p0.zm.z);
    }
    if (threadIdx.x < ns) {
        const int i = tile.sink_begin + threadIdx.x;
        const SplitPos pi = a.sp[i];
        s_sink[threadIdx.x] = pi;
        s_act[threadIdx.x] = 0 < g.id[i];
        s_R[threadIdx.x] = SCREEN ? g.rf[i] : 0.0f;
        s_rho[threadIdx.x] = (SCREEN && g.hill) ? star_dist_f(pi, p0) : 0.0f;
        s_m[threadIdx.x] = pi.zm.z;
        s_close2[threadIdx.x] = close_r2(pi);
    }
    __syncthreads();
    Acc2 acc[SMAX][3];  // compensated sums of the thread's sources (a few per chunk)
#pragma unroll
    for (int s = 0; s < SMAX; s++)
#pragma unroll
        for (int c = 0; c < 3; c++) acc[s][c] = Acc2{0.0f, 0.0f};
    const int c1 = min(nsrc, c0 + a.chunk);
    for (int q = c0 + (int)threadIdx.x; q < c1; q += blockDim.x) {
        const int j = tile.src_begin + q;
        if (g.id[j] < 0) continue;
        const SplitPos pj = a.sp[j];
        float Rj = 0.0f, rhoj = 0.0f;
        if (SCREEN) {
            Rj = g.rf[j];
            rhoj = g.hill ? star_dist_f(pj, p0) : 0.0f;
        }
#pragma unroll
        for (int s = 0; s < SMAX; s++) {
            if (s < ns) {
                const int i = tile.sink_begin + s;
                if (s_act[s] && j != i) {
                    DF tx, ty, tz;
                    float r2f;
                    df_term(s_sink[s], pj, tx, ty, tz, r2f);
                    if (r2f < s_close2[s])
                        df_term_fp64(g.px[i], g.py[i], g.pz[i], g.px[j], g.py[j], g.pz[j], pj.zm.z, pj.zm.w, tx, ty,
                                     tz, r2f);
                    acc_df(acc[s][0], tx);
                    acc_df(acc[s][1], ty);
                    acc_df(acc[s][2], tz);
                    if (SCREEN) df_screen(g, tile, i, j, r2f, s_R[s], Rj, s_rho[s], rhoj, s_m[s], pj.zm.z, inv3M, frad);
                }
            }
        }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int s = 0; s < SMAX; s++) {
        if (s < ns) {  // uniform over the CTA
#pragma unroll
            for (int c = 0; c < 3; c++) {
                // the warp's compensated sums merged pairwise (a two-sum of the leading parts
                // and one addition of the corrections: a third of a double-float addition)
                Acc2 v = acc[s][c];
#pragma unroll
                for (int off = 16; off > 0; off >>= 1) {
                    const Acc2 o{__shfl_xor_sync(0xffffffffu, v.s, off), __shfl_xor_sync(0xffffffffu, v.c, off)};
                    v = two_sum_merge(v, o);
                }
                if (lane == 0) s_red[warp][3 * s + c] = df_two_sum(v.s, v.c);
            }
        }
    }
    __syncthreads();
    if ((int)threadIdx.x < 3 * ns) {
        const int s = threadIdx.x / 3, c = threadIdx.x % 3;
        DF v = s_red[0][threadIdx.x];
        for (int w = 1; w < (int)(blockDim.x >> 5); w++) v = df_add(v, s_red[w][threadIdx.x]);
        const int row = a.tile_row0[blockIdx.y] + s;
        a.partial[((long long)c * a.rows + row) * a.pitch + blockIdx.x] = df_to_double(v);
    }
}

// Heavy-light pairs once for both directions.  A system whose SI block is a few heavy
// bodies (star, giant planets: rows over every massive body) and whose NSI block takes the
// row kernel over them (light bodies: rows over the SI bodies) has each (heavy h, light i)
// pair in two rows.  The displacement, r^2, y = 1/r and y^3 are the same for both; this
// kernel forms them once and both terms from them:
//   i's row:  (y^3 m_h) (r_h - r_i)   -- grav_df_rowseq's term, bit for bit, in its source order
//   h's row: -(y^3 m_i) (r_h - r_i)   -- summed over the thread's light bodies in compensated
//                                        accumulators, then over the CTA
// The light bodies of all such systems, end to end, are cut into one equal range per CTA (the
// grid is a whole wave); a range is split into segments at system boundaries, and each
// segment is one part of its system's heavy rows: partial[(comp * rows + row) * pitch +
// part].  The segment with part 1 also forms the heavy-heavy pairs (grav_df_few's terms and
// screens) into part 0.  The system's last segment to finish (a ticket per system, reset by
// it) adds the parts in order into the heavy rows.  The close-pair FP64 displacement is taken
// when either body's split positions would be too coarse for it (the row kernel's and the
// few kernel's thresholds).
// a body's split record from its FP64 coordinates and its split mass (split_positions_kernel's)
__device__ __forceinline__ SplitPos split_record(double x, double y, double z, float2 m)
{
    SplitPos p;
    split_coord(x, p.xy.x, p.xy.y);
    split_coord(y, p.xy.z, p.xy.w);
    split_coord(z, p.zm.x, p.zm.y);
    p.zm.z = m.x;
    p.zm.w = m.y;
    return p;
}

struct DfSymArgs {
    GravArgs g;             // tiles: the segments (Tile::part from 1)
    const int* cta_seg;     // CTA c takes segments [cta_seg[c], cta_seg[c + 1])
    const SplitPos* sp;
    const int* tile_row0;   // per segment: its system's first heavy row
    double* partial;
    int rows;
    long long pitch;
    const int* row_sink;    // the heavy rows' bodies
    const int* row_nparts;  // parts per heavy row: 1 + the system's segments
    unsigned int* ticket;   // per system, zero between launches
    const float2* mass_f2;  // FROM64: the split masses; the coordinates are split here from FP64
};

// FROM64: the split records are formed here from the FP64 coordinates and mass_f2 (a later
// stage of an attempt, whose coordinates the split records do not hold): 32 B read per light
// body, where a separate split pass would read 24 and write 32 before this kernel's 32
template <bool SCREEN, int HMAX, bool FROM64>
__global__ void __launch_bounds__(256, DF_SYM_RESIDENT) grav_df_sym(DfSymArgs a)
{
    pdl_wait();  // first: every CTA waits for the kernel before it (the launch may overlap them)
    const GravArgs& g = a.g;
    __shared__ SplitPos s_h[HMAX];
    __shared__ float s_R[HMAX], s_rho[HMAX], s_close2[HMAX];
    __shared__ double s_x[HMAX], s_y[HMAX], s_z[HMAX];
    __shared__ int s_src[HMAX], s_sink[HMAX];
    __shared__ DF s_red[8][3 * HMAX];
    __shared__ DF s_hh[HMAX][HMAX][3];
    __shared__ int s_last;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int sg = a.cta_seg[blockIdx.x]; sg < a.cta_seg[blockIdx.x + 1]; sg++) {
        const Tile tile = g.tiles[sg];
        if (g.sys_active && !g.sys_active[tile.sys]) continue;  // uniform over the CTA
        const int nh = tile.src_end - tile.src_begin;          // <= HMAX (the launcher's choice)
        SplitPos p0{};
        float inv3M = 0.0f;
        const float frad = SCREEN ? tile_frad_f(g, tile) : 0.0f;
        if (SCREEN && g.hill) {
            p0 = FROM64 ? split_record(g.px[tile.base], g.py[tile.base], g.pz[tile.base], a.mass_f2[tile.base])
                        : a.sp[tile.base];
            inv3M = 1.0f / (3.0f * p0.zm.z);
        }
        __syncthreads();  // the previous segment's shared data are consumed
        if ((int)threadIdx.x < nh) {
            const int h = tile.src_begin + threadIdx.x;
            const SplitPos ph = FROM64 ? split_record(g.px[h], g.py[h], g.pz[h], a.mass_f2[h]) : a.sp[h];
            const int id = g.id[h];
            s_h[threadIdx.x] = ph;
            s_src[threadIdx.x] = 0 <= id;  // a source term (pp_disk.cu:246-247)
            s_sink[threadIdx.x] = 0 < id;  // a sink's row (pp_disk.cu:235-236)
            s_R[threadIdx.x] = SCREEN ? g.rf[h] : 0.0f;
            s_rho[threadIdx.x] = (SCREEN && g.hill) ? star_dist_f(ph, p0) : 0.0f;
            s_close2[threadIdx.x] = close_r2(ph);
            s_x[threadIdx.x] = g.px[h];
            s_y[threadIdx.x] = g.py[h];
            s_z[threadIdx.x] = g.pz[h];
        }
        __syncthreads();
        const int row0 = a.tile_row0[sg];
        if (tile.part == 1) {  // part 0: the heavy-heavy pairs, as grav_df_few forms them
            const int t = threadIdx.x;
            if (t < nh * nh) {
                const int hs = t / nh, hq = t % nh;  // sink, source
                DF tx{0.0f, 0.0f}, ty{0.0f, 0.0f}, tz{0.0f, 0.0f};
                if (hs != hq && s_sink[hs] && s_src[hq]) {
                    float r2f;
                    df_term(s_h[hs], s_h[hq], tx, ty, tz, r2f);
                    if (r2f < s_close2[hs])
                        df_term_fp64(s_x[hs], s_y[hs], s_z[hs], s_x[hq], s_y[hq], s_z[hq], s_h[hq].zm.z,
                                     s_h[hq].zm.w, tx, ty, tz, r2f);
                    if (SCREEN)
                        df_screen(g, tile, tile.src_begin + hs, tile.src_begin + hq, r2f, s_R[hs], s_R[hq],
                                  s_rho[hs], s_rho[hq], s_h[hs].zm.z, s_h[hq].zm.z, inv3M, frad);
                }
                s_hh[hs][hq][0] = tx;
                s_hh[hs][hq][1] = ty;
                s_hh[hs][hq][2] = tz;
            }
            __syncthreads();
            if (t < 3 * nh) {
                const int hs = t / 3, c = t % 3;
                Acc2 v{0.0f, 0.0f};
                for (int q = 0; q < nh; q++) acc_df(v, s_hh[hs][q][c]);
                a.partial[((long long)c * a.rows + row0 + hs) * a.pitch] = f2d_bits(v.s) + f2d_bits(v.c);
            }
        }
        Acc2 racc[HMAX][3];
#pragma unroll
        for (int h = 0; h < HMAX; h++)
#pragma unroll
            for (int c = 0; c < 3; c++) racc[h][c] = Acc2{0.0f, 0.0f};
        // the next light body's record is loaded while the current one's pairs are formed
        int i = tile.sink_begin + (int)threadIdx.x;
        SplitPos pn{};
        double xn = 0.0, yn = 0.0, zn = 0.0;
        float2 mn{0.0f, 0.0f};
        int idn = -1;
        float Rn = 0.0f;
        auto fetch = [&](int j) {
            if constexpr (FROM64) {
                xn = g.px[j];
                yn = g.py[j];
                zn = g.pz[j];
                mn = a.mass_f2[j];
            } else {
                pn = a.sp[j];
            }
            idn = g.id[j];
            if (SCREEN) Rn = g.rf[j];
        };
        if (i < tile.sink_end) fetch(i);
        for (; i < tile.sink_end; i += blockDim.x) {
            const SplitPos pi = FROM64 ? split_record(xn, yn, zn, mn) : pn;
            const int idi = idn;
            const float Ri = Rn;
            if (i + (int)blockDim.x < tile.sink_end) fetch(i + blockDim.x);
            const bool sink_ok = 0 < idi, src_ok = 0 <= idi;
            Acc2 ox{0.0f, 0.0f}, oy{0.0f, 0.0f}, oz{0.0f, 0.0f};
            if (src_ok) {
                const float rhoi = (SCREEN && g.hill) ? star_dist_f(pi, p0) : 0.0f;
                const float close_i = close_r2(pi);
                const DF mi{pi.zm.z, pi.zm.w};
#pragma unroll
                for (int h = 0; h < HMAX; h++) {
                    if (h >= nh) continue;
                    const bool own = sink_ok && s_src[h];
                    const bool rev = s_sink[h] != 0;
                    if (!(own || rev)) continue;
                    const SplitPos ph = s_h[h];
                    DF dx = df_diff(ph.xy.x, ph.xy.y, pi.xy.x, pi.xy.y);
                    DF dy = df_diff(ph.xy.z, ph.xy.w, pi.xy.z, pi.xy.w);
                    DF dz = df_diff(ph.zm.x, ph.zm.y, pi.zm.x, pi.zm.y);
                    DF r2 = df_add_same_sign(df_add_same_sign(df_mul(dx, dx), df_mul(dy, dy)), df_mul(dz, dz));
                    if (r2.hi < fmaxf(close_i, s_close2[h])) {  // the FP64 displacement (df_term_fp64)
                        dx = split_df(__dadd_rn(s_x[h], -g.px[i]));
                        dy = split_df(__dadd_rn(s_y[h], -g.py[i]));
                        dz = split_df(__dadd_rn(s_z[h], -g.pz[i]));
                        r2 = df_add_same_sign(df_add_same_sign(df_mul(dx, dx), df_mul(dy, dy)), df_mul(dz, dz));
                    }
                    if (!(r2.hi < 1.0e30f)) r2 = DF{1.0e30f, 0.0f};  // a merged body parked at 1e20 AU
                    const float y0 = rsqrt_approx(r2.hi);
                    const DF p = df_mul(r2, df_two_prod(y0, y0));
                    const float hh = (1.0f - p.hi) - p.lo;
                    const DF y = df_fast_sum(y0, 0.5f * y0 * hh);
                    const DF y3 = df_mul(df_mul(y, y), y);
                    if (own) {
                        const DF w = df_mul(y3, DF{ph.zm.z, ph.zm.w});
                        acc_df(ox, df_mul(w, dx));
                        acc_df(oy, df_mul(w, dy));
                        acc_df(oz, df_mul(w, dz));
                        if (SCREEN)
                            df_screen(g, tile, i, tile.src_begin + h, r2.hi, Ri, s_R[h], rhoi, s_rho[h], pi.zm.z,
                                      ph.zm.z, inv3M, frad);
                    }
                    if (rev) {
                        const DF w = df_mul(y3, mi);
                        const DF tx = df_mul(w, dx), ty = df_mul(w, dy), tz = df_mul(w, dz);
                        acc_df(racc[h][0], DF{-tx.hi, -tx.lo});
                        acc_df(racc[h][1], DF{-ty.hi, -ty.lo});
                        acc_df(racc[h][2], DF{-tz.hi, -tz.lo});
                    }
                }
            }
            if (g.acc_f2) {
                const DF x = df_two_sum(ox.s, ox.c), y = df_two_sum(oy.s, oy.c), z = df_two_sum(oz.s, oz.c);
                reinterpret_cast<float2*>(g.ax)[i] = make_float2(x.hi, x.lo);
                reinterpret_cast<float2*>(g.ay)[i] = make_float2(y.hi, y.lo);
                reinterpret_cast<float2*>(g.az)[i] = make_float2(z.hi, z.lo);
            } else {
                g.ax[i] = f2d_bits(ox.s) + f2d_bits(ox.c);
                g.ay[i] = f2d_bits(oy.s) + f2d_bits(oy.c);
                g.az[i] = f2d_bits(oz.s) + f2d_bits(oz.c);
            }
        }
#pragma unroll
        for (int h = 0; h < HMAX; h++) {
            if (h < nh) {  // uniform over the CTA
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    Acc2 v = racc[h][c];
#pragma unroll
                    for (int off = 16; off > 0; off >>= 1) {
                        const Acc2 o{__shfl_xor_sync(0xffffffffu, v.s, off), __shfl_xor_sync(0xffffffffu, v.c, off)};
                        v = two_sum_merge(v, o);
                    }
                    if (lane == 0) s_red[warp][3 * h + c] = df_two_sum(v.s, v.c);
                }
            }
        }
        __syncthreads();
        if ((int)threadIdx.x < 3 * nh) {
            const int h = threadIdx.x / 3, c = threadIdx.x % 3;
            DF v = s_red[0][threadIdx.x];
            for (int w = 1; w < (int)(blockDim.x >> 5); w++) v = df_add(v, s_red[w][threadIdx.x]);
            a.partial[((long long)c * a.rows + row0 + h) * a.pitch + tile.part] = df_to_double(v);
        }
        // the system's last segment adds its heavy rows' parts in order (no waiting: the
        // others are done)
        const int np = a.row_nparts[row0];
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            s_last = atomicAdd(&a.ticket[tile.sys], 1u) == (unsigned int)(np - 2);  // np - 1 segments
        }
        __syncthreads();
        if (s_last) {
            __threadfence();
            if (threadIdx.x == 0) a.ticket[tile.sys] = 0u;
            if ((int)threadIdx.x < 3 * nh) {
                const int h = threadIdx.x / 3, c = threadIdx.x % 3;
                const double* P = a.partial + ((long long)c * a.rows + row0 + h) * a.pitch;
                double v = 0.0;
                for (int q = 0; q < np; q++) v += __ldcg(P + q);
                double* out = c == 0 ? g.ax : (c == 1 ? g.ay : g.az);
                store_acc(g, out, a.row_sink[row0 + h], v);
            }
        }
    }
}

struct DfFinalArgs {
    int acc_f2;
    const double* partial;
    int rows, row0, nrows;
    long long pitch;
    const int* row_sink;
    const int* row_nsrc;
    const int* row_sys;     // nullptr for one disk
    const int* sys_active;
    double *ax, *ay, *az;
    int chunk;
};

// one thread per (row, component): the row's chunk sums in order
__global__ void df_few_final(DfFinalArgs a)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= 3 * a.nrows) return;
    const int comp = k / a.nrows, row = a.row0 + k % a.nrows;
    if (a.sys_active && a.row_sys && !a.sys_active[a.row_sys[row]]) return;
    const int nch = (a.row_nsrc[row] + a.chunk - 1) / a.chunk;
    const double* P = a.partial + ((long long)comp * a.rows + row) * a.pitch;
    double s = 0.0;
    for (int c = 0; c < nch; c++) s += P[c];
    double* out = comp == 0 ? a.ax : (comp == 1 ? a.ay : a.az);
    if (a.acc_f2)
        reinterpret_cast<float2*>(out)[a.row_sink[row]] = to_f2(s);
    else
        out[a.row_sink[row]] = s;
}

int launch_grav_df_rowseq(const GravArgs& g, const void* split, cudaStream_t st)
{
    if (g.n_tiles <= 0) return 0;
    const SplitPos* sp = (const SplitPos*)split;
    if (g.record || g.hill)
        grav_df_rowseq<true><<<g.n_tiles, DF_ROW_NT, 0, st>>>(g, sp);
    else
        grav_df_rowseq<false><<<g.n_tiles, DF_ROW_NT, 0, st>>>(g, sp);
    RG_CUDA_CHECK(cudaGetLastError());
    return 0;
}

int launch_grav_df_few(const GravArgs& g, const void* split, const int* tile_row0, int max_src, int max_sinks,
                       int chunk_hint, double* partial, int rows, long long pitch, const int* row_sink,
                       const int* row_nsrc, const int* row_sys, int group_row0, int group_rows, cudaStream_t st)
{
    if (g.n_tiles <= 0 || group_rows <= 0) return 0;
    if (max_sinks > FEW_SINKS_MAX) return set_error(RG_ERR_STATE, "few-sink tile wider than FEW_SINKS_MAX");
    int chunk = DF_FEW_CHUNK_MAX;
    if (chunk_hint > 0)  // a tuned chunk: a multiple of the CTA's 256 threads
        chunk = std::max(DF_FEW_CHUNK_MIN, std::min(DF_FEW_CHUNK_MAX, chunk_hint / 256 * 256));
    else
        while (chunk > DF_FEW_CHUNK_MIN && (long long)g.n_tiles * ((max_src + chunk - 1) / chunk) < DF_FEW_GRID_MIN)
            chunk /= 2;
    const int chunks = std::max(1, (max_src + chunk - 1) / chunk);
    if ((long long)chunks > pitch) return set_error(RG_ERR_STATE, "few-sink partial buffer too narrow");
    DfFewArgs a{g, (const SplitPos*)split, tile_row0, partial, rows, pitch, chunk};
    const dim3 grid(chunks, g.n_tiles);
    const bool screen = g.record || g.hill;
    if (max_sinks <= 4) {
        if (screen)
            grav_df_few<true, 4><<<grid, 256, 0, st>>>(a);
        else
            grav_df_few<false, 4><<<grid, 256, 0, st>>>(a);
    } else {
        if (screen)
            grav_df_few<true, FEW_SINKS_MAX><<<grid, 256, 0, st>>>(a);
        else
            grav_df_few<false, FEW_SINKS_MAX><<<grid, 256, 0, st>>>(a);
    }
    RG_CUDA_CHECK(cudaGetLastError());
    DfFinalArgs f{g.acc_f2, partial, rows, group_row0, group_rows, pitch, row_sink, row_nsrc, row_sys, g.sys_active,
                  g.ax, g.ay, g.az, chunk};
    df_few_final<<<(3 * group_rows + 127) / 128, 128, 0, st>>>(f);
    RG_CUDA_CHECK(cudaGetLastError());
    return 0;
}

int launch_grav_df_sym(const GravArgs& g, const int* cta_seg, int n_cta, const void* split, const int* tile_row0,
                       int max_heavy, double* partial, int rows, long long pitch, const int* row_sink,
                       const int* row_nparts, unsigned int* ticket, cudaStream_t st, const float2* mass_f2)
{
    if (g.n_tiles <= 0 || n_cta <= 0) return 0;
    if (max_heavy < 1 || max_heavy > DF_SYM_MAX_HEAVY) return set_error(RG_ERR_STATE, "symmetric tile: heavy bodies");
    DfSymArgs b{g, cta_seg, (const SplitPos*)split, tile_row0, partial, rows, pitch, row_sink, row_nparts, ticket,
                mass_f2};
    const bool screen = g.record || g.hill;
    // may be scheduled while the kernel before it finishes (programmatic dependent launch)
    cudaLaunchAttribute pdl[1];
    pdl[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    pdl[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3((unsigned)n_cta);
    cfg.blockDim = dim3(256);
    cfg.stream = st;
    cfg.attrs = pdl;
    cfg.numAttrs = 1;
#define RG_SYM2(H, F)                                                                   \
    do {                                                                                \
        if (screen)                                                                     \
            RG_CUDA_CHECK(cudaLaunchKernelEx(&cfg, grav_df_sym<true, H, F>, b));        \
        else                                                                            \
            RG_CUDA_CHECK(cudaLaunchKernelEx(&cfg, grav_df_sym<false, H, F>, b));       \
    } while (0)
#define RG_SYM(H)               \
    do {                        \
        if (mass_f2)            \
            RG_SYM2(H, true);   \
        else                    \
            RG_SYM2(H, false);  \
    } while (0)
    if (max_heavy <= 3)
        RG_SYM(3);
    else
        RG_SYM(DF_SYM_MAX_HEAVY);
#undef RG_SYM
#undef RG_SYM2
    RG_CUDA_CHECK(cudaGetLastError());
    return 0;
}

// the coordinates alone of a later stage (the masses, radii and ids change only at events, and
// the step start's split has written them): 24 B read and written per body instead of 80
__global__ void split_coords_kernel(const double* __restrict__ x, const double* __restrict__ y,
                                    const double* __restrict__ z, int n, SplitPos* __restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 xy;
    float2 zz;
    split_coord(x[i], xy.x, xy.y);
    split_coord(y[i], xy.z, xy.w);
    split_coord(z[i], zz.x, zz.y);
    out[i].xy = xy;
    *reinterpret_cast<float2*>(&out[i].zm) = zz;
}

int launch_split_coords(const double* x, const double* y, const double* z, int n, SplitPos* out, cudaStream_t st)
{
    if (n <= 0) return 0;
    split_coords_kernel<<<(n + 255) / 256, 256, 0, st>>>(x, y, z, n, out);
    RG_CUDA_CHECK(cudaGetLastError());
    return 0;
}

int launch_split_positions(const double* x, const double* y, const double* z, const double* m, const int* id,
                           const int* base_of, const int* screen_slot, const double* radius, int n,
                           SplitPos* out, float* rf, unsigned int* smax, bool hill, cudaStream_t st, float2* mass_f2)
{
    if (n <= 0) return 0;
    split_positions_kernel<<<(n + 255) / 256, 256, 0, st>>>(x, y, z, m, id, base_of, screen_slot, radius, n, out,
                                                            rf, smax, hill, mass_f2);
    RG_CUDA_CHECK(cudaGetLastError());
    return 0;
}

int launch_grav_mixed_tiles(const GravArgs& g, const void* split, const int* heavy_end, float near_ratio,
                            int n_chunks, int chunk, double* partial, int n_part, unsigned int* err, bool hold,
                            cudaStream_t st)
{
    if (g.n_tiles <= 0) return 0;
    constexpr int smem = (int)sizeof(MixedSmem);
    // the shared-memory opt-in is a per-device attribute of each kernel: set once per device
    // (setting it again from another thread is harmless)
    static std::atomic<bool> attr_set[64];
    int dev = 0;
    RG_CUDA_CHECK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64 || !attr_set[dev].load(std::memory_order_acquire)) {
        RG_CUDA_CHECK(cudaFuncSetAttribute(grav_mixed_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        RG_CUDA_CHECK(cudaFuncSetAttribute(grav_mixed_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        if (dev >= 0 && dev < 64) attr_set[dev].store(true, std::memory_order_release);
    }
    MixedArgs a;
    a.err = err;
    a.g = g;
    a.sp = (const SplitPos*)split;
    a.heavy_end = heavy_end;
    a.near_ratio = near_ratio;
    a.chunk = n_chunks > 1 ? chunk : (1 << 30);
    a.partial = n_chunks > 1 ? partial : nullptr;
    a.n_part = n_part;
    a.hold = hold ? 1 : 0;
    const dim3 grid(g.n_tiles, n_chunks > 1 ? n_chunks : 1);
    if (g.record || g.hill)
        grav_mixed_kernel<true><<<grid, 256, smem, st>>>(a);
    else
        grav_mixed_kernel<false><<<grid, 256, smem, st>>>(a);
    RG_CUDA_CHECK(cudaGetLastError());
    if (n_chunks > 1) {
        mixed_reduce_kernel<<<g.n_tiles, MX_S, 0, st>>>(partial, n_chunks, n_part, g.tiles, g.n_tiles, g.sys_active,
                                                        g.ax, g.ay, g.az, g.acc_f2);
        RG_CUDA_CHECK(cudaGetLastError());
    }
    return 0;
}

}  // namespace redgb
