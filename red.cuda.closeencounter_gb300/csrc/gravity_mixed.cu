// gravity_mixed.cu -- mixed-precision direct-summation gravity for GB300.
//
// Same interaction model and event tests as the FP64 kernel (pp_disk.cu:217-296), but
// the arithmetic is placed on the pipes GB300 has: its FP64 rate is about 1/64 of its
// FP32 rate, so every FP64 operation per pair costs as much as ~64 FP32 operations.
//
//  * Heavy sources (the leading SI bodies: star, giant and rocky planets -- `heavy_end`
//    per tile) contribute the exact FP64 term of the reference (sqrt, divide), summed in
//    FP64.  They dominate every force, so their terms stay at FP64 accuracy.
//  * Every other pair uses the FP64 positions split into FP32 (hi, lo) pairs once per
//    force evaluation (split_positions, O(N) FP64 work).  The displacement is
//    (x_j^hi - x_i^hi) + (x_j^lo - x_i^lo): the hi difference is exact for neighbours
//    (Sterbenz), so the displacement carries the FP64 positions' information down to
//    FP32 resolution of the displacement itself.  1/r comes from the FP32 rsqrt refined
//    by one Newton step, and the terms are summed with compensated (two-sum) FP32
//    accumulators per component.
//  * Near pairs (m_j / r^2 above `near_ratio` times the sink's heavy-source pull) fall
//    back to the FP64 displacement and an FP32 rsqrt seed refined by one FP64 Newton
//    step, summed in FP64: close approaches keep FP64-quality forces.
//  * Event tests (collision radius, Hill sphere) are re-evaluated in FP64 for every pair
//    whose FP32 distance is within a 1e-3 relative margin of a threshold, so the event
//    list is decided in FP64 exactly as in the FP64 kernel.
//
// Work split: a CTA holds 32 sinks x 2 (lane x register) and 8 warps; warp w walks the
// w-th slice of each source tile, so all 256 threads work however few sinks a tile has.
// Sources are staged in shared memory as FP32 (hi, lo) quads; per-warp partial sums are
// combined with two-sum at the end.
#include "common.cuh"
#include "kernels.h"

namespace redgb {

struct SplitPos {
    float4 xy;  // x_hi, x_lo, y_hi, y_lo
    float4 zm;  // z_hi, z_lo, m, (unused)
};

__global__ void split_positions_kernel(const double* __restrict__ x, const double* __restrict__ y,
                                       const double* __restrict__ z, const double* __restrict__ m, int n,
                                       SplitPos* __restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double xd = x[i], yd = y[i], zd = z[i];
    const float xh = (float)xd, yh = (float)yd, zh = (float)zd;
    out[i].xy = make_float4(xh, (float)(xd - (double)xh), yh, (float)(yd - (double)yh));
    out[i].zm = make_float4(zh, (float)(zd - (double)zh), (float)m[i], 0.0f);
}

// compensated accumulation: s + c tracks the exact sum of the added terms to ~2^-46
struct Acc2 {
    float s, c;
};

__device__ __forceinline__ void two_sum_add(Acc2& a, float t)
{
    const float s = a.s + t;
    const float bp = s - a.s;
    const float err = (a.s - (s - bp)) + (t - bp);
    a.s = s;
    a.c += err;
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
};

constexpr int MX_WARPS = 8;
constexpr int MX_R = 2;         // sinks per lane
constexpr int MX_S = 32 * MX_R; // sinks per CTA
static_assert(MX_S == MIXED_SINKS_PER_TILE, "tile size");
static_assert(sizeof(SplitPos) == SPLIT_POS_BYTES, "split size");
constexpr int MX_T = 256;       // sources per shared-memory tile

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
    const bool rad = g.record && li > 0 && li > lj && d < __dmul_rn(g.f_rad, __dadd_rn(Ri, g.radius[j]));
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
        if (slot < eb.cap) {
            DevEvent* e = &eb.rec[slot];
            e->seq = g.seq;
            e->kind = kind;
            e->i = i;
            e->j = j;
            e->sys = tile.sys;
            e->pad = 0;
            e->d = d;
            const int b0 = tile.base;
            e->ri[0] = xi; e->ri[1] = yi; e->ri[2] = zi;
            e->rj[0] = xj; e->rj[1] = yj; e->rj[2] = zj;
            e->vi[0] = g.vx[i]; e->vi[1] = g.vy[i]; e->vi[2] = g.vz[i];
            e->vj[0] = g.vx[j]; e->vj[1] = g.vy[j]; e->vj[2] = g.vz[j];
            e->r0[0] = g.px[b0]; e->r0[1] = g.py[b0]; e->r0[2] = g.pz[b0];
            e->v0[0] = g.vx[b0]; e->v0[1] = g.vy[b0]; e->v0[2] = g.vz[b0];
        }
    }
}

__global__ void __launch_bounds__(256) grav_mixed_kernel(MixedArgs a)
{
    const GravArgs& g = a.g;
    __shared__ float4 s_xy[MX_T];
    __shared__ float4 s_zm[MX_T];
    __shared__ float s_R[MX_T];
    __shared__ float s_rho[MX_T];
    __shared__ int s_id[MX_T];
    __shared__ float s_red[MX_WARPS][6][MX_S];  // per-warp (s, c) x 3 components
    __shared__ double s_redh[MX_WARPS][3][MX_S];

    const Tile tile = g.tiles[blockIdx.x];
    const int heavy_end = a.heavy_end[blockIdx.x];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;

    int si[MX_R];
    bool act[MX_R];
    double xi[MX_R], yi[MX_R], zi[MX_R], Ri[MX_R], mi[MX_R], rhoi[MX_R];
    float xh[MX_R], xl[MX_R], yh[MX_R], yl[MX_R], zh[MX_R], zl[MX_R];
    float Rf[MX_R], rhof[MX_R];
    Acc2 ax[MX_R], ay[MX_R], az[MX_R];
    double hx[MX_R], hy[MX_R], hz[MX_R];
    float heavy_pull[MX_R];
#pragma unroll
    for (int r = 0; r < MX_R; r++) {
        const int i = tile.sink_begin + lane + 32 * r;
        si[r] = i;
        act[r] = false;
        xi[r] = yi[r] = zi[r] = Ri[r] = mi[r] = rhoi[r] = 0.0;
        xh[r] = xl[r] = yh[r] = yl[r] = zh[r] = zl[r] = 0.0f;
        Rf[r] = rhof[r] = 0.0f;
        if (i < tile.sink_end) {
            act[r] = 0 < g.id[i];
            xi[r] = g.px[i]; yi[r] = g.py[i]; zi[r] = g.pz[i];
            Ri[r] = g.radius[i]; mi[r] = g.mass[i];
            rhoi[r] = g.hill ? g.rho[i] : 0.0;
            const SplitPos sp = a.sp[i];
            xh[r] = sp.xy.x; xl[r] = sp.xy.y; yh[r] = sp.xy.z; yl[r] = sp.xy.w;
            zh[r] = sp.zm.x; zl[r] = sp.zm.y;
            Rf[r] = (float)Ri[r];
            rhof[r] = (float)rhoi[r];
        }
        ax[r] = ay[r] = az[r] = Acc2{0.0f, 0.0f};
        hx[r] = hy[r] = hz[r] = 0.0;
        heavy_pull[r] = 0.0f;
    }

    // heavy sources: exact FP64 terms, split over the warps
    for (int j = tile.src_begin + warp; j < heavy_end; j += MX_WARPS) {
        const double xj = g.px[j], yj = g.py[j], zj = g.pz[j], mj = g.mass[j];
        const bool ok = 0 <= g.id[j];
#pragma unroll
        for (int r = 0; r < MX_R; r++) {
            if (!act[r] || !ok || j == si[r]) continue;
            const double dx = xj - xi[r], dy = yj - yi[r], dz = zj - zi[r];
            const double r2 = dx * dx + dy * dy + dz * dz;
            const double d = sqrt(r2);
            const double w = mj / (d * r2);
            hx[r] += w * dx;
            hy[r] += w * dy;
            hz[r] += w * dz;
            heavy_pull[r] = fmaxf(heavy_pull[r], (float)(mj / r2));
            const int li = si[r] - tile.base, lj = j - tile.base;
            if ((g.record && li > 0 && li > lj && d < 1.001 * g.f_rad * (Ri[r] + g.radius[j])) ||
                (g.hill && tile.block != 2 && li > 0 && li > lj && lj > 0))
                exact_event_tests(g, tile, si[r], j, xi[r], yi[r], zi[r], Ri[r], mi[r], rhoi[r]);
        }
    }
    // the near-pair criterion needs the heavy pull of the whole sink: max over warps
    __shared__ float s_pull[MX_WARPS][MX_S];
#pragma unroll
    for (int r = 0; r < MX_R; r++) s_pull[warp][lane + 32 * r] = heavy_pull[r];
    __syncthreads();
    float near_lim[MX_R];
#pragma unroll
    for (int r = 0; r < MX_R; r++) {
        float p = 0.0f;
        for (int w = 0; w < MX_WARPS; w++) p = fmaxf(p, s_pull[w][lane + 32 * r]);
        near_lim[r] = p > 0.0f ? a.near_ratio * p : 3.0e38f;
    }

    const float f_rad = (float)g.f_rad;
    const float margin = 1.001f;
    const bool screen_rad = g.record != 0;
    const bool screen_hill = g.hill != 0 && tile.block != 2;
    const float hill_f3 = (float)g.hill_f3;
    const float inv3M = (float)(1.0 / (3.0 * g.mass[tile.base]));

    for (int j0 = max(heavy_end, tile.src_begin); j0 < tile.src_end; j0 += MX_T) {
        const int nj = min(MX_T, tile.src_end - j0);
        __syncthreads();
        for (int q = threadIdx.x; q < nj; q += blockDim.x) {
            const SplitPos sp = a.sp[j0 + q];
            s_xy[q] = sp.xy;
            s_zm[q] = sp.zm;
            s_R[q] = (float)g.radius[j0 + q];
            s_rho[q] = g.hill ? (float)g.rho[j0 + q] : 0.0f;
            s_id[q] = g.id[j0 + q];
        }
        __syncthreads();
        const int q_begin = warp * (MX_T / MX_WARPS);
        const int q_end = min(nj, q_begin + MX_T / MX_WARPS);
        for (int q = q_begin; q < q_end; q++) {
            const float4 pxy = s_xy[q];
            const float4 pzm = s_zm[q];
            const int idj = s_id[q];
            const int j = j0 + q;
            if (idj < 0) continue;
#pragma unroll
            for (int r = 0; r < MX_R; r++) {
                if (!act[r] || j == si[r]) continue;
                const float dx = (pxy.x - xh[r]) + (pxy.y - xl[r]);
                const float dy = (pxy.z - yh[r]) + (pxy.w - yl[r]);
                const float dz = (pzm.x - zh[r]) + (pzm.y - zl[r]);
                const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                const float mj = pzm.z;
                if (mj > near_lim[r] * r2) {
                    // near pair: FP64 displacement, FP32 rsqrt seed + one FP64 Newton step
                    const double ddx = g.px[j] - xi[r], ddy = g.py[j] - yi[r], ddz = g.pz[j] - zi[r];
                    const double dr2 = ddx * ddx + ddy * ddy + ddz * ddz;
                    const double y0 = (double)rsqrtf((float)dr2);
                    const double y1 = y0 * (1.5 - 0.5 * dr2 * y0 * y0);
                    const double w = g.mass[j] * (y1 * y1 * y1);
                    hx[r] += w * ddx;
                    hy[r] += w * ddy;
                    hz[r] += w * ddz;
                } else {
                    float y = rsqrtf(r2);
                    y = y * fmaf(-0.5f * r2, y * y, 1.5f);
                    const float w = mj * (y * y * y);
                    two_sum_add(ax[r], w * dx);
                    two_sum_add(ay[r], w * dy);
                    two_sum_add(az[r], w * dz);
                }
                // event screens with a relative margin, decided in FP64
                const int li = si[r] - tile.base, lj = j - tile.base;
                if (li > 0 && li > lj) {
                    bool cand = false;
                    if (screen_rad) {
                        const float lim = f_rad * (Rf[r] + s_R[q]) * margin;
                        cand = r2 < lim * lim;
                    }
                    if (screen_hill && lj > 0) {
                        const float h = 0.5f * (rhof[r] + s_rho[q]);
                        const float d3 = r2 * sqrtf(r2);
                        cand = cand || (d3 < hill_f3 * ((float)mi[r] + mj) * inv3M * (h * h * h) * margin * margin * margin);
                    }
                    if (cand) exact_event_tests(g, tile, si[r], j, xi[r], yi[r], zi[r], Ri[r], mi[r], rhoi[r]);
                }
            }
        }
    }
    // combine the warps' partial sums
#pragma unroll
    for (int r = 0; r < MX_R; r++) {
        const int s = lane + 32 * r;
        s_red[warp][0][s] = ax[r].s; s_red[warp][1][s] = ax[r].c;
        s_red[warp][2][s] = ay[r].s; s_red[warp][3][s] = ay[r].c;
        s_red[warp][4][s] = az[r].s; s_red[warp][5][s] = az[r].c;
        s_redh[warp][0][s] = hx[r]; s_redh[warp][1][s] = hy[r]; s_redh[warp][2][s] = hz[r];
    }
    __syncthreads();
    // threads 0..3*MX_S-1: one (sink, component) each
    for (int t = threadIdx.x; t < 3 * MX_S; t += blockDim.x) {
        const int comp = t / MX_S, s = t % MX_S;
        const int i = tile.sink_begin + s;
        if (i >= tile.sink_end) continue;
        Acc2 acc{0.0f, 0.0f};
        double h = 0.0;
        for (int w = 0; w < MX_WARPS; w++) {
            acc = two_sum_merge(acc, Acc2{s_red[w][2 * comp][s], s_red[w][2 * comp + 1][s]});
            h += s_redh[w][comp][s];
        }
        const double v = h + ((double)acc.s + (double)acc.c);
        (comp == 0 ? g.ax : (comp == 1 ? g.ay : g.az))[i] = v;
    }
}

int launch_split_positions(const double* x, const double* y, const double* z, const double* m, int n, SplitPos* out,
                           cudaStream_t st)
{
    if (n <= 0) return 0;
    split_positions_kernel<<<(n + 255) / 256, 256, 0, st>>>(x, y, z, m, n, out);
    RG_CUDA_CHECK(cudaGetLastError());
    return 0;
}

int launch_grav_mixed_tiles(const GravArgs& g, const void* split, const int* heavy_end, float near_ratio,
                            cudaStream_t st)
{
    if (g.n_tiles <= 0) return 0;
    MixedArgs a;
    a.g = g;
    a.sp = (const SplitPos*)split;
    a.heavy_end = heavy_end;
    a.near_ratio = near_ratio;
    grav_mixed_kernel<<<g.n_tiles, 256, 0, st>>>(a);
    RG_CUDA_CHECK(cudaGetLastError());
    return 0;
}

}  // namespace redgb
