// gravity_fp64.cu -- FP64 direct-summation gravity with collision / close-encounter
// screening, bit-identical to the reference's FP64 path.
//
// Reference: kernel_pp_disk::calc_grav_accel (pp_disk.cu:217-296) and its CPU twin
// pp_disk::cpu_calc_grav_accel_SI (pp_disk.cu:404-572).  For every sink i the reference
// adds the source terms m_j (r_j - r_i) / (|r_j - r_i| * |r_j - r_i|^2) one after the
// other in ascending j.  This file is compiled with -fmad=false and keeps that operation
// order, so the accelerations equal the CPU path's bit for bit.
//
// GB300 design.  GB300 retires about two FP64 lanes per SM and clock, so the FP64 pipe
// bounds this file.  The square root and the division of each pair term, about half of its
// FP64 instructions in hardware form, are computed exactly (correctly rounded, the same
// bits) with integer arithmetic on the other pipes (exact_fp64.h); the FP64 pipe keeps the
// 15 subtractions, multiplications and additions.  The serial sum is only 3 FP64 adds per
// pair; the pair terms do not depend on the order.  The pair-parallel
// kernel therefore lets all 256 threads of a CTA compute the S x J pair terms of a tile
// (S sinks x J sources) into shared memory, and 3 S threads then add them in source
// order.  That keeps every SM's FP64 pipe busy however few sinks a block has (3 sinks x
// 1027 sources in the planetesimal disk), which thread-per-sink scheduling cannot.
// The row-serial kernel (thread per sink) serves blocks with few sources per sink
// (planetesimals x 3 massive bodies).  Sources are staged through shared memory in both.
#include <string>

#include "../../include/redgb.h"
#include "common.cuh"
#include "exact_fp64.h"
#include "kernels.h"

namespace redgb {

int set_error(int code, const std::string& msg);

struct PairOut {
    double tx, ty, tz;
};

// One (sink, source) pair: the term added to a_i and the event tests of pp_disk.cu:265
// (radius criterion) and of the mutual Hill sphere (cube form, no cube root).
__device__ __forceinline__ void pair_term(const GravArgs& g, const Tile& tile, int i, int j, double xi, double yi,
                                          double zi, double Ri, double mi, double rhoi, double xj, double yj,
                                          double zj, double mj, double Rj, double rhoj, PairOut& o)
{
    const double dx = xj - xi;
    const double dy = yj - yi;
    const double dz = zj - zi;
    const double r2 = dx * dx + dy * dy + dz * dz;
    const double d = rn_sqrt(r2);         // sqrt.rn, computed on the integer pipes
    const double w = rn_div(mj, d * r2);  // div.rn, likewise (exact_fp64.h)
    o.tx = w * dx;
    o.ty = w * dy;
    o.tz = w * dz;
    const int li = i - tile.base, lj = j - tile.base;
    bool rad = g.record && li > 0 && li > lj && d < tile_f_rad(g, tile) * (Ri + Rj);
    bool hill = false;
    if (g.hill && tile.block != 2 && li > 0 && li > lj && lj > 0) {
        const double h = 0.5 * (rhoi + rhoj);
        const double lhs = d * d * d;
        const double rhs = ((g.hill_f3 * (mi + mj)) / (3.0 * g.mass[tile.base])) * (h * h * h);
        hill = lhs < rhs;
    }
    if (rad || hill) {
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
                e->vi[0] = g.vx[i]; e->vi[1] = g.vy[i]; e->vi[2] = g.vz[i];
                e->vj[0] = g.vx[j]; e->vj[1] = g.vy[j]; e->vj[2] = g.vz[j];
                e->r0[0] = g.px[b0]; e->r0[1] = g.py[b0]; e->r0[2] = g.pz[b0];
                e->v0[0] = g.vx[b0]; e->v0[1] = g.vy[b0]; e->v0[2] = g.vz[b0];
            }
        }
    }
}

// ---------------------------------------------------------------------------------------
// Pair-parallel kernel: CTA = S sinks, source tiles of J = 1024 / S.  ASTRO: the
// astrocentric frame of the reference's CPU path -- each sink starts from the star's pull
// and, for every source it interacts with, adds the direct term and then subtracts the
// source's indirect term (pp_disk.cu:413-454), in source order.
// RG_PAIRPAR_RESIDENT (kernels.h): resident CTAs per SM the register budget is cut for (the
// pair term's integer square root and division hold many values; more resident warps hide
// their latency)

// S sinks x STRIDE threads per CTA, four pair terms per thread and tile (J = 4 STRIDE sources).
// S sets the number of CTAs, ceil(sinks / S): the tuner picks the S whose grid fills the last
// wave of resident CTAs best (16 385 sinks at S = 36: 456 CTAs, exactly three per SM of a
// 152-SM GB300), since every CTA of a block runs the same sources and so takes the same time.
template <int S, int STRIDE, bool ASTRO>
__global__ void __launch_bounds__(S * STRIDE, RG_PAIRPAR_RESIDENT) grav_fp64_pairpar(GravArgs g)
{
    constexpr int NT = S * STRIDE;
    constexpr int JPT = 4;           // terms per thread per tile
    constexpr int J = JPT * STRIDE;  // sources per tile
    constexpr int JA = ASTRO ? J : 1;
    __shared__ double tx[J * S], ty[J * S], tz[J * S];
    __shared__ double sx[J], sy[J], sz[J], sm[J], sR[J], srho[J];
    __shared__ double sind[3][JA];  // ASTRO: the sources' indirect terms
    __shared__ int sid[J];

    const Tile tile = g.tiles[blockIdx.x];
    if (g.sys_active && !g.sys_active[tile.sys]) return;
    const int t = threadIdx.x;
    const int s = t % S;
    const int q0 = t / S;
    const int i = tile.sink_begin + s;
    const bool sink_ok = i < tile.sink_end;
    double xi = 0, yi = 0, zi = 0, Ri = 0, mi = 0, rhoi = 0;
    bool active = false;
    if (sink_ok) {
        xi = g.px[i]; yi = g.py[i]; zi = g.pz[i];
        Ri = g.radius[i]; mi = g.mass[i];
        rhoi = g.hill ? g.rho[i] : 0.0;
        active = 0 < g.id[i];
    }
    const int bc = t / S;  // phase-B component (0, 1, 2) for t < 3 S
    const double* Tb = bc == 0 ? tx : (bc == 1 ? ty : tz);
    double acc = 0.0;
    if (ASTRO && t < 3 * S && sink_ok) acc = g.astro[bc * g.astro_stride + i];

    for (int j0 = tile.src_begin; j0 < tile.src_end; j0 += J) {
        const int nj = min(J, tile.src_end - j0);
        for (int q = t; q < nj; q += NT) {
            const int j = j0 + q;
            sx[q] = g.px[j]; sy[q] = g.py[j]; sz[q] = g.pz[j];
            sm[q] = g.mass[j]; sR[q] = g.radius[j]; sid[q] = g.id[j];
            srho[q] = g.hill ? g.rho[j] : 0.0;
            if (ASTRO) {
                sind[0][q] = g.astro[3 * g.astro_stride + j];
                sind[1][q] = g.astro[4 * g.astro_stride + j];
                sind[2][q] = g.astro[5 * g.astro_stride + j];
            }
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < JPT; k++) {
            const int q = q0 + k * STRIDE;
            const int j = j0 + q;
            PairOut o{0.0, 0.0, 0.0};
            if (active && q < nj && j != i && 0 <= sid[q])
                pair_term(g, tile, i, j, xi, yi, zi, Ri, mi, rhoi, sx[q], sy[q], sz[q], sm[q], sR[q], srho[q], o);
            tx[q * S + s] = o.tx;
            ty[q * S + s] = o.ty;
            tz[q * S + s] = o.tz;
        }
        __syncthreads();
        if (t < 3 * S) {
            if (ASTRO) {
                if (active) {
                    const double* Ib = sind[bc < 3 ? bc : 0];
                    for (int q = 0; q < nj; q++)
                        if (j0 + q != i && 0 <= sid[q]) {
                            acc = acc + Tb[q * S + s];
                            acc = acc - Ib[q];
                        }
                }
            } else {
                for (int q = 0; q < nj; q++) acc = acc + Tb[q * S + s];
            }
        }
        __syncthreads();
    }
    if (t < 3 * S && sink_ok) {
        double* out = bc == 0 ? g.ax : (bc == 1 ? g.ay : g.az);
        out[i] = acc;
    }
}

// ---------------------------------------------------------------------------------------
// Row-serial kernel: one thread per sink, sources staged through shared memory.
__global__ void __launch_bounds__(128) grav_fp64_rowseq(GravArgs g)
{
    constexpr int NT = 128;
    __shared__ double sx[NT], sy[NT], sz[NT], sm[NT], sR[NT], srho[NT];
    __shared__ int sid[NT];
    const Tile tile = g.tiles[blockIdx.x];
    if (g.sys_active && !g.sys_active[tile.sys]) return;
    const int t = threadIdx.x;
    const int i = tile.sink_begin + t;
    const bool sink_ok = i < tile.sink_end;
    double xi = 0, yi = 0, zi = 0, Ri = 0, mi = 0, rhoi = 0;
    bool active = false;
    if (sink_ok) {
        xi = g.px[i]; yi = g.py[i]; zi = g.pz[i];
        Ri = g.radius[i]; mi = g.mass[i];
        rhoi = g.hill ? g.rho[i] : 0.0;
        active = 0 < g.id[i];
    }
    double ax = 0.0, ay = 0.0, az = 0.0;
    for (int j0 = tile.src_begin; j0 < tile.src_end; j0 += NT) {
        const int nj = min(NT, tile.src_end - j0);
        if (t < nj) {
            const int j = j0 + t;
            sx[t] = g.px[j]; sy[t] = g.py[j]; sz[t] = g.pz[j];
            sm[t] = g.mass[j]; sR[t] = g.radius[j]; sid[t] = g.id[j];
            srho[t] = g.hill ? g.rho[j] : 0.0;
        }
        __syncthreads();
        if (active) {
            for (int q = 0; q < nj; q++) {
                const int j = j0 + q;
                if (j == i || 0 > sid[q]) continue;
                PairOut o;
                pair_term(g, tile, i, j, xi, yi, zi, Ri, mi, rhoi, sx[q], sy[q], sz[q], sm[q], sR[q], srho[q], o);
                ax = ax + o.tx;
                ay = ay + o.ty;
                az = az + o.tz;
            }
        }
        __syncthreads();
    }
    if (sink_ok) {
        g.ax[i] = ax;
        g.ay[i] = ay;
        g.az[i] = az;
    }
}

// Distance of every body from its disk's body 0 (the star), for the Hill test:
// sqrt(SQR(x_i - x_0) + SQR(y_i - y_0) + SQR(z_i - z_0)).
__global__ void star_distance(const double* __restrict__ x, const double* __restrict__ y,
                              const double* __restrict__ z, const int* __restrict__ base_of, int n,
                              double* __restrict__ rho)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int b = base_of ? base_of[i] : 0;
    const double dx = x[i] - x[b], dy = y[i] - y[b], dz = z[i] - z[b];
    rho[i] = rn_sqrt(dx * dx + dy * dy + dz * dz);  // sqrt.rn's bits, off the FP64 pipe
}

// ---------------------------------------------------------------------------------------
// Few-sink path: blocks with a handful of sinks and many sources (the star and giants
// of a planetesimal disk).  Kernel A spreads the pair terms of up to FEW_MAX sinks over
// the whole GPU, one thread per source, into a terms buffer (3 x rows x n_src); kernel B
// adds each row in ascending source order -- one thread per (sink, component), which is
// the reference's serial sum -- or, for the mixed-precision kernel's heavy rows, as a
// compensated tree reduction.
constexpr int FEW_MAX = 8;

struct FewArgs {
    GravArgs g;
    const int* tile_row0;  // first row of each tile in the terms buffer
    double* terms;         // 3 x rows x pitch
    int rows;              // rows of the buffer
    long long pitch;       // >= largest source count
};

__global__ void __launch_bounds__(256) grav_fp64_few_terms(FewArgs a)
{
    const GravArgs& g = a.g;
    const Tile tile = g.tiles[blockIdx.y];
    if (g.sys_active && !g.sys_active[tile.sys]) return;
    if ((int)(blockIdx.x * blockDim.x) >= tile.src_end - tile.src_begin) return;
    const int row0 = a.tile_row0[blockIdx.y];
    const int q = blockIdx.x * blockDim.x + threadIdx.x;  // source offset within the tile
    const int j = tile.src_begin + q;
    __shared__ double sx[FEW_MAX], sy[FEW_MAX], sz[FEW_MAX], sR[FEW_MAX], sm[FEW_MAX], srho[FEW_MAX];
    __shared__ int sact[FEW_MAX];
    const int ns = tile.sink_end - tile.sink_begin;
    if (threadIdx.x < ns) {
        const int i = tile.sink_begin + threadIdx.x;
        sx[threadIdx.x] = g.px[i]; sy[threadIdx.x] = g.py[i]; sz[threadIdx.x] = g.pz[i];
        sR[threadIdx.x] = g.radius[i]; sm[threadIdx.x] = g.mass[i];
        srho[threadIdx.x] = g.hill ? g.rho[i] : 0.0;
        sact[threadIdx.x] = 0 < g.id[i];
    }
    __syncthreads();
    if (j >= tile.src_end) return;
    const double xj = g.px[j], yj = g.py[j], zj = g.pz[j], mj = g.mass[j], Rj = g.radius[j];
    const double rhoj = g.hill ? g.rho[j] : 0.0;
    const bool src_ok = 0 <= g.id[j];
    const long long plane = (long long)a.rows * a.pitch;
    for (int s = 0; s < ns; s++) {
        const int i = tile.sink_begin + s;
        PairOut o{0.0, 0.0, 0.0};
        if (sact[s] && src_ok && j != i)
            pair_term(g, tile, i, j, sx[s], sy[s], sz[s], sR[s], sm[s], srho[s], xj, yj, zj, mj, Rj, rhoj, o);
        const long long e = (long long)(row0 + s) * a.pitch + q;
        a.terms[e] = o.tx;
        a.terms[plane + e] = o.ty;
        a.terms[2 * plane + e] = o.tz;
    }
}

struct FewSumArgs {
    const double* terms;
    int rows;         // rows of the whole buffer
    int row0, nrows;  // the rows this launch sums
    long long pitch;
    const int* row_sink;   // sink index of each row
    const int* row_nsrc;   // sources of each row
    const int* row_sys;    // system of each row (ensembles) or nullptr
    const int* sys_active;
    double* ax;
    double* ay;
    double* az;
};

// exact: one warp per (row, component).  The warp streams the row through shared memory
// in coalesced chunks (the next chunk's loads are in flight while the current one is added)
// and adds the terms in ascending source order with the bits of the reference's serial sum:
// warp_serial_sum (exact_fp64.h) takes 32 terms per pass on the integer pipes, where a chain
// of dependent FP64 additions would wait on GB300's FP64 latency for each term.
constexpr int SUM_CHUNK = 256;

__global__ void __launch_bounds__(128) few_sum_serial(FewSumArgs a)
{
    __shared__ double buf[4][2][SUM_CHUNK];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int t = blockIdx.x * 4 + warp;
    if (t >= 3 * a.nrows) return;
    const int comp = t / a.nrows, row = a.row0 + t % a.nrows;
    if (a.sys_active && !a.sys_active[a.row_sys[row]]) return;
    const double* T = a.terms + ((long long)comp * a.rows + row) * a.pitch;
    const int n = a.row_nsrc[row];
    double (*B)[SUM_CHUNK] = buf[warp];
    double reg[SUM_CHUNK / 32];
    auto load = [&](int c0) {
#pragma unroll
        for (int k = 0; k < SUM_CHUNK / 32; k++) {
            const int q = c0 + k * 32 + lane;
            reg[k] = q < n ? T[q] : 0.0;
        }
    };
    double acc = 0.0;
    SerialSumState sst{0, 0};
    int cur = 0;
    load(0);
    for (int c0 = 0; c0 < n; c0 += SUM_CHUNK) {
#pragma unroll
        for (int k = 0; k < SUM_CHUNK / 32; k++) B[cur][k * 32 + lane] = reg[k];
        __syncwarp();
        if (c0 + SUM_CHUNK < n) load(c0 + SUM_CHUNK);
        const int m = min(SUM_CHUNK, n - c0);
        for (int b = 0; b < m; b += 32) {
            const int mb = min(32, m - b);
            acc = warp_serial_sum(acc, &B[cur][b], mb, sst);
        }
        __syncwarp();
        cur ^= 1;
    }
    if (lane == 0) {
        double* out = comp == 0 ? a.ax : (comp == 1 ? a.ay : a.az);
        out[a.row_sink[row]] = acc;
    }
}

// The astrocentric frame's per-body terms (pp_disk.cu:413-420 and 447-454) for bodies
// [1, n): the star's pull on body i, -mu / (r2 sqrt(r2)) r_i with mu = m_star + m_i, and the
// indirect term m_i / (r2 sqrt(r2)) r_i, r2 = |r_i|^2, each component evaluated as the
// reference writes it (division first, then the product).  Body 0 (the star) gets zeros.
__global__ void astro_terms_kernel(const double* __restrict__ x, const double* __restrict__ y,
                                   const double* __restrict__ z, const double* __restrict__ mass, int n,
                                   double m_star, double* __restrict__ out, long long stride)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double sx = 0.0, sy = 0.0, sz = 0.0, ix = 0.0, iy = 0.0, iz = 0.0;
    if (i > 0) {
        const double xi = x[i], yi = y[i], zi = z[i], m = mass[i];
        const double r2 = xi * xi + yi * yi + zi * zi;
        const double den = r2 * rn_sqrt(r2);
        const double mu = m_star + m;
        const double ws = -mu / den;
        const double wi = rn_div(m, den);
        sx = ws * xi; sy = ws * yi; sz = ws * zi;
        ix = wi * xi; iy = wi * yi; iz = wi * zi;
    }
    out[i] = sx;
    out[stride + i] = sy;
    out[2 * stride + i] = sz;
    out[3 * stride + i] = ix;
    out[4 * stride + i] = iy;
    out[5 * stride + i] = iz;
}

// ---------------------------------------------------------------------------------------
// Host launchers
int launch_grav_fp64_pairpar(const GravArgs& g, int S, cudaStream_t st)
{
    if (g.n_tiles <= 0) return 0;
    if (g.astro) {
        switch (S) {
        case 8: grav_fp64_pairpar<8, 32, true><<<g.n_tiles, 256, 0, st>>>(g); break;
        case 16: grav_fp64_pairpar<16, 16, true><<<g.n_tiles, 256, 0, st>>>(g); break;
        case 32: grav_fp64_pairpar<32, 8, true><<<g.n_tiles, 256, 0, st>>>(g); break;
        default: return set_error(RG_ERR_ARG, "pair-parallel sinks per CTA: 8, 16 or 32 in the astrocentric frame");
        }
    } else {
        switch (S) {
        case 8: grav_fp64_pairpar<8, 32, false><<<g.n_tiles, 256, 0, st>>>(g); break;
        case 12: grav_fp64_pairpar<12, 21, false><<<g.n_tiles, 252, 0, st>>>(g); break;
        case 16: grav_fp64_pairpar<16, 16, false><<<g.n_tiles, 256, 0, st>>>(g); break;
        case 18: grav_fp64_pairpar<18, 14, false><<<g.n_tiles, 252, 0, st>>>(g); break;
        case 24: grav_fp64_pairpar<24, 10, false><<<g.n_tiles, 240, 0, st>>>(g); break;
        case 32: grav_fp64_pairpar<32, 8, false><<<g.n_tiles, 256, 0, st>>>(g); break;
        case 36: grav_fp64_pairpar<36, 7, false><<<g.n_tiles, 252, 0, st>>>(g); break;
        default: return set_error(RG_ERR_ARG, "pair-parallel sinks per CTA: 8, 12, 16, 18, 24, 32 or 36");
        }
    }
    RG_CUDA_CHECK(cudaGetLastError());
    return 0;
}

int launch_astro_terms(const double* x, const double* y, const double* z, const double* mass, int n, double m_star,
                       double* out, long long stride, cudaStream_t st)
{
    if (n <= 0) return 0;
    astro_terms_kernel<<<(n + 255) / 256, 256, 0, st>>>(x, y, z, mass, n, m_star, out, stride);
    RG_CUDA_CHECK(cudaGetLastError());
    return 0;
}

int launch_grav_fp64_rowseq(const GravArgs& g, cudaStream_t st)
{
    if (g.n_tiles <= 0) return 0;
    grav_fp64_rowseq<<<g.n_tiles, 128, 0, st>>>(g);
    RG_CUDA_CHECK(cudaGetLastError());
    return 0;
}

// Few-sink tiles (at most FEW_MAX sinks each) -> terms -> exact serial row sums, one launch
// each for all tiles of the group.  Rows are numbered tile by tile; tile_row0 (device) gives
// each tile's first row, max_src bounds the tiles' source counts, and the row arrays
// (dev_row_sink, dev_row_nsrc, dev_row_sys) are on the device.
int launch_grav_fp64_few(const GravArgs& g, const int* tile_row0, int max_src, double* terms, int rows,
                         long long pitch, const int* dev_row_sink, const int* dev_row_nsrc, const int* dev_row_sys,
                         int group_row0, int group_rows, cudaStream_t st)
{
    if (g.n_tiles <= 0 || rows <= 0 || group_rows <= 0 || max_src <= 0) return 0;
    FewArgs a{g, tile_row0, terms, rows, pitch};
    // 256 sources per CTA, or 64 when that would leave most SMs idle (one disk's few heavy rows)
    const int nt = (long long)((max_src + 255) / 256) * g.n_tiles < 2 * NUM_SMS_HINT ? 64 : 256;
    grav_fp64_few_terms<<<dim3((max_src + nt - 1) / nt, g.n_tiles), nt, 0, st>>>(a);
    RG_CUDA_CHECK(cudaGetLastError());
    FewSumArgs b{terms, rows, group_row0, group_rows, pitch, dev_row_sink, dev_row_nsrc, dev_row_sys, g.sys_active,
                 g.ax, g.ay, g.az};
    few_sum_serial<<<(3 * group_rows + 3) / 4, 128, 0, st>>>(b);
    RG_CUDA_CHECK(cudaGetLastError());
    return 0;
}

int launch_star_distance(const double* x, const double* y, const double* z, const int* base_of, int n, double* rho,
                         cudaStream_t st)
{
    if (n <= 0) return 0;
    star_distance<<<(n + 255) / 256, 256, 0, st>>>(x, y, z, base_of, n, rho);
    RG_CUDA_CHECK(cudaGetLastError());
    return 0;
}

}  // namespace redgb
