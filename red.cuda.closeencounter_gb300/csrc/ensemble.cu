// ensemble.cu -- many independent disks on one GPU, each following the reference's
// RKF7(8) adaptive step (int_rungekutta8.cu:704-797) with its own step size and clock.
//
// Layout: the disks' bodies are concatenated (disk s owns [base_s, base_s + n_s)), with the
// same structure-of-arrays rows as a single context (common.cuh).  Per-disk scalars (clock,
// trial step, status, error maximum, counters) live on the device, so one attempt of every
// running disk is a fixed sequence of launches:
//
//   stage 0 (disks that start a new step) -> Hill-sphere records -> 12 stage combines +
//   force evaluations -> y_{n+1} -> error maximum per disk -> step-size controller (one
//   thread per disk) -> accepted disks copy y_{n+1} into y and screen for ejection /
//   hit-star -> finalize -> event handling (merges, ejections, hit-star, ens_events.cu) ->
//   loop condition.
//
// That sequence is captured once as the body of a CUDA graph's conditional while-node, whose
// last kernel sets the condition, so one graph launch runs attempt after attempt until every
// disk is done (bounded chunks of attempts per launch).  Kernels take per-disk activity
// masks, so finished disks cost nothing but an early exit.  Differences from the single-disk
// path: the controller's pow and the merged radius's pow are the device's (trial steps and
// merged radii may differ from glibc's in the last bit), and inactive bodies are not
// compacted away.
//
// Built with -fmad=false: the stage combinations and the error norm keep the reference's
// operation order.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/redgb.h"
#include "abi_guard.h"
#include "common.cuh"
#include "dfloat.cuh"
#include "ens_events.h"
#include "host_tools.h"
#include "kernels.h"
#include "plan_tools.h"
#include "tma.cuh"
#include "rk_tables.h"
#include "mlp.h"
#include <cuda_bf16.h>

namespace redgb {
int set_error(int code, const std::string& msg);
const void* mlp_device_weights(const rg_mlp* m);
void mlp_normalisation(const rg_mlp* m, float* mean, float* stdev);

// bodies [b0, b1) of disk `sys`; the error norm covers [b0, e1)
struct StageTile {
    int sys, b0, b1, e1;
};

struct EnsStageArgs {
    const StageTile* tiles;
    const int* active;    // per disk
    const double* dt;     // per disk trial step
    const double* y;      // 6 rows
    const double* k[MAXT];
    double c[MAXT];
    int nterm;
    int stride;
    double* out_lo;       // rows 0..2
    double* out_hi;       // rows 3..5
    // y_{n+1} in the mixed form: also the error norm's signed maximum (k[7] = k11, k[8] = k12;
    // the error reads k0 = k[0] and k10 = k[6]), per disk into max_bits; nullptr: none
    unsigned long long* max_bits;
};

// FORM_SUM (stage rows) or FORM_RK8_NP1 (y_{n+1}), one CTA per stage tile, in the
// reference's operation order, y + dt * (c_0 k_0 + c_1 k_1 + ...), without contraction (the
// bit-exact FP64 mode).
template <int FORM, int NTERM>
__device__ __forceinline__ double ens_combine_one(const EnsStageArgs& a, double dt, long long e)
{
    const double y = a.y[e];
    if (FORM == FORM_SUM) {
        double sum = a.c[0] * a.k[0][e];
#pragma unroll
        for (int q = 1; q < NTERM; q++) sum = sum + a.c[q] * a.k[q][e];
        return y + dt * sum;
    }
    return y + dt * (a.c[0] * a.k[0][e] + a.c[1] * a.k[1][e] + a.c[2] * (a.k[2][e] + a.k[3][e]) +
                     a.c[3] * (a.k[4][e] + a.k[5][e]) + a.c[4] * a.k[6][e]);
}

// Rows one after another, two independent elements per thread and iteration (their loads
// and FP64 chains interleave: these kernels are bound by FP64 issue and load latency).
template <int FORM, int NTERM>
__global__ void __launch_bounds__(256) ens_combine_kernel(EnsStageArgs a)
{
    const StageTile t = a.tiles[blockIdx.x];
    if (!a.active[t.sys]) return;
    const double dt = a.dt[t.sys];
    const int nb = t.b1 - t.b0;
    for (int row = 0; row < 6; row++) {
        const long long base = (long long)row * a.stride + t.b0;
        double* out = row < 3 ? a.out_lo + base : a.out_hi + base - 3LL * a.stride;
        for (int i = threadIdx.x; i < nb; i += 2 * blockDim.x) {
            const int i2 = i + blockDim.x;
            const double o1 = ens_combine_one<FORM, NTERM>(a, dt, base + i);
            if (i2 < nb) {
                const double o2 = ens_combine_one<FORM, NTERM>(a, dt, base + i2);
                out[i] = o1;
                out[i2] = o2;
            } else {
                out[i] = o1;
            }
        }
    }
}

// Mixed form with double-float stage vectors (each element of k_q a float2 hi + lo, written
// by the gravity kernels and by these combinations): y + sum_q (dt c_q) k_q with the products
// and the sum in double-float on the FP32 pipes and two FP64 additions per element (the sum
// onto y), where the FP64 form's FMAs kept GB300's FP64 pipe busy; the kernel is then bound
// by HBM.  Stage rows: positions (rows 0-2) as FP64 for the next evaluation, velocities (the
// next stage vector's rows 0-2) as double-float; y_{n+1}: FP64.
__device__ __forceinline__ DF ldf(const double* k, long long e)
{
    const float2 f = __ldg(reinterpret_cast<const float2*>(k) + e);  // read-only for the kernel
    return DF{f.x, f.y};
}

template <int FORM, int NTERM>
__device__ __forceinline__ double ens_combine_df_sum(const DF* w, const DF* k, double y)
{
    DF sum;
    if (FORM == FORM_SUM) {
        sum = df_mul(w[0], k[0]);
#pragma unroll
        for (int q = 1; q < NTERM; q++) sum = df_add(sum, df_mul(w[q], k[q]));
    } else {
        sum = df_mul(w[0], k[0]);
        sum = df_add(sum, df_mul(w[1], k[1]));
        sum = df_add(sum, df_mul(w[2], df_add(k[2], k[3])));
        sum = df_add(sum, df_mul(w[3], df_add(k[4], k[5])));
        sum = df_add(sum, df_mul(w[4], k[6]));
    }
    return y + (f2d_bits(sum.hi) + f2d_bits(sum.lo));
}

template <int FORM, int NTERM>
__global__ void __launch_bounds__(256) ens_combine_df_kernel(EnsStageArgs a)
{
    pdl_wait();  // first: every CTA waits for the kernel before it (launch_stage may overlap them)
    const StageTile t = a.tiles[blockIdx.x];
    if (!a.active[t.sys]) return;
    const double dt = a.dt[t.sys];
    constexpr int NW = FORM == FORM_SUM ? NTERM : 5;  // the coefficients the form reads
    constexpr bool NP1 = FORM == FORM_RK8_NP1;
    constexpr int NL = FORM == FORM_SUM ? NTERM : 9;  // the stage vectors it reads (y_{n+1}: + error)
    // elements per thread and iteration, all their loads issued before any arithmetic (the
    // kernel is bound by memory latency otherwise): 20-40 loaded registers
    constexpr int U = NL <= 4 ? 4 : 2;
    DF w[MAXT];
#pragma unroll
    for (int q = 0; q < NW; q++) w[q] = split_df(dt * a.c[q]);
    const int nb = t.b1 - t.b0;
    const int ne = t.e1 - t.b0;  // y_{n+1}: the elements the error norm covers
    DF mdf{0.0f, 0.0f};          // the error's running maximum (normalised double-float)
    for (int row = 0; row < 6; row++) {
        const long long base = (long long)row * a.stride + t.b0;
        const bool f2 = FORM == FORM_SUM && row >= 3;  // the next stage vector's velocity rows
        double* out = row < 3 ? a.out_lo + base : a.out_hi + base - 3LL * a.stride;
        for (int i = threadIdx.x; i < nb; i += U * blockDim.x) {
            DF kv[U][NL];
            double yv[U];
#pragma unroll
            for (int u = 0; u < U; u++) {
                const int iu = min(i + u * (int)blockDim.x, nb - 1);  // in range; excess lanes repeat the last
                yv[u] = __ldg(a.y + base + iu);
#pragma unroll
                for (int q = 0; q < NL; q++) kv[u][q] = ldf(a.k[q], base + iu);
            }
#pragma unroll
            for (int u = 0; u < U; u++) {
                const int iu = i + u * blockDim.x;
                if (iu < nb) {
                    const double o = ens_combine_df_sum<FORM, NTERM>(w, kv[u], yv[u]);
                    if (f2)
                        reinterpret_cast<float2*>(out)[iu] = to_f2(o);
                    else
                        out[iu] = o;

                    if (NP1 && iu < ne) {  // e = ((k0 + k10) - k11) - k12 (integrator.cu:240-255)
                        const DF d = df_add(df_add(df_add(kv[u][0], kv[u][6]), DF{-kv[u][7].hi, -kv[u][7].lo}),
                                            DF{-kv[u][8].hi, -kv[u][8].lo});
                        if (mdf.hi < d.hi || (mdf.hi == d.hi && mdf.lo < d.lo)) mdf = d;
                    }
                }
            }
        }
    }
    if (NP1) {  // the CTA's signed maximum (starting at 0) into the disk's word
        double m = f2d_bits(mdf.hi) + f2d_bits(mdf.lo);  // rounding is monotone
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            const double o = __shfl_xor_sync(0xffffffffu, m, off);
            if (m < o) m = o;
        }
        __shared__ double wmax[8];
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        if (lane == 0) wmax[warp] = m;
        __syncthreads();
        if (warp == 0) {
            m = lane < (int)(blockDim.x >> 5) ? wmax[lane] : 0.0;
#pragma unroll
            for (int off = 4; off > 0; off >>= 1) {
                const double o = __shfl_xor_sync(0xffffffffu, m, off);
                if (m < o) m = o;
            }
            if (lane == 0 && m > 0.0) atomicMax(&a.max_bits[t.sys], (unsigned long long)__double_as_longlong(m));
        }
    }
}

// rows [r0, r0 + nr) of FP64 src -> double-float rows [d0, d0 + nr) of dst, for disks whose
// mask is set (the step start's velocities into the first stage vector, mixed form)
__global__ void ens_copy_to_f2_kernel(const StageTile* tiles, const int* mask, const double* src, int r0, double* dst,
                                      int d0, int nr, int stride)
{
    const StageTile t = tiles[blockIdx.x];
    if (!mask[t.sys]) return;
    const int nb = t.b1 - t.b0;
    for (int f = threadIdx.x; f < nr * nb; f += blockDim.x) {
        const int r = f / nb, i = t.b0 + f - r * nb;
        reinterpret_cast<float2*>(dst + (long long)(d0 + r) * stride)[i] = to_f2(src[(long long)(r0 + r) * stride + i]);
    }
}

// the stage vectors' storage between FP64 and double-float pairs, in place (n elements)
__global__ void k_format_kernel(double* k, long long n, int to_f2_pairs)
{
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        if (to_f2_pairs)
            reinterpret_cast<float2*>(k)[e] = to_f2(k[e]);
        else
            k[e] = f2_to_double(reinterpret_cast<const float2*>(k)[e]);
    }
}

// rows [r0, r0 + nr) of src -> rows [d0, d0 + nr) of dst, for disks whose mask is set
__global__ void ens_copy_kernel(const StageTile* tiles, const int* mask, const double* src, int r0, double* dst,
                                int d0, int nr, int stride)
{
    const StageTile t = tiles[blockIdx.x];
    if (!mask[t.sys]) return;
    const int nb = t.b1 - t.b0;
    // four elements per thread and iteration, loads first (the copy is bound by memory latency)
    constexpr int U = 4;
    for (int f0 = threadIdx.x; f0 < nr * nb; f0 += U * blockDim.x) {
        double v[U];
        long long o[U];
        int row[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int f = min(f0 + u * (int)blockDim.x, nr * nb - 1);
            row[u] = f / nb;
            o[u] = (long long)t.b0 + (f - row[u] * nb);
            v[u] = __ldg(src + (long long)(r0 + row[u]) * stride + o[u]);
        }
#pragma unroll
        for (int u = 0; u < U; u++)
            if (f0 + u * (int)blockDim.x < nr * nb) dst[(long long)(d0 + row[u]) * stride + o[u]] = v[u];
    }
}

// e = ((k0 + k10) - k11) - k12, signed maximum starting at 0 (integrator.cu:240-255)
__global__ void __launch_bounds__(256) ens_error_kernel(const StageTile* tiles, const int* active, const double* k0,
                                                        const double* k10, const double* k11, const double* k12,
                                                        int stride, unsigned long long* max_bits)
{
    const StageTile t = tiles[blockIdx.x];
    if (!active[t.sys]) return;
    const int nb = t.e1 - t.b0;
    double m = 0.0;
    for (int f = threadIdx.x; f < 6 * nb; f += blockDim.x) {
        const int row = f / nb;
        const long long e = (long long)row * stride + t.b0 + (f - row * nb);
        const double v = (k0[e] + k10[e] - k11[e] - k12[e]);
        if (m < v) m = v;
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const double o = __shfl_xor_sync(0xffffffffu, m, off);
        if (m < o) m = o;
    }
    __shared__ double wmax[8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) wmax[warp] = m;
    __syncthreads();
    if (warp == 0) {
        m = lane < (int)(blockDim.x >> 5) ? wmax[lane] : 0.0;
#pragma unroll
        for (int off = 4; off > 0; off >>= 1) {
            const double o = __shfl_xor_sync(0xffffffffu, m, off);
            if (m < o) m = o;
        }
        if (lane == 0 && m > 0.0) atomicMax(&max_bits[t.sys], (unsigned long long)__double_as_longlong(m));
    }
}

struct EnsSys {
    int n;
    int* status;
    int* active;
    int* active_f0;
    int* acc;
    int* ej;
    unsigned int* events;
    unsigned long long* max_bits;
    double* t;
    double* t_prev;
    double* t_stop;
    double* dt_try;
    double* dt_did;
    long long* n_tried;
    long long* n_passed;
    long long* n_failed;
    unsigned int* attempt;   // per disk: attempts so far (event records carry it)
    unsigned int* acc_attempt;
    unsigned int* n_f0;      // per disk: step-start force evaluations so far
    double tol;
    rg_step_rec_t* log;      // attempt log (nullptr: off)
    unsigned int* log_count;
    unsigned int log_cap;
    // learned proposer: per-disk history and features
    float* feat;             // n x 8, features of the current step
    double* dt_last;         // last accepted step
    double* ideal_last;      // the error model's ideal step for the last accepted step
    float* hist;             // n x 5: err_last, acc_last, ir0, ir1, ir2 (log ideal-step ratios)
    int* proposed;           // the current attempt's step came from the network
    int* step_prop_rej;      // a proposal of the current step was rejected
    int* prop_rej_steps;     // consecutive steps with a rejected proposal
    int* cool;               // steps left on the plain controller
    long long* n_prop;
    long long* n_prop_acc;
    long long* n_fallback;
    int cooldown;
    float dither;                    // > 0: plain trial steps scaled by exp(dither * U[-1, 1))
    unsigned long long dither_seed;
};

// the controller of rungekutta8::step, one thread per disk
__global__ void ens_controller_kernel(EnsSys s)
{
    const int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= s.n) return;
    if (!s.active[d]) {
        s.acc[d] = 0;
        return;
    }
    const double raw = __longlong_as_double((long long)s.max_bits[d]);
    const double dt = s.dt_try[d];
    const double max_err = fabs(dt * (41.0 / 840.0) * raw);
    const double new_dt = dt * (0.9 * pow(s.tol / max_err, 1.0 / 8.0));
    const bool accepted = !(max_err > s.tol);
    const int proposed = s.proposed[d];
    if (s.log) {
        const unsigned int slot = atomicAdd(s.log_count, 1u);
        if (slot < s.log_cap) {
            rg_step_rec_t& rec = s.log[slot];
            rec.sys = d;
            rec.accepted = accepted;
            rec.proposed = proposed;
            rec.step = (int)s.n_passed[d];
            rec.dt = dt;
            rec.err = max_err;
            for (int q = 0; q < 8; q++) rec.feat[q] = s.feat[8 * d + q];
        }
    }
    s.n_tried[d]++;
    float* h = s.hist + 5 * d;
    h[0] = (float)log10(max_err / s.tol);
    h[1] = accepted ? 1.0f : 0.0f;
    if (proposed) {
        s.n_prop[d]++;
        if (accepted) s.n_prop_acc[d]++;
        else s.step_prop_rej[d] = 1;
    }
    s.proposed[d] = 0;
    if (accepted) {
        s.t_prev[d] = s.t[d];
        s.t[d] = s.t[d] + dt;
        s.dt_did[d] = dt;
        s.n_passed[d]++;
        s.acc[d] = 1;
        s.acc_attempt[d] = s.attempt[d];
        // the step that would have met the tolerance exactly (the error scales as dt^8)
        const double ideal = max_err > 0.0 ? dt * pow(s.tol / max_err, 1.0 / 8.0) : 8.0 * dt;
        const double last = s.ideal_last[d];
        h[4] = h[3];
        h[3] = h[2];
        h[2] = last > 0.0 && isfinite(ideal) ? fminf(fmaxf((float)log(ideal / last), -3.0f), 3.0f) : 0.0f;
        s.dt_last[d] = dt;
        if (isfinite(ideal)) s.ideal_last[d] = ideal;
        // fallback: two steps in a row whose proposals were rejected
        if (s.step_prop_rej[d]) {
            if (++s.prop_rej_steps[d] >= 2) {
                s.cool[d] = s.cooldown;
                s.prop_rej_steps[d] = 0;
                s.n_fallback[d]++;
            }
        } else if (proposed) {
            s.prop_rej_steps[d] = 0;
        }
        s.step_prop_rej[d] = 0;
        if (s.cool[d] > 0) s.cool[d]--;
    } else {
        s.n_failed[d]++;
        s.acc[d] = 0;
    }
    s.dt_try[d] = new_dt;
}

// ejection / hit-star screen of the accepted disks' new states (kernel_pp_disk::
// check_for_ejection_hit_centrum, pp_disk.cu:72-142); the host applies the handlers
__global__ void ens_eject_screen_kernel(const StageTile* tiles, const int* mask, const double* y, int stride,
                                        const int* id, const int* type, const double* thr, int* ej)
{
    const StageTile t = tiles[blockIdx.x];
    if (!mask[t.sys]) return;
    const double* th = thr + 5 * t.sys;
    if (!(0.0 < th[0]) && !(0.0 < th[1])) return;
    for (int i = t.b0 + threadIdx.x; i < t.b1; i += blockDim.x) {
        if (!(0 < id[i] && type[i] != 0)) continue;
        const double x = y[i], yy = y[stride + i], z = y[2LL * stride + i];
        const double r2 = x * x + yy * yy + z * z;
        if ((0.0 < th[1] && th[4] < r2) || (0.0 < th[0] && th[3] > r2)) ej[t.sys] = 1;
    }
}

__global__ void ens_finalize_kernel(EnsSys s)
{
    const int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= s.n) return;
    if (s.active_f0[d]) s.n_f0[d]++;
    if (s.active[d]) {
        s.attempt[d]++;
        if (s.acc[d]) {
            if (s.events[d] > 0 || s.ej[d])
                s.status[d] = RG_SYS_HELD;
            else if (!(s.t[d] <= s.t_stop[d]))
                s.status[d] = RG_SYS_DONE;
        }
        if (s.status[d] == RG_SYS_RUNNING && (!isfinite(s.dt_try[d]) || s.dt_try[d] == 0.0))
            s.status[d] = RG_SYS_ERROR;
    }
    const int run = s.status[d] == RG_SYS_RUNNING;
    s.active_f0[d] = run && (s.acc[d] || !s.active[d]);
    s.active[d] = run;
    s.events[d] = 0;
    s.ej[d] = 0;
    s.max_bits[d] = 0ull;
}

// features of a step start: max |a| and min (d / mutual Hill radius)^3 over the pairs of
// every body with a massive non-star self-interacting body, in FP32 (the features are
// logarithms fed to an FP32 network).  FP64 values become FP32 on their bit patterns
// (split_bits, integer operations): a hardware conversion runs on GB300's FP64 pipe.
constexpr int FEAT_MAX_SI = 16;  // self-interacting bodies per disk staged in shared memory
constexpr unsigned int FEAT_H3_NONE_BITS = 0x7f61b1e6u;  // 3e38f: no pair seen

__device__ __forceinline__ float to_f32(double v)
{
    float hi, lo;
    split_bits(v, hi, lo);
    return hi;
}

// the accepted disks' y_{n+1} into y (6 rows), with the ejection / hit-star screen of the new
// positions (ens_eject_screen_kernel's tests) taken on the way: r^2 in FP32 from the
// coordinates' leading parts first (relative error below 1e-6), the reference's FP64 test only
// where that lies within 1e-5 of a threshold -- so the screen costs no FP64 work for bodies
// far from both
__global__ void ens_accept_kernel(const StageTile* tiles, const int* acc, const double* __restrict__ src,
                                  double* __restrict__ dst, int stride, const int* id, const int* type,
                                  const double* thr, int* ej)
{
    const StageTile t = tiles[blockIdx.x];
    if (!acc[t.sys]) return;
    const double* th = thr + 5 * t.sys;
    const bool hit_on = 0.0 < th[0], ej_on = 0.0 < th[1];
    const float hit_f = hit_on ? to_f32(th[3]) * (1.0f + 1e-5f) : 0.0f;
    const float ej_f = ej_on ? to_f32(th[4]) * (1.0f - 1e-5f) : 0.0f;
    // two bodies per thread and iteration, their six rows' loads first (memory latency)
    constexpr int U = 2;
    bool hit = false;
    for (int i0 = t.b0 + threadIdx.x; i0 < t.b1; i0 += U * blockDim.x) {
        double v[U][6];
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int i = min(i0 + u * (int)blockDim.x, t.b1 - 1);
#pragma unroll
            for (int r = 0; r < 6; r++) v[u][r] = __ldg(src + (long long)r * stride + i);
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int i = i0 + u * (int)blockDim.x;
            if (i >= t.b1) continue;
#pragma unroll
            for (int r = 0; r < 6; r++) dst[(long long)r * stride + i] = v[u][r];
            if (!(hit_on || ej_on) || !(0 < id[i] && type[i] != 0)) continue;
            const float xf = to_f32(v[u][0]), yf = to_f32(v[u][1]), zf = to_f32(v[u][2]);
            const float r2f = xf * xf + yf * yf + zf * zf;
            if (!((ej_on && !(r2f < ej_f)) || (hit_on && !(r2f > hit_f)))) continue;
            const double x = v[u][0], yy = v[u][1], z = v[u][2];
            const double r2 = x * x + yy * yy + z * z;  // pp_disk.cu:72-142, in FP64
            if ((ej_on && th[4] < r2) || (hit_on && th[3] > r2)) hit = true;
        }
    }
    if (hit) ej[t.sys] = 1;
}

// one body's contribution; si: the disk's first FEAT_MAX_SI SI bodies (positions relative to
// body 0, masses, distance from body 0) in shared memory, ns of them in all (the rest are read
// from the state rows), M = body 0's mass.  The body's values are loaded before any test, so
// that the loads of consecutive bodies overlap.
__device__ __forceinline__ void body_features(const double* y, const double* k0, bool k_f2, const double* mass,
                                              const int* id, long long stride, int b, int ns, const float4* si,
                                              const float* si_r, float x0, float y0, float z0, float M, int i,
                                              float& am, float& h3)
{
    const int idi = id[i];
    // the step start's acceleration: FP64, or a double-float pair (the mixed form) whose
    // leading float is all a feature needs
    const double kx = k0[3LL * stride + i], ky = k0[4LL * stride + i], kz = k0[5LL * stride + i];
    const double px = y[i], py = y[stride + i], pz = y[2LL * stride + i];
    const double pm = mass[i];
    if (idi <= 0) return;
    float ax, ay, az;
    if (k_f2) {
        ax = __uint_as_float((unsigned)__double_as_longlong(kx));  // the pair's first float
        ay = __uint_as_float((unsigned)__double_as_longlong(ky));
        az = __uint_as_float((unsigned)__double_as_longlong(kz));
    } else {
        ax = to_f32(kx);
        ay = to_f32(ky);
        az = to_f32(kz);
    }
    am = fmaxf(am, sqrtf(ax * ax + ay * ay + az * az));
    const float xi = to_f32(px) - x0, yi = to_f32(py) - y0, zi = to_f32(pz) - z0;
    const float ri = sqrtf(xi * xi + yi * yi + zi * zi);
    const float mi = to_f32(pm);
    const float inv3M = 1.0f / (3.0f * M);
    for (int q = 1; q < ns; q++) {
        const int j = b + q;
        float4 sj;
        float rj;
        if (q < FEAT_MAX_SI) {
            sj = si[q];
            rj = si_r[q];
        } else {
            sj = make_float4(to_f32(y[j]) - x0, to_f32(y[stride + j]) - y0, to_f32(y[2LL * stride + j]) - z0,
                             id[j] > 0 ? to_f32(mass[j]) : -1.0f);
            rj = sqrtf(sj.x * sj.x + sj.y * sj.y + sj.z * sj.z);
        }
        if (j == i || !(sj.w >= 0.0f)) continue;  // inactive SI bodies carry w = -1
        const float dx = sj.x - xi, dy = sj.y - yi, dz = sj.z - zi;
        const float d2 = dx * dx + dy * dy + dz * dz;
        const float hh = 0.5f * (ri + rj);
        const float rh3 = (mi + sj.w) * inv3M * hh * hh * hh;
        if (rh3 > 0.0f) h3 = fminf(h3, d2 * sqrtf(d2) / rh3);
    }
}

struct PropArgs {
    EnsSys s;
    int k_f2;  // the stage vectors are double-float pairs (the mixed form)
    const StageTile* tiles;  // the stage tiles (a disk's tiles are consecutive)
    const int* tiles_of;     // per disk: its stage tiles
    unsigned int* red;       // per disk: max |a| bits, min h3 bits, tiles done (reset by the last)
    const double* y;
    const double* k0;
    const double* mass;
    const int* id;
    const int* base;  // per disk: body 0
    const int* nsi;   // per disk: self-interacting bodies
    const int* ntot;  // per disk: bodies
    long long stride;
    const __nv_bfloat16* w;  // nullptr: features only
    float mean[8], inv_std[8];
    float safety;
};

// uniform in [-1, 1) from (seed, disk, step): splitmix64 finaliser
__device__ __forceinline__ double dither_uniform(unsigned long long seed, int d, long long step)
{
    unsigned long long z = seed + 0x9E3779B97F4A7C15ull * (((unsigned long long)(unsigned)d << 40) ^ (unsigned long long)step);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (double)(z >> 11) * (2.0 / 9007199254740992.0) - 1.0;
}

// one CTA per stage tile of the disks that start a step: the tile's feature partials (max |a|,
// min (d / mutual Hill radius)^3) go to the disk's slots by atomics; the disk's last tile to
// finish (a ticket per disk, no waiting) takes the disk's features, resets the slots for the
// next launch, and in its first warp evaluates the network and sets the trial step.  That CTA
// stages the network's weights in shared memory first (as float, W2 transposed so that the
// lanes of a warp read consecutive words).
constexpr int PROP_THREADS = 256;

__global__ void __launch_bounds__(PROP_THREADS) ens_propose_kernel(PropArgs a)
{
    const StageTile tile = a.tiles[blockIdx.x];
    const int d = tile.sys;
    const EnsSys& s = a.s;
    if (!s.active_f0[d]) return;  // uniform over the CTA
    __shared__ float red_am[PROP_THREADS / 32], red_h3[PROP_THREADS / 32];
    __shared__ float4 si[FEAT_MAX_SI];
    __shared__ float si_r[FEAT_MAX_SI];
    __shared__ float sw1[MLP_HIDDEN * MLP_IN], sb1[MLP_HIDDEN], sw2t[MLP_HIDDEN * MLP_HIDDEN], sb2[MLP_HIDDEN],
        sw3[MLP_HIDDEN];
    __shared__ int last_sh;
    __shared__ float feat_sh[2];
    float am = 0.0f, h3 = 3.0e38f;
    {
        const int b = a.base[d], ns = a.nsi[d];
        const float x0 = to_f32(a.y[b]), y0 = to_f32(a.y[a.stride + b]), z0 = to_f32(a.y[2LL * a.stride + b]);
        const float M = to_f32(a.mass[b]);
        if ((int)threadIdx.x < min(ns, FEAT_MAX_SI)) {
            const int j = b + threadIdx.x;
            const float xj = to_f32(a.y[j]) - x0, yj = to_f32(a.y[a.stride + j]) - y0, zj = to_f32(a.y[2LL * a.stride + j]) - z0;
            si[threadIdx.x] = make_float4(xj, yj, zj, a.id[j] > 0 ? to_f32(a.mass[j]) : -1.0f);
            si_r[threadIdx.x] = sqrtf(xj * xj + yj * yj + zj * zj);
        }
        __syncthreads();
#pragma unroll 2
        for (int i = tile.b0 + threadIdx.x; i < tile.b1; i += blockDim.x)
            body_features(a.y, a.k0, a.k_f2 != 0, a.mass, a.id, a.stride, b, ns, si, si_r, x0, y0, z0, M, i, am, h3);
        for (int off = 16; off > 0; off >>= 1) {
            am = fmaxf(am, __shfl_xor_sync(0xffffffffu, am, off));
            h3 = fminf(h3, __shfl_xor_sync(0xffffffffu, h3, off));
        }
        if ((threadIdx.x & 31) == 0) {
            red_am[threadIdx.x >> 5] = am;
            red_h3[threadIdx.x >> 5] = h3;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            for (int w = 1; w < PROP_THREADS / 32; w++) {
                am = fmaxf(am, red_am[w]);
                h3 = fminf(h3, red_h3[w]);
            }
            // non-negative floats order as their bit patterns
            unsigned int* r = a.red + 3 * d;
            atomicMax(r, __float_as_uint(am));
            atomicMin(r + 1, __float_as_uint(h3));
            __threadfence();
            const unsigned int done = atomicAdd(r + 2, 1u);
            last_sh = done + 1 == (unsigned int)a.tiles_of[d];
            if (last_sh) {
                __threadfence();
                feat_sh[0] = __uint_as_float(atomicExch(r, 0u));
                feat_sh[1] = __uint_as_float(atomicExch(r + 1, FEAT_H3_NONE_BITS));
                atomicExch(r + 2, 0u);
            }
        }
        __syncthreads();
        if (!last_sh) return;
        am = feat_sh[0];
        h3 = feat_sh[1];
    }
    const bool use_net = a.w && !(s.cool[d] > 0 || s.n_passed[d] < 4 || !(s.ideal_last[d] > 0.0));
    if (use_net) {
        for (int k = threadIdx.x; k < MLP_HIDDEN * MLP_HIDDEN; k += blockDim.x) {
            const int u = k / MLP_HIDDEN, v = k % MLP_HIDDEN;  // W2[u][v] -> sw2t[v][u]
            sw2t[v * MLP_HIDDEN + u] = __bfloat162float(a.w[MLP_OFF_W2 + k]);
        }
        for (int k = threadIdx.x; k < MLP_HIDDEN * MLP_IN; k += blockDim.x)
            sw1[k] = __bfloat162float(a.w[MLP_OFF_W1 + k]);
        for (int k = threadIdx.x; k < MLP_HIDDEN; k += blockDim.x) {
            sb1[k] = __bfloat162float(a.w[MLP_OFF_B1 + k]);
            sb2[k] = __bfloat162float(a.w[MLP_OFF_B2 + k]);
            sw3[k] = __bfloat162float(a.w[MLP_OFF_W3 + k]);
        }
        __syncthreads();
    }
    if (threadIdx.x >= 32) return;
    const int lane = threadIdx.x & 31;
    const float* h = s.hist + 5 * d;
    float f[8];
    f[0] = h3 < 1.0e38f ? log10f(fmaxf(h3, 1e-30f)) / 3.0f : 6.0f;
    f[1] = log10f(fmaxf(am, 1e-30f));
    f[2] = s.dt_last[d] > 0.0 ? log10f(to_f32(s.dt_last[d]) * (1.0f / 1.720209895e-2f)) : -3.0f;
    f[3] = h[0];
    f[4] = h[1];
    f[5] = h[2];
    f[6] = h[3];
    f[7] = h[4];
    if (lane < 8) s.feat[8 * d + lane] = f[lane];
    if (!use_net) {
        if (lane == 0 && s.dither > 0.0f)
            s.dt_try[d] *= exp((double)s.dither * dither_uniform(s.dither_seed, d, s.n_passed[d]));
        return;
    }
    float x[8];
#pragma unroll
    for (int q = 0; q < 8; q++) x[q] = fminf(fmaxf((f[q] - a.mean[q]) * a.inv_std[q], -6.0f), 6.0f);
    // hidden layer 1: lane owns units lane and lane + 32
    float h1[2];
#pragma unroll
    for (int r = 0; r < 2; r++) {
        const int u = lane + 32 * r;
        float z = sb1[u];
#pragma unroll
        for (int q = 0; q < 8; q++) z = fmaf(sw1[u * 8 + q], x[q], z);
        h1[r] = z / (1.0f + __expf(-z));
    }
    float h2[2];
#pragma unroll
    for (int r = 0; r < 2; r++) {
        const int u = lane + 32 * r;
        float z = sb2[u];
#pragma unroll 16
        for (int v = 0; v < 64; v++) {
            const float hv = __shfl_sync(0xffffffffu, h1[v >> 5], v & 31);
            z = fmaf(sw2t[v * MLP_HIDDEN + u], hv, z);
        }
        h2[r] = z / (1.0f + __expf(-z));
    }
    float o = sw3[lane] * h2[0] + sw3[lane + 32] * h2[1];
    for (int off = 16; off > 0; off >>= 1) o += __shfl_xor_sync(0xffffffffu, o, off);
    o += __bfloat162float(a.w[MLP_OFF_B3]);
    if (lane == 0 && isfinite(o)) {
        // the network predicts log(ideal step / last ideal step); the plain controller bounds
        // the proposal to [1/2, 2] of its own estimate
        const double plain = s.dt_try[d];
        double dt = (double)a.safety * s.ideal_last[d] * (double)expf(o);
        dt = fmin(fmax(dt, 0.5 * plain), 2.0 * plain);
        if (isfinite(dt) && dt > 0.0) {
            s.dt_try[d] = dt;
            s.proposed[d] = 1;
        }
    }
}

// per-body energy partials of an ensemble (as energy_kernel, with disk offsets)
__global__ void ens_energy_kernel(const double* y, const double* mass, const int* id, int stride, int base, int n,
                                  int n_si, int n_massive, double* part)
{
    const int li = blockIdx.x * blockDim.x + threadIdx.x;
    if (li >= n) return;
    const int i = base + li;
    const long long sd = stride;
    const double *rx = y, *ry = y + sd, *rz = y + 2 * sd, *vx = y + 3 * sd, *vy = y + 4 * sd, *vz = y + 5 * sd;
    double T = 0, U = 0, Uc = 0, Lx = 0, Ly = 0, Lz = 0;
    if (id[i] > 0) {
        const double m = mass[i];
        T = 0.5 * m * (vx[i] * vx[i] + vy[i] * vy[i] + vz[i] * vz[i]);
        Lx = m * (ry[i] * vz[i] - rz[i] * vy[i]);
        Ly = m * (rz[i] * vx[i] - rx[i] * vz[i]);
        Lz = m * (rx[i] * vy[i] - ry[i] * vx[i]);
        if (li >= 1 && li < n_massive) {
            const int jmax = li < n_si ? li : n_si;
            for (int lj = 0; lj < jmax; lj++) {
                const int j = base + lj;
                if (id[j] <= 0) continue;
                const double dx = rx[j] - rx[i], dy = ry[j] - ry[i], dz = rz[j] - rz[i];
                const double d = sqrt(dx * dx + dy * dy + dz * dz);
                const double term = -(m * mass[j]) / d;
                const double tt = U + term;
                if (fabs(U) >= fabs(term))
                    Uc += (U - tt) + term;
                else
                    Uc += (term - tt) + U;
                U = tt;
            }
        }
    }
    part[li] = T;
    part[n + li] = U + Uc;
    part[2 * n + li] = Lx;
    part[3 * n + li] = Ly;
    part[4 * n + li] = Lz;
}

}  // namespace redgb

using namespace redgb;

// ============================================================================ host side
struct rg_ens {
    int n_sys = 0;
    int cap = 0;
    int device = 0, n_sm = 152;
    // gravity launch shapes (rg_ens_autotune): row-kernel source limit, sinks per FP64
    // pair-parallel CTA, sources per few-sink CTA (0: automatic)
    int rowseq_max_src = 64, pairpar_S = 16, few_chunk = 0;
    std::vector<int> base, ntot;
    std::vector<std::array<int, 7>> cnt;
    std::vector<rg_param_t> p;
    std::vector<rg_body_metadata_t> md;
    std::vector<double> thr;  // 5 per disk
    cudaStream_t st = nullptr;
    // the row kernels of an evaluation (planetesimals against the star and giants) run on a
    // side stream beside the other groups: forked after the split, joined before the combine
    cudaStream_t st2 = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    // device, per body
    double* d_y = nullptr;
    double* d_yout = nullptr;
    double* d_k[13] = {};
    int k_f2_now = 0;  // the first stage vector (kept across a rejected attempt) holds double-float pairs
    double* d_P = nullptr;
    double* d_mass = nullptr;
    double* d_radius = nullptr;
    double* d_rho = nullptr;
    int* d_id = nullptr;
    int* d_type = nullptr;
    void* d_split = nullptr;
    float* d_rf = nullptr;  // FP32 radii of the mixed kernels' event screens
    float2* d_mass_f2 = nullptr;  // the split masses (the symmetric kernel's later stages)
    unsigned int* d_smax = nullptr;  // the screens' maxima per disk (split_positions)
    int* d_screen_slot = nullptr;    // per body: its disk for a light body, -1 for a heavy one
    std::vector<int> screen_slot;
    double* d_partial = nullptr;
    size_t partial_cap = 0;
    double* d_thr = nullptr;
    // device, per disk
    int *d_status = nullptr, *d_active = nullptr, *d_active_f0 = nullptr, *d_acc = nullptr, *d_ej = nullptr;
    unsigned int* d_sys_events = nullptr;
    unsigned long long* d_maxbits = nullptr;
    double *d_t = nullptr, *d_tprev = nullptr, *d_tstop = nullptr, *d_dt_try = nullptr, *d_dt_did = nullptr;
    long long *d_ntried = nullptr, *d_npassed = nullptr, *d_nfailed = nullptr;
    unsigned int *d_attempt = nullptr, *d_acc_attempt = nullptr, *d_nf0 = nullptr;
    // stage tiles
    std::vector<StageTile> stiles;
    StageTile* d_stiles = nullptr;
    std::vector<int> tiles_of;      // per disk: its stage tiles
    int* d_tiles_of = nullptr;
    unsigned int* d_feat_red = nullptr;  // per disk: max |a| bits, min h3 bits, tiles done
    std::vector<unsigned int> feat_red_init;
    // gravity plan
    struct Group {
        int kind;
        size_t off;
        int n;
        int row_base, rows, max_src;
        int max_sinks = 0;  // few-sink groups: widest tile
    };
    std::vector<Group> plan[2];
    std::vector<Tile> tiles;
    std::vector<int> heavy, few_row0, row_sink, row_nsrc, row_sys, row_nparts;
    int few_rows = 0;
    int sym_chunk = 0;  // light bodies per symmetric heavy-light tile, about (mixed plan)
    long long few_pitch = 0;
    Tile* d_tiles = nullptr;
    int* d_heavy = nullptr;
    int* d_few_row0 = nullptr;
    int *d_row_sink = nullptr, *d_row_nsrc = nullptr, *d_row_sys = nullptr, *d_row_nparts = nullptr;
    unsigned int* d_sym_ticket = nullptr;  // per disk: the symmetric kernel's last-segment tickets
    std::vector<int> sym_cta;              // the symmetric kernel's CTAs: first segments (+ end)
    int* d_sym_cta = nullptr;
    double* d_terms = nullptr;
    int64_t pairs_per_eval = 0;
    // events: raw records of one attempt, handled on the device (ens_events.cu)
    DevEvent* d_ev = nullptr;
    unsigned int* d_ev_count = nullptr;
    DevEvent* d_hill = nullptr;
    unsigned int* d_hill_count = nullptr;
    unsigned int* d_kerr = nullptr;  // set by a gravity kernel whose tile copy timed out
    unsigned int ev_cap = 0;
    rg_param_t* d_prm = nullptr;     // authoritative body parameters (merges change them)
    double* d_f_rad = nullptr;       // per disk collision factor
    int *d_base = nullptr, *d_ntot = nullptr, *d_nsi = nullptr;
    long long* d_hill_set = nullptr;  // per disk 2 x HILL_SET_CAP pair keys
    int *d_hill_n = nullptr, *d_hill_which = nullptr;
    EnsLogRec* d_elog = nullptr;     // the event log, drained when an advance ends
    unsigned int* d_elog_count = nullptr;
    unsigned int elog_cap = 0;
    unsigned int* d_elog_seq = nullptr;
    unsigned int* d_flags = nullptr;  // ENS_FLAG_* bits
    unsigned int* d_hit_slots = nullptr;
    int* d_keep = nullptr;
    long long* d_attempts = nullptr;  // [0] attempts of the current advance, [1] its limit,
                                      // [2] the end of the current launch's chunk
    std::vector<std::pair<int, rg_event_t>> log;
    // options
    int has_int = 0, ectp = 0, gravity_mode = RG_GRAVITY_FP64, use_graph = 1;
    double tol = 1e-10, dt0 = 0.0, hill_factor = 0.0;
    float near_ratio = 1.0e-5f;
    int started = 0;
    // graph: a conditional while-node whose body is one attempt (its last kernel sets the
    // condition), so that one launch runs attempts until every disk is done
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaGraphConditionalHandle cond = 0;
    bool graph_valid = false;
    int64_t n_kernels = 0, n_graph_launches = 0, n_attempts = 0;
    int64_t kernels_per_attempt = 0;
    // profiling (rg_ens_set_profiling): CUDA events around each launch group of an attempt,
    // by kind (0 gravity, 1 stage combination / error norm, 2 the rest); attempts are then
    // launched directly instead of through the graph
    int profiling = 0;
    std::vector<cudaEvent_t> ev_pool;
    std::vector<int> ev_kind;
    size_t ev_used = 0;
    double* d_part = nullptr;
    int* d_base_of = nullptr;  // per body: index of its disk's body 0
    rg_step_rec_t* d_log = nullptr;
    unsigned int* d_log_count = nullptr;
    unsigned int log_cap = 0;
    std::vector<rg_step_rec_t> host_log;
    // learned proposer
    float* d_feat = nullptr;
    double* d_dt_last = nullptr;
    double* d_ideal_last = nullptr;
    float* d_hist = nullptr;
    int *d_proposed = nullptr, *d_step_prop_rej = nullptr, *d_prop_rej_steps = nullptr, *d_cool = nullptr;
    long long *d_nprop = nullptr, *d_nprop_acc = nullptr, *d_nfallback = nullptr;
    const rg_mlp* mlp = nullptr;
    float mlp_mean[8] = {0}, mlp_inv_std[8] = {1, 1, 1, 1, 1, 1, 1, 1};
    float safety = 0.95f;
    int cooldown = 16;
    float dither = 0.0f;
    unsigned long long dither_seed = 0;

    int n_si(int s) const { return cnt[s][0] + cnt[s][1] + cnt[s][2] + cnt[s][3]; }
    int n_massive(int s) const { return n_si(s) + cnt[s][4] + cnt[s][5]; }
    EnsSys sys() const
    {
        return EnsSys{n_sys, d_status, d_active, d_active_f0, d_acc, d_ej, d_sys_events, d_maxbits, d_t, d_tprev,
                      d_tstop, d_dt_try, d_dt_did, d_ntried, d_npassed, d_nfailed, d_attempt, d_acc_attempt, d_nf0,
                      tol, d_log, d_log_count, log_cap, d_feat, d_dt_last, d_ideal_last, d_hist, d_proposed,
                      d_step_prop_rej, d_prop_rej_steps, d_cool, d_nprop, d_nprop_acc, d_nfallback, cooldown,
                      dither, dither_seed};
    }
};

namespace {

constexpr double GAUSS = 1.720209895e-2;
constexpr double GAUSS2 = 2.959122082855911025e-4;
// bodies per stage tile (one CTA of the per-element kernels): the tiles of a disk are equal but
// its last, so smaller tiles spread the stage combinations' bytes more evenly over the SMs
// (1024 against 2048: 0.93 against 1.03 ms of stage kernels per 256-disk attempt)
constexpr int STAGE_TILE = 1024;
constexpr int ENS_FEW_BLOCK = 32;
constexpr int HILL_SET_CAP = 256;  // pairs inside their Hill spheres per disk
constexpr int HIT_CAP = 64;        // hit-star records per disk and check
constexpr long long ATTEMPT_CHUNK = 4096;  // attempts per graph launch at most
// the FP64 plan uses the first three kinds; the mixed-precision plan uses MIXED, DF_ROWSEQ,
// DF_FEW and DF_SYM (double-float heavy pairs)
enum {
    GROUP_PAIRPAR = 0,
    GROUP_ROWSEQ = 1,
    GROUP_FEW_SERIAL = 2,
    GROUP_MIXED = 3,
    GROUP_DF_ROWSEQ = 4,
    GROUP_DF_FEW = 5,
    GROUP_DF_SYM = 6,  // heavy-light pairs once for both rows, with its systems' heavy rows
    GROUP_KINDS = 7
};
constexpr int ENS_SYM_CHUNK = 2048;  // light bodies per symmetric tile about, unless tuned

template <class T>
int dalloc(T** p, size_t count)
{
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc((void**)p, count * sizeof(T));
    if (e != cudaSuccess) {
        *p = nullptr;
        return set_error(RG_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    }
    return RG_OK;
}

void free_all(rg_ens* e)
{
    if (e->exec) cudaGraphExecDestroy(e->exec);
    if (e->graph) cudaGraphDestroy(e->graph);
    void* ptrs[] = {e->d_y, e->d_yout, e->d_P, e->d_mass, e->d_radius, e->d_rho, e->d_id, e->d_type, e->d_split,
                    e->d_partial, e->d_thr, e->d_status, e->d_active, e->d_active_f0, e->d_acc, e->d_ej,
                    e->d_sys_events, e->d_maxbits, e->d_t, e->d_tprev, e->d_tstop, e->d_dt_try, e->d_dt_did,
                    e->d_ntried, e->d_npassed, e->d_nfailed, e->d_attempt, e->d_acc_attempt, e->d_nf0, e->d_stiles,
                    e->d_tiles, e->d_heavy, e->d_few_row0, e->d_row_sink, e->d_row_nsrc, e->d_row_sys, e->d_row_nparts,
                    e->d_sym_ticket, e->d_sym_cta, e->d_terms, e->d_ev, e->d_ev_count, e->d_hill, e->d_hill_count, e->d_part, e->d_base_of, e->d_log,
                    e->d_log_count, e->d_feat, e->d_dt_last, e->d_ideal_last, e->d_hist, e->d_proposed, e->d_step_prop_rej,
                    e->d_prop_rej_steps, e->d_cool, e->d_nprop, e->d_nprop_acc, e->d_nfallback,
                    e->d_kerr, e->d_rf, e->d_mass_f2, e->d_smax, e->d_screen_slot, e->d_prm,
                    e->d_f_rad, e->d_base, e->d_ntot, e->d_nsi, e->d_hill_set, e->d_hill_n, e->d_hill_which,
                    e->d_elog, e->d_elog_count, e->d_elog_seq, e->d_flags, e->d_hit_slots, e->d_keep,
                    e->d_attempts, e->d_tiles_of, e->d_feat_red};
    for (void* q : ptrs) cudaFree(q);
    for (auto& k : e->d_k) cudaFree(k);
    if (e->st) cudaStreamDestroy(e->st);
    if (e->st2) cudaStreamDestroy(e->st2);
    if (e->ev_fork) cudaEventDestroy(e->ev_fork);
    if (e->ev_join) cudaEventDestroy(e->ev_join);
    for (auto ev : e->ev_pool) cudaEventDestroy(ev);
}

// ------------------------------------------------------------------- profiling
constexpr size_t ENS_MAX_PROFILE_PAIRS = 1 << 18;

// opens a timed launch group of `kind` on the ensemble's stream; returns its index or -1
long prof_begin(rg_ens* e, int kind)
{
    if (!e->profiling || e->ev_used / 2 >= ENS_MAX_PROFILE_PAIRS) return -1;
    while (e->ev_pool.size() < e->ev_used + 2) {
        cudaEvent_t ev;
        if (cudaEventCreate(&ev) != cudaSuccess) return -1;
        e->ev_pool.push_back(ev);
    }
    cudaEventRecord(e->ev_pool[e->ev_used], e->st);
    e->ev_kind.push_back(kind);
    const long idx = (long)e->ev_used;
    e->ev_used += 2;
    return idx;
}

void prof_end(rg_ens* e, long idx)
{
    if (idx >= 0) cudaEventRecord(e->ev_pool[(size_t)idx + 1], e->st);
}

// ------------------------------------------------------------------- plans
void build_stage_tiles(rg_ens* e)
{
    e->stiles.clear();
    e->tiles_of.assign(e->n_sys, 0);
    for (int s = 0; s < e->n_sys; s++) {
        const int b = e->base[s], n = e->ntot[s];
        const int nerr = e->ectp ? n : e->n_massive(s);
        for (int o = 0; o < n; o += STAGE_TILE) {
            const int b0 = b + o, b1 = b + std::min(n, o + STAGE_TILE);
            e->stiles.push_back(StageTile{s, b0, b1, std::max(b0, std::min(b1, b + nerr))});
            e->tiles_of[s]++;
        }
    }
}

void build_gravity_plan(rg_ens* e)
{
    e->tiles.clear();
    e->heavy.clear();
    e->few_row0.clear();
    e->row_sink.clear();
    e->row_nsrc.clear();
    e->row_sys.clear();
    e->row_nparts.clear();
    e->few_rows = 0;
    e->few_pitch = 0;
    e->pairs_per_eval = 0;
    struct Pending {
        int kind, mode;
        std::vector<Tile> t;
        std::vector<int> heavy;
    };
    // group tiles of all disks by (mode, kind)
    std::vector<Tile> by[2][GROUP_KINDS];
    std::vector<int> hv[2][GROUP_KINDS];
    e->screen_slot.assign(e->cap, -1);
    // mixed plan: a system whose SI block is a few heavy bodies (a few-sink block over every
    // massive body) and whose NSI block takes the row kernel over them evaluates the pairs
    // between the two blocks once, for both rows (grav_df_sym, the heavy-heavy pairs with
    // them).  The light bodies of all such systems, end to end, are cut into ranges of equal
    // cost (plan_tools.h), about sym_chunk bodies each, one per CTA, their count whole waves of
    // resident CTAs; a range's pieces in different systems are its segments, each one part of
    // its system's heavy rows.
    e->sym_chunk = e->few_chunk > 0 ? e->few_chunk : ENS_SYM_CHUNK;
    std::vector<char> sym(e->n_sys, 0);
    std::vector<Tile> sym_systems;
    std::vector<int> sym_parts(e->n_sys, 0), sym_row0(e->n_sys, 0);
    double sym_light = 0.0;
    for (int s = 0; s < e->n_sys; s++) {
        const int nsi = e->n_si(s), nm = e->n_massive(s), b = e->base[s];
        sym[s] = nsi >= 1 && nsi <= DF_SYM_MAX_HEAVY && nm > nsi && nsi <= e->rowseq_max_src &&
                 nm > e->rowseq_max_src && nsi <= ENS_FEW_BLOCK;
        if (!sym[s]) continue;
        sym_light += nm - nsi;
        sym_systems.push_back(Tile{b + nsi, b + nm, b, b + nsi, s, b, 1, 0});
    }
    e->sym_cta.clear();
    if (!sym_systems.empty()) {
        const int slots = DF_SYM_RESIDENT * e->n_sm;
        const int waves = std::max(1, (int)std::lround(sym_light / ((double)slots * e->sym_chunk)));
        const int n_cta = (int)std::min<double>(waves * slots, std::ceil(sym_light / DF_SYM_PASS));
        std::vector<int> parts;
        build_sym_segments(sym_systems, n_cta, DF_SYM_PASS, DF_SYM_SEGMENT_COST, by[1][GROUP_DF_SYM], e->sym_cta,
                           parts);
        hv[1][GROUP_DF_SYM].assign(by[1][GROUP_DF_SYM].size(), 0);
        for (size_t k = 0; k < sym_systems.size(); k++) sym_parts[sym_systems[k].sys] = parts[k];
    }
    for (int s = 0; s < e->n_sys; s++) {
        const int b = e->base[s];
        const int nsi = e->n_si(s), nm = e->n_massive(s), nt = e->ntot[s];
        const int n_heavy = std::min(nsi, e->cnt[s][0] + e->cnt[s][1] + e->cnt[s][2]);
        for (int q = n_heavy; q < nt; q++) e->screen_slot[b + q] = s;
        e->pairs_per_eval += (int64_t)nsi * (nm > 0 ? nm - 1 : 0) + (int64_t)(nm - nsi) * nsi + (int64_t)(nt - nm) * nm;
        struct Blk {
            int s0, s1, src1, block;
        } blks[3] = {{0, nsi, nm, 0}, {nsi, nm, nsi, 1}, {nm, nt, nm, 2}};
        auto add = [&](int mode, int kind, int s0, int s1, int src1, int block, int step) {
            for (int q = s0; q < s1; q += step) {
                by[mode][kind].push_back(Tile{b + q, b + std::min(q + step, s1), b, b + src1, s, b, block, 0});
                hv[mode][kind].push_back(b + std::min(n_heavy, src1));
            }
        };
        for (const auto& k : blks) {
            if (k.s1 <= k.s0) continue;
            if (k.src1 <= e->rowseq_max_src) {
                add(0, GROUP_ROWSEQ, k.s0, k.s1, k.src1, k.block, 128);
                if (!(sym[s] && k.block == 1))  // a symmetric system's light rows: the segments above
                    add(1, GROUP_DF_ROWSEQ, k.s0, k.s1, k.src1, k.block, 128);
            } else if (k.s1 - k.s0 <= ENS_FEW_BLOCK) {
                add(0, GROUP_FEW_SERIAL, k.s0, k.s1, k.src1, k.block, FEW_SINKS_MAX);
                if (!(sym[s] && k.block == 0))  // a symmetric system's heavy rows come with its tiles
                    add(1, GROUP_DF_FEW, k.s0, k.s1, k.src1, k.block, FEW_SINKS_MAX);
            } else {
                add(0, GROUP_PAIRPAR, k.s0, k.s1, k.src1, k.block, e->pairpar_S);  // S sinks per CTA and tile
                const int light0 = k.block == 0 ? std::max(k.s0, std::min(n_heavy, k.s1)) : k.s0;
                add(1, GROUP_DF_FEW, k.s0, light0, k.src1, k.block, FEW_SINKS_MAX);
                add(1, GROUP_MIXED, light0, k.s1, k.src1, k.block, MIXED_SINKS_PER_TILE);
            }
        }
    }
    for (int mode = 0; mode < 2; mode++) {
        e->plan[mode].clear();
        for (int kind = 0; kind < GROUP_KINDS; kind++) {
            auto& T = by[mode][kind];
            if (T.empty()) continue;
            rg_ens::Group gr{kind, e->tiles.size(), (int)T.size(), e->few_rows, 0, 0};
            for (size_t k = 0; k < T.size(); k++) {
                e->tiles.push_back(T[k]);
                e->heavy.push_back(hv[mode][kind][k]);
                if (kind == GROUP_FEW_SERIAL || kind == GROUP_DF_FEW) {
                    e->few_row0.push_back(e->few_rows);
                    const int nsrc = T[k].src_end - T[k].src_begin;
                    for (int i = T[k].sink_begin; i < T[k].sink_end; i++) {
                        e->row_sink.push_back(i);
                        e->row_nsrc.push_back(nsrc);
                        e->row_sys.push_back(T[k].sys);
                        e->row_nparts.push_back(0);
                        e->few_rows++;
                        gr.rows++;
                    }
                    gr.max_src = std::max(gr.max_src, nsrc);
                    gr.max_sinks = std::max(gr.max_sinks, T[k].sink_end - T[k].sink_begin);
                    e->few_pitch = std::max<long long>(e->few_pitch, nsrc);
                } else if (kind == GROUP_DF_SYM) {
                    const int sy = T[k].sys, nh = T[k].src_end - T[k].src_begin;
                    if (T[k].part == 1) {  // the system's heavy rows: the heavy-heavy part + one per segment
                        sym_row0[sy] = e->few_rows;
                        for (int h = 0; h < nh; h++) {
                            e->row_sink.push_back(T[k].src_begin + h);
                            e->row_nsrc.push_back(e->n_massive(sy));
                            e->row_sys.push_back(sy);
                            e->row_nparts.push_back(sym_parts[sy]);
                            e->few_rows++;
                            gr.rows++;
                        }
                        e->few_pitch = std::max<long long>(e->few_pitch, sym_parts[sy]);
                    }
                    e->few_row0.push_back(sym_row0[sy]);
                    gr.max_src = std::max(gr.max_src, nh);
                } else {
                    e->few_row0.push_back(0);
                }
            }
            e->plan[mode].push_back(gr);
        }
    }
}

int upload_plans(rg_ens* e)
{
    const size_t nt = e->tiles.size();
    int rc = RG_OK;
    auto chk = [&](int x) {
        if (!rc) rc = x;
    };
    cudaFree(e->d_stiles);
    cudaFree(e->d_tiles);
    cudaFree(e->d_heavy);
    cudaFree(e->d_few_row0);
    cudaFree(e->d_row_sink);
    cudaFree(e->d_row_nsrc);
    cudaFree(e->d_row_nparts);
    cudaFree(e->d_sym_cta);
    cudaFree(e->d_row_sys);
    cudaFree(e->d_terms);
    cudaFree(e->d_tiles_of);
    e->d_stiles = nullptr;
    e->d_tiles_of = nullptr;
    e->d_tiles = nullptr;
    e->d_heavy = e->d_few_row0 = e->d_row_sink = e->d_row_nsrc = e->d_row_sys = e->d_row_nparts = nullptr;
    e->d_sym_cta = nullptr;
    e->d_terms = nullptr;
    chk(dalloc(&e->d_stiles, e->stiles.size()));
    chk(dalloc(&e->d_tiles_of, e->tiles_of.size()));
    chk(dalloc(&e->d_tiles, nt));
    chk(dalloc(&e->d_heavy, nt));
    chk(dalloc(&e->d_few_row0, nt));
    chk(dalloc(&e->d_row_sink, (size_t)e->few_rows));
    chk(dalloc(&e->d_row_nsrc, (size_t)e->few_rows));
    chk(dalloc(&e->d_row_nparts, (size_t)e->few_rows));
    chk(dalloc(&e->d_sym_cta, e->sym_cta.size()));
    chk(dalloc(&e->d_row_sys, (size_t)e->few_rows));
    chk(dalloc(&e->d_terms, (size_t)3 * e->few_rows * (size_t)std::max<long long>(e->few_pitch, 1)));
    if (rc) return rc;
    auto up = [&](void* dst, const void* src, size_t bytes) {
        if (bytes && !rc) {
            cudaError_t err = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, e->st);
            if (err != cudaSuccess) rc = cuda_fail(err, "upload", __FILE__, __LINE__);
        }
    };
    up(e->d_stiles, e->stiles.data(), e->stiles.size() * sizeof(StageTile));
    up(e->d_tiles_of, e->tiles_of.data(), e->tiles_of.size() * sizeof(int));
    up(e->d_tiles, e->tiles.data(), nt * sizeof(Tile));
    up(e->d_heavy, e->heavy.data(), nt * sizeof(int));
    up(e->d_screen_slot, e->screen_slot.data(), e->screen_slot.size() * sizeof(int));
    up(e->d_few_row0, e->few_row0.data(), nt * sizeof(int));
    up(e->d_row_sink, e->row_sink.data(), e->row_sink.size() * sizeof(int));
    up(e->d_row_nsrc, e->row_nsrc.data(), e->row_nsrc.size() * sizeof(int));
    up(e->d_row_nparts, e->row_nparts.data(), e->row_nparts.size() * sizeof(int));
    up(e->d_sym_cta, e->sym_cta.data(), e->sym_cta.size() * sizeof(int));
    up(e->d_row_sys, e->row_sys.data(), e->row_sys.size() * sizeof(int));
    if (!rc) RG_CUDA_CHECK(cudaStreamSynchronize(e->st));
    e->graph_valid = false;
    return rc;
}

// ------------------------------------------------------------------- one attempt
int ens_gravity(rg_ens* e, const double* pos, const double* vel, double* acc, int stage, const int* mask,
                bool hill)
{
    const size_t cap = (size_t)e->cap;
    GravArgs g{};
    g.px = pos;
    g.py = pos + cap;
    g.pz = pos + 2 * cap;
    g.vx = vel;
    g.vy = vel + cap;
    g.vz = vel + 2 * cap;
    g.mass = e->d_mass;
    g.radius = e->d_radius;
    g.id = e->d_id;
    g.rho = e->d_rho;
    g.rf = e->gravity_mode == RG_GRAVITY_MIXED ? e->d_rf : nullptr;
    g.ax = acc;
    g.ay = acc + cap;
    g.az = acc + 2 * cap;
    // each disk's own collision factor (sys_f_rad); the largest decides whether any records
    g.f_rad = 0.0;
    for (int s2 = 0; s2 < e->n_sys; s2++) g.f_rad = std::max(g.f_rad, e->thr[5 * (size_t)s2 + 2]);
    g.sys_f_rad = e->d_f_rad;
    g.hill_f3 = e->hill_factor * e->hill_factor * e->hill_factor;
    g.f_rad_f = (float)g.f_rad;
    g.hill_f3_f = (float)g.hill_f3;
    g.record = (stage > 0 && g.f_rad > 0.0) ? 1 : 0;
    g.hill = hill ? 1 : 0;
    // the mixed form's stage vectors are double-float pairs: the accelerations written, and the
    // velocities read for records after the step start (stage 0 reads the FP64 state's)
    g.acc_f2 = e->gravity_mode == RG_GRAVITY_MIXED ? 1 : 0;
    g.vel_f2 = g.acc_f2 && stage > 0 ? 1 : 0;
    g.seq = (uint32_t)stage;
    g.ev = EventBuf{e->d_ev, e->d_ev_count, e->ev_cap};
    g.hv = EventBuf{e->d_hill, e->d_hill_count, e->ev_cap};
    g.sys_active = mask;
    g.sys_events = e->d_sys_events;
    g.sys_attempt = e->d_attempt;
    g.sys_f0 = e->d_nf0;
    g.sys_t = e->d_t;
    int rc = RG_OK;
    if (hill) {
        // distance from each disk's body 0 (the per-body base is the tile's base: use a
        // base-of array built from the stage tiles)
        rc = launch_star_distance(g.px, g.py, g.pz, e->d_base_of, e->cap, e->d_rho, e->st);
        if (rc) return rc;
        e->n_kernels++;
    }
    // the screens' maxima serve the mixed kernel's per-sink cutoffs (light sinks x light sources)
    bool mixed_tiles = false;
    for (const auto& gr : e->plan[1]) mixed_tiles = mixed_tiles || gr.kind == GROUP_MIXED;
    if (e->gravity_mode == RG_GRAVITY_MIXED && (g.record || g.hill) && mixed_tiles) {
        RG_CUDA_CHECK(cudaMemsetAsync(e->d_smax, 0, (size_t)SCREEN_MAX_WORDS * e->n_sys * sizeof(unsigned int),
                                      e->st));
        g.smax = e->d_smax;
    }
    const auto& plan = e->plan[e->gravity_mode == RG_GRAVITY_MIXED ? 1 : 0];
    bool split_done = false;
    // a later stage of the attempt needs only the coordinates split again: the step start's
    // split wrote the masses and radii, which change only at events (after the attempt); when
    // the symmetric kernel is the only one, it splits the coordinates itself (from the FP64
    // positions and the step start's split masses)
    bool sym_only = !plan.empty();
    for (const auto& gr : plan) sym_only = sym_only && gr.kind == GROUP_DF_SYM;
    const bool sym_splits = e->gravity_mode == RG_GRAVITY_MIXED && sym_only && stage > 0 && !g.smax;
    if (e->gravity_mode == RG_GRAVITY_MIXED && !plan.empty() && !sym_splits) {
        // (Writing the split from the stage combination instead was slower: its 8-byte stores
        // at a 32-byte stride cost the combination more than this kernel takes.)
        if (stage > 0 && !g.smax)
            rc = launch_split_coords(g.px, g.py, g.pz, e->cap, (SplitPos*)e->d_split, e->st);
        else
            rc = launch_split_positions(g.px, g.py, g.pz, e->d_mass, e->d_id, e->d_base_of, e->d_screen_slot,
                                        e->d_radius, e->cap, (SplitPos*)e->d_split, e->d_rf,
                                        g.smax ? e->d_smax : nullptr, g.hill != 0, e->st, e->d_mass_f2);
        split_done = true;
        e->n_kernels++;
        if (rc) return rc;
    }
    // fork the row groups onto the side stream when other groups run beside them
    bool has_row = false, has_other = false;
    for (const auto& gr : plan) {
        const bool row = gr.kind == GROUP_ROWSEQ || gr.kind == GROUP_DF_ROWSEQ;
        has_row = has_row || row;
        has_other = has_other || !row;
    }
    const bool fork = has_row && has_other;
    if (fork) {
        RG_CUDA_CHECK(cudaEventRecord(e->ev_fork, e->st));
        RG_CUDA_CHECK(cudaStreamWaitEvent(e->st2, e->ev_fork, 0));
    }
    cudaStream_t row_st = fork ? e->st2 : e->st;
    for (const auto& gr : plan) {
        g.tiles = e->d_tiles + gr.off;
        g.n_tiles = gr.n;
        switch (gr.kind) {
        case GROUP_PAIRPAR: rc = launch_grav_fp64_pairpar(g, e->pairpar_S, e->st); e->n_kernels++; break;
        case GROUP_ROWSEQ: rc = launch_grav_fp64_rowseq(g, row_st); e->n_kernels++; break;
        case GROUP_FEW_SERIAL:
            rc = launch_grav_fp64_few(g, e->d_few_row0 + gr.off, gr.max_src, e->d_terms, e->few_rows, e->few_pitch,
                                      e->d_row_sink, e->d_row_nsrc, e->d_row_sys, gr.row_base, gr.rows, e->st);
            e->n_kernels += 2;
            break;
        case GROUP_DF_ROWSEQ:
        case GROUP_DF_FEW:
            if (!split_done) {
                rc = launch_split_positions(g.px, g.py, g.pz, e->d_mass, e->d_id, e->d_base_of, e->d_screen_slot,
                                            e->d_radius, e->cap, (SplitPos*)e->d_split, e->d_rf,
                                            g.smax ? e->d_smax : nullptr, g.hill != 0, e->st);
                split_done = true;
                e->n_kernels++;
            }
            if (rc) break;
            if (gr.kind == GROUP_DF_ROWSEQ) {
                rc = launch_grav_df_rowseq(g, e->d_split, row_st);
                e->n_kernels++;
            } else {
                rc = launch_grav_df_few(g, e->d_split, e->d_few_row0 + gr.off, gr.max_src, gr.max_sinks, e->few_chunk,
                                        e->d_terms,
                                        e->few_rows,
                                        e->few_pitch, e->d_row_sink, e->d_row_nsrc, e->d_row_sys, gr.row_base, gr.rows,
                                        e->st);
                e->n_kernels += 2;
            }
            break;
        case GROUP_DF_SYM:
            rc = launch_grav_df_sym(g, e->d_sym_cta, (int)e->sym_cta.size() - 1, e->d_split, e->d_few_row0 + gr.off,
                                    gr.max_src, e->d_terms, e->few_rows, e->few_pitch, e->d_row_sink, e->d_row_nparts,
                                    e->d_sym_ticket, e->st, sym_splits ? e->d_mass_f2 : nullptr);
            e->n_kernels++;
            break;
        case GROUP_MIXED:
            if (!split_done) {
                rc = launch_split_positions(g.px, g.py, g.pz, e->d_mass, e->d_id, e->d_base_of, e->d_screen_slot,
                                            e->d_radius, e->cap, (SplitPos*)e->d_split, e->d_rf,
                                            g.smax ? e->d_smax : nullptr, g.hill != 0, e->st);
                split_done = true;
                e->n_kernels++;
            }
            if (!rc) {
                // one source chunk: the disks' source counts differ, so a chunked split would
                // need a partial buffer per disk
                rc = launch_grav_mixed_tiles(g, e->d_split, e->d_heavy + gr.off, e->near_ratio, 1, MIXED_SOURCE_TILE,
                                             nullptr, e->cap, e->d_kerr, false, e->st);
                e->n_kernels++;
            }
            break;
        }
        if (rc) break;
    }
    if (fork) {  // join (also after an error: a capture must not end with the side stream open)
        RG_CUDA_CHECK(cudaEventRecord(e->ev_join, e->st2));
        RG_CUDA_CHECK(cudaStreamWaitEvent(e->st, e->ev_join, 0));
    }
    return rc;
}

int launch_stage(rg_ens* e, int form, int nterm, const int* stages, const double* coef, double* out_lo,
                 double* out_hi)
{
    EnsStageArgs a{};
    a.tiles = e->d_stiles;
    a.active = e->d_active;
    a.dt = e->d_dt_try;
    a.y = e->d_y;
    for (int q = 0; q < nterm; q++) {
        a.k[q] = e->d_k[stages[q]];
        a.c[q] = coef[q];
    }
    a.nterm = nterm;
    a.stride = e->cap;
    a.out_lo = out_lo;
    a.out_hi = out_hi;
    a.max_bits = nullptr;
    if (form == FORM_RK8_NP1 && e->gravity_mode == RG_GRAVITY_MIXED) {  // the error norm folded in
        a.k[7] = e->d_k[11];
        a.k[8] = e->d_k[12];
        a.max_bits = e->d_maxbits;
    }
    const int g = (int)e->stiles.size();
    if (g <= 0) return RG_OK;
    const bool df = e->gravity_mode == RG_GRAVITY_MIXED;  // double-float stage vectors
    // the mixed form's combination may be scheduled while the gravity kernel before it
    // finishes (programmatic dependent launch; the kernel waits before it reads anything)
    cudaLaunchAttribute pdl[1];
    pdl[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    pdl[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3((unsigned)g);
    cfg.blockDim = dim3(256);
    cfg.stream = e->st;
    cfg.attrs = pdl;
    cfg.numAttrs = 1;
#define RG_ENS(F, T)                                                     \
    do {                                                                 \
        if (df)                                                          \
            RG_CUDA_CHECK(cudaLaunchKernelEx(&cfg, ens_combine_df_kernel<F, T>, a)); \
        else                                                             \
            ens_combine_kernel<F, T><<<g, 256, 0, e->st>>>(a);           \
    } while (0)
    if (form == FORM_RK8_NP1) {
        RG_ENS(FORM_RK8_NP1, 7);
    } else {
        switch (nterm) {
        case 1: RG_ENS(FORM_SUM, 1); break;
        case 2: RG_ENS(FORM_SUM, 2); break;
        case 3: RG_ENS(FORM_SUM, 3); break;
        case 4: RG_ENS(FORM_SUM, 4); break;
        case 6: RG_ENS(FORM_SUM, 6); break;
        case 7: RG_ENS(FORM_SUM, 7); break;
        case 8: RG_ENS(FORM_SUM, 8); break;
        case 9: RG_ENS(FORM_SUM, 9); break;
        default: return set_error(RG_ERR_ARG, "stage row length");
        }
    }
#undef RG_ENS
    RG_CUDA_CHECK(cudaGetLastError());
    e->n_kernels++;
    return RG_OK;
}

EnsEventArgs event_args(rg_ens* e)
{
    EnsEventArgs a{};
    a.n_sys = e->n_sys;
    a.base = e->d_base;
    a.ntot = e->d_ntot;
    a.nsi = e->d_nsi;
    a.stride = e->cap;
    a.y = e->d_y;
    a.mass = e->d_mass;
    a.radius = e->d_radius;
    a.prm = e->d_prm;
    a.id = e->d_id;
    a.type = e->d_type;
    a.thr = e->d_thr;
    a.status = e->d_status;
    a.active = e->d_active;
    a.active_f0 = e->d_active_f0;
    a.t = e->d_t;
    a.t_prev = e->d_tprev;
    a.t_stop = e->d_tstop;
    a.dt_did = e->d_dt_did;
    a.acc_attempt = e->d_acc_attempt;
    a.ej = e->d_ej;
    a.ev = e->d_ev;
    a.ev_count = e->d_ev_count;
    a.ev_cap = e->ev_cap;
    a.hill = e->d_hill;
    a.hill_count = e->d_hill_count;
    a.hill_set = e->d_hill_set;
    a.hill_n = e->d_hill_n;
    a.hill_which = e->d_hill_which;
    a.hill_set_cap = HILL_SET_CAP;
    a.log = e->d_elog;
    a.log_count = e->d_elog_count;
    a.log_cap = e->elog_cap;
    a.log_seq = e->d_elog_seq;
    a.flags = e->d_flags;
    a.hit_slots = e->d_hit_slots;
    a.hit_cap = HIT_CAP;
    for (int r = 0; r < 13; r++) a.stage_c[r] = rk8_c[r];
    return a;
}

EnsLoopArgs loop_args(rg_ens* e, bool in_graph)
{
    EnsLoopArgs l{};
    l.n_sys = e->n_sys;
    l.status = e->d_status;
    l.active = e->d_active;
    l.active_f0 = e->d_active_f0;
    l.flags = e->d_flags;
    l.kerr = e->d_kerr;
    l.step_log_count = e->d_log_count;
    l.step_log_cap = e->log_cap;
    l.ev_count = e->d_ev_count;
    l.hill_count = e->d_hill_count;
    l.ev_cap = e->ev_cap;
    l.attempts = e->d_attempts;
    l.keep = e->d_keep;
    l.cond = e->cond;
    l.use_cond = in_graph ? 1 : 0;
    return l;
}

// The launch sequence of one attempt of every running disk, with the handling of its events
// and the loop condition (captured as the body of the graph's while-node).
int record_attempt(rg_ens* e, bool in_graph)
{
    const size_t cap = (size_t)e->cap;
    const int ns = (int)e->stiles.size();
    const int nb = (e->n_sys + 127) / 128;
    // stage 0 for the disks that start a new step: k0 = (v, a(y))
    long pr = prof_begin(e, 2);
    if (e->gravity_mode == RG_GRAVITY_MIXED)  // the stage vectors are double-float pairs
        ens_copy_to_f2_kernel<<<ns, 256, 0, e->st>>>(e->d_stiles, e->d_active_f0, e->d_y, 3, e->d_k[0], 0, 3, e->cap);
    else
        ens_copy_kernel<<<ns, 256, 0, e->st>>>(e->d_stiles, e->d_active_f0, e->d_y, 3, e->d_k[0], 0, 3, e->cap);
    prof_end(e, pr);
    RG_CUDA_CHECK(cudaGetLastError());
    e->n_kernels++;
    pr = prof_begin(e, 0);
    int rc = ens_gravity(e, e->d_y, e->d_y + 3 * cap, e->d_k[0] + 3 * cap, 0, e->d_active_f0, e->hill_factor > 0.0);
    prof_end(e, pr);
    if (rc) return rc;
    pr = prof_begin(e, 2);
    if (e->d_log || e->mlp || e->dither > 0.0f) {
        // step-start features (and, with a network attached, the proposed trial step): one
        // kernel, a CTA per stage tile, the network in each disk's last tile
        PropArgs pa{};
        pa.s = e->sys();
        pa.y = e->d_y;
        pa.k0 = e->d_k[0];
        pa.k_f2 = e->gravity_mode == RG_GRAVITY_MIXED ? 1 : 0;
        pa.mass = e->d_mass;
        pa.id = e->d_id;
        pa.base = e->d_base;
        pa.nsi = e->d_nsi;
        pa.ntot = e->d_ntot;
        pa.stride = e->cap;
        pa.w = (const __nv_bfloat16*)mlp_device_weights(e->mlp);
        for (int q = 0; q < 8; q++) {
            pa.mean[q] = e->mlp_mean[q];
            pa.inv_std[q] = e->mlp_inv_std[q];
        }
        pa.safety = e->safety;
        pa.tiles = e->d_stiles;
        pa.tiles_of = e->d_tiles_of;
        pa.red = e->d_feat_red;
        ens_propose_kernel<<<(int)e->stiles.size(), PROP_THREADS, 0, e->st>>>(pa);
        RG_CUDA_CHECK(cudaGetLastError());
        e->n_kernels += 1;
    }
    if (e->hill_factor > 0.0) {  // the pairs that entered their Hill spheres at this step start
        rc = launch_ens_hill(event_args(e), e->st);
        if (rc) return rc;
        e->n_kernels++;
    }
    prof_end(e, pr);
    for (int r = 1; r <= 12 && !rc; r++) {
        double a[9];
        for (int q = 0; q < rk8_nterm[r]; q++) a[q] = rk8_a[rk8_aidx[r][q]];
        pr = prof_begin(e, 1);
        rc = launch_stage(e, FORM_SUM, rk8_nterm[r], rk8_stage[r], a, e->d_P, e->d_k[r]);
        prof_end(e, pr);
        pr = prof_begin(e, 0);
        if (!rc) rc = ens_gravity(e, e->d_P, e->d_k[r], e->d_k[r] + 3 * cap, r, e->d_active, false);
        prof_end(e, pr);
    }
    if (rc) return rc;
    const int snp[7] = {0, 5, 6, 7, 8, 9, 10};
    const double bnp[7] = {rk8_b[0], rk8_b[5], rk8_b[6], rk8_b[8], rk8_b[10], 0.0, 0.0};
    pr = prof_begin(e, 1);
    rc = launch_stage(e, FORM_RK8_NP1, 7, snp, bnp, e->d_yout, e->d_yout + 3 * cap);
    if (rc) return rc;
    if (e->gravity_mode != RG_GRAVITY_MIXED)  // the mixed form's y_{n+1} kernel takes the error norm too
        ens_error_kernel<<<ns, 256, 0, e->st>>>(e->d_stiles, e->d_active, e->d_k[0], e->d_k[10], e->d_k[11],
                                                e->d_k[12], e->cap, e->d_maxbits);
    prof_end(e, pr);
    RG_CUDA_CHECK(cudaGetLastError());
    pr = prof_begin(e, 2);
    ens_controller_kernel<<<nb, 128, 0, e->st>>>(e->sys());
    RG_CUDA_CHECK(cudaGetLastError());
    ens_accept_kernel<<<ns, 256, 0, e->st>>>(e->d_stiles, e->d_acc, e->d_yout, e->d_y, e->cap, e->d_id, e->d_type,
                                             e->d_thr, e->d_ej);
    RG_CUDA_CHECK(cudaGetLastError());
    ens_finalize_kernel<<<nb, 128, 0, e->st>>>(e->sys());
    RG_CUDA_CHECK(cudaGetLastError());
    // merges, ejections and hit-star merges of the held disks, then the loop condition
    rc = launch_ens_handle(event_args(e), 0, e->st);
    if (!rc) rc = launch_ens_loop(loop_args(e, in_graph), e->st);
    prof_end(e, pr);
    if (rc) return rc;
    e->n_kernels += e->gravity_mode == RG_GRAVITY_MIXED ? 5 : 6;  // (error norm,) controller ... loop
    return RG_OK;
}

int launch_attempt(rg_ens* e)
{
    const int64_t k0 = e->n_kernels;
    int rc = record_attempt(e, false);
    e->kernels_per_attempt = e->n_kernels - k0;
    return rc;
}

// the graph: one conditional while-node whose body, captured from record_attempt, ends with
// the kernel that sets the condition; rebuilt when a launch parameter it freezes changes
int build_loop_graph(rg_ens* e)
{
    if (e->exec) cudaGraphExecDestroy(e->exec);
    if (e->graph) cudaGraphDestroy(e->graph);
    e->exec = nullptr;
    e->graph = nullptr;
    e->graph_valid = false;
    RG_CUDA_CHECK(cudaGraphCreate(&e->graph, 0));
    RG_CUDA_CHECK(cudaGraphConditionalHandleCreate(&e->cond, e->graph, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams np{};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = e->cond;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t node = nullptr;
    RG_CUDA_CHECK(cudaGraphAddNode(&node, e->graph, nullptr, nullptr, 0, &np));
    cudaGraph_t body = np.conditional.phGraph_out[0];
    RG_CUDA_CHECK(cudaStreamBeginCaptureToGraph(e->st, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    const int64_t k0 = e->n_kernels;
    int rc = record_attempt(e, true);
    e->kernels_per_attempt = e->n_kernels - k0;
    e->n_kernels = k0;
    cudaGraph_t captured = nullptr;
    const cudaError_t err = cudaStreamEndCapture(e->st, &captured);
    if (rc) return rc;
    if (err != cudaSuccess) return cuda_fail(err, "cudaStreamEndCapture", __FILE__, __LINE__);
    RG_CUDA_CHECK(cudaGraphInstantiate(&e->exec, e->graph, 0));
    e->graph_valid = true;
    return RG_OK;
}

}  // namespace

// ============================================================================ C ABI

namespace {

template <class T>
int upload(rg_ens* e, T* dst, const std::vector<T>& src)
{
    if (!src.empty())
        RG_CUDA_CHECK(cudaMemcpyAsync(dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice, e->st));
    return RG_OK;
}

template <class T>
int download(rg_ens* e, std::vector<T>& dst, const T* src, size_t n)
{
    dst.resize(n);
    if (n) RG_CUDA_CHECK(cudaMemcpyAsync(dst.data(), src, n * sizeof(T), cudaMemcpyDeviceToHost, e->st));
    return RG_OK;
}

int create_impl(int n_sys, const rg_counts_t* counts, const rg_vec_t* r, const rg_vec_t* v, const rg_param_t* p,
                const rg_body_metadata_t* md, const double* thr, int event_capacity, rg_ens** out)
{
    if (n_sys <= 0 || !counts || !r || !v || !p || !md || !thr || !out) return set_error(RG_ERR_ARG, "bad argument");
    *out = nullptr;
    int dev_count = 0;
    if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count <= 0) {
        cudaGetLastError();
        return set_error(RG_ERR_NO_DEVICE, "no CUDA device");
    }
    rg_ens* e = new rg_ens();
    e->n_sys = n_sys;
    int64_t tot = 0;
    for (int s = 0; s < n_sys; s++) {
        std::array<int, 7> c;
        const int32_t* cn = &counts[s].n_s;
        int n = 0;
        for (int k = 0; k < 7; k++) {
            if (cn[k] < 0) {
                delete e;
                return set_error(RG_ERR_ARG, "negative body count");
            }
            c[k] = cn[k];
            n += cn[k];
        }
        if (n <= 0) {
            delete e;
            return set_error(RG_ERR_ARG, "empty disk");
        }
        e->cnt.push_back(c);
        e->base.push_back((int)tot);
        e->ntot.push_back(n);
        tot += n;
    }
    if (tot > (1 << 28)) {
        delete e;
        return set_error(RG_ERR_ARG, "too many bodies");
    }
    e->cap = (int)tot;
    cudaGetDevice(&e->device);
    cudaDeviceGetAttribute(&e->n_sm, cudaDevAttrMultiProcessorCount, e->device);
    e->ev_cap = (unsigned int)(event_capacity > 0 ? event_capacity : std::max<int64_t>(tot, 4096));
    const size_t nt = (size_t)tot, ns = (size_t)n_sys;
    int rc = RG_OK;
    auto chk = [&](int x) {
        if (!rc) rc = x;
    };
    if (cudaStreamCreateWithFlags(&e->st, cudaStreamNonBlocking) != cudaSuccess) chk(set_error(RG_ERR_CUDA, "stream"));
    if (!rc && cudaStreamCreateWithFlags(&e->st2, cudaStreamNonBlocking) != cudaSuccess)
        chk(set_error(RG_ERR_CUDA, "stream"));
    if (!rc && (cudaEventCreateWithFlags(&e->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
                cudaEventCreateWithFlags(&e->ev_join, cudaEventDisableTiming) != cudaSuccess))
        chk(set_error(RG_ERR_CUDA, "event"));
    chk(dalloc(&e->d_y, 6 * nt));
    chk(dalloc(&e->d_yout, 6 * nt));
    for (auto& k : e->d_k) chk(dalloc(&k, 6 * nt));
    chk(dalloc(&e->d_P, 3 * nt));
    chk(dalloc(&e->d_mass, nt));
    chk(dalloc(&e->d_radius, nt));
    chk(dalloc(&e->d_rho, nt));
    chk(dalloc(&e->d_id, nt));
    chk(dalloc(&e->d_type, nt));
    chk(dalloc(&e->d_base_of, nt));
    chk(dalloc((char**)&e->d_split, SPLIT_POS_BYTES * nt));
    chk(dalloc(&e->d_rf, nt));
    chk(dalloc(&e->d_mass_f2, nt));
    chk(dalloc(&e->d_smax, (size_t)SCREEN_MAX_WORDS * ns));
    chk(dalloc(&e->d_screen_slot, nt));
    chk(dalloc(&e->d_thr, 5 * ns));
    chk(dalloc(&e->d_status, ns));
    chk(dalloc(&e->d_active, ns));
    chk(dalloc(&e->d_active_f0, ns));
    chk(dalloc(&e->d_acc, ns));
    chk(dalloc(&e->d_ej, ns));
    chk(dalloc(&e->d_sys_events, ns));
    chk(dalloc(&e->d_maxbits, ns));
    chk(dalloc(&e->d_t, ns));
    chk(dalloc(&e->d_tprev, ns));
    chk(dalloc(&e->d_tstop, ns));
    chk(dalloc(&e->d_dt_try, ns));
    chk(dalloc(&e->d_dt_did, ns));
    chk(dalloc(&e->d_ntried, ns));
    chk(dalloc(&e->d_npassed, ns));
    chk(dalloc(&e->d_nfailed, ns));
    chk(dalloc(&e->d_attempt, ns));
    chk(dalloc(&e->d_acc_attempt, ns));
    chk(dalloc(&e->d_nf0, ns));
    chk(dalloc(&e->d_feat, 8 * ns));
    chk(dalloc(&e->d_feat_red, 3 * ns));
    chk(dalloc(&e->d_dt_last, ns));
    chk(dalloc(&e->d_ideal_last, ns));
    chk(dalloc(&e->d_hist, 5 * ns));
    chk(dalloc(&e->d_proposed, ns));
    chk(dalloc(&e->d_step_prop_rej, ns));
    chk(dalloc(&e->d_prop_rej_steps, ns));
    chk(dalloc(&e->d_cool, ns));
    chk(dalloc(&e->d_nprop, ns));
    chk(dalloc(&e->d_nprop_acc, ns));
    chk(dalloc(&e->d_nfallback, ns));
    chk(dalloc(&e->d_ev, e->ev_cap));
    chk(dalloc(&e->d_ev_count, 1));
    chk(dalloc(&e->d_hill, e->ev_cap));
    chk(dalloc(&e->d_hill_count, 1));
    chk(dalloc(&e->d_kerr, 1));
    chk(dalloc(&e->d_prm, nt));
    chk(dalloc(&e->d_f_rad, ns));
    chk(dalloc(&e->d_base, ns));
    chk(dalloc(&e->d_ntot, ns));
    chk(dalloc(&e->d_nsi, ns));
    chk(dalloc(&e->d_hill_set, 2 * (size_t)HILL_SET_CAP * ns));
    chk(dalloc(&e->d_hill_n, ns));
    chk(dalloc(&e->d_hill_which, ns));
    chk(dalloc(&e->d_sym_ticket, ns));
    // the event log holds every record of one advance: 16 per body, at least 4096, at most
    // 2^18 (128 MiB); more records end the advance with RG_ERR_EVENT_OVERFLOW
    e->elog_cap = (unsigned int)std::min<int64_t>(1 << 18, std::max<int64_t>(4096, 16 * tot));
    chk(dalloc(&e->d_elog, e->elog_cap));
    chk(dalloc(&e->d_elog_count, 1));
    chk(dalloc(&e->d_elog_seq, ns));
    chk(dalloc(&e->d_flags, 1));
    chk(dalloc(&e->d_hit_slots, (size_t)HIT_CAP * ns));
    chk(dalloc(&e->d_keep, 1));
    chk(dalloc(&e->d_attempts, 3));
    if (rc) {
        free_all(e);
        delete e;
        return rc;
    }
    e->p.assign(p, p + nt);
    e->md.assign(md, md + nt);
    e->thr.assign(thr, thr + 5 * ns);
    // per disk: barycentric transform and time rescale as rg_create does
    std::vector<double> h(6 * nt);
    std::vector<int> base_of(nt);
    for (int s = 0; s < n_sys; s++) {
        const int b = e->base[s], n = e->ntot[s];
        std::vector<rg_vec_t> rr(r + b, r + b + n), vv(v + b, v + b + n);
        if (0 == std::fabs(rr[0].x) && 0 == std::fabs(rr[0].y) && 0 == std::fabs(rr[0].z) && 0 == std::fabs(vv[0].x) &&
            0 == std::fabs(vv[0].y) && 0 == std::fabs(vv[0].z)) {
            rg_vec_t R0{0, 0, 0, 0}, V0{0, 0, 0, 0};
            for (int j = n - 1; j >= 0; j--) {
                const double m = e->p[b + j].mass;
                R0.x += m * rr[j].x; R0.y += m * rr[j].y; R0.z += m * rr[j].z;
                V0.x += m * vv[j].x; V0.y += m * vv[j].y; V0.z += m * vv[j].z;
            }
            double M0 = 0.0;
            for (int j = n - 1; j >= 0; j--) M0 += e->p[b + j].mass;
            R0.x /= M0; R0.y /= M0; R0.z /= M0;
            V0.x /= M0; V0.y /= M0; V0.z /= M0;
            for (int j = n - 1; j >= 0; j--) {
                rr[j].x -= R0.x; rr[j].y -= R0.y; rr[j].z -= R0.z;
                vv[j].x -= V0.x; vv[j].y -= V0.y; vv[j].z -= V0.z;
            }
        }
        for (int j = 0; j < n; j++) {
            const size_t i = (size_t)b + j;
            h[i] = rr[j].x;
            h[nt + i] = rr[j].y;
            h[2 * nt + i] = rr[j].z;
            h[3 * nt + i] = vv[j].x / GAUSS;
            h[4 * nt + i] = vv[j].y / GAUSS;
            h[5 * nt + i] = vv[j].z / GAUSS;
            base_of[i] = b;
        }
    }
    std::vector<double> m(nt), R(nt);
    std::vector<int> id(nt), ty(nt);
    for (size_t i = 0; i < nt; i++) {
        m[i] = e->p[i].mass;
        R[i] = e->p[i].radius;
        id[i] = e->md[i].id;
        ty[i] = e->md[i].body_type;
    }
    chk(upload(e, e->d_y, h));
    chk(upload(e, e->d_mass, m));
    chk(upload(e, e->d_radius, R));
    chk(upload(e, e->d_id, id));
    chk(upload(e, e->d_type, ty));
    chk(upload(e, e->d_base_of, base_of));
    {
        std::vector<float> zf(8 * ns, 0.0f), zh(5 * ns, 0.0f);
        chk(upload(e, e->d_feat, zf));
        chk(upload(e, e->d_hist, zh));
        e->feat_red_init.assign(3 * ns, 0u);
        for (int d = 0; d < ns; d++) e->feat_red_init[3 * d + 1] = FEAT_H3_NONE_BITS;
        chk(upload(e, e->d_feat_red, e->feat_red_init));
    }
    chk(upload(e, e->d_thr, e->thr));
    chk(upload(e, e->d_prm, e->p));
    {
        std::vector<double> fr(ns);
        std::vector<int> nsi(ns);
        for (int s2 = 0; s2 < n_sys; s2++) {
            fr[s2] = e->thr[5 * (size_t)s2 + RG_THRESHOLD_RADII_ENHANCE_FACTOR];
            nsi[s2] = e->n_si(s2);
        }
        chk(upload(e, e->d_f_rad, fr));
        chk(upload(e, e->d_base, e->base));
        chk(upload(e, e->d_ntot, e->ntot));
        chk(upload(e, e->d_nsi, nsi));
    }
    std::vector<int> zi(ns, 0);
    std::vector<double> zd(ns, 0.0);
    std::vector<long long> zl(ns, 0);
    std::vector<unsigned int> zu(ns, 0);
    std::vector<unsigned long long> zb(ns, 0);
    chk(upload(e, e->d_status, zi));
    chk(upload(e, e->d_acc, zi));
    chk(upload(e, e->d_ej, zi));
    chk(upload(e, e->d_t, zd));
    chk(upload(e, e->d_tprev, zd));
    chk(upload(e, e->d_dt_did, zd));
    chk(upload(e, e->d_ntried, zl));
    chk(upload(e, e->d_npassed, zl));
    chk(upload(e, e->d_nfailed, zl));
    chk(upload(e, e->d_attempt, zu));
    chk(upload(e, e->d_acc_attempt, zu));
    chk(upload(e, e->d_nf0, zu));
    chk(upload(e, e->d_sys_events, zu));
    chk(upload(e, e->d_maxbits, zb));
    chk(upload(e, e->d_dt_last, zd));
    chk(upload(e, e->d_ideal_last, zd));
    chk(upload(e, e->d_proposed, zi));
    chk(upload(e, e->d_step_prop_rej, zi));
    chk(upload(e, e->d_prop_rej_steps, zi));
    chk(upload(e, e->d_cool, zi));
    chk(upload(e, e->d_nprop, zl));
    chk(upload(e, e->d_nprop_acc, zl));
    chk(upload(e, e->d_nfallback, zl));
    if (!rc && cudaMemsetAsync(e->d_ev_count, 0, sizeof(unsigned int), e->st) != cudaSuccess) chk(RG_ERR_CUDA);
    if (!rc && cudaMemsetAsync(e->d_hill_count, 0, sizeof(unsigned int), e->st) != cudaSuccess) chk(RG_ERR_CUDA);
    if (!rc && cudaMemsetAsync(e->d_kerr, 0, sizeof(unsigned int), e->st) != cudaSuccess) chk(RG_ERR_CUDA);
    for (auto z : {std::make_pair((void*)e->d_hill_n, ns * sizeof(int)),
                   std::make_pair((void*)e->d_hill_which, ns * sizeof(int)),
                   std::make_pair((void*)e->d_sym_ticket, ns * sizeof(unsigned int)),
                   std::make_pair((void*)e->d_elog_count, sizeof(unsigned int)),
                   std::make_pair((void*)e->d_elog_seq, ns * sizeof(unsigned int)),
                   std::make_pair((void*)e->d_flags, sizeof(unsigned int)),
                   std::make_pair((void*)e->d_attempts, 3 * sizeof(long long))})
        if (!rc && cudaMemsetAsync(z.first, 0, z.second, e->st) != cudaSuccess) chk(RG_ERR_CUDA);
    if (!rc && cudaStreamSynchronize(e->st) != cudaSuccess) chk(set_error(RG_ERR_CUDA, "upload"));
    if (rc) {
        free_all(e);
        delete e;
        return rc;
    }
    build_stage_tiles(e);
    build_gravity_plan(e);
    rc = upload_plans(e);
    if (rc) {
        free_all(e);
        delete e;
        return rc;
    }
    *out = e;
    return RG_OK;
}

// host view of the per-disk control arrays
struct Ctl {
    std::vector<int> status, active, active_f0;
    std::vector<double> t, t_stop;
};

int set_control(rg_ens* e, const std::vector<int>& status, bool fresh_f0)
{
    std::vector<int> active(e->n_sys), f0(e->n_sys);
    for (int s = 0; s < e->n_sys; s++) {
        active[s] = status[s] == RG_SYS_RUNNING;
        f0[s] = active[s] && fresh_f0;
    }
    int rc = upload(e, e->d_status, status);
    if (!rc) rc = upload(e, e->d_active, active);
    if (!rc) rc = upload(e, e->d_active_f0, f0);
    return rc;
}

int drain_log(rg_ens* e)
{
    if (!e->d_log) return RG_OK;
    unsigned int n = 0;
    RG_CUDA_CHECK(cudaMemcpyAsync(&n, e->d_log_count, sizeof(unsigned int), cudaMemcpyDeviceToHost, e->st));
    RG_CUDA_CHECK(cudaStreamSynchronize(e->st));
    if (n > e->log_cap) return set_error(RG_ERR_EVENT_OVERFLOW, "attempt log full between two host synchronisations");
    if (n == 0) return RG_OK;
    const size_t old = e->host_log.size();
    e->host_log.resize(old + n);
    RG_CUDA_CHECK(cudaMemcpyAsync(e->host_log.data() + old, e->d_log, n * sizeof(rg_step_rec_t), cudaMemcpyDeviceToHost,
                                  e->st));
    RG_CUDA_CHECK(cudaMemsetAsync(e->d_log_count, 0, sizeof(unsigned int), e->st));
    RG_CUDA_CHECK(cudaStreamSynchronize(e->st));
    // one thread per disk appended in slot order; within a disk the attempts are ordered
    std::stable_sort(e->host_log.begin() + old, e->host_log.end(),
                     [](const rg_step_rec_t& a, const rg_step_rec_t& b) { return a.sys < b.sys; });
    return RG_OK;
}

// After an advance: the device's event log (ordered per disk by record number), the body
// parameters and ids the merges changed (host mirrors), and the error bits.
int collect(rg_ens* e)
{
    int rc = drain_log(e);
    if (rc) return rc;
    unsigned int flags = 0, kerr = 0, n_log = 0;
    RG_CUDA_CHECK(cudaMemcpyAsync(&flags, e->d_flags, sizeof(unsigned int), cudaMemcpyDeviceToHost, e->st));
    RG_CUDA_CHECK(cudaMemcpyAsync(&kerr, e->d_kerr, sizeof(unsigned int), cudaMemcpyDeviceToHost, e->st));
    RG_CUDA_CHECK(cudaMemcpyAsync(&n_log, e->d_elog_count, sizeof(unsigned int), cudaMemcpyDeviceToHost, e->st));
    std::vector<rg_param_t> prm;
    std::vector<int> id;
    rc = download(e, prm, e->d_prm, (size_t)e->cap);
    if (!rc) rc = download(e, id, e->d_id, (size_t)e->cap);
    if (rc) return rc;
    RG_CUDA_CHECK(cudaStreamSynchronize(e->st));
    for (int i = 0; i < e->cap; i++) {
        e->p[i] = prm[i];
        e->md[i].id = id[i];
    }
    const unsigned int m = std::min(n_log, e->elog_cap);
    if (m > 0) {
        std::vector<EnsLogRec> recs;
        rc = download(e, recs, e->d_elog, m);
        if (rc) return rc;
        RG_CUDA_CHECK(cudaMemsetAsync(e->d_elog_count, 0, sizeof(unsigned int), e->st));
        RG_CUDA_CHECK(cudaStreamSynchronize(e->st));
        std::stable_sort(recs.begin(), recs.end(), [](const EnsLogRec& a, const EnsLogRec& b) {
            return a.sys != b.sys ? a.sys < b.sys : a.seqno < b.seqno;
        });
        for (const EnsLogRec& r : recs) e->log.emplace_back(r.sys, r.ev);
    }
    if (kerr) {
        RG_CUDA_CHECK(cudaMemsetAsync(e->d_kerr, 0, sizeof(unsigned int), e->st));
        return set_error(RG_ERR_CUDA, "a gravity tile copy did not arrive within the wait limit");
    }
    if (flags) {
        RG_CUDA_CHECK(cudaMemsetAsync(e->d_flags, 0, sizeof(unsigned int), e->st));
        RG_CUDA_CHECK(cudaStreamSynchronize(e->st));
        if (flags & ENS_FLAG_SUPERPLANETESIMAL)
            return set_error(RG_ERR_NOT_IMPLEMENTED, "collision with a super-planetesimal is not implemented");
        if (flags & ENS_FLAG_EVENT_OVERFLOW)
            return set_error(RG_ERR_EVENT_OVERFLOW, "more collision records in one attempt than the event buffer holds");
        if (flags & ENS_FLAG_HILL_OVERFLOW)
            return set_error(RG_ERR_EVENT_OVERFLOW, "more Hill records in one step start than the event buffer holds");
        if (flags & ENS_FLAG_LOG_OVERFLOW)
            return set_error(RG_ERR_EVENT_OVERFLOW, "the ensemble's event log is full (drain it with rg_ens_events)");
        if (flags & ENS_FLAG_HILL_SET)
            return set_error(RG_ERR_EVENT_OVERFLOW, "more pairs inside their Hill spheres than a disk's set holds");
        if (flags & ENS_FLAG_HIT_OVERFLOW)
            return set_error(RG_ERR_EVENT_OVERFLOW, "more hit-star records in one check than a disk's list holds");
        if (flags & ENS_FLAG_STEP_LOG_OVERFLOW)
            return set_error(RG_ERR_EVENT_OVERFLOW, "the attempt log is full (drain it with rg_ens_step_log)");
        return set_error(RG_ERR_STATE, "ensemble error flag");
    }
    return RG_OK;
}

// The stage vectors' storage follows the gravity mode (double-float pairs in the mixed form);
// the first one outlives an attempt (a rejected attempt retries from it), so after a change of
// mode it is converted in place before the next launch.
int ensure_k_format(rg_ens* e)
{
    const int want = e->gravity_mode == RG_GRAVITY_MIXED ? 1 : 0;
    if (e->k_f2_now == want) return RG_OK;
    const long long n = 6LL * e->cap;
    if (n > 0) {
        const long long blocks = std::min<long long>((n + 255) / 256, (long long)NUM_SMS_HINT * 16);
        k_format_kernel<<<(unsigned)blocks, 256, 0, e->st>>>(e->d_k[0], n, want);
        RG_CUDA_CHECK(cudaGetLastError());
    }
    e->k_f2_now = want;
    return RG_OK;
}

int advance_impl(rg_ens* e, double t_stop_day, int64_t max_attempts, int64_t* n_attempts)
{
    if (!e->has_int) return set_error(RG_ERR_STATE, "no integrator set (rg_ens_set_integrator)");
    if (int krc = ensure_k_format(e)) return krc;
    if (n_attempts) *n_attempts = 0;
    const double stop = t_stop_day * GAUSS;
    std::vector<int> status;
    std::vector<double> t;
    int rc = download(e, status, e->d_status, e->n_sys);
    if (!rc) rc = download(e, t, e->d_t, e->n_sys);
    if (rc) return rc;
    RG_CUDA_CHECK(cudaStreamSynchronize(e->st));
    for (int s = 0; s < e->n_sys; s++)
        if (status[s] != RG_SYS_ERROR) status[s] = (t[s] <= stop) ? RG_SYS_RUNNING : RG_SYS_DONE;
    std::vector<double> tstop(e->n_sys, stop);
    rc = upload(e, e->d_tstop, tstop);
    if (!rc) rc = set_control(e, status, true);
    if (rc) return rc;
    if (!e->started) {
        // the reference checks for ejection / hit-star before the first step (main.cu:201)
        ens_eject_screen_kernel<<<(int)e->stiles.size(), 256, 0, e->st>>>(e->d_stiles, e->d_active, e->d_y, e->cap,
                                                                          e->d_id, e->d_type, e->d_thr, e->d_ej);
        RG_CUDA_CHECK(cudaGetLastError());
        rc = launch_ens_handle(event_args(e), 1, e->st);
        if (rc) return rc;
        e->n_kernels += 2;
        e->started = 1;
    }
    // attempts in bounded chunks: a graph launch (or, with graphs off, a run of direct
    // launches) ends after ATTEMPT_CHUNK attempts at most, and the host starts the next chunk
    // while disks are running -- reading three words, handling nothing
    const long long limit = max_attempts > 0 ? (long long)max_attempts : 0;
    long long att = 0;
    for (;;) {
        const long long ctl[3] = {att, limit, att + ATTEMPT_CHUNK};
        const int one = 1;
        RG_CUDA_CHECK(cudaMemcpyAsync(e->d_attempts, ctl, sizeof(ctl), cudaMemcpyHostToDevice, e->st));
        RG_CUDA_CHECK(cudaMemcpyAsync(e->d_keep, &one, sizeof(int), cudaMemcpyHostToDevice, e->st));
        if (e->use_graph && !e->profiling) {
            // one launch: the while-node repeats the attempt until its last kernel clears the
            // condition (every disk done, an error bit, a limit)
            if (!e->graph_valid) rc = build_loop_graph(e);
            if (rc) return rc;
            RG_CUDA_CHECK(cudaGraphLaunch(e->exec, e->st));
            e->n_graph_launches++;
        } else {
            int keep = 1;
            while (keep) {  // direct launches, the condition read after each attempt
                rc = launch_attempt(e);
                if (rc) return rc;
                RG_CUDA_CHECK(cudaMemcpyAsync(&keep, e->d_keep, sizeof(int), cudaMemcpyDeviceToHost, e->st));
                RG_CUDA_CHECK(cudaStreamSynchronize(e->st));
            }
        }
        long long now = 0;
        int keep = 0;
        RG_CUDA_CHECK(cudaMemcpyAsync(&now, e->d_attempts, sizeof(long long), cudaMemcpyDeviceToHost, e->st));
        RG_CUDA_CHECK(cudaMemcpyAsync(&keep, e->d_keep, sizeof(int), cudaMemcpyDeviceToHost, e->st));
        RG_CUDA_CHECK(cudaStreamSynchronize(e->st));
        if (e->use_graph && !e->profiling) e->n_kernels += e->kernels_per_attempt * (now - att);
        att = now;
        // the loop stopped at the chunk's end only when nothing else stopped it
        if (keep || att < ctl[2] || (limit > 0 && att >= limit)) break;
        unsigned int flags = 0;
        std::vector<int> st;
        RG_CUDA_CHECK(cudaMemcpyAsync(&flags, e->d_flags, sizeof(unsigned int), cudaMemcpyDeviceToHost, e->st));
        rc = download(e, st, e->d_status, e->n_sys);
        if (rc) return rc;
        RG_CUDA_CHECK(cudaStreamSynchronize(e->st));
        bool running = false;
        for (int s = 0; s < e->n_sys; s++) running = running || st[s] == RG_SYS_RUNNING;
        if (!running || flags) break;
    }
    e->n_attempts += att;
    if (n_attempts) *n_attempts = att;
    rc = collect(e);
    if (rc) return rc;
    rc = download(e, status, e->d_status, e->n_sys);
    if (rc) return rc;
    RG_CUDA_CHECK(cudaStreamSynchronize(e->st));
    for (int s = 0; s < e->n_sys; s++)
        if (status[s] == RG_SYS_ERROR)
            return set_error(RG_ERR_DT_NONFINITE, "a disk's step-size controller produced a non-finite or zero step");
    return RG_OK;
}

int get_state_impl(rg_ens* e, int s, rg_vec_t* r, rg_vec_t* v, rg_param_t* p, rg_body_metadata_t* md, double* t_day)
{
    const int b = e->base[s], n = e->ntot[s];
    std::vector<double> h((size_t)6 * n);
    double t = 0.0;
    RG_CUDA_CHECK(cudaMemcpy2DAsync(h.data(), n * sizeof(double), e->d_y + b, e->cap * sizeof(double),
                                    n * sizeof(double), 6, cudaMemcpyDeviceToHost, e->st));
    RG_CUDA_CHECK(cudaMemcpyAsync(&t, e->d_t + s, sizeof(double), cudaMemcpyDeviceToHost, e->st));
    RG_CUDA_CHECK(cudaStreamSynchronize(e->st));
    for (int i = 0; i < n; i++) {
        if (r) r[i] = rg_vec_t{h[i], h[(size_t)n + i], h[(size_t)2 * n + i], 0.0};
        if (v)
            v[i] = rg_vec_t{h[(size_t)3 * n + i] * GAUSS, h[(size_t)4 * n + i] * GAUSS, h[(size_t)5 * n + i] * GAUSS, 0.0};
    }
    if (p) std::memcpy(p, e->p.data() + b, (size_t)n * sizeof(rg_param_t));
    if (md) std::memcpy(md, e->md.data() + b, (size_t)n * sizeof(rg_body_metadata_t));
    if (t_day) *t_day = t / GAUSS;
    return RG_OK;
}

int stats_impl(rg_ens* e, int s, rg_ens_stats_t* o)
{
    double t, dtt, dtd;
    long long a, b, c;
    int st;
    RG_CUDA_CHECK(cudaMemcpyAsync(&t, e->d_t + s, sizeof(double), cudaMemcpyDeviceToHost, e->st));
    RG_CUDA_CHECK(cudaMemcpyAsync(&dtt, e->d_dt_try + s, sizeof(double), cudaMemcpyDeviceToHost, e->st));
    RG_CUDA_CHECK(cudaMemcpyAsync(&dtd, e->d_dt_did + s, sizeof(double), cudaMemcpyDeviceToHost, e->st));
    RG_CUDA_CHECK(cudaMemcpyAsync(&a, e->d_ntried + s, sizeof(long long), cudaMemcpyDeviceToHost, e->st));
    RG_CUDA_CHECK(cudaMemcpyAsync(&b, e->d_npassed + s, sizeof(long long), cudaMemcpyDeviceToHost, e->st));
    RG_CUDA_CHECK(cudaMemcpyAsync(&c, e->d_nfailed + s, sizeof(long long), cudaMemcpyDeviceToHost, e->st));
    RG_CUDA_CHECK(cudaMemcpyAsync(&st, e->d_status + s, sizeof(int), cudaMemcpyDeviceToHost, e->st));
    RG_CUDA_CHECK(cudaStreamSynchronize(e->st));
    std::memset(o, 0, sizeof(*o));
    o->t_day = t / GAUSS;
    o->dt_try_day = dtt / GAUSS;
    o->dt_did_day = dtd / GAUSS;
    o->n_tried_step = a;
    o->n_passed_step = b;
    o->n_failed_step = c;
    o->status = st;
    o->n_total = e->ntot[s];
    long long pr, pa, fb;
    RG_CUDA_CHECK(cudaMemcpyAsync(&pr, e->d_nprop + s, sizeof(long long), cudaMemcpyDeviceToHost, e->st));
    RG_CUDA_CHECK(cudaMemcpyAsync(&pa, e->d_nprop_acc + s, sizeof(long long), cudaMemcpyDeviceToHost, e->st));
    RG_CUDA_CHECK(cudaMemcpyAsync(&fb, e->d_nfallback + s, sizeof(long long), cudaMemcpyDeviceToHost, e->st));
    RG_CUDA_CHECK(cudaStreamSynchronize(e->st));
    o->n_proposed = pr;
    o->n_proposal_accepted = pa;
    o->n_fallback = fb;
    return RG_OK;
}

int energy_impl(rg_ens* e, int s, double* energy, double* angmom)
{
    const int n = e->ntot[s];
    if (!e->d_part) {
        int rc = dalloc(&e->d_part, (size_t)5 * e->cap);
        if (rc) return rc;
    }
    ens_energy_kernel<<<(n + 127) / 128, 128, 0, e->st>>>(e->d_y, e->d_mass, e->d_id, e->cap, e->base[s], n, e->n_si(s),
                                                          e->n_massive(s), e->d_part);
    RG_CUDA_CHECK(cudaGetLastError());
    e->n_kernels++;
    std::vector<double> h;
    int rc = download(e, h, e->d_part, (size_t)5 * n);
    if (rc) return rc;
    RG_CUDA_CHECK(cudaStreamSynchronize(e->st));
    double sum[5], comp[5];
    for (int q = 0; q < 5; q++) {
        sum[q] = comp[q] = 0.0;
        for (int i = 0; i < n; i++) {
            const double x = h[(size_t)q * n + i];
            const double tt = sum[q] + x;
            comp[q] += std::fabs(sum[q]) >= std::fabs(x) ? (sum[q] - tt) + x : (x - tt) + sum[q];
            sum[q] = tt;
        }
    }
    if (energy) *energy = (sum[0] + comp[0]) + (sum[1] + comp[1]);
    if (angmom)
        for (int q = 0; q < 3; q++) angmom[q] = sum[2 + q] + comp[2 + q];
    return RG_OK;
}

}  // namespace

extern "C" {

int rg_ens_create(int n_sys, const rg_counts_t* counts, const rg_vec_t* r, const rg_vec_t* v, const rg_param_t* p,
                  const rg_body_metadata_t* md, const double* thr, int event_capacity, rg_ens** out)
{
    RG_GUARD(create_impl(n_sys, counts, r, v, p, md, thr, event_capacity, out));
}

int rg_ens_destroy(rg_ens* e)
{
    if (!e) return set_error(RG_ERR_ARG, "null ensemble");
    cudaStreamSynchronize(e->st);
    free_all(e);
    delete e;
    return RG_OK;
}

int rg_ens_set_integrator(rg_ens* e, double dt_day, double tol, int error_check_for_tp)
{
    if (!e || !(dt_day > 0.0) || !(tol > 0.0)) return set_error(RG_ERR_ARG, "bad argument");
    e->tol = tol;
    e->dt0 = dt_day * GAUSS;
    e->ectp = error_check_for_tp ? 1 : 0;
    std::vector<double> dt(e->n_sys, e->dt0);
    int rc = upload(e, e->d_dt_try, dt);
    if (rc) return rc;
    RG_CUDA_CHECK(cudaStreamSynchronize(e->st));
    build_stage_tiles(e);
    rc = upload_plans(e);
    if (!rc) e->has_int = 1;
    return rc;
}

int rg_ens_set_options(rg_ens* e, int gravity_mode, double hill_factor, int use_graph)
{
    if (!e || (gravity_mode != RG_GRAVITY_FP64 && gravity_mode != RG_GRAVITY_MIXED) || !(hill_factor >= 0.0))
        return set_error(RG_ERR_ARG, "bad option");
    e->gravity_mode = gravity_mode;
    e->hill_factor = hill_factor;
    e->use_graph = use_graph ? 1 : 0;
    e->graph_valid = false;
    return RG_OK;
}

int rg_ens_advance(rg_ens* e, double t_stop_day, int64_t max_attempts, int64_t* n_attempts)
{
    if (!e) return set_error(RG_ERR_ARG, "null ensemble");
    RG_GUARD(advance_impl(e, t_stop_day, max_attempts, n_attempts));
}

int rg_ens_get_state(rg_ens* e, int sys, rg_vec_t* r, rg_vec_t* v, rg_param_t* p, rg_body_metadata_t* md,
                     double* t_day)
{
    if (!e || sys < 0 || sys >= e->n_sys) return set_error(RG_ERR_ARG, "bad disk index");
    RG_GUARD(get_state_impl(e, sys, r, v, p, md, t_day));
}

int rg_ens_get_stats(rg_ens* e, int sys, rg_ens_stats_t* o)
{
    if (!e || !o || sys < 0 || sys >= e->n_sys) return set_error(RG_ERR_ARG, "bad argument");
    RG_GUARD(stats_impl(e, sys, o));
}

int rg_ens_events(rg_ens* e, rg_event_t* out, int* sys_of_event, int cap, int* n)
{
    if (!e || !n || cap < 0 || (cap > 0 && !out)) return set_error(RG_ERR_ARG, "bad argument");
    const int m = std::min<int>((int)e->log.size(), cap);
    for (int k = 0; k < m; k++) {
        out[k] = e->log[k].second;
        if (sys_of_event) sys_of_event[k] = e->log[k].first;
    }
    e->log.erase(e->log.begin(), e->log.begin() + m);
    *n = m;
    return RG_OK;
}

int rg_ens_event_count(rg_ens* e, int* n)
{
    if (!e || !n) return set_error(RG_ERR_ARG, "bad argument");
    *n = (int)e->log.size();
    return RG_OK;
}

int rg_ens_set_step_log(rg_ens* e, int capacity)
{
    if (!e || capacity < 0) return set_error(RG_ERR_ARG, "bad argument");
    cudaFree(e->d_log);
    cudaFree(e->d_log_count);
    e->d_log = nullptr;
    e->d_log_count = nullptr;
    e->log_cap = 0;
    if (capacity > 0) {
        int rc = dalloc(&e->d_log, (size_t)capacity);
        if (!rc) rc = dalloc(&e->d_log_count, 1);
        if (rc) return rc;
        RG_CUDA_CHECK(cudaMemsetAsync(e->d_log_count, 0, sizeof(unsigned int), e->st));
        RG_CUDA_CHECK(cudaStreamSynchronize(e->st));
        e->log_cap = (unsigned int)capacity;
    }
    e->graph_valid = false;
    return RG_OK;
}

int rg_ens_step_log(rg_ens* e, rg_step_rec_t* out, int cap, int* n)
{
    if (!e || !n || cap < 0 || (cap > 0 && !out)) return set_error(RG_ERR_ARG, "bad argument");
    int rc = drain_log(e);
    if (rc) return rc;
    // records of one disk stay in attempt order across drains: stable by disk on output
    std::stable_sort(e->host_log.begin(), e->host_log.end(),
                     [](const rg_step_rec_t& a, const rg_step_rec_t& b) { return a.sys < b.sys; });
    const int m = std::min<int>((int)e->host_log.size(), cap);
    if (m > 0) std::memcpy(out, e->host_log.data(), (size_t)m * sizeof(rg_step_rec_t));
    e->host_log.erase(e->host_log.begin(), e->host_log.begin() + m);
    *n = m;
    return RG_OK;
}

int rg_ens_energy(rg_ens* e, int sys, double* energy, double angmom[3])
{
    if (!e || sys < 0 || sys >= e->n_sys) return set_error(RG_ERR_ARG, "bad disk index");
    RG_GUARD(energy_impl(e, sys, energy, angmom));
}

int rg_ens_set_proposer(rg_ens* e, rg_mlp* mlp, double safety, int cooldown)
{
    if (!e || (mlp && !(safety > 0.0 && safety <= 1.5)) || cooldown < 0) return set_error(RG_ERR_ARG, "bad argument");
    e->mlp = mlp;
    if (mlp) {
        float mean[8], sd[8];
        redgb::mlp_normalisation(mlp, mean, sd);
        for (int q = 0; q < 8; q++) {
            e->mlp_mean[q] = mean[q];
            e->mlp_inv_std[q] = 1.0f / sd[q];
        }
        e->safety = (float)safety;
        e->cooldown = cooldown;
    }
    e->graph_valid = false;
    return RG_OK;
}

int rg_ens_set_dither(rg_ens* e, double sigma, uint64_t seed)
{
    if (!e || !(sigma >= 0.0 && sigma <= 1.0)) return set_error(RG_ERR_ARG, "dither must be in [0, 1]");
    e->dither = (float)sigma;
    e->dither_seed = (unsigned long long)seed;
    e->graph_valid = false;
    return RG_OK;
}

int rg_ens_get_stream(rg_ens* e, void** stream)
{
    if (!e || !stream) return set_error(RG_ERR_ARG, "bad argument");
    *stream = (void*)e->st;
    return RG_OK;
}

// CUDA-event time of one gravity evaluation of every disk (stage-0 form, no event records)
// on the step-start state, written to a stage buffer; `reps` evaluations after a warm-up
static int time_ens_evaluations(rg_ens* e, int reps, double* ms)
{
    const size_t cap = (size_t)e->cap;
    double* acc = e->d_k[0] + 3 * cap;
    int rc = ens_gravity(e, e->d_y, e->d_y + 3 * cap, acc, 0, nullptr, false);
    if (rc) return rc;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    RG_CUDA_CHECK(cudaEventCreate(&e0));
    if (cudaEventCreate(&e1) != cudaSuccess) {
        cudaEventDestroy(e0);
        return set_error(RG_ERR_CUDA, "cudaEventCreate");
    }
    cudaEventRecord(e0, e->st);
    for (int k = 0; k < reps && !rc; k++) rc = ens_gravity(e, e->d_y, e->d_y + 3 * cap, acc, 0, nullptr, false);
    cudaEventRecord(e1, e->st);
    cudaError_t err = cudaEventSynchronize(e1);
    float t = 0.0f;
    if (!rc && err == cudaSuccess) err = cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    if (err != cudaSuccess) return set_error(RG_ERR_CUDA, "autotune timing");
    *ms = t / std::max(1, reps);
    return RG_OK;
}

// the ensemble's tile shapes, timed on its own disks: FP64 mode sinks per pair-parallel CTA x
// the row-kernel source limit (each candidate sums in the reference's order: results stay
// bit-exact), mixed mode sources per few-sink CTA x the row-kernel limit
static int ens_autotune_impl(rg_ens* e, int reps, rg_tune_t* out)
{
    if (int krc = ensure_k_format(e)) return krc;
    struct Shape {
        int S, rowseq, chunk;
    };
    std::vector<Shape> cand;
    const int rows[3] = {32, 64, 128};
    if (e->gravity_mode == RG_GRAVITY_MIXED) {
        const int ch[4] = {0, 512, 1024, 2048};
        for (int r : rows)
            for (int k : ch) cand.push_back({e->pairpar_S, r, k});
    } else {
        const int ss[3] = {8, 16, 32};
        for (int r : rows)
            for (int S : ss) cand.push_back({S, r, e->few_chunk});
    }
    const int64_t kernels = e->n_kernels;
    const Shape before{e->pairpar_S, e->rowseq_max_src, e->few_chunk};
    double ms_before = 0.0;
    int rc = time_ens_evaluations(e, reps, &ms_before);
    Shape best = before;
    double best_ms = ms_before;
    for (const Shape& sh : cand) {
        if (rc) break;
        e->pairpar_S = sh.S;
        e->rowseq_max_src = sh.rowseq;
        e->few_chunk = sh.chunk;
        build_gravity_plan(e);
        rc = upload_plans(e);
        double ms = 0.0;
        if (!rc) rc = time_ens_evaluations(e, reps, &ms);
        if (!rc && ms < best_ms) {
            best_ms = ms;
            best = sh;
        }
    }
    e->pairpar_S = best.S;
    e->rowseq_max_src = best.rowseq;
    e->few_chunk = best.chunk;
    build_gravity_plan(e);
    const int rc2 = upload_plans(e);
    if (!rc) rc = rc2;
    e->n_kernels = kernels;
    if (rc) return rc;
    if (out) {
        out->pairpar_sinks = best.S;
        out->rowseq_max_src = best.rowseq;
        out->mixed_chunks = best.chunk;
        out->candidates = (int32_t)cand.size();
        out->ms_per_eval = best_ms;
        out->ms_before = ms_before;
    }
    return RG_OK;
}

int rg_ens_autotune(rg_ens* e, int reps, rg_tune_t* out)
{
    if (!e || reps < 1) return set_error(RG_ERR_ARG, "bad argument");
    RG_GUARD(ens_autotune_impl(e, reps, out));
}

int rg_ens_set_profiling(rg_ens* e, int on)
{
    if (!e) return set_error(RG_ERR_ARG, "null ensemble");
    e->profiling = on ? 1 : 0;
    return RG_OK;
}

int rg_ens_get_profile(rg_ens* e, rg_profile_t* prof)
{
    if (!e || !prof) return set_error(RG_ERR_ARG, "bad argument");
    std::memset(prof, 0, sizeof(*prof));
    RG_CUDA_CHECK(cudaStreamSynchronize(e->st));
    for (size_t k = 0; k < e->ev_kind.size(); k++) {
        float ms = 0.0f;
        RG_CUDA_CHECK(cudaEventElapsedTime(&ms, e->ev_pool[2 * k], e->ev_pool[2 * k + 1]));
        if (e->ev_kind[k] == 0) {
            prof->gravity_launches++;
            prof->gravity_ms += ms;
        } else if (e->ev_kind[k] == 1) {
            prof->stage_launches++;
            prof->stage_ms += ms;
        } else {
            prof->other_launches++;
            prof->other_ms += ms;
        }
    }
    e->ev_kind.clear();
    e->ev_used = 0;
    return RG_OK;
}

int rg_ens_kernel_count(rg_ens* e, int64_t* n_kernels, int64_t* n_graph_launches)
{
    if (!e) return set_error(RG_ERR_ARG, "null ensemble");
    if (n_kernels) *n_kernels = e->n_kernels;
    if (n_graph_launches) *n_graph_launches = e->n_graph_launches;
    return RG_OK;
}

}  // extern "C"
