// stages.cu -- Runge-Kutta stage combination, the embedded error norm and the
// ejection / hit-star screen.  Compiled with -fmad=false: every expression keeps the
// reference's operation order so the results equal its CPU path bit for bit.
//
// The state and the stage derivatives are 6 rows of n doubles ([r | v] and [dr/dt | dv/dt],
// common.cuh), so one elementwise pass covers positions and velocities.  A stage combine
// writes its positions to the stage position rows (read by the gravity kernel) and its
// velocities straight into the dr/dt rows of the new stage: the reference's device-to-device
// copy dy <- v (pp_disk.cu:1013) disappears.  The error kernel reduces to the one number the
// step controller needs (signed maximum, integrator.cu:211-256) with warp shuffles and one
// 64-bit atomic per CTA instead of materialising the error vectors.
//
// Roofline: all kernels here are HBM-bound streams (algorithmic bytes per body are listed
// with each kernel).
#include "common.cuh"
#include "kernels.h"

namespace redgb {




template <int FORM, int NTERM>
__global__ void __launch_bounds__(256) combine_kernel(CombineArgs a)
{
    const double dt = *a.dt;
    const long long total = 6LL * a.n;
    for (long long f = blockIdx.x * (long long)blockDim.x + threadIdx.x; f < total;
         f += (long long)gridDim.x * blockDim.x) {
        const int row = (int)(f / a.n);
        const long long b = f - (long long)row * a.n;
        const long long e = (long long)row * a.stride + b;
        const double y = a.y[e];
        double out;
        if (FORM == FORM_SUM) {
            double sum = a.c[0] * a.k[0][e];
#pragma unroll
            for (int q = 1; q < NTERM; q++) sum = sum + a.c[q] * a.k[q][e];
            out = y + dt * sum;
        } else if (FORM == FORM_SCALED) {
            out = y + (a.c[0] * dt) * a.k[0][e];
        } else if (FORM == FORM_ACC) {
            double acc = y;
#pragma unroll
            for (int q = 0; q < NTERM; q++) acc = acc + dt * a.c[q] * a.k[q][e];
            out = acc;
        } else if (FORM == FORM_RK4_NP1) {
            const double b0 = a.c[0] * dt, b1 = a.c[1] * dt;
            out = y + b0 * (a.k[0][e] + a.k[3][e]) + b1 * (a.k[1][e] + a.k[2][e]);
        } else {  // FORM_RK8_NP1: k = {k0, k5, k6, k7, k8, k9, k10}, c = {b0, b5, b6, b8, b10}
            out = y + dt * (a.c[0] * a.k[0][e] + a.c[1] * a.k[1][e] + a.c[2] * (a.k[2][e] + a.k[3][e]) +
                            a.c[3] * (a.k[4][e] + a.k[5][e]) + a.c[4] * a.k[6][e]);
        }
        if (row < 3)
            a.out_lo[e] = out;
        else
            a.out_hi[e - 3LL * a.stride] = out;
    }
}

static int grid_for(long long total, int threads = 256)
{
    long long b = (total + threads - 1) / threads;
    if (b > 152LL * 16) b = 152LL * 16;  // grid-stride beyond 16 CTAs per SM
    return (int)(b < 1 ? 1 : b);
}

int launch_combine(const CombineArgs& a, cudaStream_t st)
{
    const int g = grid_for(6LL * a.n);
#define RG_LAUNCH(F, T) combine_kernel<F, T><<<g, 256, 0, st>>>(a)
    switch (a.form) {
    case FORM_SUM:
        switch (a.nterm) {
        case 1: RG_LAUNCH(FORM_SUM, 1); break;
        case 2: RG_LAUNCH(FORM_SUM, 2); break;
        case 3: RG_LAUNCH(FORM_SUM, 3); break;
        case 4: RG_LAUNCH(FORM_SUM, 4); break;
        case 5: RG_LAUNCH(FORM_SUM, 5); break;
        case 6: RG_LAUNCH(FORM_SUM, 6); break;
        case 7: RG_LAUNCH(FORM_SUM, 7); break;
        case 8: RG_LAUNCH(FORM_SUM, 8); break;
        case 9: RG_LAUNCH(FORM_SUM, 9); break;
        default: return -1;
        }
        break;
    case FORM_SCALED: RG_LAUNCH(FORM_SCALED, 1); break;
    case FORM_ACC:
        switch (a.nterm) {
        case 1: RG_LAUNCH(FORM_ACC, 1); break;
        case 2: RG_LAUNCH(FORM_ACC, 2); break;
        case 3: RG_LAUNCH(FORM_ACC, 3); break;
        case 4: RG_LAUNCH(FORM_ACC, 4); break;
        case 5: RG_LAUNCH(FORM_ACC, 5); break;
        default: return -1;
        }
        break;
    case FORM_RK4_NP1: RG_LAUNCH(FORM_RK4_NP1, 4); break;
    case FORM_RK8_NP1: RG_LAUNCH(FORM_RK8_NP1, 7); break;
    default: return -1;
    }
#undef RG_LAUNCH
    RG_CUDA_CHECK(cudaGetLastError());
    return 0;
}

// ---------------------------------------------------------------------------------------
// Embedded error estimate fused with its maximum.
//   ERR_RK4 : e = k3 - k4                                 (int_rungekutta4.cu:63-74)
//   ERR_RK5 : e = (bh0-b0) k0 + sum_{q>=1} (bhq-bq) kq     (int_rungekutta5.cu:79-93)
//   ERR_RK8 : e = ((k0 + k10) - k11) - k12                 (int_rungekutta8.cu:307-319)
// Over the first n_err bodies of each of the 6 rows (massive bodies, or all with
// error_check_for_tp).  The maximum starts at 0 and ignores NaN exactly as the CPU branch
// of integrator::get_max_error does; the result is >= 0, so its bit pattern orders like
// an unsigned integer and one atomicMax per CTA combines the blocks.


template <int FORM>
__global__ void __launch_bounds__(256) error_max_kernel(ErrArgs a)
{
    double m = 0.0;
    const long long total = 6LL * a.n_err;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const long long row = e / a.n_err;
        const long long idx = row * a.stride + (e - row * a.n_err);
        double v;
        if (FORM == ERR_RK4) {
            v = a.k[0][idx] - a.k[1][idx];
        } else if (FORM == ERR_RK5) {
            v = a.c[0] * a.k[0][idx];
#pragma unroll
            for (int q = 1; q < 6; q++) v = v + a.c[q] * a.k[q][idx];
        } else {
            v = (a.k[0][idx] + a.k[1][idx] - a.k[2][idx] - a.k[3][idx]);
        }
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
        m = lane < (blockDim.x >> 5) ? wmax[lane] : 0.0;
#pragma unroll
        for (int off = 4; off > 0; off >>= 1) {
            const double o = __shfl_xor_sync(0xffffffffu, m, off);
            if (m < o) m = o;
        }
        if (lane == 0 && m > 0.0) atomicMax(a.max_bits, (unsigned long long)__double_as_longlong(m));
    }
}

int launch_error_max(const ErrArgs& a, cudaStream_t st)
{
    const int g = grid_for(6LL * (a.n_err > 0 ? a.n_err : 1));
    if (a.n_err <= 0) return 0;
    switch (a.form) {
    case ERR_RK4: error_max_kernel<ERR_RK4><<<g, 256, 0, st>>>(a); break;
    case ERR_RK5: error_max_kernel<ERR_RK5><<<g, 256, 0, st>>>(a); break;
    default: error_max_kernel<ERR_RK8><<<g, 256, 0, st>>>(a); break;
    }
    RG_CUDA_CHECK(cudaGetLastError());
    return 0;
}

// ---------------------------------------------------------------------------------------
// Ejection / hit-star screen (kernel_pp_disk::check_for_ejection_hit_centrum,
// pp_disk.cu:72-142; CPU twin 934-976): distance from the origin of every active body
// that is not a star.  Candidates are listed as (index, kind, r^2); the host applies them
// in index order, as the CPU loop does.

__global__ void ejection_kernel(const double* __restrict__ x, const double* __restrict__ y,
                                const double* __restrict__ z, const int* __restrict__ id,
                                const int* __restrict__ type, int n, double thr_hit, double thr_ej, double thr_hit2,
                                double thr_ej2, EjectRec* rec, unsigned int* count, unsigned int cap)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (0 < id[i] && type[i] != 0) {
        const double r2 = x[i] * x[i] + y[i] * y[i] + z[i] * z[i];
        int kind = 0;
        if (0.0 < thr_ej && thr_ej2 < r2)
            kind = 2;
        else if (0.0 < thr_hit && thr_hit2 > r2)
            kind = 1;
        if (kind) {
            unsigned int slot = atomicAdd(count, 1u);
            if (slot < cap) {
                rec[slot].i = i;
                rec[slot].kind = kind;
                rec[slot].r2 = r2;
            }
        }
    }
}

int launch_ejection(const double* x, const double* y, const double* z, const int* id, const int* type, int n,
                    const double* thr, EjectRec* rec, unsigned int* count, unsigned int cap, cudaStream_t st)
{
    if (n <= 0) return 0;
    ejection_kernel<<<(n + 255) / 256, 256, 0, st>>>(x, y, z, id, type, n, thr[0], thr[1], thr[3], thr[4], rec, count,
                                                     cap);
    RG_CUDA_CHECK(cudaGetLastError());
    return 0;
}

// ---------------------------------------------------------------------------------------
// State records <-> the state rows.  Records are the reference's vec_t {x, y, z, w} (4
// doubles; r in AU, v in AU/day, w = 0), rows the integrator's SoA (v in AU per k-scaled
// day).  On the way in velocities are divided by k (the load transform, pp_disk.cu:1498-1551),
// on the way out multiplied by it (print_result_ascii, pp_disk.cu:1720-1722) when `scale`:
// single IEEE operations, as the host loops round them.

__global__ void records_to_rows_kernel(const double* __restrict__ r, const double* __restrict__ v, int n,
                                       int stride, double k, double* __restrict__ y)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const size_t s = (size_t)stride;
    for (int c = 0; c < 3; c++) {
        y[c * s + i] = r[4 * (size_t)i + c];
        y[(3 + c) * s + i] = __ddiv_rn(v[4 * (size_t)i + c], k);
    }
}

__global__ void rows_to_records_kernel(const double* __restrict__ y, int n, int stride, double k, bool scale,
                                       double* __restrict__ r, double* __restrict__ v)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const size_t s = (size_t)stride;
    for (int c = 0; c < 3; c++) {
        r[4 * (size_t)i + c] = y[c * s + i];
        const double vc = y[(3 + c) * s + i];
        v[4 * (size_t)i + c] = scale ? __dmul_rn(vc, k) : vc;
    }
    r[4 * (size_t)i + 3] = 0.0;
    v[4 * (size_t)i + 3] = 0.0;
}

int launch_records_to_rows(const double* r, const double* v, int n, int stride, double k, double* y, cudaStream_t st)
{
    if (n <= 0) return 0;
    records_to_rows_kernel<<<(n + 255) / 256, 256, 0, st>>>(r, v, n, stride, k, y);
    RG_CUDA_CHECK(cudaGetLastError());
    return 0;
}

int launch_rows_to_records(const double* y, int n, int stride, double k, bool scale, double* r, double* v,
                           cudaStream_t st)
{
    if (n <= 0) return 0;
    rows_to_records_kernel<<<(n + 255) / 256, 256, 0, st>>>(y, n, stride, k, scale, r, v);
    RG_CUDA_CHECK(cudaGetLastError());
    return 0;
}

// Compaction of the state rows (the device side of pp_disk::remove_inactive_bodies,
// pp_disk.cu:1324-1409): dst row c, column k = src row c, column keep[k], for the 6 rows of
// positions and velocities.  Pure data movement, so the compacted state is bit-identical to
// the one a host copy makes.
__global__ void gather_rows_kernel(const double* __restrict__ src, double* __restrict__ dst, int stride,
                                   const int* __restrict__ keep, int n)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const size_t s = (size_t)stride;
    const int i = keep[k];
    for (int c = 0; c < 6; c++) dst[c * s + k] = src[c * s + i];
}

int launch_gather_rows(const double* src, double* dst, int stride, const int* keep, int n, cudaStream_t st)
{
    if (n <= 0) return 0;
    gather_rows_kernel<<<(n + 255) / 256, 256, 0, st>>>(src, dst, stride, keep, n);
    RG_CUDA_CHECK(cudaGetLastError());
    return 0;
}

// ---------------------------------------------------------------------------------------
// Energy and angular momentum partials (not in the reference).  Per body i: kinetic
// energy, the potential of the pairs (i, j < i) the force model couples (all j < i for a
// self-interacting body, j < n_si for a planetesimal), and m r x v, each summed with a
// Neumaier compensation.  The host adds the per-body partials in index order.

__global__ void energy_kernel(EnergyArgs a)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const int n = a.n;
    const long long sd = a.stride;
    const double* rx = a.y;
    const double* ry = a.y + sd;
    const double* rz = a.y + 2 * sd;
    const double* vx = a.y + 3 * sd;
    const double* vy = a.y + 4 * sd;
    const double* vz = a.y + 5 * sd;
    double T = 0, U = 0, Uc = 0, Lx = 0, Ly = 0, Lz = 0;
    if (a.id[i] > 0) {
        const double m = a.mass[i];
        T = 0.5 * m * (vx[i] * vx[i] + vy[i] * vy[i] + vz[i] * vz[i]);
        Lx = m * (ry[i] * vz[i] - rz[i] * vy[i]);
        Ly = m * (rz[i] * vx[i] - rx[i] * vz[i]);
        Lz = m * (rx[i] * vy[i] - ry[i] * vx[i]);
        if (i >= 1 && i < a.n_massive) {
            const int jmax = i < a.n_si ? i : a.n_si;
            for (int j = 0; j < jmax; j++) {
                if (a.id[j] <= 0) continue;
                const double dx = rx[j] - rx[i], dy = ry[j] - ry[i], dz = rz[j] - rz[i];
                const double d = sqrt(dx * dx + dy * dy + dz * dz);
                const double term = -(m * a.mass[j]) / d;
                const double t = U + term;
                if (fabs(U) >= fabs(term))
                    Uc += (U - t) + term;
                else
                    Uc += (term - t) + U;
                U = t;
            }
        }
    }
    a.part[i] = T;
    a.part[n + i] = U + Uc;
    a.part[2 * (long long)n + i] = Lx;
    a.part[3 * (long long)n + i] = Ly;
    a.part[4 * (long long)n + i] = Lz;
}

int launch_energy(const EnergyArgs& a, cudaStream_t st)
{
    if (a.n <= 0) return 0;
    energy_kernel<<<(a.n + 127) / 128, 128, 0, st>>>(a);
    RG_CUDA_CHECK(cudaGetLastError());
    return 0;
}

// ---------------------------------------------------------------------------------------
// Pipe-peak microbenchmark: CH independent FMA chains per thread, every SM busy.
template <class T, int CH>
__global__ void __launch_bounds__(256) fma_peak_kernel(T a, T b, int iters, T* sink)
{
    T acc[CH];
#pragma unroll
    for (int k = 0; k < CH; k++) acc[k] = (T)(threadIdx.x + k);
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int k = 0; k < CH; k++) acc[k] = fma(acc[k], a, b);
    }
    T s = 0;
#pragma unroll
    for (int k = 0; k < CH; k++) s += acc[k];
    if (s == (T)-1.2345) sink[0] = s;  // keeps the chains alive
}

int measure_pipe_peak(int kind, double* tflops)
{
    int dev = 0, sms = 0;
    RG_CUDA_CHECK(cudaGetDevice(&dev));
    RG_CUDA_CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    double* sink = nullptr;
    RG_CUDA_CHECK(cudaMalloc(&sink, 64));
    cudaEvent_t e0, e1;
    RG_CUDA_CHECK(cudaEventCreate(&e0));
    RG_CUDA_CHECK(cudaEventCreate(&e1));
    const int blocks = sms * 8, threads = 256;
    const int iters = kind == 0 ? 8192 : 256;
    constexpr int CH = 8;
    float best = 1e30f;
    for (int rep = 0; rep < 4; rep++) {
        RG_CUDA_CHECK(cudaEventRecord(e0));
        if (kind == 0)
            fma_peak_kernel<float, CH><<<blocks, threads>>>(0.999f, 1e-3f, iters, (float*)sink);
        else
            fma_peak_kernel<double, CH><<<blocks, threads>>>(0.999, 1e-3, iters, sink);
        RG_CUDA_CHECK(cudaGetLastError());
        RG_CUDA_CHECK(cudaEventRecord(e1));
        RG_CUDA_CHECK(cudaEventSynchronize(e1));
        float ms = 0.0f;
        RG_CUDA_CHECK(cudaEventElapsedTime(&ms, e0, e1));
        if (rep > 0 && ms < best) best = ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(sink);
    const double flops = 2.0 * (double)blocks * threads * (double)iters * CH;
    *tflops = flops / (best * 1e-3) / 1e12;
    return 0;
}

}  // namespace redgb
