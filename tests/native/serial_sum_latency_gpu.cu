// Latencies on one warp, measured with clock64 over dependent chains of 2 048 operations:
// the serial FP64 row sum as lane 0 runs it (shared-memory loads, __dadd_rn), the same sum by
// warp_serial_sum (exact_fp64.h), a dependent FP64 multiply chain, a dependent 64-bit integer
// chain (three operations per step) and a shuffle chain; both sums must give the same bits.
//
//   serial_sum_latency_gpu  ->  one line per row family of serial_sum_cases.h (0 gravity-like,
//                               3 cancelling, 2 tie-rich): cycles per term of each
#include <cstdio>
#include "../../red.cuda.closeencounter_gb300/csrc/exact_fp64.h"
#include "serial_sum_cases.h"

constexpr int N = 2048;

__global__ void probe(const double* t, long long* out)
{
    __shared__ double s[N];
    for (int k = threadIdx.x; k < N; k += 32) s[k] = t[k];
    __syncwarp();
    const int lane = threadIdx.x & 31;
    // 1: lane 0 serial loop from shared memory, 8-unrolled (the old few_sum_serial)
    long long c0 = clock64();
    double acc = 0.0;
    if (lane == 0) {
        for (int q = 0; q < N; q += 8) {
            const double t0 = s[q], t1 = s[q + 1], t2 = s[q + 2], t3 = s[q + 3];
            const double t4 = s[q + 4], t5 = s[q + 5], t6 = s[q + 6], t7 = s[q + 7];
            acc = __dadd_rn(acc, t0); acc = __dadd_rn(acc, t1); acc = __dadd_rn(acc, t2); acc = __dadd_rn(acc, t3);
            acc = __dadd_rn(acc, t4); acc = __dadd_rn(acc, t5); acc = __dadd_rn(acc, t6); acc = __dadd_rn(acc, t7);
        }
    }
    __syncwarp();
    long long c1 = clock64();
    // 2: warp_serial_sum
    double acc2 = 0.0;
    redgb::SerialSumState sst{0, 0};
    for (int b = 0; b < N; b += 32) acc2 = redgb::warp_serial_sum(acc2, s + b, 32, sst);
    __syncwarp();
    long long c2 = clock64();
    // 3: dependent DMUL chain
    double p = 1.0000001;
    for (int k = 0; k < N; k++) p = __dmul_rn(p, s[k & 7] * 0.0 + 1.0000001);
    long long c3 = clock64();
    // 4: dependent 64-bit integer chain (shift/add)
    unsigned long long u = (unsigned long long)__double_as_longlong(s[1]);
    for (int k = 0; k < N; k++) u = (u >> (k & 7)) + (u << 1) + k;
    long long c4 = clock64();
    // 5: shfl chain
    int v = lane;
    for (int k = 0; k < N; k++) v = __shfl_sync(0xffffffffu, v, (v + 1) & 31);
    long long c5 = clock64();
    if (lane == 0) {
        out[0] = c1 - c0; out[1] = c2 - c1; out[2] = c3 - c2; out[3] = c4 - c3; out[4] = c5 - c4;
        out[5] = __double_as_longlong(acc); out[6] = __double_as_longlong(acc2);
        out[7] = __double_as_longlong(p) ^ (long long)u ^ v;
    }
}

int main()
{
    for (int fam : {0, 3, 2}) {
        double h[N];
        double acc0;
        int n = 0;
        for (unsigned long long row = 0; n < N; row++) {
            double tmp[SC_MAX_LEN];
            int m = sc_row(99, fam, row, &acc0, tmp);
            for (int k = 0; k < m && n < N; k++) h[n++] = tmp[k];
        }
        double* d; long long* o;
        cudaMalloc(&d, sizeof(h)); cudaMalloc(&o, 8 * sizeof(long long));
        cudaMemcpy(d, h, sizeof(h), cudaMemcpyHostToDevice);
        for (int rep = 0; rep < 3; rep++) probe<<<1, 32>>>(d, o);
        long long r[8];
        if (cudaMemcpy(r, o, sizeof(r), cudaMemcpyDeviceToHost) != cudaSuccess) { printf("err\n"); return 1; }
        printf("family %d cycles per term: lane0 serial DADD %.1f | warp_serial_sum %.1f | DMUL chain %.1f | int64 chain %.1f | shfl %.1f | same %d\n",
               fam, r[0] / (double)N, r[1] / (double)N, r[2] / (double)N, r[3] / (double)N, r[4] / (double)N, (int)(r[5] == r[6]));
        cudaFree(d); cudaFree(o);
    }
    return 0;
}
