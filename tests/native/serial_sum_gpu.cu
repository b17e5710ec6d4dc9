// GPU check of warp_serial_sum (exact_fp64.h) as the gravity kernels compile it: one warp
// per row of serial_sum_cases.h, the warp's rounds of 32 terms against lane 0's plain serial
// loop of __dadd_rn, counted on the device.
//
//   serial_sum_gpu ROWS  ->  one line per family: "family F rows R bad B"
#include <cstdio>
#include <cstdlib>

#include "../../red.cuda.closeencounter_gb300/csrc/exact_fp64.h"
#include "serial_sum_cases.h"

constexpr int WARPS = 4;

__global__ void __launch_bounds__(32 * WARPS) check(uint64_t seed, int fam, long long rows, double* buf,
                                                     unsigned long long* bad)
{
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long gw = (long long)blockIdx.x * WARPS + warp;
    double* t = buf + gw * SC_MAX_LEN;
    for (long long row = gw; row < rows; row += (long long)gridDim.x * WARPS) {
        double acc0 = 0.0;
        int n = 0;
        if (lane == 0) n = sc_row(seed, fam, (uint64_t)row, &acc0, t);
        n = __shfl_sync(0xffffffffu, n, 0);
        acc0 = __shfl_sync(0xffffffffu, acc0, 0);
        __syncwarp();
        double ref = acc0;
        if (lane == 0)
            for (int k = 0; k < n; k++) ref = __dadd_rn(ref, t[k]);
        ref = __shfl_sync(0xffffffffu, ref, 0);
        double acc = acc0;
        redgb::SerialSumState st{0, 0};
        for (int b = 0; b < n; b += 32) {
            const int m = n - b < 32 ? n - b : 32;
            acc = redgb::warp_serial_sum(acc, t + b, m, st);
        }
        const bool ok = (acc != acc && ref != ref) || __double_as_longlong(acc) == __double_as_longlong(ref);
        if (lane == 0 && !ok) atomicAdd(bad, 1ull);
        __syncwarp();
    }
}

int main(int argc, char** argv)
{
    const long long rows = argc > 1 ? atoll(argv[1]) : 20000;
    const int grid = 152 * 4;
    double* buf = nullptr;
    unsigned long long* bad = nullptr;
    if (cudaMalloc(&buf, (size_t)grid * WARPS * SC_MAX_LEN * sizeof(double)) != cudaSuccess) return 2;
    if (cudaMalloc(&bad, 5 * sizeof(unsigned long long)) != cudaSuccess) return 2;
    cudaMemset(bad, 0, 5 * sizeof(unsigned long long));
    for (int fam = 0; fam < 5; fam++) check<<<grid, 32 * WARPS>>>(12345, fam, rows, buf, bad + fam);
    unsigned long long h[5];
    if (cudaMemcpy(h, bad, sizeof(h), cudaMemcpyDeviceToHost) != cudaSuccess) {
        printf("cuda error %s\n", cudaGetErrorString(cudaGetLastError()));
        return 3;
    }
    int rc = 0;
    for (int fam = 0; fam < 5; fam++) {
        printf("family %d rows %lld bad %llu\n", fam, rows, h[fam]);
        rc |= h[fam] != 0;
    }
    cudaFree(buf);
    cudaFree(bad);
    return rc;
}
