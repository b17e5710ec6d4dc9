// GPU check of exact_fp64.h as the gravity kernels compile it (rcp/rsqrt.approx seeds):
// rn_sqrt / rn_div against the hardware's correctly rounded __dsqrt_rn / __ddiv_rn on the
// operand families of exact_fp64_cases.h, counted on the device.
//
//   exact_fp64_gpu LOG2N  ->  one line per family: "family F cases C bad B fast_div D fast_sqrt S"
#include <cstdio>
#include <cstdlib>

#include "../../red.cuda.closeencounter_gb300/csrc/exact_fp64.h"
#include "exact_fp64_cases.h"

struct Counts {
    unsigned long long bad, fast_div, fast_sqrt;
    unsigned long long first_a, first_b;
};

__global__ void check(uint64_t seed, int family, unsigned long long n, Counts* c)
{
    unsigned long long fd = 0, fs = 0;
    for (unsigned long long k = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; k < n;
         k += (unsigned long long)gridDim.x * blockDim.x) {
        uint64_t ab, bb;
        xc_case(seed, k, family, &ab, &bb);
        const double a = __longlong_as_double((long long)ab), b = __longlong_as_double((long long)bb);
        double q, s;
        const bool okd = redgb::xf::div_rn_fast(a, b, &q);
        const bool oks = redgb::xf::sqrt_rn_fast(a, &s);
        fd += okd;
        fs += oks;
        const bool wrong = (okd && __double_as_longlong(q) != __double_as_longlong(__ddiv_rn(a, b))) ||
                           (oks && __double_as_longlong(s) != __double_as_longlong(__dsqrt_rn(a))) ||
                           __double_as_longlong(redgb::rn_div(a, b)) != __double_as_longlong(__ddiv_rn(a, b)) ||
                           __double_as_longlong(redgb::rn_sqrt(a)) != __double_as_longlong(__dsqrt_rn(a));
        if (wrong) {
            if (atomicAdd(&c->bad, 1ull) == 0) {
                c->first_a = ab;
                c->first_b = bb;
            }
        }
    }
    atomicAdd(&c->fast_div, fd);
    atomicAdd(&c->fast_sqrt, fs);
}

int main(int argc, char** argv)
{
    const int lg = argc > 1 ? atoi(argv[1]) : 26;
    const unsigned long long n = 1ull << lg;
    Counts* c = nullptr;
    if (cudaMalloc(&c, sizeof(Counts)) != cudaSuccess) return 2;
    int rc = 0;
    for (int fam = 0; fam < 5; fam++) {
        cudaMemset(c, 0, sizeof(Counts));
        check<<<152 * 8, 256>>>(0xC0FFEEull + fam, fam, n, c);
        Counts h;
        if (cudaMemcpy(&h, c, sizeof(h), cudaMemcpyDeviceToHost) != cudaSuccess) return 2;
        printf("family %d cases %llu bad %llu fast_div %llu fast_sqrt %llu", fam, n, h.bad, h.fast_div, h.fast_sqrt);
        if (h.bad) {
            printf(" first %a %a", redgb::xf::bitsd(h.first_a), redgb::xf::bitsd(h.first_b));
            rc = 1;
        }
        printf("\n");
    }
    cudaFree(c);
    return rc;
}
