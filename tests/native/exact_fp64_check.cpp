// CPU check of exact_fp64.h: the integer square root and division against the host's IEEE
// binary64 sqrt and '/', with the FP32 seeds exact (the host's) and perturbed by up to
// 1e-5 relative -- the GPU's rcp/rsqrt.approx seeds are within about 1e-7.  Also every
// combination of extreme significands and exponents.
//
//   exact_fp64_check N   ->  prints "bad B fallback_div F fallback_sqrt G", exit status 1 if B > 0
#include <cmath>
#include <cstdio>
#include <cstdlib>

static double g_pert = 0.0;
static float pert_rcp(float x) { return (float)((1.0 / x) * (1.0 + g_pert)); }
static float pert_rsqrt(float x) { return (float)((1.0 / std::sqrt((double)x)) * (1.0 + g_pert)); }
#define XF_APPROX_RCP(x) pert_rcp(x)
#define XF_APPROX_RSQRT(x) pert_rsqrt(x)
#include "../../red.cuda.closeencounter_gb300/csrc/exact_fp64.h"
#include "exact_fp64_cases.h"

using namespace redgb::xf;

int main(int argc, char** argv)
{
    const long n = argc > 1 ? atol(argv[1]) : 200000;
    const double perts[] = {0.0, 3e-7, -3e-7, 2e-6, -2e-6, 1e-5, -1e-5};
    long bad = 0, fb_d = 0, fb_s = 0;
    for (double p : perts) {
        g_pert = p;
        for (int fam = 0; fam < 5; fam++)
            for (long k = 0; k < n; k++) {
                uint64_t ab, bb;
                xc_case(1234567 + fam, (uint64_t)k, fam, &ab, &bb);
                const double a = bitsd(ab), b = bitsd(bb);
                double q, s;
                if (div_rn_fast(a, b, &q)) {
                    if (dbits(q) != dbits(a / b) && bad++ < 10) printf("div %a / %a -> %a, IEEE %a\n", a, b, q, a / b);
                } else {
                    fb_d++;
                }
                if (sqrt_rn_fast(a, &s)) {
                    if (dbits(s) != dbits(std::sqrt(a)) && bad++ < 10) printf("sqrt %a -> %a, IEEE %a\n", a, s, std::sqrt(a));
                } else {
                    fb_s++;
                }
            }
    }
    g_pert = 0.0;
    const uint64_t sig[] = {0, 1, 2, 3, M52 - 2, M52 - 1, M52, H52 >> 1, (H52 >> 1) + 1, (H52 >> 1) - 1,
                            0x5555555555555ull, 0xAAAAAAAAAAAAAull};
    const int ex[] = {1, 2, 500, 1022, 1023, 1024, 1500, 2045, 2046};
    for (uint64_t sa : sig)
        for (uint64_t sb : sig)
            for (int xa : ex)
                for (int xb : ex) {
                    const double a = bitsd(sa | ((uint64_t)xa << 52)), b = bitsd(sb | ((uint64_t)xb << 52));
                    double q, s;
                    if (div_rn_fast(a, b, &q) && dbits(q) != dbits(a / b) && bad++ < 10) printf("corner div %a / %a\n", a, b);
                    if (sqrt_rn_fast(a, &s) && dbits(s) != dbits(std::sqrt(a)) && bad++ < 10) printf("corner sqrt %a\n", a);
                }
    printf("bad %ld fallback_div %ld fallback_sqrt %ld\n", bad, fb_d, fb_s);
    return bad ? 1 : 0;
}
