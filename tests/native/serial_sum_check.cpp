// CPU check of the exact serial sum's integer steps (exact_fp64.h: xf::quantize,
// xf::quanta_of, xf::from_quanta, xf::inside_binade): the warp algorithm of
// warp_serial_sum replayed lane by lane, in rounds of 32 terms, against the plain serial
// loop acc = acc + t_k, on the row families of serial_sum_cases.h.
//
//   serial_sum_check ROWS  ->  "rows R terms T bad B fast F fallback A"
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "../../red.cuda.closeencounter_gb300/csrc/exact_fp64.h"
#include "serial_sum_cases.h"

using namespace redgb;

// one round of up to 32 terms, as the warp computes it (warp_serial_sum, with its state)
struct State {
    int skip, backoff;
};

static double round_emulated(double acc, const double* t, int m, State& st, long long* fast, long long* slow)
{
    if (m <= 0) return acc;
    auto tail = [&](int from, int to) {
        for (int k = from; k < to; k++) acc = acc + t[k];
        *slow += to - from;
        return acc;
    };
    if (st.skip > 0) {
        st.skip--;
        return tail(0, m);
    }
    int pos = 0;
    while (pos < m) {
        const int ea = (int)((xf::dbits(acc) >> 52) & 0x7ff);
        if (ea == 0 || ea == 2047) {
            tail(pos, pos + 1);
            pos++;
            continue;
        }
        const int64_t A = xf::quanta_of(acc);
        int64_t P = 0, Sc = 0;
        int stop = m;
        for (int k = pos; k < m; k++) {
            int64_t r = 0;
            const bool ok = xf::quantize(t[k], ea, &r);
            if (!ok) r = 0;
            P += r;
            const int64_t S = A + P;
            if (!(ok && xf::inside_binade(A, S))) {
                stop = k;
                break;
            }
            Sc = S;
        }
        if (stop > pos) {
            acc = xf::from_quanta(Sc, ea);
            *fast += stop - pos;
        }
        if (stop >= m) break;
        if (stop - pos < 8) {  // SERIAL_GOOD_PASS
            st.skip = st.backoff;
            st.backoff = st.backoff ? (st.backoff * 2 < 8 ? st.backoff * 2 : 8) : 1;
            return tail(stop, m);
        }
        tail(stop, stop + 1);
        pos = stop + 1;
    }
    st.backoff = 0;
    return acc;
}

static bool same(double a, double b)
{
    return (std::isnan(a) && std::isnan(b)) || xf::dbits(a) == xf::dbits(b);
}

int main(int argc, char** argv)
{
    const long long rows = argc > 1 ? atoll(argv[1]) : 2000;
    std::vector<double> t(SC_MAX_LEN);
    long long terms = 0, bad = 0, fast = 0, slow = 0;
    for (int fam = 0; fam < 5; fam++) {
        const long long f0 = fast, s0 = slow;
        for (long long row = 0; row < rows; row++) {
            double acc0;
            const int n = sc_row(12345, fam, (uint64_t)row, &acc0, t.data());
            double ref = acc0, got = acc0;
            for (int k = 0; k < n; k++) ref = ref + t[k];
            State st{0, 0};
            for (int b = 0; b < n; b += 32)
                got = round_emulated(got, t.data() + b, n - b < 32 ? n - b : 32, st, &fast, &slow);
            terms += n;
            if (!same(ref, got)) {
                if (bad < 5)
                    printf("mismatch family %d row %lld: %a vs %a\n", fam, row, got, ref);
                bad++;
            }
        }
        printf("family %d fast %lld fallback %lld\n", fam, fast - f0, slow - s0);
    }
    // quantize against long double arithmetic on single terms (independent of the rounds)
    long long qbad = 0;
    ScRng g{777};
    for (long long k = 0; k < 20 * rows; k++) {
        const double acc = (g.below(2) ? -1.0 : 1.0) * sc_random_mag(g, -20, 20);
        const int ea = (int)((xf::dbits(acc) >> 52) & 0x7ff);
        const double tq = (g.below(2) ? -1.0 : 1.0) * sc_random_mag(g, -80, 24);
        int64_t r;
        if (!xf::quantize(tq, ea, &r)) continue;
        // acc + r Q inside the binade must be the rounded sum whenever inside_binade holds
        const int64_t S = xf::quanta_of(acc) + r;
        if (xf::inside_binade(xf::quanta_of(acc), S) && !same(xf::from_quanta(S, ea), acc + tq)) qbad++;
    }
    printf("rows %lld terms %lld bad %lld fast %lld fallback %lld qbad %lld\n", 5 * rows, terms, bad, fast, slow, qbad);
    return bad || qbad ? 1 : 0;
}
