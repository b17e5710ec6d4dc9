// CPU check of build_sym_segments (plan_tools.h): random systems of 1 to 9000 light bodies,
// CTA counts from 1 to past the pass count.  Every system's light bodies are covered once, in
// order, by its segments (parts 1, 2, ...), each made of whole passes of 256 from the
// system's first light body; parts[k] = 1 + its segments; the CTA table is monotone and
// complete; and every CTA's cost (passes + 0.6 per system start) is within one pass and one
// segment cost of the mean, unless there are fewer passes than CTAs.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "../../red.cuda.closeencounter_gb300/csrc/plan_tools.h"

struct T {
    int sink_begin, sink_end, sys, part;
};

int main()
{
    const int unit = 256;
    const double seg = 0.6;
    unsigned seed = 12345u;
    auto rnd = [&](int n) {
        seed = seed * 1664525u + 1013904223u;
        return (int)((seed >> 8) % (unsigned)n);
    };
    int cases = 0, bad = 0;
    for (int trial = 0; trial < 400; trial++) {
        const int ns = 1 + rnd(trial < 200 ? 8 : 300);
        std::vector<T> sys;
        int base = 0;
        long long passes = 0;
        double total = 0.0;
        for (int k = 0; k < ns; k++) {
            const int nh = 1 + rnd(4), nl = 1 + rnd(rnd(3) == 0 ? 20 : 9000);
            sys.push_back(T{base + nh, base + nh + nl, k, 0});
            base += nh + nl;
            passes += (nl + unit - 1) / unit;
            total += (nl + unit - 1) / unit + seg;
        }
        const int cands[6] = {1, 7, 456, 912, (int)(passes / 3) + 1, (int)passes + 3};
        for (int n_cta : cands) {
            if (n_cta < 1) continue;
            cases++;
            std::vector<T> tiles{T{-1, -1, -1, -1}};  // appended after an existing tile
            std::vector<int> cta, parts;
            redgb::build_sym_segments(sys, n_cta, unit, seg, tiles, cta, parts);
            bool ok = (int)cta.size() == n_cta + 1 && cta[0] == 0 && cta[n_cta] == (int)tiles.size() - 1;
            for (int c = 0; ok && c < n_cta; c++) {
                ok = cta[c] <= cta[c + 1];
                double cost = 0.0;
                for (int q = cta[c]; q < cta[c + 1]; q++) {
                    const T& t = tiles[1 + q];
                    const T& s = sys[t.sys];
                    cost += std::ceil((t.sink_end - t.sink_begin) / (double)unit);
                    if (t.sink_begin == s.sink_begin) cost += seg;
                }
                if (passes >= n_cta) ok = ok && std::fabs(cost - total / n_cta) <= 1.0 + seg + 1e-9;
            }
            std::vector<int> next(ns), seen(ns, 0);
            for (int k = 0; k < ns; k++) next[k] = sys[k].sink_begin;
            for (size_t q = 1; ok && q < tiles.size(); q++) {
                const T& t = tiles[q];
                ok = t.sys >= 0 && t.sys < ns && t.sink_begin == next[t.sys] && t.sink_end > t.sink_begin &&
                     (t.sink_begin - sys[t.sys].sink_begin) % unit == 0 &&
                     (t.sink_end == sys[t.sys].sink_end || (t.sink_end - sys[t.sys].sink_begin) % unit == 0) &&
                     t.part == ++seen[t.sys];
                if (ok) next[t.sys] = t.sink_end;
            }
            for (int k = 0; ok && k < ns; k++) ok = next[k] == sys[k].sink_end && parts[k] == 1 + seen[k];
            if (!ok) {
                bad++;
                if (bad < 5) printf("bad: trial %d systems %d n_cta %d\n", trial, ns, n_cta);
            }
        }
    }
    printf("cases %d bad %d\n", cases, bad);
    return bad ? 1 : 0;
}
