// plan_tools.h -- host-side launch-plan helpers shared by the single-disk and the ensemble
// plans (header-only, no CUDA types: the CPU tests compile it alone).
#pragma once

#include <algorithm>
#include <cstdint>
#include <vector>

namespace redgb {

// Segments of the symmetric heavy-light kernel (grav_df_sym).  `systems` holds one tile per
// system: its light bodies [sink_begin, sink_end) (and whatever else the kernel reads, copied
// into every segment).  The kernel's CTA takes a segment in passes of `unit` bodies (one per
// thread), then reduces the segment's heavy-row sums, so a segment costs its passes plus a
// fixed `seg_cost` (in passes).  The light bodies of all systems, end to end, are cut into
// passes (a system's last one partial), and the passes into n_cta contiguous ranges of equal
// cost, a system's first pass carrying the segment cost; a range's pieces in different
// systems are its segments.  Appends the segments, each with its part of its system's heavy
// rows (from 1, in the order of its light bodies), to `tiles`; CTA c takes the segments
// [cta_seg[c], cta_seg[c + 1]) of those appended (n_cta + 1 entries); parts[k] = 1 + the
// segments of system k (the heavy-heavy part is part 0).
template <class TileT>
void build_sym_segments(const std::vector<TileT>& systems, int n_cta, int unit, double seg_cost,
                        std::vector<TileT>& tiles, std::vector<int>& cta_seg, std::vector<int>& parts)
{
    const size_t t0 = tiles.size();
    struct Pass {
        int sys, b0, b1;
        double cost;
    };
    std::vector<Pass> pass;
    double total = 0.0;
    for (size_t k = 0; k < systems.size(); k++)
        for (int b = systems[k].sink_begin; b < systems[k].sink_end; b += unit) {
            const double c = 1.0 + (b == systems[k].sink_begin ? seg_cost : 0.0);
            pass.push_back(Pass{(int)k, b, std::min(b + unit, systems[k].sink_end), c});
            total += c;
        }
    parts.assign(systems.size(), 1);
    cta_seg.clear();
    size_t q = 0;
    double done = 0.0;
    for (int c = 0; c < n_cta; c++) {
        cta_seg.push_back((int)(tiles.size() - t0));
        // this CTA's passes: up to the cost boundary (c + 1) total / n_cta, the pass that
        // crosses it going to the side nearer to it; the last CTA takes the rest
        const double goal = total * (c + 1) / n_cta;
        int prev_sys = -1;
        while (q < pass.size()) {
            const bool last = c == n_cta - 1;
            if (!last && done + pass[q].cost * 0.5 > goal) break;
            const Pass& p = pass[q];
            if (p.sys == prev_sys) {
                tiles.back().sink_end = p.b1;  // the same segment goes on
            } else {
                TileT t = systems[p.sys];
                t.sink_begin = p.b0;
                t.sink_end = p.b1;
                t.part = parts[p.sys]++;
                tiles.push_back(t);
                prev_sys = p.sys;
            }
            done += p.cost;
            q++;
        }
    }
    cta_seg.push_back((int)(tiles.size() - t0));
}

}  // namespace redgb
