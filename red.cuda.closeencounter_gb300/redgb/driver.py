"""The reference's time loop (red.cuda/src/red.cuda/main.cu:159-281) over a `System`,
with its snapshot cadence, so runs can be compared with the reference's result files.

The loop is the sequence of C entry points the reference's main() calls through
pp_disk / integrator: output check, ejection / hit-star check, step, collision (or
close-encounter) handling and storage compaction.  Snapshots are taken exactly when the
reference prints a result record (main.cu:166-199,266-281).
"""
from __future__ import annotations

from . import types as T


def run_main_loop(system, stop_day, output_interval_day, *, radii_enhance_factor, close_encounter=False,
                  inner_steps=True, start_day=0.0, max_steps=0, keep_inactive=False):
    """Returns (snapshots, events, n_steps); a snapshot is (t_day, r, v, p, md) in file units,
    the active records only, or the whole storage (inactive records until the next
    compaction included, storage order) with keep_inactive."""
    snaps = []
    events = []
    stop = stop_day * T.GAUSS
    oi = output_interval_day * T.GAUSS
    ps = 0.0

    def snap():
        r, v, p, md, t = system.state()
        if keep_inactive:
            snaps.append((t, r.copy(), v.copy(), p.copy(), md.copy()))
            return
        active = (md["id"] > 0) & (md["body_type"] < T.BODY_PADDINGPARTICLE)
        snaps.append((t, r[active].copy(), v[active].copy(), p[active].copy(), md[active].copy()))

    snap()
    n = 0
    while True:
        t = system.time(internal=True)
        if not t <= stop or (max_steps and n >= max_steps):
            break
        if oi <= abs(ps):
            ps = 0.0
            snap()
        system.check_for_ejection_hit_centrum()
        events.extend(system.events())
        dt = system.step() * T.GAUSS
        n += 1
        ps += abs(dt)
        if close_encounter and inner_steps:
            if 0.0 < radii_enhance_factor:
                system.check_for_close_encounter()
        elif not close_encounter and inner_steps:
            if 0.0 < radii_enhance_factor:
                system.check_for_collision()
            system.check_for_rebuild_vectors(8)
        events.extend(system.events())
    if 0.0 < ps:
        snap()
    return snaps, events, n
