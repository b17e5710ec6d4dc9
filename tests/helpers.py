"""Shared test helpers: golden fixtures, systems under test, bit-exact comparisons."""
from __future__ import annotations

import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "red.cuda.closeencounter_gb300")
for p in (PKG, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

from redgb import bodies, types as T  # noqa: E402
from redgb.driver import run_main_loop  # noqa: E402
from redgb.types import event_key  # noqa: E402,F401

GOLDEN = os.path.join(ROOT, "tests", "golden")
INT_TYPES = {"e": T.INT_EULER, "rk4": T.INT_RK4, "rk5": T.INT_RK5, "rkf8": T.INT_RKF78}


def load_fixture(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False)
    counts = tuple(int(c) for c in z["counts"])
    disk = bodies.Disk(counts, z["r"].copy(), z["v"].copy(), z["p"].copy(), z["md"].copy(), z["epoch"].copy(),
                       [f"b{i}" for i in range(sum(counts))])
    params = json.loads(str(z["params"]))
    return disk, params, z["result"], z["events"]


def thresholds_of(params):
    ej = params.get("ejection", 0.0) or 0.0
    hit = params.get("hit_centrum", 0.0) or 0.0
    cf = params.get("collision_factor", 0.0) or 0.0
    return bodies.thresholds(ejection=ej, hit_centrum=hit, collision_factor=cf)


def frame_of(params):
    return T.FRAME_ASTRO if params.get("frame_center") == "astro" else T.FRAME_BARY


def configure(system, params):
    system.set_integrator(INT_TYPES[params["integrator"]], 0.001, params.get("tolerance") is not None,
                          params.get("tolerance") or 1e-10, params.get("error_check_for_tp", False))
    system.set_event_options(close_encounter=params.get("close_encounter", False))
    return system


def run_fixture(system, params, max_steps=0):
    configure(system, params)
    return run_main_loop(system, params["length_yr"] * T.YEAR, params["output_interval_yr"] * T.YEAR,
                         radii_enhance_factor=params.get("collision_factor", 0.0) or 0.0,
                         close_encounter=params.get("close_encounter", False), max_steps=max_steps)


def same(a, b):
    """Bit-exact equality that treats every NaN as equal to every NaN."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return a.shape == b.shape and bool(np.all((a == b) | (np.isnan(a) & np.isnan(b))))


def snapshots_as_result(snaps):
    """Flatten snapshots into the reference's result-record layout."""
    rows = []
    for t, r, v, p, md in snaps:
        for i in range(len(r)):
            rows.append((int(md[i]["id"]), int(md[i]["body_type"]), t, p[i]["mass"], p[i]["radius"], p[i]["density"],
                         p[i]["cd"], int(md[i]["mig_type"]), md[i]["mig_stop_at"],
                         [r[i]["x"], r[i]["y"], r[i]["z"]], [v[i]["x"], v[i]["y"], v[i]["z"]]))
    return rows


def compare_result(rows, result, velocity_scale=1.0):
    """Compare snapshot rows with the reference's result records; returns a list of problems."""
    bad = []
    if len(rows) != len(result):
        return [f"row count {len(rows)} != {len(result)}"]
    for k, (row, ref) in enumerate(zip(rows, result)):
        if row[0] != ref["id"] or row[1] != ref["type"]:
            bad.append(f"row {k}: id/type {row[:2]} != {(ref['id'], ref['type'])}")
        if not same(row[2], ref["t"]):
            bad.append(f"row {k}: t {row[2]!r} != {ref['t']!r}")
        if not same(row[3:7], [ref["mass"], ref["radius"], ref["density"], ref["cd"]]):
            bad.append(f"row {k}: params differ")
        if not same(row[9], ref["r"]):
            bad.append(f"row {k}: r {row[9]} != {ref['r']}")
        if not same(np.asarray(row[10]) * velocity_scale, ref["v"]):
            bad.append(f"row {k}: v {row[10]} != {ref['v']}")
        if len(bad) > 10:
            break
    return bad


def compare_events(events, ref):
    """Compare rg_event_t records with the reference's printed event records."""
    bad = []
    if len(events) != len(ref):
        return [f"event count {len(events)} != {len(ref)}"]
    for k, (e, g) in enumerate(zip(events, ref)):
        mine = [e["t"] / T.GAUSS, e["d"],
                e["p1"]["mass"], e["p1"]["density"], e["p1"]["radius"], *[e["r1"][c] for c in "xyz"],
                *[e["v1"][c] * T.GAUSS for c in "xyz"], *[e["oe1"][f] for f in T.ORBELEM.names],
                e["p2"]["mass"], e["p2"]["density"], e["p2"]["radius"], *[e["r2"][c] for c in "xyz"],
                *[e["v2"][c] * T.GAUSS for c in "xyz"], *[e["oe2"][f] for f in T.ORBELEM.names],
                e["ps"]["mass"], e["ps"]["density"], e["ps"]["radius"], *[e["rs"][c] for c in "xyz"],
                *[e["vs"][c] * T.GAUSS for c in "xyz"], *[e["oes"][f] for f in T.ORBELEM.names]]
        theirs = [g["t"], g["d"], *g["p1"], *g["r1"], *g["v1"], *g["oe1"], *g["p2"], *g["r2"], *g["v2"], *g["oe2"],
                  *g["ps"], *g["rs"], *g["vs"], *g["oes"]]
        if int(e["event_name"]) != int(g["name"]) or int(e["id1"]) != int(g["id1"]) or int(e["id2"]) != int(g["id2"]):
            bad.append(f"event {k}: ({e['event_name']},{e['id1']},{e['id2']}) != ({g['name']},{g['id1']},{g['id2']})")
        elif not same(mine, theirs):
            diff = [i for i, (a, b) in enumerate(zip(mine, theirs)) if not same(a, b)]
            bad.append(f"event {k}: fields {diff} differ")
        if len(bad) > 10:
            break
    return bad


FIXTURES = ["twobody_euler", "n1_massive_n3", "disk_nsi_rkf78", "disk_si_rkf78_collide", "disk_si_rkf78_ce",
            "disk_si_rk4_fixed", "disk_si_rk4_adaptive", "disk_eject_hit", "planetesimal_disk_1000yr",
            "disk_si_astro_collide", "disk_si_astro_ce"]
