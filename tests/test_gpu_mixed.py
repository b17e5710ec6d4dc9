"""Mixed-precision gravity (FP32 rsqrt / two-sum FP32 accumulation, FP64 displacements
for near pairs, FP64 heavy sources) against the FP64 oracle.

Tolerances: the relative force error |a_mixed - a_fp64| / |a_fp64| per body must stay
below 1e-10 (max) and 3e-11 (RMS) on the benchmark disks; event lists must be identical
to the FP64 path's, because every event decision is re-evaluated in FP64.
"""
import json
import os

import numpy as np
import pytest

import helpers as H
import pyoracle
from redgb import bodies, lib, types as T

pytestmark = pytest.mark.gpu

MAX_REL, RMS_REL = 1e-10, 3e-11


def force_error(disk):
    g = lib.System(disk, bodies.thresholds())
    g.set_gravity_mode(T.GRAVITY_MIXED)
    am = g.calc_accel()
    g.set_gravity_mode(T.GRAVITY_FP64)
    ae = g.calc_accel()
    a_m = np.stack([am[f] for f in "xyz"], 1)
    a_e = np.stack([ae[f] for f in "xyz"], 1)
    norm = np.linalg.norm(a_e, axis=1)
    ok = norm > 0
    rel = np.linalg.norm(a_m - a_e, axis=1)[ok] / norm[ok]
    return float(rel.max()), float(np.sqrt(np.mean(rel ** 2))), ae, disk


@pytest.mark.parametrize("config,n", [("planetesimal_disk", None), ("self_gravitating", 4096),
                                      ("self_gravitating", None), ("dense_ring", 8192)])
def test_mixed_force_error(gpulib, config, n):
    disk = bodies.config_disk(config, n=n)
    mx, rms, ae, _ = force_error(disk)
    out = os.environ.get("RG_FORCE_ERROR_LOG")
    if out:
        with open(out, "a") as f:
            f.write(json.dumps({"config": config, "n": disk.n_total, "max_rel": mx, "rms_rel": rms}) + "\n")
    print(f"{config} n={disk.n_total}: max rel {mx:.3e} rms rel {rms:.3e}")
    assert mx < MAX_REL and rms < RMS_REL


def test_mixed_close_pairs_force_error(gpulib):
    """Pairs closer than the split positions resolve (2^-48 |x| ~ 4e-15 AU at 1 AU): light
    pairs 1e-7 to 1e-5 AU apart (near pairs of the mixed kernel) and planetesimals within
    0.002 AU of a giant (double-float kernels).  Their displacements come from the FP64
    positions, so the force error stays within the same bounds."""
    disk = bodies.config_disk("self_gravitating", n=4096)
    for k in range(8):
        a, b = 10 + k, 2000 + k
        for f, c in zip("xyz", (1.0, 2.0, -1.0)):
            disk.r[f][b] = disk.r[f][a] + c * 10.0 ** (-7 + 2 * (k % 2)) * (k + 1)
    mx, rms, _, _ = force_error(disk)
    print(f"close light pairs: max rel {mx:.3e} rms rel {rms:.3e}")
    assert mx < MAX_REL and rms < RMS_REL
    disk = bodies.config_disk("planetesimal_disk")
    for k, off in enumerate(((2e-3, 1e-3, 0.0), (0.0, -5e-4, 1e-4), (1e-4, 1e-4, 1e-4))):
        for f, c in zip("xyz", off):
            disk.r[f][3 + k] = disk.r[f][1] + c
    mx, rms, _, _ = force_error(disk)
    print(f"planetesimals near a giant: max rel {mx:.3e} rms rel {rms:.3e}")
    assert mx < MAX_REL and rms < RMS_REL


def test_mixed_crowded_clump_force_error(gpulib):
    """256 self-gravitating bodies within 5e-4 AU of one point: every pair of the clump is a
    near pair, so a warp-slice over the clump flags up to 32 x 128 pairs (self pairs included)
    and the kernel's exact pass runs many rounds of 32 shared items; the clump's own pairs
    take the double-float term from FP64 displacements."""
    disk = bodies.config_disk("self_gravitating", n=4096)
    rng = np.random.default_rng(7)
    centre = [float(disk.r[f][1000]) for f in "xyz"]
    for k in range(100, 356):
        off = rng.uniform(-5e-4, 5e-4, 3)
        for f, o, c in zip("xyz", off, centre):
            disk.r[f][k] = c + o
    mx, rms, _, _ = force_error(disk)
    print(f"crowded clump: max rel {mx:.3e} rms rel {rms:.3e}")
    assert mx < MAX_REL and rms < RMS_REL


def test_mixed_planetesimal_events_from_the_heavy_rows(gpulib):
    """Planetesimals (NSI) against the star and the giants in the double-float kernels (the
    giants' rows in the few-sink kernel, the planetesimals' rows in the row kernel, each with
    its block's event screens): planetesimals placed inside the giants' Hill spheres and two
    overlapping a giant give the FP64 path's close-encounter and collision records over two
    fixed steps."""
    disk = bodies.config_disk("planetesimal_disk")
    offsets = [(0.05 * k, 0.03, 0.01) for k in range(1, 9)] + [(3e-4, 0.0, 0.0), (0.0, -2e-4, 1e-4)]
    for k, off in enumerate(offsets):
        g = 1 + k % 2
        for f, c in zip("xyz", off):
            disk.r[f][3 + k] = disk.r[f][g] + c
    thr = bodies.thresholds(collision_factor=1.0)
    lists = {}
    for mode in (T.GRAVITY_FP64, T.GRAVITY_MIXED):
        s = lib.System(disk, thr)
        s.set_gravity_mode(mode)
        s.set_integrator(T.INT_RKF78, 0.01, False)
        s.set_event_options(hill_factor=3.0)
        s.advance(0.02)
        lists[mode] = [(int(e["event_name"]), int(e["id1"]), int(e["id2"])) for e in s.events()]
    kinds = {k for k, _, _ in lists[T.GRAVITY_FP64]}
    assert {T.EVENT_CLOSE_ENCOUNTER, T.EVENT_COLLISION} <= kinds, lists[T.GRAVITY_FP64]
    assert lists[T.GRAVITY_MIXED] == lists[T.GRAVITY_FP64]


@pytest.mark.parametrize("case", ["star_only", "star_and_one_planet", "test_particles", "inactive_and_massless",
                                  "large_protoplanet_block"])
def test_mixed_edge_cases(gpulib, case):
    """Small and ragged inputs through the mixed plan: one body, one pair, test particles (NI
    block), inactive and massless bodies, and an SI block large enough for the mixed kernel
    with test particles behind it.  Inactive bodies feel nothing; everything else within the
    force-error bound of the FP64 path."""
    if case == "star_only":
        disk = bodies.make_disk(n_pl=0, seed=1, giants=())
    elif case == "star_and_one_planet":
        disk = bodies.make_disk(n_pl=0, seed=1, giants=((9.55e-4, 5.2, 0.05),))
    elif case == "test_particles":
        disk = bodies.make_disk(n_pl=300, seed=2, n_tp=57)
    elif case == "inactive_and_massless":
        disk = bodies.make_disk(n_pl=400, pl_type=T.BODY_PROTOPLANET, seed=5, n_tp=9, m_range=(1e-9, 1e-7))
        disk.md["id"][[5, 17, 40, 300]] *= -1
        disk.p["mass"][[7, 8, 301]] = 0.0
    else:
        disk = bodies.make_disk(n_pl=2500, pl_type=T.BODY_PROTOPLANET, seed=6, n_tp=33, m_range=(1e-9, 1e-7))
    g = lib.System(disk, bodies.thresholds())
    ae = g.calc_accel()
    g.set_gravity_mode(T.GRAVITY_MIXED)
    am = g.calc_accel()
    a_m = np.stack([am[f] for f in "xyz"], 1)
    a_e = np.stack([ae[f] for f in "xyz"], 1)
    inactive = disk.md["id"] <= 0
    assert np.all(a_m[inactive] == 0.0) and np.all(a_e[inactive] == 0.0)
    norm = np.linalg.norm(a_e, axis=1)
    ok = norm > 0
    assert np.array_equal(np.linalg.norm(a_m, axis=1) > 0, ok)
    if ok.any():
        rel = np.linalg.norm(a_m - a_e, axis=1)[ok] / norm[ok]
        assert rel.max() < MAX_REL, (case, rel.max())


def test_mixed_fp64_reference_matches_oracle_rows(gpulib):
    """The FP64 accelerations used as the yardstick above are the oracle's."""
    disk = bodies.config_disk("self_gravitating", n=2048)
    _, _, ae, _ = force_error(disk)
    o = pyoracle.OracleSystem(disk, bodies.thresholds())
    ao = o.calc_accel()
    for f in "xyz":
        assert H.same(ae[f], ao[f])


def test_mixed_event_list_identical(gpulib, planetesimal_disk_1000yr_oracle):
    """The planetesimal-disk workload (star, two giants, 1024 planetesimals) over its full 1000
    years with the mixed kernels, close encounters at 3 mutual Hill radii: the event list
    equals the FP64 oracle's record for record -- type and pair of every record, none missing
    or added -- and so does the number of steps.  Event decisions are taken in FP64 on the
    mixed run's own state; the step sizes differ in their last digits, so the records' times
    (step starts) agree to 1e-3 relative, not bit for bit."""
    disk, thr, params, n_o, eo, _ = planetesimal_disk_1000yr_oracle
    s = lib.System(disk, thr)
    s.set_gravity_mode(T.GRAVITY_MIXED)
    s.set_integrator(T.INT_RKF78, 0.001, True, params["tolerance"])
    s.set_event_options(hill_factor=3.0)
    assert s.advance(params["length_yr"] * T.YEAR) == n_o
    mine = s.events()
    assert len(eo) >= 20
    assert [(int(e["event_name"]), int(e["id1"]), int(e["id2"])) for e in mine] == \
           [(int(e["event_name"]), int(e["id1"]), int(e["id2"])) for e in eo]
    assert np.allclose(mine["t"], eo["t"], rtol=1e-3, atol=0.0)


def test_mixed_screen_cutoffs_keep_every_event(gpulib):
    """A crowded ring (planetesimal radii x 300, Hill factor 3: about 150 overlapping and
    250 Hill pairs at the start, masses spread over a factor of 100): the mixed kernels
    skip the detailed screens beyond each sink's cutoff from the evaluation's largest
    radius, mass and star distance, and still find exactly the FP64 path's events."""
    disk = bodies.config_disk("dense_ring", n=16384)
    disk.p["radius"][1:] *= 300.0
    thr = bodies.thresholds(collision_factor=1.0)
    lists = {}
    for mode in (T.GRAVITY_FP64, T.GRAVITY_MIXED):
        s = lib.System(disk, thr, event_capacity=1 << 16)
        s.set_gravity_mode(mode)
        s.set_integrator(T.INT_RKF78, 0.02, False)
        s.set_event_options(hill_factor=3.0)
        s.advance(0.04)
        lists[mode] = [(int(e["event_name"]), int(e["id1"]), int(e["id2"])) for e in s.events()]
    names = {k for k, _, _ in lists[T.GRAVITY_FP64]}
    assert len(lists[T.GRAVITY_FP64]) > 100 and len(names) >= 2, (len(lists[T.GRAVITY_FP64]), names)
    assert lists[T.GRAVITY_MIXED] == lists[T.GRAVITY_FP64]


def test_mixed_wait_limit_reports_an_error(gpulib):
    """Failure path of the mixed kernel without a fault: with the tile copies held back, every
    CTA's bounded wait (one second of the GPU's global timer) runs out, the kernel records it
    and returns, the host reports RG_ERR_CUDA, and the same context then evaluates normally."""
    import time
    from redgb.api import RedError
    disk = bodies.config_disk("self_gravitating", n=4096)
    s = lib.System(disk, bodies.thresholds())
    s.set_gravity_mode(T.GRAVITY_MIXED)
    ref = s.calc_accel()
    s.test_hold_tile_copies(True)
    t0 = time.perf_counter()
    with pytest.raises(RedError) as ei:
        s.calc_accel()
    assert ei.value.status == -2 and "wait limit" in str(ei.value)
    assert time.perf_counter() - t0 < 30.0
    s.test_hold_tile_copies(False)
    again = s.calc_accel()
    for f in "xyz":
        assert np.array_equal(again[f], ref[f])
