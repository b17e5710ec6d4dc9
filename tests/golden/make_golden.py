"""Regenerates the golden fixtures of tests/golden/ from the reference itself.

Run in a checkout that has the reference sources (this is the only script that reads
them; nothing in the test suite does):

    make -f oracle/ref.mk REF=<reference checkout> -j8   # builds oracle/_ref/red (CPU path)
    python tests/golden/make_golden.py --ref <reference checkout>

The checkout can also be named by the RED_REFERENCE environment variable.

Each case writes a body list and a parameter file, runs ``red -cpu -ef`` (the
reference's FP64 CPU path, single thread) and stores inputs, result snapshots and event
records in <case>.npz.  The reference prints with 17 significant digits, so the parsed
numbers are the reference's doubles exactly.  The reference's own test fixtures
(TestRun/InputTest) are stored the same way.
"""
from __future__ import annotations

import argparse
import json
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "red.cuda.closeencounter_gb300"))

from redgb import bodies, types as T  # noqa: E402

RED = os.path.join(ROOT, "oracle", "_ref", "red")

# body records printed by pp_disk::print_result_ascii (pp_disk.cu:1685-1725)
RESULT = np.dtype([("id", "<i4"), ("type", "<i4"), ("t", "<f8"), ("mass", "<f8"), ("radius", "<f8"),
                   ("density", "<f8"), ("cd", "<f8"), ("mig_type", "<i4"), ("mig_stop_at", "<f8"),
                   ("r", "<f8", 3), ("v", "<f8", 3)])
# event records printed by pp_disk::print_event_data (pp_disk.cu:1772-1848)
EVREC = np.dtype([("name", "<i4"), ("t", "<f8"), ("d", "<f8"), ("id1", "<i4"), ("id2", "<i4"),
                  ("p1", "<f8", 3), ("r1", "<f8", 3), ("v1", "<f8", 3), ("oe1", "<f8", 6),
                  ("p2", "<f8", 3), ("r2", "<f8", 3), ("v2", "<f8", 3), ("oe2", "<f8", 6),
                  ("ps", "<f8", 3), ("rs", "<f8", 3), ("vs", "<f8", 3), ("oes", "<f8", 6)])


def parse_result(path):
    rows = []
    for line in open(path):
        f = line.split()
        if not f:
            continue
        rows.append((int(f[0]), int(f[2]), float(f[3]), float(f[4]), float(f[5]), float(f[6]), float(f[7]),
                     int(f[8]), float(f[9]), [float(x) for x in f[10:13]], [float(x) for x in f[13:16]]))
    return np.array(rows, RESULT)


def parse_events(path):
    rows = []
    for line in open(path):
        f = line.split()
        if not f:
            continue
        name = T.EVENT_NAMES.index(f[0])
        x = [float(v) for v in f[5:]]
        assert len(x) == 45, len(x)
        rows.append((name, float(f[1]), float(f[2]), int(f[3]), int(f[4]),
                     x[0:3], x[3:6], x[6:9], x[9:15], x[15:18], x[18:21], x[21:24], x[24:30],
                     x[30:33], x[33:36], x[36:39], x[39:45]))
    return np.array(rows, EVREC)


def run_case(name, disk, params, workdir, timeout=600):
    d = os.path.join(workdir, name)
    os.makedirs(d, exist_ok=True)
    bodies.write_body_file(os.path.join(d, "bodies.txt"), disk)
    bodies.write_parameter_file(os.path.join(d, "parameters.txt"), **params)
    subprocess.run([RED, "-cpu", "-ef", "-iDir", d, "-p", "parameters.txt", "-ic", "bodies.txt"], cwd=d,
                   check=True, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL, timeout=timeout)
    prefix = os.path.join(d, "R_cpu_ns_" + ("as" if params.get("tolerance") is not None else "fs") + "_")
    short = {"e": "E", "rk4": "RK4", "rkf8": "RKF8"}[params["integrator"]]
    result = parse_result(prefix + short + "_result.txt")
    events = parse_events(prefix + short + "_event.txt")
    return result, events


def save_text(name, disk, params, workdir, events_only=False):
    """The reference's own output files of one case, kept verbatim (gzip) to pin the
    writers of redgb.io byte for byte: text result, binary result, event lines."""
    import gzip
    for out_type in (("text",) if events_only else ("text", "binary")):
        d = os.path.join(workdir, name + "_" + out_type)
        os.makedirs(d, exist_ok=True)
        bodies.write_body_file(os.path.join(d, "bodies.txt"), disk)
        bodies.write_parameter_file(os.path.join(d, "parameters.txt"), output_type=out_type, **params)
        subprocess.run([RED, "-cpu", "-ef", "-iDir", d, "-p", "parameters.txt", "-ic", "bodies.txt"], cwd=d,
                       check=True, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL, timeout=600)
        prefix = os.path.join(d, "R_cpu_ns_" + ("as" if params.get("tolerance") is not None else "fs") + "_")
        short = {"e": "E", "rk4": "RK4", "rkf8": "RKF8"}[params["integrator"]]
        files = [("_event.txt", "_event.txt")] if events_only else []
        if not events_only:
            files += [("_result.txt", "_result.txt")] if out_type == "text" else [("_result.bin", "_result.bin")]
            if out_type == "text":
                files.append(("_event.txt", "_event.txt"))
        for src, dst in files:
            with open(prefix + short + src, "rb") as fi, gzip.open(os.path.join(HERE, name + dst + ".gz"), "wb") as fo:
                fo.write(fi.read())
            print(f"{name}{dst}.gz")


def save(name, disk, params, result, events):
    np.savez_compressed(os.path.join(HERE, name + ".npz"), counts=np.array(disk.counts, np.int32), r=disk.r,
                        v=disk.v, p=disk.p, md=disk.md, epoch=disk.epoch, params=json.dumps(params),
                        result=result, events=events)
    print(f"{name}: {len(result)} result rows, {len(events)} events")


def cases():
    """(name, disk, params): small seeded disks exercising each integrator and event type."""
    out = []
    d = bodies.make_disk(n_pl=48, seed=3)
    out.append(("disk_nsi_rkf78", d, dict(integrator="rkf8", tolerance=1e-10, length_yr=2.0, output_interval_yr=0.25,
                                          ejection=100.0, hit_centrum=0.05, collision_factor=1.0)))
    d = bodies.make_disk(n_pl=120, pl_type=T.BODY_PROTOPLANET, seed=5, m_range=(1e-7, 1e-5),
                         giants=((9.55e-4, 5.2, 0.05),), a_range=(1.0, 1.3), sigma_e=0.05, sigma_i=0.02)
    # collision radii inflated 150x: ~30 merges in 2 yr and several storage compactions, while
    # every step stays below the reference's unchecked n_total-record event buffer
    out.append(("disk_si_rkf78_collide", d, dict(integrator="rkf8", tolerance=1e-10, length_yr=2.0,
                                                 output_interval_yr=0.25, ejection=100.0, hit_centrum=0.05,
                                                 collision_factor=150.0)))
    out.append(("disk_si_rkf78_ce", d, dict(integrator="rkf8", tolerance=1e-10, length_yr=0.5, output_interval_yr=0.1,
                                            ejection=100.0, hit_centrum=0.05, collision_factor=40.0,
                                            close_encounter=True)))
    d = bodies.make_disk(n_pl=24, pl_type=T.BODY_PROTOPLANET, seed=7, m_range=(1e-9, 1e-7), giants=())
    out.append(("disk_si_rk4_fixed", d, dict(integrator="rk4", length_yr=0.02, output_interval_yr=0.005,
                                             ejection=100.0, hit_centrum=0.05, collision_factor=1.0)))
    out.append(("disk_si_rk4_adaptive", d, dict(integrator="rk4", tolerance=1e-12, length_yr=0.5,
                                                output_interval_yr=0.1, ejection=100.0, hit_centrum=0.05,
                                                collision_factor=1.0)))
    d = bodies.make_disk(n_pl=16, seed=11, a_range=(1.0, 3.0), sigma_e=0.3, sigma_i=0.05, n_tp=4)
    out.append(("disk_eject_hit", d, dict(integrator="rkf8", tolerance=1e-10, length_yr=3.0, output_interval_yr=0.5,
                                          ejection=3.2, hit_centrum=0.3, collision_factor=1.0)))
    # the astrocentric frame (frame_center = astro) on a self-interacting disk -- the reference's
    # own CPU path gives NaN once planetesimals or test particles are present (their blocks take
    # the star at the origin as a source) -- from barycentric input, so that the astrocentric
    # transform at load (options.cpp:217-220) moves every body to the star
    d = bodies.make_disk(n_pl=120, pl_type=T.BODY_PROTOPLANET, seed=17, m_range=(1e-7, 1e-5),
                         giants=((9.55e-4, 5.2, 0.05), (2.86e-4, 9.54, 0.05)), a_range=(1.0, 1.3), sigma_e=0.05,
                         sigma_i=0.02)
    m = d.p["mass"]
    for f in "xyz":
        d.r[f] -= np.sum(m * d.r[f]) / np.sum(m)
        d.v[f] -= np.sum(m * d.v[f]) / np.sum(m)
    out.append(("disk_si_astro_collide", d, dict(integrator="rkf8", tolerance=1e-10, length_yr=2.0,
                                                 output_interval_yr=0.25, ejection=100.0, hit_centrum=0.05,
                                                 collision_factor=150.0, frame_center="astro")))
    out.append(("disk_si_astro_ce", d, dict(integrator="rkf8", tolerance=1e-10, length_yr=0.5, output_interval_yr=0.1,
                                            ejection=100.0, hit_centrum=0.05, collision_factor=150.0,
                                            close_encounter=True, frame_center="astro")))
    # the plain FP64 planetesimal-disk workload: star, two giants, 1024 planetesimals (seed 0),
    # RKF7(8) at 1e-10 for 1000 years with collisions, ejection (100 AU) and hit-star (0.05 AU)
    # on; snapshots every 250 years
    out.append(("planetesimal_disk_1000yr", bodies.config_disk("planetesimal_disk"),
                dict(integrator="rkf8", tolerance=1e-10, length_yr=1000.0, output_interval_yr=250.0, ejection=100.0,
                     hit_centrum=0.05, collision_factor=1.0)))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("RED_REFERENCE"),
                    help="the reference checkout (default: $RED_REFERENCE)")
    ap.add_argument("--only", default=None)
    args = ap.parse_args()
    if not args.ref:
        sys.exit("name the reference checkout: --ref <dir> or RED_REFERENCE=<dir>")
    if not os.path.exists(RED):
        sys.exit("oracle/_ref/red missing: make -f oracle/ref.mk REF=<reference> first")
    tin = os.path.join(args.ref, "red.cuda", "TestRun", "InputTest")
    work = tempfile.mkdtemp(prefix="redgolden_")
    try:
        if args.only in (None, "twobody_euler"):
            # the reference's own golden run (Debug/TwoBody, Euler, 2 yr, output every 0.1 yr)
            src = os.path.join(tin, "Debug", "TwoBody")
            disk = bodies.read_body_file(os.path.join(src, "TwoBody2.txt"))
            result = parse_result(os.path.join(src, "D_cpu_ns_fs_E_result.txt"))
            params = dict(integrator="e", length_yr=2.0, output_interval_yr=0.1)
            save("twobody_euler", disk, params, result, np.zeros(0, EVREC))
        if args.only in (None, "n1_massive_n3"):
            # Release/N1_massive_N3_test: test particle 12 sits on protoplanet 2
            src = os.path.join(tin, "Release", "N1_massive_N3_test")
            disk = bodies.read_body_file(os.path.join(src, "N1_massive_N3_test.txt"))
            params = dict(integrator="rkf8", tolerance=1e-10, length_yr=1000.0, output_interval_yr=1.0,
                          ejection=100.0, hit_centrum=0.1, collision_factor=100.0)
            result, events = run_case("n1_massive_n3", disk, params, work)
            save("n1_massive_n3", disk, params, result, events)
        for name, disk, params in cases():
            if args.only not in (None, name):
                continue
            result, events = run_case(name, disk, params, work)
            save(name, disk, params, result, events)
            # verbatim output files for the format tests of redgb.io
            if name == "disk_eject_hit":
                save_text(name, disk, params, work)
            elif name == "disk_si_rkf78_ce":
                save_text(name, disk, params, work, events_only=True)
    finally:
        shutil.rmtree(work, ignore_errors=True)


if __name__ == "__main__":
    main()
