"""Benchmark of the gravity + Runge-Kutta hot path on GB300 (one JSON line).

Workload (default): 16384 self-gravitating planetesimals (m log-uniform 1e-9..1e-7 Msun,
Sigma ~ r^-1.5 on 1..4 AU) around a 1 Msun star, RK4 with a fixed 0.1-day step.  A
bench step is one RK4 step: 4 force evaluations of 16385 x 16384 pairs plus the stage
combinations.  Metric: simulated years per second (and interacting pairs per second).

  python bench.py [--gpus N --steps K --warmup W] [--impl ours|reference] [--mode mixed|fp64]

--impl reference times the FP64 CPU path (the oracle port of the reference's CPU code,
one core, the reference is single threaded) on the same workload.

The line also carries an "ensemble" section: 256 independent disks (N ~ U[512, 8192],
giants scaled by U[0.5, 2], seeds 65-320), RKF7(8) at tolerance 1e-10 with per-disk
adaptive steps, integrated over the same interval in four forms -- learned step proposer +
mixed-precision gravity + batching (the proposer trained first, untimed, on dithered attempt
logs of disks with seeds 1-64), the plain controller with mixed gravity, the plain
controller with FP64 gravity, both batched, and the plain FP64 form one disk at a time
through the single-disk API (a sample of the disks, the rate scaled to all of them).  Each
reports aggregate simulated years per second, the largest |dE/E| over the interval, the
rejected-attempt fraction and the event list.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "red.cuda.closeencounter_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from redgb import bodies, types as T  # noqa: E402
from redgb.replicas import max_over_ranks  # noqa: E402

WORKLOADS = {
    # name: (config, n, integrator, dt_day, adaptive)
    "self_gravitating_16384_rk4": ("self_gravitating", 16384, T.INT_RK4, 0.1, False),
    "planetesimal_disk_rkf78": ("planetesimal_disk", 1024, T.INT_RKF78, 0.001, True),
}
FLOP_PER_PAIR = 36  # the reference's own count (pp_disk.cu:170-184,293)
# DRAM bytes (read + write) per launch of the dominant kernel of the default workload, from
# one ncu capture of `python bench.py --no-ensemble --no-dense-ring --no-cpu-baseline --no-autotune
# --steps 3 --warmup 3`
# (profiles/grav_mixed_kernel_self_gravitating_16384.md, .../grav_fp64_pairpar_...md)
NCU_TRAFFIC = {("self_gravitating_16384_rk4", "mixed"): 1332224, ("self_gravitating_16384_rk4", "fp64"): 819712}


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return 0, 1, None
    import torch
    import torch.distributed as dist
    rank = int(os.environ["RANK"])
    local = int(os.environ.get("LOCAL_RANK", rank))
    torch.cuda.set_device(local)
    dist.init_process_group("nccl")
    return rank, ws, dist


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for k, name in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def flush_l2(buf):
    """Writes a buffer larger than the 129 MB L2 between timed steps."""
    buf.zero_()


def run_ours(args, rank, ws, dist):
    import torch

    from redgb import lib

    cfg, n, int_type, dt_day, adaptive = WORKLOADS[args.workload]
    dev = torch.cuda.current_device()
    disk = bodies.config_disk(cfg, n=n, seed=rank)
    thr = bodies.thresholds(collision_factor=0.0)
    mode = T.GRAVITY_MIXED if args.mode == "mixed" else T.GRAVITY_FP64
    pairs = disk.pairs_per_eval()
    evals_per_step = {T.INT_RK4: 4 + (1 if adaptive else 0), T.INT_RKF78: 13 if adaptive else 11,
                      T.INT_RK5: 6}[int_type]
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def make(mode_):
        s = lib.System(disk, thr)
        s.set_integrator(int_type, dt_day, adaptive, 1e-10)
        s.set_gravity_mode(mode_)
        return s

    def timed_steps(s, k, prof=False):
        """Per-step CUDA-event time on the library's stream, L2 flushed between steps."""
        ext = torch.cuda.ExternalStream(s.stream())
        tot = 0.0
        days = 0.0
        if prof:
            s.set_profiling(True)
            s.profile()
        for _ in range(k):
            flush_l2(flush)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(ext)
            days += s.step()
            e1.record(ext)
            e1.synchronize()
            tot += e0.elapsed_time(e1)
        p = s.profile() if prof else None
        if prof:
            s.set_profiling(False)
        return tot / 1e3, days, p

    sysm = make(mode)
    tune = sysm.autotune(3) if not args.no_autotune else None
    for _ in range(args.warmup):
        sysm.step()
    E0, _ = sysm.energy()
    k0 = sysm.counters()["n_kernels"]
    clocks = ClockSampler(dev)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    secs, days, prof = timed_steps(sysm, args.steps, prof=True)
    torch.cuda.synchronize()
    clk = clocks.stop()
    if dist:
        secs = max_over_ranks(secs, dist, device="cuda")
        dist.barrier()
    launches = sysm.counters()["n_kernels"] - k0
    E1, _ = sysm.energy()
    years = days / T.YEAR
    value = ws * years / secs
    pairs_per_s = ws * args.steps * evals_per_step * pairs / secs

    # e2e: the public API with pinned host buffers every step (state in, step, state out)
    r_h, v_h = (torch.empty(4 * disk.n_total, dtype=torch.float64, pin_memory=True).numpy().view(T.VEC)
                for _ in range(2))
    sysm.state(out=(r_h, v_h), params=False)
    nbytes = r_h.nbytes + v_h.nbytes
    t_e2e = 0.0
    e2e_days = 0.0
    for _ in range(args.steps):
        flush_l2(flush)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sysm.set_state(r_h, v_h)
        e2e_days += sysm.step()
        sysm.state(out=(r_h, v_h), params=False)
        t_e2e += time.perf_counter() - t0
    if dist:
        t_e2e = max_over_ranks(t_e2e, dist, device="cuda")
    e2e = {"value": ws * (e2e_days / T.YEAR) / t_e2e, "unit": "sim-years/s", "h2d_bytes_per_step": nbytes,
           "d2h_bytes_per_step": nbytes}

    out = None
    if rank == 0:
        from redgb import lib as L
        kind = 0 if mode == T.GRAVITY_MIXED else 1
        peak = L.measure_pipe_peak(kind)
        avg_ms = prof["gravity_ms"] / max(prof["gravity_launches"], 1)
        achieved = pairs * FLOP_PER_PAIR / (avg_ms * 1e-3) / 1e12
        # the FP64 form of the same step, for the mixed/FP64 comparison
        fp = make(T.GRAVITY_FP64)
        tune_fp = fp.autotune(1) if not args.no_autotune else None
        for _ in range(min(args.warmup, 3)):
            fp.step()
        k_fp = max(2, min(args.steps, 5))
        s_fp, d_fp, _ = timed_steps(fp, k_fp)
        ae = fp.calc_accel()
        fp.set_gravity_mode(T.GRAVITY_MIXED)
        am = fp.calc_accel()
        a_e = np.stack([ae[f] for f in "xyz"], 1)
        a_m = np.stack([am[f] for f in "xyz"], 1)
        rel = np.linalg.norm(a_m - a_e, axis=1) / np.linalg.norm(a_e, axis=1)
        out = {
            "metric": "sim-years/s", "value": value, "unit": "sim-years/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * secs / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64+f32" if mode == T.GRAVITY_MIXED else "f64",
            "data": "synthetic seeded disk (no public dataset exists)",
            "config": {"workload": args.workload, "bodies": disk.n_total, "integrator": "RK4 fixed 0.1 day",
                       "gravity": args.mode, "pairs_per_eval": pairs, "evals_per_step": evals_per_step,
                       "l2": "flushed between timed steps (256 MB write)", "parallelism": f"replicas x{ws}"},
            "pairs_per_s": pairs_per_s,
            "dE_over_E": abs((E1 - E0) / E0),
            "e2e": e2e,
            "gpu_launches": int(launches),
            "roofline": {"bound": "fp32" if kind == 0 else "fp64", "achieved": achieved, "peak": peak,
                         "unit": "TFLOP/s", "frac": achieved / peak,
                         "traffic": NCU_TRAFFIC.get((args.workload, args.mode)),
                         "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum, one capture",
                         "kernel": "grav_mixed_kernel" if kind == 0 else "grav_fp64_pairpar",
                         "peak_source": "measured FMA-chain microbenchmark on this GPU (rg_measure_pipe_peak)",
                         "flop_per_pair": FLOP_PER_PAIR, "avg_launch_ms": avg_ms},
            "fp64_form": {"value": (d_fp / T.YEAR) / s_fp, "ms_per_step": 1e3 * s_fp / k_fp,
                          "pairs_per_s": k_fp * evals_per_step * pairs / s_fp,
                          "fp64_peak_tflops": L.measure_pipe_peak(1),
                          "achieved_tflops": k_fp * evals_per_step * pairs * FLOP_PER_PAIR / s_fp / 1e12},
            "mixed_force_error": {"max_rel": float(rel.max()), "rms_rel": float(np.sqrt(np.mean(rel ** 2)))},
            "autotune": {"timed_form": tune, "fp64_form": tune_fp},
            "clocks": clk,
        }
        if ws == 1 and not args.no_cpu_baseline:
            out["cpu_baseline"] = cpu_baseline(args, disk, int_type, dt_day, adaptive, samples=args.cpu_steps)
        if not args.no_ensemble:
            out["ensemble"] = ensemble_section(args)
        if not args.no_dense_ring:
            out["dense_ring"] = dense_ring_section(args)
    return out


def cpu_baseline(args, disk, int_type, dt_day, adaptive, samples):
    """The oracle (the reference's CPU path restated in C, single thread) on the same disk."""
    import pyoracle
    o = pyoracle.OracleSystem(disk, bodies.thresholds(collision_factor=0.0))
    o.set_integrator(int_type, dt_day, adaptive, 1e-10)
    t0 = time.perf_counter()
    days = 0.0
    for _ in range(samples):
        days += o.step()
    secs = time.perf_counter() - t0
    return {"value": (days / T.YEAR) / secs, "unit": "sim-years/s", "cores": 1, "kind": "port",
            "sample": f"{samples} integrator steps of the same {disk.n_total}-body workload",
            "seconds": secs}


def run_reference(args, rank, ws):
    if rank != 0:
        return None
    cfg, n, int_type, dt_day, adaptive = WORKLOADS[args.workload]
    disk = bodies.config_disk(cfg, n=n, seed=0)
    import pyoracle
    o = pyoracle.OracleSystem(disk, bodies.thresholds(collision_factor=0.0))
    o.set_integrator(int_type, dt_day, adaptive, 1e-10)
    for _ in range(args.warmup):
        o.step()
    t0 = time.perf_counter()
    days = 0.0
    for _ in range(args.steps):
        days += o.step()
    secs = time.perf_counter() - t0
    value = (days / T.YEAR) / secs
    return {"metric": "sim-years/s", "value": value, "unit": "sim-years/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * secs / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "impl": "reference",
            "data": "synthetic seeded disk (no public dataset exists)",
            "config": {"workload": args.workload, "bodies": disk.n_total, "integrator": "RK4 fixed 0.1 day"},
            "cpu_baseline": {"value": value, "unit": "sim-years/s", "cores": 1, "kind": "port",
                             "sample": f"{args.steps} full integrator steps, single thread (the reference's "
                                       "CPU path is serial)"},
            "e2e": {"value": value, "unit": "sim-years/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def _oracle_disk(task):
    """One disk through the oracle on one host core (a spawned worker: no CUDA)."""
    import pyoracle
    seed, years, hill = task
    disk = bodies.config_disk("ensemble_member", seed=seed)
    o = pyoracle.OracleSystem(disk, bodies.thresholds(ejection=100.0, hit_centrum=0.05, collision_factor=1.0))
    o.set_integrator(T.INT_RKF78, 0.001, True, 1e-10)
    o.set_event_options(close_encounter=False, hill_factor=hill)
    t0 = time.perf_counter()
    o.advance(years * T.YEAR)
    return years, time.perf_counter() - t0


def cpu_ensemble(seeds, years, hill, processes):
    """The reference's CPU path (oracle) on `processes` host cores, one disk per process,
    all running at once: aggregate simulated years over the slowest process's time."""
    import multiprocessing as mp
    with mp.get_context("spawn").Pool(processes) as pool:
        res = pool.map(_oracle_disk, [(s, years, hill) for s in seeds], chunksize=1)
    yrs = sum(r[0] for r in res)
    slowest = max(r[1] for r in res)
    return {"value": yrs / slowest, "unit": "sim-years/s", "cores": processes, "kind": "port",
            "sample": f"{len(seeds)} disks of the same ensemble (seeds {seeds[0]}-{seeds[-1]}), {years} yr each, "
                      f"one process per core, all at once; slowest process {slowest:.2f} s"}


def dense_ring_section(args):
    """BASELINE config 4: 131 072 self-gravitating bodies in a narrow ring (a in [0.9, 1.1]
    AU, e, i ~ R(0.002)) around a 1 Msun star plus a 3e-6 Msun embryo at 1 AU, masses
    log-uniform in [1e-11, 1e-9] Msun; RKF5 adaptive at tolerance 1e-9, collisions at R1 + R2,
    close encounters at 3 mutual Hill radii.  A bounded sample of the 10-year run: mixed
    precision over `--dense-ring-steps` steps, and the first `--dense-ring-fp64-steps` steps
    in both precisions from the same state, whose event lists (type, pair, step) must agree."""
    import torch

    from redgb import lib

    disk = bodies.config_disk("dense_ring", n=args.dense_ring_n)
    thr = bodies.thresholds(ejection=100.0, hit_centrum=0.05, collision_factor=1.0)

    def make(mode):
        s = lib.System(disk, thr)
        s.set_integrator(T.INT_RK5, 0.001, True, 1e-9)
        s.set_event_options(close_encounter=False, hill_factor=3.0)
        s.set_gravity_mode(mode)
        return s

    def run(s, steps):
        events = []
        E0 = s.energy()[0]
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        days = 0.0
        for k in range(steps):  # the main loop's order (main.cu:201-251)
            s.check_for_ejection_hit_centrum()
            days += s.step()
            for name in ("check_for_collision", "check_for_close_encounter"):
                getattr(s, name)()
            for e in s.events():
                events.append((k, int(e["event_name"]), int(e["id1"]), int(e["id2"])))
        torch.cuda.synchronize()
        secs = time.perf_counter() - t0
        c = s.counters()
        return days, secs, events, abs((s.energy()[0] - E0) / E0), (c["n_passed_step"], c["n_tried_step"])

    mixed = make(T.GRAVITY_MIXED)
    tune = mixed.autotune(1)
    days, secs, ev_m, dE, att = run(mixed, args.dense_ring_steps)
    evals = 6 * args.dense_ring_steps
    pairs = disk.pairs_per_eval()
    cmp_m = make(T.GRAVITY_MIXED)
    _, _, ev_a, _, _ = run(cmp_m, args.dense_ring_fp64_steps)
    fp = make(T.GRAVITY_FP64)
    d_fp, s_fp, ev_f, dE_fp, _ = run(fp, args.dense_ring_fp64_steps)
    return {
        "workload": f"dense ring, {disk.n_total} bodies, RKF5 tol 1e-9, {args.dense_ring_steps} steps "
                    "(a sample of the 10-year run)",
        "mixed": {"sim_years_per_s": (days / T.YEAR) / secs, "steps": args.dense_ring_steps,
                  "ms_per_step": 1e3 * secs / args.dense_ring_steps, "simulated_days": days,
                  "pairs_per_s_lower_bound": evals * pairs / secs, "events": len(ev_m), "dE_over_E": dE,
                  "steps_passed_tried": att,
                  "autotune": tune},
        "fp64": {"sim_years_per_s": (d_fp / T.YEAR) / s_fp, "steps": args.dense_ring_fp64_steps,
                 "ms_per_step": 1e3 * s_fp / args.dense_ring_fp64_steps, "dE_over_E": dE_fp},
        "event_list_vs_fp64": {"steps": args.dense_ring_fp64_steps, "identical": ev_a == ev_f,
                               "n_mixed": len(ev_a), "n_fp64": len(ev_f)},
    }


def _compare_events(a, b, n_disks):
    """Two event lists of (disk, type, id1, id2, t_day): identical, or how many records
    differ, how many disks' lists are identical, and the earliest simulated time of a record
    found in one list only.  Over a long interval the trajectories of two precisions part
    chaotically near the giants, so grazing close encounters may be recorded in one run and
    not the other; every decision on a given state is taken in FP64 by both."""
    from collections import Counter, defaultdict
    ka, kb = [x[:4] for x in a], [x[:4] for x in b]
    ca, cb = Counter(ka), Counter(kb)
    only = (ca - cb) + (cb - ca)
    ta, tb = defaultdict(list), defaultdict(list)
    for x in a:
        ta[x[:4]].append(x[4])
    for x in b:
        tb[x[:4]].append(x[4])
    first = None
    for k in only:  # the first record of a pair beyond the count both lists share
        u, w = sorted(ta[k]), sorted(tb[k])
        t = (u if len(u) > len(w) else w)[min(len(u), len(w))]
        first = t if first is None else min(first, t)
    differing = {k[0] for k in only}
    return {"identical": ka == kb, "n": len(a), "n_fp64": len(b),
            "only_here": sum((ca - cb).values()), "only_fp64": sum((cb - ca).values()),
            "disks_identical": n_disks - len(differing), "disks": n_disks,
            "first_difference_yr": None if first is None else first / T.YEAR}


def ensemble_section(args):
    """The batched / mixed / learned forms against the plain FP64 form (module docstring)."""
    import torch

    from redgb import lib
    from redgb.ensemble import Ensemble
    from redgb.proposer import dataset_from_log, fit, set_dither

    tol = 1e-10
    hill = 3.0
    thr = bodies.thresholds(ejection=100.0, hit_centrum=0.05, collision_factor=1.0)
    warm_day = 10.0
    span_day = args.ensemble_years * T.YEAR

    def advance_timed(ens, t_stop):
        ext = torch.cuda.ExternalStream(ens.stream())
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        n = ens.advance(t_stop)
        e1.record(ext)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 1e3, n

    # proposer training (untimed): dithered plain-controller logs of seeds 1-64
    t0 = time.perf_counter()
    train = [bodies.config_disk("ensemble_member", seed=s) for s in range(1, 65)]
    ens = Ensemble(train, thr)
    ens.set_integrator(0.001, tol)
    ens.set_options(gravity_mode=T.GRAVITY_MIXED, hill_factor=hill)
    ens.set_step_log(1 << 22)
    set_dither(ens, 0.15, seed=7)
    ens.advance(args.train_years * T.YEAR)
    x, y = dataset_from_log(ens.step_log(1 << 22), tol)
    ens.close()
    del train
    net, loss = fit(x, y, seed=0, epochs=30)
    train_s = time.perf_counter() - t0

    t_cpu = time.perf_counter()
    disks = [bodies.config_disk("ensemble_member", seed=s) for s in range(65, 65 + args.ensemble_disks)]
    t_cpu = time.perf_counter() - t_cpu
    n_bodies = sum(d.n_total for d in disks)
    # the same ensemble's shapes from the GPU generator (its own random streams)
    from redgb.icgen import generate_disks, spec_like
    specs = [spec_like("ensemble_member", seed=s) for s in range(65, 65 + args.ensemble_disks)]
    generate_disks(specs[:1])  # first use: module load
    t_gpu = time.perf_counter()
    gen = generate_disks(specs)
    t_gpu = time.perf_counter() - t_gpu
    ic_generator = {"disks": len(gen), "bodies": int(sum(d.n_total for d in gen)), "gpu_seconds": t_gpu,
                    "cpu_python_seconds": t_cpu, "note": "GPU: rg_generate_disks incl. copies to the host; CPU: "
                    "bodies.config_disk (numpy draws, scalar Kepler solver per body)"}
    del gen
    # the reference's initial-condition program on the GPU: 256 of its Dvorak disks (2000
    # protoplanets each, scaled to the MMSN solids, moved to the barycentre)
    from redgb.icgen import dvorak_disk, populate_disks
    dv = [dvorak_disk(seed=s, n_pp=2000) for s in range(1, 257)]
    populate_disks(dv[:1])
    t_pop = time.perf_counter()
    pop = populate_disks(dv)
    t_pop = time.perf_counter() - t_pop
    ic_generator["populate"] = {"disks": len(pop), "bodies": int(sum(d.n_total for d in pop)), "gpu_seconds": t_pop,
                                "note": "rg_populate_disks incl. copies to the host"}
    del pop
    if not args.no_cpu_baseline:
        import icgen_ref  # the restatement, timed as the CPU figure on a sample of 4 disks
        t_ref = time.perf_counter()
        for d in dv[:4]:
            icgen_ref.populate(d)
        t_ref = (time.perf_counter() - t_ref) / 4
        ic_generator["populate"]["cpu_restatement_seconds_per_disk"] = t_ref
        ic_generator["populate"]["cpu_sample"] = "4 disks through oracle/icgen_ref.populate (numpy, one thread)"
    del dv

    def batched(mode, proposer):
        e = Ensemble(disks, thr)
        e.set_integrator(0.001, tol)
        e.set_options(gravity_mode=mode, hill_factor=hill)
        tune = None if args.no_autotune else e.autotune(2)  # tile shapes for these disks
        if proposer is not None:
            proposer.attach(e)
        e.advance(warm_day)
        E0 = [e.energy(k)[0] for k in range(len(disks))]
        st0 = [e.stats(k) for k in range(len(disks))]
        _, g0 = e.kernel_count()
        secs, _ = advance_timed(e, warm_day + span_day)
        _, g1 = e.kernel_count()
        st = [e.stats(k) for k in range(len(disks))]
        dE = max(abs((e.energy(k)[0] - E0[k]) / E0[k]) for k in range(len(disks)))
        sim_years = sum(a["t_day"] - b["t_day"] for a, b in zip(st, st0)) / T.YEAR
        tried = sum(a["n_tried_step"] - b["n_tried_step"] for a, b in zip(st, st0))
        failed = sum(a["n_failed_step"] - b["n_failed_step"] for a, b in zip(st, st0))
        ev, sysv = e.events()
        out = {"sim_years_per_s": sim_years / secs, "seconds": secs, "sim_years": sim_years, "attempts": tried,
               "rejected_frac": failed / max(tried, 1), "max_dE_over_E": dE, "events": int(len(ev)),
               "all_done": all(a["status"] == T.SYS_DONE for a in st),
               "iterations": int(g1 - g0), "ms_per_iteration": 1e3 * secs / max(g1 - g0, 1), "autotune": tune}
        if proposer is not None:
            out["proposed"] = sum(a["n_proposed"] for a in st)
            out["proposals_accepted"] = sum(a["n_proposal_accepted"] for a in st)
            out["fallbacks"] = sum(a["n_fallback"] for a in st)
        keys = sorted((int(k), int(r["event_name"]), int(r["id1"]), int(r["id2"]), float(r["t"]) / T.GAUSS)
                      for r, k in zip(ev, sysv))
        e.close()
        return out, keys

    learned, ev_l = batched(T.GRAVITY_MIXED, net)
    plain_mixed, ev_m = batched(T.GRAVITY_MIXED, None)
    plain_fp64, ev_f = batched(T.GRAVITY_FP64, None)

    # the plain FP64 form, one disk at a time through the single-disk API
    sample = disks[::max(1, len(disks) // args.sequential_sample)][:args.sequential_sample]
    seq_s, seq_years, seq_dE = 0.0, 0.0, 0.0
    for d in sample:
        s = lib.System(d, thr)
        s.set_integrator(T.INT_RKF78, 0.001, True, tol)
        s.set_event_options(close_encounter=False, hill_factor=hill)
        s.set_gravity_mode(T.GRAVITY_FP64)
        s.advance(warm_day)
        E0 = s.energy()[0]
        t_a = s.state()[4]
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        s.advance(warm_day + span_day)
        torch.cuda.synchronize()
        seq_s += time.perf_counter() - t1
        seq_years += (s.state()[4] - t_a) / T.YEAR
        seq_dE = max(seq_dE, abs((s.energy()[0] - E0) / E0))
        s.close()
    sequential = {"sim_years_per_s": seq_years / seq_s, "seconds": seq_s, "sim_years": seq_years,
                  "max_dE_over_E": seq_dE, "sample": f"{len(sample)} of {len(disks)} disks (every "
                  f"{max(1, len(disks) // args.sequential_sample)}th), the rate applies to all of them"}
    procs = max(1, min(os.cpu_count() or 1, 32))
    cpu = cpu_ensemble([65 + k for k in range(procs)], args.cpu_ensemble_years, hill, procs)
    return {
        "cpu_baseline": cpu,
        "speedup_vs_cpu_cores": learned["sim_years_per_s"] / cpu["value"],
        "workload": f"{len(disks)} disks, {n_bodies} bodies (N ~ U[512, 8192]), RKF7(8) tol 1e-10, "
                    f"{args.ensemble_years} yr per disk after a {warm_day:g}-day warm-up; CE at {hill:g} mutual "
                    "Hill radii, collisions at R1+R2, ejection 100 AU, hit-star 0.05 AU",
        "learned_mixed_batched": learned,
        "plain_mixed_batched": plain_mixed,
        "plain_fp64_batched": plain_fp64,
        "plain_fp64_sequential": sequential,
        "ic_generator": ic_generator,
        "speedup_vs_plain_fp64_sequential": learned["sim_years_per_s"] / sequential["sim_years_per_s"],
        "speedup_vs_plain_fp64_batched": learned["sim_years_per_s"] / plain_fp64["sim_years_per_s"],
        "learned_vs_plain_attempts": plain_mixed["attempts"] / max(learned["attempts"], 1),
        "event_lists": {name: _compare_events(ev, ev_f, len(disks)) for name, ev in (("learned_vs_fp64", ev_l),
                                                                                     ("mixed_vs_fp64", ev_m))},
        "proposer": {"train_records": int(len(x)), "train_disks": "seeds 1-64, dither 0.15",
                     "train_years": args.train_years, "loss": loss, "drift_std": float(np.std(y)),
                     "residual_std": net.residual_std, "safety": net.safety, "setup_seconds": train_s},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--mode", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--workload", default="self_gravitating_16384_rk4", choices=sorted(WORKLOADS))
    ap.add_argument("--cpu-steps", type=int, default=3)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-ensemble", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default launch shapes")
    ap.add_argument("--only-ensemble", action="store_true", help="the ensemble section alone (profiling)")
    ap.add_argument("--only-dense-ring", action="store_true", help="the dense-ring section alone (profiling)")
    ap.add_argument("--ensemble-disks", type=int, default=256)
    ap.add_argument("--ensemble-years", type=float, default=10.0)
    ap.add_argument("--train-years", type=float, default=10.0)
    ap.add_argument("--sequential-sample", type=int, default=8)
    ap.add_argument("--cpu-ensemble-years", type=float, default=1.0)
    ap.add_argument("--no-dense-ring", action="store_true")
    ap.add_argument("--dense-ring-steps", type=int, default=20)
    ap.add_argument("--dense-ring-n", type=int, default=None, help="planetesimals of the ring (default 131072)")
    ap.add_argument("--dense-ring-fp64-steps", type=int, default=2)
    args = ap.parse_args()
    if args.only_ensemble:
        print(json.dumps({"ensemble": ensemble_section(args)}))
        return
    if args.only_dense_ring:
        print(json.dumps({"dense_ring": dense_ring_section(args)}))
        return
    if args.impl == "reference":
        rank, ws = int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1"))
        out = run_reference(args, rank, ws)
    else:
        rank, ws, dist = dist_init()
        out = run_ours(args, rank, ws, dist)
        if dist:
            dist.destroy_process_group()
    if out is not None:
        print(json.dumps(out))


if __name__ == "__main__":
    main()
