"""Benchmark of the gravity + Runge-Kutta hot path on GB300 (one JSON line).

Headline workload: 16384 self-gravitating planetesimals (m log-uniform 1e-9..1e-7 Msun,
Sigma ~ r^-1.5 on 1..4 AU) around a 1 Msun star, RK4 with a fixed 0.1-day step.  A bench
step is one RK4 step: 4 force evaluations of 16385 x 16384 pairs plus the stage
combinations.  Metric: simulated years per second (and interacting pairs per second).  The
headline runs the FP64 form, whose results are bit-identical to the reference's FP64 CPU
path (the reference arm's arithmetic); `mixed_form` reports the mixed-precision form of the
same step beside it.

  python bench.py [--gpus N --steps K --warmup W] [--impl ours|reference] [--mode fp64|mixed]

--impl reference times the FP64 CPU path (the oracle port of the reference's CPU code,
one core, the reference is single threaded) on the same workload.

Further sections: `planetesimal_disk` (the plain FP64 1024-planetesimal disk through the
single-disk main loop against the oracle over the same interval); `ensemble` -- 256
independent disks (N ~ U[512, 8192], giants scaled by U[0.5, 2], seeds 65-320), RKF7(8) at
tolerance 1e-10 with per-disk adaptive steps, integrated over the same interval in four
forms: learned step proposer + mixed-precision gravity + batching (the proposer trained
first, untimed, on dithered attempt logs of disks with seeds 1-64), the plain controller
with mixed gravity, the plain controller with FP64 gravity, both batched, and the plain FP64
form one disk at a time through the single-disk API (a sample of the disks, the rate scaled
to all of them).  Each reports aggregate simulated years per second, the largest |dE/E|
over the interval, the rejected-attempt fraction and the event list (records found in one
list only, with their margins to the event thresholds); `kernel_time` splits an attempt by
kernel class with the stage combinations' HBM roofline; `dense_ring` samples the 131 072-body
ring.
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
# DRAM bytes (read + write) of one launch of each gravity kernel of the default workload, from
# one ncu capture of one launch (`-k <kernel> -c 1`) of `python bench.py --no-ensemble
# --no-dense-ring --no-cpu-baseline --no-planetesimal-disk --no-autotune --steps 3 --warmup 3`
NCU_TRAFFIC = {("self_gravitating_16384_rk4", "mixed"): 1332224, ("self_gravitating_16384_rk4", "fp64"): 809216}

def _hbm_peak():
    """The measured HBM copy bandwidth of the GB300s (MEASURED_PEAKS.json, written
    beside this file by the machine's set-up), else the figure it held when this was written."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"])
    except (OSError, KeyError, ValueError):
        return 6773.5


HBM_PEAK_GBS = _hbm_peak()


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


def stage_bytes_per_step(int_type, adaptive, n):
    """Algorithmic HBM bytes of one step's stage combinations and error norm: each combine
    reads y and its NTERM stage vectors and writes one vector, each vector 6 FP64 values per
    body (48 B, positions and velocities); the error norm reads its stage vectors.  RK4 fixed:
    three stage rows of one term and y_{n+1} of four (15 vectors); RKF7(8) adaptive (the
    reference's count, int_rungekutta8.cu:140-333): 93 vectors per attempt."""
    vectors = {(T.INT_RK4, False): 15, (T.INT_RKF78, True): 93}[(int_type, adaptive)]
    return vectors * 48 * n


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

    def e2e_steps(s, k):
        """The public API with pinned host buffers every step: state in, step, state out."""
        r_h, v_h = (torch.empty(4 * disk.n_total, dtype=torch.float64, pin_memory=True).numpy().view(T.VEC)
                    for _ in range(2))
        s.state(out=(r_h, v_h), params=False)
        nbytes = r_h.nbytes + v_h.nbytes
        t_e2e = 0.0
        days = 0.0
        for _ in range(k):
            flush_l2(flush)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            s.set_state(r_h, v_h)
            days += s.step()
            s.state(out=(r_h, v_h), params=False)
            t_e2e += time.perf_counter() - t0
        return t_e2e, days, nbytes

    def gravity_roofline(prof, kind, peak, traffic):
        avg_ms = prof["gravity_ms"] / max(prof["gravity_launches"], 1)
        achieved = pairs * FLOP_PER_PAIR / (avg_ms * 1e-3) / 1e12
        return {"bound": "fp32" if kind == 0 else "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                "frac": achieved / peak, "traffic": traffic,
                "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum, one capture of one launch",
                "kernel": "grav_mixed_kernel" if kind == 0 else "grav_fp64_pairpar",
                "peak_source": "measured " + ("FP32" if kind == 0 else "FP64") +
                               " FMA-chain microbenchmark on this GPU (rg_measure_pipe_peak)",
                "flop_per_pair": FLOP_PER_PAIR, "avg_launch_ms": avg_ms}

    def stage_roofline(prof, steps):
        """The stage-combine kernels of the timed steps against the measured HBM copy peak."""
        if not prof or not prof["stage_launches"]:
            return None
        nbytes = steps * stage_bytes_per_step(int_type, adaptive, disk.n_total)
        achieved = nbytes / (prof["stage_ms"] * 1e-3) / 1e9
        return {"bound": "hbm", "achieved": achieved, "peak": HBM_PEAK_GBS, "unit": "GB/s",
                "frac": achieved / HBM_PEAK_GBS, "launches": prof["stage_launches"],
                "avg_launch_us": 1e3 * prof["stage_ms"] / prof["stage_launches"],
                "bytes_per_step": nbytes / steps,
                "note": "algorithmic bytes (y and the stage vectors read, one vector written per combine) over "
                        "the combine kernels' CUDA-event time; at 16 385 bodies one combine moves 1.6-3.1 MB, "
                        "so launch latency, not bandwidth, sets its time",
                "peak_source": "MEASURED_PEAKS.json hbm_gbs (copy)"}

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
    t_e2e, e2e_days, nbytes = e2e_steps(sysm, args.steps)
    if dist:
        t_e2e = max_over_ranks(t_e2e, dist, device="cuda")
    e2e = {"value": ws * (e2e_days / T.YEAR) / t_e2e, "unit": "sim-years/s", "h2d_bytes_per_step": nbytes,
           "d2h_bytes_per_step": nbytes}

    out = None
    if rank == 0:
        from redgb import lib as L
        kind = 0 if mode == T.GRAVITY_MIXED else 1
        peak = L.measure_pipe_peak(kind)
        out = {
            "metric": "sim-years/s", "value": value, "unit": "sim-years/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * secs / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64+f32" if mode == T.GRAVITY_MIXED else "f64",
            "data": "synthetic seeded disk (no public dataset exists)",
            "config": {"workload": args.workload, "bodies": disk.n_total,
                       "integrator": "RK4 fixed 0.1 day" if int_type == T.INT_RK4 else "RKF7(8) tol 1e-10",
                       "gravity": args.mode + (" (bit-identical to the reference's FP64 CPU path)"
                                               if mode == T.GRAVITY_FP64 else ""),
                       "pairs_per_eval": pairs, "evals_per_step": evals_per_step,
                       "l2": "flushed between timed steps (256 MB write)", "parallelism": f"replicas x{ws}"},
            "e2e": e2e,
            "gpu_launches": int(launches),
            "roofline": gravity_roofline(prof, kind, peak, NCU_TRAFFIC.get((args.workload, args.mode))),
            "clocks": clk,
            "pairs_per_s": pairs_per_s,
            "dE_over_E": abs((E1 - E0) / E0),
            "stage_roofline": stage_roofline(prof, args.steps),
        }
        if ws == 1 and not args.no_cpu_baseline:
            out["cpu_baseline"] = cpu_baseline(args, disk, int_type, dt_day, adaptive, samples=args.cpu_steps)
        # the other gravity form of the same step: mixed precision next to the FP64 headline
        other = T.GRAVITY_FP64 if mode == T.GRAVITY_MIXED else T.GRAVITY_MIXED
        o_kind = 0 if other == T.GRAVITY_MIXED else 1
        fo = make(other)
        tune_o = fo.autotune(1) if not args.no_autotune else None
        for _ in range(min(args.warmup, 3)):
            fo.step()
        k_o = args.steps if other == T.GRAVITY_MIXED else max(2, min(args.steps, 5))
        s_o, d_o, p_o = timed_steps(fo, k_o, prof=True)
        t_oe, d_oe, _ = e2e_steps(fo, k_o)
        ae = (fo if other == T.GRAVITY_FP64 else sysm).calc_accel()
        am = (fo if other == T.GRAVITY_MIXED else sysm).calc_accel()
        a_e = np.stack([ae[f] for f in "xyz"], 1)
        a_m = np.stack([am[f] for f in "xyz"], 1)
        rel = np.linalg.norm(a_m - a_e, axis=1) / np.linalg.norm(a_e, axis=1)
        name = "mixed_form" if other == T.GRAVITY_MIXED else "fp64_form"
        out[name] = {
            "value": (d_o / T.YEAR) / s_o, "unit": "sim-years/s", "ms_per_step": 1e3 * s_o / k_o, "steps": k_o,
            "dtype": "f64+f32" if other == T.GRAVITY_MIXED else "f64",
            "e2e": {"value": (d_oe / T.YEAR) / t_oe, "unit": "sim-years/s"},
            "pairs_per_s": k_o * evals_per_step * pairs / s_o,
            "roofline": gravity_roofline(p_o, o_kind, L.measure_pipe_peak(o_kind),
                                         NCU_TRAFFIC.get((args.workload, "mixed" if o_kind == 0 else "fp64"))),
            "note": "mixed precision: FP32 pair terms (FP64-split displacements, rsqrt with a first-order r^-3 "
                    "correction), double-float heavy pairs, event decisions re-taken in FP64"
                    if other == T.GRAVITY_MIXED else "bit-identical FP64 form"}
        out["mixed_force_error"] = {"max_rel": float(rel.max()), "rms_rel": float(np.sqrt(np.mean(rel ** 2)))}
        out["autotune"] = {"timed_form": tune, "other_form": tune_o}
        if not args.no_planetesimal_disk:
            out["planetesimal_disk"] = planetesimal_disk_section(args)
        if not args.no_ensemble:
            out["ensemble"] = ensemble_section(args)
        if not args.no_dense_ring:
            out["dense_ring"] = dense_ring_section(args)
    return out


def planetesimal_disk_section(args):
    """The plain FP64 planetesimal-disk workload (star, giants of 9.55e-4 and 2.86e-4 Msun at
    5.2 and 9.54 AU, 1024 planetesimals, seed 0; RKF7(8) tol 1e-10; close encounters at 3
    mutual Hill radii, collisions at R1 + R2, ejection 100 AU, hit-star 0.05 AU) over a
    stated sample of its 1000 years, through the single-disk C ABI's main loop (rg_advance),
    against the oracle (the reference's CPU path, one thread) over the same interval: both
    rates, and whether event lists, step counts and final states are identical bit for bit."""
    import torch

    import pyoracle
    from redgb import lib

    disk = bodies.config_disk("planetesimal_disk")
    thr = bodies.thresholds(ejection=100.0, hit_centrum=0.05, collision_factor=1.0)
    stop = args.c0_years * T.YEAR
    res = {}
    runs = {}
    for name, mk in (("gpu_fp64", lambda: lib.System(disk, thr)), ("gpu_mixed", lambda: lib.System(disk, thr)),
                     ("oracle", lambda: pyoracle.OracleSystem(disk, thr))):
        s = mk()
        if name == "gpu_mixed":
            s.set_gravity_mode(T.GRAVITY_MIXED)
        s.set_integrator(T.INT_RKF78, 0.001, True, 1e-10)
        s.set_event_options(hill_factor=3.0)
        if name != "oracle":
            torch.cuda.synchronize()
        t0 = time.perf_counter()
        n = s.advance(stop)
        if name != "oracle":
            torch.cuda.synchronize()
        secs = time.perf_counter() - t0
        ev = s.events()
        runs[name] = (n, ev, s.state(internal=True))
        res[name] = {"sim_years_per_s": args.c0_years / secs, "seconds": secs, "steps": int(n),
                     "ms_per_step": 1e3 * secs / max(n, 1), "events": int(len(ev))}
    res["oracle"].update({"cores": 1, "kind": "port"})
    n_f, ev_f, st_f = runs["gpu_fp64"]
    n_o, ev_o, st_o = runs["oracle"]
    same_state = all(a.tobytes() == b.tobytes() for a, b in zip(st_f[:2], st_o[:2])) and st_f[4] == st_o[4]
    km = [(int(e["event_name"]), int(e["id1"]), int(e["id2"])) for e in runs["gpu_mixed"][1]]
    ko = [(int(e["event_name"]), int(e["id1"]), int(e["id2"])) for e in ev_o]
    return {
        "workload": f"planetesimal disk, {disk.n_total} bodies, RKF7(8) tol 1e-10, {args.c0_years:g} of its "
                    "1000 years (the whole run is a GPU test against the oracle)",
        **res,
        "gpu_fp64_vs_oracle": {"events_identical": ev_f.tobytes() == ev_o.tobytes(), "steps_equal": n_f == n_o,
                               "state_identical": bool(same_state)},
        "gpu_mixed_vs_oracle": {"event_keys_identical": km == ko, "steps_equal": runs["gpu_mixed"][0] == n_o},
        "speedup_gpu_fp64_vs_oracle": res["gpu_fp64"]["sim_years_per_s"] / res["oracle"]["sim_years_per_s"],
    }


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
    """The dense-ring stress workload: 131 072 self-gravitating bodies in a narrow ring (a in [0.9, 1.1]
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
    fp = make(T.GRAVITY_FP64)
    d_fp, s_fp, _, dE_fp, _ = run(fp, args.dense_ring_fp64_steps)
    # the event-list comparison on the same ring with the bodies' collision radii x RADIUS_X:
    # a few hundred overlapping and Hill pairs, so that both precisions record events
    crowded = disk.copy()
    crowded.p["radius"][2:] *= args.dense_ring_radius_x
    disk_saved = disk
    disk = crowded
    _, _, ev_a, _, _ = run(make(T.GRAVITY_MIXED), args.dense_ring_fp64_steps)
    _, _, ev_f, _, _ = run(make(T.GRAVITY_FP64), args.dense_ring_fp64_steps)
    disk = disk_saved
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
                               "n_mixed": len(ev_a), "n_fp64": len(ev_f),
                               "types": sorted({T.EVENT_NAMES[x[1]] for x in ev_f}),
                               "ring": f"the same ring with collision radii x{args.dense_ring_radius_x:g}"},
    }


def event_margin(rec, f_rad=1.0, hill=3.0, m_star=1.0, ejection=100.0, hit=0.05):
    """How far a record sits inside its event's threshold, relative: COLLISION
    d / (f (R1 + R2)) - 1; CLOSE_ENCOUNTER (mutual Hill sphere) d / (hill R_H) - 1 with
    R_H^3 = (m1 + m2) / (3 M_star) h^3, h the mean of the two star distances, taken here as
    the bodies' distances from the barycentre (the star sits within 0.01 AU of it, so the
    figure is good to about 1e-3); EJECTION d / R_ej - 1; HIT_CENTRUM d / R_hit - 1.  Near 0:
    a grazing event that a last-digit difference of the trajectory can flip."""
    name = int(rec["event_name"])
    d = float(rec["d"])
    if name == T.EVENT_COLLISION:
        return d / (f_rad * (float(rec["p1"]["radius"]) + float(rec["p2"]["radius"]))) - 1.0
    if name == T.EVENT_CLOSE_ENCOUNTER:
        r1 = np.sqrt(sum(float(rec["r1"][c]) ** 2 for c in "xyz"))
        r2 = np.sqrt(sum(float(rec["r2"][c]) ** 2 for c in "xyz"))
        h = 0.5 * (r1 + r2)
        rh = ((float(rec["p1"]["mass"]) + float(rec["p2"]["mass"])) / (3.0 * m_star)) ** (1.0 / 3.0) * h
        return d / (hill * rh) - 1.0
    if name == T.EVENT_EJECTION:
        return d / ejection - 1.0
    if name == T.EVENT_HIT_CENTRUM:
        return d / hit - 1.0
    return None


def _compare_events(a, b, n_disks):
    """Two event lists of records (disk, type, id1, id2, t_day, margin): identical, or how
    many records differ, how many disks' lists are identical, and every record found in one
    list only, with its time and its margin to the event's threshold.  Over a long interval
    the trajectories of two precisions part chaotically near the giants, so grazing close
    encounters may be recorded in one run and not the other; every decision on a given
    state is taken in FP64 by both."""
    from collections import Counter, defaultdict
    ka, kb = [x[:4] for x in a], [x[:4] for x in b]
    ca, cb = Counter(ka), Counter(kb)
    only = (ca - cb) + (cb - ca)
    ra, rb = defaultdict(list), defaultdict(list)
    for x in a:
        ra[x[:4]].append(x)
    for x in b:
        rb[x[:4]].append(x)
    diffs = []
    for k in only:  # the records of a pair beyond the count both lists share
        u, w = sorted(ra[k], key=lambda x: x[4]), sorted(rb[k], key=lambda x: x[4])
        side, extra = ("here", u[len(w):]) if len(u) > len(w) else ("fp64", w[len(u):])
        for x in extra:
            diffs.append({"list": side, "disk": x[0], "type": T.EVENT_NAMES[x[1]], "id1": x[2], "id2": x[3],
                          "t_yr": x[4] / T.YEAR, "margin": x[5]})
    diffs.sort(key=lambda r: r["t_yr"])
    differing = {k[0] for k in only}
    margins = [abs(r["margin"]) for r in diffs if r["margin"] is not None]
    return {"identical": ka == kb, "n": len(a), "n_fp64": len(b),
            "only_here": sum((ca - cb).values()), "only_fp64": sum((cb - ca).values()),
            "disks_identical": n_disks - len(differing), "disks": n_disks,
            "first_difference_yr": diffs[0]["t_yr"] if diffs else None,
            "largest_abs_margin": max(margins) if margins else None,
            "differing_records": diffs[:40]}


def ensemble_attempts(args):
    """Profiling aid: the benchmark ensemble (`--ensemble-disks` disks) in one form, attempts
    launched directly rather than from the graph (so that a profiler sees every kernel), with
    the device time of each kernel class.  A proposer form uses an untrained network (its
    launches and their cost are those of a trained one)."""
    from redgb.ensemble import Ensemble
    from redgb.proposer import Proposer

    thr = bodies.thresholds(ejection=100.0, hit_centrum=0.05, collision_factor=1.0)
    disks = [bodies.config_disk("ensemble_member", seed=s) for s in range(65, 65 + args.ensemble_disks)]
    e = Ensemble(disks, thr)
    e.set_integrator(0.001, 1e-10)
    e.set_options(gravity_mode=T.GRAVITY_FP64 if args.ensemble_form == "fp64" else T.GRAVITY_MIXED, hill_factor=3.0,
                  use_graph=False)
    net = None
    if args.ensemble_form == "learned":
        net = Proposer(seed=0)
        net.set_normalisation([0.0] * 8, [1.0] * 8)
        net.attach(e, safety=0.98)
    e.advance(1e9, max_attempts=args.ensemble_attempts)
    e.set_profiling(True)
    e.profile()
    e.advance(1e9, max_attempts=args.ensemble_attempts)
    p = e.profile()
    e.close()
    k = args.ensemble_attempts
    return {"form": args.ensemble_form, "disks": len(disks), "bodies": int(sum(d.n_total for d in disks)),
            "attempts": k, "ms_per_attempt": (p["gravity_ms"] + p["stage_ms"] + p["other_ms"]) / k,
            "gravity_ms_per_attempt": p["gravity_ms"] / k, "stage_ms_per_attempt": p["stage_ms"] / k,
            "other_ms_per_attempt": p["other_ms"] / k}


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
    x, y, grp = dataset_from_log(ens.step_log(1 << 22), tol, with_groups=True)
    ens.close()
    del train
    net, loss = fit(x, y, seed=0, epochs=30, groups=grp)
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
        secs, n_att = advance_timed(e, warm_day + span_day)
        _, g1 = e.kernel_count()
        st = [e.stats(k) for k in range(len(disks))]
        dEk = [abs((e.energy(k)[0] - E0[k]) / E0[k]) for k in range(len(disks))]
        sim_years = sum(a["t_day"] - b["t_day"] for a, b in zip(st, st0)) / T.YEAR
        tried = sum(a["n_tried_step"] - b["n_tried_step"] for a, b in zip(st, st0))
        failed = sum(a["n_failed_step"] - b["n_failed_step"] for a, b in zip(st, st0))
        ev, sysv = e.events()
        # a merge is inelastic (the pair's relative kinetic energy is lost) and an ejection or a
        # hit-star merger removes a body: energy conservation is judged on the disks without one
        merged = {int(k) for r, k in zip(ev, sysv) if int(r["event_name"]) != T.EVENT_CLOSE_ENCOUNTER}
        dE_free = [v for k, v in enumerate(dEk) if k not in merged]
        out = {"sim_years_per_s": sim_years / secs, "seconds": secs, "sim_years": sim_years, "attempts": tried,
               "rejected_frac": failed / max(tried, 1), "max_dE_over_E": max(dEk),
               "max_dE_over_E_disks_without_merges": max(dE_free) if dE_free else None,
               "disks_with_merges": len(merged), "events": int(len(ev)),
               "all_done": all(a["status"] == T.SYS_DONE for a in st),
               "iterations": int(n_att), "ms_per_iteration": 1e3 * secs / max(n_att, 1),
               "graph_launches": int(g1 - g0), "autotune": tune}
        if proposer is not None:
            out["proposed"] = sum(a["n_proposed"] for a in st)
            out["proposals_accepted"] = sum(a["n_proposal_accepted"] for a in st)
            out["fallbacks"] = sum(a["n_fallback"] for a in st)
        keys = sorted((int(k), int(r["event_name"]), int(r["id1"]), int(r["id2"]), float(r["t"]) / T.GAUSS,
                       event_margin(r)) for r, k in zip(ev, sysv))
        e.close()
        return out, keys

    learned, ev_l = batched(T.GRAVITY_MIXED, net)
    plain_mixed, ev_m = batched(T.GRAVITY_MIXED, None)
    plain_fp64, ev_f = batched(T.GRAVITY_FP64, None)

    def profiled(mode, attempts=16, proposer=None):
        """Device time by kernel class over `attempts` attempts launched directly with CUDA
        events (rg_ens_set_profiling), every disk running: the stage-combine and error-norm
        kernels against the measured HBM peak at the reference's algorithmic bytes
        (93 vectors of 48 B per body and attempt, int_rungekutta8.cu:140-333)."""
        e = Ensemble(disks, thr)
        e.set_integrator(0.001, tol)
        e.set_options(gravity_mode=mode, hill_factor=hill)
        if not args.no_autotune:
            e.autotune(2)
        if proposer is not None:
            proposer.attach(e)
        e.advance(warm_day)
        e.set_profiling(True)
        e.profile()
        e.advance(1e9, max_attempts=attempts)
        p = e.profile()
        e.set_profiling(False)
        e.close()
        nbytes = attempts * stage_bytes_per_step(T.INT_RKF78, True, n_bodies)
        achieved = nbytes / (p["stage_ms"] * 1e-3) / 1e9
        return {"attempts": attempts, "ms_per_attempt": (p["gravity_ms"] + p["stage_ms"] + p["other_ms"]) / attempts,
                "gravity_ms_per_attempt": p["gravity_ms"] / attempts, "stage_ms_per_attempt": p["stage_ms"] / attempts,
                "other_ms_per_attempt": p["other_ms"] / attempts,
                "stage_roofline": {"bound": "hbm", "achieved": achieved, "peak": HBM_PEAK_GBS, "unit": "GB/s",
                                   "frac": achieved / HBM_PEAK_GBS, "bytes_per_attempt": nbytes / attempts,
                                   "launches": p["stage_launches"],
                                   "peak_source": "MEASURED_PEAKS.json hbm_gbs (copy)"}}

    kernel_time = {"learned_mixed": profiled(T.GRAVITY_MIXED, proposer=net), "mixed": profiled(T.GRAVITY_MIXED),
                   "fp64": profiled(T.GRAVITY_FP64)}

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
        s.advance(warm_day + args.sequential_years * T.YEAR)
        torch.cuda.synchronize()
        seq_s += time.perf_counter() - t1
        seq_years += (s.state()[4] - t_a) / T.YEAR
        seq_dE = max(seq_dE, abs((s.energy()[0] - E0) / E0))
        s.close()
    sequential = {"sim_years_per_s": seq_years / seq_s, "seconds": seq_s, "sim_years": seq_years,
                  "max_dE_over_E": seq_dE, "sample": f"{len(sample)} of {len(disks)} disks (every "
                  f"{max(1, len(disks) // args.sequential_sample)}th), {args.sequential_years:g} yr each; the rate "
                  "applies to all of them"}
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
        "kernel_time": kernel_time,
        "ic_generator": ic_generator,
        "speedup_vs_plain_fp64_sequential": learned["sim_years_per_s"] / sequential["sim_years_per_s"],
        "speedup_vs_plain_fp64_batched": learned["sim_years_per_s"] / plain_fp64["sim_years_per_s"],
        "learned_vs_plain_attempts": plain_mixed["attempts"] / max(learned["attempts"], 1),
        "event_lists": {name: _compare_events(ev, ev_f, len(disks)) for name, ev in (("learned_vs_fp64", ev_l),
                                                                                     ("mixed_vs_fp64", ev_m))},
        "proposer": {"train_records": int(len(x)), "train_disks": "seeds 1-64, dither 0.15",
                     "holdout": "whole disks (10% for the safety factor, 10% for the epoch kept)", "expected_cost": getattr(net, "expected_cost", None),
                     "train_years": args.train_years, "loss": loss, "drift_std": float(np.std(y)),
                     "residual_std": net.residual_std, "holdout_drift_std": net.holdout_drift_std,
                     "best_epoch": net.best_epoch,
                     "safety": net.safety, "setup_seconds": train_s},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--mode", default="fp64", choices=["mixed", "fp64"],
                    help="gravity form of the headline (fp64: bit-identical to the reference's CPU path)")
    ap.add_argument("--workload", default="self_gravitating_16384_rk4", choices=sorted(WORKLOADS))
    ap.add_argument("--cpu-steps", type=int, default=3)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-ensemble", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default launch shapes")
    ap.add_argument("--only-ensemble", action="store_true", help="the ensemble section alone (profiling)")
    ap.add_argument("--only-dense-ring", action="store_true", help="the dense-ring section alone (profiling)")
    ap.add_argument("--only-planetesimal-disk", action="store_true",
                    help="the planetesimal-disk section alone (profiling; see --c0-years)")
    ap.add_argument("--ensemble-attempts", type=int, default=0,
                    help="profiling: the ensemble's attempts launched directly (no graph), after as many "
                         "warm-up attempts, in the form --ensemble-form; prints their device times")
    ap.add_argument("--ensemble-form", default="mixed", choices=["mixed", "learned", "fp64"])
    ap.add_argument("--ensemble-disks", type=int, default=256)
    ap.add_argument("--ensemble-years", type=float, default=100.0,
                    help="simulated years per disk of the batched ensemble forms (the configuration's 100)")
    ap.add_argument("--sequential-years", type=float, default=10.0,
                    help="simulated years per disk of the one-disk-at-a-time FP64 sample")
    ap.add_argument("--train-years", type=float, default=450.0,
                    help="years of dithered training runs of the 64 training disks (about 1e6 step records)")
    ap.add_argument("--sequential-sample", type=int, default=8)
    ap.add_argument("--cpu-ensemble-years", type=float, default=1.0)
    ap.add_argument("--no-dense-ring", action="store_true")
    ap.add_argument("--no-planetesimal-disk", action="store_true")
    ap.add_argument("--c0-years", type=float, default=100.0, help="planetesimal-disk sample (years)")
    ap.add_argument("--dense-ring-steps", type=int, default=20)
    ap.add_argument("--dense-ring-n", type=int, default=None, help="planetesimals of the ring (default 131072)")
    ap.add_argument("--dense-ring-fp64-steps", type=int, default=2)
    ap.add_argument("--dense-ring-radius-x", type=float, default=40.0,
                    help="collision-radius factor of the ring whose event lists are compared")
    args = ap.parse_args()
    if args.only_ensemble:
        print(json.dumps({"ensemble": ensemble_section(args)}))
        return
    if args.only_dense_ring:
        print(json.dumps({"dense_ring": dense_ring_section(args)}))
        return
    if args.only_planetesimal_disk:
        print(json.dumps({"planetesimal_disk": planetesimal_disk_section(args)}))
        return
    if args.ensemble_attempts > 0:
        print(json.dumps({"ensemble_attempts": ensemble_attempts(args)}))
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
