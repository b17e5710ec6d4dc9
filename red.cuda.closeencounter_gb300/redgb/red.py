"""Command-line driver with the reference's options, inputs and output files.

    python -m redgb.red [-gpu] [-ef] -iDir DIR -p parameters.txt -ic bodies.txt
                        [-result NAME] [-event NAME] [-info NAME] [-log NAME] [-id_dev K] [-v]

The options are those of the reference's ``red`` (options.cpp:57-196); the parameter file
(parameter.cpp:55-285) and the body list (pp_disk.cu:1576-1683) are read in the reference's
formats, and the result, event, info and log files are written into the input directory
under the reference's names (main.cu:28-71: with ``-ef`` the prefix is
``R_gpu_{ns}_{as|fs}_{E|RK4|RK5|RKF8}_``).  Result and event files are byte-identical to
the reference's for the same run (redgb.io).  The integration runs on the GPU only: this
library has no CPU path, so ``-cpu`` is refused; ``-ups`` (padded storage), ``-n_tpb`` and
``-gd`` (gas disk) belong to the reference's own kernels and are refused too.
"""
from __future__ import annotations

import os
import sys
import time

from . import bodies, io as rio, types as T

SHORT_NAME = {T.INT_EULER: "E", T.INT_RK4: "RK4", T.INT_RK5: "RK5", T.INT_RKF78: "RKF8"}
INTEGRATORS = {"e": T.INT_EULER, "euler": T.INT_EULER, "rk4": T.INT_RK4, "rungekutta4": T.INT_RK4,
               "rk5": T.INT_RK5, "rungekutta5": T.INT_RK5, "rkf8": T.INT_RKF78, "rungekuttafehlberg8": T.INT_RKF78}


class UsageError(ValueError):
    pass


def parse_options(argv):
    o = {"iDir": ".", "p": None, "ic": None, "ef": False, "verbose": False, "device": 0,
         "result": "result", "event": "event", "info": "info", "log": "log"}
    names = {"-iDir": "iDir", "--inputDir": "iDir", "-p": "p", "--parameters": "p", "-ic": "ic",
             "--initial_conditions": "ic", "-result": "result", "--result-filename": "result", "-event": "event",
             "--event-filename": "event", "-info": "info", "--info-filename": "info", "-log": "log",
             "--log-filename": "log"}
    i = 0
    while i < len(argv):
        a = argv[i]
        if a in names:
            if i + 1 >= len(argv):
                raise UsageError(f"missing value after {a}")
            o[names[a]] = argv[i + 1]
            i += 2
            continue
        if a in ("-id_dev", "--id_active_device"):
            o["device"] = int(argv[i + 1])
            i += 2
            continue
        if a == "-ef":
            o["ef"] = True
        elif a in ("-v", "--verbose"):
            o["verbose"] = True
        elif a in ("-gpu", "--gpu"):
            pass
        elif a in ("-cpu", "--cpu"):
            raise UsageError("-cpu: this implementation runs on the GPU only (no CPU path)")
        elif a in ("-ups", "--use-padded-storage", "-n_tpb", "--n_thread-per-block", "-gd", "--gas_disk"):
            raise UsageError(f"{a} is not supported (the reference's kernel launch options and gas disk)")
        elif a in ("-h", "--help"):
            raise UsageError(__doc__)
        else:
            raise UsageError(f"unknown option {a}")
        i += 1
    if not o["p"] or not o["ic"]:
        raise UsageError("-p <parameter file> and -ic <body file> are required")
    return o


def read_parameter_file(path):
    """key = value lines (parameter.cpp:55-285): keys are case-insensitive, times in years."""
    prm = {"name": "", "description": "", "int_type": T.INT_RKF78, "adaptive": False, "tolerance": 1e-10,
           "error_check_for_tp": False, "close_encounter": False, "inner_steps": True, "start_time": 0.0,
           "length": 0.0, "output_interval": 0.0, "ejection": 0.0, "hit_centrum": 0.0, "collision_factor": 0.0,
           "output_type": "text"}

    def boolean(k, v):
        if v not in ("true", "false"):
            raise ValueError(f"Invalid value at: {k}")
        return v == "true"

    for line in open(path).read().splitlines():
        if not line.strip():
            continue
        if "=" not in line:
            raise ValueError(f"Invalid key/value pair: {line}.")
        key, value = (x.strip() for x in line.split("=", 1))
        key = key.lower()
        if key in ("name", "description"):
            prm[key] = value
        elif key == "integrator":
            if value.lower() not in INTEGRATORS:
                raise ValueError(f"Invalid integrator type: {value}")
            prm["int_type"] = INTEGRATORS[value.lower()]
        elif key == "tolerance":
            prm["adaptive"], prm["tolerance"] = True, float(value)
        elif key in ("error_check_for_tp", "close_encounter", "inner_steps"):
            prm[key] = boolean(key, value)
        elif key in ("start_time", "length", "output_interval"):
            prm[key] = float(value) * T.YEAR
        elif key in ("ejection", "hit_centrum"):
            prm[key] = float(value)
        elif key in ("radii_enhance_factor", "collision_factor"):
            prm["collision_factor"] = float(value)
        elif key == "output_type":
            if value not in ("text", "ascii", "binary"):
                raise ValueError(f"Invalid value at: {key}")
            prm["output_type"] = "binary" if value == "binary" else "text"
        elif key == "frame_center":
            # parameter.cpp:257-266
            if value.lower() == "astro":
                prm["frame"] = T.FRAME_ASTRO
            elif value.lower() == "bary":
                prm["frame"] = T.FRAME_BARY
            else:
                raise ValueError(f"Invalid value at: {key}")
        else:
            raise ValueError(f"Invalid parameter: {key}")
    return prm


def output_paths(opt, prm):
    prefix = ""
    if opt["ef"]:
        prefix = "_".join(["R", "gpu", "ns", "as" if prm["adaptive"] else "fs", SHORT_NAME[prm["int_type"]]]) + "_"
    d = opt["iDir"]
    result_ext = "bin" if prm["output_type"] == "binary" else "txt"
    return {k: os.path.join(d, prefix + opt[k] + "." + (result_ext if k == "result" else "txt"))
            for k in ("result", "event", "info", "log")}


def run(argv):
    from . import lib

    opt = parse_options(argv)
    prm = read_parameter_file(os.path.join(opt["iDir"], opt["p"]))
    disk = bodies.read_body_file(os.path.join(opt["iDir"], opt["ic"]))
    paths = output_paths(opt, prm)
    thr = bodies.thresholds(ejection=prm["ejection"], hit_centrum=prm["hit_centrum"],
                            collision_factor=prm["collision_factor"])
    binary = prm["output_type"] == "binary"
    s = lib.System(disk, thr, frame=prm.get("frame", T.FRAME_BARY))
    s.set_integrator(prm["int_type"], 0.001, prm["adaptive"], prm["tolerance"], prm["error_check_for_tp"])
    s.set_event_options(close_encounter=prm["close_encounter"], inner_steps=prm["inner_steps"])
    s.set_time(prm["start_time"])
    stop = (prm["start_time"] + prm["length"]) * T.GAUSS
    oi = prm["output_interval"] * T.GAUSS
    f_rad = prm["collision_factor"]
    t0 = time.time()
    with open(paths["result"], "wb" if binary else "w") as res, open(paths["event"], "w") as evf, \
            open(paths["log"], "w") as logf, open(paths["info"], "w") as info:
        logf.write(time.strftime("%Y-%m-%d %H:%M:%S") + " starting: " + " ".join(["red"] + list(argv)) + "\n")

        def snapshot():
            r, v, p, md, t = s.state()
            (rio.write_result_binary if binary else rio.write_result_ascii)(res, t, r, v, p, md, disk.names)

        def events():
            ev = s.events()
            rio.write_events(evf, ev)
            for e in ev:
                logf.write(time.strftime("%Y-%m-%d %H:%M:%S") + " " + T.EVENT_NAMES[int(e["event_name"])] +
                           f" {int(e['id1']):8d} {int(e['id2']):8d} \n")

        snapshot()
        ps, n = 0.0, 0
        while s.time(internal=True) <= stop:  # main.cu:176-263
            if oi <= abs(ps):
                ps = 0.0
                snapshot()
            s.check_for_ejection_hit_centrum()
            events()
            dt = s.step() * T.GAUSS
            n += 1
            ps += abs(dt)
            if prm["close_encounter"] and prm["inner_steps"]:
                if 0.0 < f_rad:
                    s.check_for_close_encounter()
            elif not prm["close_encounter"] and prm["inner_steps"]:
                if 0.0 < f_rad:
                    s.check_for_collision()
                s.check_for_rebuild_vectors(8)
            events()
        if 0.0 < ps:  # the last snapshot, unless it was just written (main.cu:266-279)
            snapshot()
        c = s.counters()
        info.write(f"steps: {n}, passed: {c['n_passed_step']}, failed: {c['n_failed_step']}, "
                   f"events: {c['n_event'][0]}, wall: {time.time() - t0:.3f} s\n")
    return paths


def main(argv=None):
    """Exit status 0 on success, 2 for a usage error, 1 for an unreadable or invalid input
    file (the reference prints the message and exits, main.cu:288-303)."""
    try:
        paths = run(sys.argv[1:] if argv is None else argv)
    except UsageError as x:
        print(x, file=sys.stderr)
        return 2
    except (OSError, ValueError) as x:
        print(f"red: {x}", file=sys.stderr)
        return 1
    if "-v" in (sys.argv if argv is None else argv):
        print("\n".join(paths.values()))
    return 0


if __name__ == "__main__":
    sys.exit(main())
