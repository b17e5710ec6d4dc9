"""rg_autotune: the chosen launch shape is at least as fast as the one before, FP64 results
stay bit-exact (every candidate sums in the reference's order) and mixed-mode forces stay
within their tolerance."""
import numpy as np
import pytest

import helpers as H
from redgb import bodies, lib, types as T

pytestmark = pytest.mark.gpu


def test_fp64_autotune_keeps_bit_exact_run(gpulib):
    disk, params, result, events = H.load_fixture("disk_si_rkf78_collide")
    s = lib.System(disk, H.thresholds_of(params))
    t = s.autotune(reps=2)
    assert t["candidates"] == 9
    assert t["pairpar_sinks"] in (8, 16, 32) and t["rowseq_max_src"] in (32, 64, 128)
    assert t["ms_per_eval"] <= t["ms_before"] * 1.001
    assert s.counters()["n_gravity_evals"] == 0
    snaps, evs, _ = H.run_fixture(s, params)
    assert H.compare_result(H.snapshots_as_result(snaps), result) == []
    assert H.compare_events(evs, events) == []


def test_mixed_autotune_keeps_force_error(gpulib):
    disk = bodies.config_disk("self_gravitating", n=4096)
    s = lib.System(disk, bodies.thresholds())
    ref = s.calc_accel()
    s.set_gravity_mode(T.GRAVITY_MIXED)
    t = s.autotune(reps=2)
    # 3 row limits, then 0 (automatic) and the chunk sizes in tiles of 256 sources: for each
    # chunk count up to 24, the smallest size giving it and one tile less
    tiles = -(-disk.n_total // 256)
    sizes = {k for n in range(1, 25) for k in (-(-tiles // n), -(-tiles // n) - 1) if k >= 1}
    assert t["candidates"] == 3 + 1 + len(sizes)
    assert t["mixed_chunks"] == 0 or t["mixed_chunks"] // 256 in sizes
    assert t["ms_per_eval"] <= t["ms_before"] * 1.001
    am = s.calc_accel()
    a_m = np.stack([am[f] for f in "xyz"], 1)
    a_e = np.stack([ref[f] for f in "xyz"], 1)
    rel = np.linalg.norm(a_m - a_e, axis=1) / np.linalg.norm(a_e, axis=1)
    assert rel.max() < 1e-10
