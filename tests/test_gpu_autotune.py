"""rg_autotune: the chosen launch shape is at least as fast as the one before, FP64 results
stay bit-exact (every candidate sums in the reference's order) and mixed-mode forces stay
within their tolerance."""
import numpy as np
import pytest

import helpers as H
import pyoracle
from redgb import bodies, lib, types as T
from redgb.api import RedError

pytestmark = pytest.mark.gpu


def test_fp64_autotune_keeps_bit_exact_run(gpulib):
    disk, params, result, events = H.load_fixture("disk_si_rkf78_collide")
    s = lib.System(disk, H.thresholds_of(params))
    t = s.autotune(reps=2)
    assert t["candidates"] == 7 + 3  # sinks per pair-parallel CTA, then the row-kernel limit
    assert t["pairpar_sinks"] in (8, 12, 16, 18, 24, 32, 36) and t["rowseq_max_src"] in (32, 64, 128)
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


@pytest.mark.parametrize("S", [8, 12, 16, 18, 24, 32, 36])
def test_every_pair_parallel_shape_is_bit_exact(gpulib, S):
    """Each sink count per pair-parallel CTA the tuner may choose (set with
    rg_set_launch_shape) gives the oracle's accelerations bit for bit, on a disk whose last
    sink tile is partial for every S and whose sources span several tiles of each shape."""
    disk = bodies.make_disk(n_pl=1000, pl_type=T.BODY_PROTOPLANET, giants=(), seed=S)
    g = lib.System(disk, bodies.thresholds())
    g.set_launch_shape(pairpar_sinks=S, rowseq_max_src=64)
    ag, ao = g.calc_accel(), pyoracle.OracleSystem(disk, bodies.thresholds()).calc_accel()
    for f in "xyzw":
        assert H.same(ag[f], ao[f]), (S, f)


def test_launch_shape_refusals(gpulib):
    disk = bodies.make_disk(n_pl=100, pl_type=T.BODY_PROTOPLANET, giants=(), seed=1)
    g = lib.System(disk, bodies.thresholds())
    for kw in ({"pairpar_sinks": 20}, {"rowseq_max_src": 0}, {"mixed_chunks": 100}):
        with pytest.raises(RedError):
            g.set_launch_shape(**kw)
    astro = lib.System(disk, bodies.thresholds(), frame=T.FRAME_ASTRO)
    with pytest.raises(RedError):
        astro.set_launch_shape(pairpar_sinks=36)
    astro.set_launch_shape(pairpar_sinks=32)
