"""CUDA library vs the reference's FP64 path: bit-exact parity through the C ABI.

Every comparison here is exact (NaN == NaN): the FP64 kernels keep the reference's
operation order and build without FMA contraction, so states, accelerations and event
records must equal the oracle's and the reference's own outputs bit for bit.
"""
import numpy as np
import pytest

import helpers as H
import pyoracle
from redgb import bodies, lib, types as T
from redgb.api import RedError

pytestmark = pytest.mark.gpu


def gpu_system(disk, thr, **kw):
    return lib.System(disk, thr, **kw)


@pytest.mark.parametrize("name", H.FIXTURES[1:])
def test_reference_runs_bit_exact(gpulib, name):
    """Whole reference runs: RKF7(8) with merges and compactions, close-encounter
    records with orbital elements, ejection / hit-star, RK4 fixed and adaptive."""
    disk, params, result, events = H.load_fixture(name)
    s = gpu_system(disk, H.thresholds_of(params), frame=H.frame_of(params))
    snaps, evs, _ = H.run_fixture(s, params)
    assert H.compare_result(H.snapshots_as_result(snaps), result) == []
    assert H.compare_events(evs, events) == []


def test_twobody_golden(gpulib):
    disk, params, result, _ = H.load_fixture("twobody_euler")
    s = gpu_system(disk, H.thresholds_of(params))
    snaps, _, n = H.run_fixture(s, params, max_steps=36526)
    rows = H.snapshots_as_result(snaps)
    for row, ref in zip(rows[:4], result[:4]):
        assert H.same(row[9], ref["r"])


def _pair(disk, thr, setup):
    g = gpu_system(disk, thr)
    o = pyoracle.OracleSystem(disk, thr)
    for s in (g, o):
        setup(s)
    return g, o


def _assert_same_state(g, o):
    rg, vg, pg, mg, tg = g.state(internal=True)
    ro, vo, po, mo, to = o.state(internal=True)
    assert tg == to
    for f in "xyz":
        assert H.same(rg[f], ro[f]), f
        assert H.same(vg[f], vo[f]), f
    assert np.array_equal(mg["id"], mo["id"])
    for f in ("mass", "radius", "density"):
        assert H.same(pg[f], po[f])


DISKS = {
    "nsi": lambda: bodies.make_disk(n_pl=300, seed=21),
    "si": lambda: bodies.make_disk(n_pl=200, pl_type=T.BODY_PROTOPLANET, seed=22, m_range=(1e-8, 1e-6)),
    "mixed_types": lambda: bodies.make_disk(n_pl=150, seed=23, n_tp=40, embryos=((1e-6, 1.5, 0.05), (2e-6, 2.2, 0.02))),
}
INTEGRATORS = [(T.INT_EULER, False, 0.5), (T.INT_RK4, False, 2.0), (T.INT_RK4, True, 2.0), (T.INT_RK5, False, 2.0),
               (T.INT_RK5, True, 2.0), (T.INT_RKF78, False, 4.0), (T.INT_RKF78, True, 4.0)]


@pytest.mark.parametrize("kind", sorted(DISKS))
@pytest.mark.parametrize("int_type,adaptive,dt", INTEGRATORS)
def test_steps_bit_exact(gpulib, kind, int_type, adaptive, dt):
    disk = DISKS[kind]()
    thr = bodies.thresholds(collision_factor=0.0)

    def setup(s):
        s.set_integrator(int_type, dt, adaptive, 1e-12, error_check_for_tp=(kind == "mixed_types"))

    g, o = _pair(disk, thr, setup)
    for _ in range(6):
        assert g.step() == o.step()
        _assert_same_state(g, o)
    assert g.counters()["n_tried_step"] == o.counters()["n_tried_step"]
    assert g.dt() == o.dt()


@pytest.mark.parametrize("n", [2, 3, 33, 1000, 4097])
def test_acceleration_bit_exact(gpulib, n):
    """Both FP64 kernels (pair-parallel for the many-source blocks, row-serial for the
    rest) against the oracle, all-self-interacting and planetesimal disks."""
    for disk in (bodies.make_disk(n_pl=max(n - 1, 0), pl_type=T.BODY_PROTOPLANET, giants=(), seed=n),
                 bodies.make_disk(n_pl=max(n - 3, 0), seed=n, n_tp=5)):
        g = gpu_system(disk, bodies.thresholds())
        o = pyoracle.OracleSystem(disk, bodies.thresholds())
        ag, ao = g.calc_accel(), o.calc_accel()
        for f in "xyzw":
            assert H.same(ag[f], ao[f]), (n, f)


def test_acceleration_full_size_sampled(gpulib):
    """16384 self-gravitating bodies + star (the gravity-throughput workload): 1 088 rows
    against the oracle -- the star, every pair-parallel tile boundary region sampled in 17
    runs of 64 consecutive sinks spread over the whole disk (each row sums all 16 384
    sources), and the last rows."""
    disk = bodies.config_disk("self_gravitating")
    g = gpu_system(disk, bodies.thresholds())
    ag = g.calc_accel()
    r = g.state(internal=True)[0]
    n = disk.n_total
    starts = np.linspace(0, n - 64, 17).astype(int)
    for i0 in starts:
        ao = pyoracle.grav_accel_rows(disk, r, int(i0), int(i0) + 64)
        for f in "xyz":
            assert H.same(ag[f][i0:i0 + 64], ao[f]), (i0, f)


def test_inactive_and_zero_mass_bodies(gpulib):
    disk = bodies.make_disk(n_pl=60, pl_type=T.BODY_PROTOPLANET, seed=5, n_tp=4)
    disk.md["id"][[5, 17, 40]] *= -1
    disk.p["mass"][[7, 8]] = 0.0
    g, o = _pair(disk, bodies.thresholds(), lambda s: s.set_integrator(T.INT_RKF78, 3.0, True, 1e-10))
    for _ in range(3):
        g.step()
        o.step()
    _assert_same_state(g, o)


def test_compaction_matches_oracle(gpulib):
    """pp_disk::remove_inactive_bodies on the device (the state rows gathered by the list of
    kept bodies): the same state, ids and counts as the oracle's host compaction, bit for bit,
    and the same next step.  With n = 0 the rebuild check always compacts."""
    disk = bodies.make_disk(n_pl=200, pl_type=T.BODY_PROTOPLANET, seed=9, n_tp=6)
    disk.md["id"][[3, 50, 51, 150, disk.n_total - 1]] *= -1
    g, o = _pair(disk, bodies.thresholds(), lambda s: s.set_integrator(T.INT_RKF78, 3.0, True, 1e-10))
    assert g.check_for_rebuild_vectors(0) and o.check_for_rebuild_vectors(0)
    (cg, ng), (co, no) = g.n_total(), o.n_total()
    assert ng == no == disk.n_total - 5
    assert [getattr(cg, f) for f, _ in cg._fields_] == [getattr(co, f) for f, _ in co._fields_]
    _assert_same_state(g, o)
    g.step()
    o.step()
    _assert_same_state(g, o)


def test_hill_close_encounters_match_oracle(gpulib):
    disk = bodies.make_disk(n_pl=120, pl_type=T.BODY_PROTOPLANET, seed=5, m_range=(1e-7, 1e-5),
                            giants=((9.55e-4, 5.2, 0.05),), a_range=(1.0, 1.3), sigma_e=0.05, sigma_i=0.02)
    thr = bodies.thresholds(collision_factor=1.0)

    def setup(s):
        s.set_integrator(T.INT_RKF78, 0.001, True, 1e-10)
        s.set_event_options(hill_factor=3.0)

    g, o = _pair(disk, thr, setup)
    g.advance(120.0)
    o.advance(120.0)
    eg, eo = g.events(), o.events()
    assert len(eo) > 0
    assert [H.event_key(e) for e in eg] == [H.event_key(e) for e in eo]
    assert H.same(eg["d"], eo["d"]) and H.same(eg["t"], eo["t"])
    _assert_same_state(g, o)


def test_planetesimal_disk_1000yr_hill_events(gpulib, planetesimal_disk_1000yr_oracle):
    """The plain FP64 planetesimal-disk workload (star, two giants, 1024 planetesimals, seed
    0) over its full 1000 years through rg_advance (main.cu:176-263), with close encounters
    logged at 3 mutual Hill radii as the workload asks: the GPU's event list (every field of
    every record), step count and final state equal the oracle's bit for bit.  The same
    disk's snapshots against the reference's own run are test_reference_runs_bit_exact."""
    disk, thr, params, n_o, eo, o = planetesimal_disk_1000yr_oracle
    g = gpu_system(disk, thr)
    g.set_integrator(T.INT_RKF78, 0.001, True, params["tolerance"])
    g.set_event_options(hill_factor=3.0)
    assert g.advance(params["length_yr"] * T.YEAR) == n_o
    eg = g.events()
    assert len(eo) >= 20
    assert eg.tobytes() == eo.tobytes()
    _assert_same_state(g, o)
    assert g.counters()["n_tried_step"] == o.counters()["n_tried_step"]


def test_astrocentric_frame_refusals(gpulib):
    """The astrocentric frame takes self-interacting systems only: with planetesimals or
    test particles the reference's own CPU path turns NaN at the first step (their blocks
    take the star at the origin as a source, pp_disk.cu:447-454), so the context refuses
    them, as the oracle does; mixed-precision gravity is refused in that frame; the
    astrocentric transform needs the star as body 0."""
    thr = bodies.thresholds()
    for disk in (bodies.make_disk(n_pl=20, seed=6), bodies.make_disk(n_pl=20, pl_type=T.BODY_PROTOPLANET, seed=6,
                                                                     n_tp=3)):
        with pytest.raises(RedError) as ei:
            gpu_system(disk, thr, frame=T.FRAME_ASTRO)
        assert ei.value.status == -6
        with pytest.raises(RedError) as ei:
            pyoracle.OracleSystem(disk, thr, frame=T.FRAME_ASTRO)
        assert ei.value.status == -6
    si = bodies.make_disk(n_pl=30, pl_type=T.BODY_PROTOPLANET, seed=6, m_range=(1e-8, 1e-6))
    s = gpu_system(si, thr, frame=T.FRAME_ASTRO)
    with pytest.raises(RedError) as ei:
        s.set_gravity_mode(T.GRAVITY_MIXED)
    assert ei.value.status == -6
    bad = si.copy()
    bad.md["body_type"][0] = T.BODY_GIANTPLANET
    bad.r["x"][0] = 0.01  # not at rest in the origin: the transform looks for the star
    with pytest.raises(RedError):
        gpu_system(bad, thr, frame=T.FRAME_ASTRO)


def test_astrocentric_steps_bit_exact(gpulib):
    """Accelerations and RKF7(8) steps in the astrocentric frame against the oracle, state by
    state: the star's starting pull, direct and indirect terms in source order, the star
    pinned at the origin."""
    disk = bodies.make_disk(n_pl=300, pl_type=T.BODY_PROTOPLANET, seed=31, m_range=(1e-9, 1e-6),
                            embryos=((1e-6, 1.5, 0.05),))
    thr = bodies.thresholds(collision_factor=0.0)
    g = gpu_system(disk, thr, frame=T.FRAME_ASTRO)
    o = pyoracle.OracleSystem(disk, thr, frame=T.FRAME_ASTRO)
    ag, ao = g.calc_accel(), o.calc_accel()
    for f in "xyz":
        assert H.same(ag[f], ao[f]), f
    for s in (g, o):
        s.set_integrator(T.INT_RKF78, 1.0, True, 1e-12)
    for _ in range(5):
        assert g.step() == o.step()
        _assert_same_state(g, o)
    r = g.state(internal=True)[0]
    assert r["x"][0] == 0.0 and r["y"][0] == 0.0 and r["z"][0] == 0.0


def test_state_records_in_and_out(gpulib):
    """rg_set_state / rg_get_state: vec_t records in file units, converted on the device
    (v / k in, v * k out: the reference's load and print transforms, one IEEE operation
    each); pinned host buffers through out= give the same records as fresh arrays."""
    import torch
    disk = bodies.make_disk(n_pl=300, seed=12)
    s = gpu_system(disk, bodies.thresholds())
    r, v = s.state()[:2]
    rng = np.random.RandomState(4)
    for f in "xyz":
        r[f] *= 1.0 + 1e-3 * rng.standard_normal(len(r))
        v[f] *= 1.0 + 1e-3 * rng.standard_normal(len(v))
    s.set_state(r, v)
    ri, vi = s.state(internal=True)[:2]
    for f in "xyz":
        assert H.same(ri[f], r[f])
        assert H.same(vi[f], v[f] / T.GAUSS)
    rf, vf, p, md, _ = s.state()
    for f in "xyz":
        assert H.same(vf[f], vi[f] * T.GAUSS)
    assert np.all(rf["w"] == 0.0) and np.all(vf["w"] == 0.0)
    n = len(r)
    pin = [torch.empty(4 * n, dtype=torch.float64, pin_memory=True).numpy().view(T.VEC) for _ in range(2)]
    r2, v2, p2, md2, _ = s.state(out=pin, params=False)
    assert p2 is None and md2 is None and r2 is pin[0]
    assert r2.tobytes() == rf.tobytes() and v2.tobytes() == vf.tobytes()
    with pytest.raises(ValueError):
        s.state(out=(np.zeros(n - 1, T.VEC), np.zeros(n, T.VEC)))


def test_nan_in_the_state_is_reported(gpulib):
    """A NaN position: the first step spreads it exactly as the oracle does (states equal, NaN
    for NaN); the controller's next step is then infinite, which rg_step (like the
    reference's integrator) returns and rg_advance's main loop reports as
    RG_ERR_DT_NONFINITE."""
    disk = bodies.make_disk(n_pl=40, pl_type=T.BODY_PROTOPLANET, seed=8, n_tp=3)
    g, o = _pair(disk, bodies.thresholds(), lambda s: s.set_integrator(T.INT_RKF78, 0.01, False))
    for s in (g, o):
        r, v = s.state()[:2]
        r["x"][7] = np.nan
        s.set_state(r, v)
    g.step()
    o.step()
    _assert_same_state(g, o)
    g.set_integrator(T.INT_RKF78, 0.01, True, 1e-10)
    with pytest.raises(RedError) as ei:
        g.advance(1.0e9, max_steps=3)
    assert ei.value.status == -4


def test_energy_matches_oracle(gpulib):
    disk = bodies.make_disk(n_pl=500, seed=3, n_tp=10, embryos=((1e-6, 1.5, 0.0),))
    g = gpu_system(disk, bodies.thresholds())
    o = pyoracle.OracleSystem(disk, bodies.thresholds())
    (eg, lg), (eo, lo) = g.energy(), o.energy()
    assert abs(eg - eo) <= 1e-14 * abs(eo)
    assert np.allclose(lg, lo, rtol=1e-13, atol=0)


def test_event_overflow_is_reported(gpulib):
    disk, params, _, _ = H.load_fixture("disk_si_rkf78_collide")
    thr = H.thresholds_of(params)
    thr[T.THRESHOLD_RADII_ENHANCE_FACTOR] = 5000.0
    s = gpu_system(disk, thr, event_capacity=4)
    s.set_integrator(T.INT_RKF78, 0.001, True, 1e-10)
    with pytest.raises(RedError) as ei:
        for _ in range(20):
            s.step()
    assert ei.value.status == -3


def test_bad_arguments_are_rejected(gpulib):
    disk = bodies.make_disk(n_pl=4, seed=1)
    s = gpu_system(disk, bodies.thresholds())
    with pytest.raises(RedError) as ei:
        s.step()  # no integrator yet
    assert ei.value.status == -5
    with pytest.raises(RedError):
        s.set_integrator(99, 1.0)
    with pytest.raises(RedError):
        s.set_event_options(hill_factor=-1.0)
