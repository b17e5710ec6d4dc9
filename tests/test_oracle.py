"""The oracle (oracle/redoracle.c) against the reference's own test vectors and runs.

Golden fixtures (tests/golden/*.npz) were produced by running the reference's CPU path
(`red -cpu`, built from its sources by oracle/ref.mk) with tests/golden/make_golden.py;
the TwoBody case is the reference's own committed result file.
"""
import ctypes
import math

import numpy as np
import pytest

import helpers as H
import pyoracle
from redgb import bodies, types as T

CPU_FIXTURES = [f for f in H.FIXTURES if f != "twobody_euler"]


@pytest.mark.parametrize("name", CPU_FIXTURES)
def test_oracle_reproduces_reference_run(name):
    disk, params, result, events = H.load_fixture(name)
    s = pyoracle.OracleSystem(disk, H.thresholds_of(params), frame=H.frame_of(params))
    snaps, evs, _ = H.run_fixture(s, params)
    assert H.compare_result(H.snapshots_as_result(snaps), result) == []
    assert H.compare_events(evs, events) == []


def test_oracle_twobody_golden_positions():
    """TestRun/InputTest/Debug/TwoBody: Euler, 2 yr.  The golden file was written by an
    older build that printed time and velocity in internal units: positions must match
    bit for bit, velocities to 2 ulp after the k rescale."""
    disk, params, result, _ = H.load_fixture("twobody_euler")
    s = pyoracle.OracleSystem(disk, H.thresholds_of(params))
    snaps, _, n = H.run_fixture(s, params)
    assert n == 730500
    rows = H.snapshots_as_result(snaps)
    assert len(rows) == len(result)
    for row, ref in zip(rows, result):
        assert H.same(row[9], ref["r"])
        v_int = np.asarray(row[10]) / T.GAUSS
        assert np.allclose(v_int, ref["v"], rtol=3e-16, atol=0)


def test_n1_massive_n3_collision_record():
    """Release/N1_massive_N3_test: test particle 12 sits on protoplanet 2, so the first
    step records COLLISION (2, 12) at t = 0 with d = 1.0235750533041806e-15."""
    disk, params, _, events = H.load_fixture("n1_massive_n3")
    assert events[0]["d"] == 1.0235750533041806e-15
    s = pyoracle.OracleSystem(disk, H.thresholds_of(params))
    H.configure(s, params)
    s.check_for_ejection_hit_centrum()
    s.step()
    assert s.check_for_collision() == 1
    ev = s.events()
    assert (ev[0]["event_name"], ev[0]["id1"], ev[0]["id2"]) == (T.EVENT_COLLISION, 2, 12)
    assert ev[0]["d"] == 1.0235750533041806e-15 and ev[0]["t"] == 0.0


def test_red_test_kats():
    """Known-answer values of red.cuda.utility/red_test.cpp:592-840."""
    L = pyoracle.lib()
    assert abs(L.ro_calculate_radius(1.0, 1.0) - 0.62035049089940001666800681204778) <= 1e-15
    assert abs(L.ro_calculate_mass(1.0, 1.0) - 4.1887902047863909846168578443727) <= 1e-15
    assert abs(L.ro_calculate_density(1.0, 1.0) - 0.23873241463784300365332564505877) <= 1e-15
    r1 = np.array([(1.0, 1.0, 1.0, 0.0)], T.VEC)
    r2 = np.array([(4.0, 3.0, 1.0, 0.0)], T.VEC)
    out = np.zeros(1, T.VEC)
    L.ro_calc_position_after_collision(1.0, 1.0, T.ptr(r1), T.ptr(r2), T.ptr(out))
    assert tuple(out[0]) == (2.5, 2.0, 1.0, 0.0)
    v1 = np.array([(1.0, 0.0, 0.0, 0.0)], T.VEC)
    v2 = np.array([(-1.0, 0.0, 0.0, 0.0)], T.VEC)
    L.ro_calc_velocity_after_collision(1.0, 1.0, T.ptr(v1), T.ptr(v2), T.ptr(out))
    assert tuple(out[0])[:3] == (0.0, 0.0, 0.0)
    v1[0] = (-1.0, 0.0, 0.0, 0.0)
    v2[0] = (-1.0, 0.0, 0.0, 0.0)
    L.ro_calc_velocity_after_collision(1.0, 1.0, T.ptr(v1), T.ptr(v2), T.ptr(out))
    assert tuple(out[0])[:3] == (-1.0, 0.0, 0.0)
    p1 = np.array([(1.0, 1.0, 1.0, 1.0)], T.PARAM)
    p2 = np.array([(1.0, 1.0, 1.0, 1.0)], T.PARAM)
    p = np.zeros(1, T.PARAM)
    L.ro_calc_physical_properties(T.ptr(p1), T.ptr(p2), T.ptr(p))
    assert p[0]["mass"] == 2.0 and p[0]["cd"] == 1.0
    assert abs(p[0]["density"] - 0.23873241463784300365332564505877) <= 1e-15
    assert abs(p[0]["radius"] - L.ro_calculate_radius(2.0, 0.23873241463784300365332564505877)) <= 1e-15
    E = ctypes.c_double()
    d2r = 1.745329251994329509e-2
    L.ro_kepler_equation_solver(0.5, 27.0 * d2r, 1e-15, ctypes.byref(E))
    assert abs(48.43417991487915 - E.value * (1.0 / d2r)) <= 1e-13
    L.ro_kepler_equation_solver(0.5, 225.0 * d2r, 1e-15, ctypes.byref(E))
    assert abs(210.47211284530107 - E.value * (1.0 / d2r)) <= 1e-13


def test_barycentre_transform():
    """red_test.cpp's 4-body barycentre fixture: after the transform the mass-weighted
    position and velocity vanish."""
    n = 4
    p = np.zeros(n, T.PARAM)
    p["mass"] = [1.0, 1e-3, 2e-3, 1e-5]
    r = np.zeros(n, T.VEC)
    v = np.zeros(n, T.VEC)
    r["x"] = [0.0, 1.0, -2.0, 3.5]
    r["y"] = [0.0, 0.5, 1.0, -1.0]
    v["y"] = [0.0, 1.0, -0.7, 0.5]
    pyoracle.lib().ro_transform_to_bc(n, T.ptr(p), T.ptr(r), T.ptr(v))
    for f in "xyz":
        assert abs(np.sum(p["mass"] * r[f])) < 1e-15
        assert abs(np.sum(p["mass"] * v[f])) < 1e-15


def test_body_file_round_trip(tmp_path):
    d = bodies.make_disk(n_pl=20, seed=1, n_tp=3)
    path = tmp_path / "b.txt"
    bodies.write_body_file(str(path), d)
    e = bodies.read_body_file(str(path))
    assert e.counts == d.counts
    for f in ("r", "v", "p", "md"):
        assert np.array_equal(getattr(e, f), getattr(d, f))


def test_synthetic_disk_shapes():
    d = bodies.config_disk("planetesimal_disk")
    assert d.counts == (1, 2, 0, 0, 0, 1024, 0)
    a = np.hypot(d.r["x"][3:], d.r["y"][3:])
    assert 0.9 < a.min() and a.max() < 4.5
    m = d.p["mass"][3:]
    assert m.min() >= 1e-10 and m.max() <= 1e-8
    g = bodies.config_disk("self_gravitating", n=512)
    assert g.counts == (1, 0, 0, 512, 0, 0, 0)
    ring = bodies.config_disk("dense_ring", n=256)
    assert ring.counts == (1, 0, 0, 257, 0, 0, 0)
    assert d.pairs_per_eval() == 3 * 1026 + 1024 * 3


def test_oracle_energy_matches_direct_sum():
    d = bodies.make_disk(n_pl=30, pl_type=T.BODY_PROTOPLANET, seed=2)
    s = pyoracle.OracleSystem(d, bodies.thresholds())
    E, L = s.energy()
    r, v, p, md, _ = s.state(internal=True)
    m = p["mass"]
    T_kin = 0.5 * np.sum(m * (v["x"] ** 2 + v["y"] ** 2 + v["z"] ** 2))
    U = 0.0
    for i in range(len(m)):
        for j in range(i):
            U -= m[i] * m[j] / math.sqrt((r["x"][i] - r["x"][j]) ** 2 + (r["y"][i] - r["y"][j]) ** 2
                                        + (r["z"][i] - r["z"][j]) ** 2)
    assert abs(E - (T_kin + U)) <= 1e-14 * abs(E)


@pytest.mark.parametrize("int_type,order,dts", [(T.INT_RK4, 4, (4.0, 2.0)), (T.INT_RK5, 4, (8.0, 4.0)),
                                               (T.INT_RKF78, 7, (16.0, 8.0))])
def test_oracle_convergence_order(int_type, order, dts):
    """Fixed-step global error of an eccentric orbit scales as dt^order (RKF5 propagates
    its fourth-order weights, as int_rungekutta5.cu:60-77 does)."""
    d = bodies.make_disk(n_pl=0, giants=((1e-3, 1.0, 0.2),), seed=4)
    span = 256.0
    s = pyoracle.OracleSystem(d, np.zeros(5))
    s.set_integrator(T.INT_RKF78, 1.0, False, 1e-10)
    for _ in range(int(span)):
        s.step()
    ref = s.state()[0]
    e = []
    for dt in dts:
        s = pyoracle.OracleSystem(d, np.zeros(5))
        s.set_integrator(int_type, dt, False, 1e-10)
        for _ in range(int(round(span / dt))):
            s.step()
        r = s.state()[0]
        e.append(max(abs(r["x"] - ref["x"]).max(), abs(r["y"] - ref["y"]).max()))
    rate = math.log2(e[0] / e[1])
    assert rate > order - 0.7, (e, rate)
