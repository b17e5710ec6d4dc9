"""Ensemble (many disks, one GPU): every disk reproduces the FP64 oracle bit for bit when
the oracle replays the trial steps the ensemble's device controller chose (the device pow
may round differently from glibc's, so the step sizes are the only free input)."""
import numpy as np
import pytest

import helpers as H
import pyoracle
from redgb import bodies, types as T
from redgb.ensemble import Ensemble

pytestmark = pytest.mark.gpu


def _replay_check(ens, disks, thr, log, events=None):
    for s, disk in enumerate(disks):
        mine = log[log["sys"] == s]
        assert len(mine) > 0
        st = ens.stats(s)
        assert st["n_tried_step"] == len(mine)
        assert st["n_passed_step"] == int(mine["accepted"].sum())
        o = pyoracle.OracleSystem(disk, thr[s] if np.ndim(thr) == 2 else thr)
        o.set_integrator(T.INT_RKF78, 0.001, True, 1e-10)
        o.set_dt_replay(mine["dt"])
        n_steps = st["n_passed_step"]
        o.advance(1e30, max_steps=n_steps)
        rg, vg, pg, mg, tg = ens.state(s)
        ro, vo, po, mo, to = o.state()
        # inactive bodies stay in the ensemble's storage; the oracle compacts them away
        act = (mg["id"] > 0)
        assert np.array_equal(mg["id"][act], mo["id"][mo["id"] > 0])
        for f in "xyz":
            assert H.same(rg[f][act], ro[f][mo["id"] > 0]), (s, f)
            assert H.same(vg[f][act], vo[f][mo["id"] > 0]), (s, f)
        assert tg == to


@pytest.mark.parametrize("use_graph", [True, False])
def test_ensemble_replay_bit_exact(gpulib, use_graph):
    disks = [bodies.make_disk(n_pl=120 + 60 * k, seed=30 + k, giant_scale=(0.5 + 0.4 * k, 1.0)) for k in range(3)]
    disks.append(bodies.make_disk(n_pl=80, pl_type=T.BODY_PROTOPLANET, seed=40, m_range=(1e-9, 1e-7), giants=()))
    thr = bodies.thresholds(collision_factor=0.0)
    ens = Ensemble(disks, thr)
    ens.set_integrator(0.001, 1e-10)
    ens.set_options(use_graph=use_graph)
    ens.set_step_log(1 << 16)
    ens.advance(40.0)
    log = ens.step_log()
    _replay_check(ens, disks, thr, log)
    for s in range(len(disks)):
        assert ens.stats(s)["status"] == T.SYS_DONE


def test_ensemble_autotune(gpulib):
    """rg_ens_autotune: FP64 shapes keep the bit-exact replay; mixed shapes keep the energy."""
    disks = [bodies.make_disk(n_pl=150 + 90 * k, seed=60 + k) for k in range(3)]
    disks.append(bodies.make_disk(n_pl=200, pl_type=T.BODY_PROTOPLANET, seed=63, m_range=(1e-9, 1e-7), giants=()))
    thr = bodies.thresholds(collision_factor=0.0)
    ens = Ensemble(disks, thr)
    ens.set_integrator(0.001, 1e-10)
    t = ens.autotune(reps=2)
    assert t["candidates"] == 9 and t["pairpar_sinks"] in (8, 16, 32) and t["rowseq_max_src"] in (32, 64, 128)
    assert t["ms_per_eval"] <= t["ms_before"] * 1.001
    ens.set_step_log(1 << 16)
    ens.advance(20.0, max_attempts=4000)  # bounded: a wrong shape would collapse the steps
    _replay_check(ens, disks, thr, ens.step_log())
    mixed = Ensemble(disks, thr)
    mixed.set_integrator(0.001, 1e-10)
    mixed.set_options(gravity_mode=T.GRAVITY_MIXED, hill_factor=3.0)
    t = mixed.autotune(reps=2)
    assert t["candidates"] == 12 and t["mixed_chunks"] in (0, 512, 1024, 2048)
    E0 = [mixed.energy(s)[0] for s in range(len(disks))]
    mixed.advance(60.0, max_attempts=4000)
    for s in range(len(disks)):
        assert abs((mixed.energy(s)[0] - E0[s]) / E0[s]) < 1e-10
        assert mixed.stats(s)["status"] == T.SYS_DONE


def test_ensemble_collisions_match_oracle(gpulib):
    """The reference's collision-merge run as a one-disk ensemble next to a second disk with
    its own (smaller) collision factor: merges, their event records and the resulting states
    match the oracle; the merges are applied on the device inside one graph launch (the host
    handles nothing until the interval ends).  A merged radius is the device's pow of the
    merged volume, so radii are compared to 2 ulp; everything else bit for bit."""
    disk, params, _, ref_events = H.load_fixture("disk_si_rkf78_collide")
    other = bodies.make_disk(n_pl=64, seed=9)
    thr = np.stack([H.thresholds_of(params), bodies.thresholds(collision_factor=1.0)])
    ens = Ensemble([disk, other], thr)
    ens.set_integrator(0.001, 1e-10)
    ens.set_step_log(1 << 18)
    _, g0 = ens.kernel_count()
    n_att = ens.advance(0.5 * T.YEAR)
    _, g1 = ens.kernel_count()
    assert g1 - g0 == (n_att + 4095) // 4096
    log = ens.step_log()
    ev, sysv = ens.events()
    mine = ev[sysv == 0]
    # replay disk 0 in the oracle's full loop (with its merges and compactions)
    o = pyoracle.OracleSystem(disk, thr[0])
    o.set_integrator(T.INT_RKF78, 0.001, True, 1e-10)
    d0 = log[log["sys"] == 0]
    o.set_dt_replay(d0["dt"])
    o.advance(1e30, max_steps=ens.stats(0)["n_passed_step"])
    eo = o.events()
    assert len(mine) == len(eo) and len(eo) > 0
    for a, b in zip(mine, eo):
        assert (a["event_name"], a["id1"], a["id2"]) == (b["event_name"], b["id1"], b["id2"])
        assert H.same(a["t"], b["t"]) and H.same(a["d"], b["d"])
        for f in ("rs", "vs"):
            for c in "xyz":
                assert H.same(a[f][c], b[f][c])
    rg, vg, pg, mg, tg = ens.state(0)
    ro, vo, po, mo, to = o.state()
    act_g, act_o = mg["id"] > 0, mo["id"] > 0
    assert np.array_equal(mg["id"][act_g], mo["id"][act_o])
    for f in "xyz":
        assert H.same(rg[f][act_g], ro[f][act_o])
    assert H.same(pg["mass"][act_g], po["mass"][act_o])
    assert np.allclose(pg["radius"][act_g], po["radius"][act_o], rtol=4.5e-16, atol=0.0)
    assert all(int(e["event_name"]) != T.EVENT_COLLISION for e in ev[sysv == 1])  # R1 + R2: none


def test_ensemble_ejection_and_hit_star_match_oracle(gpulib):
    """The reference's ejection run (16 planetesimals on eccentric orbits, 4 test particles,
    ejection beyond 3.2 AU: 11 ejections in 3 years) and a disk with two planetesimals let
    fall towards the star from rest (hit-star inside 0.3 AU) as one ensemble: the screen of
    each accepted state (taken in FP32 first, in FP64 near a threshold) finds the same bodies
    at the same steps as the oracle's replay of each disk's step sizes, and the records and
    the final states match it bit for bit."""
    disk, params, _, _ = H.load_fixture("disk_eject_hit")
    fall = bodies.make_disk(n_pl=16, seed=12, a_range=(1.0, 3.0))
    for k in (5, 9):
        for f in "xyz":
            fall.v[f][k] = 0.0
    thr = np.stack([H.thresholds_of(params)] * 2)
    ens = Ensemble([disk, fall], thr)
    ens.set_integrator(0.001, 1e-10)
    ens.set_step_log(1 << 18)
    ens.advance(params["length_yr"] * T.YEAR)
    log = ens.step_log()
    ev, sysv = ens.events()
    for s, (d, kind) in enumerate(((disk, T.EVENT_EJECTION), (fall, T.EVENT_HIT_CENTRUM))):
        o = pyoracle.OracleSystem(d, thr[s])
        o.set_integrator(T.INT_RKF78, 0.001, True, 1e-10)
        o.set_dt_replay(log[log["sys"] == s]["dt"])
        o.advance(1e30, max_steps=ens.stats(s)["n_passed_step"])
        eo, mine = o.events(), ev[sysv == s]
        assert kind in {int(e["event_name"]) for e in eo}
        assert len(mine) == len(eo)
        for a, b in zip(mine, eo):
            assert (a["event_name"], a["id1"], a["id2"]) == (b["event_name"], b["id1"], b["id2"])
            assert H.same(a["t"], b["t"]) and H.same(a["d"], b["d"])
        rg, vg, pg, mg, _ = ens.state(s)
        ro, vo, po, mo, _ = o.state()
        act_g, act_o = mg["id"] > 0, mo["id"] > 0
        assert np.array_equal(mg["id"][act_g], mo["id"][act_o])
        for f in "xyz":
            assert H.same(rg[f][act_g], ro[f][act_o]) and H.same(vg[f][act_g], vo[f][act_o])


def test_ensemble_mixed_and_energy(gpulib):
    disks = [bodies.config_disk("ensemble_member", seed=s, n=600) for s in (1, 2, 3)]
    ens = Ensemble(disks, bodies.thresholds(collision_factor=0.0))
    ens.set_integrator(0.001, 1e-10)
    ens.set_options(gravity_mode=T.GRAVITY_MIXED, hill_factor=3.0)
    E0 = [ens.energy(s)[0] for s in range(3)]
    ens.advance(365.25)
    for s in range(3):
        E1 = ens.energy(s)[0]
        assert abs((E1 - E0[s]) / E0[s]) < 1e-10
        assert ens.stats(s)["status"] == T.SYS_DONE
    n_k, n_g = ens.kernel_count()
    assert n_g > 0 and n_k > n_g


def test_ensemble_close_encounter_times(gpulib):
    """A close-encounter record carries the step start at which the pair was found inside the
    Hill sphere (a wide sphere, 10 mutual Hill radii, so that pairs enter it within 60 days)."""
    disks = [bodies.config_disk("ensemble_member", seed=s, n=600) for s in (4, 5)]
    ens = Ensemble(disks, bodies.thresholds(collision_factor=0.0))
    ens.set_integrator(0.001, 1e-10)
    ens.set_options(gravity_mode=T.GRAVITY_MIXED, hill_factor=10.0)
    ens.set_step_log(1 << 18)
    ens.advance(60.0, max_attempts=20000)
    ev, sysv = ens.events()
    log = ens.step_log()
    later = 0
    for s in range(len(disks)):
        mine = log[(log["sys"] == s) & (log["accepted"] == 1)]
        starts = np.concatenate([[0.0], np.cumsum(mine["dt"])])  # internal units
        for r, k in zip(ev, sysv):
            if k == s and r["event_name"] == T.EVENT_CLOSE_ENCOUNTER:
                assert np.min(np.abs(starts - r["t"])) <= 1e-12 * max(1.0, starts[-1]), (s, r["t"])
                later += r["t"] > 0.0
    assert later > 0


def test_ensemble_mixed_screen_cutoffs_keep_every_event(gpulib):
    """Three crowded disks (3000 protoplanets with radii x 300 and a giant; Hill factor 3:
    about 20 overlapping and 50 Hill pairs each at the start).  The mixed kernels skip the
    detailed screens beyond each sink's cutoff from its own disk's largest light-body
    radius, mass and star distance, screen the star and the giant always, and record the
    FP64 ensemble's events.  One step (the first trial step, 0.001 day): the next step sizes
    follow error estimates far below the tolerance, i.e. rounding noise, which differs
    between the two arithmetics."""
    disks = []
    for seed in (51, 52, 53):
        d = bodies.make_disk(n_pl=3000, pl_type=T.BODY_PROTOPLANET, seed=seed, m_range=(1e-9, 1e-7),
                             giants=((9.55e-4, 5.2, 0.05),), a_range=(1.0, 1.3), sigma_e=0.05, sigma_i=0.02)
        d.p["radius"][2:] *= 300.0
        disks.append(d)
    thr = bodies.thresholds(collision_factor=1.0)
    out = {}
    for mode in (T.GRAVITY_FP64, T.GRAVITY_MIXED):
        ens = Ensemble(disks, thr)
        ens.set_integrator(0.001, 1e-10)
        ens.set_options(gravity_mode=mode, hill_factor=3.0)
        ens.advance(0.0005)  # runs while t <= t_stop: one step of the first trial size
        ev, sysv = ens.events()
        out[mode] = [(int(s), int(e["event_name"]), int(e["id1"]), int(e["id2"])) for e, s in zip(ev, sysv)]
        assert all(ens.stats(s)["n_tried_step"] == 1 for s in range(len(disks)))
    assert len(out[T.GRAVITY_FP64]) > 60 and len({k for _, k, _, _ in out[T.GRAVITY_FP64]}) >= 2
    assert out[T.GRAVITY_MIXED] == out[T.GRAVITY_FP64]


def test_ensemble_heavy_light_events_match_fp64(gpulib):
    """Disks of star, giants and planetesimals (the symmetric heavy-light kernel's plans: each
    heavy-light pair screened once, in the planetesimal's row), with planetesimals placed
    inside the giants' Hill spheres and two overlapping a giant: over one step the mixed
    ensemble records the FP64 ensemble's close-encounter and collision records, pair for
    pair."""
    disks = []
    for seed in (4, 5):
        d = bodies.config_disk("ensemble_member", seed=seed, n=600)
        offsets = [(0.05 * k, 0.03, 0.01) for k in range(1, 9)] + [(3e-4, 0.0, 0.0), (0.0, -2e-4, 1e-4)]
        for k, off in enumerate(offsets):
            g = 1 + k % 2
            for f, c in zip("xyz", off):
                d.r[f][3 + k] = d.r[f][g] + c
        disks.append(d)
    thr = bodies.thresholds(collision_factor=1.0)
    out = {}
    for mode in (T.GRAVITY_FP64, T.GRAVITY_MIXED):
        ens = Ensemble(disks, thr)
        ens.set_integrator(0.001, 1e-10)
        ens.set_options(gravity_mode=mode, hill_factor=3.0)
        ens.advance(0.0005)  # runs while t <= t_stop: one step of the first trial size
        ev, sysv = ens.events()
        out[mode] = [(int(s), int(e["event_name"]), int(e["id1"]), int(e["id2"])) for e, s in zip(ev, sysv)]
    kinds = {k for _, k, _, _ in out[T.GRAVITY_FP64]}
    assert {T.EVENT_CLOSE_ENCOUNTER, T.EVENT_COLLISION} <= kinds, out[T.GRAVITY_FP64]
    assert out[T.GRAVITY_MIXED] == out[T.GRAVITY_FP64]


def test_proposer_fallback_keeps_the_run_correct(gpulib):
    """A proposer that always asks for the largest step it may (twice the plain controller's):
    the embedded error estimate rejects its proposals, each disk falls back to the plain
    controller after two rejections in a row, and the run still ends with |dE/E| < 1e-10."""
    from redgb.proposer import N_IN, N_PARAM, Proposer
    disks = [bodies.config_disk("ensemble_member", seed=s, n=600) for s in (7, 8)]
    ens = Ensemble(disks, bodies.thresholds(collision_factor=0.0))
    ens.set_integrator(0.001, 1e-10)
    ens.set_options(gravity_mode=T.GRAVITY_MIXED, hill_factor=0.0)
    net = Proposer(seed=1)
    w = np.zeros(N_PARAM, np.float32)
    w[-1] = 5.0  # the output bias: log(proposed / ideal step) = 5 for every input
    net.set_params(w)
    net.set_normalisation(np.zeros(N_IN), np.ones(N_IN))
    net.attach(ens, safety=1.0, cooldown=16)
    E0 = [ens.energy(s)[0] for s in range(len(disks))]
    ens.advance(120.0, max_attempts=20000)
    st = [ens.stats(s) for s in range(len(disks))]
    assert all(x["status"] == T.SYS_DONE for x in st)
    assert sum(x["n_fallback"] for x in st) > 0
    assert sum(x["n_proposed"] for x in st) > sum(x["n_proposal_accepted"] for x in st)
    for s in range(len(disks)):
        assert abs((ens.energy(s)[0] - E0[s]) / E0[s]) < 1e-10


@pytest.mark.parametrize("mode", [T.GRAVITY_FP64, T.GRAVITY_MIXED])
def test_graph_replay_equals_direct_launches(gpulib, mode):
    """One attempt of every running disk is captured once as a CUDA graph and replayed; the
    graph freezes the kernels' arguments (row stride, tile lists, control-array pointers,
    thresholds).  The configuration in which an earlier, discarded form of the stage
    combination faulted only inside the graph -- Hill-sphere detection on, with merges
    changing masses, radii and ids between replays -- must give bit for bit the same states,
    event records, step counts and energies as the same attempts launched directly."""
    coll, params, _, _ = H.load_fixture("disk_si_rkf78_collide")
    disks = [coll, bodies.config_disk("ensemble_member", seed=11, n=700),
             bodies.make_disk(n_pl=90, pl_type=T.BODY_PROTOPLANET, seed=12, m_range=(1e-9, 1e-7), giants=())]
    thr = np.stack([H.thresholds_of(params), bodies.thresholds(collision_factor=1.0),
                    bodies.thresholds(collision_factor=1.0)])
    runs = []
    for use_graph in (True, False):
        ens = Ensemble(disks, thr)
        ens.set_integrator(0.001, 1e-10)
        ens.set_options(gravity_mode=mode, hill_factor=3.0, use_graph=use_graph)
        ens.advance(0.25 * T.YEAR)
        ev, sysv = ens.events()
        states = [ens.state(s) for s in range(len(disks))]
        stats = [ens.stats(s) for s in range(len(disks))]
        energy = [ens.energy(s) for s in range(len(disks))]
        _, n_graph = ens.kernel_count()
        runs.append((ev, sysv, states, stats, energy, n_graph))
        ens.close()
    (ev_g, sys_g, st_g, stat_g, en_g, ng_g), (ev_d, sys_d, st_d, stat_d, en_d, ng_d) = runs
    assert ng_g > 0 and ng_d == 0
    assert sum(e["event_name"] == T.EVENT_COLLISION for e in ev_g) >= 5
    assert np.array_equal(sys_g, sys_d) and ev_g.tobytes() == ev_d.tobytes()
    for a, b in zip(st_g, st_d):
        for x, y in zip(a[:4], b[:4]):
            assert x.tobytes() == y.tobytes()
        assert a[4] == b[4]
    for a, b in zip(stat_g, stat_d):
        assert (a["n_tried_step"], a["n_passed_step"], a["t_day"]) == (b["n_tried_step"], b["n_passed_step"], b["t_day"])
    for (ea, la), (eb, lb) in zip(en_g, en_d):
        assert ea == eb and np.array_equal(la, lb)


def test_mode_switch_keeps_the_first_stage_vector(gpulib):
    """The mixed form keeps its stage vectors as double-float pairs and the FP64 form as FP64;
    the first stage vector outlives a rejected attempt, so a change of gravity mode converts it
    in place.  Dithered trial steps make rejections, and the mode changes between advances of
    a few attempts each: the run stays finite and conserves energy as an unswitched one does."""
    from redgb.proposer import set_dither
    disks = [bodies.config_disk("ensemble_member", seed=s, n=600) for s in (1, 2)]
    thr = bodies.thresholds(collision_factor=0.0)
    ens = Ensemble(disks, thr)
    ens.set_integrator(0.001, 1e-10)
    set_dither(ens, 0.3, seed=11)
    E0 = [ens.energy(s)[0] for s in range(2)]
    for k, mode in enumerate([T.GRAVITY_MIXED, T.GRAVITY_FP64] * 6):
        ens.set_options(gravity_mode=mode, hill_factor=3.0)
        ens.advance(1e9, max_attempts=7 + k)
    failed = sum(ens.stats(s)["n_failed_step"] for s in range(2))
    assert failed > 0  # some switches came after a rejected attempt
    for s in range(2):
        E1 = ens.energy(s)[0]
        assert np.isfinite(E1) and abs((E1 - E0[s]) / E0[s]) < 1e-10
        assert ens.stats(s)["status"] == T.SYS_RUNNING


def test_mixed_heavy_light_pairs_match_fp64(gpulib):
    """The mixed form evaluates each (heavy, light) pair once for both rows: the planetesimal's
    row term and the star's or giant's row term come from one displacement and one y^3, and
    the heavy rows add one part per tile of up to 2048 light bodies after the heavy-heavy part.
    Over one accepted 0.01-day step (one attempt) from rest -- so that the velocity after the
    step is the velocity change itself, to full precision -- every body's agrees with the FP64
    form's to the mixed force tolerance, and the star's and the giants' to 1e-11, on disks of
    one light tile and of several (5000 and 2049 planetesimals: tiles are balanced over the
    ensemble, so their sizes differ)."""
    disks = [bodies.config_disk("ensemble_member", seed=s, n=n) for s, n in ((1, 600), (2, 5000), (3, 2049))]
    for d in disks:
        for f in "xyz":
            d.v[f][:] = 0.0
    thr = bodies.thresholds(collision_factor=0.0)
    dv, t_end = {}, {}
    for mode in (T.GRAVITY_FP64, T.GRAVITY_MIXED):
        ens = Ensemble(disks, thr)
        ens.set_integrator(0.01, 1e-10)
        ens.set_options(gravity_mode=mode)
        v0 = [ens.state(s)[1] for s in range(len(disks))]
        ens.advance(1.0, max_attempts=1)
        out = []
        for s in range(len(disks)):
            assert ens.stats(s)["n_passed_step"] == 1
            _, v1, _, _, t = ens.state(s)
            out.append(np.stack([v1[f] - v0[s][f] for f in "xyz"], 1))
            t_end[mode, s] = t
        dv[mode] = out
        ens.close()
    for s, d in enumerate(disks):
        assert t_end[T.GRAVITY_MIXED, s] == t_end[T.GRAVITY_FP64, s]
        a_e, a_m = dv[T.GRAVITY_FP64][s], dv[T.GRAVITY_MIXED][s]
        rel = np.linalg.norm(a_m - a_e, axis=1) / np.linalg.norm(a_e, axis=1)
        print(f"disk {s} ({d.n_total} bodies): max rel {rel.max():.3e}, heavy rows {rel[:3].max():.3e}")
        assert rel.max() < 1e-10 and rel[:3].max() < 1e-11
