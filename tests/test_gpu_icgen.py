"""rg_generate_disks against its numpy restatement (oracle/icgen_ref.py): the same random
streams (body order, types and counts exact; masses to the last bits of exp), positions and
velocities to the rounding of the transcendental functions; a disk does not depend on the
other disks generated with it; generated disks integrate as an ensemble."""
import numpy as np
import pytest

import icgen_ref as ref
from redgb import bodies, types as T
from redgb.ensemble import Ensemble
from redgb.icgen import DiskSpec, generate_disks, spec_like

pytestmark = pytest.mark.gpu


def _check(disk, spec):
    r, v, m, R, rho, typ = ref.generate(spec)
    assert disk.n_total == spec.n_total
    assert np.array_equal(disk.md["body_type"], typ)
    assert np.array_equal(disk.md["id"], np.arange(1, spec.n_total + 1))
    assert np.allclose(disk.p["mass"], m, rtol=1e-14, atol=0)
    assert np.allclose(disk.p["radius"], R, rtol=1e-14, atol=0)
    assert np.allclose(disk.p["density"], rho, rtol=1e-15, atol=0)
    rg = np.stack([disk.r[f] for f in "xyz"], 1)
    vg = np.stack([disk.v[f] for f in "xyz"], 1)
    assert np.all(np.linalg.norm(rg - r, axis=1) <= 1e-11 * np.maximum(np.linalg.norm(r, axis=1), 1e-300))
    assert np.all(np.linalg.norm(vg - v, axis=1) <= 1e-11 * np.maximum(np.linalg.norm(v, axis=1), 1e-300))
    assert np.all(disk.r["w"] == 0.0) and np.all(disk.v["w"] == 0.0)


def test_generator_matches_restatement(gpulib):
    specs = [spec_like("planetesimal_disk", seed=4, n=3000),
             DiskSpec(seed=9, n_pl=700, pl_type=T.BODY_PROTOPLANET, n_tp=50, giants=((1e-3, 5.0, 0.1),),
                      m_range=(1e-9, 1e-7)),
             spec_like("dense_ring", seed=2, n=5000),
             DiskSpec(seed=11, n_pl=0, giants=())]
    disks = generate_disks(specs)
    for d, s in zip(disks, specs):
        _check(d, s)
    counts = disks[1].counts
    assert counts[0] == 1 and counts[1] == 1 and counts[3] == 700 and counts[6] == 50


def test_disks_do_not_depend_on_their_batch(gpulib):
    a = DiskSpec(seed=21, n_pl=513)
    alone = generate_disks([a])[0]
    batch = generate_disks([DiskSpec(seed=5, n_pl=300), a, DiskSpec(seed=6, n_pl=1000, n_tp=7)])[1]
    for f in ("r", "v", "p", "md"):
        assert getattr(alone, f).tobytes() == getattr(batch, f).tobytes()


def test_generated_ensemble_integrates(gpulib):
    disks = generate_disks([spec_like("ensemble_member", seed=s, n=500) for s in (70, 71, 72)])
    ens = Ensemble(disks, bodies.thresholds(collision_factor=0.0))
    ens.set_integrator(0.001, 1e-10)
    ens.set_options(gravity_mode=T.GRAVITY_MIXED, hill_factor=3.0)
    E0 = [ens.energy(s)[0] for s in range(3)]
    ens.advance(30.0, max_attempts=10000)
    for s in range(3):
        assert ens.stats(s)["status"] == T.SYS_DONE
        assert abs((ens.energy(s)[0] - E0[s]) / E0[s]) < 1e-10


def test_invalid_spec_is_refused(gpulib):
    from redgb.api import RedError
    with pytest.raises(RedError) as ei:
        generate_disks([DiskSpec(seed=1, n_pl=10, pl_type=T.BODY_TESTPARTICLE)])
    assert ei.value.status == -1


# ------------------------------------------------------------------ rg_populate_disks
from redgb import icgen as I  # noqa: E402


def _mixed_disk(seed):
    """Every distribution kind on some body type: a star (mass and radius given), giants on
    uniform elements, protoplanets with power-law a, lognormal masses, Rayleigh e, and
    planetesimals with exponential e, normal i, log-uniform masses (radius and density given
    for them: the mass is derived), test particles with elements only."""
    n_body = (1, 3, 0, 400, 0, 300, 60)
    two_pi = 2.0 * np.pi
    angles = {I.OE_PERI: I.uniform(0.0, two_pi), I.OE_NODE: I.uniform(0.0, two_pi), I.OE_MEAN: I.uniform(0.0, two_pi)}
    return I.BodyDisk(
        seed=seed, n_body=n_body, to_bc=True, pp_total_mass=3.0e-5,
        pp={T.BODY_STAR: {I.PP_MASS: I.uniform(1.0, 1.0), I.PP_RADIUS: I.uniform(I.SOLAR_RADIUS_AU, I.SOLAR_RADIUS_AU)},
            T.BODY_GIANTPLANET: {I.PP_MASS: I.uniform(3e-4, 1e-3), I.PP_DENSITY: I.uniform(1.0 * I.GRAM_PER_CM3,
                                                                                          2.0 * I.GRAM_PER_CM3)},
            T.BODY_PROTOPLANET: {I.PP_MASS: I.lognormal(0.1, 3.0, 0.0, 0.25),
                                 I.PP_DENSITY: I.uniform(2.7 * I.GRAM_PER_CM3, 2.7 * I.GRAM_PER_CM3)},
            T.BODY_PLANETESIMAL: {I.PP_RADIUS: I.log_uniform(1e-9, 1e-8), I.PP_DENSITY: I.uniform(1e6, 3e6),
                                  I.PP_DRAG_COEFF: I.uniform(1.0, 2.7)},
            T.BODY_TESTPARTICLE: {I.PP_MASS: I.uniform(0.0, 0.0), I.PP_RADIUS: I.uniform(0.0, 0.0)}},
        oe={T.BODY_GIANTPLANET: {I.OE_SMA: I.uniform(5.0, 10.0), I.OE_ECC: I.uniform(0.0, 0.1),
                                 I.OE_INC: I.uniform(0.0, 0.1), **angles},
            T.BODY_PROTOPLANET: {I.OE_SMA: I.power_law(0.9, 2.7, -1.5), I.OE_ECC: I.rayleigh(0.01), **angles},
            T.BODY_PLANETESIMAL: {I.OE_SMA: I.power_law(1.0, 4.0, -0.5), I.OE_ECC: I.exponential(100.0),
                                  I.OE_INC: I.normal(0.0, 0.01), **angles},
            T.BODY_TESTPARTICLE: {I.OE_SMA: I.uniform(1.0, 4.0), I.OE_ECC: I.uniform(0.0, 0.05), **angles}})


def _check_populated(disk, spec):
    r, v, m, R, rho, cd, typ = ref.populate(spec)
    assert disk.n_total == spec.n_total
    assert np.array_equal(disk.md["body_type"], typ)
    assert np.array_equal(disk.md["id"], np.arange(1, spec.n_total + 1))
    for got, want in ((disk.p["mass"], m), (disk.p["radius"], R), (disk.p["density"], rho), (disk.p["cd"], cd)):
        assert np.allclose(got, want, rtol=1e-12, atol=0)
    rg = np.stack([disk.r[f] for f in "xyz"], 1)
    vg = np.stack([disk.v[f] for f in "xyz"], 1)
    rs, vs = np.abs(r).max(), np.abs(v).max()
    assert np.abs(rg - r).max() <= 1e-11 * rs and np.abs(vg - v).max() <= 1e-11 * vs


def test_populate_matches_restatement(gpulib):
    specs = [_mixed_disk(31), I.dvorak_disk(seed=8, n_pp=2000)]
    disks = I.populate_disks(specs)
    for d, s in zip(disks, specs):
        _check_populated(d, s)
    dv = disks[1]
    m = dv.p["mass"]
    assert abs(m[1:].sum() - specs[1].pp_total_mass) < 1e-15  # scaled to the nebula's solids
    rv = np.stack([dv.r[f] for f in "xyz"], 1)
    assert np.abs((m[:, None] * rv).sum(0)).max() < 1e-15  # at its barycentre


def test_populated_disks_do_not_depend_on_their_batch(gpulib):
    a = _mixed_disk(40)
    alone = I.populate_disks([a])[0]
    batch = I.populate_disks([I.dvorak_disk(seed=1, n_pp=100), a, _mixed_disk(41)])[1]
    for f in ("r", "v", "p", "md"):
        assert getattr(alone, f).tobytes() == getattr(batch, f).tobytes()


def test_dvorak_disk_integrates(gpulib):
    """The reference's Dvorak disk, drawn on the GPU, through the FP64 integrator."""
    disk = I.populate_disks([I.dvorak_disk(seed=12, n_pp=500)])[0]
    from redgb import lib
    s = lib.System(disk, bodies.thresholds(collision_factor=0.0))
    s.set_integrator(T.INT_RKF78, tolerance=1e-10)
    E0, _ = s.energy()
    s.advance(20.0)
    E1, _ = s.energy()
    assert abs((E1 - E0) / E0) < 1e-10


def test_populate_refusals(gpulib):
    from redgb.api import RedError
    bad = _mixed_disk(1)
    bad.pp[T.BODY_PROTOPLANET] = {I.PP_MASS: I.uniform(1e-8, 1e-7)}  # radius and density both missing
    with pytest.raises(RedError) as ei:
        I.populate_disks([bad])
    assert ei.value.status == -1 and "missing physical parameters" in str(ei.value)
    bad = _mixed_disk(1)
    bad.oe[T.BODY_PROTOPLANET][I.OE_SMA] = I.power_law(0.0, 2.7, -1.5)  # x_min must be positive
    with pytest.raises(RedError):
        I.populate_disks([bad])


def test_initial_command_line_writes_body_files(gpulib, tmp_path):
    """python -m redgb.initial: two of the reference's n_pl disks drawn on the GPU, written as
    body files that read back as the restatement's disks and load into a context."""
    from redgb import initial, lib
    assert initial.main(["n_pl", "--n", "50", "--seed", "7", "--count", "2", "-o", str(tmp_path / "disk")]) == 0
    for k, seed in ((1, 7), (2, 8)):
        disk = bodies.read_body_file(tmp_path / f"disk_{k}.txt")
        r, v, m, R, rho, cd, typ = ref.populate(I.reference_preset("n_pl", seed, 50))
        assert disk.counts == (1, 0, 0, 0, 0, 50, 0) and np.array_equal(disk.md["body_type"], typ)
        np.testing.assert_allclose(disk.p["mass"], m, rtol=1e-12)
        rg = np.stack([disk.r[f] for f in "xyz"], 1)
        assert np.abs(rg - r).max() <= 1e-11 * np.abs(r).max()
    s = lib.System(bodies.read_body_file(tmp_path / "disk_1.txt"), bodies.thresholds())
    s.set_integrator(T.INT_RKF78, tolerance=1e-10)
    s.advance(10.0)
