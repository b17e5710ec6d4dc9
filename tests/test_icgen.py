"""The disk generator's numpy restatement (oracle/icgen_ref.py, the checker of the GPU
generator): determinism, independence of the streams, and the requested distributions."""
import math

import numpy as np
import pytest

import icgen_ref as ref
from redgb.icgen import DiskSpec, spec_like
from redgb import types as T


def test_streams_are_keyed_and_counted():
    a = ref.draw2(7, np.arange(1, 100), 0)
    b = ref.draw2(7, np.arange(1, 100), 0)
    c = ref.draw2(8, np.arange(1, 100), 0)
    d = ref.draw2(7, np.arange(1, 100), 1)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert not np.any(a[0] == c[0]) and not np.any(a[0] == d[0])
    u = np.concatenate(ref.draw2(12345, np.arange(200000), 0))
    assert 0.0 <= u.min() and u.max() < 1.0
    assert abs(u.mean() - 0.5) < 3e-3 and abs(u.var() - 1.0 / 12.0) < 2e-3


def test_disk_follows_the_spec():
    spec = spec_like("planetesimal_disk", seed=3, n=20000)
    r, v, m, R, rho, typ = ref.generate(spec)
    pl = typ == T.BODY_PLANETESIMAL
    assert pl.sum() == 20000 and typ[0] == T.BODY_STAR and list(typ[1:3]) == [1, 1]
    lm = np.log(m[pl])
    lo, hi = math.log(1e-10), math.log(1e-8)
    assert lo <= lm.min() and lm.max() <= hi
    assert abs(lm.mean() - 0.5 * (lo + hi)) < 0.02 * (hi - lo)  # log-uniform
    # Sigma ~ r^-1.5 on [1, 4]: sqrt(a) is uniform on [1, 2] for circular-ish orbits
    rr = np.linalg.norm(r[pl], axis=1)
    assert 0.95 < rr.min() and rr.max() < 4.3
    assert abs(np.median(np.sqrt(rr)) - 1.5) < 0.02
    # circular speeds, Kepler's third law through calculate_phase
    vv = np.linalg.norm(v[pl], axis=1)
    assert np.allclose(vv, np.sqrt(ref.GAUSS2 * (1.0 + m[pl]) / rr), rtol=0.05)
    # radii from the density
    assert np.allclose(m[pl], ref.FOUR_PI_OVER_THREE * R[pl] ** 3 * rho[pl], rtol=1e-12)


def test_kepler_solver_matches_the_scalar_restatement():
    from redgb import bodies
    ecc = np.array([0.0, 0.01, 0.3, 0.7, 0.9, 0.05])
    mean = np.array([1.0, 0.0, 2.0, 5.5, 3.0, math.pi])
    E = ref.kepler(ecc, mean)
    for k in range(len(ecc)):
        assert E[k] == pytest.approx(bodies.kepler_equation_solver(float(ecc[k]), float(mean[k]), 1.0e-14),
                                     rel=1e-14, abs=1e-15)


def test_spec_validation_constants():
    s = DiskSpec(seed=1, n_pl=10)
    assert s.n_total == 13 and s.to_c().n_giants == 2
    with pytest.raises(ValueError):
        spec_like("no_such_config", 1)


# ---------------------------------------------------------------- rg_populate_disks (CPU)
def _reference_power_law(rng, x0, x1, pw, n):
    """distribution.cpp:187-207 with numpy's generator in place of the Mersenne twister."""
    y_min, y_max = sorted((0.0 if pw == 0 else x0 ** pw, 1.0 if pw == 0 else x1 ** pw))
    d_y, d_x = y_max - y_min, x1 - x0
    out = []
    while len(out) < n:
        x = rng.uniform(0.0, d_x * d_y, n) / d_y + x0
        y = rng.uniform(y_min, y_max, n)
        out.extend(x[~(y > x ** pw)])
    return np.array(out[:n])


def _reference_lognormal(rng, x0, x1, mu, sigma, n):
    """distribution.cpp:223-249 with numpy's generator."""
    def pdf(x):
        return 1.0 / (np.sqrt(2.0 * np.pi) * sigma * x) * np.exp(-(np.log(x) - mu) ** 2 / (2.0 * sigma ** 2))
    y_max = pdf(np.exp(mu - sigma ** 2))
    out = []
    while len(out) < n:
        x = rng.uniform(0.0, (x1 - x0) * y_max, n) / y_max + x0
        y = rng.uniform(0.0, y_max, n)
        out.extend(x[~(y > pdf(x))])
    return np.array(out[:n])


@pytest.mark.parametrize("kind,params", [(ref.DIST_POWER_LAW, (0.9, 2.7, -1.5)), (ref.DIST_POWER_LAW, (1.0, 4.0, 0.5)),
                                         (ref.DIST_LOGNORMAL, (0.1, 3.0, 0.0, 0.25)),
                                         (ref.DIST_LOGNORMAL, (0.5, 20.0, 1.0, 0.8))])
def test_distributions_follow_the_reference_samplers(kind, params):
    """The populate draws (restated) and the reference's rejection samplers give the same
    distribution: two-sample Kolmogorov-Smirnov test on 20 000 draws each."""
    stats = pytest.importorskip("scipy.stats")
    n = 20000
    ours = ref.sample_dist(kind, params, 123456789, np.arange(n), ref.POP_ITEM0)
    rng = np.random.default_rng(5)
    theirs = (_reference_power_law(rng, *params, n) if kind == ref.DIST_POWER_LAW else
              _reference_lognormal(rng, *params, n))
    assert stats.ks_2samp(ours, theirs).pvalue > 1e-3
    assert ours.min() >= params[0] and ours.max() <= params[1]


def test_closed_form_distributions():
    """Exponential, Rayleigh and the reference's Box-Muller normal against their laws."""
    stats = pytest.importorskip("scipy.stats")
    k = np.arange(20000)
    x = ref.sample_dist(ref.DIST_EXPONENTIAL, (2.5,), 7, k, ref.POP_ITEM0)
    assert stats.kstest(x, stats.expon(0.0, 1.0 / 2.5).cdf).pvalue > 1e-3
    x = ref.sample_dist(ref.DIST_RAYLEIGH, (0.01,), 7, k, ref.POP_ITEM0 + 1)
    assert stats.kstest(x, stats.rayleigh(0.0, 0.01).cdf).pvalue > 1e-3
    x = ref.sample_dist(ref.DIST_NORMAL, (3.0, 0.5), 7, k, ref.POP_ITEM0 + 2)
    assert stats.kstest(x, stats.norm(3.0, 0.5).cdf).pvalue > 1e-3
    x = ref.sample_dist(ref.DIST_UNIFORM, (2.0, 5.0), 7, k, ref.POP_ITEM0 + 3)
    assert x.min() > 2.0 and x.max() <= 5.0 and stats.kstest(x, stats.uniform(2.0, 3.0).cdf).pvalue > 1e-3


@pytest.mark.parametrize("r_SL", [0.5, 2.7, 5.0, 50.0])
@pytest.mark.parametrize("p", [-1.5, -2.0])
def test_mmsn_masses(r_SL, p):
    """rg_mmsn_gas_mass / rg_mmsn_solid_mass (host arithmetic only) equal the restatement of
    nebula.cpp bit for bit, snow line below, inside and beyond the disk, and p = -2 (the
    logarithmic integral)."""
    from redgb import icgen
    kw = dict(r_1=0.9, r_2=2.7 if r_SL != 50.0 else 30.0, r_SL=r_SL, f_neb=3.0, Sigma_1=7.0 * icgen.GRAM_PER_CM2, p=p)
    assert icgen.mmsn_solid_mass(f_ice=4.2, **kw) == ref.mmsn_solid(f_ice=4.2, **kw)
    assert icgen.mmsn_gas_mass(f_gas=240.0, **kw) == ref.mmsn_gas(f_gas=240.0, **kw)
    if p == -1.5 and r_SL == 2.7:  # the solids lie inside the snow line: 2 pi f Sigma_1 (r^0.5) / 0.5
        s1 = kw["Sigma_1"]
        assert icgen.mmsn_solid_mass(f_ice=4.2, **kw) == pytest.approx(
            2 * np.pi * 3.0 * s1 / 0.5 * (2.7 ** 0.5 - 0.9 ** 0.5), rel=1e-14)


def test_dvorak_disk_spec():
    from redgb import icgen, types as T
    d = icgen.dvorak_disk(seed=3, n_pp=10)
    assert d.n_total == 11 and d.names()[:2] == ["star", "proto1"] and d.to_bc
    assert d.pp_total_mass == icgen.mmsn_solid_mass(**icgen.DVORAK_SOLIDS)
    r, v, m, R, rho, cd, typ = ref.populate(d)
    assert m[0] == 1.0 and R[0] == icgen.SOLAR_RADIUS_AU and list(typ) == [0] + [T.BODY_PROTOPLANET] * 10
    assert abs(m[1:].sum() - d.pp_total_mass) < 1e-15
    np.testing.assert_allclose(rho[1:], 2.7 * icgen.GRAM_PER_CM3, rtol=0)
    assert abs((m[:, None] * r).sum(0)).max() < 1e-15 and abs((m[:, None] * v).sum(0)).max() < 1e-17


@pytest.mark.parametrize("name", ["dvorak", "n_gp", "n_pp", "n_spl", "n_pl"])
def test_reference_presets_restated(name, tmp_path):
    """The reference's disk set-ups as specs: counts, derived properties, barycentre, and a
    body file written from the restatement reads back the same."""
    from redgb import bodies, icgen
    spec = icgen.reference_preset(name, seed=4, n=40)
    r, v, m, R, rho, cd, typ = ref.populate(spec)
    assert spec.n_total == 41 and typ[0] == T.BODY_STAR and np.all(typ[1:] == typ[1])
    assert np.all(np.isfinite(r)) and np.all(np.isfinite(v)) and np.all(np.isfinite(R))
    assert abs((m[:, None] * r).sum(0)).max() < 1e-12 * abs(m[:, None] * r).max()
    if name == "n_pp":  # radius and density given: mass = 4 pi / 3 R^3 rho
        np.testing.assert_allclose(m[1:], 4.0 / 3.0 * np.pi * R[1:] ** 3 * rho[1:], rtol=1e-14)
    if name == "n_spl":  # superplanetesimals keep all three as drawn
        assert np.all((m[1:] >= 1e-10) & (m[1:] <= 1e-9))
    disk = bodies.empty_disk(list(spec.n_body))
    for f, col in zip("xyz", range(3)):
        disk.r[f], disk.v[f] = r[:, col], v[:, col]
    disk.p["mass"], disk.p["radius"], disk.p["density"], disk.p["cd"] = m, R, rho, cd
    disk.md["id"], disk.md["body_type"] = np.arange(1, 42), typ
    disk.names = spec.names()
    path = tmp_path / f"{name}.txt"
    bodies.write_body_file(path, disk)
    back = bodies.read_body_file(path)
    assert back.counts == disk.counts and back.names == disk.names
    np.testing.assert_allclose(back.p["mass"], m, rtol=1e-15)
    np.testing.assert_allclose(back.r["x"], r[:, 0], rtol=1e-15, atol=0)


def test_initial_command_line_arguments():
    """redgb.initial refuses a non-positive disk count and the set-ups it does not offer
    before it draws anything."""
    from redgb import initial
    for argv in (["n_pl", "--count", "0", "-o", "x"], ["n_tp", "-o", "x"], ["two_body", "-o", "x"],
                 ["n_pl", "--n", "-1", "-o", "x"]):
        with pytest.raises(SystemExit):
            initial.main(argv)
