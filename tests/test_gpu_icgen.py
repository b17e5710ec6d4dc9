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
