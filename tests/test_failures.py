"""Failures injected on the host (no GPU): malformed or missing input files, and a NaN in the
state, which the reference's integrator carries along without an error (its maximum of the
error estimate skips NaN, integrator.cu:211-256) until its step becomes infinite."""
import numpy as np
import pytest

import pyoracle
from redgb import bodies, red, types as T


def _write_disk(path, n_pl=5):
    disk = bodies.make_disk(n_pl=n_pl, seed=2)
    bodies.write_body_file(str(path), disk)
    return disk


def test_truncated_body_file_is_refused(tmp_path):
    p = tmp_path / "bodies.txt"
    _write_disk(p)
    text = p.read_text().split()
    p.write_text(" ".join(text[:-5]) + "\n")
    with pytest.raises(ValueError):
        bodies.read_body_file(str(p))


def test_non_numeric_body_field_is_refused(tmp_path):
    p = tmp_path / "bodies.txt"
    _write_disk(p)
    text = p.read_text().split()
    text[7 + 4] = "heavy"  # the first record's mass
    p.write_text(" ".join(text) + "\n")
    with pytest.raises(ValueError):
        bodies.read_body_file(str(p))


def test_cli_reports_missing_and_invalid_files(tmp_path, capsys):
    assert red.main(["-iDir", str(tmp_path), "-p", "nope.txt", "-ic", "b.txt"]) == 1
    (tmp_path / "p.txt").write_text("integrator = rk99\n")
    _write_disk(tmp_path / "b.txt")
    assert red.main(["-iDir", str(tmp_path), "-p", "p.txt", "-ic", "b.txt"]) == 1
    assert "Invalid integrator" in capsys.readouterr().err


def test_nan_in_the_state_reaches_a_non_finite_step():
    """The reference's behaviour, restated by the oracle: a NaN body spreads to every body it
    attracts, the error maximum skips NaN and reads 0, and the controller's next step is
    infinite; the oracle goes on without an error (the CUDA library reports
    RG_ERR_DT_NONFINITE there instead, test_gpu_parity.py)."""
    disk = bodies.make_disk(n_pl=30, seed=3)
    o = pyoracle.OracleSystem(disk, bodies.thresholds())
    o.set_integrator(T.INT_RKF78, 0.01, True, 1e-10)
    r, v = o.state()[:2]
    r["x"][7] = np.nan
    o.set_state(r, v)
    o.step()
    assert np.isnan(o.state()[0]["x"]).sum() > 1  # every body feels the NaN body
    o.step()
    assert not all(np.isfinite(o.dt()))
