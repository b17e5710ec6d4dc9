"""The reference-compatible command line (redgb.red): options, parameter file, output names,
and (GPU) a whole run whose result and event files are the reference's, byte for byte."""
import gzip
import importlib.util
import os

import pytest

import helpers as H
from redgb import bodies, red, types as T


def _case(name):
    """Stored initial state (exact arrays) with the case's body names."""
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(H.GOLDEN, "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    names = next(d.names for n, d, _ in mg.cases() if n == name)
    disk, params, _, _ = H.load_fixture(name)
    disk.names = list(names)
    return disk, params


def test_options_and_refusals():
    o = red.parse_options(["-gpu", "-ef", "-iDir", "D", "-p", "p.txt", "-ic", "b.txt", "-result", "res"])
    assert (o["iDir"], o["p"], o["ic"], o["ef"], o["result"]) == ("D", "p.txt", "b.txt", True, "res")
    for bad in (["-cpu", "-p", "a", "-ic", "b"], ["-p", "a"], ["-ups", "-p", "a", "-ic", "b"], ["-x"]):
        with pytest.raises(red.UsageError):
            red.parse_options(bad)


def test_parameter_file_and_output_names(tmp_path):
    path = tmp_path / "parameters.txt"
    bodies.write_parameter_file(str(path), integrator="rkf8", tolerance=1e-10, length_yr=3.0, output_interval_yr=0.5,
                                ejection=3.2, hit_centrum=0.3, collision_factor=1.0, output_type="binary")
    prm = red.read_parameter_file(str(path))
    assert prm["int_type"] == T.INT_RKF78 and prm["adaptive"] and prm["tolerance"] == 1e-10
    assert prm["length"] == 3.0 * T.YEAR and prm["output_interval"] == 0.5 * T.YEAR
    assert (prm["ejection"], prm["hit_centrum"], prm["collision_factor"]) == (3.2, 0.3, 1.0)
    o = red.parse_options(["-ef", "-iDir", str(tmp_path), "-p", "parameters.txt", "-ic", "b.txt"])
    paths = red.output_paths(o, prm)
    assert os.path.basename(paths["result"]) == "R_gpu_ns_as_RKF8_result.bin"
    assert os.path.basename(paths["event"]) == "R_gpu_ns_as_RKF8_event.txt"
    with open(path, "a") as f:
        f.write("frame_center = astro\n")
    assert red.read_parameter_file(str(path))["frame"] == T.FRAME_ASTRO
    with open(path, "a") as f:
        f.write("frame_center = galactic\n")
    with pytest.raises(ValueError):
        red.read_parameter_file(str(path))


@pytest.mark.gpu
def test_cli_run_writes_the_reference_files(gpulib, tmp_path):
    disk, params = _case("disk_eject_hit")
    bodies.write_body_file(str(tmp_path / "bodies.txt"), disk)
    bodies.write_parameter_file(str(tmp_path / "parameters.txt"), **params)
    assert red.main(["-gpu", "-ef", "-iDir", str(tmp_path), "-p", "parameters.txt", "-ic", "bodies.txt"]) == 0
    for mine, ref in (("R_gpu_ns_as_RKF8_result.txt", "disk_eject_hit_result.txt.gz"),
                      ("R_gpu_ns_as_RKF8_event.txt", "disk_eject_hit_event.txt.gz")):
        with open(tmp_path / mine, "rb") as f, gzip.open(os.path.join(H.GOLDEN, ref), "rb") as g:
            assert f.read() == g.read(), mine
