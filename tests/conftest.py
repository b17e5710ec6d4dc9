import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "red.cuda.closeencounter_gb300"), os.path.join(ROOT, "oracle"),
          os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the CUDA library)")


@pytest.fixture(scope="session")
def gpulib():
    from redgb import lib
    L = lib.load()
    if L.rg_device_count() <= 0:
        pytest.fail("no CUDA device visible to libredgb.so")
    return L


@pytest.fixture(scope="session")
def planetesimal_disk_1000yr_oracle():
    """The oracle's run of the 1000-year planetesimal-disk workload with close encounters at
    3 mutual Hill radii: (disk, thresholds, steps, events, oracle system), computed once."""
    import helpers as H
    import pyoracle
    from redgb import types as T
    disk, params, _, _ = H.load_fixture("planetesimal_disk_1000yr")
    thr = H.thresholds_of(params)
    o = pyoracle.OracleSystem(disk, thr)
    o.set_integrator(T.INT_RKF78, 0.001, True, params["tolerance"])
    o.set_event_options(hill_factor=3.0)
    n = o.advance(params["length_yr"] * T.YEAR)
    return disk, thr, params, n, o.events(), o
