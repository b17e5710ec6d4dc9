"""rg_energy_noalloc against rg_energy, through the C ABI.

rg_energy_noalloc gives rg_energy's energy / angular-momentum diagnostic for bodies the
caller keeps in device memory, with a fixed device scratch in place of any allocation.
The caller here is this test: it copies a context's state, in the reference's record
layouts and internal units (rg_get_state_internal), into device memory it owns and calls
the entry point twice in a row (default stream, then a stream of its own); both results
must agree with rg_energy on the same state within REL_TOL.  The two entry points run the
same operations in the same order, so they are expected to agree to the last bit; the
tolerance only leaves room for a future change of summation order.

The file is named to be collected last, so that in a full run it also shows the scratch
set-up working after every other GPU test has used the library in the same process.
"""
import ctypes

import numpy as np
import pytest
import torch

import helpers as H
from redgb import bodies, lib, types as T

pytestmark = pytest.mark.gpu

REL_TOL = 1e-14
MAX_BODIES = 65536  # RG_ENERGY_NOALLOC_MAX_BODIES
RG_ERR_ARG = -1


def _entry(L):
    f = L.rg_energy_noalloc
    vp, dp = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)
    f.argtypes = [ctypes.POINTER(T.Counts), vp, vp, vp, vp, vp, dp, dp]
    f.restype = ctypes.c_int
    return f


def _on_device(rec):
    """A device copy of a record array, in memory the caller owns."""
    return torch.from_numpy(np.ascontiguousarray(rec).view(np.uint8).copy()).to("cuda")


def _call(f, counts, dev, stream):
    e = ctypes.c_double()
    L = (ctypes.c_double * 3)()
    rc = f(ctypes.byref(counts), *[ctypes.c_void_p(t.data_ptr()) for t in dev], ctypes.c_void_p(stream),
           ctypes.byref(e), L)
    return rc, e.value, np.array(list(L))


def _check_twice(gpulib, system):
    """Two calls in a row on the system's current state, each against rg_energy."""
    f = _entry(gpulib)
    E0, L0 = system.energy()
    counts, n = system.n_total()
    r, v, p, md, _ = system.state(internal=True)
    dev = [_on_device(a) for a in (r, v, p, md)]
    torch.cuda.synchronize()
    side = torch.cuda.Stream()
    for stream in (None, side.cuda_stream):
        rc, E, L = _call(f, counts, dev, stream)
        assert rc == 0, gpulib.rg_last_error().decode()
        assert abs(E - E0) <= REL_TOL * abs(E0), (E, E0)
        assert np.all(np.abs(L - L0) <= REL_TOL * np.linalg.norm(L0)), (L, L0)
    return n


def test_matches_rg_energy_before_and_after_merges(gpulib):
    """A small disk with every body type, then the same disk after collisions have merged
    bodies (inactive records are skipped by both entry points)."""
    disk, params, _, _ = H.load_fixture("disk_si_rkf78_collide")
    s = lib.System(disk, H.thresholds_of(params))
    H.configure(s, params)
    _check_twice(gpulib, s)
    H.run_fixture(s, params)
    _, _, _, md, _ = s.state(internal=True)
    assert np.any(md["id"] <= 0) or len(md) < len(disk.md)
    _check_twice(gpulib, s)


def test_matches_rg_energy_self_gravitating(gpulib):
    s = lib.System(bodies.config_disk("self_gravitating", n=4096), bodies.thresholds())
    assert _check_twice(gpulib, s) == 4097


def test_largest_accepted_size_and_rejection_beyond(gpulib):
    """Exactly RG_ENERGY_NOALLOC_MAX_BODIES bodies run; one more is refused with
    RG_ERR_ARG before any device work (the body pointers are not read)."""
    disk = bodies.config_disk("planetesimal_disk", n=MAX_BODIES - 3)
    s = lib.System(disk, bodies.thresholds())
    assert _check_twice(gpulib, s) == MAX_BODIES
    f = _entry(gpulib)
    counts = T.Counts()
    counts.n_s, counts.n_pl = 1, MAX_BODIES
    e = ctypes.c_double()
    L = (ctypes.c_double * 3)()
    rc = f(ctypes.byref(counts), None, None, None, None, None, ctypes.byref(e), L)
    assert rc == RG_ERR_ARG
    assert str(MAX_BODIES) in gpulib.rg_last_error().decode()
