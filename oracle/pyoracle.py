"""ORACLE (test infrastructure only): ctypes view of oracle/_build/libredoracle.so.

The CPU restatement of the reference's FP64 path (redoracle.c).  Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg import this module, always as
the checker or the timed CPU baseline; the product never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
PKG = os.path.join(ROOT, "red.cuda.closeencounter_gb300")
if PKG not in sys.path:
    sys.path.insert(0, PKG)

from redgb import types as T  # noqa: E402
from redgb.api import System, bind  # noqa: E402

LIB_PATH = os.path.join(HERE, "_build", "libredoracle.so")
_lib = None


def build(force=False):
    """Compile the oracle library (a few seconds, plain gcc)."""
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(
            os.path.join(HERE, "redoracle.c")):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        bind(L, "ro_", has_last_error=False)
        vp, ci, cd = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
        L.ro_set_dt_replay.argtypes = [vp, vp, ci]
        L.ro_grav_accel_rows.argtypes = [ctypes.POINTER(T.Counts), vp, vp, vp, ci, ci, vp]
        L.ro_calculate_radius.restype = cd
        L.ro_calculate_radius.argtypes = [cd, cd]
        L.ro_calculate_density.restype = cd
        L.ro_calculate_density.argtypes = [cd, cd]
        L.ro_calculate_mass.restype = cd
        L.ro_calculate_mass.argtypes = [cd, cd]
        L.ro_calc_position_after_collision.argtypes = [cd, cd, vp, vp, vp]
        L.ro_calc_velocity_after_collision.argtypes = [cd, cd, vp, vp, vp]
        L.ro_calc_physical_properties.argtypes = [vp, vp, vp]
        L.ro_kepler_equation_solver.argtypes = [cd, cd, cd, ctypes.POINTER(cd)]
        L.ro_calculate_phase.argtypes = [cd, vp, vp, vp]
        L.ro_calculate_orbital_element.argtypes = [cd, vp, vp, vp]
        L.ro_transform_to_bc.argtypes = [ci, vp, vp, vp]
        _lib = L
    return _lib


class OracleSystem(System):
    """The CPU oracle behind the same Python interface as the CUDA library."""

    prefix = "ro_"

    def __init__(self, disk, thr, frame=T.FRAME_BARY):
        super().__init__(lib(), disk, thr, _create_extra=False, frame=frame)

    def set_dt_replay(self, dts_internal):
        a = np.ascontiguousarray(dts_internal, np.float64)
        self._call("set_dt_replay", self.handle, T.ptr(a), int(a.size))


def grav_accel_rows(disk, r_internal, i_begin, i_end):
    """Reference FP64 accelerations of sinks [i_begin, i_end) for positions r_internal."""
    out = np.zeros(i_end - i_begin, T.VEC)
    c = disk.counts_struct()
    rc = lib().ro_grav_accel_rows(ctypes.byref(c), T.ptr(np.ascontiguousarray(r_internal)),
                                  T.ptr(np.ascontiguousarray(disk.p)), T.ptr(np.ascontiguousarray(disk.md)),
                                  int(i_begin), int(i_end), T.ptr(out))
    if rc:
        raise RuntimeError(f"ro_grav_accel_rows: {rc}")
    return out
