"""Loads libredgb.so and declares the C ABI (include/redgb.h).

There is no CPU fallback: if the library is missing or no CUDA device is visible the
calls raise.
"""
from __future__ import annotations

import ctypes
import os

from . import api
from . import types as T
from . import build as _build

_lib = None


def load(auto_build=True):
    """The loaded library (built first if its sources changed and nvcc is available)."""
    global _lib
    if _lib is not None:
        return _lib
    if auto_build and _build.stale():
        _build.build()
    if not os.path.exists(_build.LIB):
        raise RuntimeError(f"{_build.LIB} is missing: build it with `python -m redgb.build`")
    L = ctypes.CDLL(_build.LIB)
    api.bind(L, "rg_")
    vp, ci = ctypes.c_void_p, ctypes.c_int
    L.rg_set_gravity_mode.argtypes = [vp, ci]
    L.rg_set_gravity_mode.restype = ci
    L.rg_version.restype = ctypes.c_char_p
    L.rg_device_count.restype = ci
    L.rg_get_stream.argtypes = [vp, ctypes.POINTER(ctypes.c_void_p)]
    L.rg_set_profiling.argtypes = [vp, ci]
    L.rg_get_profile.argtypes = [vp, ctypes.POINTER(T.Profile)]
    L.rg_measure_pipe_peak.argtypes = [ci, ctypes.POINTER(ctypes.c_double)]
    L.rg_autotune.argtypes = [vp, ci, ctypes.POINTER(T.Tune)]
    L.rg_set_launch_shape.argtypes = [vp, ctypes.POINTER(T.Tune)]
    L.rg_test_hold_tile_copies.argtypes = [vp, ci]
    _lib = L
    return L


def device_count():
    return load().rg_device_count()


class System(api.System):
    """One disk on the GPU through the C ABI (pp_disk + integrator of the reference)."""

    prefix = "rg_"

    def __init__(self, disk, thr, event_capacity=0, frame=T.FRAME_BARY):
        super().__init__(load(), disk, thr, event_capacity=event_capacity, frame=frame)

    def set_gravity_mode(self, mode):
        self._call("set_gravity_mode", self.handle, int(mode))
        return self

    def stream(self):
        p = ctypes.c_void_p()
        self._call("get_stream", self.handle, ctypes.byref(p))
        return p.value

    def set_profiling(self, on=True):
        self._call("set_profiling", self.handle, int(bool(on)))

    def profile(self):
        prof = T.Profile()
        self._call("get_profile", self.handle, ctypes.byref(prof))
        return {f: getattr(prof, f) for f, _ in prof._fields_}

    def test_hold_tile_copies(self, on=True):
        """Test hook: the mixed kernel issues no tile copies, so its bounded waits run out
        and the evaluation reports RG_ERR_CUDA (rg_test_hold_tile_copies)."""
        self._call("test_hold_tile_copies", self.handle, int(bool(on)))

    def autotune(self, reps=3):
        """Time the candidate launch shapes of the current gravity mode and keep the fastest
        (rg_autotune); returns the choice."""
        t = T.Tune()
        self._call("autotune", self.handle, int(reps), ctypes.byref(t))
        return {f: getattr(t, f) for f, _ in t._fields_}

    def set_launch_shape(self, pairpar_sinks=16, rowseq_max_src=64, mixed_chunks=0):
        """Pin the launch shape (rg_set_launch_shape), e.g. one an earlier autotune chose."""
        t = T.Tune()
        t.pairpar_sinks, t.rowseq_max_src, t.mixed_chunks = int(pairpar_sinks), int(rowseq_max_src), int(mixed_chunks)
        self._call("set_launch_shape", self.handle, ctypes.byref(t))


def measure_pipe_peak(kind):
    """Measured FP32 (kind 0) or FP64 (kind 1) FMA throughput of the device, TFLOP/s."""
    L = load()
    out = ctypes.c_double()
    rc = L.rg_measure_pipe_peak(int(kind), ctypes.byref(out))
    if rc:
        raise api.RedError("rg_measure_pipe_peak", rc, L.rg_last_error().decode())
    return out.value
