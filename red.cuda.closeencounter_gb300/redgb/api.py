"""Python view of the C ABI: one planetesimal disk driven through its context.

`System` mirrors the reference's pp_disk + integrator pair (pp_disk.h:14-195,
integrator.h:17-88) one call per C entry point; it is a thin ctypes layer, every number
is computed by the CUDA library (libredgb.so).  The same class drives the CPU oracle's
library, whose functions carry the same names with an ``ro_`` prefix, so parity tests
call both implementations the same way.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import types as T

_c_int_p = ctypes.POINTER(ctypes.c_int)
_c_i64_p = ctypes.POINTER(ctypes.c_int64)
_c_dbl_p = ctypes.POINTER(ctypes.c_double)


class RedError(RuntimeError):
    """A C entry point returned a non-zero status."""

    def __init__(self, func, status, msg=""):
        self.status = status
        name = T.STATUS.get(status, str(status))
        super().__init__(f"{func} failed: {name}{(': ' + msg) if msg else ''}")


def bind(lib, prefix, has_last_error=True):
    """Declare argument types of the context entry points of `lib`."""
    vp, ci, cd = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
    sigs = {
        "create": None,
        "create_in_frame": None,
        "destroy": [vp],
        "set_integrator": [vp, ci, cd, ci, cd, ci],
        "set_event_options": [vp, ci, ci, cd, ci],
        "set_time": [vp, cd],
        "step": [vp, _c_dbl_p],
        "check_for_ejection_hit_centrum": [vp, _c_int_p],
        "check_for_collision": [vp, _c_int_p],
        "check_for_close_encounter": [vp, _c_int_p],
        "check_for_rebuild_vectors": [vp, ci, _c_int_p],
        "advance": [vp, cd, ctypes.c_int64, _c_i64_p],
        "events": [vp, vp, ci, _c_int_p],
        "event_count": [vp, _c_int_p],
        "get_n_total": [vp, ctypes.POINTER(T.Counts), _c_int_p],
        "get_state": [vp, vp, vp, vp, vp, _c_dbl_p],
        "get_state_internal": [vp, vp, vp, vp, vp, _c_dbl_p],
        "set_state": [vp, vp, vp],
        "calc_accel": [vp, vp],
        "get_counters": [vp, ctypes.POINTER(T.Counters)],
        "energy": [vp, _c_dbl_p, _c_dbl_p],
        "get_dt": [vp, _c_dbl_p, _c_dbl_p],
    }
    for name, args in sigs.items():
        f = getattr(lib, prefix + name)
        if args is not None:
            f.argtypes = args
        f.restype = ctypes.c_int if name != "destroy" or prefix == "rg_" else None
    if has_last_error:
        lib.rg_last_error.restype = ctypes.c_char_p
        lib.rg_last_error.argtypes = []
    return lib


class System:
    """One disk: the reference's pp_disk + integrator behind the C ABI."""

    prefix = "rg_"

    def __init__(self, lib, disk, thr, event_capacity=0, _create_extra=True, frame=T.FRAME_BARY):
        self._lib = lib
        self._f = lambda name: getattr(lib, self.prefix + name)
        self.handle = ctypes.c_void_p()
        self._disk = disk
        counts = disk.counts_struct()
        thr = np.ascontiguousarray(thr, np.float64)
        args = [ctypes.byref(counts), T.ptr(np.ascontiguousarray(disk.r)), T.ptr(np.ascontiguousarray(disk.v)),
                T.ptr(np.ascontiguousarray(disk.p)), T.ptr(np.ascontiguousarray(disk.md)),
                T.ptr(np.ascontiguousarray(disk.epoch)), T.ptr(thr)]
        if _create_extra:
            args.append(ctypes.c_int(event_capacity))
        if frame != T.FRAME_BARY:
            args.append(ctypes.c_int(frame))
        args.append(ctypes.byref(self.handle))
        self._call("create" if frame == T.FRAME_BARY else "create_in_frame", *args)

    # ------------------------------------------------------------------ plumbing
    def _msg(self):
        try:
            return self._lib.rg_last_error().decode()
        except AttributeError:
            return ""

    def _call(self, name, *args):
        rc = self._f(name)(*args)
        if rc != 0:
            raise RedError(self.prefix + name, rc, self._msg())
        return rc

    def close(self):
        if self.handle:
            self._f("destroy")(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ------------------------------------------------------------------ set-up
    def set_integrator(self, int_type, dt_day=0.001, adaptive=True, tolerance=1e-10, error_check_for_tp=False):
        self._call("set_integrator", self.handle, int(int_type), float(dt_day), int(bool(adaptive)),
                   float(tolerance), int(bool(error_check_for_tp)))
        return self

    def set_event_options(self, close_encounter=False, inner_steps=True, hill_factor=0.0,
                          event_time_mode=T.EVENT_TIME_CPU):
        self._call("set_event_options", self.handle, int(bool(close_encounter)), int(bool(inner_steps)),
                   float(hill_factor), int(event_time_mode))
        return self

    def set_time(self, t_day):
        self._call("set_time", self.handle, float(t_day))

    # ------------------------------------------------------------------ stepping
    def step(self):
        dt = ctypes.c_double()
        self._call("step", self.handle, ctypes.byref(dt))
        return dt.value

    def check_for_ejection_hit_centrum(self):
        n = ctypes.c_int()
        self._call("check_for_ejection_hit_centrum", self.handle, ctypes.byref(n))
        return n.value

    def check_for_collision(self):
        n = ctypes.c_int()
        self._call("check_for_collision", self.handle, ctypes.byref(n))
        return n.value

    def check_for_close_encounter(self):
        n = ctypes.c_int()
        self._call("check_for_close_encounter", self.handle, ctypes.byref(n))
        return n.value

    def check_for_rebuild_vectors(self, n=8):
        out = ctypes.c_int()
        self._call("check_for_rebuild_vectors", self.handle, int(n), ctypes.byref(out))
        return bool(out.value)

    def advance(self, t_stop_day, max_steps=0):
        n = ctypes.c_int64()
        self._call("advance", self.handle, float(t_stop_day), int(max_steps), ctypes.byref(n))
        return n.value

    # ------------------------------------------------------------------ read-out
    def events(self):
        n = ctypes.c_int()
        self._call("event_count", self.handle, ctypes.byref(n))
        out = np.zeros(max(n.value, 1), T.EVENT)
        got = ctypes.c_int()
        self._call("events", self.handle, T.ptr(out), int(n.value), ctypes.byref(got))
        return out[:got.value]

    def n_total(self):
        c = T.Counts()
        n = ctypes.c_int()
        self._call("get_n_total", self.handle, ctypes.byref(c), ctypes.byref(n))
        return c, n.value

    def state(self, internal=False, out=None, params=True):
        """(r, v, p, md, t): positions and velocities as vec_t records (AU, AU/day; internal
        units with `internal`), parameters, metadata and the time.  `out`: two vec_t arrays of
        n_total records to fill instead of new ones (e.g. pinned host buffers); with
        params=False, p and md are not copied and come back as None."""
        _, n = self.n_total()
        if out is None:
            r, v = np.zeros(n, T.VEC), np.zeros(n, T.VEC)
        else:
            r, v = out
            for a in (r, v):
                if a.dtype != T.VEC or a.shape != (n,) or not a.flags["C_CONTIGUOUS"]:
                    raise ValueError("out: two contiguous vec_t arrays of n_total records")
        p, md = (np.zeros(n, T.PARAM), np.zeros(n, T.BODY_MD)) if params else (None, None)
        t = ctypes.c_double()
        self._call("get_state_internal" if internal else "get_state", self.handle, T.ptr(r), T.ptr(v), T.ptr(p),
                   T.ptr(md), ctypes.byref(t))
        return r, v, p, md, t.value

    def time(self, internal=True):
        """The clock alone (internal units, or days with internal=False); copies no state."""
        t = ctypes.c_double()
        self._call("get_state_internal" if internal else "get_state", self.handle, None, None, None, None,
                   ctypes.byref(t))
        return t.value

    def set_state(self, r, v):
        self._call("set_state", self.handle, T.ptr(np.ascontiguousarray(r)), T.ptr(np.ascontiguousarray(v)))

    def calc_accel(self):
        _, n = self.n_total()
        a = np.zeros(n, T.VEC)
        self._call("calc_accel", self.handle, T.ptr(a))
        return a

    def counters(self):
        c = T.Counters()
        self._call("get_counters", self.handle, ctypes.byref(c))
        return c.as_dict()

    def energy(self):
        e = ctypes.c_double()
        L = (ctypes.c_double * 3)()
        self._call("energy", self.handle, ctypes.byref(e), L)
        return e.value, np.array(list(L))

    def dt(self):
        a, b = ctypes.c_double(), ctypes.c_double()
        self._call("get_dt", self.handle, ctypes.byref(a), ctypes.byref(b))
        return a.value, b.value


def vec3(a):
    """(n, 3) float64 view of a VEC array."""
    return np.stack([a["x"], a["y"], a["z"]], axis=1)
