"""Python view of the ensemble C ABI (rg_ens_*): many independent disks on one GPU."""
from __future__ import annotations

import ctypes

import numpy as np

from . import lib, types as T
from .api import RedError


def _bind(L):
    if getattr(L, "_ens_bound", False):
        return L
    vp, ci, cd, i64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_int64
    sig = {
        "rg_ens_create": [ci, vp, vp, vp, vp, vp, vp, ci, ctypes.POINTER(vp)],
        "rg_ens_destroy": [vp],
        "rg_ens_set_integrator": [vp, cd, cd, ci],
        "rg_ens_set_options": [vp, ci, cd, ci],
        "rg_ens_advance": [vp, cd, i64, ctypes.POINTER(i64)],
        "rg_ens_get_state": [vp, ci, vp, vp, vp, vp, ctypes.POINTER(cd)],
        "rg_ens_get_stats": [vp, ci, ctypes.POINTER(T.EnsStats)],
        "rg_ens_events": [vp, vp, vp, ci, ctypes.POINTER(ci)],
        "rg_ens_event_count": [vp, ctypes.POINTER(ci)],
        "rg_ens_set_step_log": [vp, ci],
        "rg_ens_step_log": [vp, vp, ci, ctypes.POINTER(ci)],
        "rg_ens_energy": [vp, ci, ctypes.POINTER(cd), vp],
        "rg_ens_get_stream": [vp, ctypes.POINTER(vp)],
        "rg_ens_kernel_count": [vp, ctypes.POINTER(i64), ctypes.POINTER(i64)],
        "rg_ens_autotune": [vp, ci, ctypes.POINTER(T.Tune)],
        "rg_ens_set_profiling": [vp, ci],
        "rg_ens_get_profile": [vp, ctypes.POINTER(T.Profile)],
    }
    for name, args in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = ci
    L._ens_bound = True
    return L


class Ensemble:
    """Independent disks integrated together (RKF7(8), per-disk adaptive steps)."""

    def __init__(self, disks, thr, event_capacity=0):
        self._lib = _bind(lib.load())
        self.disks = list(disks)
        self.n_sys = len(self.disks)
        counts = (T.Counts * self.n_sys)(*[d.counts_struct() for d in self.disks])
        cat = lambda f: np.ascontiguousarray(np.concatenate([getattr(d, f) for d in self.disks]))
        thr = np.asarray(thr, np.float64)
        if thr.ndim == 1:
            thr = np.tile(thr, (self.n_sys, 1))
        thr = np.ascontiguousarray(thr.reshape(-1))
        self._keep = (cat("r"), cat("v"), cat("p"), cat("md"), thr)
        self.handle = ctypes.c_void_p()
        self._call("rg_ens_create", self.n_sys, ctypes.cast(counts, ctypes.c_void_p), *[T.ptr(a) for a in self._keep],
                   int(event_capacity), ctypes.byref(self.handle))

    def _call(self, name, *args):
        rc = getattr(self._lib, name)(*args)
        if rc != 0:
            raise RedError(name, rc, self._lib.rg_last_error().decode())

    def close(self):
        if self.handle:
            self._lib.rg_ens_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_integrator(self, dt_day=0.001, tolerance=1e-10, error_check_for_tp=False):
        self._call("rg_ens_set_integrator", self.handle, float(dt_day), float(tolerance), int(bool(error_check_for_tp)))
        return self

    def set_options(self, gravity_mode=T.GRAVITY_FP64, hill_factor=0.0, use_graph=True):
        self._call("rg_ens_set_options", self.handle, int(gravity_mode), float(hill_factor), int(bool(use_graph)))
        return self

    def set_step_log(self, capacity):
        self._call("rg_ens_set_step_log", self.handle, int(capacity))

    def advance(self, t_stop_day, max_attempts=0):
        n = ctypes.c_int64()
        self._call("rg_ens_advance", self.handle, float(t_stop_day), int(max_attempts), ctypes.byref(n))
        return n.value

    def state(self, sys):
        n = self.disks[sys].n_total
        r, v, p, md = np.zeros(n, T.VEC), np.zeros(n, T.VEC), np.zeros(n, T.PARAM), np.zeros(n, T.BODY_MD)
        t = ctypes.c_double()
        self._call("rg_ens_get_state", self.handle, int(sys), T.ptr(r), T.ptr(v), T.ptr(p), T.ptr(md), ctypes.byref(t))
        return r, v, p, md, t.value

    def stats(self, sys):
        st = T.EnsStats()
        self._call("rg_ens_get_stats", self.handle, int(sys), ctypes.byref(st))
        return st.as_dict()

    def events(self):
        n = ctypes.c_int()
        self._call("rg_ens_event_count", self.handle, ctypes.byref(n))
        out = np.zeros(max(n.value, 1), T.EVENT)
        sysv = np.zeros(max(n.value, 1), np.int32)
        got = ctypes.c_int()
        self._call("rg_ens_events", self.handle, T.ptr(out), T.ptr(sysv), int(n.value), ctypes.byref(got))
        return out[:got.value], sysv[:got.value]

    def step_log(self, cap=1 << 22):
        out = np.zeros(cap, T.STEP_REC)
        got = ctypes.c_int()
        self._call("rg_ens_step_log", self.handle, T.ptr(out), int(cap), ctypes.byref(got))
        return out[:got.value].copy()

    def energy(self, sys):
        e = ctypes.c_double()
        L = (ctypes.c_double * 3)()
        self._call("rg_ens_energy", self.handle, int(sys), ctypes.byref(e), L)
        return e.value, np.array(list(L))

    def stream(self):
        p = ctypes.c_void_p()
        self._call("rg_ens_get_stream", self.handle, ctypes.byref(p))
        return p.value

    def autotune(self, reps=3):
        """Time the candidate tile shapes of the current gravity mode on these disks and keep
        the fastest (rg_ens_autotune); returns the choice (`mixed_chunks`: sources per
        few-sink CTA, 0 = automatic)."""
        t = T.Tune()
        self._call("rg_ens_autotune", self.handle, int(reps), ctypes.byref(t))
        return {f: getattr(t, f) for f, _ in t._fields_}

    def set_profiling(self, on=True):
        """Time each launch group of every attempt with CUDA events (direct launches)."""
        self._call("rg_ens_set_profiling", self.handle, int(bool(on)))

    def profile(self):
        """Summed device times since the last call: gravity, stage and other kernels."""
        prof = T.Profile()
        self._call("rg_ens_get_profile", self.handle, ctypes.byref(prof))
        return {f: getattr(prof, f) for f, _ in prof._fields_}

    def kernel_count(self):
        a, b = ctypes.c_int64(), ctypes.c_int64()
        self._call("rg_ens_kernel_count", self.handle, ctypes.byref(a), ctypes.byref(b))
        return a.value, b.value
