"""Seeded synthetic disks generated on the GPU (rg_generate_disks).

A DiskSpec describes one disk: a 1 Msun star at rest in the origin, up to four giants on given
orbits, n_pl planetesimals (pl_type 5) or self-gravitating protoplanets (pl_type 3) and n_tp
test particles.  Each body's random numbers come from Philox4x32-10 keyed by the disk's seed,
so the disks do not depend on how many are generated together.  `spec_like(config, seed, n)`
gives the spec of one of the benchmark configurations.
"""
from __future__ import annotations

import ctypes
import dataclasses

import numpy as np

from . import bodies, lib, types as T
from .api import RedError


class DiskSpecC(ctypes.Structure):
    """rg_disk_spec_t."""
    _fields_ = [("seed", ctypes.c_uint64), ("n_pl", ctypes.c_int32), ("pl_type", ctypes.c_int32),
                ("n_tp", ctypes.c_int32), ("n_giants", ctypes.c_int32), ("giant_m", ctypes.c_double * 4),
                ("giant_a", ctypes.c_double * 4), ("giant_e", ctypes.c_double * 4), ("m_lo", ctypes.c_double),
                ("m_hi", ctypes.c_double), ("a_lo", ctypes.c_double), ("a_hi", ctypes.c_double),
                ("a_mode", ctypes.c_int32), ("pad", ctypes.c_int32), ("sigma_e", ctypes.c_double),
                ("sigma_i", ctypes.c_double), ("rho_pl", ctypes.c_double)]


@dataclasses.dataclass
class DiskSpec:
    seed: int
    n_pl: int
    pl_type: int = T.BODY_PLANETESIMAL
    n_tp: int = 0
    giants: tuple = ((9.55e-4, 5.2, 0.05), (2.86e-4, 9.54, 0.05))  # (m [Msun], a [AU], e)
    m_range: tuple = (1e-10, 1e-8)
    a_range: tuple = (1.0, 4.0)
    a_mode: int = 0  # 0: Sigma ~ r^-1.5, 1: uniform
    sigma_e: float = 0.01
    sigma_i: float = 0.005
    rho_pl: float = 2.0

    def to_c(self):
        c = DiskSpecC()
        c.seed, c.n_pl, c.pl_type, c.n_tp, c.n_giants = self.seed, self.n_pl, self.pl_type, self.n_tp, len(self.giants)
        for g, (m, a, e) in enumerate(self.giants):
            c.giant_m[g], c.giant_a[g], c.giant_e[g] = m, a, e
        c.m_lo, c.m_hi = self.m_range
        c.a_lo, c.a_hi = self.a_range
        c.a_mode, c.sigma_e, c.sigma_i, c.rho_pl = self.a_mode, self.sigma_e, self.sigma_i, self.rho_pl
        return c

    @property
    def n_total(self):
        return 1 + len(self.giants) + self.n_pl + self.n_tp


def spec_like(config, seed, n=None):
    """The spec of a benchmark configuration (the distributions of bodies.config_disk, drawn
    from this generator's streams instead of numpy's)."""
    if config == "planetesimal_disk":
        return DiskSpec(seed=seed, n_pl=1024 if n is None else n)
    if config == "self_gravitating":
        return DiskSpec(seed=seed, n_pl=16384 if n is None else n, pl_type=T.BODY_PROTOPLANET, giants=(),
                        m_range=(1e-9, 1e-7))
    if config == "ensemble_member":
        rng = np.random.RandomState(1_000_003 + seed)
        n_pl = int(rng.randint(512, 8193)) if n is None else n
        scale = rng.uniform(0.5, 2.0, 2)
        return DiskSpec(seed=seed, n_pl=n_pl, giants=((9.55e-4 * scale[0], 5.2, 0.05), (2.86e-4 * scale[1], 9.54, 0.05)))
    if config == "dense_ring":
        return DiskSpec(seed=seed, n_pl=131072 if n is None else n, pl_type=T.BODY_PROTOPLANET, giants=(),
                        m_range=(1e-11, 1e-9), a_range=(0.9, 1.1), a_mode=1, sigma_e=0.002, sigma_i=0.002)
    raise ValueError(f"unknown config {config!r}")


def _bind(L):
    if getattr(L, "_icgen_bound", False):
        return L
    vp = ctypes.c_void_p
    L.rg_generate_disks.argtypes = [ctypes.c_int, vp, vp, vp, vp, vp, vp]
    L.rg_generate_disks.restype = ctypes.c_int
    L._icgen_bound = True
    return L


def generate_disks(specs):
    """One bodies.Disk per spec, generated on the GPU."""
    L = _bind(lib.load())
    specs = list(specs)
    arr = (DiskSpecC * max(len(specs), 1))(*[s.to_c() for s in specs])
    total = sum(s.n_total for s in specs)
    counts = (T.Counts * max(len(specs), 1))()
    r, v = np.zeros(max(total, 1), T.VEC), np.zeros(max(total, 1), T.VEC)
    p, md = np.zeros(max(total, 1), T.PARAM), np.zeros(max(total, 1), T.BODY_MD)
    vp = ctypes.c_void_p
    rc = L.rg_generate_disks(len(specs), ctypes.cast(arr, vp), ctypes.cast(counts, vp), T.ptr(r), T.ptr(v), T.ptr(p),
                             T.ptr(md))
    if rc:
        raise RedError("rg_generate_disks", rc, L.rg_last_error().decode())
    out, o = [], 0
    for s, spec in enumerate(specs):
        c = counts[s]
        disk = bodies.empty_disk([c.n_s, c.n_gp, c.n_rp, c.n_pp, c.n_spl, c.n_pl, c.n_tp])
        n = spec.n_total
        disk.r[:], disk.v[:], disk.p[:], disk.md[:] = r[o:o + n], v[o:o + n], p[o:o + n], md[o:o + n]
        ng = len(spec.giants)
        disk.names = (["star"] + [f"giant{g}" for g in range(ng)] + [f"pl{q}" for q in range(spec.n_pl)] +
                      [f"tp{q}" for q in range(spec.n_tp)])
        out.append(disk)
        o += n
    return out
