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


# ------------------------------------------------------------------ rg_populate_disks
# The reference's initial-condition program (red.cuda.initial): per body type, one
# distribution per orbital element and physical property (distribution.h, main.cu:29-86).
(DIST_NONE, DIST_UNIFORM, DIST_EXPONENTIAL, DIST_RAYLEIGH, DIST_NORMAL, DIST_POWER_LAW, DIST_LOGNORMAL,
 DIST_LOG_UNIFORM) = range(8)
OE_SMA, OE_ECC, OE_INC, OE_PERI, OE_NODE, OE_MEAN = range(6)
PP_MASS, PP_RADIUS, PP_DENSITY, PP_DRAG_COEFF = range(4)
TYPE_NAMES = ("star", "giant", "rocky", "proto", "superpl", "pl", "testp")  # util_init.cpp:16-29

# unit conversions of the reference's constants (red_constants.h): 1 Msun = 1.98911e33 g,
# 1 AU = 1.495978707e11 m = 215.094 solar radii
SOLAR_RADIUS_AU = 1.0 / 215.094
_GRAM_TO_SOLAR = 1.0 / (1.0e3 * 1.98911e30)
_CM_TO_AU = 1.0e-2 * (1.0 / 1.495978707e11)
GRAM_PER_CM2 = _GRAM_TO_SOLAR / (_CM_TO_AU * _CM_TO_AU)              # g/cm^2 -> Msun/AU^2
GRAM_PER_CM3 = _GRAM_TO_SOLAR / (_CM_TO_AU * _CM_TO_AU * _CM_TO_AU)  # g/cm^3 -> Msun/AU^3


class DistC(ctypes.Structure):
    """rg_dist_t."""
    _fields_ = [("kind", ctypes.c_int32), ("pad", ctypes.c_int32), ("p", ctypes.c_double * 4)]


class BodyDiskC(ctypes.Structure):
    """rg_body_disk_t."""
    _fields_ = [("seed", ctypes.c_uint64), ("n_body", ctypes.c_int32 * 7), ("to_bc", ctypes.c_int32),
                ("pp_total_mass", ctypes.c_double), ("oe", (DistC * 6) * 7), ("pp", (DistC * 4) * 7)]


class MmsnC(ctypes.Structure):
    """rg_mmsn_component_t."""
    _fields_ = [(f, ctypes.c_double) for f in ("r_1", "r_2", "r_SL", "f_neb", "Sigma_1", "f", "p")]


@dataclasses.dataclass(frozen=True)
class Dist:
    """One distribution: `kind` (DIST_*) and its parameters (see rg_dist_t)."""
    kind: int = DIST_NONE
    p: tuple = ()


def uniform(x_min, x_max):
    return Dist(DIST_UNIFORM, (x_min, x_max))


def exponential(lam):
    return Dist(DIST_EXPONENTIAL, (lam,))


def rayleigh(sigma):
    return Dist(DIST_RAYLEIGH, (sigma,))


def normal(mean, scale):
    return Dist(DIST_NORMAL, (mean, scale))


def power_law(x_min, x_max, power):
    return Dist(DIST_POWER_LAW, (x_min, x_max, power))


def lognormal(x_min, x_max, mu, sigma):
    return Dist(DIST_LOGNORMAL, (x_min, x_max, mu, sigma))


def log_uniform(x_min, x_max):
    return Dist(DIST_LOG_UNIFORM, (x_min, x_max))


@dataclasses.dataclass
class BodyDisk:
    """One disk for rg_populate_disks: body counts per type (the reference's order), and per
    type {OE_*: Dist} and {PP_*: Dist}; what is not given is DIST_NONE."""
    seed: int
    n_body: tuple
    oe: dict = dataclasses.field(default_factory=dict)
    pp: dict = dataclasses.field(default_factory=dict)
    pp_total_mass: float = 0.0
    to_bc: bool = False

    def to_c(self):
        c = BodyDiskC()
        c.seed = self.seed
        for t in range(7):
            c.n_body[t] = self.n_body[t]
        c.to_bc = 1 if self.to_bc else 0
        c.pp_total_mass = self.pp_total_mass
        for table, field in ((self.oe, c.oe), (self.pp, c.pp)):
            for t, items in table.items():
                for e, d in items.items():
                    field[t][e].kind = d.kind
                    for q, x in enumerate(d.p):
                        field[t][e].p[q] = x
        return c

    @property
    def n_total(self):
        return int(sum(self.n_body))

    def names(self):
        out = []
        for t, n in enumerate(self.n_body):
            out += ["star"] if (t == 0 and n == 1) else [f"{TYPE_NAMES[t]}{i + 1}" for i in range(n)]
        return out


def _bind_populate(L):
    if getattr(L, "_populate_bound", False):
        return L
    vp = ctypes.c_void_p
    L.rg_populate_disks.argtypes = [ctypes.c_int, vp, vp, vp, vp, vp, vp]
    L.rg_populate_disks.restype = ctypes.c_int
    for f in ("rg_mmsn_gas_mass", "rg_mmsn_solid_mass"):
        getattr(L, f).argtypes = [vp, ctypes.POINTER(ctypes.c_double)]
        getattr(L, f).restype = ctypes.c_int
    L._populate_bound = True
    return L


def populate_disks(disks):
    """One bodies.Disk per BodyDisk, drawn on the GPU (rg_populate_disks)."""
    L = _bind_populate(lib.load())
    disks = list(disks)
    arr = (BodyDiskC * max(len(disks), 1))(*[d.to_c() for d in disks])
    total = sum(d.n_total for d in disks)
    counts = (T.Counts * max(len(disks), 1))()
    r, v = np.zeros(max(total, 1), T.VEC), np.zeros(max(total, 1), T.VEC)
    p, md = np.zeros(max(total, 1), T.PARAM), np.zeros(max(total, 1), T.BODY_MD)
    vp = ctypes.c_void_p
    rc = L.rg_populate_disks(len(disks), ctypes.cast(arr, vp), ctypes.cast(counts, vp), T.ptr(r), T.ptr(v), T.ptr(p),
                             T.ptr(md))
    if rc:
        raise RedError("rg_populate_disks", rc, L.rg_last_error().decode())
    out, o = [], 0
    for d in disks:
        n = d.n_total
        disk = bodies.empty_disk(list(d.n_body))
        disk.r[:], disk.v[:], disk.p[:], disk.md[:] = r[o:o + n], v[o:o + n], p[o:o + n], md[o:o + n]
        disk.names = d.names()
        out.append(disk)
        o += n
    return out


def _mmsn(fn, r_1, r_2, r_SL, f_neb, Sigma_1, f, p):
    L = _bind_populate(lib.load())
    c = MmsnC(r_1, r_2, r_SL, f_neb, Sigma_1, f, p)
    m = ctypes.c_double()
    rc = getattr(L, fn)(ctypes.cast(ctypes.byref(c), ctypes.c_void_p), ctypes.byref(m))
    if rc:
        raise RedError(fn, rc, L.rg_last_error().decode())
    return m.value


def mmsn_gas_mass(r_1, r_2, r_SL, f_neb, Sigma_1, f_gas, p):
    """Gas mass of a minimum-mass solar nebula (rg_mmsn_gas_mass; host arithmetic only)."""
    return _mmsn("rg_mmsn_gas_mass", r_1, r_2, r_SL, f_neb, Sigma_1, f_gas, p)


def mmsn_solid_mass(r_1, r_2, r_SL, f_neb, Sigma_1, f_ice, p):
    """Solid mass of a minimum-mass solar nebula (rg_mmsn_solid_mass; host arithmetic only)."""
    return _mmsn("rg_mmsn_solid_mass", r_1, r_2, r_SL, f_neb, Sigma_1, f_ice, p)


# the reference's "Dvorak disk" (main.cu:88-137, 440-470): a 1 Msun star and protoplanets in
# the solid component of an MMSN with f_neb = 3, Sigma_1 = 7 g/cm^2, the snow line at 2.7 AU
DVORAK_SOLIDS = dict(r_1=0.9, r_2=2.7, r_SL=2.7, f_neb=3.0, Sigma_1=7.0 * GRAM_PER_CM2, f_ice=4.2, p=-1.5)
DVORAK_GAS = dict(r_1=0.025, r_2=33.0, r_SL=2.7, f_neb=3.0, Sigma_1=7.0 * GRAM_PER_CM2, f_gas=240.0, p=-1.5)


def dvorak_disk(seed, n_pp=2000, m_solid=None):
    """The reference's Dvorak disk as a BodyDisk: protoplanets with a ~ a^-1.5 on [0.9, 2.7] AU,
    Rayleigh e (0.01), i = 0, lognormal masses scaled to the nebula's solid mass, basalt
    density (2.7 g/cm^3); moved to the barycentre."""
    if m_solid is None:
        m_solid = mmsn_solid_mass(**DVORAK_SOLIDS)
    s = DVORAK_SOLIDS
    star, proto = T.BODY_STAR, T.BODY_PROTOPLANET
    n_body = [0] * 7
    n_body[star], n_body[proto] = 1, n_pp
    return BodyDisk(
        seed=seed, n_body=tuple(n_body), to_bc=True, pp_total_mass=m_solid,
        pp={star: {PP_MASS: uniform(1.0, 1.0), PP_RADIUS: uniform(SOLAR_RADIUS_AU, SOLAR_RADIUS_AU),
                   PP_DRAG_COEFF: uniform(0.0, 0.0)},
            proto: {PP_MASS: lognormal(0.1, 3.0, 0.0, 0.25), PP_DENSITY: uniform(2.7 * GRAM_PER_CM3, 2.7 * GRAM_PER_CM3),
                    PP_DRAG_COEFF: uniform(0.0, 0.0)}},
        oe={proto: {OE_SMA: power_law(s["r_1"], s["r_2"], s["p"]), OE_ECC: rayleigh(0.01), OE_INC: uniform(0.0, 0.0),
                    OE_PERI: uniform(0.0, 2.0 * np.pi), OE_NODE: uniform(0.0, 0.0),
                    OE_MEAN: uniform(0.0, 2.0 * np.pi)}})


# the other disks of the reference's initial-condition program (main.cu:187-385): a star and
# n bodies of one type on uniform elements; each moved to the barycentre, no mass scaling
_DEG = 1.745329251994329509e-2                 # DegreeToRadian
_JUPITER = 1.0 / 1.0473486e3                   # JupiterToSolar
_CERES = 1.0 / 2.109342e9                      # CeresToSolar
_KM = 1.0 / (1.495978707e11 / 1.0e3)           # KilometerToAu
PRESETS = ("dvorak", "n_gp", "n_pp", "n_spl", "n_pl")
_PRESET_N = {"dvorak": 2000, "n_gp": 10, "n_pp": 1000, "n_spl": 10, "n_pl": 10}


def reference_preset(name, seed, n=None):
    """The BodyDisk of one of the reference's disk set-ups (PRESETS), with n bodies besides the
    star (the reference's own count when None).  Its `n_tp` set-up (mass, radius and density
    all given: the reference refuses it) and its two-body set-up (a radius from 0/0) are not
    offered."""
    n = _PRESET_N[name] if n is None else n
    if name == "dvorak":
        return dvorak_disk(seed, n_pp=n)
    two_pi = 2.0 * np.pi
    star = {PP_MASS: uniform(1.0, 1.0), PP_RADIUS: uniform(SOLAR_RADIUS_AU, SOLAR_RADIUS_AU),
            PP_DRAG_COEFF: uniform(0.0, 0.0)}
    wide = {OE_SMA: uniform(1.0, 10.0), OE_ECC: uniform(0.0, 0.1), OE_INC: uniform(0.0, 10.0 * _DEG),
            OE_PERI: uniform(0.0, two_pi), OE_NODE: uniform(0.0, two_pi), OE_MEAN: uniform(0.0, two_pi)}
    if name == "n_gp":
        t, oe = T.BODY_GIANTPLANET, wide
        pp = {PP_MASS: uniform(0.1 * _JUPITER, 1.0 * _JUPITER), PP_DENSITY: uniform(1.0 * GRAM_PER_CM3, 2.0 * GRAM_PER_CM3),
              PP_DRAG_COEFF: uniform(0.0, 0.0)}
    elif name == "n_pp":
        t = T.BODY_PROTOPLANET
        oe = {OE_SMA: uniform(100.0, 100.0001), OE_ECC: uniform(0.0, 0.01), OE_INC: uniform(0.0, 0.0),
              OE_PERI: uniform(0.0, two_pi), OE_NODE: uniform(0.0, 0.0), OE_MEAN: uniform(0.0, two_pi)}
        pp = {PP_RADIUS: uniform(1.0e3 * _KM, 1.0e3 * _KM), PP_DENSITY: uniform(2.7 * GRAM_PER_CM3, 2.7 * GRAM_PER_CM3),
              PP_DRAG_COEFF: uniform(0.0, 0.0)}
    elif name == "n_spl":
        t, oe = T.BODY_SUPERPLANETESIMAL, wide
        pp = {PP_MASS: uniform(1.0e-10, 1.0e-9), PP_RADIUS: uniform(10.0 * _KM, 30.0 * _KM),
              PP_DENSITY: uniform(1.0 * GRAM_PER_CM3, 3.0 * GRAM_PER_CM3), PP_DRAG_COEFF: uniform(1.0, 2.7)}
    elif name == "n_pl":
        t, oe = T.BODY_PLANETESIMAL, wide
        pp = {PP_MASS: uniform(1.0e-3 * _CERES, 1.0e-2 * _CERES),
              PP_DENSITY: uniform(1.0 * GRAM_PER_CM3, 3.0 * GRAM_PER_CM3), PP_DRAG_COEFF: uniform(0.0, 0.0)}
    else:
        raise ValueError(f"unknown disk set-up {name!r}; one of {PRESETS}")
    n_body = [0] * 7
    n_body[T.BODY_STAR], n_body[t] = 1, n
    return BodyDisk(seed=seed, n_body=tuple(n_body), to_bc=True, pp={T.BODY_STAR: star, t: pp}, oe={t: oe})
