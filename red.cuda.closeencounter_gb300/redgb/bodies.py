"""Body lists: the reference's text format and seeded synthetic planetesimal disks.

File format: the body-list file read by pp_disk::get_number_of_bodies / load /
read_body_record (red.cuda/src/red.cuda/pp_disk.cu:1307-1322,1576-1683): a header line
with the seven counts (stars, giants, rocky planets, protoplanets, super-planetesimals,
planetesimals, test particles), then one record per body
``id name type epoch mass radius density cd mig_type mig_stop_at x y z vx vy vz``
in AU, solar masses, days and AU/day.  Numbers are written with 17 significant digits so
that a file round-trips bit-exactly through the reference's iostream parser.

Synthetic disks: orbital elements are drawn with numpy's MT19937 (RandomState) and turned
into positions and velocities by the reference's element-to-phase conversion
(red.cuda/src/red.cuda.utility/tools.cpp:292-359, restated here), with mu = k^2 (M* + m).
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

from . import types as T

# red.cuda/red.type/red_constants.h: GramPerCm3ToSolarPerAu3
_SOLAR_TO_GRAM = 1.0e3 * 1.98911e30
_METER_TO_AU = 1.0 / 1.495978707e11
GRAM_PER_CM3_TO_SOLAR_PER_AU3 = (1.0 / _SOLAR_TO_GRAM) / (1.0e-2 * _METER_TO_AU) ** 3
FOUR_PI_OVER_THREE = 4.1887902047863909846168578443727


@dataclasses.dataclass
class Disk:
    """One body list in the reference's storage order (SI, NSI, NI blocks)."""
    counts: tuple  # (n_s, n_gp, n_rp, n_pp, n_spl, n_pl, n_tp)
    r: np.ndarray  # VEC[n], AU
    v: np.ndarray  # VEC[n], AU/day
    p: np.ndarray  # PARAM[n]
    md: np.ndarray  # BODY_MD[n]
    epoch: np.ndarray  # f8[n], day
    names: list

    @property
    def n_total(self):
        return int(sum(self.counts))

    @property
    def n_si(self):
        return int(sum(self.counts[:4]))

    @property
    def n_massive(self):
        return int(sum(self.counts[:6]))

    def counts_struct(self):
        return T.Counts(*self.counts)

    def copy(self):
        return Disk(tuple(self.counts), self.r.copy(), self.v.copy(), self.p.copy(), self.md.copy(),
                    self.epoch.copy(), list(self.names))

    def pairs_per_eval(self):
        """Interacting (sink, source) pairs of one force evaluation, all bodies active
        (number_of_bodies.cpp:196-258: SI x massive, NSI x SI, NI x massive, minus i == j)."""
        nsi, nm, nt = self.n_si, self.n_massive, self.n_total
        nnsi, nni = nm - nsi, nt - nm
        return nsi * (nm - 1) + nnsi * nsi + nni * nm


def empty_disk(counts):
    n = int(sum(counts))
    return Disk(tuple(int(c) for c in counts), np.zeros(n, T.VEC), np.zeros(n, T.VEC), np.zeros(n, T.PARAM),
                np.zeros(n, T.BODY_MD), np.zeros(n, np.float64), [f"b{i}" for i in range(n)])


def _fmt(x):
    return repr(float(x))


def write_body_file(path, disk: Disk):
    """Write a body list in the reference's input format (pp_disk.cu:1576-1612)."""
    with open(path, "w") as f:
        f.write(" ".join(str(int(c)) for c in disk.counts) + "\n")
        for i in range(disk.n_total):
            r, v, p, md = disk.r[i], disk.v[i], disk.p[i], disk.md[i]
            name = disk.names[i][:30].replace(" ", "_")
            f.write(" ".join([str(int(md["id"])), name, str(int(md["body_type"])), _fmt(disk.epoch[i]),
                              _fmt(p["mass"]), _fmt(p["radius"]), _fmt(p["density"]), _fmt(p["cd"]),
                              str(int(md["mig_type"])), _fmt(md["mig_stop_at"]),
                              _fmt(r["x"]), _fmt(r["y"]), _fmt(r["z"]),
                              _fmt(v["x"]), _fmt(v["y"]), _fmt(v["z"])]) + "\n")


def read_body_file(path) -> Disk:
    """Read a body list in the reference's input format (pp_disk.cu:1307-1322,1576-1683)."""
    with open(path) as f:
        tokens = f.read().split()
    counts = tuple(int(t) for t in tokens[:7])
    disk = empty_disk(counts)
    k = 7
    for i in range(disk.n_total):
        rec = tokens[k:k + 16]
        if len(rec) < 16:
            raise ValueError(f"{path}: truncated record {i}")
        k += 16
        disk.md[i]["id"] = int(rec[0])
        disk.names[i] = rec[1][:30]
        disk.md[i]["body_type"] = int(rec[2])
        disk.epoch[i] = float(rec[3])
        disk.p[i] = (float(rec[4]), float(rec[5]), float(rec[6]), float(rec[7]))
        disk.md[i]["mig_type"] = int(rec[8])
        disk.md[i]["mig_stop_at"] = float(rec[9])
        disk.r[i] = (float(rec[10]), float(rec[11]), float(rec[12]), 0.0)
        disk.v[i] = (float(rec[13]), float(rec[14]), float(rec[15]), 0.0)
    return disk


def write_parameter_file(path, *, integrator="rkf8", tolerance=None, length_yr=1.0, output_interval_yr=None,
                         ejection=None, hit_centrum=None, collision_factor=None, error_check_for_tp=False,
                         close_encounter=False, name="synthetic", output_type=None, frame_center="bary"):
    """key = value parameter file read by parameter::parse (parameter.cpp:55-285)."""
    lines = [f"name = {name}", "description = seeded synthetic disk", f"frame_center = {frame_center}",
             f"integrator = {integrator}"]
    if tolerance is not None:
        lines.append(f"tolerance = {tolerance!r}")
    lines.append(f"error_check_for_tp = {'true' if error_check_for_tp else 'false'}")
    if close_encounter:
        lines.append("close_encounter = true")
    lines += ["start_time = 0.0", f"length = {length_yr!r}",
              f"output_interval = {output_interval_yr if output_interval_yr is not None else length_yr!r}"]
    if ejection is not None:
        lines.append(f"ejection = {ejection!r}")
    if hit_centrum is not None:
        lines.append(f"hit_centrum = {hit_centrum!r}")
    if collision_factor is not None:
        lines.append(f"collision_factor = {collision_factor!r}")
    if output_type is not None:  # "text" or "binary" (parameter.cpp:242-256)
        lines.append(f"output_type = {output_type}")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


# ---------------------------------------------------------------------- orbital elements

def kepler_equation_solver(ecc, mean, eps=1.0e-14):
    """tools.cpp:292-315."""
    if ecc == 0.0 or mean == 0.0 or mean == math.pi:
        return mean
    E = mean + ecc * math.sin(mean) / (1.0 - math.sin(mean + ecc) + math.sin(mean))
    step = 0
    while True:
        E1 = E - (E - ecc * math.sin(E) - mean) / (1.0 - ecc * math.cos(E))
        error = abs(E1 - E)
        E = E1
        cont = error > eps
        if cont:
            cont = step <= 15
            step += 1
        if not cont:
            break
    return E


def calculate_phase(mu, sma, ecc, inc, peri, node, mean):
    """tools.cpp:317-359: orbital elements -> position and velocity."""
    E = kepler_equation_solver(ecc, mean, 1.0e-14)
    v = 2.0 * math.atan(math.sqrt((1.0 + ecc) / (1.0 - ecc)) * math.tan(E / 2.0))
    p = sma * (1.0 - ecc * ecc)
    r = p / (1.0 + ecc * math.cos(v))
    kszi, eta = r * math.cos(v), r * math.sin(v)
    vkszi = -math.sqrt(mu / p) * math.sin(v)
    veta = math.sqrt(mu / p) * (ecc + math.cos(v))
    cw, sw = math.cos(peri), math.sin(peri)
    cO, sO = math.cos(node), math.sin(node)
    ci, si = math.cos(inc), math.sin(inc)
    P = (cw * cO - sw * sO * ci, cw * sO + sw * cO * ci, sw * si)
    Q = (-sw * cO - cw * sO * ci, -sw * sO + cw * cO * ci, cw * si)
    rv = tuple(kszi * P[k] + eta * Q[k] for k in range(3))
    vv = tuple(vkszi * P[k] + veta * Q[k] for k in range(3))
    return rv, vv


def radius_from_density(m, rho_gcc):
    """tools.cpp:238-243 calculate_radius with the density in g/cm^3."""
    rho = rho_gcc * GRAM_PER_CM3_TO_SOLAR_PER_AU3
    return (1.0 / FOUR_PI_OVER_THREE * m / rho) ** (1.0 / 3.0), rho


# ---------------------------------------------------------------------- disk recipes

STAR_RADIUS_AU = 0.004649130148  # TestRun/InputTest body lists
STAR_DENSITY = 2375725.607


def make_disk(*, n_pl, pl_type=T.BODY_PLANETESIMAL, seed=0, giants=((9.55e-4, 5.2, 0.05), (2.86e-4, 9.54, 0.05)),
              giant_scale=(1.0, 1.0), embryos=(), m_range=(1e-10, 1e-8), a_mode="sigma", a_range=(1.0, 4.0),
              sigma_e=0.01, sigma_i=0.005, rho_pl=2.0, n_tp=0):
    """A star, giant planets, optional embryos and a planetesimal swarm.

    Masses log-uniform in m_range, radii from density rho_pl g/cm^3, semi-major axes either
    from a surface density Sigma ~ r^-1.5 on a_range (dN/da ~ a^-0.5, a_mode="sigma") or
    uniform (a_mode="uniform"); e and i Rayleigh(sigma_e / sigma_i); angles uniform.
    pl_type 5 gives the reference's non-self-interacting planetesimals, 3 (protoplanet)
    makes every body self-gravitating.  The star sits at rest in the origin, so creating a
    system moves it to the barycentre exactly as the reference does (options.cpp:206).
    """
    rng = np.random.RandomState(seed)
    n_gp = len(giants)
    n_emb = len(embryos)
    si_pl = pl_type <= T.BODY_PROTOPLANET
    counts = [1, n_gp, 0, n_emb + (n_pl if si_pl else 0), 0, 0 if si_pl else n_pl, n_tp]
    if pl_type == T.BODY_SUPERPLANETESIMAL:
        counts[4], counts[5] = n_pl, 0
    disk = empty_disk(counts)
    m_star = 1.0
    disk.p[0] = (m_star, STAR_RADIUS_AU, STAR_DENSITY, 0.0)
    disk.md[0] = (1, T.BODY_STAR, 0, 0.0)
    disk.names[0] = "star"
    k = 1
    for g, (m, a, e) in enumerate(giants):
        m = m * giant_scale[g]
        R, rho = radius_from_density(m, 1.33)
        mean = rng.uniform(0.0, 2.0 * math.pi)
        peri = rng.uniform(0.0, 2.0 * math.pi)
        rv, vv = calculate_phase(T.GAUSS2 * (m_star + m), a, e, 0.0, peri, 0.0, mean)
        disk.p[k] = (m, R, rho, 0.0)
        disk.md[k] = (k + 1, T.BODY_GIANTPLANET, 0, 0.0)
        disk.r[k] = rv + (0.0,)
        disk.v[k] = vv + (0.0,)
        disk.names[k] = f"giant{g}"
        k += 1
    for q, (m, a, e) in enumerate(embryos):
        R, rho = radius_from_density(m, 3.0)
        mean = rng.uniform(0.0, 2.0 * math.pi)
        rv, vv = calculate_phase(T.GAUSS2 * (m_star + m), a, e, 0.0, 0.0, 0.0, mean)
        disk.p[k] = (m, R, rho, 0.0)
        disk.md[k] = (k + 1, T.BODY_PROTOPLANET, 0, 0.0)
        disk.r[k] = rv + (0.0,)
        disk.v[k] = vv + (0.0,)
        disk.names[k] = f"embryo{q}"
        k += 1
    lo, hi = math.log(m_range[0]), math.log(m_range[1])
    m = np.exp(rng.uniform(lo, hi, n_pl))
    u = rng.uniform(0.0, 1.0, n_pl)
    if a_mode == "sigma":
        s0, s1 = math.sqrt(a_range[0]), math.sqrt(a_range[1])
        a = (s0 + u * (s1 - s0)) ** 2
    else:
        a = a_range[0] + u * (a_range[1] - a_range[0])
    e = np.minimum(rng.rayleigh(sigma_e, n_pl), 0.9)
    inc = rng.rayleigh(sigma_i, n_pl)
    ang = rng.uniform(0.0, 2.0 * math.pi, (n_pl, 3))
    ptype = pl_type
    for q in range(n_pl):
        R, rho = radius_from_density(m[q], rho_pl)
        rv, vv = calculate_phase(T.GAUSS2 * (m_star + m[q]), a[q], e[q], inc[q], ang[q, 0], ang[q, 1], ang[q, 2])
        disk.p[k] = (m[q], R, rho, 0.0)
        disk.md[k] = (k + 1, ptype, 0, 0.0)
        disk.r[k] = rv + (0.0,)
        disk.v[k] = vv + (0.0,)
        disk.names[k] = f"pl{q}"
        k += 1
    for q in range(n_tp):
        aa = rng.uniform(a_range[0], a_range[1])
        rv, vv = calculate_phase(T.GAUSS2 * m_star, aa, rng.rayleigh(sigma_e), rng.rayleigh(sigma_i),
                                 *rng.uniform(0.0, 2.0 * math.pi, 3))
        disk.md[k] = (k + 1, T.BODY_TESTPARTICLE, 0, 0.0)
        disk.r[k] = rv + (0.0,)
        disk.v[k] = vv + (0.0,)
        disk.names[k] = f"tp{q}"
        k += 1
    assert k == disk.n_total
    return disk


def config_disk(config, seed=None, n=None):
    """The seeded synthetic disks of the benchmark workloads.

    planetesimal_disk   1 Msun star, giants 9.55e-4 Msun at 5.2 AU and 2.86e-4 Msun at
                        9.54 AU (e = 0.05, i = 0), 1024 planetesimals m in [1e-10, 1e-8],
                        rho 2 g/cm^3, Sigma ~ r^-1.5 on [1, 4] AU, e ~ R(0.01), i ~ R(0.005).
    self_gravitating    the same swarm with 16384 self-gravitating bodies (type 3),
                        m in [1e-9, 1e-7], star only.
    ensemble_member     planetesimal_disk with its own seed, N ~ U[512, 8192] and giant
                        masses scaled by U[0.5, 2].
    dense_ring          1 Msun star + one 3e-6 Msun embryo at 1 AU + 131072 self-gravitating
                        bodies, a ~ U[0.9, 1.1], e, i ~ R(0.002), m in [1e-11, 1e-9].
    """
    if config == "planetesimal_disk":
        return make_disk(n_pl=1024 if n is None else n, seed=0 if seed is None else seed)
    if config == "self_gravitating":
        return make_disk(n_pl=16384 if n is None else n, pl_type=T.BODY_PROTOPLANET, giants=(),
                         m_range=(1e-9, 1e-7), seed=0 if seed is None else seed)
    if config == "ensemble_member":
        seed = 1 if seed is None else seed
        rng = np.random.RandomState(1_000_003 + seed)
        n_pl = int(rng.randint(512, 8193)) if n is None else n
        scale = tuple(rng.uniform(0.5, 2.0, 2))
        return make_disk(n_pl=n_pl, seed=seed, giant_scale=scale)
    if config == "dense_ring":
        return make_disk(n_pl=131072 if n is None else n, pl_type=T.BODY_PROTOPLANET, giants=(),
                         embryos=((3e-6, 1.0, 0.0),), m_range=(1e-11, 1e-9), a_mode="uniform",
                         a_range=(0.9, 1.1), sigma_e=0.002, sigma_i=0.002, seed=0 if seed is None else seed)
    raise ValueError(f"unknown config {config!r}")


def thresholds(ejection=100.0, hit_centrum=0.05, collision_factor=1.0):
    """The five threshold_t values (red_type.h:46-54; parameter.cpp:216-241)."""
    return np.array([hit_centrum, ejection, collision_factor, hit_centrum * hit_centrum, ejection * ejection],
                    np.float64)
