"""Test infrastructure: a numpy restatement of the GPU disk generator (rg_generate_disks,
csrc/icgen.cu), used only by the tests as the checker.

Same Philox4x32-10 streams (Salmon, Moraes, Dror & Shaw, SC 2011: ten rounds, multipliers
0xD2511F53 / 0xCD9E8D57, key bumps 0x9E3779B9 / 0xBB67AE85; key = the disk's seed, counter =
(body slot, draw block, 0, 0)), the same 53-bit uniforms and transforms, and the reference's
Kepler solver and calculate_phase (tools.cpp:292-359), vectorised.  numpy's transcendental
functions may round differently from the GPU's in the last bit, so the tests compare with a
small tolerance; the random streams themselves are compared exactly (through the masses'
uniforms and the body order).
"""
import math

import numpy as np

MASK = np.uint64(0xFFFFFFFF)
GAUSS2 = 2.959122082855911025e-4
FOUR_PI_OVER_THREE = 4.1887902047863909846168578443727
STAR_RADIUS = 0.004649130148
STAR_DENSITY = 2375725.607
GRAM_CC = (1.0 / (1.0e3 * 1.98911e30)) / math.pow(1.0e-2 * (1.0 / 1.495978707e11), 3.0)


def philox4x32_10(c0, c1, c2, c3, k0, k1):
    c = [np.asarray(x, np.uint64) & MASK for x in (c0, c1, c2, c3)]
    k0, k1 = np.uint64(k0) & MASK, np.uint64(k1) & MASK
    for r in range(10):
        if r > 0:
            k0 = (k0 + np.uint64(0x9E3779B9)) & MASK
            k1 = (k1 + np.uint64(0xBB67AE85)) & MASK
        p0 = np.uint64(0xD2511F53) * c[0]
        p1 = np.uint64(0xCD9E8D57) * c[2]
        hi0, lo0 = p0 >> np.uint64(32), p0 & MASK
        hi1, lo1 = p1 >> np.uint64(32), p1 & MASK
        c = [hi1 ^ c[1] ^ k0, lo1, hi0 ^ c[3] ^ k1, lo0]
    return c


def uniform53(a, b):
    return ((a >> np.uint64(5)).astype(np.float64) * 67108864.0 + (b >> np.uint64(6)).astype(np.float64)) * \
        (1.0 / 9007199254740992.0)


def draw2(seed, k, blk):
    k = np.asarray(k, np.uint64)
    c = philox4x32_10(k, np.full_like(k, blk), np.zeros_like(k), np.zeros_like(k), seed & 0xFFFFFFFF, seed >> 32)
    return uniform53(c[0], c[1]), uniform53(c[2], c[3])


def kepler(ecc, mean, eps=1.0e-14):
    """tools.cpp:292-315, element-wise."""
    ecc, mean = np.asarray(ecc, np.float64), np.asarray(mean, np.float64)
    E = mean + ecc * np.sin(mean) / (1.0 - np.sin(mean + ecc) + np.sin(mean))
    special = (ecc == 0.0) | (mean == 0.0) | (mean == math.pi)
    active = ~special
    step = np.zeros(E.shape, np.int64)
    while active.any():
        E1 = E - (E - ecc * np.sin(E) - mean) / (1.0 - ecc * np.cos(E))
        error = np.abs(E1 - E)
        E = np.where(active, E1, E)
        cont = active & (error > eps)
        active = cont & (step <= 15)
        step = np.where(cont, step + 1, step)
    return np.where(special, mean, E)


def calculate_phase(mu, sma, ecc, inc, peri, node, mean):
    """tools.cpp:317-359, element-wise: (r [n, 3], v [n, 3])."""
    E = kepler(ecc, mean)
    nu = 2.0 * np.arctan(np.sqrt((1.0 + ecc) / (1.0 - ecc)) * np.tan(E / 2.0))
    p = sma * (1.0 - ecc * ecc)
    rr = p / (1.0 + ecc * np.cos(nu))
    kszi, eta = rr * np.cos(nu), rr * np.sin(nu)
    vkszi = -np.sqrt(mu / p) * np.sin(nu)
    veta = np.sqrt(mu / p) * (ecc + np.cos(nu))
    cw, sw, cO, sO, ci, si = np.cos(peri), np.sin(peri), np.cos(node), np.sin(node), np.cos(inc), np.sin(inc)
    P = np.stack([cw * cO - sw * sO * ci, cw * sO + sw * cO * ci, sw * si], 1)
    Q = np.stack([-sw * cO - cw * sO * ci, -sw * sO + cw * cO * ci, cw * si], 1)
    return kszi[:, None] * P + eta[:, None] * Q, vkszi[:, None] * P + veta[:, None] * Q


def radius_of(m, rho):
    return np.power(1.0 / FOUR_PI_OVER_THREE * m / rho, 1.0 / 3.0)


def generate(spec):
    """(r [n, 3], v [n, 3], mass, radius, density, body type) of one DiskSpec."""
    ng, npl, ntp = len(spec.giants), spec.n_pl, spec.n_tp
    n = 1 + ng + npl + ntp
    r, v = np.zeros((n, 3)), np.zeros((n, 3))
    m, R, rho, typ = np.zeros(n), np.zeros(n), np.zeros(n), np.zeros(n, np.int32)
    m[0], R[0], rho[0] = 1.0, STAR_RADIUS, STAR_DENSITY
    if ng:
        k = np.arange(1, 1 + ng)
        um, uw = draw2(spec.seed, k, 0)
        gm = np.array([g[0] for g in spec.giants]); ga = np.array([g[1] for g in spec.giants])
        ge = np.array([g[2] for g in spec.giants])
        r[k], v[k] = calculate_phase(GAUSS2 * (1.0 + gm), ga, ge, np.zeros(ng), 2.0 * math.pi * uw, np.zeros(ng),
                                     2.0 * math.pi * um)
        m[k], rho[k] = gm, 1.33 * GRAM_CC
        R[k] = radius_of(gm, rho[k])
        typ[k] = 1
    if npl:
        k = np.arange(1 + ng, 1 + ng + npl)
        um, ua = draw2(spec.seed, k, 0)
        ue, ui = draw2(spec.seed, k, 1)
        uw, uO = draw2(spec.seed, k, 2)
        uM, _ = draw2(spec.seed, k, 3)
        lo, hi = math.log(spec.m_range[0]), math.log(spec.m_range[1])
        mm = np.exp(lo + um * (hi - lo))
        if spec.a_mode == 0:
            s0, s1 = math.sqrt(spec.a_range[0]), math.sqrt(spec.a_range[1])
            x = s0 + ua * (s1 - s0)
            sma = x * x
        else:
            sma = spec.a_range[0] + ua * (spec.a_range[1] - spec.a_range[0])
        ecc = np.minimum(spec.sigma_e * np.sqrt(-2.0 * np.log(1.0 - ue)), 0.9)
        inc = spec.sigma_i * np.sqrt(-2.0 * np.log(1.0 - ui))
        r[k], v[k] = calculate_phase(GAUSS2 * (1.0 + mm), sma, ecc, inc, 2.0 * math.pi * uw, 2.0 * math.pi * uO,
                                     2.0 * math.pi * uM)
        m[k], rho[k] = mm, spec.rho_pl * GRAM_CC
        R[k] = radius_of(mm, rho[k])
        typ[k] = spec.pl_type
    if ntp:
        k = np.arange(1 + ng + npl, n)
        ua, ue = draw2(spec.seed, k, 0)
        ui, uw = draw2(spec.seed, k, 1)
        uO, uM = draw2(spec.seed, k, 2)
        sma = spec.a_range[0] + ua * (spec.a_range[1] - spec.a_range[0])
        ecc = np.minimum(spec.sigma_e * np.sqrt(-2.0 * np.log(1.0 - ue)), 0.9)
        inc = spec.sigma_i * np.sqrt(-2.0 * np.log(1.0 - ui))
        r[k], v[k] = calculate_phase(np.full(ntp, GAUSS2), sma, ecc, inc, 2.0 * math.pi * uw, 2.0 * math.pi * uO,
                                     2.0 * math.pi * uM)
        typ[k] = 6
    return r, v, m, R, rho, typ


# ------------------------------------------------------------------ rg_populate_disks
# Restatement of the GPU populate steps (csrc/icgen.cu), which follow the reference's
# red.cuda.initial: populate_disk (main.cu:29-86), the mass scaling and re-derivation
# (main.cu:472-509), the phases (main.cu:511-536) and tools::transform_to_bc
# (tools.cpp:122-176).  Distributions: distribution.cpp:117-249, the lognormal density
# sampled by its inverse distribution function and the power law by the reference's own
# rejection steps.
POP_ITEM0 = 16
(DIST_NONE, DIST_UNIFORM, DIST_EXPONENTIAL, DIST_RAYLEIGH, DIST_NORMAL, DIST_POWER_LAW, DIST_LOGNORMAL,
 DIST_LOG_UNIFORM) = range(8)
BODY_STAR, BODY_PROTOPLANET, BODY_SUPERPLANETESIMAL = 0, 3, 4


def draw2a(seed, k, blk, att):
    """draw2 with the attempt counter (attempt 0 is draw2)."""
    k = np.asarray(k, np.uint64)
    c = philox4x32_10(k, np.full_like(k, blk), np.full_like(k, att), np.zeros_like(k), seed & 0xFFFFFFFF, seed >> 32)
    return uniform53(c[0], c[1]), uniform53(c[2], c[3])


def sample_dist(kind, p, seed, k, blk):
    """One value per body slot k from draw block blk (see csrc/icgen.cu sample_dist)."""
    from scipy.special import ndtr, ndtri
    u0, u1 = draw2(seed, k, blk)
    u = 1.0 - u0
    if kind == DIST_UNIFORM:
        return p[0] + (p[1] - p[0]) * u
    if kind == DIST_EXPONENTIAL:
        return -1.0 / p[0] * np.log(u)
    if kind == DIST_RAYLEIGH:
        return p[0] * np.sqrt(-2.0 * np.log(u))
    if kind == DIST_NORMAL:
        return p[0] + p[1] * np.sqrt(-2.0 * np.log(u)) * np.cos(2.0 * math.pi * (1.0 - u1))
    if kind == DIST_POWER_LAW:  # the reference's rejection steps (distribution.cpp:187-207)
        x0, x1, pw = p[0], p[1], p[2]
        y_min = 0.0 if pw == 0.0 else math.pow(x0, pw)
        y_max = 1.0 if pw == 0.0 else math.pow(x1, pw)
        y_min, y_max = min(y_min, y_max), max(y_min, y_max)
        d_y, d_x = y_max - y_min, x1 - x0
        area_max = d_x * d_y
        k = np.asarray(k)
        if not d_y > 0.0:
            return np.full(k.shape, x0)
        out = np.full(k.shape, np.nan)
        todo = np.ones(k.shape, bool)
        for att in range(10000):
            if att > 0:
                u0, u1 = draw2a(seed, k, blk, att)
            x = area_max * (1.0 - u0) / d_y + x0
            y = y_min + (y_max - y_min) * (1.0 - u1)
            ok = todo & ~(y > np.power(x, pw))
            out[ok] = x[ok]
            todo &= ~ok
            if not todo.any():
                return out
        raise ValueError("a power-law draw reached its attempt limit")
    if kind == DIST_LOGNORMAL:
        x0, x1, mu, sg = p
        c0 = ndtr((math.log(x0) - mu) / sg) if x0 > 0 else 0.0
        c1 = ndtr((math.log(x1) - mu) / sg)
        x = np.exp(mu + sg * ndtri(c0 + u0 * (c1 - c0)))
        return np.minimum(np.maximum(x, x0), x1)
    if kind == DIST_LOG_UNIFORM:
        return np.exp(math.log(p[0]) + u0 * (math.log(p[1]) - math.log(p[0])))
    return np.zeros_like(u0)


def density_of(m, R):
    """tools.cpp:245-254."""
    R = np.asarray(R, np.float64)
    with np.errstate(divide="ignore", invalid="ignore"):
        return np.where(R == 0.0, 0.0, m / (FOUR_PI_OVER_THREE * (R * R * R)))


def mass_of(R, rho):
    """tools.cpp:256-261."""
    return FOUR_PI_OVER_THREE * (R * R * R) * rho


def _protoplanet_mass(m, typ):
    tot = 0.0
    for j in range(len(m) - 1, -1, -1):  # tools::get_total_mass: from the last body down
        if typ[j] == BODY_PROTOPLANET:
            tot += float(m[j])
    return tot


def populate(disk):
    """(r [n, 3], v [n, 3], mass, radius, density, cd, body type) of one BodyDisk (redgb.icgen);
    raises ValueError where rg_populate_disks returns RG_ERR_ARG after drawing."""
    n_body = list(disk.n_body)
    n = int(sum(n_body))
    typ = np.repeat(np.arange(7, dtype=np.int32), n_body)
    k = np.arange(n)
    pp = np.zeros((n, 4))
    oe = np.zeros((n, 6))
    for t in range(7):
        idx = k[typ == t]
        if idx.size == 0:
            continue
        items = disk.pp.get(t, {})
        for e in range(4):
            d = items.get(e)
            if d is not None and d.kind != DIST_NONE:
                pp[idx, e] = sample_dist(d.kind, d.p, disk.seed, idx, POP_ITEM0 + e)
        if t != BODY_SUPERPLANETESIMAL:
            hm, hr, hd = (items.get(e) is not None and items[e].kind != DIST_NONE for e in range(3))
            if not hm and hr and hd:
                pp[idx, 0] = mass_of(pp[idx, 1], pp[idx, 2])
            elif not hr and hm and hd:
                pp[idx, 1] = radius_of(pp[idx, 0], pp[idx, 2])
            elif not hd and hm and hr:
                pp[idx, 2] = density_of(pp[idx, 0], pp[idx, 1])
        if t != BODY_STAR:
            for e in range(6):
                d = disk.oe.get(t, {}).get(e)
                if d is not None and d.kind != DIST_NONE:
                    oe[idx, e] = sample_dist(d.kind, d.p, disk.seed, idx, POP_ITEM0 + 4 + e)
    m = pp[:, 0]
    if disk.pp_total_mass > 0.0:
        f = disk.pp_total_mass / _protoplanet_mass(m, typ)
        m[typ == BODY_PROTOPLANET] *= f
        if abs(_protoplanet_mass(m, typ) - disk.pp_total_mass) > 1.0e-15:
            raise ValueError("the required mass was not reached")
        for t in range(7):
            sel = (typ == t) & (m > 0.0)
            items = disk.pp.get(t, {})
            hr = items.get(1) is not None and items[1].kind != DIST_NONE
            hd = items.get(2) is not None and items[2].kind != DIST_NONE
            if not hd and hr:
                pp[sel, 2] = density_of(m[sel], pp[sel, 1])
            if not hr and hd:
                pp[sel, 1] = radius_of(m[sel], pp[sel, 2])
    r, v = np.zeros((n, 3)), np.zeros((n, 3))
    if n > 1:
        mu = GAUSS2 * (m[0] + m[1:])
        r[1:], v[1:] = calculate_phase(mu, *(oe[1:, e] for e in range(6)))
    if disk.to_bc:
        R0, V0, M0 = [0.0, 0.0, 0.0], [0.0, 0.0, 0.0], 0.0
        for j in range(n - 1, -1, -1):  # compute_bc: from the last body down
            mj = float(m[j])
            for c in range(3):
                R0[c] += mj * float(r[j, c])
                V0[c] += mj * float(v[j, c])
        for j in range(n - 1, -1, -1):
            M0 += float(m[j])
        r -= np.array([x / M0 for x in R0])
        v -= np.array([x / M0 for x in V0])
    return r, v, m, pp[:, 1], pp[:, 2], pp[:, 3], typ


def mmsn_gas(r_1, r_2, r_SL, f_neb, Sigma_1, f_gas, p):
    """nebula.cpp:23-46."""
    p2 = p + 2.0
    if p2 != 0.0:
        return 2.0 * math.pi * f_neb * f_gas * Sigma_1 / p2 * (math.pow(r_2, p2) - math.pow(r_1, p2))
    return 2.0 * math.pi * f_neb * f_gas * Sigma_1 * (math.log(r_2) - math.log(r_1))


def mmsn_solid(r_1, r_2, r_SL, f_neb, Sigma_1, f_ice, p):
    """nebula.cpp:63-95."""
    p2 = p + 2.0
    C = 2.0 * math.pi * f_neb * Sigma_1 / p2 if p2 != 0.0 else 2.0 * math.pi * f_neb * Sigma_1

    def integral(a, b):
        return math.pow(b, p2) - math.pow(a, p2) if p2 != 0.0 else math.log(b) - math.log(a)

    if r_SL <= r_1:
        I = f_ice * integral(r_1, r_2)
    elif r_SL <= r_2:
        I = integral(r_1, r_SL) + f_ice * integral(r_SL, r_2)
    else:
        I = integral(r_1, r_2)
    return C * I
