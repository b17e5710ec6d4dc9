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
