"""The mixed kernel's per-slice flag cutoff (flag_cut2 in csrc/gravity_mixed.cu), restated in
IEEE float32 with numpy, and the property the pair loop relies on: a pair whose FP32 r^2 is
at or above the cutoff is not a near pair (m_j > fl(near_lim * r^2) is false for every source
of the slice, m_j <= the slice's largest mass), not a self pair (r^2 = 0) and not a screen
candidate (r^2 < cut2) -- so skipping its exact classification loses nothing.

The device code multiplies and compares without contraction (no add follows a multiply), and
numpy float32 arithmetic rounds to nearest even like the GPU's FP32 multiply and divide.
"""
import numpy as np

F = np.float32
FLT_MIN = F(1.17549435e-38)


def flag_cut2(mslice, near_lim, cut2):
    """The device function, operation by operation (float32 throughout)."""
    with np.errstate(over="ignore", under="ignore", invalid="ignore", divide="ignore"):
        inv = F(1.0) / near_lim
        c = np.where(mslice > 0, (mslice * inv) * F(1.0001), F(0.0)).astype(F)
        c = np.maximum(np.maximum(c, cut2), FLT_MIN).astype(F)
        ok = (near_lim * c) >= mslice
        return np.where(ok, c, F(3.0e38)).astype(F)


def _cases(rng, n):
    # masses and near limits over the ranges the kernel sees (Msun, 1/AU^2 scales), plus the
    # no-scale limit 3e38 of a tile without a heavy source
    mslice = (10.0 ** rng.uniform(-14, 0, n)).astype(F)
    mslice[rng.random(n) < 0.05] = F(0.0)
    near_lim = (10.0 ** rng.uniform(-12, 8, n)).astype(F)
    near_lim[rng.random(n) < 0.05] = F(3.0e38)
    cut2 = np.where(rng.random(n) < 0.5, F(-1.0), (10.0 ** rng.uniform(-12, -2, n)).astype(F)).astype(F)
    return mslice, near_lim, cut2


def test_pairs_above_the_cutoff_are_not_near_self_or_candidates():
    rng = np.random.default_rng(11)
    mslice, near_lim, cut2 = _cases(rng, 200_000)
    c = flag_cut2(mslice, near_lim, cut2)
    assert np.all(c >= FLT_MIN)  # r^2 = 0 (a self pair) is always below the cutoff
    # r^2 exactly at the cutoff, one float above it, and random values above it
    for r2 in (c, np.nextafter(c, F(np.inf)).astype(F),
               (c * (1.0 + 10.0 ** rng.uniform(-7, 3, c.size))).astype(F)):
        r2 = np.minimum(r2, F(3.0e38)).astype(F)
        above = r2 >= c
        with np.errstate(over="ignore"):
            near_test = near_lim * r2  # the pair loop's own product, m_j > near_lim * r^2
        # every source of the slice has m_j <= mslice: none can pass the near test
        assert np.all(~above | (mslice <= near_test))
        assert np.all(~above | ~(r2 < cut2))


def test_the_margin_keeps_the_cutoff_tight():
    """The cutoff flags few pairs beyond the near radius: within 1e-3 of mslice / near_lim
    wherever the quotient is a normal float above the screen cutoff."""
    rng = np.random.default_rng(12)
    mslice, near_lim, _ = _cases(rng, 100_000)
    cut2 = np.full_like(mslice, F(-1.0))
    c = flag_cut2(mslice, near_lim, cut2)
    q = mslice.astype(np.float64) / near_lim.astype(np.float64)
    sel = (mslice > 0) & (near_lim < 1e30) & (q > 1e-30)
    assert np.all(c[sel] >= q[sel])
    assert np.all(c[sel] <= q[sel] * 1.001)


def test_a_failed_check_flags_the_whole_slice():
    # an infinite near limit (a sink on top of the heavy source) makes near_lim * c NaN or
    # inf; a zero near limit makes the quotient infinite: the check sends every pair of the
    # slice to the exact pass
    c = flag_cut2(np.array([1e-8, 1e-8], F), np.array([0.0, np.inf], F), np.array([-1.0, -1.0], F))
    assert c[0] == F(3.0e38)
    assert c[1] == FLT_MIN or c[1] == F(3.0e38)
