"""The section kernel's exact skip of cubic segments (csrc/hg_section.cu):
where its convex-hull or Hermite-basis test says a same-signed segment cannot
cross, every sub-interval value the reference evaluates (its Hermite form,
poincare/utils.py:53-147, restated by the oracle's herm_s) keeps the end
values' sign -- so skipping the scan changes no result.  Segments are drawn
at random and adversarially, with the hull's control values or the basis
bound just above the skip margin."""
import numpy as np


def _skip(gk, gk1, d0, d1, dt):
    """The kernel's test, operation for operation (float64 arrays)."""
    m0, m1 = d0 * dt, d1 * dt
    am0, am1 = np.abs(m0), np.abs(m1)
    margin = 2.0 ** -46 * ((np.abs(gk) + np.abs(gk1)) + (am0 + am1))
    sg = np.where(gk > 0.0, 1.0, -1.0)
    b1, b2 = sg * (gk + m0 / 3.0), sg * (gk1 - m1 / 3.0)
    hull = (b1 > margin) & (b2 > margin) & (np.abs(gk) > margin) & (np.abs(gk1) > margin)
    lo = np.minimum(np.abs(gk), np.abs(gk1))
    basis = lo > (4.0 / 27.0) * (am0 + am1) * (1.0 + 1e-12) + margin
    return hull | basis


def _herm(s, y0, y1, dy0, dy1, dt):
    """The reference's cubic Hermite value at s (numba's squares: x * x)."""
    h00 = (1.0 + 2.0 * s) * ((1.0 - s) * (1.0 - s))
    h10 = s * ((1.0 - s) * (1.0 - s))
    h01 = (s * s) * (3.0 - 2.0 * s)
    h11 = (s * s) * (s - 1.0)
    return ((h00 * y0 + (h10 * dy0) * dt) + h01 * y1) + (h11 * dy1) * dt


def _segments(rng, n):
    sign = rng.choice([-1.0, 1.0], n)
    scale = 10.0 ** rng.uniform(-12, 2, n)
    g0 = sign * scale * rng.uniform(0.01, 1.0, n)
    g1 = sign * scale * rng.uniform(0.01, 1.0, n)
    dt = 10.0 ** rng.uniform(-4, 0, n)
    kind = rng.integers(0, 4, n)
    m0 = scale * rng.normal(0, 3, n)
    m1 = scale * rng.normal(0, 3, n)
    # hull control values a hair above the margin: g0 + m0/3 ~ g0 * delta
    delta = 2.0 ** rng.uniform(-56, -20, n)  # down to below the margin: those must not be skipped
    m0 = np.where(kind == 1, 3.0 * g0 * (delta - 1.0), m0)
    m1 = np.where(kind == 2, -3.0 * g1 * (delta - 1.0), m1)
    # basis bound a hair above the margin: |m0| + |m1| ~ 27/4 min(|g0|, |g1|) (1 - delta)
    lo = np.minimum(np.abs(g0), np.abs(g1))
    split = rng.uniform(0, 1, n)
    tot = 6.75 * lo * (1.0 - delta)
    m0 = np.where(kind == 3, -sign * tot * split, m0)
    m1 = np.where(kind == 3, sign * tot * (1.0 - split), m1)
    return g0, g1, m0 / dt, m1 / dt, dt


def test_skipped_segments_never_change_sign():
    rng = np.random.default_rng(12)
    r = 50
    step = 1.0 / (r + 1)
    s = np.arange(r + 2) * step  # every sub-interval end the reference evaluates (mm * step)
    total = skipped = 0
    for _ in range(20):
        g0, g1, d0, d1, dt = _segments(rng, 20000)
        sk = _skip(g0, g1, d0, d1, dt)
        total += sk.size
        skipped += int(sk.sum())
        v = _herm(s[:, None], g0[sk], g1[sk], d0[sk], d1[sk], dt[sk])
        assert np.all(np.sign(v) == np.sign(g0[sk])), "a skipped segment changes sign"
    # the adversarial draws reach the skip often enough to mean something
    assert skipped > total // 4


def _skips_scan(g0, g1, d0, d1, dt, cubic, dir_any, tiny_any=2.0 ** -490):
    """The kernel's decision to skip a segment's sub-interval scan (no end value
    near the surface): same-signed ends, neither below the tiny threshold and,
    for cubic segments, the hull or basis bound."""
    tiny_end = tiny_any if dir_any else 1e-280
    same = ((g0 > 0) & (g1 > 0)) | ((g0 < 0) & (g1 < 0))
    ok = same & (np.abs(g0) >= tiny_end) & (np.abs(g1) >= tiny_end)
    if cubic:
        ok &= _skip(g0, g1, d0, d1, dt)
    return ok


def _reference_crosses_any(g0, g1, d0, d1, dt, cubic, r=50):
    """Whether the reference's direction=None test (g_lo * g_hi <= 0 and
    g_lo != g_hi, synodic/backend.py:588) fires on any sub-interval."""
    step = 1.0 / (r + 1)
    s = np.arange(r + 2) * step
    if cubic:
        v = _herm(s[:, None], g0, g1, d0, d1, dt)
    else:
        v = (1.0 - s[:, None]) * g0 + s[:, None] * g1
    lo, hi = v[:-1], v[1:]
    return np.any((lo * hi <= 0.0) & (lo != hi), axis=0)


def _tiny_segments(rng, n):
    sign = rng.choice([-1.0, 1.0], n)
    g0 = sign * 2.0 ** rng.uniform(-560, -380, n)
    g1 = sign * 2.0 ** rng.uniform(-560, -380, n)
    dt = 10.0 ** rng.uniform(-3, 0, n)
    m0 = np.abs(g0) * rng.normal(0, 1, n)
    m1 = np.abs(g1) * rng.normal(0, 1, n)
    return g0, g1, m0 / dt, m1 / dt, dt


def test_direction_free_skip_never_hides_an_underflowing_product():
    """Without a direction the reference's product g_lo * g_hi underflows to
    zero for same-signed values below about 2^-537 and reports a crossing:
    no segment the kernel skips may be one of those (linear and cubic)."""
    rng = np.random.default_rng(5)
    for cubic in (False, True):
        g0, g1, d0, d1, dt = _tiny_segments(rng, 40000)
        sk = _skips_scan(g0, g1, d0, d1, dt, cubic, dir_any=True)
        assert sk.sum() > 1000
        assert not np.any(_reference_crosses_any(g0[sk], g1[sk], d0[sk], d1[sk], dt[sk], cubic))


def test_direction_free_skip_check_catches_a_loose_threshold():
    """The check above fails for the threshold used with a direction (1e-280):
    the reference does report crossings on segments that rule would skip."""
    rng = np.random.default_rng(5)
    g0, g1, d0, d1, dt = _tiny_segments(rng, 40000)
    sk = _skips_scan(g0, g1, d0, d1, dt, False, dir_any=True, tiny_any=1e-280)
    assert np.any(_reference_crosses_any(g0[sk], g1[sk], d0[sk], d1[sk], dt[sk], False))
