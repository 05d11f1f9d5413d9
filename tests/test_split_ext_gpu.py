"""Split form above lmax = 256: Legendre rows with 2-bit exponents (extended range),
and the FP64 plain path at lmax = 512 pinned to the oracle.

Sectoral seeds P_mm ~ sin^m(theta) leave the range of FP32 rows scaled by 2^100 for
m above ~256; the extended rows keep them exact down to ~2^-520.  Above lmax 256 the
split form always takes the Reinsch-modified rows (P_l and D_l sharing one exponent per
value; 'split' and 'split_accurate' are the same computation there).  The results are
held to the same error measures as below lmax = 256 against the FP64 plain path with
exact j_l (or with j_l from its FP64 polynomials), which is itself pinned to the oracle
at lmax = 512 here.
"""
import numpy as np
import pytest

import catana_gb300 as catana
from oracle import oracle as O
from conftest import uniform_ball
from test_raw_split_gpu import _check

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sm103(cuda_device):
    if tuple(cuda_device) != (10, 3):
        pytest.skip("split form needs sm_103")


def test_plain_lmax512_vs_oracle(cuda_device):
    pts = uniform_ball(48, 1500.0, seed=41)
    res = catana.sfb_decomposition(catana.PointContainer(pts), 512, 6, 1500.0, True, False, interpolation="off")
    k, c, f = O.sfb_raw(pts, 512, 6, 1500.0, interpolated=False)
    assert np.array_equal(res.k_ln, k)
    fmax = max(np.abs(x).max() for x in f)
    err = max(np.abs(a - b).max() for a, b in zip(res.f_lmn, f)) / fmax
    assert err <= 1e-10, err


@pytest.mark.parametrize("n,lmax,nmax,weighted", [
    (4000, 300, 40, True),
    (3000, 512, 24, False),
    (2000, 400, 160, True),   # extended rows and two radial halves
])
def test_split_extended_vs_plain(sm103, n, lmax, nmax, weighted):
    pts = uniform_ball(n, 1500.0, seed=500 + lmax)
    w = np.random.default_rng(lmax).uniform(0.5, 1.5, n) if weighted else None
    pc = catana.PointContainer(pts)
    rs = catana.sfb_decomposition(pc, lmax, nmax, 1500.0, True, False, weights=w, precision="split")
    rp = catana.sfb_decomposition(pc, lmax, nmax, 1500.0, True, False, weights=w, interpolation="off")
    assert np.array_equal(rs.k_ln, rp.k_ln)
    _check(rs, rp.f_lmn, rp.c_ln, "split ext n=%d lmax=%d nmax=%d" % (n, lmax, nmax))


def test_split_forms_agree_above_256(sm103):
    """Above lmax 256 both precision names run the Reinsch-modified rows: same bits."""
    pts = uniform_ball(1500, 1000.0, seed=77)
    pc = catana.PointContainer(pts)
    a = catana.sfb_decomposition(pc, 300, 20, 1000.0, True, False, precision="split")
    b = catana.sfb_decomposition(pc, 300, 20, 1000.0, True, False, precision="split_accurate")
    assert np.array_equal(a.c_ln, b.c_ln)
    for x, y in zip(a.f_lmn, b.f_lmn):
        assert np.array_equal(x, y)


def _rms_by_l(res, ref):
    return np.array([np.sqrt(np.mean(np.abs(a - b) ** 2) / np.mean(np.abs(b) ** 2))
                     for a, b in zip(res.f_lmn, ref.f_lmn)])


def test_split_extended_polar_points(sm103):
    """30% of the points within 0.05 rad of a pole, lmax 400: near the poles the FP32
    three-term recurrence's rounding builds up through its cancellation (rms(df_l) /
    rms(f_l) up to 7.8e-5 at l >= 256 with three-term extended rows); the
    Reinsch-modified rows, carried through the extended range with their exponents,
    keep the usual error measures (measured 1.0e-6)."""
    rng = np.random.default_rng(11)
    n = 3000
    pts = uniform_ball(n, 1000.0, seed=12)
    pol = rng.random(n) < 0.3
    th = rng.uniform(0.0, 0.05, pol.sum())
    pts[pol, 1] = np.where(rng.random(pol.sum()) < 0.5, th, np.pi - th)
    pc = catana.PointContainer(pts)
    rp = catana.sfb_decomposition(pc, 400, 16, 1000.0, True, False, interpolation="off")
    ra = catana.sfb_decomposition(pc, 400, 16, 1000.0, True, False, precision="split")
    ea = _rms_by_l(ra, rp)
    print("polar band, rms(df_l)/rms(f_l) max over l >= 256: %.2e" % ea[256:].max())
    _check(ra, rp.f_lmn, rp.c_ln, "split ext polar band")
    assert ea[256:].max() <= 3e-6


def _masked_survey(n, seed, rmax=1500.0, a=300.0):
    """(r, theta, phi): r ~ r^2 exp(-(r/a)^2) below rmax, |theta - pi/2| < 20 deg masked, phi uniform."""
    rng = np.random.default_rng(seed)
    r = a / np.sqrt(2.0) * np.sqrt((rng.standard_normal((n, 3)) ** 2).sum(1))
    r = np.minimum(r, 0.999 * rmax)
    ct = rng.uniform(np.sin(np.deg2rad(20.0)), 1.0, n) * np.where(rng.random(n) < 0.5, -1.0, 1.0)
    return np.column_stack([r, np.arccos(ct), rng.uniform(0.0, 2.0 * np.pi, n)])


def test_split_survey_outermost_point_near_pole(sm103):
    """A masked survey at lmax 512 whose outermost point lies 0.15 rad from a pole.  A
    mode that reaches the data only in j_l's evanescent zone (k_ln r well below l at
    every radius) is carried by that one point -- j_l(k r) grows like r^l there -- so
    its Legendre rows enter those C_ln undiluted.  Three-term extended rows lose a few
    1e-6 of sum_m P_lm^2 at theta = 0.15 and l > 200 (C_ln p99 5.0e-6 here); the
    Reinsch-modified rows hold C_ln to the usual bar (measured 5.0e-7)."""
    n = 20000
    pts = _masked_survey(n, seed=21)
    o = np.argmax(pts[:, 0])
    pts[o, 1] = 0.15
    pc = catana.PointContainer(pts)
    rp = catana.sfb_decomposition(pc, 512, 32, 1500.0, True, False, interpolation="poly")
    keep = rp.c_ln >= 1e-40 * rp.c_ln.max()  # below: outside FP32's range, returned as 0
    r = catana.sfb_decomposition(pc, 512, 32, 1500.0, True, False, precision="split")
    rel = np.abs(r.c_ln - rp.c_ln)[keep] / rp.c_ln[keep]
    print("survey, outermost point near a pole: C rel median %.2e p99 %.2e max %.2e, %d above 1e-6 (of %d)"
          % (np.median(rel), np.percentile(rel, 99), rel.max(), int((rel > 1e-6).sum()), int(keep.sum())))
    assert np.percentile(rel, 99) <= 1e-6


def test_split_extended_mid_latitude_points(sm103):
    """40% of the points at 0.3 < theta < 0.6 (or the mirror band): their sectoral
    seeds sin(theta)^m drop below the plain scaled-row range for m above ~150, yet
    they reach the oscillatory zone (l > m / sin(theta)) before lmax = 512, so their
    contributions at high l come through the extended rows alone."""
    rng = np.random.default_rng(7)
    n = 3000
    pts = uniform_ball(n, 1000.0, seed=8)
    band = rng.random(n) < 0.4
    th = rng.uniform(0.3, 0.6, band.sum())
    pts[band, 1] = np.where(rng.random(band.sum()) < 0.5, th, np.pi - th)
    pc = catana.PointContainer(pts)
    rp = catana.sfb_decomposition(pc, 512, 16, 1000.0, True, False, interpolation="off")
    rs = catana.sfb_decomposition(pc, 512, 16, 1000.0, True, False, precision="split")
    _check(rs, rp.f_lmn, rp.c_ln, "split ext mid-latitude band")
