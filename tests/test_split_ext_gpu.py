"""Split form above lmax = 256: Legendre rows with 2-bit exponents (extended range),
and the FP64 plain path at lmax = 512 pinned to the oracle.

Sectoral seeds P_mm ~ sin^m(theta) leave the range of FP32 rows scaled by 2^100 for
m above ~256; the extended rows keep them exact down to ~2^-520.  The split results
are held to the same error measures as below lmax = 256 against the FP64 plain path
with exact j_l, which is itself pinned to the oracle at lmax = 512 here.
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
    rs = catana.sfb_decomposition(pc, 512, 16, 1000.0, True, False, precision="split")
    rp = catana.sfb_decomposition(pc, 512, 16, 1000.0, True, False, interpolation="off")
    _check(rs, rp.f_lmn, rp.c_ln, "split ext mid-latitude band")
