"""_sfb_reverse on the GPU (catana_gpu_sfb_reverse) against the oracle's restatement
of the dense per-pixel sum (sfb_reverse.cpp:13-112), <= 1e-10 of max|f|; and the
reference's own test of the method (sfb_test.cpp:101-133) on the golden catalog."""
import numpy as np
import pytest

import catana_gb300 as catana
from oracle import oracle as O
from conftest import uniform_ball

pytestmark = pytest.mark.gpu


def _cmp(res, k, c, f):
    assert np.array_equal(res.k_ln, k)
    fmax = max(np.abs(x).max() for x in f)
    err = max(np.abs(a - b).max() for a, b in zip(res.f_lmn, f)) / fmax
    assert err <= 1e-10, err
    assert np.allclose(res.c_ln, c, rtol=1e-9, atol=0)


@pytest.mark.parametrize("nside,n,lmax,nmax,interp", [
    (8, 3000, 20, 8, False),    # rings of 4..32 pixels: m mod rpix past rpix/2 everywhere
    (8, 3000, 20, 8, True),
    (32, 20000, 40, 10, True),
])
def test_reverse_vs_oracle(cuda_device, nside, n, lmax, nmax, interp):
    pts = uniform_ball(n, 700.0, seed=nside + lmax)
    ppc = catana.PixelizedPointContainer(nside, catana.PointContainer(pts))
    res = catana.sfb_reverse(ppc, lmax, nmax, 700.0, store_flmn=True, verbose=False, interpolated=interp)
    k, c, f = O.sfb_reverse(nside, ppc.offsets, ppc.r_sorted, lmax, nmax, 700.0, interpolated=interp)
    _cmp(res, k, c, f)


def test_reverse_golden(cuda_device, golden):
    pts = O.cartesian_to_spherical(golden["xyz"])
    ppc = catana.PixelizedPointContainer(64, catana.PointContainer(pts))
    for interp in (False, True):
        res = catana.sfb_reverse(ppc, 10, 10, 2500, store_flmn=True, verbose=False, interpolated=interp)
        k, c, f = O.sfb_reverse(64, ppc.offsets, ppc.r_sorted, 10, 10, 2500, interpolated=interp)
        _cmp(res, k, c, f)
        assert np.allclose(res.c_ln * golden["correction_factor"] ** 2, golden["c_ln"], rtol=1e-1)


def test_reverse_large_rings_vs_raw(cuda_device):
    """Points on pixel centres: the pixelized sum equals the raw sum over the same points
    (the oracle's two restatements agree to 2e-16 at nside 8), so at nside 1024 -- the
    2048- and 4096-pixel rings through the FFT from l = 40 and 44 on, the polar rings of
    4 i pixels through the folded sums -- the reverse path matches the FP64 raw path."""
    nside = 1024
    rng = np.random.default_rng(11)
    pix = rng.choice(12 * nside * nside, 4000, replace=False).astype(np.int64)
    th, ph = O.pix2ang_ring(nside, pix)
    pts = np.stack([700.0 * rng.random(pix.size) ** (1 / 3), th, ph], 1)
    lmax, nmax = 48, 3
    raw = catana.sfb_decomposition(catana.PointContainer(pts), lmax, nmax, 700.0, True, False, interpolation="off")
    ppc = catana.PixelizedPointContainer(nside, catana.PointContainer(pts))
    assert np.count_nonzero(np.diff(ppc.offsets)) == pix.size  # one point per pixel
    rev = catana.sfb_reverse(ppc, lmax, nmax, 700.0, store_flmn=True, verbose=False, interpolated=False)
    fmax = max(np.abs(x).max() for x in raw.f_lmn)
    err = max(np.abs(a - b).max() for a, b in zip(rev.f_lmn, raw.f_lmn)) / fmax
    assert err <= 1e-10, err
    assert np.allclose(rev.c_ln, raw.c_ln, rtol=1e-9, atol=0)
