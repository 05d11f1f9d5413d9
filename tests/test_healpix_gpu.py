"""HEALPix path on the GPU: RING ang2pix / pix2ang and binning bit-exact against
the oracle's restatement of the published algorithm, and the pixelized SFB
(sfb_reverse_fft.cpp:43-209) against the oracle at 1e-10 of max|f_lmn|."""
import numpy as np
import pytest

import catana_gb300 as catana
from catana_gb300 import _lib
from oracle import oracle as O
from conftest import uniform_ball

pytestmark = pytest.mark.gpu


def _ang2pix_gpu(nside, th, ph):
    pix = np.zeros(th.size, dtype=np.int64)
    _lib.check(_lib.lib.catana_gpu_ang2pix_ring(nside, _lib.ptr(th), _lib.ptr(ph), th.size, _lib.ptr(pix), None))
    return pix


def test_ang2pix_bitexact(cuda_device):
    rng = np.random.default_rng(0)
    n = 200000
    th = np.arccos(rng.uniform(-1, 1, n))
    ph = rng.uniform(0, 2 * np.pi, n)
    # near-polar, boundary-ish and exact-pixel-centre angles
    th = np.concatenate([th, rng.uniform(0, 0.02, 2000), np.pi - rng.uniform(0, 0.02, 2000), [0.0, np.pi]])
    ph = np.concatenate([ph, rng.uniform(-7, 14, 4000), [0.0, 1.0]])
    for nside in [1, 2, 16, 64, 256, 1024]:
        gpu = _ang2pix_gpu(nside, th, ph)
        cpu = O.ang2pix_ring(nside, th, ph)
        assert np.array_equal(gpu, cpu), nside


def test_pix2ang_roundtrip(cuda_device):
    for nside in [1, 4, 32, 256]:
        npix = 12 * nside * nside
        pix = np.arange(npix, dtype=np.int64)
        th = np.zeros(npix)
        ph = np.zeros(npix)
        _lib.check(_lib.lib.catana_gpu_pix2ang_ring(nside, _lib.ptr(pix), npix, _lib.ptr(th), _lib.ptr(ph), None))
        oth, oph = O.pix2ang_ring(nside, pix) if nside <= 32 else (None, None)
        if oth is not None:
            assert np.array_equal(th, oth) or np.max(np.abs(th - oth)) < 1e-15
            assert np.array_equal(ph, oph)
        assert np.array_equal(_ang2pix_gpu(nside, th, ph), pix)


def test_binning_matches_oracle(cuda_device):
    pts = uniform_ball(50000, 100.0, seed=3)
    for nside in [2, 16, 128]:
        ppc = catana.PixelizedPointContainer(nside, catana.PointContainer(pts))
        offs, rs = O.bin_points(nside, pts)
        assert np.array_equal(ppc.offsets, offs)
        assert np.array_equal(ppc.r_sorted, rs)  # point order kept inside each pixel
        assert ppc.get_npoints() == 50000


def test_countmap_known_answers(cuda_device):
    """point_test.py:55-62 and point_types_tests.cpp:86-109."""
    pc = catana.PointContainer(np.array([[1, 0, 0], [1, 0, 0], [1, np.pi, 0]], dtype=float))
    cm = catana.PixelizedPointContainer(32, pc).get_countmap()
    assert cm.shape == (32 ** 2 * 12,) and cm.sum() == 3 and np.count_nonzero(cm) == 2
    xyz = np.array([[-1, 2, 3], [-4, 1, 0], [0, 1, 2], [1, 4, 0], [1, 2, 3]], dtype=float)
    ppc = catana.PixelizedPointContainer(16, catana.PointContainer(xyz, "cartesian"))
    assert ppc.get_npoints() == 5 and ppc.get_countmap().sum() == 5
    with pytest.raises(ValueError):
        catana.PixelizedPointContainer(16, catana.PointContainer(np.array([[1.0, 4.0, 0.0]])))  # theta > pi


def _compare(res, k, c, f, tol=1e-10):
    assert np.array_equal(res.k_ln, k)
    fmax = max(np.abs(x).max() for x in f)
    err = max(np.abs(a - b).max() for a, b in zip(res.f_lmn, f)) / fmax
    assert err <= tol, err
    assert np.max(np.abs(res.c_ln - c) / np.abs(c)) <= 1e-9


def test_golden_healpix(cuda_device, golden):
    """decomposition_test.py:38-49: nside 64, lmax = nmax = 10, rmax 2500, rtol 1e-2."""
    pc = catana.PointContainer(golden["xyz"], "cartesian")
    ppc = catana.PixelizedPointContainer(64, pc)
    res = catana.sfb_decomposition(ppc, 10, 10, 2500, True, False)
    assert np.allclose(res.k_ln, golden["k_ln_rev"])
    assert np.allclose(res.c_ln * golden["correction_factor"] ** 2, golden["c_ln_rev"], rtol=1e-2)
    k, c, f = O.sfb_healpix(64, ppc.offsets, ppc.r_sorted, 10, 10, 2500, interpolated=False)
    _compare(res, k, c, f)


@pytest.mark.parametrize("nside,n,lmax,nmax", [(8, 3000, 40, 12), (16, 1500, 20, 10), (32, 5000, 16, 40),
                                                (64, 20000, 30, 17), (4, 4000, 48, 9), (2, 1200, 20, 5),
                                                (1, 1500, 12, 4)])
def test_healpix_vs_oracle(cuda_device, nside, n, lmax, nmax):
    """Polar rings shorter than 2l exercise the reference's unconjugated alias.  Rings of
    power-of-two length go through the FFT once l + 1 > 4 log2(length) - 4 (equatorial
    rings at nside 1 to 8 and 64, polar rings of 4 to 32 pixels; both packed radial
    orders, odd nmax); the other polar rings (4 i pixels, i not a power of two: 12, 20,
    24, 28, ...) through the folded direct sum.  nside 1: every ring has 4 pixels."""
    pts = uniform_ball(n, 500.0, seed=nside)
    ppc = catana.PixelizedPointContainer(nside, catana.PointContainer(pts))
    res = catana.sfb_decomposition(ppc, lmax, nmax, 500.0, True, False)
    k, c, f = O.sfb_healpix(nside, ppc.offsets, ppc.r_sorted, lmax, nmax, 500.0, interpolated=n > 1000)
    _compare(res, k, c, f)


def test_healpix_conj_fix_changes_only_aliased(cuda_device):
    pts = uniform_ball(2000, 500.0, seed=1)
    ppc = catana.PixelizedPointContainer(2, catana.PointContainer(pts))
    a = catana.sfb_decomposition(ppc, 8, 4, 500.0, True, False)
    b = catana.sfb_decomposition(ppc, 8, 4, 500.0, True, False, conj_fix=True)
    # m <= 2 is never aliased at nside 2 (shortest ring: 4 pixels)
    for l in range(8):
        assert np.array_equal(a.f_lmn[l][:3], b.f_lmn[l][:3])
    assert any(not np.array_equal(a.f_lmn[l], b.f_lmn[l]) for l in range(3, 8))
