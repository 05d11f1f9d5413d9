"""The oracle (CPU restatement, oracle/catana_oracle.c) pinned against the
reference's golden vectors, known answers and, where it was built, the reference's
own besseltools sources."""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O
from conftest import uniform_ball


def test_golden_raw_exact(golden):
    """decomposition_test.py:23-36 (raw, N=445 <= 1000 so exact j_l), tightened."""
    pts = O.cartesian_to_spherical(golden["xyz"])
    assert pts.shape == (445, 3)
    k, c, _ = O.sfb_raw(pts, 10, 10, 2500, interpolated=False, store_flmn=False)
    assert np.allclose(k, golden["k_ln"])
    cc = c * golden["correction_factor"] ** 2
    assert np.allclose(cc, golden["c_ln"], rtol=1e-2)
    # the golden file was made with converged zeros; the reference's k_ln stop early
    # (SphericalBesselZeros.cpp:53-59), which moves C_ln by ~1e-6
    assert np.max(np.abs(cc / golden["c_ln"] - 1)) < 1e-5


def test_golden_raw_interpolated(golden):
    """sfb_test.cpp:53-63: the interpolated raw method also within 1% of the golden C_ln."""
    pts = O.cartesian_to_spherical(golden["xyz"])
    k, c, _ = O.sfb_raw(pts, 10, 10, 2500, interpolated=True, store_flmn=False)
    assert np.allclose(c * golden["correction_factor"] ** 2, golden["c_ln"], rtol=1e-2)


def test_golden_healpix(golden):
    """decomposition_test.py:38-49 (pixelized method, nside 64)."""
    pts = O.cartesian_to_spherical(golden["xyz"])
    offs, rs = O.bin_points(64, pts)
    assert offs[-1] == 445
    k, c, _ = O.sfb_healpix(64, offs, rs, 10, 10, 2500, interpolated=False, store_flmn=False)
    assert np.allclose(k, golden["k_ln_rev"])
    cc = c * golden["correction_factor"] ** 2
    assert np.allclose(cc, golden["c_ln_rev"], rtol=1e-2)
    assert np.max(np.abs(cc / golden["c_ln_rev"] - 1)) < 1e-5


def test_zeros_known_answers():
    """SphericalBesselZeros_test.cpp:7-16 and besseltools_test.py:11-19."""
    z0 = O.sbessel_zeros(0, 3)
    assert z0 == pytest.approx([np.pi, 6.283185307179586, 9.42477796076938])
    assert O.sbessel_zeros(5, 10)[9] == pytest.approx(38.8836, abs=1e-4)


def test_kln_boundary_condition():
    """return_types_test.cpp:26-29: |j_l(k_{l,nmax-1} rmax)| < 1e-15 for l < 10, nmax 20."""
    rmax = 5.4
    k = O.compute_kln(10, 20, rmax)
    for l in range(10):
        assert abs(O.sbessel_jl(l, k[l, 19] * rmax)) < 1e-15


def test_zeros_and_tables_match_reference_sources():
    """The reference's own SphericalBesselZeros / SBesselInterpolator (compiled by
    `make -C oracle ref` against the oracle's j_l) agree with the restatement bit for bit."""
    R = O.ref_lib()
    if R is None:
        pytest.skip("reference sources not built here (no reference tree)")
    for l in [0, 1, 5, 31, 100, 255, 511]:
        a = O.sbessel_zeros(l, 140)
        b = np.zeros(140)
        R.ref_sbessel_zeros(l, 140, b.ctypes.data_as(ctypes.c_void_p))
        assert np.array_equal(a, b), l
    for l, nmax in [(0, 10), (7, 32), (31, 32), (200, 128)]:
        z = O.sbessel_zeros(l, nmax + 1)[nmax]
        y, _ = O.lerp_table(l, z, 1000 * nmax)
        yr = np.zeros(1000 * nmax)
        zr = np.zeros(1)
        R.ref_interp_table(l, nmax, 1000 * nmax, yr.ctypes.data_as(ctypes.c_void_p), zr.ctypes.data_as(ctypes.c_void_p))
        assert zr[0] == z
        assert np.array_equal(y, yr)


def test_interpolator_accuracy():
    """SBesselLookUp_test.cpp:20-42: lerp within 5% (or 1e-8) of j_l; value at zmax ~ 0."""
    rng = np.random.default_rng(1)
    for l in range(10):
        z4 = O.sbessel_zeros(l, 5)[4]
        y, dxi = O.lerp_table(l, z4, 4000)
        err = ctypes.c_int(0)
        for z in rng.uniform(0, z4, 200):
            v = O.lib().co_lerp_eval_pub(y.ctypes.data_as(ctypes.c_void_p), 4000, dxi, z4, z, ctypes.byref(err))
            ex = O.sbessel_jl(l, z)
            assert abs(v - ex) <= max(1e-8, abs(0.05 * ex))
        v = O.lib().co_lerp_eval_pub(y.ctypes.data_as(ctypes.c_void_p), 4000, dxi, z4, z4 - 1e-10, ctypes.byref(err))
        assert abs(v) < 1e-8
        assert err.value == 0


def test_special_functions_vs_scipy():
    special = pytest.importorskip("scipy.special")
    rng = np.random.default_rng(2)
    for l in [0, 1, 3, 10, 32, 100, 255]:
        x = np.concatenate([rng.uniform(0, 3, 20), rng.uniform(0, 3 * l + 30, 60)])
        ours = np.array([O.sbessel_jl(l, v) for v in x])
        ref = special.spherical_jn(l, x)
        env = np.minimum(1.0, 1.0 / np.maximum(x, 1e-300))
        assert np.max(np.abs(ours - ref) / env) < 1e-11, l
    for l in [0, 1, 5, 20, 64, 150]:
        for m in range(0, l + 1, max(1, l // 7)):
            x = rng.uniform(-1, 1, 15)
            ours = np.array([O.sph_plm(l, m, v) for v in x])
            ref = special.sph_legendre_p(l, m, np.arccos(x))
            assert np.max(np.abs(ours - ref)) < 1e-11 * max(1.0, np.abs(ref).max()), (l, m)


def test_point_conversion_known_values():
    """point_types_tests.cpp:11-27."""
    p = O.cartesian_to_spherical(np.array([[0, 0, 1], [1, 1, 1], [-380, -800, 200]], dtype=float))
    assert p[0] == pytest.approx([1, 0, 0])
    assert p[1] == pytest.approx([1.73205081, 9.55316618e-01, 7.85398163e-01])
    assert p[2] == pytest.approx([9.07964757e+02, 1.34870213e+00, 4.26894064e+00])


def test_healpix_roundtrip_and_counts():
    for nside in [1, 2, 4, 8, 32]:
        npix = 12 * nside * nside
        th, ph = O.pix2ang_ring(nside, np.arange(npix))
        assert np.array_equal(O.ang2pix_ring(nside, th, ph), np.arange(npix))
    # point_test.py:55-62: two points at the pole and one at the other pole
    pts = np.array([[1, 0, 0], [1, 0, 0], [1, np.pi, 0]], dtype=float)
    offs, _ = O.bin_points(32, pts)
    cm = np.diff(offs)
    assert cm.shape == (32 * 32 * 12,) and cm.sum() == 3 and np.count_nonzero(cm) == 2
    # rings tile the map
    nside = 16
    tot = 0
    for ring in range(1, 4 * nside):
        s, n = O.ring_info(nside, ring)
        assert s == tot
        tot += n
    assert tot == 12 * nside * nside


def test_oracle_weights_reduce_to_unweighted():
    pts = uniform_ball(300, 100.0, 5)
    k1, c1, f1 = O.sfb_raw(pts, 6, 5, 100.0, interpolated=False)
    k2, c2, f2 = O.sfb_raw(pts, 6, 5, 100.0, interpolated=False, weights=np.ones(300))
    assert np.allclose(c1, c2, rtol=1e-13)
    # doubling every weight changes nothing (normalised by the weight sum)
    k3, c3, f3 = O.sfb_raw(pts, 6, 5, 100.0, interpolated=False, weights=2 * np.ones(300))
    assert np.allclose(c1, c3, rtol=1e-13)


def test_golden_reverse(golden):
    """sfb_test.cpp:101-133: _sfb_reverse (nside 64, lmax = nmax = 10, rmax 2500; exact
    and interpolated j_l) against the golden raw C_ln at the test's 10% bar, tightened:
    within 1e-5 of the pixelized golden file (the same pixel sums; this catalog has no
    ring where the FFT method's unconjugated alias matters at l < 10)."""
    pts = O.cartesian_to_spherical(golden["xyz"])
    offs, rs = O.bin_points(64, pts)
    for interp in (False, True):
        k, c, _ = O.sfb_reverse(64, offs, rs, 10, 10, 2500, interpolated=interp)
        cc = c * golden["correction_factor"] ** 2
        assert np.allclose(cc, golden["c_ln"], rtol=1e-1)
        assert np.allclose(k, golden["k_ln_rev"])
    k, c, _ = O.sfb_reverse(64, offs, rs, 10, 10, 2500, interpolated=False)
    assert np.max(np.abs(c * golden["correction_factor"] ** 2 / golden["c_ln_rev"] - 1)) < 1e-5


def test_reverse_equals_fft_path_away_from_aliasing():
    """_sfb_reverse and _sfb_reverse_fft sum the same pixel maps; at l = 0, 1 no m
    exceeds half of any ring's length (the shortest ring has 4 pixels), so the FFT
    method's unconjugated alias does not enter and the two agree to rounding."""
    pts = uniform_ball(4000, 300.0, seed=17)
    offs, rs = O.bin_points(16, pts)
    k1, c1, f1 = O.sfb_reverse(16, offs, rs, 8, 6, 300.0, interpolated=False)
    k2, c2, f2 = O.sfb_healpix(16, offs, rs, 8, 6, 300.0, interpolated=False)
    # l = 0, 1: every ring has >= 4 pixels > 2 l, no alias
    for l in (0, 1):
        assert np.max(np.abs(f1[l] - f2[l])) <= 1e-12 * np.max(np.abs(f2[l]))


@pytest.mark.parametrize("nside,n,lmax,nmax,interp", [(2, 1500, 8, 4, True), (8, 3000, 40, 12, True),
                                                       (8, 800, 12, 5, False)])
def test_healpix_fft_restatement_equals_direct(nside, n, lmax, nmax, interp):
    """The FFT form of the HEALPix oracle (per-ring r2c transforms, as the reference
    computes them) equals the direct-DFT restatement, aliased frequencies included."""
    pts = uniform_ball(n, 500.0, seed=nside)
    offs, rs = O.bin_points(nside, pts)
    k1, c1, f1 = O.sfb_healpix(nside, offs, rs, lmax, nmax, 500.0, interpolated=interp)
    k2, c2, f2 = O.sfb_healpix_fft(nside, offs, rs, lmax, nmax, 500.0, interpolated=interp)
    assert np.array_equal(k1, k2)
    fmax = max(np.abs(x).max() for x in f1)
    assert max(np.abs(a - b).max() for a, b in zip(f1, f2)) <= 1e-13 * fmax
    assert np.allclose(c2, c1, rtol=1e-12, atol=0)


def test_oracle_ingest_filters():
    """Ingest restatement: conversion as Point(x, y, z); the tophat keeps exactly r < R0;
    the Gaussian window keeps a fraction matching its expectation; the mask keeps
    exactly the points whose RING pixel is 1; chunked calls (index0) reproduce one call."""
    rng = np.random.default_rng(3)
    xyz = rng.normal(size=(20000, 3)) * 300.0
    rtp = O.cartesian_to_spherical(xyz)
    assert np.array_equal(O.ingest(xyz, cartesian=True), rtp)
    top = O.ingest(rtp, tophat_r0=400.0)
    assert np.array_equal(top, rtp[rtp[:, 0] < 400.0])
    g = O.ingest(rtp, gauss_r0=300.0, seed=11)
    expect = np.exp(-(rtp[:, 0] / 300.0) ** 2).sum()
    assert abs(g.shape[0] - expect) < 5 * np.sqrt(expect)
    nside = 8
    mask = (np.arange(12 * nside * nside) % 3 == 0).astype(np.float32)
    pix = O.ang2pix_ring(nside, rtp[:, 1], rtp[:, 2])
    assert np.array_equal(O.ingest(rtp, mask=mask), rtp[mask[pix] == 1.0])
    both = O.ingest(rtp, gauss_r0=300.0, seed=11, mask=mask)
    parts = np.concatenate([O.ingest(rtp[:7000], gauss_r0=300.0, seed=11, mask=mask),
                            O.ingest(rtp[7000:], gauss_r0=300.0, seed=11, mask=mask, index0=7000)])
    assert np.array_equal(both, parts)


def test_oracle_dsb_integral_known_values():
    """besseltools_test.py:26-37 and sbessel_integrator.cpp:8-14: known integrals with
    w = 1, and symmetry in k1 <-> k2."""
    one = np.ones(3)
    assert O.dsb_integral(one, (0.0, 100.0 + 1e-9), 0, 100, 1, 1) == pytest.approx(1.56582, abs=1e-5)
    assert O.dsb_integral(one, (0.0, 100.0 + 1e-9), 0, 100, 1, 2) == pytest.approx(0.785393, abs=1e-5)
    assert O.dsb_integral(one, (0.0, 100.0 + 1e-9), 4, 100, 1, 4.2) == pytest.approx(0.000133933, abs=1e-9)
    x = np.linspace(0.0, 100.0, 100000)
    w = np.exp(-(x / 40) ** 2) * x ** 2
    assert O.dsb_integral(w, (0, 100), 6, 100, 2.3, 4.5) == O.dsb_integral(w, (0, 100), 6, 100, 4.5, 2.3)
