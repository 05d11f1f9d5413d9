"""Parity of the plain FP64 raw path (the drop-in) with the oracle, through the
C ABI on the GPU.  Bar: max|f_gpu - f_oracle| <= 1e-10 * max|f_oracle| and C_ln to
1e-9 relative, with identical k_ln (both use the reference's zero finder)."""
import ctypes

import numpy as np
import pytest

import catana_gb300 as catana
from catana_gb300 import _lib
from oracle import oracle as O
from conftest import uniform_ball

pytestmark = pytest.mark.gpu
TOL_F = 1e-10


def _compare(res, k, c, f, tol=TOL_F):
    assert np.array_equal(res.k_ln, k)
    fmax = max([np.abs(x).max() for x in f] + [0.0])
    if fmax > 0:
        err = max(np.abs(a - b).max() for a, b in zip(res.f_lmn, f)) / fmax
        assert err <= tol, err
    cmax = np.abs(c).max()
    assert np.max(np.abs(res.c_ln - c)) <= 10 * tol * max(cmax, 1e-300)


def test_golden_catalog(cuda_device, golden):
    """decomposition_test.py:23-36 through the GPU path, plus parity with the oracle."""
    pc = catana.PointContainer(golden["xyz"], "cartesian")
    res = catana.sfb_decomposition(pc, 10, 10, 2500, False, False)
    assert np.allclose(res.k_ln, golden["k_ln"])
    assert np.allclose(res.c_ln * golden["correction_factor"] ** 2, golden["c_ln"], rtol=1e-2)
    res = catana.sfb_decomposition(pc, 10, 10, 2500, True, False)
    k, c, f = O.sfb_raw(np.asarray(pc), 10, 10, 2500, interpolated=False)
    _compare(res, k, c, f)


@pytest.mark.parametrize("n,lmax,nmax,interp", [
    (2000, 16, 16, "auto"),   # N > 1000: interpolated, the reference's rule
    (700, 12, 20, "auto"),    # N <= 1000: exact j_l
    (3000, 40, 24, "on"),     # 64-wide tiles in m
    (1500, 8, 70, "on"),      # 64-wide tiles in n, ragged
    (1200, 33, 33, "off"),    # exact j_l above the threshold
])
def test_random_catalogs(cuda_device, n, lmax, nmax, interp):
    pts = uniform_ball(n, 1000.0, seed=n + lmax)
    res = catana.sfb_decomposition(catana.PointContainer(pts), lmax, nmax, 1000.0, True, False, interpolation=interp)
    interpolated = {"auto": n > 1000, "on": True, "off": False}[interp]
    k, c, f = O.sfb_raw(pts, lmax, nmax, 1000.0, interpolated=interpolated)
    _compare(res, k, c, f)


@pytest.mark.parametrize("interp", ["auto", "off"])
def test_config1_size(cuda_device, interp):
    """Plain raw SFB at the reference's CPU-runnable case: 100k points uniform in a
    ball of rmax=1000, lmax=nmax=32, seed 0, in the interpolated mode (the reference's
    rule for N > 1000) and with exact j_l."""
    pts = uniform_ball(100000, 1000.0, seed=0)
    res = catana.sfb_decomposition(catana.PointContainer(pts), 32, 32, 1000.0, True, False, interpolation=interp)
    k, c, f = O.sfb_raw(pts, 32, 32, 1000.0, interpolated=(interp == "auto"))
    _compare(res, k, c, f)


def test_weights(cuda_device):
    pts = uniform_ball(2500, 500.0, seed=7)
    w = np.random.default_rng(7).uniform(0.5, 1.5, 2500)
    res = catana.sfb_decomposition(catana.PointContainer(pts), 12, 12, 500.0, True, False, weights=w)
    k, c, f = O.sfb_raw(pts, 12, 12, 500.0, interpolated=True, weights=w)
    _compare(res, k, c, f)


def test_store_flmn_false_and_small_shapes(cuda_device):
    pts = uniform_ball(50, 10.0, seed=3)
    pc = catana.PointContainer(pts)
    res = catana.sfb_decomposition(pc, 5, 4, 10.0, False, False)
    assert res.f_lmn == [] and res.c_ln.shape == (5, 4)
    k, c, f = O.sfb_raw(pts, 5, 4, 10.0, interpolated=False)
    assert np.allclose(res.c_ln, c, rtol=1e-10)
    res = catana.sfb_decomposition(catana.PointContainer(pts[:1]), 3, 3, 10.0, True, False)
    k, c, f = O.sfb_raw(pts[:1], 3, 3, 10.0, interpolated=False)
    _compare(res, k, c, f)
    res = catana.sfb_decomposition(pc, 0, 4, 10.0, True, False)
    assert res.k_ln.shape == (0, 4) and res.f_lmn == []


def test_empty_catalog_matches_reference_nan(cuda_device):
    """No points: the reference divides by N = 0, so f = 0 * inf = NaN."""
    res = catana.sfb_decomposition(catana.PointContainer(), 3, 3, 10.0, True, False)
    k, c, f = O.sfb_raw(np.zeros((0, 3)), 3, 3, 10.0, interpolated=False)
    assert np.array_equal(res.k_ln, k)
    assert np.all(np.isnan(res.c_ln)) and np.all(np.isnan(c))


def test_domain_error(cuda_device):
    """A radius far beyond rmax leaves the interpolation table: ValueError, as the
    reference's std::domain_error (SBesselInterpolator.cpp:20-23)."""
    pts = uniform_ball(1500, 100.0, seed=4)
    pts[17, 0] = 400.0
    with pytest.raises(ValueError):
        catana.sfb_decomposition(catana.PointContainer(pts), 6, 6, 100.0, False, False)
    # exact mode evaluates j_l anywhere
    catana.sfb_decomposition(catana.PointContainer(pts), 6, 6, 100.0, False, False, interpolation="off")


def test_device_entry_point(cuda_device):
    """catana_gpu_sfb_raw_dev on device-resident tensors equals the host entry point."""
    torch = pytest.importorskip("torch")
    pts = uniform_ball(5000, 1000.0, seed=11)
    lmax, nmax = 10, 12
    host = catana.sfb_decomposition(catana.PointContainer(pts), lmax, nmax, 1000.0, True, False)
    d_pts = torch.from_numpy(pts).cuda()
    d_k = torch.zeros(lmax * nmax, dtype=torch.float64, device="cuda")
    d_c = torch.zeros_like(d_k)
    d_f = torch.zeros(2 * int(_lib.lib.catana_gpu_flmn_size(lmax, nmax)), dtype=torch.float64, device="cuda")
    st = _lib.lib.catana_gpu_sfb_raw_dev(ctypes.c_void_p(d_pts.data_ptr()), None, 5000, lmax, nmax, 1000.0, 0,
                                         ctypes.c_void_p(d_k.data_ptr()), ctypes.c_void_p(d_c.data_ptr()),
                                         ctypes.c_void_p(d_f.data_ptr()), None,
                                         ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0
    torch.cuda.synchronize()
    assert np.array_equal(d_k.cpu().numpy().reshape(lmax, nmax), host.k_ln)
    assert np.array_equal(d_c.cpu().numpy().reshape(lmax, nmax), host.c_ln)


@pytest.mark.parametrize("n,lmax,nmax,weighted", [
    (1500, 12, 20, False),
    (2500, 40, 70, True),     # 64-wide tiles in m and n, ragged
    (3000, 256, 128, True),   # the split form's headline shape: l up to 255, z up to ~670
])
def test_poly_jl_vs_oracle_exact(cuda_device, n, lmax, nmax, weighted):
    """CATANA_JL_POLY (piecewise FP64 polynomials, degree 11 per unit interval of
    z = k r) against the oracle with exact j_l on the same points: the same 1e-10 bar
    as the drop-in.  This mode is the FP64 reference the split form is measured
    against at full catalog sizes (the exact branch costs O(l) per j_l)."""
    pts = uniform_ball(n, 1000.0, seed=31 + n)
    w = np.random.default_rng(n).uniform(0.5, 1.5, n) if weighted else None
    res = catana.sfb_decomposition(catana.PointContainer(pts), lmax, nmax, 1000.0, True, False, weights=w,
                                   interpolation="poly")
    k, c, f = O.sfb_raw(pts, lmax, nmax, 1000.0, interpolated=False, weights=w)
    fmax = max(np.abs(x).max() for x in f)
    err = max(np.abs(a - b).max() for a, b in zip(res.f_lmn, f)) / fmax
    print("poly n=%d lmax=%d nmax=%d: max|df|/max|f| = %.2e" % (n, lmax, nmax, err))
    _compare(res, k, c, f)


def test_poly_jl_radius_beyond_rmax_and_domain(cuda_device):
    """The polynomial table is sized from the catalog's largest radius, so radii past
    rmax are fine (unlike the lerp table); a negative radius is a ValueError."""
    pts = uniform_ball(1200, 100.0, seed=4)
    pts[17, 0] = 400.0
    res = catana.sfb_decomposition(catana.PointContainer(pts), 6, 6, 100.0, True, False, interpolation="poly")
    k, c, f = O.sfb_raw(pts, 6, 6, 100.0, interpolated=False)
    _compare(res, k, c, f)
    pts[3, 0] = -1.0
    with pytest.raises(ValueError):
        catana.sfb_decomposition(catana.PointContainer(pts), 6, 6, 100.0, False, False, interpolation="poly")
