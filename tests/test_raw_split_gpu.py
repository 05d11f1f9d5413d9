"""The split-precision tensor-core form (tcgen05, 3-term FP16 hi+lo products, FP32
accumulation folded per 32-point tile, FP32 partial per work item, FP64 across items)
against the FP64 oracle with exact j_l (or, at sizes the oracle does not finish in seconds,
the FP64 GPU path with j_l from its FP64 polynomials, itself pinned to the oracle).
Both split variants: the default three-term Legendre rows and the Reinsch-modified
rows of CATANA_SPLIT_ACCURATE.

Error measures (measured values are ~2e-7 median, ~6e-7 p99 on 100k points):
  C_ln   median relative error <= 5e-7 and 99th percentile <= 2e-6; every entry
         within 1e-5 of max(C_ln, median_n C_l) -- a single C_ln can be
         statistically tiny (a chi-square draw over 2l+1 complex terms), which
         inflates its own relative error without a larger absolute error;
  f_lmn  max |df| <= 1e-5 max|f|, and per l: rms(df) <= 2e-5 rms(f_l).
"""
import numpy as np
import pytest

import catana_gb300 as catana
from oracle import oracle as O
from conftest import uniform_ball

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sm103(cuda_device):
    if tuple(cuda_device) != (10, 3):
        pytest.skip("split form needs sm_103")


def _check(res, f, c, tag):
    fmax = max(np.abs(x).max() for x in f)
    ef = max(np.abs(a - b).max() for a, b in zip(res.f_lmn, f)) / fmax
    efl = max(np.sqrt(np.mean(np.abs(a - b) ** 2) / np.mean(np.abs(b) ** 2)) for a, b in zip(res.f_lmn, f))
    rel = np.abs(res.c_ln - c) / np.abs(c)
    typ = np.abs(res.c_ln - c) / np.maximum(np.abs(c), np.median(c, axis=1, keepdims=True))
    print("%s: max|df|/max|f|=%.2e max_l rms(df)/rms(f)=%.2e | C rel: median %.2e p99 %.2e max %.2e | "
          "max |dC|/max(C, median_l C) %.2e" % (tag, ef, efl, np.median(rel), np.percentile(rel, 99), rel.max(), typ.max()))
    assert ef <= 1e-5
    assert efl <= 2e-5
    assert np.median(rel) <= 5e-7
    assert np.percentile(rel, 99) <= 2e-6
    assert typ.max() <= 1e-5


FORMS = ["split", "split_accurate"]


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("n,lmax,nmax,weighted", [
    (3000, 8, 8, False),
    (5000, 33, 20, True),
    (2000, 130, 64, False),   # l >= 128: two m-blocks per slab
    (20000, 40, 100, False),  # several tiles per CTA: per-tile folds
    (3000, 24, 200, True),    # nmax > 128: two radial halves
])
def test_split_vs_oracle(sm103, n, lmax, nmax, weighted, form):
    pts = uniform_ball(n, 1000.0, seed=100 + n)
    w = np.random.default_rng(n).uniform(0.5, 1.5, n) if weighted else None
    res = catana.sfb_decomposition(catana.PointContainer(pts), lmax, nmax, 1000.0, True, False,
                                   weights=w, precision=form)
    k, c, f = O.sfb_raw(pts, lmax, nmax, 1000.0, interpolated=False, weights=w)
    assert np.array_equal(res.k_ln, k)
    _check(res, f, c, "%s n=%d lmax=%d nmax=%d" % (form, n, lmax, nmax))


@pytest.mark.parametrize("form", FORMS)
def test_split_full_shape_vs_fp64_gpu(sm103, form):
    """lmax=256, nmax=128 (the precision form's headline shape) on a 20k-point
    subsample of the uniform ball with weights U[0.5,1.5]: split vs the plain FP64
    GPU path in exact-j_l mode (itself pinned to the oracle)."""
    n = 20000
    pts = uniform_ball(n, 1000.0, seed=2)
    w = np.random.default_rng(2).uniform(0.5, 1.5, n)
    pc = catana.PointContainer(pts)
    rs = catana.sfb_decomposition(pc, 256, 128, 1000.0, True, False, weights=w, precision=form)
    rp = catana.sfb_decomposition(pc, 256, 128, 1000.0, True, False, weights=w, interpolation="poly")
    _check(rs, rp.f_lmn, rp.c_ln, "%s lmax=256 nmax=128 n=20000" % form)


@pytest.mark.parametrize("form", FORMS)
def test_split_long_items_vs_fp64_gpu(sm103, form):
    """2M points: about 400 tiles per work item, so each item folds into its TMEM sum
    and flushes it into its running FP32 partial several times (read-modify-write of
    the partial) before the last flush; split vs the plain FP64 GPU path with exact j_l
    on the same points.  At this size the catalog's monopole (a sum that grows like N)
    leaks through any error of Y_l0 with a nonzero mean over the sphere; the m = 0
    Legendre steps round A x P_{l-1} - B P_{l-2} once for that reason."""
    n = 2_000_000
    pts = uniform_ball(n, 1000.0, seed=77)
    w = np.random.default_rng(77).uniform(0.5, 1.5, n)
    pc = catana.PointContainer(pts)
    rs = catana.sfb_decomposition(pc, 64, 32, 1000.0, True, False, weights=w, precision=form)
    rp = catana.sfb_decomposition(pc, 64, 32, 1000.0, True, False, weights=w, interpolation="poly")
    _check(rs, rp.f_lmn, rp.c_ln, "%s lmax=64 nmax=32 n=2M" % form)


def test_split_multi_chunk_linearity(sm103):
    """f is a sum over points: the split result for A+B equals the weighted
    combination of the results for A and B (size-independent property)."""
    pts = uniform_ball(8000, 500.0, seed=9)
    a, b = pts[:3000], pts[3000:]
    pc = catana.PointContainer
    r_all = catana.sfb_decomposition(pc(pts), 16, 16, 500.0, True, False, precision="split")
    r_a = catana.sfb_decomposition(pc(a), 16, 16, 500.0, True, False, precision="split")
    r_b = catana.sfb_decomposition(pc(b), 16, 16, 500.0, True, False, precision="split")
    fmax = max(np.abs(x).max() for x in r_all.f_lmn)
    for fa, fb, ft in zip(r_a.f_lmn, r_b.f_lmn, r_all.f_lmn):
        # f carries V/N: recombine with the point counts
        comb = (fa * 3000 + fb * 5000) / 8000
        assert np.abs(comb - ft).max() <= 1e-5 * fmax
