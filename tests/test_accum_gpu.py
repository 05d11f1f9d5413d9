"""Chunked accumulation (catana_gpu_accum_*): a catalog fed in chunks gives the
one-shot decomposition of the whole catalog.

Plain form: the same FP64 arithmetic, summed in a different order (<= 1e-12 of
max|f|).  Split form: against the one-shot split call and the FP64 plain path with
the split form's error measures.  float32 records: against the oracle on the same
float32 values widened to float64.
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


def _chunks(a, k):
    return np.array_split(a, k)


def test_accum_plain_equals_one_shot(cuda_device):
    pts = uniform_ball(9000, 800.0, seed=60)
    w = np.random.default_rng(60).uniform(0.5, 1.5, 9000)
    with catana.SFBAccumulator(24, 20, 800.0, precision="plain", interpolation="off") as acc:
        for p, ww in zip(_chunks(pts, 4), _chunks(w, 4)):
            acc.add(p, ww)
        r = acc.finish(store_flmn=True)
    one = catana.sfb_decomposition(catana.PointContainer(pts), 24, 20, 800.0, True, False, weights=w,
                                   interpolation="off")
    assert np.array_equal(r.k_ln, one.k_ln)
    fmax = max(np.abs(x).max() for x in one.f_lmn)
    assert max(np.abs(a - b).max() for a, b in zip(r.f_lmn, one.f_lmn)) <= 1e-12 * fmax
    assert np.allclose(r.c_ln, one.c_ln, rtol=1e-11, atol=0)


def test_accum_split_vs_one_shot_and_fp64(sm103):
    pts = uniform_ball(12000, 1000.0, seed=61)
    with catana.SFBAccumulator(64, 48, 1000.0, precision="split") as acc:
        for p in _chunks(pts, 3):
            acc.add(p)
        r = acc.finish(store_flmn=True)
    one = catana.sfb_decomposition(catana.PointContainer(pts), 64, 48, 1000.0, True, False, precision="split")
    fmax = max(np.abs(x).max() for x in one.f_lmn)
    assert max(np.abs(a - b).max() for a, b in zip(r.f_lmn, one.f_lmn)) <= 2e-6 * fmax
    rp = catana.sfb_decomposition(catana.PointContainer(pts), 64, 48, 1000.0, True, False, interpolation="off")
    _check(r, rp.f_lmn, rp.c_ln, "accum split 3 chunks")


def test_accum_float32_records_vs_oracle(sm103):
    pts32 = uniform_ball(6000, 1500.0, seed=62).astype(np.float32)
    w32 = np.random.default_rng(62).uniform(0.5, 1.5, 6000).astype(np.float32)
    with catana.SFBAccumulator(40, 30, 1500.0, precision="split") as acc:
        for p, ww in zip(_chunks(pts32, 2), _chunks(w32, 2)):
            acc.add(p, ww)
        r = acc.finish(store_flmn=True)
    k, c, f = O.sfb_raw(pts32.astype(np.float64), 40, 30, 1500.0, interpolated=False, weights=w32.astype(np.float64))
    assert np.array_equal(r.k_ln, k)
    _check(r, f, c, "accum float32 records")


def test_accum_float32_large_shape(sm103):
    """lmax = 512, nmax = 256 (extended Reinsch-modified rows, two radial halves) through
    float32 chunks."""
    form = "split"
    pts32 = uniform_ball(3000, 1500.0, seed=63).astype(np.float32)
    with catana.SFBAccumulator(512, 256, 1500.0, precision=form) as acc:
        for p in _chunks(pts32, 2):
            acc.add(p)
        r = acc.finish(store_flmn=True)
    rp = catana.sfb_decomposition(catana.PointContainer(pts32.astype(np.float64)), 512, 256, 1500.0, True, False,
                                  interpolation="off")
    _check(r, rp.f_lmn, rp.c_ln, "accum float32 lmax 512 nmax 256 %s" % form)


def test_accum_errors(cuda_device):
    pts = uniform_ball(100, 10.0, seed=64)
    acc = catana.SFBAccumulator(4, 4, 10.0, precision="plain")
    acc.add(pts)
    with pytest.raises(ValueError):
        acc.add(pts, np.ones(100))  # weights after an unweighted chunk
    with pytest.raises(ValueError):
        acc.add(pts, np.ones(7))
    acc.finish()
    with pytest.raises(ValueError):
        acc.finish()
    with pytest.raises(ValueError):
        acc.add(pts)
    acc.close()
    bad = pts.copy()
    bad[3, 0] = -1.0
    with catana.SFBAccumulator(4, 4, 10.0, precision="plain") as acc2:
        with pytest.raises(ValueError):
            acc2.add(bad)


def _survey(n, seed, rmax=1500.0, a=300.0):
    """float32 (r, theta, phi): radial pdf ~ r^2 exp(-(r/a)^2) cut at rmax, the band
    |theta - pi/2| < 20 deg masked out, phi uniform (the streamed survey's shape)."""
    rng = np.random.default_rng(seed)
    out = []
    smin = np.sin(np.deg2rad(20.0))
    while sum(len(x) for x in out) < n:
        r = a / np.sqrt(2.0) * np.sqrt((rng.standard_normal((n, 3)) ** 2).sum(1))
        r = r[r < rmax]
        ct = rng.uniform(smin, 1.0, r.size) * np.where(rng.random(r.size) < 0.5, -1.0, 1.0)
        out.append(np.stack([r, np.arccos(ct), rng.uniform(0.0, 2.0 * np.pi, r.size)], 1))
    return np.concatenate(out)[:n].astype(np.float32)


def test_accum_13_chunks_matches_one_shot(sm103):
    """The streamed survey's chunk count: 13 float32 chunks from pinned host memory
    (copies of chunk k+1 overlapping the decomposition of chunk k) give the one-shot
    split result of the whole catalog, and the split error measures against the FP64
    plain path (polynomial j_l) on the same float32 values."""
    torch = pytest.importorskip("torch")
    n, k = 26000, 13
    pts32 = _survey(n, seed=65)
    pinned = [torch.from_numpy(np.ascontiguousarray(c)).pin_memory() for c in _chunks(pts32, k)]
    lmax, nmax = 96, 64
    with catana.SFBAccumulator(lmax, nmax, 1500.0, precision="split") as acc:
        for c in pinned:
            acc.add(c.numpy())
        r = acc.finish(store_flmn=True)
    pts64 = pts32.astype(np.float64)
    one = catana.sfb_decomposition(catana.PointContainer(pts64), lmax, nmax, 1500.0, True, False, precision="split")
    fmax = max(np.abs(x).max() for x in one.f_lmn)
    assert max(np.abs(a - b).max() for a, b in zip(r.f_lmn, one.f_lmn)) <= 2e-6 * fmax
    rp = catana.sfb_decomposition(catana.PointContainer(pts64), lmax, nmax, 1500.0, True, False, interpolation="poly")
    fmax = max(np.abs(x).max() for x in rp.f_lmn)
    assert max(np.abs(a - b).max() for a, b in zip(r.f_lmn, rp.f_lmn)) <= 1e-5 * fmax
    # the radial profile leaves some (l, n) with j_l(k r) deep in its evanescent zone
    # at every point: compare C_ln above 1e-30 of the largest (FP32 operand range)
    keep = rp.c_ln >= 1e-30 * rp.c_ln.max()
    rel = np.abs(r.c_ln - rp.c_ln)[keep] / rp.c_ln[keep]
    print("accum split 13 chunks: C rel median %.2e p99 %.2e (%d of %d modes)" %
          (np.median(rel), np.percentile(rel, 99), keep.sum(), keep.size))
    assert keep.mean() > 0.9
    assert np.median(rel) <= 5e-7 and np.percentile(rel, 99) <= 2e-6
