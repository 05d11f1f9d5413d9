"""Batched raw decomposition (catana_gpu_sfb_raw_batched): catalogs of uneven size,
lmax, rmax and kmax cut in one call.

Each catalog's result is checked against the FP64 oracle run on that catalog alone
(exact j_l), with the split form's error measures restricted to the modes the kmax
cut keeps (k_ln <= kmax); the cut modes must be exactly zero.  The plain form must
equal the single-catalog plain call bit for bit on the kept modes.
"""
import numpy as np
import pytest

import catana_gb300 as catana
from catana_gb300 import _lib
from oracle import oracle as O
from conftest import uniform_ball

pytestmark = pytest.mark.gpu

# (n, lmax, nmax, rmax, kmax)
CATS = [
    (700, 12, 24, 500.0, 0.05),
    (3000, 40, 32, 1500.0, 0.05),
    (12000, 20, 48, 1000.0, 0.0),
    (40, 8, 8, 800.0, 0.0),
    (5000, 33, 40, 1200.0, 0.08),
    (1500, 130, 16, 600.0, 0.0),   # l >= 128: two m-blocks
]


@pytest.fixture(scope="module")
def sm103(cuda_device):
    if tuple(cuda_device) != (10, 3):
        pytest.skip("split form needs sm_103")


@pytest.fixture(scope="module")
def batch():
    pts, ws, ref = [], [], []
    for i, (n, lmax, nmax, rmax, kmax) in enumerate(CATS):
        p = uniform_ball(n, rmax, seed=300 + i)
        w = np.random.default_rng(300 + i).uniform(0.5, 1.5, n) if i % 2 else None
        pts.append(p)
        ws.append(w)
        ref.append(O.sfb_raw(p, lmax, nmax, rmax, interpolated=False, weights=w))
    return pts, ws, ref


def _run(pts, ws, precision="split", waves=2.0, graph=True, mblock=128):
    return catana.sfb_decomposition_batched(
        [catana.PointContainer(p) for p in pts], [c[1] for c in CATS], [c[2] for c in CATS],
        [c[3] for c in CATS], kmax=[c[4] for c in CATS], weights=ws, store_flmn=True, verbose=False,
        precision=precision, waves=waves, graph=graph, mblock=mblock)


def _keep(k, kmax):
    return np.ones_like(k, dtype=bool) if kmax <= 0 else (k <= kmax)


def _check_cut(res, k, c, f, kmax, tag):
    keep = _keep(k, kmax)
    assert np.array_equal(res.k_ln, k)
    # cut modes: exactly zero
    assert np.all(res.c_ln[~keep] == 0.0)
    for l, fl in enumerate(res.f_lmn):
        assert np.all(fl[:, ~keep[l]] == 0.0)
    # kept modes: the split form's error measures
    fk = [fl[:, keep[l]] for l, fl in enumerate(f) if keep[l].any()]
    rk = [fl[:, keep[l]] for l, fl in enumerate(res.f_lmn) if keep[l].any()]
    fmax = max(np.abs(x).max() for x in fk)
    ef = max(np.abs(a - b).max() for a, b in zip(rk, fk)) / fmax
    efl = max(np.sqrt(np.mean(np.abs(a - b) ** 2) / np.mean(np.abs(b) ** 2)) for a, b in zip(rk, fk))
    ck, rc = c[keep], res.c_ln[keep]
    rel = np.abs(rc - ck) / np.abs(ck)
    med_l = np.array([np.median(c[l][keep[l]]) if keep[l].any() else 0.0 for l in range(c.shape[0])])
    typ = np.abs(res.c_ln - c) / np.maximum(np.abs(c), med_l[:, None])
    typ = typ[keep]
    print("%s: max|df|/max|f|=%.2e max_l rms %.2e | C rel median %.2e p99 %.2e | typ %.2e" %
          (tag, ef, efl, np.median(rel), np.percentile(rel, 99), typ.max()))
    assert ef <= 1e-5
    assert efl <= 2e-5
    assert np.median(rel) <= 5e-7
    assert np.percentile(rel, 99) <= 2e-6
    assert typ.max() <= 1e-5


def test_batched_split_vs_oracle(sm103, batch):
    pts, ws, ref = batch
    res = _run(pts, ws)
    for i, (r, (k, c, f)) in enumerate(zip(res, ref)):
        _check_cut(r, k, c, f, CATS[i][4], "catalog %d %s" % (i, CATS[i]))


def test_batched_graph_equals_direct_launches(sm103, batch):
    """The CUDA-graph replay and direct launches of the same schedule are bit-identical."""
    pts, ws, _ = batch
    a = _run(pts, ws, waves=3.0, graph=True)
    b = _run(pts, ws, waves=3.0, graph=False)
    for x, y in zip(a, b):
        assert np.array_equal(x.c_ln, y.c_ln)
        for fx, fy in zip(x.f_lmn, y.f_lmn):
            assert np.array_equal(fx, fy)


def test_batched_mblock64(sm103, batch):
    """Work items of at most 64 complex m (the MMA tile's N = 128): levels l >= 64 split
    into two or three m-blocks; every catalog keeps the bar against the oracle."""
    pts, ws, ref = batch
    res = _run(pts, ws, waves=2.0, mblock=64)
    assert _lib.lib.catana_gpu_batch_mblk() == 64
    for i, (r, (k, c, f)) in enumerate(zip(res, ref)):
        _check_cut(r, k, c, f, CATS[i][4], "mblock 64 catalog %d" % i)
    with pytest.raises(ValueError):
        _run(pts, ws, mblock=32)


def test_batched_autotune(sm103, batch):
    """waves <= 0 picks a schedule and a tile shape from the candidate sets; the result
    keeps the bar."""
    pts, ws, ref = batch
    res = _run(pts, ws, waves=0.0)
    assert _lib.lib.catana_gpu_batch_waves() in (1.0, 2.0, 3.0, 4.0, 6.0, 8.0, 12.0)
    assert _lib.lib.catana_gpu_batch_mblk() in (128, 64)
    for i, (r, (k, c, f)) in enumerate(zip(res, ref)):
        _check_cut(r, k, c, f, CATS[i][4], "autotuned catalog %d" % i)
    again = _run(pts, ws, waves=0.0)  # cached choice: same schedule, same bits
    for x, y in zip(res, again):
        assert np.array_equal(x.c_ln, y.c_ln)


def test_batched_matches_single_split(sm103, batch):
    """A catalog decomposed alone and inside the batch agree to the split form's accuracy."""
    pts, ws, _ = batch
    res = _run(pts, ws)
    i = 2  # no cut
    n, lmax, nmax, rmax, _k = CATS[i]
    single = catana.sfb_decomposition(catana.PointContainer(pts[i]), lmax, nmax, rmax, True, False,
                                      weights=ws[i], precision="split")
    fmax = max(np.abs(x).max() for x in single.f_lmn)
    for a, b in zip(res[i].f_lmn, single.f_lmn):
        assert np.abs(a - b).max() <= 2e-6 * fmax


def test_batched_plain_equals_single_plain(cuda_device, batch):
    pts, ws, _ = batch
    res = _run(pts, ws, precision="plain")
    for i, r in enumerate(res):
        n, lmax, nmax, rmax, kmax = CATS[i]
        s = catana.sfb_decomposition(catana.PointContainer(pts[i]), lmax, nmax, rmax, True, False, weights=ws[i])
        keep = _keep(s.k_ln, kmax)
        assert np.array_equal(r.k_ln, s.k_ln)
        assert np.array_equal(r.c_ln[keep], s.c_ln[keep])
        assert np.all(r.c_ln[~keep] == 0.0)
        for l in range(lmax):
            assert np.array_equal(r.f_lmn[l][:, keep[l]], s.f_lmn[l][:, keep[l]])
            assert np.all(r.f_lmn[l][:, ~keep[l]] == 0.0)


def test_batched_empty_catalog(sm103):
    """An empty catalog in a batch gives what the single call gives (NaN from N = 0,
    like the reference's normalisation) and leaves the others untouched."""
    p = uniform_ball(2000, 700.0, seed=5)
    pcs = [catana.PointContainer(p), catana.PointContainer(np.zeros((0, 3))), catana.PointContainer(p)]
    res = catana.sfb_decomposition_batched(pcs, 10, 12, 700.0, store_flmn=True, verbose=False, waves=1.0)
    alone = catana.sfb_decomposition(catana.PointContainer(np.zeros((0, 3))), 10, 12, 700.0, False, False,
                                     precision="split")
    assert np.array_equal(res[1].c_ln, alone.c_ln, equal_nan=True)
    assert np.array_equal(res[0].c_ln, res[2].c_ln)
