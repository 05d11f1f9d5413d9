"""Bounded device-side waits of the split (tcgen05) kernel.

Every mbarrier wait in k_split_l gives up after a limit; the kernel then stops
issuing work, lets the copies and MMAs already in flight land (bounded as well),
frees its tensor memory and records CATANA_ERR_CUDA, which the entry point returns.
The reference has no such path (its GSL errors are switched off, sfb_raw.cpp:26).

The failure is made without faulting anything: catana_gpu_test_split_stall arms one
run in which every work item withholds the hand-off of its first tile's operands (a
flag that nothing sets), with the wait limit cut to a few milliseconds so that the
run ends quickly.  The test checks the returned status, then that the next run on
the same context -- which needs the tensor memory the aborted CTAs released -- is
normal and matches the oracle."""
import time

import numpy as np
import pytest

import catana_gb300 as catana
from catana_gb300 import _lib
from oracle import oracle as O
from conftest import uniform_ball
from test_raw_split_gpu import _check

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sm103(cuda_device):
    if tuple(cuda_device) != (10, 3):
        pytest.skip("split form needs sm_103")


def test_stalled_handoff_times_out_and_context_recovers(sm103):
    pts = uniform_ball(3000, 1000.0, seed=5)
    pc = catana.PointContainer(pts)
    lmax, nmax = 4, 8
    assert _lib.lib.catana_gpu_test_split_stall(3000) == _lib.OK  # 3 ms limit for the armed run
    t0 = time.perf_counter()
    with pytest.raises(_lib.CatanaError) as ei:
        catana.sfb_decomposition(pc, lmax, nmax, 1000.0, True, False, precision="split")
    dt = time.perf_counter() - t0
    assert "error 3" in str(ei.value) and "timed-out" in str(ei.value)
    assert dt < 30.0  # the waits ran out after milliseconds, not the 1 s default per CTA
    # the hook armed one run only: the same call now completes and matches the oracle
    res = catana.sfb_decomposition(pc, lmax, nmax, 1000.0, True, False, precision="split")
    k, c, f = O.sfb_raw(pts, lmax, nmax, 1000.0, interpolated=False)
    assert np.array_equal(res.k_ln, k)
    _check(res, f, c, "split after a timed-out run")
    # and a larger run on the same context (every SM's tensor memory in use again)
    pts2 = uniform_ball(20000, 1000.0, seed=6)
    res2 = catana.sfb_decomposition(catana.PointContainer(pts2), 40, 100, 1000.0, True, False, precision="split")
    k2, c2, f2 = O.sfb_raw(pts2, 40, 100, 1000.0, interpolated=False)
    _check(res2, f2, c2, "split n=20000 after a timed-out run")


def test_stall_hook_validates_its_argument():
    assert _lib.lib.catana_gpu_test_split_stall(0) == _lib.ERR_ARG
    assert _lib.lib.catana_gpu_test_split_stall(2000000) == _lib.ERR_ARG
