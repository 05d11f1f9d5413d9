"""The allocation-free entry point, catana_gpu_sfb_raw_noalloc.

Some callers cannot allocate device memory: code running inside a caller-owned
memory pool or under a fixed memory budget, or code that must not trigger the
implicit device synchronisation of cudaMalloc/cudaFree.  For them the library runs
the plain FP64 raw path out of one static 32 MiB device array per device.  This
test calls that entry point twice in a row through the C ABI (different catalogs,
weights and shapes, so stale scratch from the first call would show) and checks
each result against the allocating entry point catana_gpu_sfb_raw_dev with the
tolerance the plain-path tests use: identical k_ln, f_lmn within 1e-10 of max|f|,
C_ln within 1e-9 relative.  The file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

from catana_gb300 import _lib
from conftest import uniform_ball

pytestmark = pytest.mark.gpu


def _run(entry, pts, w, lmax, nmax, rmax, torch):
    n = pts.shape[0]
    d_pts = torch.from_numpy(pts).cuda()
    d_w = torch.from_numpy(w).cuda() if w is not None else None
    fc = int(_lib.lib.catana_gpu_flmn_size(lmax, nmax))
    d_k = torch.zeros(lmax * nmax, dtype=torch.float64, device="cuda")
    d_c = torch.zeros_like(d_k)
    d_f = torch.full((2 * fc,), float("nan"), dtype=torch.float64, device="cuda")
    sp = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    wp = ctypes.c_void_p(d_w.data_ptr()) if d_w is not None else None
    args = [ctypes.c_void_p(d_pts.data_ptr()), wp, n, lmax, nmax, rmax, _lib.JL_AUTO,
            ctypes.c_void_p(d_k.data_ptr()), ctypes.c_void_p(d_c.data_ptr()), ctypes.c_void_p(d_f.data_ptr())]
    if entry == "noalloc":
        st = _lib.lib.catana_gpu_sfb_raw_noalloc(*args, sp)
    else:
        st = _lib.lib.catana_gpu_sfb_raw_dev(*args, None, sp)
    _lib.check(st, entry)
    torch.cuda.synchronize()
    return d_k.cpu().numpy(), d_c.cpu().numpy(), d_f.cpu().numpy()


def test_noalloc_matches_allocating_entry_twice(cuda_device):
    torch = pytest.importorskip("torch")
    cases = [
        (uniform_ball(20000, 1000.0, seed=0), np.random.default_rng(0).uniform(0.5, 1.5, 20000), 32, 32, 1000.0),
        (uniform_ball(3000, 250.0, seed=1), None, 16, 20, 250.0),
        # about 26k points fit the fixed array per chunk at lmax = nmax = 32: 60k points
        # run the chunk loop three times (Legendre rows restarted, partials accumulated)
        (uniform_ball(60000, 1000.0, seed=2), np.random.default_rng(2).uniform(0.5, 1.5, 60000), 32, 32, 1000.0),
    ]
    for pts, w, lmax, nmax, rmax in cases:
        k0, c0, f0 = _run("dev", pts, w, lmax, nmax, rmax, torch)
        k1, c1, f1 = _run("noalloc", pts, w, lmax, nmax, rmax, torch)
        assert np.array_equal(k0, k1)
        fmax = np.abs(f0).max()
        assert np.all(np.isfinite(f1))
        assert np.abs(f1 - f0).max() <= 1e-10 * fmax
        assert np.max(np.abs(c1 - c0) / np.abs(c0)) <= 1e-9


def test_noalloc_rejects_oversize(cuda_device):
    torch = pytest.importorskip("torch")
    d = torch.zeros(64 * 64, dtype=torch.float64, device="cuda")
    st = _lib.lib.catana_gpu_sfb_raw_noalloc(ctypes.c_void_p(d.data_ptr()), None, 2000, 64, 64, 1.0,
                                             _lib.JL_INTERP, ctypes.c_void_p(d.data_ptr()),
                                             ctypes.c_void_p(d.data_ptr()), ctypes.c_void_p(d.data_ptr()), None)
    assert st == _lib.ERR_ARG
    assert "MiB" in _lib.last_error()
