"""The HEALPix SFB at its full workload size -- nside 256, 1M points (90% uniform in a
ball of radius 1000, 10% in 1000 Gaussian clumps of sigma 5, seed 1), lmax 128, nmax
64 -- against the FFT form of the oracle's restatement of sfb_reverse_fft.cpp:43-209
(per-ring r2c transforms, as the reference computes them), at the bar of the smaller
HEALPix parity tests: f_lmn within 1e-10 of max|f|, C_ln to rtol 1e-9.  Here every
path of the GPU ring transform is exercised at scale: the FFT on the 513 equatorial
rings of 1024 pixels once l + 1 > 36, the folded direct sums on the polar rings, the
range-proven map levels.  The oracle needs one to two minutes of host CPU."""
import numpy as np
import pytest

import catana_gb300 as catana
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _catalog(n=1_000_000, radius=1000.0, seed=1):
    rng = np.random.default_rng(seed)
    nu = int(0.9 * n)
    nc = n - nu

    def ball(k):
        r = radius * rng.random(k) ** (1 / 3)
        ct = rng.uniform(-1, 1, k)
        ph = rng.uniform(0, 2 * np.pi, k)
        st = np.sqrt(1 - ct ** 2)
        return np.stack([r * st * np.cos(ph), r * st * np.sin(ph), r * ct], 1)

    xyz = [ball(nu)]
    centres = ball(1000)
    got = 0
    while got < nc:
        p = centres[rng.integers(0, 1000, nc)] + rng.normal(0, 5.0, (nc, 3))
        p = p[np.sum(p ** 2, 1) < radius ** 2][:nc - got]
        xyz.append(p)
        got += p.shape[0]
    return np.concatenate(xyz)


def test_healpix_full_size_vs_fft_oracle(cuda_device):
    radius = 1000.0
    ppc = catana.PixelizedPointContainer(256, catana.PointContainer(_catalog(radius=radius), "cartesian"))
    res = catana.sfb_decomposition(ppc, 128, 64, radius, True, False)
    k, c, f = O.sfb_healpix_fft(256, ppc.offsets, ppc.r_sorted, 128, 64, radius, interpolated=True)
    assert np.array_equal(res.k_ln, k)
    fmax = max(np.abs(x).max() for x in f)
    err = max(np.abs(a - b).max() for a, b in zip(res.f_lmn, f)) / fmax
    print("nside 256, 1M points, lmax 128, nmax 64: max|df|/max|f| = %.2e" % err)
    assert err <= 1e-10
    assert np.allclose(res.c_ln, c, rtol=1e-9, atol=0)
