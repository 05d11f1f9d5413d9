"""Batched double spherical-Bessel integrals on the GPU against the oracle (adaptive
Gauss-Legendre to 1e-14 on the same breakpoints) and the reference's own known values
(besseltools_test.py:26-58)."""
import numpy as np
import pytest

import catana_gb300 as catana
from catana_gb300 import besseltools
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_known_values(cuda_device):
    w = lambda r: np.ones_like(r)
    assert besseltools.double_sbessel_integrator(w, 0, 100, 1, 1) == pytest.approx(1.56582, abs=1e-5)
    assert besseltools.double_sbessel_integrator(w, 0, 100, 1, 2) == pytest.approx(0.785393, abs=1e-5)
    assert besseltools.double_sbessel_integrator(w, 4, 100, 1, 4.2) == pytest.approx(0.000133933, abs=1e-9)


def test_symmetric_and_interpolator(cuda_device):
    w = lambda r: np.exp(-(r / 40) ** 2) * r ** 2
    r1 = besseltools.double_sbessel_integrator(w, 6, 100, 2.3, 4.5)
    r2 = besseltools.double_sbessel_integrator(w, 6, 100, 4.5, 2.3)
    assert r1 == r2
    fi = catana.FunctionInterpolator(w, 100000, 0, 100)
    assert besseltools.double_sbessel_integrator(fi, 6, 100, 2.3, 4.5) == pytest.approx(r1, rel=1e-5)


@pytest.mark.parametrize("l,rmax,nodes,nk", [(0, 100.0, 20001, 6), (6, 100.0, 20001, 6), (20, 1000.0, 8001, 5),
                                          (100, 1000.0, 4001, 4)])
def test_vs_oracle(cuda_device, l, rmax, nodes, nk):
    """A batch of (k1, k2) pairs: zeros-of-j_l wave numbers as in a C_l^SN matrix."""
    fi = catana.FunctionInterpolator(lambda r: np.exp(-(r / (0.4 * rmax)) ** 2) * r ** 2, nodes, 0.0, rmax)
    k = catana.compute_kln(l + 1, nk, rmax)[l]
    k1, k2 = np.meshgrid(k, k)
    got = besseltools.double_sbessel_integrator(fi, l, rmax, k1, k2)
    scale = np.max(np.abs(got))
    for i in range(nk):
        for j in range(nk):
            ref = O.dsb_integral(fi.y_values, (fi.x_min, fi.x_max), l, rmax, k1[i, j], k2[i, j])
            assert abs(got[i, j] - ref) <= 1e-10 * scale, (i, j, got[i, j], ref)
