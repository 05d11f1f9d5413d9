"""besseltools: zeros of the spherical Bessel functions (python/py_besseltools.cpp:15-44).

``SphericalBesselZeros(l)[n]`` returns the n-th zero of j_l computed exactly as the
reference's SphericalBesselZeros (SphericalBesselZeros.cpp:11-100), including its
Newton stopping rule; the zeros are cached per process by the library.
"""
import ctypes

import numpy as np

from . import _lib
from .basictypes import FunctionInterpolator


class SphericalBesselZeros(object):
    """Root generator for j_l at a fixed multipole l."""

    def __init__(self, l):
        if isinstance(l, bool) or not isinstance(l, (int, np.integer)) or l < 0:
            raise TypeError("l must be a non-negative integer")
        self.l = int(l)
        self._z = np.zeros(0)

    def _ensure(self, count):
        if self._z.size < count:
            out = np.zeros(count)
            _lib.check(_lib.lib.catana_gpu_sbessel_zeros(self.l, count, _lib.ptr(out)), "sbessel_zeros")
            self._z = out

    def __getitem__(self, n):
        n = int(n)
        if n < 0:
            raise IndexError("zero index must be >= 0")
        self._ensure(n + 1)
        return float(self._z[n])

    def compute_up_to(self, z_max):
        """Compute zeros until the largest exceeds z_max (SphericalBesselZeros.cpp:70-74)."""
        count = max(2, self._z.size)
        self._ensure(count)
        while self._z[-1] < z_max:
            count *= 2
            self._ensure(count)

    def next_zero(self, z):
        """Index of the first zero above z (SphericalBesselZeros.cpp:76-80)."""
        self.compute_up_to(z)
        return int(np.argmax(self._z > z))


def double_sbessel_integrator(w, l, r_max, k1, k2):
    """int_0^r_max w(r) j_l(k1 r) j_l(k2 r) dr (py_besseltools.cpp:45-84), vectorised in
    k1, k2 and computed on the GPU in one batch.  w: a FunctionInterpolator (used as is)
    or a callable, tabulated here on 2^18 + 1 equally spaced nodes of [0, r_max]
    (linear between them, error ~1e-10 of the integral for smooth w)."""
    if isinstance(w, FunctionInterpolator):
        fi = w
    else:
        fi = FunctionInterpolator(w, (1 << 18) + 1, 0.0, float(r_max) * (1.0 + 1e-12))
    if isinstance(l, bool) or not isinstance(l, (int, np.integer)) or l < 0:
        raise TypeError("l must be a non-negative integer")
    a, b = np.broadcast_arrays(np.asarray(k1, dtype=np.float64), np.asarray(k2, dtype=np.float64))
    shape = a.shape
    a = np.ascontiguousarray(a.ravel())
    b = np.ascontiguousarray(b.ravel())
    out = np.zeros(max(a.size, 1))
    _lib.check(_lib.lib.catana_gpu_sbessel_integrals(_lib.ptr(fi.y_values), fi.n, fi.x_min, fi.x_max, int(l),
                                                     float(r_max), _lib.ptr(a), _lib.ptr(b), a.size, _lib.ptr(out),
                                                     None), "sbessel_integrals")
    res = out[:a.size].reshape(shape)
    return float(res) if res.ndim == 0 else res
