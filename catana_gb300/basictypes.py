"""Point, PointContainer and PixelizedPointContainer -- the input side of the
reference's Python API (python/py_basictypes.cpp), with the same constructors,
buffer layout and error behaviour.

* ``Point``: one (r, theta, phi) triple (Point.hpp:10-19).  ``Point(x, y, z)`` is
  the Cartesian constructor of Point.cpp:5-10: r = |v|, theta = atan2(rho, z),
  phi = atan2(y, x) reduced into [0, 2 pi).
* ``PointContainer``: an (N, 3) float64 row-major array of (r, theta, phi), the
  buffer the reference exposes through the buffer protocol (py_basictypes.cpp:126-135).
* ``PixelizedPointContainer(nside[, point_container])``: the catalog binned into
  HEALPix RING pixels (PixelizedPointContainer.cpp:11-30).  Binning runs on the GPU
  (``catana_gpu_bin_points``); the result is kept as CSR arrays (pixel offsets and
  radii grouped by pixel in point order).
"""
import numpy as np

from . import _lib

_TWO_PI = 2.0 * np.pi


def _cartesian_to_spherical(xyz):
    """Point(x, y, z) of Point.cpp:5-10 for an (N, 3) array."""
    x, y, z = xyz[:, 0], xyz[:, 1], xyz[:, 2]
    rho = np.sqrt(x * x + y * y)
    r = np.sqrt(x * x + y * y + z * z)
    theta = np.arctan2(rho, z)
    phi = np.where((x == 0.0) & (y == 0.0), 0.0, np.arctan2(y, x))
    phi = np.where(phi < 0.0, phi + _TWO_PI, phi)
    phi = np.where(phi >= _TWO_PI, np.fmod(phi, _TWO_PI), phi)
    return np.ascontiguousarray(np.stack([r, theta, phi], axis=1))


class Point(object):
    """Representation of a particle in 3-d space in spherical coordinates.

    ``Point()`` is the origin; ``Point(x, y, z)`` converts Cartesian coordinates.
    ``np.array(point)`` gives (r, theta, phi).
    """

    __slots__ = ("_rtp",)

    def __init__(self, x=None, y=None, z=None):
        if x is None and y is None and z is None:
            self._rtp = np.zeros(3)
        else:
            self._rtp = _cartesian_to_spherical(np.array([[x, y, z]], dtype=np.float64))[0]

    @classmethod
    def from_spherical(cls, r, theta, phi):
        p = cls()
        p._rtp = np.array([r, theta, phi], dtype=np.float64)
        return p

    def spherical(self):
        return (float(self._rtp[0]), float(self._rtp[1]), float(self._rtp[2]))

    def cartesian(self):
        r, th, ph = self._rtp
        st = np.sin(th)
        return (float(r * st * np.cos(ph)), float(r * st * np.sin(ph)), float(r * np.cos(th)))

    def __array__(self, dtype=None, copy=None):
        a = self._rtp.copy()
        return a if dtype is None else a.astype(dtype)

    def __repr__(self):
        return "Point(r=%g, theta=%g, phi=%g)" % tuple(self._rtp)


class PointContainer(object):
    """Collection of Points, stored as an (N, 3) float64 array of (r, theta, phi).

    ``PointContainer(coordinates, coordinate_type='spherical')`` with coordinates of
    shape (N, 3); 'cartesian' converts x, y, z like ``Point(x, y, z)``.
    """

    def __init__(self, coordinates=None, coordinate_type="spherical"):
        if coordinates is None:
            self._data = np.zeros((0, 3))
            return
        if coordinate_type == "cartesian":
            spherical = False
        elif coordinate_type == "spherical":
            spherical = True
        else:
            raise RuntimeError("coord_type either 'cartesian' or 'spherical'")
        arr = np.asarray(coordinates)
        if arr.ndim != 2:
            raise RuntimeError("Incompatible number of dimensions of array (needs 2)")
        if arr.shape[1] != 3:
            raise RuntimeError("Incompatible number of columns of array (needs 3)")
        if arr.dtype == np.float64 and arr.shape[0] > 1 and arr.strides[1] != arr.itemsize:
            raise RuntimeError("Data ordering of array is ColumnMajor, but RowMajor needed.")
        arr = np.ascontiguousarray(arr, dtype=np.float64)
        self._data = arr.copy() if spherical else _cartesian_to_spherical(arr)

    @classmethod
    def _from_array(cls, rtp):
        pc = cls()
        pc._data = np.ascontiguousarray(rtp, dtype=np.float64).reshape(-1, 3)
        return pc

    def __len__(self):
        return self._data.shape[0]

    def __getitem__(self, i):
        if i < 0 or i >= len(self):
            raise IndexError("index out of bounds!")
        return Point.from_spherical(*self._data[i])

    def add_point(self, point):
        self._data = np.concatenate([self._data, np.asarray(point, dtype=np.float64).reshape(1, 3)])

    def __array__(self, dtype=None, copy=None):
        return self._data if dtype is None else self._data.astype(dtype)

    @property
    def data(self):
        """The (N, 3) float64 (r, theta, phi) array (no copy)."""
        return self._data


def _is_power_of_2(n):
    return (n & (n - 1)) == 0


class PixelizedPointContainer(object):
    """A catalog binned into HEALPix RING pixels of resolution nside.

    ``PixelizedPointContainer(nside)`` is empty; ``PixelizedPointContainer(nside,
    point_container)`` bins every point (ang2pix on the GPU).  nside must be a power
    of two (ValueError otherwise, like the reference's std::invalid_argument).
    """

    def __init__(self, nside, point_container=None):
        nside = int(nside)
        if nside < 1 or not _is_power_of_2(nside):
            raise ValueError("argument (nside) must be a power of 2")
        self.nside = nside
        self.npix = 12 * nside * nside
        self.offsets = np.zeros(self.npix + 1, dtype=np.int64)
        self.r_sorted = np.zeros(0, dtype=np.float64)
        if point_container is not None:
            self._bin(np.asarray(point_container, dtype=np.float64).reshape(-1, 3))

    def _bin(self, pts):
        pts = np.ascontiguousarray(pts, dtype=np.float64)
        n = pts.shape[0]
        offs = np.zeros(self.npix + 1, dtype=np.int64)
        rs = np.zeros(max(n, 1), dtype=np.float64)
        st = _lib.lib.catana_gpu_bin_points(self.nside, _lib.ptr(pts), n, _lib.ptr(offs), _lib.ptr(rs), None)
        _lib.check(st, "bin_points")
        if self.r_sorted.size == 0:
            self.offsets, self.r_sorted = offs, rs[:n]
        else:  # merge: existing points first in every pixel (point order)
            self._merge(offs, rs[:n])

    def _merge(self, offs, rs):
        old_o, old_r = self.offsets, self.r_sorted
        new_counts = np.diff(old_o) + np.diff(offs)
        merged_o = np.zeros(self.npix + 1, dtype=np.int64)
        np.cumsum(new_counts, out=merged_o[1:])
        merged_r = np.empty(merged_o[-1], dtype=np.float64)
        for p in np.nonzero(new_counts)[0]:
            a = old_r[old_o[p]:old_o[p + 1]]
            b = rs[offs[p]:offs[p + 1]]
            merged_r[merged_o[p]:merged_o[p + 1]] = np.concatenate([a, b])
        self.offsets, self.r_sorted = merged_o, merged_r

    def add_point(self, point):
        self._bin(np.asarray(point, dtype=np.float64).reshape(1, 3))

    def get_nside(self):
        return self.nside

    def get_npoints(self):
        return int(self.offsets[-1])

    def get_countmap(self):
        """HEALPix RING map of the number of points per pixel (int32)."""
        return np.diff(self.offsets).astype(np.int32)

    def __len__(self):
        return self.npix


class FunctionInterpolator(object):
    """Linear interpolation of a function on equally spaced nodes
    (FunctionInterpolator.cpp:6-30; python/py_basictypes.cpp:173-215):
    ``FunctionInterpolator(fct, interpolation_points, x_min, x_max)``; calling it
    outside [x_min, x_max) raises ValueError.  The table also feeds the GPU integrals
    of ``besseltools.double_sbessel_integrator``."""

    def __init__(self, fct, interpolation_points, x_min, x_max):
        n = int(interpolation_points)
        if n < 2 or not (x_max > x_min):
            raise ValueError("need interpolation_points >= 2 and x_min < x_max")
        self.x_min, self.x_max, self.n = float(x_min), float(x_max), n
        dx = (self.x_max - self.x_min) / (n - 1)
        self._dx_inv = 1.0 / dx
        xs = self.x_min + np.arange(n) * dx
        try:
            ys = np.asarray(fct(xs), dtype=np.float64)
            if ys.shape != xs.shape:
                raise ValueError
        except Exception:
            ys = np.array([float(fct(float(x))) for x in xs])
        self.y_values = np.ascontiguousarray(ys)

    def __call__(self, x):
        x = float(x)
        if x < self.x_min or x >= self.x_max:
            raise ValueError("argument outside range for which this FunctionInterpolator is defined")
        ia = (x - self.x_min) * self._dx_inv
        i = int(ia)
        return float(self.y_values[i] + (self.y_values[i + 1] - self.y_values[i]) * (ia - i))
