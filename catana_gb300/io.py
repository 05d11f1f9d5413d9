"""Raw binary point files: the reference's RawBinarySource / RawBinarySink record
format (RawBinarySource.cpp:6-61, RawBinarySink.cpp:6-62, record_types.hpp:15-160):
consecutive fixed-size records of three float32 or float64 values, either Cartesian
(x, y, z) -- read back through Point(x, y, z) -- or spherical (r, theta, phi), with no
header.  Large files are better streamed to the GPU with
``SFBAccumulator.add_file``."""
import numpy as np

from .basictypes import PointContainer, _cartesian_to_spherical


def _dt(dtype):
    dt = np.dtype(dtype)
    if dt not in (np.dtype(np.float32), np.dtype(np.float64)):
        raise ValueError("dtype must be float32 or float64")
    return dt


def read_raw_binary(filename, record="spherical", dtype=np.float32):
    """All records of a raw binary file as a PointContainer (a trailing partial record
    is ignored, as the reference counts size / sizeof(record))."""
    dt = _dt(dtype)
    raw = np.fromfile(filename, dtype=dt)
    raw = raw[:raw.size - raw.size % 3].reshape(-1, 3).astype(np.float64)
    if record == "cartesian":
        return PointContainer(_cartesian_to_spherical(raw))
    if record != "spherical":
        raise ValueError("record must be 'spherical' or 'cartesian'")
    return PointContainer(raw)


def write_raw_binary(filename, points, record="spherical", dtype=np.float32, append=False):
    """Write points (PointContainer or (N, 3) r, theta, phi) as raw binary records;
    Cartesian records are r (sin t cos p, sin t sin p, cos t) (CartesianRecord(point, 0))."""
    dt = _dt(dtype)
    rtp = np.asarray(points, dtype=np.float64).reshape(-1, 3)
    if record == "cartesian":
        r, t, p = rtp[:, 0], rtp[:, 1], rtp[:, 2]
        out = np.stack([r * np.sin(t) * np.cos(p), r * np.sin(t) * np.sin(p), r * np.cos(t)], axis=1)
    elif record == "spherical":
        out = rtp
    else:
        raise ValueError("record must be 'spherical' or 'cartesian'")
    with open(filename, "ab" if append else "wb") as fh:
        np.ascontiguousarray(out, dtype=dt).tofile(fh)
