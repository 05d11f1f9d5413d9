"""sfb_decomposition and KClkk -- the decomposition module of the reference's
Python API (python/py_decomposition.cpp), over the C ABI of libcatana_gpu.

``sfb_decomposition(point_container, lmax, nmax, rmax, store_flmn=False,
verbose=True)`` is the raw (direct-sum) method (py_decomposition.cpp:114-133,
sfb_decomposition.cpp:15-19); called with a ``PixelizedPointContainer`` it is the
HEALPix method (py_decomposition.cpp:135-153, sfb_decomposition.cpp:22-26).
``sfb_decomposition_healpix`` is an alias of the second form.

Keyword extensions (absent in the reference, defaults reproduce it):
  weights=None         per-point weights; f is normalised by V/sum(w)
  precision='plain'    'plain': FP64 on CUDA cores (the drop-in);
                       'split': tcgen05 tensor cores, 3-term FP16 hi+lo products;
                       'split_accurate': the same with Reinsch-modified Legendre
                       rows: half the f_lmn error at high l (ten times less near
                       the poles), ~12% slower; above lmax 256 'split' always
                       takes these rows
  interpolation='auto' 'auto' (interpolated iff N > 1000, the reference's rule),
                       'on' (linear table), 'off' (exact j_l) or 'poly' (piecewise
                       FP64 polynomials, as accurate as 'off' at the cost of 'on';
                       raw path, plain form)
  conj_fix=False       HEALPix only: conjugate aliased ring coefficients instead of
                       reproducing the reference's unconjugated read.
"""
import ctypes
import sys
import time

import numpy as np

from . import _lib
from .basictypes import PixelizedPointContainer, PointContainer

_INTERP = {"auto": _lib.JL_AUTO, "on": _lib.JL_INTERP, "off": _lib.JL_EXACT, "poly": _lib.JL_POLY}
_FORM = {"plain": _lib.FORM_PLAIN, "split": _lib.FORM_SPLIT,
         "split_accurate": _lib.FORM_SPLIT | _lib.SPLIT_ACCURATE}


class KClkk(object):
    """Return type of the SFB decomposition methods (return_types.hpp:19-38).

    k_ln, c_ln: (lmax, nmax) float64, read-only.  f_lmn: list over l of (l+1, nmax)
    complex128 arrays (empty unless store_flmn).
    """

    def __init__(self, k_ln, c_ln, f_lmn):
        k_ln.setflags(write=False)
        c_ln.setflags(write=False)
        self._k, self._c, self._f = k_ln, c_ln, f_lmn

    @property
    def k_ln(self):
        return self._k

    @property
    def c_ln(self):
        return self._c

    @property
    def f_lmn(self):
        return self._f

    def savetxt(self, filename_base):
        """Write filename_base + '.k_ln' and '.c_ln' (rows l, columns n), '%.18e'
        separated by single spaces (return_types.cpp:27-64)."""
        for suffix, arr in ((".k_ln", self._k), (".c_ln", self._c)):
            with open(filename_base + suffix, "w") as fh:
                for row in arr:
                    fh.write(" ".join("%.18e" % v for v in row) + "\n")


def _unsigned_short(v, name):
    if isinstance(v, bool) or not isinstance(v, (int, np.integer)) or not (0 <= int(v) <= 65535):
        raise TypeError("%s must be an integer in [0, 65535] (C++ unsigned short)" % name)
    return int(v)


def unpack_flmn(flat, lmax, nmax):
    """Split the packed complex f_lmn buffer into the list of (l+1, nmax) arrays."""
    out, off = [], 0
    for l in range(lmax):
        s = (l + 1) * nmax
        out.append(flat[off:off + s].reshape(l + 1, nmax).copy())
        off += s
    return out


def _flags(interpolation, precision):
    if interpolation not in _INTERP:
        raise ValueError("interpolation must be one of %s" % sorted(_INTERP))
    if precision not in _FORM:
        raise ValueError("precision must be one of %s" % sorted(_FORM))
    return _INTERP[interpolation] | _FORM[precision]


def _raw(pc, lmax, nmax, rmax, store_flmn, verbose, weights, precision, interpolation):
    pts = np.ascontiguousarray(np.asarray(pc, dtype=np.float64).reshape(-1, 3))
    n = pts.shape[0]
    w = None
    if weights is not None:
        w = np.ascontiguousarray(weights, dtype=np.float64).reshape(-1)
        if w.shape[0] != n:
            raise ValueError("weights must have one entry per point")
    if verbose:
        print("SFB decomposition (raw method): lmax=%d nmax=%d Rmax=%s" % (lmax, nmax, rmax))
        print("Catalog consists of %d points." % n)
        sys.stdout.flush()
    t0 = time.perf_counter()
    k = np.zeros((lmax, nmax))
    c = np.zeros((lmax, nmax))
    fsize = int(_lib.lib.catana_gpu_flmn_size(lmax, nmax))
    f = np.zeros(fsize, dtype=np.complex128) if store_flmn else None
    st = _lib.lib.catana_gpu_sfb_raw(_lib.ptr(pts), _lib.ptr(w), n, lmax, nmax, float(rmax),
                                     _flags(interpolation, precision), _lib.ptr(k), _lib.ptr(c), _lib.ptr(f), None)
    _lib.check(st, "sfb_raw")
    if verbose:
        print("Done (%.3f s)." % (time.perf_counter() - t0))
    return KClkk(k, c, unpack_flmn(f, lmax, nmax) if store_flmn else [])


def _healpix(ppc, lmax, nmax, rmax, store_flmn, verbose, interpolation, conj_fix):
    if verbose:
        print("SFB decomposition (reverse method): lmax=%d nmax=%d NSide=%d" % (lmax, nmax, ppc.nside))
        print("Catalog consists of %d points." % ppc.get_npoints())
        sys.stdout.flush()
    t0 = time.perf_counter()
    k = np.zeros((lmax, nmax))
    c = np.zeros((lmax, nmax))
    fsize = int(_lib.lib.catana_gpu_flmn_size(lmax, nmax))
    f = np.zeros(fsize, dtype=np.complex128) if store_flmn else None
    flags = _flags(interpolation, "plain") | (_lib.HEALPIX_CONJ_FIX if conj_fix else 0)
    rs = ppc.r_sorted if ppc.r_sorted.size else np.zeros(1)
    st = _lib.lib.catana_gpu_sfb_healpix(ppc.nside, _lib.ptr(ppc.offsets), _lib.ptr(rs), lmax, nmax, float(rmax),
                                         flags, _lib.ptr(k), _lib.ptr(c), _lib.ptr(f), None)
    _lib.check(st, "sfb_healpix")
    if verbose:
        print("Done (%.3f s)." % (time.perf_counter() - t0))
    return KClkk(k, c, unpack_flmn(f, lmax, nmax) if store_flmn else [])


def sfb_decomposition(point_container, lmax, nmax, rmax, store_flmn=False, verbose=True, weights=None,
                      precision="plain", interpolation="auto", conj_fix=False):
    """Compute the SFB transform of a PointContainer (raw method) or of a
    PixelizedPointContainer (HEALPix method).  Returns a KClkk."""
    lmax = _unsigned_short(lmax, "lmax")
    nmax = _unsigned_short(nmax, "nmax")
    rmax = float(rmax)
    if isinstance(point_container, PixelizedPointContainer):
        if weights is not None or precision != "plain":
            raise ValueError("the HEALPix method takes no weights and runs in FP64 only")
        return _healpix(point_container, lmax, nmax, rmax, store_flmn, verbose, interpolation, conj_fix)
    if not isinstance(point_container, PointContainer):
        raise TypeError("sfb_decomposition expects a PointContainer or a PixelizedPointContainer")
    return _raw(point_container, lmax, nmax, rmax, store_flmn, verbose, weights, precision, interpolation)


def sfb_reverse(pixelized_point_container, lmax, nmax, rmax, store_flmn=False, verbose=True, interpolated=True):
    """The pixelized SFB without FFT, the reference's _sfb_reverse (sfb_reverse.cpp:13-112):
    per l, f = Y*_lm(pixel centres) x (per-pixel sums of j_l(k_ln r)).  `interpolated`
    picks the j_l branch as in that function.  Returns a KClkk."""
    ppc = pixelized_point_container
    if not isinstance(ppc, PixelizedPointContainer):
        raise TypeError("sfb_reverse expects a PixelizedPointContainer")
    lmax = _unsigned_short(lmax, "lmax")
    nmax = _unsigned_short(nmax, "nmax")
    if verbose:
        print("SFB decomposition (reverse method): lmax=%d nmax=%d NSide=%d" % (lmax, nmax, ppc.nside))
        print("Catalog consists of %d points." % ppc.get_npoints())
        sys.stdout.flush()
    k = np.zeros((lmax, nmax))
    c = np.zeros((lmax, nmax))
    f = np.zeros(int(_lib.lib.catana_gpu_flmn_size(lmax, nmax)), dtype=np.complex128) if store_flmn else None
    rs = ppc.r_sorted if ppc.r_sorted.size else np.zeros(1)
    flags = _lib.JL_INTERP if interpolated else _lib.JL_EXACT
    st = _lib.lib.catana_gpu_sfb_reverse(ppc.nside, _lib.ptr(ppc.offsets), _lib.ptr(rs), lmax, nmax, float(rmax),
                                         flags, _lib.ptr(k), _lib.ptr(c), _lib.ptr(f), None)
    _lib.check(st, "sfb_reverse")
    return KClkk(k, c, unpack_flmn(f, lmax, nmax) if store_flmn else [])


def sfb_decomposition_healpix(pixelized_point_container, lmax, nmax, rmax, store_flmn=False, verbose=True,
                              interpolation="auto", conj_fix=False):
    """Alias of sfb_decomposition for a PixelizedPointContainer."""
    if not isinstance(pixelized_point_container, PixelizedPointContainer):
        raise TypeError("sfb_decomposition_healpix expects a PixelizedPointContainer")
    return sfb_decomposition(pixelized_point_container, lmax, nmax, rmax, store_flmn, verbose,
                             interpolation=interpolation, conj_fix=conj_fix)


def sfb_decomposition_batched(point_containers, lmax, nmax, rmax, kmax=None, weights=None, store_flmn=False,
                              verbose=True, precision="split", interpolation="auto", waves=0.0, graph=True,
                              mblock=128):
    """Decompose many catalogs in one call (no counterpart in the reference).

    point_containers: sequence of PointContainer (or (N, 3) arrays of r, theta, phi).
    lmax, nmax, rmax, kmax, weights: one value for all catalogs or one per catalog;
    kmax > 0 keeps only the modes with k_ln <= kmax (the others have f = C = 0).
    precision='split' runs all catalogs level by level in grouped tcgen05 launches,
    captured as one CUDA graph (graph=False launches the levels directly); waves sets
    the work items per SM and mblock (128 or 64) the most complex m per work item (the
    MMA tile's N); waves <= 0 autotunes both.  precision='plain' runs the FP64 path per
    catalog.
    Returns a list of KClkk.
    """
    cats = list(point_containers)
    nc = len(cats)

    def per(v, name, conv):
        if isinstance(v, (list, tuple, np.ndarray)):
            if len(v) != nc:
                raise ValueError("%s: one value per catalog expected" % name)
            return [conv(x) for x in v]
        return [conv(v)] * nc

    lmaxs = per(lmax, "lmax", lambda x: _unsigned_short(x, "lmax"))
    nmaxs = per(nmax, "nmax", lambda x: _unsigned_short(x, "nmax"))
    rmaxs = per(rmax, "rmax", float)
    kmaxs = per(0.0 if kmax is None else kmax, "kmax", lambda x: 0.0 if x is None else float(x))
    ws = [None] * nc if weights is None else per(weights, "weights", lambda x: x)
    if mblock not in (128, 64):
        raise ValueError("mblock must be 128 or 64")
    flags = _flags(interpolation, precision) | (0 if graph else _lib.BATCH_NO_GRAPH) | \
        (_lib.BATCH_MBLK64 if mblock == 64 else 0)
    recs = (_lib.Catalog * max(nc, 1))()
    keep, out = [], []
    for i, pc in enumerate(cats):
        pts = np.ascontiguousarray(np.asarray(pc, dtype=np.float64).reshape(-1, 3))
        w = None
        if ws[i] is not None:
            w = np.ascontiguousarray(ws[i], dtype=np.float64).reshape(-1)
            if w.shape[0] != pts.shape[0]:
                raise ValueError("weights of catalog %d must have one entry per point" % i)
        k = np.zeros((lmaxs[i], nmaxs[i]))
        c = np.zeros((lmaxs[i], nmaxs[i]))
        f = np.zeros(int(_lib.lib.catana_gpu_flmn_size(lmaxs[i], nmaxs[i])), dtype=np.complex128) \
            if store_flmn else None
        r = recs[i]
        r.points, r.weights, r.npoints = pts.ctypes.data, (w.ctypes.data if w is not None else None), pts.shape[0]
        r.rmax, r.kmax, r.lmax, r.nmax = rmaxs[i], kmaxs[i], lmaxs[i], nmaxs[i]
        r.k_ln, r.c_ln, r.f_lmn = k.ctypes.data, c.ctypes.data, (f.ctypes.data if f is not None else None)
        keep.append((pts, w))
        out.append((k, c, f))
    if verbose:
        print("SFB decomposition (raw method, batched): %d catalogs, %d points" %
              (nc, sum(p.shape[0] for p, _ in keep)))
        sys.stdout.flush()
    t0 = time.perf_counter()
    st = _lib.lib.catana_gpu_sfb_raw_batched(ctypes.cast(recs, ctypes.c_void_p), nc, flags, float(waves), None)
    _lib.check(st, "sfb_raw_batched")
    if verbose:
        print("Done (%.3f s)." % (time.perf_counter() - t0))
    return [KClkk(k, c, unpack_flmn(f, lmaxs[i], nmaxs[i]) if store_flmn else [])
            for i, (k, c, f) in enumerate(out)]


def _ingest_spec(records, coordinate_type, tophat_r0, gauss_r0, window, window_range, mask, seed, index0):
    rec = np.asarray(records)
    f32 = rec.dtype == np.float32
    rec = np.ascontiguousarray(rec, dtype=np.float32 if f32 else np.float64).reshape(-1, 3)
    if coordinate_type not in ("spherical", "cartesian"):
        raise RuntimeError("coord_type either 'cartesian' or 'spherical'")
    sp = _lib.IngestSpec()
    sp.layout = (_lib.REC_FLOAT32 if f32 else _lib.REC_FLOAT64) | \
        (_lib.REC_CARTESIAN if coordinate_type == "cartesian" else _lib.REC_SPHERICAL)
    sp.tophat_r0 = float(tophat_r0 or 0.0)
    sp.gauss_r0 = float(gauss_r0 or 0.0)
    keep = [rec]
    if window is not None:
        w = np.ascontiguousarray(window, dtype=np.float64)
        keep.append(w)
        sp.window, sp.window_n = w.ctypes.data, w.size
        sp.window_min, sp.window_max = float(window_range[0]), float(window_range[1])
    if mask is not None:
        m = np.ascontiguousarray(mask, dtype=np.float32)
        nside = int(round(np.sqrt(m.size / 12)))
        if 12 * nside * nside != m.size:
            raise RuntimeError("healpix_map is not a valid map (check size!)")
        keep.append(m)
        sp.mask, sp.mask_nside = m.ctypes.data, nside
    sp.seed, sp.index0 = int(seed), int(index0)
    return rec, sp, keep


def ingest(records, coordinate_type="spherical", tophat_r0=None, gauss_r0=None, window=None, window_range=(0.0, 1.0),
           mask=None, seed=0, index0=0):
    """Convert and filter a block of records on the GPU (no counterpart in the reference's
    Python API; the filters are its TophatRadialWindowFunctionFilter,
    GaussianRadialWindowFunctionFilter, GenericRadialWindowFunctionFilter with an
    interpolated window, and AngularMaskFilter).  records: (N, 3) float32 or float64,
    (x, y, z) or (r, theta, phi).  Random windows keep record i when w(r) > u_i with u_i
    a hash of (seed, index0 + i).  Returns a PointContainer of the kept points, in order."""
    rec, sp, keep = _ingest_spec(records, coordinate_type, tophat_r0, gauss_r0, window, window_range, mask, seed,
                                 index0)
    n = rec.shape[0]
    out = np.zeros((max(n, 1), 3))
    nout = ctypes.c_int64(0)
    _lib.check(_lib.lib.catana_gpu_ingest(_lib.ptr(rec), n, ctypes.byref(sp), _lib.ptr(out), ctypes.byref(nout), None),
               "ingest")
    return PointContainer(out[:nout.value])


class SFBAccumulator(object):
    """Raw SFB decomposition of one catalog fed in chunks (no counterpart in the
    reference).  ``add(points, weights=None)`` takes an (N, 3) array of (r, theta,
    phi) -- float32 (the SphericalRecord<float> layout) or float64; pinned host
    memory (e.g. a pinned torch tensor's numpy view) lets the copy of a chunk overlap
    the decomposition of the previous one.  ``finish(store_flmn=False)`` returns the
    KClkk of all points added, normalised by the total count (or weight sum).

        with SFBAccumulator(512, 256, 1500.0, precision="split") as acc:
            for chunk in chunks:
                acc.add(chunk)
            result = acc.finish()
    """

    def __init__(self, lmax, nmax, rmax, precision="split", interpolation="auto"):
        self.lmax = _unsigned_short(lmax, "lmax")
        self.nmax = _unsigned_short(nmax, "nmax")
        self.rmax = float(rmax)
        h = ctypes.c_void_p()
        _lib.check(_lib.lib.catana_gpu_accum_create(self.lmax, self.nmax, self.rmax, _flags(interpolation, precision),
                                                    ctypes.byref(h)), "accum_create")
        self._h = h
        self._keep = []  # the last chunks stay alive until the library has copied them

    def add(self, points, weights=None):
        pts = np.asarray(points)
        f32 = pts.dtype == np.float32
        pts = np.ascontiguousarray(pts, dtype=np.float32 if f32 else np.float64).reshape(-1, 3)
        w = None
        if weights is not None:
            w = np.ascontiguousarray(weights, dtype=pts.dtype).reshape(-1)
            if w.shape[0] != pts.shape[0]:
                raise ValueError("weights must have one entry per point")
        fn = _lib.lib.catana_gpu_accum_add_f32 if f32 else _lib.lib.catana_gpu_accum_add
        _lib.check(fn(self._h, _lib.ptr(pts), _lib.ptr(w), pts.shape[0]), "accum_add")
        self._keep = (self._keep + [(pts, w)])[-2:]

    def add_records(self, records, coordinate_type="spherical", tophat_r0=None, gauss_r0=None, window=None,
                    window_range=(0.0, 1.0), mask=None, seed=0, index0=None):
        """Add a chunk of raw records, converted and filtered on the GPU as ``ingest``
        does; index0 defaults to the number of records added so far."""
        if index0 is None:
            index0 = getattr(self, "_records_seen", 0)
        rec, sp, keep = _ingest_spec(records, coordinate_type, tophat_r0, gauss_r0, window, window_range, mask, seed,
                                     index0)
        _lib.check(_lib.lib.catana_gpu_accum_add_records(self._h, _lib.ptr(rec), rec.shape[0], ctypes.byref(sp)),
                   "accum_add_records")
        self._records_seen = int(index0) + rec.shape[0]
        self._keep = (self._keep + [tuple(keep)])[-2:]

    def add_file(self, filename, coordinate_type="spherical", dtype=np.float32, first_record=0, max_records=-1,
                 chunk=8_000_000, tophat_r0=None, gauss_r0=None, window=None, window_range=(0.0, 1.0), mask=None,
                 seed=0):
        """Stream a raw binary record file (the RawBinarySource format: consecutive records
        of 3 float32 or float64, Cartesian or spherical) through the GPU ingest into this
        accumulation, `chunk` records at a time; file reads overlap the decomposition.
        Returns the number of records read."""
        dt = np.dtype(dtype)
        if dt not in (np.dtype(np.float32), np.dtype(np.float64)):
            raise ValueError("dtype must be float32 or float64")
        proto = np.zeros((1, 3), dtype=dt)
        _, sp, keep = _ingest_spec(proto, coordinate_type, tophat_r0, gauss_r0, window, window_range, mask, seed, 0)
        n = ctypes.c_int64(0)
        _lib.check(_lib.lib.catana_gpu_accum_add_file(self._h, str(filename).encode(), int(first_record),
                                                      int(max_records), int(chunk), ctypes.byref(sp),
                                                      ctypes.byref(n)), "accum_add_file")
        return n.value

    def finish(self, store_flmn=False):
        k = np.zeros((self.lmax, self.nmax))
        c = np.zeros((self.lmax, self.nmax))
        f = np.zeros(int(_lib.lib.catana_gpu_flmn_size(self.lmax, self.nmax)), dtype=np.complex128) \
            if store_flmn else None
        _lib.check(_lib.lib.catana_gpu_accum_finish(self._h, _lib.ptr(k), _lib.ptr(c), _lib.ptr(f)), "accum_finish")
        self._keep = []
        return KClkk(k, c, unpack_flmn(f, self.lmax, self.nmax) if store_flmn else [])

    def close(self):
        if self._h is not None:
            _lib.lib.catana_gpu_accum_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def compute_kln(lmax, nmax, rmax):
    """k_ln = z_{l,n} / rmax (return_types.cpp:10-20), as a (lmax, nmax) array."""
    lmax = _unsigned_short(lmax, "lmax")
    nmax = _unsigned_short(nmax, "nmax")
    k = np.zeros((lmax, nmax))
    _lib.check(_lib.lib.catana_gpu_compute_kln(lmax, nmax, float(rmax), _lib.ptr(k)), "compute_kln")
    return k
