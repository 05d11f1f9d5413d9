"""ctypes front-end of the CPU oracle (catana_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()`` as
the checker, and by ``bench.py``'s CPU-baseline leg.  The product package
(catana_gb300) never imports this module.

Builds ``oracle/_build/libcatana_oracle.so`` with the Makefile beside it on first
use when it is missing.  ``ref_lib()`` loads the reference's own besseltools
sources compiled by ``make -C oracle ref`` (only possible where the reference
tree exists); it returns None elsewhere.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libcatana_oracle.so")
_REF_PATH = os.path.join(_HERE, "_ref", "libref_besseltools.so")
_lib = None
_ref = None

_D = ctypes.c_double
_I = ctypes.c_int
_I64 = ctypes.c_int64
_P = ctypes.c_void_p


def build(force=False):
    if force or not os.path.exists(_LIB_PATH):
        subprocess.run(["make", "-s", "-C", _HERE, "all"], check=True)


def build_ref(ref_root=None):
    """Compile the reference's besseltools sources where the reference tree exists.
    The tree is ref_root, else $CATANA_REFERENCE_DIR, else the recipe's default
    location (oracle/Makefile, REF); without a tree nothing is built.  Returns
    whether oracle/_ref holds the library afterwards."""
    ref_root = ref_root or os.environ.get("CATANA_REFERENCE_DIR")
    cmd = ["make", "-s", "-C", _HERE, "ref-if-present"]
    if ref_root:
        cmd.append("REF=" + ref_root)
    subprocess.run(cmd, check=True)
    return os.path.exists(_REF_PATH)


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        L.co_sbessel_jl.restype = _D
        L.co_sbessel_jl.argtypes = [_I, _D]
        L.co_sph_plm.restype = _D
        L.co_sph_plm.argtypes = [_I, _I, _D]
        L.co_sbessel_zeros.restype = None
        L.co_sbessel_zeros.argtypes = [ctypes.c_uint, _I, _P]
        L.co_compute_kln.restype = None
        L.co_compute_kln.argtypes = [_I, _I, _D, _P]
        L.co_lerp_table.restype = None
        L.co_lerp_table.argtypes = [_I, _D, _I, _P, _P]
        L.co_lerp_eval_pub.restype = _D
        L.co_lerp_eval_pub.argtypes = [_P, _I, _D, _D, _D, _P]
        L.co_sfb_raw.restype = _I
        L.co_sfb_raw.argtypes = [_P, _P, _I64, _I, _I, _D, _I, _I, _P, _P, _P, _P]
        L.co_ang2pix_ring.restype = _I64
        L.co_ang2pix_ring.argtypes = [_I64, _D, _D]
        L.co_pix2ang_ring.restype = None
        L.co_pix2ang_ring.argtypes = [_I64, _I64, _P, _P]
        L.co_healpix_maps.restype = _I
        L.co_healpix_maps.argtypes = [_I64, _P, _P, _I, _I, _P, _D, _I, _I, _P]
        L.co_ring_info.restype = None
        L.co_ring_info.argtypes = [_I64, _I64, _P, _P]
        L.co_bin_points.restype = _I
        L.co_bin_points.argtypes = [_I64, _P, _I64, _P, _P]
        L.co_sfb_healpix.restype = _I
        L.co_sfb_healpix.argtypes = [_I64, _P, _P, _I, _I, _D, _I, _I, _P, _P, _P, _P]
        L.co_sfb_reverse.restype = _I
        L.co_sfb_reverse.argtypes = [_I64, _P, _P, _I, _I, _D, _I, _I, _P, _P, _P, _P]
        L.co_ingest.restype = _I
        L.co_ingest.argtypes = [_P, _I64, ctypes.c_uint, _D, _D, _P, _I64, _D, _D, _P, _I64, ctypes.c_uint64,
                                ctypes.c_uint64, _P, _P]
        L.co_dsb_integral.restype = _I
        L.co_dsb_integral.argtypes = [_P, _I64, _D, _D, _I, _D, _D, _D, _P]
        L.co_cartesian_to_spherical.restype = None
        L.co_cartesian_to_spherical.argtypes = [_P, _I64, _P]
        _lib = L
    return _lib


def ref_lib():
    """The reference's SphericalBesselZeros/SBesselInterpolator, or None."""
    global _ref
    if _ref is None:
        if not os.path.exists(_REF_PATH):
            return None
        R = ctypes.CDLL(_REF_PATH)
        R.ref_sbessel_zeros.restype = None
        R.ref_sbessel_zeros.argtypes = [ctypes.c_uint, _I, _P]
        R.ref_interp_table.restype = None
        R.ref_interp_table.argtypes = [ctypes.c_ushort, ctypes.c_ushort, ctypes.c_uint, _P, _P]
        R.ref_interp_eval.restype = _I
        R.ref_interp_eval.argtypes = [ctypes.c_ushort, ctypes.c_ushort, ctypes.c_uint, _P, _I, _P]
        _ref = R
    return _ref


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def sbessel_jl(l, x):
    return lib().co_sbessel_jl(int(l), float(x))


def sph_plm(l, m, x):
    return lib().co_sph_plm(int(l), int(m), float(x))


def sbessel_zeros(l, count):
    out = np.zeros(count, dtype=np.float64)
    lib().co_sbessel_zeros(int(l), int(count), _ptr(out))
    return out


def compute_kln(lmax, nmax, rmax):
    out = np.zeros((lmax, nmax), dtype=np.float64)
    lib().co_compute_kln(int(lmax), int(nmax), float(rmax), _ptr(out))
    return out


def lerp_table(l, zmax, npts):
    y = np.zeros(npts, dtype=np.float64)
    dxi = np.zeros(1, dtype=np.float64)
    lib().co_lerp_table(int(l), float(zmax), int(npts), _ptr(y), _ptr(dxi))
    return y, float(dxi[0])


def cartesian_to_spherical(xyz):
    xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
    out = np.zeros_like(xyz)
    lib().co_cartesian_to_spherical(_ptr(xyz), xyz.shape[0], _ptr(out))
    return out


def sfb_raw(pts, lmax, nmax, rmax, interpolated, weights=None, store_flmn=True, nthreads=0):
    """Raw SFB decomposition (sfb_raw.cpp:13-108).

    pts: (N, 3) float64 (r, theta, phi).  Returns (k_ln, c_ln, f_lmn) where f_lmn is
    a list of complex128 (l+1, nmax) arrays (empty when store_flmn is False).
    """
    pts = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1, 3)
    w = None if weights is None else np.ascontiguousarray(weights, dtype=np.float64)
    k = np.zeros((lmax, nmax))
    c = np.zeros((lmax, nmax))
    nf = nmax * lmax * (lmax + 1) // 2
    fre = np.zeros(nf) if store_flmn else None
    fim = np.zeros(nf) if store_flmn else None
    rc = lib().co_sfb_raw(_ptr(pts), _ptr(w), pts.shape[0], int(lmax), int(nmax), float(rmax),
                          int(bool(interpolated)), int(nthreads), _ptr(k), _ptr(c), _ptr(fre), _ptr(fim))
    if rc == 2:
        raise ValueError("argument (z) outside of defined range.")
    return k, c, _unpack_f(fre, fim, lmax, nmax) if store_flmn else []


def _unpack_f(fre, fim, lmax, nmax):
    out, off = [], 0
    for l in range(lmax):
        s = (l + 1) * nmax
        out.append((fre[off:off + s] + 1j * fim[off:off + s]).reshape(l + 1, nmax))
        off += s
    return out


def ang2pix_ring(nside, theta, phi):
    L = lib()
    th = np.asarray(theta, dtype=np.float64).ravel()
    ph = np.asarray(phi, dtype=np.float64).ravel()
    return np.array([L.co_ang2pix_ring(int(nside), float(a), float(b)) for a, b in zip(th, ph)], dtype=np.int64)


def pix2ang_ring(nside, pix):
    L = lib()
    t = np.zeros(1)
    p = np.zeros(1)
    th, ph = [], []
    for q in np.asarray(pix).ravel():
        L.co_pix2ang_ring(int(nside), int(q), _ptr(t), _ptr(p))
        th.append(t[0])
        ph.append(p[0])
    return np.array(th), np.array(ph)


def ring_info(nside, ring):
    s = np.zeros(1, dtype=np.int64)
    n = np.zeros(1, dtype=np.int64)
    lib().co_ring_info(int(nside), int(ring), _ptr(s), _ptr(n))
    return int(s[0]), int(n[0])


def bin_points(nside, pts):
    pts = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1, 3)
    npix = 12 * nside * nside
    offs = np.zeros(npix + 1, dtype=np.int64)
    rs = np.zeros(max(pts.shape[0], 1), dtype=np.float64)
    rc = lib().co_bin_points(int(nside), _ptr(pts), pts.shape[0], _ptr(offs), _ptr(rs))
    if rc != 0:
        raise ValueError("theta outside [0, pi]")
    return offs, rs[:pts.shape[0]]


def sfb_reverse(nside, offsets, r_sorted, lmax, nmax, rmax, interpolated, nthreads=0):
    """Pixelized SFB without FFT: dense Y(m, pixel) x map(pixel, n) per l (sfb_reverse.cpp:13-112)."""
    offsets = np.ascontiguousarray(offsets, dtype=np.int64)
    r_sorted = np.ascontiguousarray(r_sorted, dtype=np.float64)
    k = np.zeros((lmax, nmax))
    c = np.zeros((lmax, nmax))
    nf = nmax * lmax * (lmax + 1) // 2
    fre = np.zeros(max(nf, 1))
    fim = np.zeros(max(nf, 1))
    rc = lib().co_sfb_reverse(int(nside), _ptr(offsets), _ptr(r_sorted), int(lmax), int(nmax), float(rmax),
                              int(bool(interpolated)), int(nthreads), _ptr(k), _ptr(c), _ptr(fre), _ptr(fim))
    if rc == 2:
        raise ValueError("argument (z) outside of defined range.")
    return k, c, _unpack_f(fre, fim, lmax, nmax)


def sfb_healpix(nside, offsets, r_sorted, lmax, nmax, rmax, interpolated, store_flmn=True, nthreads=0):
    """HEALPix SFB decomposition (sfb_reverse_fft.cpp:43-209)."""
    offsets = np.ascontiguousarray(offsets, dtype=np.int64)
    r_sorted = np.ascontiguousarray(r_sorted, dtype=np.float64)
    k = np.zeros((lmax, nmax))
    c = np.zeros((lmax, nmax))
    nf = nmax * lmax * (lmax + 1) // 2
    fre = np.zeros(nf) if store_flmn else None
    fim = np.zeros(nf) if store_flmn else None
    rc = lib().co_sfb_healpix(int(nside), _ptr(offsets), _ptr(r_sorted), int(lmax), int(nmax), float(rmax),
                              int(bool(interpolated)), int(nthreads), _ptr(k), _ptr(c), _ptr(fre), _ptr(fim))
    if rc == 2:
        raise ValueError("argument (z) outside of defined range.")
    return k, c, _unpack_f(fre, fim, lmax, nmax) if store_flmn else []


def sfb_healpix_fft(nside, offsets, r_sorted, lmax, nmax, rmax, interpolated, nthreads=0):
    """HEALPix SFB decomposition with each ring's transform as an FFT, the way the
    reference computes it (sfb_reverse_fft.cpp:43-209: an FFTW r2c transform per ring;
    numpy's rfft here, rings of one length transformed together), with the same pixel
    maps (co_healpix_maps), the same m-extraction without conjugation (s = N/2 -
    |N/2 - m mod N|, imaginary part dropped at m = 0), ring phase and normalisation as
    sfb_healpix, the direct-DFT restatement it reproduces to rounding.  Returns
    (k_ln, c_ln, f_lmn) with f_lmn[l] of shape (l + 1, nmax)."""
    offsets = np.ascontiguousarray(offsets, dtype=np.int64)
    r_sorted = np.ascontiguousarray(r_sorted, dtype=np.float64)
    npix, nrings = 12 * nside * nside, 4 * nside - 1
    k = compute_kln(lmax, nmax, rmax)
    npts = int(offsets[npix])
    norm = np.sqrt(2.0 / np.pi) * (4.0 / 3.0) * np.pi * rmax ** 3 / npts
    starts = np.zeros(nrings, dtype=np.int64)
    lens = np.zeros(nrings, dtype=np.int64)
    for i in range(nrings):
        st, ln = ctypes.c_int64(), ctypes.c_int64()
        lib().co_ring_info(int(nside), i + 1, ctypes.byref(st), ctypes.byref(ln))
        starts[i], lens[i] = st.value, ln.value
    th, ph0 = pix2ang_ring(nside, starts)
    costh = np.cos(th)
    groups = {}
    for i in range(nrings):
        groups.setdefault(int(lens[i]), []).append(i)
    c = np.zeros((lmax, nmax))
    f = []
    maps = np.zeros((npix, max(nmax, 1)))
    for l in range(lmax):
        krow = np.ascontiguousarray(k[l])
        rc = lib().co_healpix_maps(int(npix), _ptr(offsets), _ptr(r_sorted), int(l), int(nmax), _ptr(krow),
                                   float(rmax), int(bool(interpolated)), int(nthreads), _ptr(maps))
        if rc == 2:
            raise ValueError("argument (z) outside of defined range.")
        y = np.empty((nrings, l + 1), dtype=np.complex128)
        for i in range(nrings):
            for m in range(l + 1):
                y[i, m] = sph_plm(l, m, costh[i]) * np.exp(-1j * m * ph0[i])
        acc = np.zeros((l + 1, nmax), dtype=np.complex128)
        for n_len, ridx in groups.items():
            ridx = np.asarray(ridx)
            block = np.stack([maps[starts[i]:starts[i] + n_len, :nmax] for i in ridx])  # (R, N, nmax)
            spec = np.fft.rfft(block, axis=1)                                          # F[s] = sum_j x_j e^{-2 pi i j s / N}
            mm = np.arange(l + 1) % n_len
            val = spec[:, n_len // 2 - np.abs(n_len // 2 - mm), :]                    # (R, l + 1, nmax)
            val[:, 0, :] = val[:, 0, :].real                                           # sign 0 at m = 0
            acc += np.einsum("rmn,rm->mn", val, y[ridx])
        f.append(acc * k[l][None, :] * norm)
        sq = np.sum(np.abs(acc) ** 2, axis=0)
        c[l] = (2.0 * sq - np.abs(acc[0]) ** 2) * (norm * k[l]) ** 2 / (2 * l + 1)
    return k, c, f


def ingest(records, cartesian=False, tophat_r0=0.0, gauss_r0=0.0, window=None, window_range=(0.0, 1.0), mask=None,
           seed=0, index0=0):
    """Record conversion and point filters (restatement of the device ingest; see
    catana_oracle.c co_ingest).  records: (N, 3) float32 or float64."""
    rec = np.ascontiguousarray(records)
    f32 = rec.dtype == np.float32
    rec = np.ascontiguousarray(rec, dtype=np.float32 if f32 else np.float64).reshape(-1, 3)
    n = rec.shape[0]
    out = np.zeros((max(n, 1), 3))
    nout = np.zeros(1, dtype=np.int64)
    win = None if window is None else np.ascontiguousarray(window, dtype=np.float64)
    msk = None if mask is None else np.ascontiguousarray(mask, dtype=np.float32)
    mnside = 0 if msk is None else int(round(np.sqrt(msk.size / 12)))
    rc = lib().co_ingest(_ptr(rec), n, (1 if f32 else 0) | (2 if cartesian else 0), float(tophat_r0), float(gauss_r0),
                         _ptr(win), 0 if win is None else win.size, float(window_range[0]), float(window_range[1]),
                         _ptr(msk), mnside, int(seed), int(index0), _ptr(out), _ptr(nout))
    if rc == 2:
        raise ValueError("ingest: radius outside the window's range or theta outside [0, pi]")
    return out[:int(nout[0])].copy()


def dsb_integral(w_table, w_range, l, rmax, k1, k2):
    """int_0^rmax w(r) j_l(k1 r) j_l(k2 r) dr with w a FunctionInterpolator table on
    w_range (restatement of sbessel_integrator.cpp:53-110; see co_dsb_integral)."""
    wt = np.ascontiguousarray(w_table, dtype=np.float64)
    out = np.zeros(1)
    rc = lib().co_dsb_integral(_ptr(wt), wt.size, float(w_range[0]), float(w_range[1]), int(l), float(rmax),
                               float(k1), float(k2), _ptr(out))
    if rc == 2:
        raise ValueError("argument outside range for which this FunctionInterpolator is defined")
    return float(out[0])
